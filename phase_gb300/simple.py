"""One SIMPLE step of the lid-driven cavity on the device, producing the
pressure-correction system fv::laplacian(rho*d, pCorr) == src::div(rho*u*).

Phase has no SIMPLE solver (its solvers are fractional-step), so this
driver is project code written over the library's own operators:

1. momentum predictor  ddt(u) + div(u_f, u) - laplacian(mu/rho, u) = 0
   (pg_assemble_momentum), solved per component on the device from the
   device matrix (pg_solver_set_eqn_component);
2. d_P = V_P / a_P from the momentum diagonal, interpolated to the faces
   with the distance weights (pg_interpolate_faces);
3. u*_f = interpolated predictor velocity on interior faces, the boundary
   values on boundary faces;
4. pCorr equation with face coefficient rho*d_f and rhs src::div(rho u*_f),
   normal-gradient on every wall (the system is singular with the constants
   as null space and a consistent rhs).

Case (Examples/LidDrivenCavity): unit square, 80 x 80 cells, rho = 1,
mu = 0.01, lid u = (1, 0) on y+, no slip elsewhere, dt = 0.005, from rest.
"""
from __future__ import annotations

import numpy as np

from . import meshes


def cavity_inputs(nx=80, ny=80, lid=1.0, faces=None):
    nodes, cptr, cind = meshes.rectilinear(nx, ny, 1.0, 1.0)
    out = dict(nodes=nodes, cptr=cptr, cind=cind, nx=nx, ny=ny)
    if faces is not None:
        patch = meshes.rect_patch_of_faces(faces["fx"], faces["fy"],
                                           faces["rcell"], 1.0, 1.0)
        bnd = faces["rcell"] < 0
        nf = faces["rcell"].size
        bc_u = np.where(bnd, 0, 1).astype(np.int32)  # FIXED walls and lid
        u_face = np.zeros((nf, 2))
        u_face[patch == 3, 0] = lid
        bc_p = np.ones(nf, np.int32)                 # NORMAL_GRADIENT
        out.update(patch=patch, bc_u=bc_u, u_face=u_face, bc_p=bc_p)
    return out


def predictor_pcorr(pg, mesh, bc_u, u_face, u0, bc_p, p_value, rho, mu, dt,
                    tol=1e-12):
    """Momentum predictor from u0 (cells) with boundary velocities u_face,
    then the pCorr equation laplacian(rho d_f, pCorr) == div(rho u*_f) with
    pressure boundary types bc_p and values p_value (per face).

    Device-resident: the momentum operator is assembled on the device, each
    velocity component is solved from it by the device solver
    (pg_solver_set_eqn_component, one factorisation for both), d = V / a_P
    comes from the device diagonal, the face values are interpolated and
    the pCorr equation assembled on the device; only the returned fields
    are copied to the host (for inspection)."""
    import torch

    dev = torch.device("cuda", torch.cuda.current_device())
    f64 = torch.float64
    n, nf = mesh.n_cells, mesh.n_faces
    on_dev = lambda a: torch.from_numpy(
        np.ascontiguousarray(a, np.float64)).to(dev)
    faces, cells = mesh.faces(), mesh.cells()
    u0_d = on_dev(np.asarray(u0).reshape(-1))
    ufb_d = on_dev(np.asarray(u_face).reshape(-1))
    torch.cuda.synchronize()
    mom = pg.MomentumEquation(mesh, bc_u).assemble_device(
        dt, mu / rho, 1.0, u0_d.data_ptr(), ufb_d.data_ptr())
    s = pg.SparseMatrixSolver(tolerance=tol, max_iters=5000)
    u_d = torch.empty((2, n), dtype=f64, device=dev)
    for d in range(2):
        s.set_eqn(mom, component=d)
        s.setGuess(None)
        s.solve()
        s.x_device(u_d[d].data_ptr())
    # the library and torch run on their own streams: each hands over after
    # a synchronisation
    a_p = torch.empty(n, dtype=f64, device=dev)
    mom.diagonal(a_p.data_ptr())
    pg.synchronize()
    dcoef = on_dev(cells["vol"]) / a_p
    gamma_f = torch.empty(nf, dtype=f64, device=dev)
    uf = torch.empty((2, nf), dtype=f64, device=dev)
    torch.cuda.synchronize()
    mesh.interpolate_faces_device(dcoef.data_ptr(), gamma_f.data_ptr())
    for d in range(2):
        mesh.interpolate_faces_device(u_d[d].data_ptr(), uf[d].data_ptr())
    pg.synchronize()
    gamma_f *= rho
    uf = uf.t().contiguous()
    bnd = on_dev((faces["rcell"] < 0).astype(np.float64)).bool()
    uf[bnd] = ufb_d.view(nf, 2)[bnd]
    rho_uf = (rho * uf).contiguous()
    pv = None if p_value is None else on_dev(p_value)
    torch.cuda.synchronize()
    eqn = pg.Equation(mesh, pg.GAMMA_FACE, bc_p).assemble_device(
        gamma_face=gamma_f.data_ptr(),
        bc_value=0 if pv is None else pv.data_ptr(), u_face=rho_uf.data_ptr())
    pg.synchronize()
    return dict(mesh=mesh, eqn=eqn, u=u_d.t().cpu().numpy(),
                d=dcoef.cpu().numpy(), gamma_f=gamma_f.cpu().numpy(),
                u_face=uf.cpu().numpy(), momentum=mom,
                momentum_iters=s.nIters())


def simple_pcorr(pg, nx=80, ny=80, rho=1.0, mu=0.01, dt=0.005, lid=1.0,
                 tol=1e-12):
    """Run the predictor on the device and return the pCorr equation and
    the intermediate fields."""
    w = cavity_inputs(nx, ny, lid)
    mesh = pg.Mesh(w["nodes"], w["cptr"], w["cind"])
    w = cavity_inputs(nx, ny, lid, mesh.faces())
    u0 = np.zeros((mesh.n_cells, 2))
    out = predictor_pcorr(pg, mesh, w["bc_u"], w["u_face"], u0, w["bc_p"],
                          None, rho, mu, dt, tol)
    out["inputs"] = w
    return out


def cylinder_pcorr(pg, mesh_args=None, u_in=1.0, re=100.0, rho=1.0, dt=0.01,
                   tol=1e-10):
    """The pressure-correction system of one PISO-style predictor step of
    the flow around a cylinder (D = 1, Re = u_in D / nu) on the graded
    triangle mesh of meshes.cylinder_channel, boundary types as
    Examples/UnstructuredFlowAroundCylinder/case/boundaries.info: u fixed
    (u_in, 0) at the inlet and 0 on the cylinder, normal gradient at the
    outlet and on the top/bottom; p fixed 0 at the outlet and top/bottom,
    normal gradient at the inlet and on the cylinder.  Starts from the
    uniform inflow u = (u_in, 0)."""
    from . import meshes
    nodes, cptr, cind = meshes.cylinder_channel(**(mesh_args or {}))
    mesh = pg.Mesh(nodes, cptr, cind)
    f = mesh.faces()
    patch = meshes.cylinder_patch_of_faces(f["fx"], f["fy"], f["rcell"])
    nf, n = mesh.n_faces, mesh.n_cells
    bc_u = np.ones(nf, np.int32)                       # NORMAL_GRADIENT
    bc_u[(patch == 0) | (patch == 3)] = 0              # FIXED
    u_face = np.zeros((nf, 2))
    u_face[patch == 0, 0] = u_in
    u_face[patch < 0, 0] = u_in
    bc_p = np.ones(nf, np.int32)
    bc_p[(patch == 1) | (patch == 2)] = 0
    u0 = np.zeros((n, 2))
    u0[:, 0] = u_in
    out = predictor_pcorr(pg, mesh, bc_u, u_face, u0, bc_p, np.zeros(nf),
                          rho, u_in * 1.0 / re * rho, dt, tol)
    out.update(patch=patch, nodes=nodes, cptr=cptr, cind=cind)
    return out
