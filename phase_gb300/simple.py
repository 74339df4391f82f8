"""One SIMPLE step of the lid-driven cavity on the device, producing the
pressure-correction system fv::laplacian(rho*d, pCorr) == src::div(rho*u*).

Phase has no SIMPLE solver (its solvers are fractional-step), so this
driver is project code written over the library's own operators:

1. momentum predictor  ddt(u) + div(u_f, u) - laplacian(mu/rho, u) = 0
   (pg_assemble_momentum), solved per component with the GPU BiCGStab;
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
    pressure boundary types bc_p and values p_value (per face)."""
    faces, cells = mesh.faces(), mesh.cells()
    n = mesh.n_cells
    mom = pg.MomentumEquation(mesh, bc_u).assemble(dt, mu / rho, 1.0, u0,
                                                   u_face)
    rp, ci, v, rhs = mom.export()
    s = pg.SparseMatrixSolver(tolerance=tol, max_iters=5000)
    s.setRank(n)
    s.set(rp, ci, v)
    u = np.empty((n, 2))
    for d in range(2):
        s.setRhs(-rhs[d * n:(d + 1) * n])
        s.setGuess(None)
        s.solve()
        u[:, d] = s.x()
    rows = np.repeat(np.arange(n), np.diff(rp))
    a_p = v[(ci == rows)]
    dcoef = cells["vol"] / a_p
    gamma_f = rho * mesh.interpolate_faces(dcoef)
    uf = np.stack([mesh.interpolate_faces(u[:, 0]),
                   mesh.interpolate_faces(u[:, 1])], 1)
    bnd = faces["rcell"] < 0
    uf[bnd] = u_face[bnd]
    eqn = pg.fv.laplacian(gamma_f, mesh, bc_p, p_value, rho * uf)
    return dict(mesh=mesh, eqn=eqn, u=u, d=dcoef, gamma_f=gamma_f, u_face=uf,
                momentum=(rp, ci, v, rhs))


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
