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


def simple_pcorr(pg, nx=80, ny=80, rho=1.0, mu=0.01, dt=0.005, lid=1.0,
                 tol=1e-12):
    """Run the predictor on the device and return the pCorr equation and
    the intermediate fields."""
    w = cavity_inputs(nx, ny, lid)
    mesh = pg.Mesh(w["nodes"], w["cptr"], w["cind"])
    faces, cells = mesh.faces(), mesh.cells()
    w = cavity_inputs(nx, ny, lid, faces)
    n, nf = mesh.n_cells, mesh.n_faces
    u0 = np.zeros((n, 2))
    mom = pg.MomentumEquation(mesh, w["bc_u"]).assemble(
        dt, mu / rho, 1.0, u0, w["u_face"])
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
    uf[bnd] = w["u_face"][bnd]
    eqn = pg.fv.laplacian(gamma_f, mesh, w["bc_p"], None, rho * uf)
    return dict(mesh=mesh, eqn=eqn, u=u, d=dcoef, gamma_f=gamma_f, u_face=uf,
                momentum=(rp, ci, v, rhs), inputs=w)
