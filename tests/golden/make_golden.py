"""Writes the golden fixtures of fv::laplacian(gamma, phi) == src::div(u):
small seeded meshes and inputs, and the output of the reference's own
CrsEquation (src/Math/CrsEquation.cpp, compiled from its sources into
oracle/_ref by oracle/Makefile) driven with the exact call sequence the
reference's Laplacian.h:49-83 / :132-167 and Source.cpp:5-25 make
(tests/refreplay.py).  The fixtures pin the oracle and the device assembly
wherever the reference sources are absent.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import oracle_bind as ob  # noqa: E402
import refreplay  # noqa: E402
from phase_gb300 import meshes  # noqa: E402


def hexagon_fan():
    """A hexagon surrounded by six triangles: the centre row has seven
    entries, so the reference's CrsEquation grows it past its five slots."""
    ang = np.linspace(0, 2 * np.pi, 7)[:-1]
    ring = np.stack([np.cos(ang), np.sin(ang)], 1)
    outer = 2.0 * np.stack([np.cos(ang + np.pi / 6), np.sin(ang + np.pi / 6)], 1)
    nodes = np.vstack([ring, outer])
    cells = [list(range(6))]
    for k in range(6):
        cells.append([k, 6 + k, (k + 1) % 6])
    cptr = np.cumsum([0] + [len(c) for c in cells]).astype(np.int64)
    cind = np.array(sum(cells, []), np.int64)
    return nodes, cptr, cind


def cases():
    rect = meshes.rectilinear(6, 5, 1.0, 2.0)
    tri = meshes.triangulated(5, 4, 1.0, 1.0, 0.2, 1)
    out = []
    for mesh_name, mesh in (("rect", rect), ("tri", tri)):
        for kind in ("scalar", "face"):
            out.append((f"laplacian_{mesh_name}_{kind}", mesh, kind, True))
    out.append(("laplacian_hexfan_scalar", hexagon_fan(), "scalar", False))
    return out


def make(name, mesh, kind, with_u, seed=7, out_dir=HERE):
    nodes, cptr, cind = mesh
    om = ob.OracleMesh(nodes, cptr, cind)
    rng = np.random.default_rng(seed)
    nf = om.n_faces
    f = om.faces()
    # boundary faces FIXED (0) or NORMAL_GRADIENT (1); interior faces 1
    bc = np.where(f["rcell"] < 0, rng.integers(0, 2, nf), 1).astype(np.int32)
    bv = rng.standard_normal(nf)
    if kind == "scalar":
        gamma = 1.7
    else:
        gamma = rng.uniform(0.0, 2.0, nf)
        gamma[::7] = 0.0  # explicit zero coefficients keep their slots
    u = rng.standard_normal((nf, 2)) if with_u else None
    r = ob.RefCrs(om.n_cells, 5)
    ops, rows, cols, vals = refreplay.laplacian_ops(om, gamma, bc, bv)
    r.apply(ops, rows, cols, vals)
    if u is not None:
        r.eq_vector(refreplay.div_u(om, u))
    rp, ci, v, rhs = r.export()
    np.savez(os.path.join(out_dir, name + ".npz"),
             nodes=nodes, cptr=cptr, cind=cind,
             gamma=np.asarray(gamma, np.float64),
             gamma_is_scalar=np.array(kind == "scalar"),
             bc_type=bc, bc_value=bv,
             u=u if u is not None else np.zeros((0, 2)),
             row_ptr=rp, col_ind=ci, vals=v, rhs=rhs)
    return rp.size - 1, int(rp[-1])


if __name__ == "__main__":
    if ob.ref_lib() is None:
        sys.exit("the reference's CrsEquation (oracle/_ref) is not built")
    for name, mesh, kind, with_u in cases():
        n, ns = make(name, mesh, kind, with_u)
        print(f"{name}: {n} rows, {ns} slots")
