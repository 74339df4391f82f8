"""Replay of the fv::laplacian call sequence (Laplacian.h:49-83, :132-167)
as CrsEquation operations, so the reference's own CrsEquation can be driven
with exactly the calls the reference makes.  Test infrastructure."""
from __future__ import annotations

import numpy as np


def link_geometry(om):
    """Per-link (cell, face, nb, coeff numerator dot(r,Sf), |r|^2, Sf)."""
    c = om.cells()
    f = om.faces()
    lp, lf, lc = om.links()
    cell_of_link = np.repeat(np.arange(om.n_cells), np.diff(lp))
    px, py = c["cx"][cell_of_link], c["cy"][cell_of_link]
    fx, fy = f["fx"][lf], f["fy"][lf]
    nx, ny = f["nx"][lf], f["ny"][lf]
    s = np.where((fx - px) * nx + (fy - py) * ny > 0.0, 1.0, -1.0)
    sfx, sfy = s * nx, s * ny
    inter = lc >= 0
    rx = np.where(inter, c["cx"][np.maximum(lc, 0)] - px, fx - px)
    ry = np.where(inter, c["cy"][np.maximum(lc, 0)] - py, fy - py)
    dot = rx * sfx + ry * sfy
    msq = rx * rx + ry * ry
    return dict(cell=cell_of_link, face=lf, nb=lc, dot=dot, msq=msq,
                sfx=sfx, sfy=sfy, lp=lp)


def laplacian_ops(om, gamma, bc_type, bc_value):
    """CrsEquation operations of fv::laplacian(gamma, phi) in call order.

    op 0 = addCoeff(row, col, val), op 1 = addRhs(row, val)."""
    g = link_geometry(om)
    face_gamma = not np.isscalar(gamma)
    ops, rows, cols, vals = [], [], [], []
    for i in range(g["cell"].size):
        c, f, nb = int(g["cell"][i]), int(g["face"][i]), int(g["nb"][i])
        gm = float(gamma[f]) if face_gamma else float(gamma)
        coeff = gm * float(g["dot"][i]) / float(g["msq"][i])
        if nb >= 0:
            if face_gamma:
                seq = [(0, c, c, -coeff), (0, c, nb, coeff)]
            else:
                seq = [(0, c, nb, coeff), (0, c, c, -coeff)]
        elif bc_type[f] == 0:  # FIXED
            seq = [(0, c, c, -coeff), (1, c, -1, coeff * float(bc_value[f]))]
        else:
            seq = []
        for o in seq:
            ops.append(o[0]); rows.append(o[1]); cols.append(o[2]); vals.append(o[3])
    return (np.array(ops, np.int32), np.array(rows, np.int32),
            np.array(cols, np.int32), np.array(vals, np.float64))


def div_u(om, u_face):
    """src::div(u) (Source.cpp:5-21) in link order."""
    g = link_geometry(om)
    u = np.asarray(u_face, np.float64).reshape(-1, 2)
    out = np.zeros(om.n_cells)
    for i in range(g["cell"].size):
        f = int(g["face"][i])
        out[int(g["cell"][i])] += u[f, 0] * g["sfx"][i] + u[f, 1] * g["sfy"][i]
    return out
