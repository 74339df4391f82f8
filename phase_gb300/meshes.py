"""Mesh and workload generators (host side, numpy).

Rectilinear meshes follow StructuredRectilinearGrid::init
(src/2D/Unstructured/FiniteVolumeGrid2D/StructuredRectilinearGrid.cpp:40-95):
node (i, j) has id j*nNodesX + i and coordinates (i*hx, j*hy) with
hx = width/nCellsX; cell (i, j) has id j*nCellsX + i and nodes
(i,j), (i+1,j), (i+1,j+1), (i,j+1) (counter-clockwise).  The patches
x-, x+, y-, y+ (:175-194) are identified here from boundary face centroids.
"""
from __future__ import annotations

import numpy as np


def rectilinear(nx: int, ny: int, width: float = 1.0, height: float = 1.0,
                origin=(0.0, 0.0)):
    """Return (nodes_xy[n_nodes,2] f64, cptr[n_cells+1] i64, cind[4*n_cells] i64)."""
    hx0 = width / nx
    hy0 = height / ny
    xs = np.arange(nx + 1, dtype=np.float64) * hx0
    ys = np.arange(ny + 1, dtype=np.float64) * hy0
    X, Y = np.meshgrid(xs, ys)  # row-major in j then i
    nodes = np.empty(((nx + 1) * (ny + 1), 2), dtype=np.float64)
    nodes[:, 0] = X.ravel() + origin[0]
    nodes[:, 1] = Y.ravel() + origin[1]
    nnx = nx + 1
    j, i = np.meshgrid(np.arange(ny, dtype=np.int64), np.arange(nx, dtype=np.int64),
                       indexing="ij")
    base = (j * nnx + i).ravel()
    cind = np.stack([base, base + 1, base + nnx + 1, base + nnx], axis=1).ravel()
    cptr = np.arange(0, 4 * nx * ny + 1, 4, dtype=np.int64)
    return nodes, cptr, cind


def rect_patch_of_faces(fx, fy, rcell, width, height, origin=(0.0, 0.0)):
    """Patch id per face for a rectilinear box: -1 interior, 0 x-, 1 x+, 2 y-, 3 y+."""
    tol = 1e-12 * max(width, height)
    patch = np.full(fx.shape, -1, dtype=np.int32)
    b = rcell < 0
    x0, y0 = origin
    patch[b & (np.abs(fx - x0) <= tol)] = 0
    patch[b & (np.abs(fx - (x0 + width)) <= tol)] = 1
    patch[b & (np.abs(fy - y0) <= tol)] = 2
    patch[b & (np.abs(fy - (y0 + height)) <= tol)] = 3
    return patch


def triangulated(nx: int, ny: int, width: float = 1.0, height: float = 1.0,
                 jitter: float = 0.0, seed: int = 0):
    """Unstructured triangle mesh: each quad of an nx-by-ny grid split along a
    diagonal whose direction alternates, interior nodes jittered by
    ``jitter`` * cell size (seeded).  Cells are counter-clockwise."""
    nodes, _, _ = rectilinear(nx, ny, width, height)
    nodes = nodes.copy()
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        hx, hy = width / nx, height / ny
        ii = np.arange(nodes.shape[0]) % (nx + 1)
        jj = np.arange(nodes.shape[0]) // (nx + 1)
        interior = (ii > 0) & (ii < nx) & (jj > 0) & (jj < ny)
        d = rng.uniform(-jitter, jitter, size=(nodes.shape[0], 2))
        nodes[interior, 0] += d[interior, 0] * hx
        nodes[interior, 1] += d[interior, 1] * hy
    nnx = nx + 1
    tris = []
    for j in range(ny):
        for i in range(nx):
            a = j * nnx + i
            b, c, d = a + 1, a + nnx + 1, a + nnx
            if (i + j) % 2 == 0:
                tris += [(a, b, c), (a, c, d)]
            else:
                tris += [(a, b, d), (b, c, d)]
    cind = np.array(tris, dtype=np.int64).ravel()
    cptr = np.arange(0, cind.size + 1, 3, dtype=np.int64)
    return nodes, cptr, cind
