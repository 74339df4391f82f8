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


def _cyl_size(d, h_near, h_far, grading):
    """Target edge length at distance d from the cylinder surface."""
    return np.minimum(h_far, h_near + (h_far - h_near) * np.maximum(d, 0.0) / grading)


def cylinder_channel(h_near: float = 0.01, h_far: float = 0.1,
                     grading: float = 9.0, length: float = 30.0,
                     height: float = 10.0, centre=(5.0, 5.0),
                     radius: float = 0.5, seed: int = 2):
    """Seeded graded triangle mesh of the channel [0, length] x [0, height]
    minus the disk of ``radius`` at ``centre`` (the geometry of
    Examples/UnstructuredFlowAroundCylinder, whose CGNS mesh cannot be read
    here).

    Points: the centres of the leaves of a quadtree refined until every
    leaf is no larger than the size function, which grows linearly from
    ``h_near`` at the cylinder to ``h_far`` over ``grading`` length units,
    each moved by a seeded jitter of 15 % of its leaf; plus points along the
    cylinder and the four channel sides at the local size.  The Delaunay
    triangulation of those points (scipy's Qhull, mesh generation only, not
    on the solve path) is cut at the cylinder, oriented counter-clockwise,
    and its cells are numbered along a Z-order curve of their centroids, as
    a mesher that writes cache-friendly files would.  Returns (nodes, cptr,
    cind) like the other generators."""
    from scipy.spatial import Delaunay

    cx, cy = centre
    rng = np.random.default_rng(seed)

    def size_at(x, y):
        d = np.hypot(x - cx, y - cy) - radius
        return _cyl_size(d, h_near, h_far, grading)

    # quadtree: unit cells refined until size <= h at the cell's nearest point
    nx0, ny0 = int(round(length)), int(round(height))
    gx, gy = np.meshgrid(np.arange(nx0, dtype=np.float64),
                         np.arange(ny0, dtype=np.float64))
    x0, y0 = gx.ravel(), gy.ravel()
    s = np.ones_like(x0)
    leaves = []
    while x0.size:
        xc, yc = x0 + 0.5 * s, y0 + 0.5 * s
        d = np.hypot(xc - cx, yc - cy) - radius - 0.7072 * s
        split = s > _cyl_size(d, h_near, h_far, grading)
        keep = ~split
        leaves.append(np.stack([x0[keep], y0[keep], s[keep]], 1))
        x0, y0, s = x0[split], y0[split], s[split] * 0.5
        x0 = np.concatenate([x0, x0 + s, x0, x0 + s])
        y0 = np.concatenate([y0, y0, y0 + s, y0 + s])
        s = np.concatenate([s, s, s, s])
    lv = np.concatenate(leaves)
    px = lv[:, 0] + 0.5 * lv[:, 2] + rng.uniform(-0.15, 0.15, len(lv)) * lv[:, 2]
    py = lv[:, 1] + 0.5 * lv[:, 2] + rng.uniform(-0.15, 0.15, len(lv)) * lv[:, 2]
    # interior points keep half a local size away from the cylinder
    far = np.hypot(px - cx, py - cy) > radius + 0.5 * lv[:, 2]
    pts = [np.stack([px[far], py[far]], 1)]
    # cylinder surface
    nc = int(np.ceil(2.0 * np.pi * radius / h_near))
    th = 2.0 * np.pi * np.arange(nc) / nc
    pts.append(np.stack([cx + radius * np.cos(th), cy + radius * np.sin(th)], 1))
    # channel sides, marched at the local quadtree size
    def march(a, b, fixed, horizontal):
        out, t = [], a
        while t < b - 1e-12:
            out.append(t)
            x, y = (t, fixed) if horizontal else (fixed, t)
            h = float(size_at(np.array([x]), np.array([y]))[0])
            t += 2.0 ** np.floor(np.log2(h))
        out.append(b)
        t = np.array(out)
        return np.stack([t, np.full_like(t, fixed)], 1) if horizontal else \
            np.stack([np.full_like(t, fixed), t], 1)
    sides = [march(0.0, length, 0.0, True), march(0.0, length, height, True),
             march(0.0, height, 0.0, False), march(0.0, height, length, False)]
    pts += sides
    pts = np.concatenate(pts)
    pts = np.unique(np.round(pts, 12), axis=0)
    tri = Delaunay(pts)
    if len(getattr(tri, "coplanar", [])):
        raise RuntimeError("cylinder_channel: Qhull dropped input points")
    t = tri.simplices.astype(np.int64)
    a, b, c = pts[t[:, 0]], pts[t[:, 1]], pts[t[:, 2]]
    g = (a + b + c) / 3.0
    t = t[np.hypot(g[:, 0] - cx, g[:, 1] - cy) > radius]
    a, b, c = pts[t[:, 0]], pts[t[:, 1]], pts[t[:, 2]]
    area2 = (b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - \
        (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0])
    flip = area2 < 0
    t[flip, 1], t[flip, 2] = t[flip, 2].copy(), t[flip, 1].copy()
    # Z-order numbering of the cells
    g = (pts[t[:, 0]] + pts[t[:, 1]] + pts[t[:, 2]]) / 3.0
    q = np.floor(g / (h_near * 0.5)).astype(np.int64)
    code = np.zeros(len(t), np.int64)
    for bit in range(24):
        code |= ((q[:, 0] >> bit) & 1) << (2 * bit)
        code |= ((q[:, 1] >> bit) & 1) << (2 * bit + 1)
    t = t[np.argsort(code, kind="stable")]
    # keep only referenced nodes, numbered in first-use order
    used, inv = np.unique(t.ravel(), return_inverse=True)
    nodes = pts[used]
    cind = inv.astype(np.int64)
    cptr = np.arange(0, cind.size + 1, 3, dtype=np.int64)
    return nodes, cptr, cind


def cylinder_patch_of_faces(fx, fy, rcell, length=30.0, height=10.0,
                            centre=(5.0, 5.0), radius=0.5):
    """Patch id per face of cylinder_channel: -1 interior, 0 inlet (x = 0),
    1 outlet (x = length), 2 bottom/top walls, 3 cylinder."""
    tol = 1e-9 * max(length, height)
    patch = np.full(fx.shape, -1, dtype=np.int32)
    b = rcell < 0
    patch[b & (np.abs(fx) <= tol)] = 0
    patch[b & (np.abs(fx - length) <= tol)] = 1
    patch[b & ((np.abs(fy) <= tol) | (np.abs(fy - height) <= tol))] = 2
    patch[b & (np.hypot(fx - centre[0], fy - centre[1]) < radius + 1e-6)] = 3
    return patch
