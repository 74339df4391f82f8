"""The direct solver's nested-dissection ordering and front structure
(host analysis, no GPU): a numpy multifrontal factorisation over the
exported fronts must reproduce a dense solve, which holds only when every
front's index list covers the fill of its subtree, children's update sets
lie in their parent's front, and the ordering is a permutation."""
import numpy as np
import pytest
import scipy.sparse as sp

from phase_gb300 import meshes


@pytest.fixture(scope="module")
def pglib():
    import __graft_entry__
    __graft_entry__.build()
    import phase_gb300
    phase_gb300.lib()
    return phase_gb300


def _multifrontal_solve(A, b, perm, fronts, lists):
    """Dense-front emulation of the device algorithm: fronts in elimination
    order, children's contribution blocks extend-added, partial pivoting
    over each front's fully summed rows."""
    n = A.shape[0]
    iperm = np.empty(n, np.int64)
    iperm[perm] = np.arange(n)
    P = A.tocoo()
    rows, cols = iperm[P.row], iperm[P.col]
    owner = np.empty(n, np.int64)
    for t, (s0, k, m, parent) in enumerate(fronts):
        owner[s0:s0 + k] = t
    ent_owner = owner[np.minimum(rows, cols)]
    cb = {}
    fac = []
    for t, (s0, k, m, parent) in enumerate(fronts):
        idx = lists[t]
        assert idx.size == m and np.array_equal(idx[:k], np.arange(s0, s0 + k))
        assert np.all(np.diff(idx[k:]) > 0) and (m == k or idx[k] >= s0 + k)
        pos = {int(v): i for i, v in enumerate(idx)}
        F = np.zeros((m, m))
        for c, U in cb.pop(t, []):
            loc = np.array([pos[int(v)] for v in U[0]])  # KeyError = bad U
            F[np.ix_(loc, loc)] += U[1]
        sel = ent_owner == t
        for r, c, v in zip(rows[sel], cols[sel], P.data[sel]):
            F[pos[int(r)], pos[int(c)]] += v  # KeyError = entry not covered
        piv = np.arange(k)
        for c in range(k):
            r = c + int(np.argmax(np.abs(F[c:k, c])))
            piv[c] = r
            F[[c, r], c:] = F[[r, c], c:]
            F[c + 1:, c] /= F[c, c]
            F[c + 1:, c + 1:] -= np.outer(F[c + 1:, c], F[c, c + 1:])
        fac.append((F, piv))
        if parent >= 0:
            cb.setdefault(int(parent), []).append((t, (idx[k:], F[k:, k:])))
        else:
            assert m == k
    bn = b[perm].copy()
    # forward (LINPACK order) and backward over the fronts
    contrib = {}
    y = np.zeros(n)
    for t, (s0, k, m, parent) in enumerate(fronts):
        idx = lists[t]
        F, piv = fac[t]
        w = np.zeros(m)
        w[:k] = bn[s0:s0 + k]
        pos = {int(v): i for i, v in enumerate(idx)}
        for U, cv in contrib.pop(t, []):
            w[[pos[int(v)] for v in U]] += cv
        for c in range(k):
            w[[c, piv[c]]] = w[[piv[c], c]]
            w[c + 1:] -= F[c + 1:, c] * w[c]
        y[s0:s0 + k] = w[:k]
        if parent >= 0:
            contrib.setdefault(int(parent), []).append((idx[k:], w[k:]))
    xn = np.zeros(n)
    for t in range(len(fronts) - 1, -1, -1):
        s0, k, m, parent = fronts[t]
        idx = lists[t]
        F, _ = fac[t]
        r = y[s0:s0 + k] - F[:k, k:] @ xn[idx[k:]]
        for c in range(k - 1, -1, -1):
            r[c] /= F[c, c]
            r[:c] -= F[:c, c] * r[c]
        xn[s0:s0 + k] = r
    x = np.empty(n)
    x[perm] = xn
    return x


@pytest.mark.parametrize("coords", [True, False])
def test_front_structure_solves_a_triangle_mesh_system(pglib, coords):
    nodes, cptr, cind = meshes.triangulated(26, 18, 2.0, 1.5, jitter=0.2,
                                            seed=4)
    n = len(cptr) - 1
    # a nonsymmetric matrix on the cells' adjacency (shared nodes)
    rng = np.random.default_rng(2)
    cells_of_node = {}
    for c in range(n):
        for v in cind[cptr[c]:cptr[c + 1]]:
            cells_of_node.setdefault(int(v), []).append(c)
    rows, cols = [], []
    for cs in cells_of_node.values():
        for a in cs:
            for b in cs:
                rows.append(a)
                cols.append(b)
    A = sp.csr_matrix((rng.standard_normal(len(rows)), (rows, cols)),
                      shape=(n, n))
    A.sum_duplicates()
    A = A + sp.diags(np.full(n, 4.0))
    A = A.tocsr()
    A.sort_indices()
    xy = None
    if coords:
        pts = nodes.reshape(-1, 2)
        xy = np.array([pts[cind[cptr[c]:cptr[c + 1]]].mean(axis=0)
                       for c in range(n)])
    perm, fronts, lists, heights = pglib.lu_analyse_pattern(A.indptr,
                                                            A.indices, xy)
    assert np.array_equal(np.sort(perm), np.arange(n))
    assert len(fronts) > 4 and heights > 2
    b = rng.standard_normal(n)
    x = _multifrontal_solve(A, b, perm, fronts, lists)
    xd = np.linalg.solve(A.toarray(), b)
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 1e-10


def test_front_structure_of_a_grid_has_line_separators(pglib):
    """Coordinate bisection of a 64 x 64 grid: the root separator is one
    grid line and the tree is about log2(4096 / 64) levels deep."""
    nodes, cptr, cind = meshes.rectilinear(64, 64)
    n = 64 * 64
    ii, jj = np.divmod(np.arange(n), 64)
    rows, cols = [np.arange(n)], [np.arange(n)]
    for di, dj in ((0, 1), (1, 0), (0, -1), (-1, 0)):
        ok = (ii + di >= 0) & (ii + di < 64) & (jj + dj >= 0) & (jj + dj < 64)
        rows.append(np.arange(n)[ok])
        cols.append(((ii + di) * 64 + jj + dj)[ok])
    r, c = np.concatenate(rows), np.concatenate(cols)
    A = sp.csr_matrix((np.where(r == c, 4.0, -1.0), (r, c)), shape=(n, n))
    A.sort_indices()
    xy = np.stack([jj + 0.5, ii + 0.5], axis=1).astype(np.float64)
    perm, fronts, lists, heights = pglib.lu_analyse_pattern(A.indptr,
                                                            A.indices, xy)
    root = fronts[-1]
    assert root[3] == -1 and root[1] == 64 and root[2] == 64
    assert 6 <= heights <= 9
    b = np.random.default_rng(0).standard_normal(n)
    x = _multifrontal_solve(A, b, perm, fronts, lists)
    assert np.linalg.norm(A @ x - b) / np.linalg.norm(b) < 1e-12
