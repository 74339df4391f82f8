"""Mesh generators (CPU): the graded cylinder-channel triangulation is a
valid, counter-clockwise, hole-respecting mesh whose boundary lies on the
channel sides and the cylinder, and it is reproducible from its seed."""
import numpy as np

from phase_gb300 import meshes


def _edges(cind):
    t = cind.reshape(-1, 3)
    e = np.concatenate([t[:, [0, 1]], t[:, [1, 2]], t[:, [2, 0]]])
    e.sort(axis=1)
    u, cnt = np.unique(e, axis=0, return_counts=True)
    return u, cnt


def test_cylinder_channel_is_a_valid_mesh():
    nodes, cptr, cind = meshes.cylinder_channel(h_near=0.05, h_far=0.5,
                                                grading=4.0, seed=2)
    t = cind.reshape(-1, 3)
    assert np.all(np.diff(cptr) == 3)
    a, b, c = nodes[t[:, 0]], nodes[t[:, 1]], nodes[t[:, 2]]
    area2 = (b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - \
        (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0])
    assert np.all(area2 > 0)
    # area = channel minus the polygonal cylinder
    nc = int(np.ceil(2 * np.pi * 0.5 / 0.05))
    poly = 0.5 * nc * 0.25 * np.sin(2 * np.pi / nc)
    assert np.isclose(area2.sum() / 2, 300.0 - poly, rtol=1e-12)
    g = (a + b + c) / 3
    assert np.all(np.hypot(g[:, 0] - 5, g[:, 1] - 5) > 0.5)
    # Euler characteristic of a disk with one hole: V - E + F = 0
    e, cnt = _edges(cind)
    assert len(nodes) - len(e) + len(t) == 0
    assert set(np.unique(cnt)) <= {1, 2}
    # boundary edges lie on the channel sides or on the cylinder
    m = 0.5 * (nodes[e[cnt == 1, 0]] + nodes[e[cnt == 1, 1]])
    on_side = (np.isclose(m[:, 0], 0) | np.isclose(m[:, 0], 30) |
               np.isclose(m[:, 1], 0) | np.isclose(m[:, 1], 10))
    on_cyl = np.abs(np.hypot(m[:, 0] - 5, m[:, 1] - 5) - 0.5) < 0.01
    assert np.all(on_side | on_cyl)
    # finer near the cylinder than far away
    h = np.sqrt(area2)
    d = np.hypot(g[:, 0] - 5, g[:, 1] - 5)
    assert np.median(h[d < 1]) < 0.3 * np.median(h[d > 6])


def test_cylinder_channel_is_reproducible():
    m1 = meshes.cylinder_channel(h_near=0.05, h_far=0.5, grading=4.0, seed=2)
    m2 = meshes.cylinder_channel(h_near=0.05, h_far=0.5, grading=4.0, seed=2)
    m3 = meshes.cylinder_channel(h_near=0.05, h_far=0.5, grading=4.0, seed=3)
    assert all(np.array_equal(a, b) for a, b in zip(m1, m2))
    assert not np.array_equal(m1[0], m3[0])
