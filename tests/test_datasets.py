"""The synthetic workloads (cuspatial_gb300/datasets.py) that stand in for the
benchmark configurations: seeded and repeatable, with the documented shapes
(closed rings, vertex counts, holes reversed, points inside the box, half
of the boundary points on polygon vertices)."""

import numpy as np

from cuspatial_gb300 import datasets as D


def _area2(x, y):
    return float(np.sum(x[:-1] * y[1:] - x[1:] * y[:-1]))


def test_precision_at_scale_shapes_and_seed():
    a = D.precision_at_scale(n_points=20000, n_polygons=300)
    b = D.precision_at_scale(n_points=20000, n_polygons=300)
    np.testing.assert_array_equal(a.x, b.x)
    np.testing.assert_array_equal(a.polygons.x, b.polygons.x)
    assert a.max_depth == 15 and a.max_size == 256 and a.scale == 10000.0 / 32768
    assert np.all((a.x >= 0) & (a.x < 10000) & (a.y >= 0) & (a.y < 10000))
    p = a.polygons
    assert p.num_polygons == 300
    holes = 0
    for pid in range(p.num_polygons):
        r0, r1 = int(p.part_offset[pid]), int(p.part_offset[pid + 1])
        rings = [(int(p.ring_offset[r]), int(p.ring_offset[r + 1])) for r in range(r0, r1)]
        outer = rings[0]
        nv = outer[1] - outer[0] - 1  # closed: the first vertex repeats
        assert 8 <= nv <= 512
        ox, oy = p.x[outer[0]:outer[1]], p.y[outer[0]:outer[1]]
        assert ox[0] == ox[-1] and oy[0] == oy[-1]
        for h in rings[1:]:
            hx, hy = p.x[h[0]:h[1]], p.y[h[0]:h[1]]
            assert hx[0] == hx[-1] and hy[0] == hy[-1]
            assert np.sign(_area2(hx, hy)) == -np.sign(_area2(ox, oy))  # reversed
            holes += 1
    assert 0 < holes < p.num_polygons * 0.25
    assert a.extra["boundary_points"] == 200
    # about half of the boundary points sit exactly on a polygon vertex
    on = 0
    verts = set(zip(p.x.tolist(), p.y.tolist()))
    for x, y in zip(a.x.tolist(), a.y.tolist()):
        if (x, y) in verts:
            on += 1
    assert on >= 50


def test_other_workloads_are_repeatable():
    for make in (lambda: D.plain_small(n_points=5000, n_polygons=16),
                 lambda: D.nearest_linestring(n_points=5000, n_linestrings=50),
                 lambda: D.unindexed_pip(n_points=5000),
                 lambda: D.pairwise_pip(n=500)):
        a, b = make(), make()
        for k in ("x", "y"):
            if hasattr(a, k):
                np.testing.assert_array_equal(getattr(a, k), getattr(b, k))
