"""contains_properly (polygons against points) in its three modes and the
polygon-contains-point predicate, against the reference's known answers
(python/cuspatial/cuspatial/tests/binpreds/test_contains_properly.py) and the
oracle's composition of the join chain (core/binpreds/contains.py:19-74)."""

import math

import numpy as np
import pytest
import torch

import cuspatial_gb300 as cs
from cuspatial_gb300 import datasets as D
from oracle import oracle as O

from helpers import gpu_polygons, to_np

pytestmark = pytest.mark.gpu


def _polys(shapes, dtype=np.float64):
    """shapes: list of multipolygons; each a list of polygons; each a list of
    rings; each a list of (x, y)."""
    xs, ys, ro, po, go = [], [], [0], [0], [0]
    for mp in shapes:
        for poly in mp:
            for ring in poly:
                xs += [p[0] for p in ring]
                ys += [p[1] for p in ring]
                ro.append(len(xs))
            po.append(len(ro) - 1)
        go.append(len(po) - 1)
    xy = np.empty(2 * len(xs), dtype)
    xy[0::2] = xs
    xy[1::2] = ys
    return cs.GeoSeries.from_polygons_xy(xy, np.array(ro, np.int32), np.array(po, np.int32),
                                         np.array(go, np.int32))


def _points(pts, dtype=np.float64):
    return cs.GeoSeries.from_points(np.array([p[0] for p in pts], dtype),
                                    np.array([p[1] for p in pts], dtype))


TRI_CW = [[(0, 0), (0, 1), (1, 1), (0, 0)]]
SQUARE_CW = [[(-0.5, -0.5), (-0.5, 0.5), (0.5, 0.5), (0.5, -0.5), (-0.5, -0.5)]]
TRI_CCW = [[(0, 0), (1, 0), (1, 1), (0, 0)]]

# test_contains_properly.py:85-194 (one point, one polygon)
SINGLE = [
    ((0.6, 0.06), [[(0, 0), (10, 1), (1, 1), (0, 0)]], False),
    ((3.333, 1.111), [[(6, 2), (3, 1), (3, 4), (6, 2)]], False),
    ((3.33, 1.11), [[(6, 2), (3, 1), (3, 4), (6, 2)]], False),
    ((0.66, 0.006), [[(0, 0), (10, 1), (1, 1), (0, 0)]], False),
    ((0.666, 0.0006), [[(0, 0), (10, 1), (1, 1), (0, 0)]], False),
    ((-0.5, -0.5), SQUARE_CW, False), ((-0.5, 0.5), SQUARE_CW, False),
    ((0.5, 0.5), SQUARE_CW, False), ((0.5, -0.5), SQUARE_CW, False),
    ((-0.5, 0.0), SQUARE_CW, False), ((0.0, 0.5), SQUARE_CW, False),
    ((0.5, 0.0), SQUARE_CW, False), ((0.0, -0.5), SQUARE_CW, False),
    ((0, 0), TRI_CW, False), ((0.0, 1.0), TRI_CW, False), ((1.0, 1.0), TRI_CW, False),
    ((0.0, 0.5), TRI_CW, False), ((0.5, 0.5), TRI_CW, False), ((0.5, 1), TRI_CW, False),
    ((0.25, 0.5), TRI_CW, True), ((0.75, 0.9), TRI_CW, True),
    ((0.0, 0.0), TRI_CCW, False), ((1.0, 0.0), TRI_CCW, False), ((1.0, 1.0), TRI_CCW, False),
    ((0.5, 0.0), TRI_CCW, False), ((0.5, 0.5), TRI_CCW, False),
    ((0.5, 0.25), TRI_CCW, True), ((0.9, 0.75), TRI_CCW, True),
]


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_single_point_single_polygon(dtype):
    for pt, poly, want in SINGLE:
        got = cs.polygons_contains_properly(_polys([[poly]], dtype), _points([pt], dtype))
        assert to_np(got).tolist() == [want], (pt, poly)


def test_reference_examples():
    tri = [[(0, 0), (1, 0), (1, 1), (0, 0)]]
    big = [[(-2, -2), (-2, 2), (2, 2), (-2, -2)]]
    up = [[(0, 0), (0, 1), (1, 1), (0, 0)]]
    # test_two_points_one_polygon, test_one_point_two_polygons (:196-218)
    got = cs.polygons_contains_properly(_polys([[tri]]), _points([(0, 0), (0, 0)]))
    assert to_np(got).tolist() == [False, False]
    got = cs.polygons_contains_properly(_polys([[tri], [big]]), _points([(0, 0)]))
    assert to_np(got).tolist() == [False]
    # test_ten_fixed_points (:221-254)
    pts = [(0, 0), (0, 0)] + [(0.5, 0.25)] * 6 + [(0, 0), (0, 0)]
    got = cs.polygons_contains_properly(_polys([[tri]] * 5 + [[up]] * 5), _points(pts))
    assert to_np(got).tolist() == [False, False, True, True, True] + [False] * 5
    # test_example_1, test_example_2 (:550-577)
    got = cs.polygons_contains_properly(_polys([[tri]]), _points([(0.5, 0.5)]))
    assert to_np(got).tolist() == [False]
    got = cs.polygons_contains_properly(
        _polys([[tri]] * 3 + [[big]] * 3),
        _points([(0, 0), (-1, 0), (-2, 0), (0, 0), (-1, 0), (-2, 0)]))
    assert to_np(got).tolist() == [False, False, False, False, True, False]


HOLE_SAME = [[(0, 0), (1, 1), (1, 0), (0, 0)], [(0, 0), (1, 1), (1, 0), (0, 0)]]
HOLE_UP = [[(0, 0), (1, 1), (1, 0), (0, 0)], [(0, 0), (1, 1), (0, 1), (0, 0)]]
TRI = [[(0, 0), (1, 1), (1, 0), (0, 0)]]


def test_multipolygons():
    # test_multi_contains (:392-434): 4 geometries, 9 points
    lhs = _polys([[TRI], [HOLE_SAME], [TRI, TRI], [TRI, HOLE_SAME]])
    rhs = _points([(0.5, 0.25)] * 8 + [(1.0, 1.0)])
    got = cs.polygons_contains_properly(lhs, rhs)
    assert to_np(got).tolist() == [True, False, True, True, False, False, False, False, False]
    # test_allpairs_with_holes (:437-474)
    lhs = _polys([[TRI, HOLE_SAME], [TRI, TRI], [HOLE_SAME], [TRI]])
    t = cs.polygons_contains_properly(lhs, _points([(0.5, 0.25)]), allpairs=True)
    assert to_np(t["polygon_index"]).tolist() == [0, 1, 3]
    # test_allpairs (:477-510)
    lhs = _polys([[TRI, HOLE_UP], [TRI, TRI], [HOLE_UP], [TRI]])
    t = cs.polygons_contains_properly(lhs, _points([(0.5, 0.25)]), allpairs=True)
    assert to_np(t["polygon_index"]).tolist() == [0, 1, 2, 3]
    assert to_np(t["point_index"]).tolist() == [0, 0, 0, 0]


def _oracle_quadtree_rows(x, y, P):
    """contains.py:44-70 on the oracle."""
    px, py = P.x.astype(x.dtype), P.y.astype(x.dtype)
    x_min, x_max, y_min, y_max = px.min(), px.max(), py.min(), py.max()
    scale = max(x_max - x_min, y_max - y_min) / ((1 << 15) + 2)
    min_size = math.ceil(math.sqrt(len(x)))
    pi, tree = O.quadtree_on_points(x, y, float(x_min), float(x_max), float(y_min),
                                    float(y_max), float(scale), 15, min_size)
    bb = O.polygon_bounding_boxes(P.part_offset, P.ring_offset, px, py)
    pairs = O.join_quadtree_and_bounding_boxes(tree, bb, float(x_min), float(x_max),
                                               float(y_min), float(y_max), float(scale), 15)
    r = O.quadtree_point_in_polygon(pairs, tree, pi, x, y, P.part_offset, P.ring_offset, px, py)
    return pi[r["point_index"]], r["polygon_index"]


def _multi(rng, n_geoms, extent=1000.0):
    """Multipolygons of 1-3 star parts (some with holes)."""
    parts = rng.integers(1, 4, n_geoms)
    centers = rng.uniform(0, extent, (int(parts.sum()), 2))
    k = rng.integers(3, 80, len(centers))
    P = D.star_polygons(rng, centers, k, lambda g, pid: g.uniform(5, 60, len(pid)),
                        hole_fraction=0.2)
    P.geometry_offset = np.concatenate([[0], np.cumsum(parts)]).astype(np.int32)
    return P


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("method", ["exact", "filtered"])
def test_quadtree_mode_against_oracle(dtype, method):
    rng = np.random.default_rng(21)
    P = _multi(rng, 300)
    x = rng.uniform(-50, 1050, 40000).astype(dtype)
    y = rng.uniform(-50, 1050, 40000).astype(dtype)
    bx, by = D._near_boundary(rng, P, 4000)
    x[:4000] = bx
    y[:4000] = by
    pts = cs.GeoSeries.from_points(x, y)
    polys = gpu_polygons(P, dtype)
    t = cs.contains_properly(polys, pts, mode="quadtree", method=method)
    wp, wa = _oracle_quadtree_rows(x, y, P)
    assert len(wa) > 1000
    np.testing.assert_array_equal(to_np(t["point_index"]), wp)
    np.testing.assert_array_equal(to_np(t["part_index"]), wa)
    # allpairs: each multipolygon once per contained point
    go = P.geometry_offset
    geom = np.searchsorted(go[1:], wa, side="right")
    key = np.unique(geom.astype(np.int64) * (1 << 32) + wp)
    a = cs.polygons_contains_properly(polys, pts, allpairs=True, method=method)
    np.testing.assert_array_equal(to_np(a["polygon_index"]), key >> 32)
    np.testing.assert_array_equal(to_np(a["point_index"]), key & 0xFFFFFFFF)


def test_modes_agree():
    rng = np.random.default_rng(22)
    centers = rng.uniform(0, 100, (31, 2))
    P = D.star_polygons(rng, centers, rng.integers(3, 40, 31),
                        lambda g, pid: g.uniform(5, 30, len(pid)), hole_fraction=0.3)
    x = rng.uniform(-10, 110, 31)
    y = rng.uniform(-10, 110, 31)
    x[:10] = centers[:10, 0]
    y[:10] = centers[:10, 1]
    pts = cs.GeoSeries.from_points(x, y)
    polys = gpu_polygons(P)
    q = cs.contains_properly(polys, pts, mode="quadtree")
    b = cs.contains_properly(polys, pts, mode="brute_force")
    pw = cs.contains_properly(polys, pts, mode="pairwise")
    qs = set(zip(to_np(q["point_index"]).tolist(), to_np(q["part_index"]).tolist()))
    bs = set(zip(to_np(b["point_index"]).tolist(), to_np(b["part_index"]).tolist()))
    assert qs == bs and len(qs) > 10
    # brute force rows are point-major
    bp = to_np(b["point_index"]) * 64 + to_np(b["part_index"])
    assert np.all(np.diff(bp) > 0)
    want = O.point_in_polygon(x, y, P.part_offset, P.ring_offset, P.x, P.y, pairwise=True)
    assert to_np(pw["pairwise_index"]).tolist() == np.nonzero(want)[0].tolist()
    assert bool(to_np(pw["result"]).all())


def test_empty_and_errors():
    pts = _points([(0.5, 0.25)])
    empty = cs.GeoSeries.from_polygons_xy(np.zeros(0), np.zeros(1, np.int32),
                                          np.zeros(1, np.int32), np.zeros(1, np.int32))
    assert cs.contains_properly(empty, pts, mode="quadtree").columns == []
    with pytest.raises(TypeError):
        cs.polygons_contains_properly(pts, pts)
    # more than 31 parts under 32 geometries: the bitmask's limit
    lhs = _polys([[TRI] * 16, [TRI] * 16])
    with pytest.raises(RuntimeError, match="Number of polygons cannot exceed 31"):
        cs.polygons_contains_properly(lhs, pts)
    # no points: no rows
    none = cs.GeoSeries.from_points(np.zeros(0), np.zeros(0))
    t = cs.contains_properly(_polys([[TRI]] * 40), none, mode="quadtree")
    assert t["point_index"].numel() == 0
    assert torch.is_tensor(cs.polygons_contains_properly(_polys([[TRI]] * 40), none))
