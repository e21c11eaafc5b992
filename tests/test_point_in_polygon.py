"""Unindexed point_in_polygon (bitmask over at most 31 polygons) and
pairwise_point_in_polygon against the reference's known answers and the
oracle (cpp/tests/point_in_polygon/point_in_polygon_test.cu,
pairwise_point_in_polygon_test.cu and
python/cuspatial/cuspatial/tests/spatial/join/test_point_in_polygon.py)."""

import numpy as np
import pytest
import torch

import cuspatial_gb300 as cs
from cuspatial_gb300 import datasets as D
from oracle import oracle as O

from helpers import gpu_polygons, to_np

pytestmark = pytest.mark.gpu

DTYPES = [np.float64, np.float32]
METHODS = ["exact", "filtered"]


def _series(x, y, po, ro, px, py, dtype):
    pts = cs.GeoSeries.from_points(np.asarray(x, dtype), np.asarray(y, dtype))
    xy = np.empty(2 * len(px), dtype)
    xy[0::2] = px
    xy[1::2] = py
    npoly = len(po) - 1
    polys = cs.GeoSeries.from_polygons_xy(xy, np.asarray(ro, np.int32), np.asarray(po, np.int32),
                                          np.arange(npoly + 1, dtype=np.int32))
    return pts, polys


def _bitmask(pts, polys, method):
    return to_np(cs.point_in_polygon_bitmask(pts, polys, method)).astype(np.int64)


def _pairwise_repeat(c, dtype):
    """Each point of a one-polygon case paired with its own copy of the polygon."""
    n = len(c["x"])
    ro = np.asarray(c["ring_offsets"], np.int64)
    po = np.asarray(c["poly_offsets"], np.int64)
    nr = po[1] - po[0]
    nv = ro[po[1]] - ro[po[0]]
    rings = np.concatenate([ro[po[0]:po[1]] - ro[po[0]] + i * nv for i in range(n)] + [[n * nv]])
    px = np.tile(np.asarray(c["px"])[ro[po[0]]:ro[po[1]]], n)
    py = np.tile(np.asarray(c["py"])[ro[po[0]]:ro[po[1]]], n)
    return _series(c["x"], c["y"], np.arange(n + 1) * nr, rings, px, py, dtype)


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("method", METHODS)
def test_point_in_polygon_known_answers(golden, dtype, method):
    # cpp/tests/point_in_polygon/point_in_polygon_test.cu:108-441
    for c in golden("point_in_polygon.json")["cases"]:
        pts, polys = _series(c["x"], c["y"], c["poly_offsets"], c["ring_offsets"], c["px"],
                             c["py"], dtype)
        got = _bitmask(pts, polys, method)
        want = np.array([int(e) for e in c["expected"]])
        np.testing.assert_array_equal(got, want, err_msg=c["name"])
        # the pairwise form on the single-polygon cases
        if len(c["poly_offsets"]) == 2:
            pp, qq = _pairwise_repeat(c, dtype)
            pw = to_np(cs.pairwise_point_in_polygon(pp, qq, method)).astype(np.int64)
            np.testing.assert_array_equal(pw, want, err_msg="pairwise " + c["name"])


def test_point_in_polygon_table_columns():
    # python/.../join/test_point_in_polygon.py: one bool column per polygon
    pts = cs.GeoSeries.from_points(np.array([0.0, -8.0, 6.0]), np.array([0.0, -8.0, 6.0]))
    px = [-10, 5, 5, -10, -10, 0, 10, 10, 0, 0]
    py = [-10, -10, 5, 5, -10, 0, 0, 10, 10, 0]
    _, polys = _series([0.0], [0.0], [0, 1, 2], [0, 5, 10], px, py, np.float64)
    t = cs.point_in_polygon(pts, polys)
    assert t.columns == [0, 1]
    assert t[0].dtype == torch.bool
    assert to_np(t[0]).tolist() == [True, True, False]
    assert to_np(t[1]).tolist() == [False, False, True]


def _random_case(rng, npoly, n, dtype):
    centers = rng.uniform(0, 100, (npoly, 2))
    k = rng.integers(3, 200, npoly)
    P = D.star_polygons(rng, centers, k, lambda g, pid: g.uniform(5, 40, len(pid)),
                        hole_fraction=0.3)
    x = rng.uniform(-20, 120, n)
    y = rng.uniform(-20, 120, n)
    bx, by = D._near_boundary(rng, P, n // 5)
    x[: n // 5] = bx
    y[: n // 5] = by
    return x.astype(dtype), y.astype(dtype), P


@pytest.mark.parametrize("dtype", DTYPES)
def test_point_in_polygon_random_against_oracle(dtype):
    rng = np.random.default_rng(11)
    for npoly in (1, 7, 31):
        x, y, P = _random_case(rng, npoly, 20000, dtype)
        pts = cs.GeoSeries.from_points(x, y)
        polys = gpu_polygons(P, dtype)
        want = O.point_in_polygon(x, y, P.part_offset, P.ring_offset, P.x.astype(dtype),
                                  P.y.astype(dtype)).astype(np.int64)
        assert want.any()
        for method in METHODS:
            got = _bitmask(pts, polys, method)
            np.testing.assert_array_equal(got, want, err_msg=f"{npoly} {method}")


def test_point_in_polygon_filtered_refines_boundary_points():
    rng = np.random.default_rng(12)
    x, y, P = _random_case(rng, 31, 50000, np.float64)
    pts = cs.GeoSeries.from_points(x, y)
    polys = gpu_polygons(P)
    _bitmask(pts, polys, "filtered")
    refined = cs.last_refined_count()
    # the on-vertex and near-edge points need float64; the bulk does not
    assert 0 < refined < 31 * 50000 // 4


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("vertices", [(3, 10), (10, 60), (40, 200), (150, 600)])
def test_pairwise_random_against_oracle(dtype, vertices):
    # covers each group width of the pairwise kernel (1, 4, 8, 32 lanes)
    w = D.pairwise_pip(6000, vertices_range=vertices, seed_offset=vertices[0])
    P = w.polygons
    x, y = w.x.astype(dtype), w.y.astype(dtype)
    pts = cs.GeoSeries.from_points(x, y)
    polys = gpu_polygons(P, dtype)
    want = O.point_in_polygon(x, y, P.part_offset, P.ring_offset, P.x.astype(dtype),
                              P.y.astype(dtype), pairwise=True)
    assert 0 < want.sum() < len(want)
    for method in METHODS:
        got = to_np(cs.pairwise_point_in_polygon(pts, polys, method))
        assert got.dtype == np.uint8
        np.testing.assert_array_equal(got, want, err_msg=method)


@pytest.mark.parametrize("method", METHODS)
def test_sequential_walk_cases(method):
    # repeated vertices, unclosed rings, tiny (denormal-scale) and non-finite
    # coordinates: the cases where the parallel edge walk hands the polygon
    # to the reference's sequential loop
    t = 1e-310
    polys_xy = [
        ([0, 4, 4, 4, 0, 0], [0, 0, 0, 4, 4, 0]),                 # repeated vertex
        ([0, 4, 4, 0], [0, 0, 4, 4]),                             # unclosed
        ([0, 4 * t, 4 * t, 0, 0], [0, 0, 4 * t, 4 * t, 0]),       # denormal scale
        ([0, 4, np.nan, 0, 0], [0, 0, 4, 4, 0]),                  # NaN vertex
        ([0, 4, np.inf, 0, 0], [0, 0, 4, 4, 0]),                  # infinite vertex
        ([0, 4, 4, 0, 0], [0, 0, 4, 4, 0]),                       # plain square
    ]
    pts_xy = [(1.0, 1.0), (2.0, 2.0), (2 * t, 2 * t), (1.0, 1.0), (1.0, 1.0), (np.nan, 1.0)]
    px = np.concatenate([np.asarray(a, float) for a, _ in polys_xy])
    py = np.concatenate([np.asarray(b, float) for _, b in polys_xy])
    ro = np.concatenate([[0], np.cumsum([len(a) for a, _ in polys_xy])])
    po = np.arange(len(polys_xy) + 1)
    x = np.array([p[0] for p in pts_xy])
    y = np.array([p[1] for p in pts_xy])
    pts, polys = _series(x, y, po, ro, px, py, np.float64)
    want = O.point_in_polygon(x, y, po, ro, px, py, pairwise=True)
    got = to_np(cs.pairwise_point_in_polygon(pts, polys, method))
    np.testing.assert_array_equal(got, want)
    # the same polygons in one bitmask call, every point against all six
    wantm = O.point_in_polygon(x, y, po, ro, px, py).astype(np.int64)
    np.testing.assert_array_equal(_bitmask(pts, polys, method), wantm)


def test_validation_and_empty_inputs():
    rng = np.random.default_rng(3)
    P = D.star_polygons(rng, rng.uniform(0, 100, (32, 2)), np.full(32, 5),
                        lambda g, pid: g.uniform(5, 10, len(pid)))
    polys = gpu_polygons(P)
    pts = cs.GeoSeries.from_points(np.zeros(4), np.zeros(4))
    # detail/point_in_polygon.cuh:93-94
    with pytest.raises(RuntimeError, match="Number of polygons cannot exceed 31"):
        cs.point_in_polygon(pts, polys)
    # point_in_polygon.cu:133-136
    with pytest.raises(RuntimeError, match="Must pass in the same number of points as polygons"):
        cs.pairwise_point_in_polygon(pts, polys)
    # no points: no polygon-count check, empty columns
    empty = cs.GeoSeries.from_points(np.zeros(0), np.zeros(0))
    t = cs.point_in_polygon(empty, polys)
    assert len(t.columns) == 32 and all(v.numel() == 0 for v in t.values())
    assert cs.pairwise_point_in_polygon(empty, cs.GeoSeries.from_polygons_xy(
        np.zeros(0), np.zeros(1, np.int32), np.zeros(1, np.int32),
        np.zeros(1, np.int32))).numel() == 0
    # no polygons: an empty table (join.py:66-67)
    nopoly = cs.GeoSeries.from_polygons_xy(np.zeros(0), np.zeros(1, np.int32),
                                           np.zeros(1, np.int32), np.zeros(1, np.int32))
    assert cs.point_in_polygon(pts, nopoly).columns == []
    # multipolygons are refused (join.py:69-74)
    multi = cs.GeoSeries.from_polygons_xy(
        np.array([0, 0, 1, 0, 1, 1, 0, 0, 2, 2, 3, 2, 3, 3, 2, 2], np.float64),
        np.array([0, 4, 8], np.int32), np.array([0, 1, 2], np.int32), np.array([0, 2], np.int32))
    with pytest.raises(ValueError, match="multipolygon"):
        cs.point_in_polygon(pts, multi)
    with pytest.raises(ValueError, match="multipolygon"):
        cs.pairwise_point_in_polygon(cs.GeoSeries.from_points(np.zeros(1), np.zeros(1)), multi)
