"""Pairwise (multi)point - (multi)linestring distance and nearest points
against the reference's known answers
(cpp/tests/distance/point_linestring_distance_test.cu,
cpp/tests/nearest_points/point_linestring_nearest_points_test.cu) and, bit
for bit, against the oracle."""

import numpy as np
import pytest
import torch

import cuspatial_gb300 as cs
from oracle import oracle as O

from helpers import to_np
from test_oracle_golden import _ulps

pytestmark = pytest.mark.gpu

DTYPES = [np.float64, np.float32]
METHODS = ["exact", "filtered"]


def _series(x, y, pgo, part_offsets, lx, ly, lgo, dtype):
    n_ls = len(part_offsets) - 1
    if pgo is None:
        pts = cs.GeoSeries.from_points(np.asarray(x, dtype), np.asarray(y, dtype))
    else:
        xy = np.empty(2 * len(x), dtype)
        xy[0::2], xy[1::2] = x, y
        pts = cs.GeoSeries.from_multipoints_xy(xy, np.asarray(pgo, np.int32))
    lxy = np.empty(2 * len(lx), dtype)
    lxy[0::2], lxy[1::2] = lx, ly
    go = np.asarray(lgo if lgo is not None else np.arange(n_ls + 1), np.int32)
    lines = cs.GeoSeries.from_linestrings_xy(lxy, np.asarray(part_offsets, np.int32), go)
    return pts, lines


def _oracle(x, y, pgo, part_offsets, lx, ly, lgo, dtype):
    return O.pairwise_point_linestring(np.asarray(x, dtype), np.asarray(y, dtype), part_offsets,
                                       np.asarray(lx, dtype), np.asarray(ly, dtype), pgo, lgo)


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("method", METHODS)
def test_distance_known_answers(golden, dtype, method):
    for c in golden("point_linestring_distance.json")["cases"]:
        args = (c["x"], c["y"], c["point_geometry_offsets"], c["part_offsets"], c["lx"],
                c["ly"], c["linestring_geometry_offsets"], dtype)
        pts, lines = _series(*args)
        got = to_np(cs.pairwise_point_linestring_distance(pts, lines, method))
        want = np.array(c["expected"], dtype)
        assert len(got) == len(want), c["name"]
        assert np.all(_ulps(got, want) <= 4), (c["name"], got, want)
        np.testing.assert_array_equal(got, _oracle(*args)["distance"], err_msg=c["name"])


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("method", METHODS)
def test_nearest_points_known_answers(golden, dtype, method):
    for c in golden("point_linestring_nearest_points.json")["cases"]:
        args = (c["x"], c["y"], c["point_geometry_offsets"], c["part_offsets"], c["lx"],
                c["ly"], c["linestring_geometry_offsets"], dtype)
        pts, lines = _series(*args)
        t = cs.pairwise_point_linestring_nearest_points(pts, lines, method)
        assert len(t) == c["num_pairs"]
        for k in ("point_geometry_id", "linestring_geometry_id", "segment_id"):
            if c[k] is not None:
                assert to_np(t[k]).tolist() == c[k], (c["name"], k)
        gx = to_np(t["geometry"].points.x)
        gy = to_np(t["geometry"].points.y)
        assert np.all(_ulps(gx, np.array(c["nearest_x"], dtype)) <= 4), c["name"]
        assert np.all(_ulps(gy, np.array(c["nearest_y"], dtype)) <= 4), c["name"]
        o = _oracle(*args)
        np.testing.assert_array_equal(gx, o["x"])
        np.testing.assert_array_equal(gy, o["y"])


def _random(rng, n, seg_range, multi, dtype):
    """n pairs: 1-3 points (multi) near random-walk linestrings, 1-3 parts."""
    npts = rng.integers(1, 4, n) if multi else np.ones(n, np.int64)
    nparts = rng.integers(1, 4, n) if multi else np.ones(n, np.int64)
    nv = rng.integers(seg_range[0] + 1, seg_range[1] + 2, int(nparts.sum()))
    centers = rng.uniform(-1e4, 1e4, (n, 2))
    part_geom = np.repeat(np.arange(n), nparts)
    steps = rng.normal(0, 3.0, (int(nv.sum()), 2))
    start = np.concatenate([[0], np.cumsum(nv)])
    lx = np.empty(int(nv.sum()))
    ly = np.empty(int(nv.sum()))
    for j in range(len(nv)):
        s = slice(start[j], start[j + 1])
        c = centers[part_geom[j]] + rng.normal(0, 5.0, 2)
        lx[s] = c[0] + np.cumsum(steps[s, 0])
        ly[s] = c[1] + np.cumsum(steps[s, 1])
    pc = np.repeat(centers, npts, axis=0)
    x = pc[:, 0] + rng.normal(0, 8.0, len(pc))
    y = pc[:, 1] + rng.normal(0, 8.0, len(pc))
    # some points exactly on vertices, some vertices repeated
    k = rng.random(len(x)) < 0.1
    idx = rng.integers(0, len(lx), int(k.sum()))
    x[k], y[k] = lx[idx], ly[idx]
    r = rng.integers(1, len(lx), len(lx) // 50)
    lx[r], ly[r] = lx[r - 1], ly[r - 1]
    pgo = np.concatenate([[0], np.cumsum(npts)]) if multi else None
    lgo = np.concatenate([[0], np.cumsum(nparts)])
    return (x.astype(dtype), y.astype(dtype), pgo, start, lx.astype(dtype), ly.astype(dtype),
            lgo, dtype)


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("segs", [(1, 8), (10, 40), (40, 150), (150, 500)])
@pytest.mark.parametrize("multi", [False, True])
def test_random_against_oracle(dtype, segs, multi):
    # covers each group width (1, 4, 8, 32 lanes per pair)
    rng = np.random.default_rng(segs[0] * 7 + int(multi))
    args = _random(rng, 3000 if segs[1] <= 150 else 600, segs, multi, dtype)
    pts, lines = _series(*args)
    o = _oracle(*args)
    for method in METHODS:
        d = to_np(cs.pairwise_point_linestring_distance(pts, lines, method))
        np.testing.assert_array_equal(d, o["distance"], err_msg=method)
        t = cs.pairwise_point_linestring_nearest_points(pts, lines, method)
        for k in ("linestring_geometry_id", "segment_id"):
            np.testing.assert_array_equal(to_np(t[k]), o[k], err_msg=f"{method} {k}")
        if multi:
            np.testing.assert_array_equal(to_np(t["point_geometry_id"]),
                                          o["point_geometry_id"])
        np.testing.assert_array_equal(to_np(t["geometry"].points.x), o["x"])
        np.testing.assert_array_equal(to_np(t["geometry"].points.y), o["y"])


def test_edge_cases_and_validation():
    d = np.float64
    # a one-vertex linestring (no segment), a degenerate segment, a NaN
    # vertex and a point without a finite coordinate
    x = [0.0, 1.0, 2.0, np.nan]
    y = [0.0, 1.0, 2.0, 0.0]
    parts = [0, 1, 3, 6, 8]
    lx = [5.0, 3.0, 3.0, 0.0, np.nan, 4.0, 0.0, 1.0]
    ly = [5.0, 3.0, 3.0, 0.0, 1.0, 4.0, 0.0, 1.0]
    args = (x, y, None, parts, lx, ly, None, d)
    pts, lines = _series(*args)
    o = _oracle(*args)
    for method in METHODS:
        got = to_np(cs.pairwise_point_linestring_distance(pts, lines, method))
        np.testing.assert_array_equal(got, o["distance"])
        assert got[0] == np.finfo(d).max  # no segment: the initial value
        t = cs.pairwise_point_linestring_nearest_points(pts, lines, method)
        np.testing.assert_array_equal(to_np(t["segment_id"]), o["segment_id"])
    # mismatched pair counts (point_linestring_distance.cu:92-93,
    # point_linestring_nearest_points.cu:233-234)
    pts2 = cs.GeoSeries.from_points(np.zeros(3), np.zeros(3))
    with pytest.raises(RuntimeError, match="Inputs should have the same number of geometries."):
        cs.pairwise_point_linestring_distance(pts2, lines)
    with pytest.raises(RuntimeError, match="Mismatch number of"):
        cs.pairwise_point_linestring_nearest_points(pts2, lines)
    with pytest.raises(ValueError):
        cs.pairwise_point_linestring_distance(lines, lines)
    # empty input
    e = cs.GeoSeries.from_points(np.zeros(0), np.zeros(0))
    el = cs.GeoSeries.from_linestrings_xy(np.zeros(0), np.zeros(1, np.int32),
                                          np.zeros(1, np.int32))
    assert cs.pairwise_point_linestring_distance(e, el).numel() == 0
    assert len(cs.pairwise_point_linestring_nearest_points(e, el)) == 0
    assert torch.is_tensor(cs.pairwise_point_linestring_distance(e, el))


def test_offsets_checked_on_the_device():
    d = np.float64
    # geometry offsets that name a part past the last one select only the
    # existing parts (as the reference's per-vertex distance kernel does)
    args = ([0.0, 5.0], [0.0, 5.0], None, [0, 2, 4], [1.0, 2.0, 4.0, 6.0], [1.0, 1.0, 5.0, 5.0],
            [0, 1, 3], d)
    pts, lines = _series(*args)
    got = to_np(cs.pairwise_point_linestring_distance(pts, lines))
    np.testing.assert_array_equal(got, _oracle(*args)["distance"])
    # point offsets past the last point are refused, nothing is read there
    xy = np.array([0.0, 0.0, 1.0, 1.0])
    mp = cs.GeoSeries.from_multipoints_xy(xy, np.array([0, 5], np.int32))
    one = cs.GeoSeries.from_linestrings_xy(np.array([0.0, 1.0, 2.0, 1.0]),
                                           np.array([0, 2], np.int32), np.array([0, 1], np.int32))
    with pytest.raises(RuntimeError, match="offsets out of range"):
        cs.pairwise_point_linestring_distance(mp, one)
