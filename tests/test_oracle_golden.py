"""The CPU oracle against the reference's own known-answer vectors.

Fixtures come from tests/golden/make_golden.py (cuSpatial's C++ tests read
as text); each test names the reference test it reproduces.
"""

import numpy as np
import pytest

from oracle import oracle as O

DTYPES = [np.float64, np.float32]


@pytest.mark.parametrize("dtype", DTYPES)
def test_quadtree_kats(golden, dtype):
    # cpp/tests/index/point_quadtree_test.cu:69-222
    for c in golden("point_quadtree.json")["cases"]:
        x = np.array(c["x"], dtype)
        y = np.array(c["y"], dtype)
        _, t = O.quadtree_on_points(x, y, c["x_min"], c["x_max"], c["y_min"], c["y_max"],
                                    c["scale"], c["max_depth"], c["max_size"])
        for k in ("key", "level", "length", "offset"):
            assert t[k].tolist() == c[k], (c["name"], k)
        assert t["is_internal_node"].astype(int).tolist() == c["is_internal_node"], c["name"]


def _small_tree(d, dtype):
    x = np.array(d["x"], dtype)
    y = np.array(d["y"], dtype)
    pi, t = O.quadtree_on_points(x, y, d["x_min"], d["x_max"], d["y_min"], d["y_max"],
                                 d["scale"], d["max_depth"], d["max_size"])
    return x, y, pi, t


@pytest.mark.parametrize("dtype", DTYPES)
def test_polygon_join_and_pip_small(golden, dtype):
    # cpp/tests/join/quadtree_point_in_polygon_test_small.cu:143-163
    d = golden("quadtree_point_in_polygon_small.json")
    x, y, pi, t = _small_tree(d, dtype)
    px = np.array(d["px"], dtype)
    py = np.array(d["py"], dtype)
    bb = O.polygon_bounding_boxes(d["part_offset"], d["ring_offset"], px, py)
    j = O.join_quadtree_and_bounding_boxes(t, bb, d["x_min"], d["x_max"], d["y_min"],
                                           d["y_max"], d["scale"], d["max_depth"])
    assert j["bbox_offset"].tolist() == d["join_bbox_offset"]
    assert j["quad_offset"].tolist() == d["join_quad_offset"]
    r = O.quadtree_point_in_polygon(j, t, pi, x, y, d["part_offset"], d["ring_offset"], px, py)
    assert r["polygon_index"].tolist() == d["polygon_index"]
    assert r["point_index"].tolist() == d["point_index"]


@pytest.mark.parametrize("dtype", DTYPES)
def test_linestring_join_and_nearest_small(golden, dtype):
    # cpp/tests/join/quadtree_point_to_nearest_linestring_test_small.cu:138-204
    d = golden("quadtree_point_to_nearest_linestring_small.json")
    x, y, pi, t = _small_tree(d, dtype)
    lx = np.array(d["lx"], dtype)
    ly = np.array(d["ly"], dtype)
    bb = O.linestring_bounding_boxes(d["part_offset"], lx, ly, d["expansion_radius"])
    j = O.join_quadtree_and_bounding_boxes(t, bb, d["x_min"], d["x_max"], d["y_min"],
                                           d["y_max"], d["scale"], d["max_depth"])
    assert j["bbox_offset"].tolist() == d["join_bbox_offset"]
    assert j["quad_offset"].tolist() == d["join_quad_offset"]
    r = O.quadtree_point_to_nearest_linestring(j, t, pi, x, y, d["part_offset"], lx, ly)
    assert r["point_index"].tolist() == d["point_index"]
    assert r["linestring_index"].tolist() == d["linestring_index"]
    expected = np.array(d["distance_f64" if dtype == np.float64 else "distance_f32"], dtype)
    # bit-exact: the oracle's dot product contraction matches the reference build
    assert np.array_equal(r["distance"], expected)


def test_point_in_polygon_boundary_rule(golden):
    # cpp/tests/point_in_polygon/point_in_polygon_test.cu:108-441 (planar cases):
    # on-edge and on-vertex points are outside, unclosed rings, holes.
    for c in golden("point_in_polygon.json")["cases"]:
        po, ro = c["poly_offsets"], c["ring_offsets"]
        for i, (x, y) in enumerate(zip(c["x"], c["y"])):
            got = 0
            for p in range(len(po) - 1):
                if O.is_point_in_polygon(x, y, ro, po[p], po[p + 1], c["px"], c["py"]):
                    got |= 1 << p
            assert got == int(c["expected"][i]), (c["name"], i)


@pytest.mark.parametrize("dtype", DTYPES)
def test_point_in_polygon_bitmask_and_pairwise(golden, dtype):
    # cpp/tests/point_in_polygon/point_in_polygon_test.cu:108-441, through
    # the unindexed entry points: the bitmask over all polygons, and each
    # point paired with its own copy of a single-polygon case
    for c in golden("point_in_polygon.json")["cases"]:
        x = np.array(c["x"], dtype)
        y = np.array(c["y"], dtype)
        px = np.array(c["px"], dtype)
        py = np.array(c["py"], dtype)
        want = [int(e) for e in c["expected"]]
        got = O.point_in_polygon(x, y, c["poly_offsets"], c["ring_offsets"], px, py)
        assert got.tolist() == want, c["name"]
        if len(c["poly_offsets"]) == 2:
            n = len(x)
            nv = len(px)
            ro = np.concatenate([np.asarray(c["ring_offsets"][:-1]) + i * nv for i in range(n)]
                                + [[n * nv]])
            nr = len(c["ring_offsets"]) - 1
            pw = O.point_in_polygon(x, y, np.arange(n + 1) * nr, ro, np.tile(px, n),
                                    np.tile(py, n), pairwise=True)
            assert pw.tolist() == want, c["name"]


@pytest.mark.parametrize("dtype", DTYPES)
def test_linestring_bounding_boxes_small(golden, dtype):
    # python/.../bounding/test_linestring_bounding_boxes.py:48-140
    d = golden("linestring_bounding_boxes_small.json")
    lx = np.array(d["lx"], dtype)
    ly = np.array(d["ly"], dtype)
    bb = O.linestring_bounding_boxes(d["part_offset"], lx, ly, d["expansion_radius"])
    for k in ("minx", "miny", "maxx", "maxy"):
        if dtype == np.float64:
            np.testing.assert_array_equal(bb[k], np.array(d[k], dtype))
        else:
            # the reference compares with cudf's default float tolerance
            np.testing.assert_allclose(bb[k], np.array(d[k], dtype), rtol=1e-5)


def test_polygon_bounding_boxes_skip_empty_polygon():
    # reduce_by_key over geometry ids (detail/bounding_boxes.cuh:75-87): a
    # polygon without vertices yields no row, later rows move up.
    po = [0, 1, 1, 2]
    ro = [0, 3, 6]
    x = np.array([0, 1, 2, 10, 11, 12], np.float64)
    y = np.array([5, 6, 7, 15, 16, 17], np.float64)
    bb = O.polygon_bounding_boxes(po, ro, x, y)
    assert bb["minx"][:2].tolist() == [0, 10]
    assert bb["maxy"][:2].tolist() == [7, 17]
    assert np.isnan(bb["minx"][2])


def _ulps(a, b):
    """Distance in units in the last place between same-dtype arrays."""
    a = np.asarray(a)
    b = np.asarray(b, dtype=a.dtype)
    it = np.int64 if a.dtype == np.float64 else np.int32
    ia = a.view(it).astype(np.int64)
    ib = b.view(it).astype(np.int64)
    top = np.int64(np.iinfo(it).min)
    ia = np.where(ia < 0, top - ia, ia)
    ib = np.where(ib < 0, top - ib, ib)
    return np.abs(ia - ib)


@pytest.mark.parametrize("dtype", DTYPES)
def test_pairwise_point_linestring_distance_kats(golden, dtype):
    # cpp/tests/distance/point_linestring_distance_test.cu:44-456; the
    # reference compares with gtest's 4-ULP float equality
    for c in golden("point_linestring_distance.json")["cases"]:
        r = O.pairwise_point_linestring(np.array(c["x"], dtype), np.array(c["y"], dtype),
                                        c["part_offsets"], np.array(c["lx"], dtype),
                                        np.array(c["ly"], dtype), c["point_geometry_offsets"],
                                        c["linestring_geometry_offsets"])
        want = np.array(c["expected"], dtype)
        assert len(r["distance"]) == len(want), c["name"]
        assert np.all(_ulps(r["distance"], want) <= 4), (c["name"], r["distance"], want)


@pytest.mark.parametrize("dtype", DTYPES)
def test_pairwise_point_linestring_nearest_points_kats(golden, dtype):
    # cpp/tests/nearest_points/point_linestring_nearest_points_test.cu:43-420
    for c in golden("point_linestring_nearest_points.json")["cases"]:
        n = c["num_pairs"]
        r = O.pairwise_point_linestring(np.array(c["x"], dtype), np.array(c["y"], dtype),
                                        c["part_offsets"], np.array(c["lx"], dtype),
                                        np.array(c["ly"], dtype), c["point_geometry_offsets"],
                                        c["linestring_geometry_offsets"])
        assert len(r["segment_id"]) == n
        for k in ("point_geometry_id", "linestring_geometry_id", "segment_id"):
            if c[k] is not None:
                assert r[k].tolist() == c[k], (c["name"], k)
        for k, ck in (("x", "nearest_x"), ("y", "nearest_y")):
            assert np.all(_ulps(r[k], np.array(c[ck], dtype)) <= 4), (c["name"], k)
