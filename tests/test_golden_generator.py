"""The reader of the reference's Python tests (tests/golden/make_golden.py)
on an inline test file of the same forms: it records each cuspatial call
chain and the expected frame, follows dtype parametrisation and helper
functions, and lists what it cannot follow."""

import os
import sys

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))

import make_golden as G  # noqa: E402

SOURCE = '''
import numpy as np
import pytest
import cudf
import cuspatial

bbox = (0, 8, 0, 8)
xs = cudf.Series([1.0, 2.0, 7.5])


def helper(dtype, expected):
    points = cuspatial.GeoSeries.from_points_xy(
        cudf.DataFrame({"x": xs.astype(dtype), "y": xs}).interleave_columns())
    order, tree = cuspatial.quadtree_on_points(points, *bbox, 1, 3, 2)
    cudf.testing.assert_frame_equal(tree, cudf.DataFrame({"key": cudf.Series(expected)}))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_tree(dtype):
    if dtype == np.float32:
        helper(dtype, [1, 2])
    else:
        helper(dtype, [3])


def test_pip():
    result = cuspatial.point_in_polygon(
        cuspatial.GeoSeries.from_points_xy(cudf.Series([0, 0], dtype="f8")),
        cuspatial.GeoSeries.from_polygons_xy(
            cudf.Series([-1, -1, 1, -1, 1, 1, -1, -1], dtype="f8"),
            cudf.Series([0, 4]), cudf.Series([0, 1]), cudf.Series([0, 1])))
    expected = cudf.DataFrame()
    expected[0] = [True]
    cudf.testing.assert_frame_equal(expected, result)


def test_unsupported():
    with pytest.raises(ValueError):
        cuspatial.point_in_polygon(None, None)
'''


def test_reader_follows_the_forms():
    cases, skipped = G.kats_from_python_source("inline.py", SOURCE)
    assert [(c["test"], c["dtype"]) for c in cases] == [
        ("test_tree", "float32"), ("test_tree", "float64"), ("test_pip", "float64")]
    t32, t64, pip = cases
    assert t32["expected"] == {"key": [1, 2]} and t64["expected"] == {"key": [3]}
    q = t32["actual"]
    assert q["op"] == "quadtree_on_points" and q["out"] == 1
    assert q["args"][0] == {"geometry": "points", "xy": [1.0, 1.0, 2.0, 2.0, 7.5, 7.5]}
    assert q["args"][1:] == [0, 8, 0, 8, 1, 3, 2]
    assert pip["actual"]["op"] == "point_in_polygon"
    poly = pip["actual"]["args"][1]
    assert poly["geometry"] == "polygons" and poly["ring_offset"] == [0, 4]
    assert pip["expected"] == {"0": [True]}
    assert [s["test"] for s in skipped] == ["test_unsupported"]
