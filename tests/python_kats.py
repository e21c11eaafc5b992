"""Replays the cases of tests/golden/python_tests.json: the reference's own
Python tests (python/cuspatial/cuspatial/tests/spatial/indexing/test_indexing.py,
tests/spatial/join/test_spatial_join.py, tests/spatial/join/test_point_in_polygon.py),
recorded by make_golden.py as chains of cuspatial calls plus the frames the
tests expect.  `run(record, dtype, impl)` evaluates a chain with the oracle
(impl="oracle") or with this library's public API (impl="gpu"), and `check`
compares the result with the expected frame (integers, booleans and the
nearest-linestring distances all exactly, although the reference's
assert_frame_equal would allow the distances a relative 1e-5)."""

import numpy as np

from oracle import oracle as O


def _xy(g, dtype):
    xy = np.asarray(g.get("xy", []), dtype=dtype)
    return xy[0::2].copy(), xy[1::2].copy()


def _offsets(g, key):
    return np.asarray(g.get(key, [0]), dtype=np.int32)


# --------------------------------------------------------------------------
# the oracle
# --------------------------------------------------------------------------
def _oracle(rec, dtype):
    op, a = rec["op"], rec["args"]
    if op == "quadtree_on_points":
        x, y = _xy(a[0], dtype)
        return O.quadtree_on_points(x, y, *a[1:8])[rec["out"]]
    if op == "polygon_bounding_boxes":
        px, py = _xy(a[0], dtype)
        return O.polygon_bounding_boxes(_offsets(a[0], "part_offset"),
                                        _offsets(a[0], "ring_offset"), px, py)
    if op == "linestring_bounding_boxes":
        lx, ly = _xy(a[0], dtype)
        return O.linestring_bounding_boxes(_offsets(a[0], "part_offset"), lx, ly, a[1])
    if op == "join_quadtree_and_bounding_boxes":
        return O.join_quadtree_and_bounding_boxes(_oracle(a[0], dtype), _oracle(a[1], dtype),
                                                  *a[2:8])
    if op in ("quadtree_point_in_polygon", "quadtree_point_to_nearest_linestring"):
        pairs, tree, pi = (_oracle(r, dtype) for r in a[:3])
        x, y = _xy(a[3], dtype)
        gx, gy = _xy(a[4], dtype)
        if op == "quadtree_point_in_polygon":
            return O.quadtree_point_in_polygon(pairs, tree, pi, x, y,
                                               _offsets(a[4], "part_offset"),
                                               _offsets(a[4], "ring_offset"), gx, gy)
        return O.quadtree_point_to_nearest_linestring(pairs, tree, pi, x, y,
                                                      _offsets(a[4], "part_offset"), gx, gy)
    if op == "point_in_polygon":
        if a[1]["geometry"] == "empty":
            return {}
        x, y = _xy(a[0], dtype)
        px, py = _xy(a[1], dtype)
        po = _offsets(a[1], "part_offset")
        mask = O.point_in_polygon(x, y, po, _offsets(a[1], "ring_offset"), px, py)
        return {str(p): ((mask >> p) & 1).astype(bool) for p in range(len(po) - 1)}
    raise ValueError(op)


# --------------------------------------------------------------------------
# this library's public API (device tensors)
# --------------------------------------------------------------------------
def _geo(g, dtype, kind):
    import cuspatial_gb300 as cs
    empty = g["geometry"] == "empty"
    xy = np.asarray(g.get("xy", []), dtype=dtype)
    if kind == "points":
        return cs.GeoSeries.from_points(xy[0::2].copy(), xy[1::2].copy())
    if kind == "polygons":
        if empty:
            return cs.GeoSeries.from_polygons_xy(xy, np.zeros(1, np.int32),
                                                 np.zeros(1, np.int32), np.zeros(1, np.int32))
        return cs.GeoSeries.from_polygons_xy(xy, _offsets(g, "ring_offset"),
                                             _offsets(g, "part_offset"),
                                             _offsets(g, "geometry_offset"))
    return cs.GeoSeries.from_linestrings_xy(xy, _offsets(g, "part_offset"),
                                            _offsets(g, "geometry_offset"))


def _gpu(rec, dtype):
    import cuspatial_gb300 as cs
    op, a = rec["op"], rec["args"]
    if op == "quadtree_on_points":
        return cs.quadtree_on_points(_geo(a[0], dtype, "points"), *a[1:8])[rec["out"]]
    if op == "polygon_bounding_boxes":
        return cs.polygon_bounding_boxes(_geo(a[0], dtype, "polygons"))
    if op == "linestring_bounding_boxes":
        return cs.linestring_bounding_boxes(_geo(a[0], dtype, "linestrings"), a[1])
    if op == "join_quadtree_and_bounding_boxes":
        return cs.join_quadtree_and_bounding_boxes(_gpu(a[0], dtype), _gpu(a[1], dtype), *a[2:8])
    if op == "quadtree_point_in_polygon":
        return cs.quadtree_point_in_polygon(*(_gpu(r, dtype) for r in a[:3]),
                                            _geo(a[3], dtype, "points"),
                                            _geo(a[4], dtype, "polygons"))
    if op == "quadtree_point_to_nearest_linestring":
        return cs.quadtree_point_to_nearest_linestring(*(_gpu(r, dtype) for r in a[:3]),
                                                       _geo(a[3], dtype, "points"),
                                                       _geo(a[4], dtype, "linestrings"))
    if op == "point_in_polygon":  # an empty polygon series gives an empty table
        return cs.point_in_polygon(_geo(a[0], dtype, "points"), _geo(a[1], dtype, "polygons"))
    raise ValueError(op)


def run(rec, dtype, impl):
    out = _oracle(rec, dtype) if impl == "oracle" else _gpu(rec, dtype)
    cols = {}
    for k, v in out.items():
        v = v.detach().cpu().numpy() if hasattr(v, "detach") else np.asarray(v)
        cols[str(k)] = v
    return cols


def _ulps(a, b):
    a = np.asarray(a)
    b = np.asarray(b, dtype=a.dtype)
    it = np.int32 if a.dtype == np.float32 else np.int64
    ia, ib = a.view(it).astype(np.int64), b.view(it).astype(np.int64)
    ia = np.where(ia < 0, np.iinfo(it).min - ia, ia)
    ib = np.where(ib < 0, np.iinfo(it).min - ib, ib)
    return np.abs(ia - ib)


def check(case, got):
    """Compares a replayed result with the case's expected frame."""
    exp = case["expected"]
    name = "%s[%s]" % (case["test"], case["dtype"])
    assert sorted(got) == sorted(exp), (name, sorted(got), sorted(exp))
    for k, want in exp.items():
        g = got[k]
        w = np.atleast_1d(np.asarray(want))
        assert g.shape == w.shape, (name, k, g.shape, w.shape)
        if k == "distance":
            assert np.all(_ulps(g, w.astype(g.dtype)) == 0), (name, g, w)
        elif g.dtype == np.bool_ or w.dtype == np.bool_:
            assert g.astype(bool).tolist() == w.astype(bool).tolist(), (name, k)
        else:
            assert g.astype(np.int64).tolist() == w.astype(np.int64).tolist(), (name, k)
