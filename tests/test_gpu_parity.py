"""GPU path (C ABI through the Python API) against the oracle.

Integer/index outputs must be identical, including order; distances must be
bit-identical to the oracle, which matches the reference's golden distances
bit for bit.  Cases follow the reference's tests (cpp/tests/index,
cpp/tests/join, cpp/tests/point_in_polygon) plus seeded synthetic workloads
of each benchmark shape at sizes the oracle finishes in seconds.
"""

import numpy as np
import pytest
import torch

import cuspatial_gb300 as cs
from cuspatial_gb300 import datasets as D
from helpers import (assert_tree_equal, gpu_linestrings, gpu_points, gpu_polygons, oracle_tree,
                     to_np, u32)
from oracle import oracle as O

pytestmark = pytest.mark.gpu

DTYPES = [np.float64, np.float32]
METHODS = ["exact", "filtered"]


def _xy(x, y, dtype):
    a = np.empty(2 * len(x), dtype)
    a[0::2] = x
    a[1::2] = y
    return a


@pytest.mark.parametrize("dtype", DTYPES)
def test_quadtree_kats(golden, dtype):
    # cpp/tests/index/point_quadtree_test.cu:69-222
    for c in golden("point_quadtree.json")["cases"]:
        pts = cs.GeoSeries.from_points(np.array(c["x"], dtype), np.array(c["y"], dtype))
        with pytest.warns(UserWarning) if c["scale"] < 0 else _nullcontext():
            pi, t = cs.quadtree_on_points(pts, c["x_min"], c["x_max"], c["y_min"], c["y_max"],
                                          c["scale"], c["max_depth"], c["max_size"])
        assert u32(t["key"]).tolist() == c["key"], c["name"]
        assert to_np(t["level"]).tolist() == c["level"], c["name"]
        assert to_np(t["is_internal_node"]).astype(int).tolist() == c["is_internal_node"]
        assert u32(t["length"]).tolist() == c["length"], c["name"]
        assert u32(t["offset"]).tolist() == c["offset"], c["name"]


class _nullcontext:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


def _small(d, dtype):
    pts = cs.GeoSeries.from_points(np.array(d["x"], dtype), np.array(d["y"], dtype))
    pi, t = cs.quadtree_on_points(pts, d["x_min"], d["x_max"], d["y_min"], d["y_max"],
                                  d["scale"], d["max_depth"], d["max_size"])
    return pts, pi, t


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("method", METHODS)
def test_pip_small_kat(golden, dtype, method):
    # cpp/tests/join/quadtree_point_in_polygon_test_small.cu:143-163
    d = golden("quadtree_point_in_polygon_small.json")
    pts, pi, t = _small(d, dtype)
    polys = cs.GeoSeries.from_polygons_xy(_xy(d["px"], d["py"], dtype), d["ring_offset"],
                                          d["part_offset"], d["geometry_offset"])
    bb = cs.polygon_bounding_boxes(polys)
    j = cs.join_quadtree_and_bounding_boxes(t, bb, d["x_min"], d["x_max"], d["y_min"],
                                            d["y_max"], d["scale"], d["max_depth"])
    assert u32(j["bbox_offset"]).tolist() == d["join_bbox_offset"]
    assert u32(j["quad_offset"]).tolist() == d["join_quad_offset"]
    r = cs.quadtree_point_in_polygon(j, t, pi, pts, polys, method=method)
    assert u32(r["polygon_index"]).tolist() == d["polygon_index"]
    assert u32(r["point_index"]).tolist() == d["point_index"]


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("method", METHODS)
def test_nearest_small_kat(golden, dtype, method):
    # cpp/tests/join/quadtree_point_to_nearest_linestring_test_small.cu:138-204
    d = golden("quadtree_point_to_nearest_linestring_small.json")
    pts, pi, t = _small(d, dtype)
    lines = cs.GeoSeries.from_linestrings_xy(_xy(d["lx"], d["ly"], dtype), d["part_offset"],
                                             d["geometry_offset"])
    bb = cs.linestring_bounding_boxes(lines, d["expansion_radius"])
    j = cs.join_quadtree_and_bounding_boxes(t, bb, d["x_min"], d["x_max"], d["y_min"],
                                            d["y_max"], d["scale"], d["max_depth"])
    assert u32(j["bbox_offset"]).tolist() == d["join_bbox_offset"]
    assert u32(j["quad_offset"]).tolist() == d["join_quad_offset"]
    r = cs.quadtree_point_to_nearest_linestring(j, t, pi, pts, lines, method=method)
    assert u32(r["point_index"]).tolist() == d["point_index"]
    assert u32(r["linestring_index"]).tolist() == d["linestring_index"]
    exp = np.array(d["distance_f64" if dtype == np.float64 else "distance_f32"], dtype)
    assert np.array_equal(to_np(r["distance"]), exp)


@pytest.mark.parametrize("dtype", DTYPES)
def test_linestring_bbox_kat(golden, dtype):
    d = golden("linestring_bounding_boxes_small.json")
    lines = cs.GeoSeries.from_linestrings_xy(_xy(d["lx"], d["ly"], dtype), d["part_offset"],
                                             d["geometry_offset"])
    bb = cs.linestring_bounding_boxes(lines, d["expansion_radius"])
    ref = O.linestring_bounding_boxes(d["part_offset"], np.array(d["lx"], dtype),
                                      np.array(d["ly"], dtype), d["expansion_radius"])
    for k in ("minx", "miny", "maxx", "maxy"):
        np.testing.assert_array_equal(to_np(bb[k]), ref[k])


def _pip_all_pairs(x, y, po, ro, px, py, dtype, method, max_depth=1):
    """Every polygon against every leaf of a shallow tree covering all points."""
    x = np.asarray(x, dtype)
    y = np.asarray(y, dtype)
    lo = min(x.min(), np.min(px)) - 1.0
    hi = max(x.max(), np.max(px), y.max(), np.max(py)) + 1.0
    lo = min(lo, y.min() - 1.0, np.min(py) - 1.0)
    pts = cs.GeoSeries.from_points(x, y)
    pi, t = cs.quadtree_on_points(pts, lo, hi, lo, hi, (hi - lo) / 2, max_depth, 1 << 20)
    nq = int(t["key"].numel())
    npoly = len(po) - 1
    pairs = {"bbox_offset": torch.arange(npoly, dtype=torch.int32).repeat_interleave(nq),
             "quad_offset": torch.arange(nq, dtype=torch.int32).repeat(npoly)}
    polys = cs.GeoSeries.from_polygons_xy(_xy(px, py, dtype), ro, po, np.arange(npoly + 1))
    r = cs.quadtree_point_in_polygon(pairs, t, pi, pts, polys, method=method)
    mask = np.zeros(len(x), np.int64)
    pimap = u32(pi)
    for poly, pos in zip(u32(r["polygon_index"]), u32(r["point_index"])):
        mask[pimap[pos]] |= 1 << int(poly)
    return mask


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("method", METHODS)
def test_boundary_rule_kats(golden, dtype, method):
    # cpp/tests/point_in_polygon/point_in_polygon_test.cu (planar cases): points on
    # edges and corners are outside; unclosed rings; holes; collinear boundary
    for c in golden("point_in_polygon.json")["cases"]:
        got = _pip_all_pairs(c["x"], c["y"], c["poly_offsets"], c["ring_offsets"], c["px"],
                             c["py"], dtype, method)
        assert got.tolist() == [int(e) for e in c["expected"]], c["name"]


def _run_pipeline(w, dtype, method):
    pts = gpu_points(w, dtype)
    pi, t = cs.quadtree_on_points(pts, w.x_min, w.x_max, w.y_min, w.y_max, w.scale, w.max_depth,
                                  w.max_size)
    polys = gpu_polygons(w.polygons, dtype)
    bb = cs.polygon_bounding_boxes(polys)
    j = cs.join_quadtree_and_bounding_boxes(t, bb, w.x_min, w.x_max, w.y_min, w.y_max, w.scale,
                                            w.max_depth)
    r = cs.quadtree_point_in_polygon(j, t, pi, pts, polys, method=method)
    return pi, t, bb, j, r


def _check_against_oracle(w, dtype, method):
    pi, t, bb, j, r = _run_pipeline(w, dtype, method)
    opi, ot = oracle_tree(w, dtype)
    assert_tree_equal(pi, t, opi, ot)
    P = w.polygons
    obb = O.polygon_bounding_boxes(P.part_offset, P.ring_offset, P.x.astype(dtype),
                                   P.y.astype(dtype))
    for k in ("minx", "miny", "maxx", "maxy"):
        np.testing.assert_array_equal(to_np(bb[k]), obb[k])
    oj = O.join_quadtree_and_bounding_boxes(ot, obb, w.x_min, w.x_max, w.y_min, w.y_max,
                                            w.scale, w.max_depth)
    np.testing.assert_array_equal(u32(j["bbox_offset"]), oj["bbox_offset"])
    np.testing.assert_array_equal(u32(j["quad_offset"]), oj["quad_offset"])
    orr = O.quadtree_point_in_polygon(oj, ot, opi, w.x.astype(dtype), w.y.astype(dtype),
                                      P.part_offset, P.ring_offset, P.x.astype(dtype),
                                      P.y.astype(dtype))
    np.testing.assert_array_equal(u32(r["polygon_index"]), orr["polygon_index"])
    np.testing.assert_array_equal(u32(r["point_index"]), orr["point_index"])
    return r


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("method", METHODS)
def test_plain_small_shape_vs_oracle(dtype, method):
    w = D.plain_small(n_points=200_000, n_polygons=64)
    r = _check_against_oracle(w, dtype, method)
    assert int(r["polygon_index"].numel()) > 1000


@pytest.mark.parametrize("method", METHODS)
def test_precision_shape_vs_oracle(method):
    # Gaussian mixture, holes, 1% of points on vertices / within 1e-9 of edges
    w = D.precision_at_scale(n_points=1_000_000, n_polygons=1500, extent=2000.0,
                             max_vertices=256)
    r = _check_against_oracle(w, np.float64, method)
    assert int(r["polygon_index"].numel()) > 10000
    if method == "filtered":
        assert cs.last_refined_count() > 0


def _square_grid_workload():
    """Axis-aligned squares and points on their edges, corners, vertical lines
    extended beyond the edges, duplicate vertices and unclosed rings."""
    rng = np.random.default_rng(7)
    sq_x, sq_y, ring_off, part_off = [], [], [0], [0]
    for i in range(6):
        for j in range(6):
            x0, y0 = 2.0 * i, 2.0 * j
            xs = [x0, x0 + 1, x0 + 1, x0, x0]
            ys = [y0, y0, y0 + 1, y0 + 1, y0]
            if (i + j) % 3 == 0:  # duplicate a vertex (degenerate edge)
                xs.insert(2, xs[1])
                ys.insert(2, ys[1])
            if (i + j) % 4 == 1:  # unclosed ring
                xs, ys = xs[:-1], ys[:-1]
            sq_x += xs
            sq_y += ys
            ring_off.append(len(sq_x))
            part_off.append(len(ring_off) - 1)
    px, py = [], []
    grid = np.arange(0, 12.5, 0.5)
    for a in grid:  # lattice points: corners, edge midpoints, vertical-line extensions
        for b in grid:
            px.append(a)
            py.append(b)
    px += list(rng.uniform(-1, 13, 3000))
    py += list(rng.uniform(-1, 13, 3000))
    return (np.array(px), np.array(py), np.array(part_off), np.array(ring_off), np.array(sq_x),
            np.array(sq_y))


@pytest.mark.parametrize("method", METHODS)
def test_axis_aligned_adversarial(method):
    px, py, po, ro, vx, vy = _square_grid_workload()
    w = D.Workload("squares", px, py, -1.0, 13.0, -1.0, 13.0, 14.0 / 64, 6, 16,
                   polygons=D.Polygons(vx, vy, ro.astype(np.int32), po.astype(np.int32),
                                       np.arange(len(po), dtype=np.int32)))
    _check_against_oracle(w, np.float64, method)


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("method", METHODS)
def test_nearest_linestring_shape_vs_oracle(dtype, method):
    w = D.nearest_linestring(n_points=60_000, n_linestrings=300, extent=1000.0)
    w.scale = (w.x_max - w.x_min) / 256  # depth 8: no clamping anywhere
    pts = gpu_points(w, dtype)
    pi, t = cs.quadtree_on_points(pts, w.x_min, w.x_max, w.y_min, w.y_max, w.scale, 8, 64)
    lines = gpu_linestrings(w.linestrings, dtype)
    bb = cs.linestring_bounding_boxes(lines, w.expansion_radius)
    j = cs.join_quadtree_and_bounding_boxes(t, bb, w.x_min, w.x_max, w.y_min, w.y_max, w.scale,
                                            8)
    r = cs.quadtree_point_to_nearest_linestring(j, t, pi, pts, lines, method=method)
    L = w.linestrings
    ox, oy = w.x.astype(dtype), w.y.astype(dtype)
    opi, ot = O.quadtree_on_points(ox, oy, w.x_min, w.x_max, w.y_min, w.y_max, w.scale, 8, 64)
    obb = O.linestring_bounding_boxes(L.part_offset, L.x.astype(dtype), L.y.astype(dtype),
                                      w.expansion_radius)
    oj = O.join_quadtree_and_bounding_boxes(ot, obb, w.x_min, w.x_max, w.y_min, w.y_max,
                                            w.scale, 8)
    np.testing.assert_array_equal(u32(j["bbox_offset"]), oj["bbox_offset"])
    orr = O.quadtree_point_to_nearest_linestring(oj, ot, opi, ox, oy, L.part_offset,
                                                 L.x.astype(dtype), L.y.astype(dtype))
    np.testing.assert_array_equal(u32(r["point_index"]), orr["point_index"])
    np.testing.assert_array_equal(u32(r["linestring_index"]), orr["linestring_index"])
    np.testing.assert_array_equal(to_np(r["distance"]), orr["distance"])


def test_empty_inputs():
    # cpp/tests/join/quadtree_point_in_polygon_test.cpp:154-348 (empty cases)
    empty = cs.GeoSeries.from_points(np.zeros(0), np.zeros(0))
    pi, t = cs.quadtree_on_points(empty, 0, 1, 0, 1, 1.0, 1, 1)
    assert pi.numel() == 0 and len(t) == 0
    pts = cs.GeoSeries.from_points(np.array([0.5]), np.array([0.5]))
    pi, t = cs.quadtree_on_points(pts, 0, 1, 0, 1, 1.0, 1, 1)
    bb = cs.Table(minx=torch.zeros(0, dtype=torch.float64, device="cuda"),
                  miny=torch.zeros(0, dtype=torch.float64, device="cuda"),
                  maxx=torch.zeros(0, dtype=torch.float64, device="cuda"),
                  maxy=torch.zeros(0, dtype=torch.float64, device="cuda"))
    j = cs.join_quadtree_and_bounding_boxes(t, bb, 0, 1, 0, 1, 1.0, 1)
    assert len(j) == 0
    polys = cs.GeoSeries.from_polygons_xy(np.array([0, 0, 1, 0, 1, 1, 0, 0.]), [0, 4], [0, 1],
                                          [0, 1])
    r = cs.quadtree_point_in_polygon(j, t, pi, pts, polys)
    assert len(r) == 0


def test_validation_errors():
    # cpp/tests/join/join_quadtree_and_bounding_boxes_test.cpp:35-122
    pts = cs.GeoSeries.from_points(np.array([0.5, 0.2]), np.array([0.5, 0.7]))
    pi, t = cs.quadtree_on_points(pts, 0, 1, 0, 1, 0.5, 2, 1)
    bb = cs.polygon_bounding_boxes(cs.GeoSeries.from_polygons_xy(
        np.array([0, 0, 1, 0, 1, 1, 0, 0.]), [0, 4], [0, 1], [0, 1]))
    lib = cs._lib if hasattr(cs, "_lib") else None
    from cuspatial_gb300 import _lib
    import ctypes
    st, keep = cs.api._tree_struct(t)
    b = [bb[k] for k in ("minx", "miny", "maxx", "maxy")]
    ob, oq, nn = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_size_t()
    lib = _lib.load()
    cases = [(0.0, 2, 0, 1, "scale must be positive"), (0.5, 0, 0, 1, "maximum depth"),
             (0.5, 16, 0, 1, "maximum depth"), (0.5, 2, 1, 0, "invalid bounding box")]
    for scale, depth, x0, x1, msg in cases:
        s = lib.cspt_join_quadtree_and_bounding_boxes(
            ctypes.byref(st), *[_lib.ptr(v) for v in b], 1, 1, float(x0), float(x1), 0.0, 1.0,
            scale, depth, None, _lib.stream_ptr(), ctypes.byref(ob), ctypes.byref(oq),
            ctypes.byref(nn))
        assert s == _lib.INVALID_ARGUMENT
        assert msg in lib.cspt_last_error_message().decode()
    with pytest.raises(RuntimeError, match="number of points"):
        cs.quadtree_point_in_polygon({"bbox_offset": torch.zeros(1, dtype=torch.int32),
                                      "quad_offset": torch.zeros(1, dtype=torch.int32)}, t,
                                     pi[:1], pts, cs.GeoSeries.from_polygons_xy(
                                         np.array([0, 0, 1, 0, 1, 1, 0, 0.]), [0, 4], [0, 1],
                                         [0, 1]))


@pytest.mark.parametrize("dtype", DTYPES)
def test_quadtree_edge_cases_vs_oracle(dtype):
    rng = np.random.default_rng(3)
    cases = []
    # duplicates and a single location
    cases.append((np.full(1000, 3.25), np.full(1000, 4.5), 0, 10, 0, 10, 10 / 16, 4, 10))
    # points outside the box share the corner cell
    x = rng.uniform(-5, 15, 5000)
    y = rng.uniform(-5, 15, 5000)
    cases.append((x, y, 0, 10, 0, 10, 10 / 64, 6, 20))
    # clamped scale (scale below the minimum), max_depth 0 and 1, max_size 1
    x = rng.uniform(0, 9.9, 3000)
    y = rng.uniform(0, 9.9, 3000)
    cases.append((x, y, 0, 10, 0, 10, 10 / 64, 0, 1))
    cases.append((x, y, 0, 10, 0, 10, 10 / 64, 1, 5))
    cases.append((x, y, 0, 10, 0, 10, 10 / 4096, 12, 1))
    # Gaussian clusters at depth 15
    x = np.clip(rng.normal(500, 3, 20000), 0, 999.9)
    y = np.clip(rng.normal(500, 3, 20000), 0, 999.9)
    cases.append((x, y, 0, 1000, 0, 1000, 1000 / 32768, 15, 32))
    # the box test at its edges: points on the bounds and one ulp either side,
    # both zeros, the smallest subnormals, infinities, a box bound of -0.0
    for x0, x1 in ((-10.0, 10.0), (-0.0, 10.0)):
        edge = np.array([x0, np.nextafter(x0, -np.inf), np.nextafter(x0, np.inf), x1,
                         np.nextafter(x1, np.inf), np.nextafter(x1, -np.inf), -0.0, 0.0,
                         5e-324, -5e-324, np.inf, -np.inf])
        x = np.concatenate([rng.choice(edge, 3000), rng.uniform(-12, 12, 3000)])
        y = np.concatenate([rng.choice(edge, 3000), rng.uniform(-12, 12, 3000)])
        cases.append((x, y, x0, x1, x0, x1, (x1 - x0) / 256, 8, 16))
    for x, y, x0, x1, y0, y1, scale, depth, size in cases:
        pts = cs.GeoSeries.from_points(x.astype(dtype), y.astype(dtype))
        import warnings
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            pi, t = cs.quadtree_on_points(pts, x0, x1, y0, y1, scale, depth, size)
        min_scale = max(x1 - x0, y1 - y0) / ((1 << depth) + 2)
        opi, ot = O.quadtree_on_points(x.astype(dtype), y.astype(dtype), x0, x1, y0, y1,
                                       max(scale, min_scale), depth, size)
        assert_tree_equal(pi, t, opi, ot)


def test_repeatable_output():
    w = D.precision_at_scale(n_points=300_000, n_polygons=400, extent=1500.0, max_vertices=128)
    a = _run_pipeline(w, np.float64, "filtered")[-1]
    b = _run_pipeline(w, np.float64, "filtered")[-1]
    assert torch.equal(a["polygon_index"], b["polygon_index"])
    assert torch.equal(a["point_index"], b["point_index"])


@pytest.mark.parametrize("method", METHODS)
def test_tiny_polygons_in_large_leaves(method):
    # sparse points -> leaves much larger than the polygons; the float32
    # filter must fall back to the exact test where its slab index is unsafe
    rng = np.random.default_rng(11)
    centers = rng.uniform(100, 9900, (200, 2))
    tiny = [1e-3 if i % 2 else 0.5 for i in range(200)]
    P = D.star_polygons(rng, centers, rng.integers(8, 40, 200),
                        lambda g, pid: np.asarray(tiny)[pid] * g.uniform(0.5, 1.0, len(pid)),
                        hole_fraction=0.2)
    x = rng.uniform(0, 10000, 20000)
    y = rng.uniform(0, 10000, 20000)
    # points inside and on the tiny polygons
    k = rng.integers(0, len(P.x), 4000)
    x = np.concatenate([x, P.x[k], centers[:, 0]])
    y = np.concatenate([y, P.y[k], centers[:, 1]])
    w = D.Workload("tiny", x, y, 0.0, 10000.0, 0.0, 10000.0, 10000.0 / 4096, 12, 64, polygons=P)
    _check_against_oracle(w, np.float64, method)


@pytest.mark.parametrize("method", METHODS)
def test_infinite_points(method):
    # +-inf coordinates take the out-of-box key and go through the exact test
    w = D.precision_at_scale(n_points=50_000, n_polygons=60, extent=300.0, max_vertices=64)
    x, y = w.x.copy(), w.y.copy()
    x[::997] = np.inf
    y[5::991] = -np.inf
    x[7::983] = -np.inf
    w.x, w.y = x, y
    _check_against_oracle(w, np.float64, method)


@pytest.mark.parametrize("method", METHODS)
def test_nearest_linestring_adversarial(method):
    # points on vertices and on segments (distance exactly 0 loses to any
    # non-zero candidate), symmetric ties (smaller id wins), zero-length
    # segments and single-vertex linestrings
    rng = np.random.default_rng(5)
    lx, ly, offs = [], [], [0]
    for i in range(40):
        y0 = 2.0 * i
        xs = [0.0, 3.0, 3.0, 6.0, 9.0]          # repeated vertex: zero-length segment
        ys = [y0, y0, y0, y0 + 1.0, y0]
        if i % 7 == 3:
            xs, ys = [4.0], [y0]               # a single vertex: no segment
        lx += xs
        ly += ys
        offs.append(len(lx))
    lx, ly = np.array(lx), np.array(ly)
    px = list(rng.uniform(-2, 11, 4000))
    py = list(rng.uniform(-2, 80, 4000))
    px += list(lx)                              # on vertices
    py += list(ly)
    px += [1.5] * 40                            # on the first segment of every line
    py += [2.0 * i for i in range(40)]
    px += [1.5] * 39                            # exactly between two lines: tie
    py += [2.0 * i + 1.0 for i in range(39)]
    px, py = np.array(px), np.array(py)
    w = D.Workload("lines", px, py, -5.0, 95.0, -5.0, 95.0, 100.0 / 64, 6, 16)
    pts = cs.GeoSeries.from_points(px, py)
    pi, t = cs.quadtree_on_points(pts, w.x_min, w.x_max, w.y_min, w.y_max, w.scale, 6, 16)
    xy = _xy(lx, ly, np.float64)
    lines = cs.GeoSeries.from_linestrings_xy(xy, np.array(offs), np.arange(len(offs)))
    bb = cs.linestring_bounding_boxes(lines, 1.5)
    j = cs.join_quadtree_and_bounding_boxes(t, bb, w.x_min, w.x_max, w.y_min, w.y_max, w.scale, 6)
    r = cs.quadtree_point_to_nearest_linestring(j, t, pi, pts, lines, method=method)
    opi, ot = O.quadtree_on_points(px, py, w.x_min, w.x_max, w.y_min, w.y_max, w.scale, 6, 16)
    obb = O.linestring_bounding_boxes(np.array(offs), lx, ly, 1.5)
    oj = O.join_quadtree_and_bounding_boxes(ot, obb, w.x_min, w.x_max, w.y_min, w.y_max,
                                            w.scale, 6)
    orr = O.quadtree_point_to_nearest_linestring(oj, ot, opi, px, py, np.array(offs), lx, ly)
    np.testing.assert_array_equal(u32(r["point_index"]), orr["point_index"])
    np.testing.assert_array_equal(u32(r["linestring_index"]), orr["linestring_index"])
    np.testing.assert_array_equal(to_np(r["distance"]), orr["distance"])


@pytest.mark.parametrize("method", METHODS)
def test_host_rows(method):
    # quadtree_point_in_polygon_host: 149,909 pairs evaluated in 8 chunks, rows
    # copied to page-locked and to pageable host tensors; the same rows as the
    # oracle, in the same order
    w = D.precision_at_scale(n_points=2_000_000, n_polygons=20_000, extent=4000.0,
                             max_vertices=64)
    pi, t, bb, j, r = _run_pipeline(w, np.float64, method)
    assert int(j["bbox_offset"].numel()) > 8 << 14
    pts, polys = gpu_points(w), gpu_polygons(w.polygons)
    m = int(r["polygon_index"].numel())
    P = w.polygons
    opi, ot = oracle_tree(w, np.float64)
    oj = O.join_quadtree_and_bounding_boxes(ot, O.polygon_bounding_boxes(
        P.part_offset, P.ring_offset, P.x, P.y), w.x_min, w.x_max, w.y_min, w.y_max, w.scale,
        w.max_depth)
    orr = O.quadtree_point_in_polygon(oj, ot, opi, w.x, w.y, P.part_offset, P.ring_offset,
                                      P.x, P.y)
    for pinned in (True, False):
        hp = torch.full((m + 5,), -1, dtype=torch.int32, pin_memory=pinned)
        hq = torch.full((m + 5,), -1, dtype=torch.int32, pin_memory=pinned)
        n = cs.quadtree_point_in_polygon_host(j, t, pi, pts, polys, hp, hq, method=method)
        assert n == m == len(orr["polygon_index"])
        np.testing.assert_array_equal(hp[:n].numpy().view(np.uint32), orr["polygon_index"])
        np.testing.assert_array_equal(hq[:n].numpy().view(np.uint32), orr["point_index"])
        assert hp[n:].tolist() == [-1] * 5
    # too few rows: the count comes back with the error (page-locked and
    # pageable arrays)
    for pinned in (True, False):
        small = torch.full((m - 1,), -1, dtype=torch.int32, pin_memory=pinned)
        with pytest.raises(cs.HostRowsTooFew) as e:
            cs.quadtree_point_in_polygon_host(j, t, pi, pts, polys, small, small.clone(),
                                              method=method)
        assert e.value.rows == m and str(m) in str(e.value)
    small = torch.empty(m - 1, dtype=torch.int32)
    # no pairs: nothing is written
    none = {"bbox_offset": j["bbox_offset"][:0], "quad_offset": j["quad_offset"][:0]}
    assert cs.quadtree_point_in_polygon_host(none, t, pi, pts, polys, small, small.clone(),
                                             method=method) == 0
    with pytest.raises(ValueError):
        cs.quadtree_point_in_polygon_host(j, t, pi, pts, polys, small.cuda(), small,
                                          method=method)


@pytest.mark.parametrize("dtype", DTYPES)
def test_quadtree_from_host(dtype):
    # quadtree_on_points_host: 9M points copied in 8 chunks (page-locked and
    # pageable), 3 chunks (an unpaired sorted run in the merge), 5M points on
    # a coarse lattice in 5 chunks (equal keys in every chunk: the merge
    # must keep them in input order), 1000 points in one chunk, and none;
    # the same tree and permutation as quadtree_on_points on the device copy,
    # and the device copy equals the input
    for n, pinned, lattice in ((9_000_000, True, False), (9_000_000, False, False),
                               (3 * (1 << 20) + 5, True, False), (5_000_000, True, True),
                               (1000, True, False), (0, True, False)):
        rng = np.random.default_rng(n + int(pinned))
        xs, ys = rng.normal(500, 150, n), rng.normal(500, 150, n)
        if lattice:
            xs, ys = np.round(xs / 25) * 25, np.round(ys / 25) * 25
        x = torch.from_numpy(xs.astype(dtype))
        y = torch.from_numpy(ys.astype(dtype))
        if pinned:
            x, y = x.pin_memory(), y.pin_memory()
        args = (0.0, 1000.0, 0.0, 1000.0, 1000.0 / (1 << 12), 12, 64)
        pts, pi, t = cs.quadtree_on_points_host(x, y, *args)
        assert torch.equal(pts.points.x.cpu(), x) and torch.equal(pts.points.y.cpu(), y)
        pi2, t2 = cs.quadtree_on_points(cs.GeoSeries.from_points(x.cuda(), y.cuda()), *args)
        assert torch.equal(pi, pi2)
        for k in t2:
            assert torch.equal(t[k], t2[k]), k
        if n:
            assert int(t["key"].numel()) > 0
    with pytest.raises(ValueError):
        cs.quadtree_on_points_host(x.cuda(), y, *args)
    with pytest.raises(TypeError):
        cs.quadtree_on_points_host(torch.zeros(3, dtype=torch.int32),
                                   torch.zeros(3, dtype=torch.int32), *args)


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_point_in_polygon_join_host(method, dtype):
    # the whole join from host columns to host rows in one call: the
    # oracle's rows, in order, with point ids mapped through its point_indices
    w = D.precision_at_scale(n_points=1_500_000, n_polygons=8000, extent=3000.0,
                             max_vertices=128)
    P = w.polygons
    px, py = P.x.astype(dtype), P.y.astype(dtype)
    opi, ot = oracle_tree(w, dtype)
    oj = O.join_quadtree_and_bounding_boxes(ot, O.polygon_bounding_boxes(
        P.part_offset, P.ring_offset, px, py), w.x_min, w.x_max, w.y_min, w.y_max, w.scale,
        w.max_depth)
    orr = O.quadtree_point_in_polygon(oj, ot, opi, w.x.astype(dtype), w.y.astype(dtype),
                                      P.part_offset, P.ring_offset, px, py)
    expect_poly = orr["polygon_index"]
    expect_point = opi.astype(np.int64)[orr["point_index"].astype(np.int64)].astype(np.uint32)
    m = len(expect_poly)
    assert m > 10_000

    def host(a, pinned):
        t = torch.from_numpy(np.ascontiguousarray(a))
        return t.pin_memory() if pinned else t

    for pinned in (True, False):
        cols = [host(w.x.astype(dtype), pinned), host(w.y.astype(dtype), pinned),
                host(P.part_offset.astype(np.int32), pinned),
                host(P.ring_offset.astype(np.int32), pinned), host(px, pinned), host(py, pinned)]
        hp = torch.full((m + 3,), -1, dtype=torch.int32, pin_memory=pinned)
        hq = torch.full((m + 3,), -1, dtype=torch.int32, pin_memory=pinned)
        # corners given swapped: ordered as join_quadtree_and_bounding_boxes does
        n = cs.point_in_polygon_join_host(cols[0], cols[1], w.x_max, w.x_min, w.y_max, w.y_min,
                                          w.scale, w.max_depth, w.max_size, *cols[2:], hp, hq,
                                          method=method)
        assert n == m
        np.testing.assert_array_equal(hp[:n].numpy().view(np.uint32), expect_poly)
        np.testing.assert_array_equal(hq[:n].numpy().view(np.uint32), expect_point)
        assert hp[n:].tolist() == [-1] * 3
    # too few rows: the count comes back with the error
    small = torch.empty(m - 1, dtype=torch.int32)
    with pytest.raises(cs.HostRowsTooFew) as e:
        cs.point_in_polygon_join_host(cols[0], cols[1], w.x_min, w.x_max, w.y_min, w.y_max,
                                      w.scale, w.max_depth, w.max_size, *cols[2:], small,
                                      small.clone(), method=method)
    assert e.value.rows == m
    # no points, no polygons: nothing written
    empty = torch.zeros(0, dtype=cols[0].dtype)
    assert cs.point_in_polygon_join_host(empty, empty, w.x_min, w.x_max, w.y_min, w.y_max,
                                         w.scale, w.max_depth, w.max_size, *cols[2:], small,
                                         small.clone(), method=method) == 0
    none = torch.zeros(1, dtype=torch.int32)
    assert cs.point_in_polygon_join_host(cols[0], cols[1], w.x_min, w.x_max, w.y_min, w.y_max,
                                         w.scale, w.max_depth, w.max_size, none, none,
                                         cols[4][:0], cols[5][:0], small, small.clone(),
                                         method=method) == 0
