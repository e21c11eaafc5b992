"""GPU path against the oracle where the float32 filters' guards decide.

Every other parity test draws coordinates below about 2e4.  These cases move
the same shapes to projected-CRS magnitudes (millions of units, where a
float64 coordinate's ULP is near 1e-9 and the anchor grid is coarse), and
build frames whose polygon and leaf anchors lie more than 2^24 grid steps
apart, so the whole-point float64 path and the slab-lookup guard
(offset * slabs-per-unit above 2^14) run.  The drop-in's own acceptance
case, the 1,000,000-point / 256-polygon plain configuration, runs at its
stated size.  Pairs and rows must equal the oracle's exactly, in order;
nearest-linestring distances bit for bit.

Differential shape as in the reference's
cpp/tests/join/quadtree_point_in_polygon_test_large.cu:190-224 and the tie
rule of quadtree_point_to_nearest_linestring.cuh:279-294.
"""

import numpy as np
import pytest

import cuspatial_gb300 as cs
from cuspatial_gb300 import datasets as D
from helpers import (assert_tree_equal, gpu_linestrings, gpu_points, gpu_polygons, oracle_tree,
                     to_np, u32)
from oracle import oracle as O

pytestmark = pytest.mark.gpu

METHODS = ["exact", "filtered"]


def _pip_vs_oracle(w, method, dtype=np.float64):
    pts = gpu_points(w, dtype)
    pi, t = cs.quadtree_on_points(pts, w.x_min, w.x_max, w.y_min, w.y_max, w.scale, w.max_depth,
                                  w.max_size)
    polys = gpu_polygons(w.polygons, dtype)
    bb = cs.polygon_bounding_boxes(polys)
    j = cs.join_quadtree_and_bounding_boxes(t, bb, w.x_min, w.x_max, w.y_min, w.y_max, w.scale,
                                            w.max_depth)
    r = cs.quadtree_point_in_polygon(j, t, pi, pts, polys, method=method)
    refined = cs.last_refined_count()
    opi, ot = oracle_tree(w, dtype)
    assert_tree_equal(pi, t, opi, ot)
    P = w.polygons
    px, py = P.x.astype(dtype), P.y.astype(dtype)
    obb = O.polygon_bounding_boxes(P.part_offset, P.ring_offset, px, py)
    for k in ("minx", "miny", "maxx", "maxy"):
        np.testing.assert_array_equal(to_np(bb[k]), obb[k])
    oj = O.join_quadtree_and_bounding_boxes(ot, obb, w.x_min, w.x_max, w.y_min, w.y_max,
                                            w.scale, w.max_depth)
    np.testing.assert_array_equal(u32(j["bbox_offset"]), oj["bbox_offset"])
    np.testing.assert_array_equal(u32(j["quad_offset"]), oj["quad_offset"])
    orr = O.quadtree_point_in_polygon(oj, ot, opi, w.x.astype(dtype), w.y.astype(dtype),
                                      P.part_offset, P.ring_offset, px, py)
    np.testing.assert_array_equal(u32(r["polygon_index"]), orr["polygon_index"])
    np.testing.assert_array_equal(u32(r["point_index"]), orr["point_index"])
    return r, refined


def _translated_precision(dx, dy, n_points=400_000, n_polygons=1200, extent=2000.0):
    """The precision configuration's shapes moved by (dx, dy); the 1% of
    points on vertices or within 1e-9 of an edge are drawn again on the moved
    polygons, so they stay that close at the new magnitude."""
    w = D.precision_at_scale(n_points=n_points, n_polygons=n_polygons, extent=extent,
                             max_vertices=256, boundary_fraction=0.0)
    P = w.polygons
    P.x = P.x + dx
    P.y = P.y + dy
    x, y = w.x + dx, w.y + dy
    rng = np.random.default_rng(41)
    nb = n_points // 100
    sel = rng.choice(n_points, nb, replace=False)
    bx, by = D._near_boundary(rng, P, nb)
    x[sel], y[sel] = bx, by
    w.x, w.y = x, y
    w.x_min, w.x_max = w.x_min + dx, w.x_max + dx
    w.y_min, w.y_max = w.y_min + dy, w.y_max + dy
    return w


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_plain_small_config_full_size(method, dtype):
    # 1,000,000 uniform points in [0,1000)^2, 256 star polygons (8-64
    # vertices), max_depth 7, scale 1000/128, max_size 128
    w = D.plain_small()
    assert len(w.x) == 1_000_000 and w.polygons.num_polygons == 256
    r, _ = _pip_vs_oracle(w, method, dtype)
    assert int(r["polygon_index"].numel()) > 100_000


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("shift", [(4.0e6, 5.0e6), (-3.3e6, 6.1e6)])
def test_precision_projected_magnitudes(method, shift):
    w = _translated_precision(*shift)
    r, refined = _pip_vs_oracle(w, method)
    assert int(r["polygon_index"].numel()) > 10_000
    if method == "filtered":
        assert refined > 0


def _far_frame_workload(n_uniform=150_000, n_near=60_000, n_polygons=300, seed=43):
    """Small polygons near the origin (|coordinate| < 8, anchor grid 2^-19,
    so 2^24 grid steps are 32 units) and points over [-1000, 1000]^2 in a
    depth-3 tree: leaves are 250 units wide, and a leaf whose first point
    (in Morton order) lies far from a polygon pairs with it across more than
    2^24 grid steps; the others sit well inside the float32 range."""
    rng = np.random.default_rng(seed)
    centers = rng.uniform(-5.0, 5.0, (n_polygons, 2))
    P = D.star_polygons(rng, centers, rng.integers(8, 200, n_polygons),
                        lambda g, pid: g.uniform(0.2, 1.5, len(pid)), hole_fraction=0.1)
    x = np.concatenate([rng.uniform(-1000, 1000, n_uniform), rng.uniform(-7, 7, n_near)])
    y = np.concatenate([rng.uniform(-1000, 1000, n_uniform), rng.uniform(-7, 7, n_near)])
    nb = (n_uniform + n_near) // 100
    sel = rng.choice(len(x), nb, replace=False)
    bx, by = D._near_boundary(rng, P, nb)
    x[sel], y[sel] = bx, by
    return D.Workload("far_frames", x, y, -1000.0, 1000.0, -1000.0, 1000.0, 250.0, 3, 64,
                      polygons=P)


@pytest.mark.parametrize("method", METHODS)
def test_frames_beyond_float32_grid_range(method):
    w = _far_frame_workload()
    r, refined = _pip_vs_oracle(w, method)
    assert int(r["polygon_index"].numel()) > 1000
    if method == "filtered":
        assert refined > 0


@pytest.mark.parametrize("method", METHODS)
def test_frames_beyond_float32_grid_range_projected(method):
    # the same shapes at +4e6 / -2e6: coarse grid and far frames together
    w = _far_frame_workload(seed=44)
    dx, dy = 4.0e6, -2.0e6
    w.x, w.y = w.x + dx, w.y + dy
    w.polygons.x = w.polygons.x + dx
    w.polygons.y = w.polygons.y + dy
    w.x_min, w.x_max, w.y_min, w.y_max = w.x_min + dx, w.x_max + dx, w.y_min + dy, w.y_max + dy
    _pip_vs_oracle(w, method)


def _nearest_vs_oracle(w, method, depth, max_size):
    pts = gpu_points(w)
    pi, t = cs.quadtree_on_points(pts, w.x_min, w.x_max, w.y_min, w.y_max, w.scale, depth,
                                  max_size)
    lines = gpu_linestrings(w.linestrings)
    bb = cs.linestring_bounding_boxes(lines, w.expansion_radius)
    j = cs.join_quadtree_and_bounding_boxes(t, bb, w.x_min, w.x_max, w.y_min, w.y_max, w.scale,
                                            depth)
    r = cs.quadtree_point_to_nearest_linestring(j, t, pi, pts, lines, method=method)
    L = w.linestrings
    opi, ot = O.quadtree_on_points(w.x, w.y, w.x_min, w.x_max, w.y_min, w.y_max, w.scale, depth,
                                   max_size)
    obb = O.linestring_bounding_boxes(L.part_offset, L.x, L.y, w.expansion_radius)
    oj = O.join_quadtree_and_bounding_boxes(ot, obb, w.x_min, w.x_max, w.y_min, w.y_max,
                                            w.scale, depth)
    np.testing.assert_array_equal(u32(j["bbox_offset"]), oj["bbox_offset"])
    np.testing.assert_array_equal(u32(j["quad_offset"]), oj["quad_offset"])
    orr = O.quadtree_point_to_nearest_linestring(oj, ot, opi, w.x, w.y, L.part_offset, L.x, L.y)
    np.testing.assert_array_equal(u32(r["point_index"]), orr["point_index"])
    np.testing.assert_array_equal(u32(r["linestring_index"]), orr["linestring_index"])
    np.testing.assert_array_equal(to_np(r["distance"]), orr["distance"])
    return orr


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("shift", [(4.0e6, 5.0e6), (-5.5e6, 3.0e6)])
def test_nearest_projected_magnitudes(method, shift):
    w = D.nearest_linestring(n_points=60_000, n_linestrings=300, extent=1000.0)
    dx, dy = shift
    w.x, w.y = w.x + dx, w.y + dy
    L = w.linestrings
    L.x, L.y = L.x + dx, L.y + dy
    # some points exactly on vertices (distance 0 loses to any other)
    k = np.random.default_rng(45).integers(0, len(L.x), 500)
    w.x[:500], w.y[:500] = L.x[k], L.y[k]
    w.x_min, w.x_max, w.y_min, w.y_max = w.x_min + dx, w.x_max + dx, w.y_min + dy, w.y_max + dy
    w.scale = 1000.0 / 256
    orr = _nearest_vs_oracle(w, method, 8, 64)
    assert int((orr["linestring_index"] != 0xFFFFFFFF).sum()) > 10_000


@pytest.mark.parametrize("method", METHODS)
def test_nearest_frames_beyond_float32_grid_range(method):
    # short random walks near the origin, points over [-1000, 1000]^2 in a
    # depth-3 tree: leaf anchors far (in grid steps) from the linestrings
    rng = np.random.default_rng(46)
    n_ls = 200
    nv = rng.integers(2, 40, n_ls)
    offs = np.concatenate([[0], np.cumsum(nv)]).astype(np.int32)
    start = rng.uniform(-5, 5, (n_ls, 2))
    steps = rng.normal(0, 0.2, (int(offs[-1]), 2))
    lx = np.repeat(start[:, 0], nv) + np.cumsum(steps[:, 0]) - np.repeat(
        np.concatenate([[0.0], np.cumsum(steps[:, 0])[offs[1:-1] - 1]]), nv)
    ly = np.repeat(start[:, 1], nv) + np.cumsum(steps[:, 1]) - np.repeat(
        np.concatenate([[0.0], np.cumsum(steps[:, 1])[offs[1:-1] - 1]]), nv)
    x = np.concatenate([rng.uniform(-1000, 1000, 40_000), rng.uniform(-8, 8, 20_000)])
    y = np.concatenate([rng.uniform(-1000, 1000, 40_000), rng.uniform(-8, 8, 20_000)])
    w = D.Workload("far_lines", x, y, -1000.0, 1000.0, -1000.0, 1000.0, 250.0, 3, 64,
                   linestrings=D.Linestrings(lx, ly, offs, np.arange(n_ls + 1, dtype=np.int32)),
                   expansion_radius=3.0)
    orr = _nearest_vs_oracle(w, method, 3, 64)
    assert int((orr["linestring_index"] != 0xFFFFFFFF).sum()) > 10_000


def _dense_quadrant_workload(n_points, depth, max_size, seed):
    """Polygons of 1,000 to 4,000 vertices (per-vertex radius factor
    U[0.5, 1]: deep spikes, dozens of entries per slab) under a coarse tree,
    so a quadrant spans more than 31 slabs or lists more edges than one warp's
    list pool holds: such quadrants leave the quadrant classification for the
    per-point slab walk, beside quadrants that stay on it."""
    rng = np.random.default_rng(seed)
    n_poly = 40
    centers = rng.uniform(100.0, 900.0, (n_poly, 2))
    P = D.star_polygons(rng, centers, rng.integers(1000, 4000, n_poly),
                        lambda g, pid: g.uniform(40.0, 120.0, len(pid)) * g.uniform(0.5, 1.0, len(pid)),
                        hole_fraction=0.2)
    x = rng.uniform(0.0, 1000.0, n_points)
    y = rng.uniform(0.0, 1000.0, n_points)
    nb = n_points // 100
    sel = rng.choice(n_points, nb, replace=False)
    bx, by = D._near_boundary(rng, P, nb)
    x[sel], y[sel] = bx, by
    return D.Workload("dense_quadrants", x, y, 0.0, 1000.0, 0.0, 1000.0, 1000.0 / 2 ** depth,
                      depth, max_size, polygons=P)


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("depth,max_size", [(5, 1024), (4, 2048), (7, 256)])
def test_dense_quadrants(method, depth, max_size):
    w = _dense_quadrant_workload(400_000, depth, max_size, seed=47 + depth)
    r, refined = _pip_vs_oracle(w, method)
    assert int(r["polygon_index"].numel()) > 10_000
    if method == "filtered":
        assert refined > 0
