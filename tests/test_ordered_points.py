"""Points in quadtree order (points_in_quadtree_order) and the *_ordered entry
points: the gathered copy equals x[point_indices], y[point_indices] exactly,
and point-in-polygon (device and host rows) and nearest-linestring results
through the ordered points equal the oracle's, in order, for both dtypes and
both methods.  No counterpart in the reference (its joins gather through
point_indices on every call)."""

import ctypes

import numpy as np
import pytest
import torch

import cuspatial_gb300 as cs
from cuspatial_gb300 import _lib
from cuspatial_gb300 import datasets as D
from helpers import gpu_linestrings, gpu_points, gpu_polygons, oracle_tree, to_np, u32
from oracle import oracle as O

pytestmark = pytest.mark.gpu

METHODS = ["exact", "filtered"]


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_gathered_copy_is_exact(dtype):
    w = D.precision_at_scale(n_points=300_000, n_polygons=10, extent=1000.0, max_vertices=16)
    pts = gpu_points(w, dtype)
    pi, t = cs.quadtree_on_points(pts, w.x_min, w.x_max, w.y_min, w.y_max, w.scale, w.max_depth,
                                  w.max_size)
    xy = cs.points_in_quadtree_order(pi, pts)
    assert xy.shape == (len(w.x), 2) and xy.dtype == pts.points.x.dtype
    p = u32(pi).astype(np.int64)
    np.testing.assert_array_equal(to_np(xy[:, 0]), w.x.astype(dtype)[p])
    np.testing.assert_array_equal(to_np(xy[:, 1]), w.y.astype(dtype)[p])


def test_out_of_range_index_gives_nan_and_misaligned_output_is_refused():
    x = torch.arange(4, dtype=torch.float64, device="cuda")
    y = -x
    pi = torch.tensor([3, 0, 7, 1], dtype=torch.int32, device="cuda")
    out = torch.empty(9, dtype=torch.float64, device="cuda")  # room for a shifted start
    lib = _lib.load()
    st = lib.cspt_points_in_quadtree_order(_lib.ptr(pi), 4, _lib.ptr(x), _lib.ptr(y), 4,
                                           _lib.FLOAT64, _lib.ptr(out), _lib.stream_ptr())
    assert st == _lib.OK
    got = out[:8].view(4, 2).cpu().numpy()
    assert got[0].tolist() == [3.0, -3.0] and got[1].tolist() == [0.0, -0.0]
    assert np.isnan(got[2]).all() and got[3].tolist() == [1.0, -1.0]
    st = lib.cspt_points_in_quadtree_order(_lib.ptr(pi), 4, _lib.ptr(x), _lib.ptr(y), 4,
                                           _lib.FLOAT64, ctypes.c_void_p(out.data_ptr() + 8),
                                           _lib.stream_ptr())
    assert st == _lib.INVALID_ARGUMENT
    assert b"16-byte boundary" in lib.cspt_last_error_message()


def _pip_oracle(w, dtype):
    P = w.polygons
    opi, ot = oracle_tree(w, dtype)
    px, py = P.x.astype(dtype), P.y.astype(dtype)
    obb = O.polygon_bounding_boxes(P.part_offset, P.ring_offset, px, py)
    oj = O.join_quadtree_and_bounding_boxes(ot, obb, w.x_min, w.x_max, w.y_min, w.y_max,
                                            w.scale, w.max_depth)
    return O.quadtree_point_in_polygon(oj, ot, opi, w.x.astype(dtype), w.y.astype(dtype),
                                       P.part_offset, P.ring_offset, px, py)


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_pip_ordered_equals_oracle(method, dtype):
    w = D.precision_at_scale(n_points=1_000_000, n_polygons=1500, extent=2000.0,
                             max_vertices=256)
    pts = gpu_points(w, dtype)
    pi, t = cs.quadtree_on_points(pts, w.x_min, w.x_max, w.y_min, w.y_max, w.scale, w.max_depth,
                                  w.max_size)
    polys = gpu_polygons(w.polygons, dtype)
    bb = cs.polygon_bounding_boxes(polys)
    j = cs.join_quadtree_and_bounding_boxes(t, bb, w.x_min, w.x_max, w.y_min, w.y_max, w.scale,
                                            w.max_depth)
    xy = cs.points_in_quadtree_order(pi, pts)
    r = cs.quadtree_point_in_polygon(j, t, pi, pts, polys, method=method, ordered_points=xy)
    orr = _pip_oracle(w, dtype)
    np.testing.assert_array_equal(u32(r["polygon_index"]), orr["polygon_index"])
    np.testing.assert_array_equal(u32(r["point_index"]), orr["point_index"])
    m = len(orr["polygon_index"])
    hp = torch.full((m + 3,), -1, dtype=torch.int32, pin_memory=True)
    hq = torch.full((m + 3,), -1, dtype=torch.int32, pin_memory=True)
    n = cs.quadtree_point_in_polygon_host(j, t, pi, pts, polys, hp, hq, method=method,
                                          ordered_points=xy)
    assert n == m
    np.testing.assert_array_equal(hp[:n].numpy().view(np.uint32), orr["polygon_index"])
    np.testing.assert_array_equal(hq[:n].numpy().view(np.uint32), orr["point_index"])
    with pytest.raises(ValueError):
        cs.quadtree_point_in_polygon(j, t, pi, pts, polys, method=method,
                                     ordered_points=xy[:-1])


@pytest.mark.parametrize("method", METHODS)
def test_nearest_ordered_equals_oracle(method):
    w = D.nearest_linestring(n_points=80_000, n_linestrings=400, extent=1000.0)
    w.scale = 1000.0 / 256
    pts = gpu_points(w)
    pi, t = cs.quadtree_on_points(pts, w.x_min, w.x_max, w.y_min, w.y_max, w.scale, 8, 64)
    lines = gpu_linestrings(w.linestrings)
    bb = cs.linestring_bounding_boxes(lines, w.expansion_radius)
    j = cs.join_quadtree_and_bounding_boxes(t, bb, w.x_min, w.x_max, w.y_min, w.y_max, w.scale,
                                            8)
    xy = cs.points_in_quadtree_order(pi, pts)
    r = cs.quadtree_point_to_nearest_linestring(j, t, pi, pts, lines, method=method,
                                                ordered_points=xy)
    L = w.linestrings
    opi, ot = O.quadtree_on_points(w.x, w.y, w.x_min, w.x_max, w.y_min, w.y_max, w.scale, 8, 64)
    obb = O.linestring_bounding_boxes(L.part_offset, L.x, L.y, w.expansion_radius)
    oj = O.join_quadtree_and_bounding_boxes(ot, obb, w.x_min, w.x_max, w.y_min, w.y_max,
                                            w.scale, 8)
    orr = O.quadtree_point_to_nearest_linestring(oj, ot, opi, w.x, w.y, L.part_offset, L.x, L.y)
    np.testing.assert_array_equal(u32(r["point_index"]), orr["point_index"])
    np.testing.assert_array_equal(u32(r["linestring_index"]), orr["linestring_index"])
    np.testing.assert_array_equal(to_np(r["distance"]), orr["distance"])


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_ordered_builds_equal_separate_gather(dtype):
    # quadtree_on_points_ordered / quadtree_on_points_host(ordered=True): the
    # same tree and permutation as quadtree_on_points, and the ordered copy
    # equal to points_in_quadtree_order (9M points: host copy in 8 chunks)
    w = D.precision_at_scale(n_points=9_000_000, n_polygons=10, extent=4000.0, max_vertices=16)
    args = (w.x_min, w.x_max, w.y_min, w.y_max, w.scale, w.max_depth, w.max_size)
    pts = gpu_points(w, dtype)
    pi, t = cs.quadtree_on_points(pts, *args)
    xy = cs.points_in_quadtree_order(pi, pts)
    pi2, t2, xy2 = cs.quadtree_on_points_ordered(pts, *args)
    assert torch.equal(pi, pi2) and torch.equal(xy, xy2)
    for k in t:
        assert torch.equal(t[k], t2[k]), k
    hx = torch.from_numpy(w.x.astype(dtype)).pin_memory()
    hy = torch.from_numpy(w.y.astype(dtype)).pin_memory()
    hpts, pi3, t3, xy3 = cs.quadtree_on_points_host(hx, hy, *args, ordered=True)
    assert torch.equal(pi, pi3) and torch.equal(xy, xy3)
    for k in t:
        assert torch.equal(t[k], t3[k]), k
    # no points: empty outputs, no error
    e = cs.GeoSeries.from_points(np.zeros(0, dtype), np.zeros(0, dtype))
    pe, te, xe = cs.quadtree_on_points_ordered(e, *args)
    assert pe.numel() == 0 and len(te) == 0 and xe.shape == (0, 2)
