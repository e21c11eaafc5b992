"""Batched point-in-polygon join: every instance's rows, sorted point order and
quadtree equal what the single-instance calls return for it alone, and a few
instances are checked against the oracle directly."""

import numpy as np
import pytest
import torch

import cuspatial_gb300 as cs
from cuspatial_gb300 import datasets as D
from cuspatial_gb300.batched import BatchedPointInPolygon
from oracle import oracle as O

from helpers import gpu_polygons, tree_np, u32

pytestmark = pytest.mark.gpu

DEPTHS = (1, 2, 3, 5, 7, 9, 12, 15)
SIZES = (1, 3, 8, 16, 40, 100, 300)


def _workload(n=24, seed=0):
    wl = D.batched_instances(n, points_range=(1, 20000), polygons_range=(1, 150),
                             side_range=(50.0, 5000.0), vertices_range=(3, 40),
                             seed_offset=seed)
    po = wl.point_offsets.copy()
    qo = wl.polygon_offsets.copy()
    po[4] = po[3]  # instance 3: no points (its points go to instance 4, outside its box)
    qo[6] = qo[5]  # instance 5: no polygons
    wl.point_offsets, wl.polygon_offsets = po, qo
    rng = np.random.default_rng(seed)
    params = []
    for i in range(wl.num_instances):
        x0, x1, y0, y1 = wl.boxes[i]
        d = int(DEPTHS[i % len(DEPTHS)])
        span = max(x1 - x0, y1 - y0)
        # scales at and above the finest the box allows
        scale = span / ((1 << d) + 2) * float(rng.choice([1.0, 1.0, 1.7]))
        params.append(dict(x_min=x0, x_max=x1, y_min=y0, y_max=y1, scale=scale, max_depth=d,
                           max_size=int(SIZES[i % len(SIZES)])))
    return wl, params


def _polygons(wl):
    return gpu_polygons(wl.polygons)


def _instance_polygons(wl, i):
    p = wl.polygons
    a, b = int(wl.polygon_offsets[i]), int(wl.polygon_offsets[i + 1])
    r0, r1 = int(p.part_offset[a]), int(p.part_offset[b])
    v0, v1 = int(p.ring_offset[r0]), int(p.ring_offset[r1])
    return (p.part_offset[a:b + 1] - r0, p.ring_offset[r0:r1 + 1] - v0, p.x[v0:v1], p.y[v0:v1])


def _single(wl, i, prm, method):
    """The single-instance pipeline through the drop-in API."""
    a, b = int(wl.point_offsets[i]), int(wl.point_offsets[i + 1])
    if b == a:
        return None
    pts = cs.GeoSeries.from_points(wl.x[a:b], wl.y[a:b])
    pi, tree = cs.quadtree_on_points(pts, prm["x_min"], prm["x_max"], prm["y_min"],
                                     prm["y_max"], prm["scale"], prm["max_depth"],
                                     prm["max_size"])
    po, ro, px, py = _instance_polygons(wl, i)
    rows = (np.zeros(0, np.uint32), np.zeros(0, np.uint32))
    if len(po) > 1:
        xy = np.empty(2 * len(px))
        xy[0::2], xy[1::2] = px, py
        polys = cs.GeoSeries.from_polygons_xy(xy, ro, po, np.arange(len(po)))
        boxes = cs.polygon_bounding_boxes(polys)
        pairs = cs.join_quadtree_and_bounding_boxes(tree, boxes, prm["x_min"], prm["x_max"],
                                                    prm["y_min"], prm["y_max"], prm["scale"],
                                                    prm["max_depth"])
        r = cs.quadtree_point_in_polygon(pairs, tree, pi, pts, polys, method=method)
        rows = (u32(r["polygon_index"]), u32(r["point_index"]))
    return u32(pi), tree_np(tree), rows


def _check_plan(plan, wl, params, method, expect=None):
    ro, pidx, qidx = plan.rows()
    ro = ro.cpu().numpy()
    pidx, qidx = u32(pidx), u32(qidx)
    total = 0
    out = []
    for i in range(wl.num_instances):
        got = (pidx[ro[i]:ro[i + 1]], qidx[ro[i]:ro[i + 1]])
        total += len(got[0])
        ref = expect[i] if expect is not None else _single(wl, i, params[i], method)
        out.append(ref)
        if ref is None:
            assert len(got[0]) == 0
            assert plan.point_indices(i).numel() == 0
            assert plan.quadtree(i)["key"].numel() == 0
            continue
        pi_ref, tree_ref, rows_ref = ref
        np.testing.assert_array_equal(u32(plan.point_indices(i)), pi_ref, err_msg=f"pi {i}")
        t = tree_np(plan.quadtree(i))
        for k in ("key", "level", "is_internal_node", "length", "offset"):
            np.testing.assert_array_equal(t[k], tree_ref[k], err_msg=f"tree {k} {i}")
        np.testing.assert_array_equal(got[0], rows_ref[0], err_msg=f"polygon_index {i}")
        np.testing.assert_array_equal(got[1], rows_ref[1], err_msg=f"point_index {i}")
    assert total == len(pidx)
    return out


@pytest.mark.parametrize("ordered", [True, False])
@pytest.mark.parametrize("method", ["exact", "filtered"])
def test_batched_matches_single_instance_calls(method, ordered):
    # ordered=False: the one-shot polygon index and its quadrant fast path
    wl, params = _workload(24, seed=1)
    plan = BatchedPointInPolygon(torch.from_numpy(wl.x).cuda(), torch.from_numpy(wl.y).cuda(),
                                 wl.point_offsets, _polygons(wl), wl.polygon_offsets, params,
                                 method=method, ordered_index=ordered)
    # the first run writes the rows from the plan's own evaluation
    plan.run(graph=False)
    torch.cuda.synchronize()
    expect = _check_plan(plan, wl, params, method)
    assert plan.info().num_rows > 500
    # a second direct run evaluates again
    plan.run(graph=False)
    torch.cuda.synchronize()
    _check_plan(plan, wl, params, method, expect)
    # graph capture, then two replays: same rows each time
    for _ in range(2):
        plan.run(graph=True)
        torch.cuda.synchronize()
        _check_plan(plan, wl, params, method, expect)
    assert plan.info().kernels_per_run >= 5
    plan.close()


def test_batched_against_oracle():
    wl, params = _workload(10, seed=2)
    plan = BatchedPointInPolygon(torch.from_numpy(wl.x).cuda(), torch.from_numpy(wl.y).cuda(),
                                 wl.point_offsets, _polygons(wl), wl.polygon_offsets, params)
    plan.run()
    torch.cuda.synchronize()
    ro, pidx, qidx = plan.rows()
    ro = ro.cpu().numpy()
    pidx, qidx = u32(pidx), u32(qidx)
    checked = 0
    for i in range(wl.num_instances):
        a, b = int(wl.point_offsets[i]), int(wl.point_offsets[i + 1])
        po, rg, px, py = _instance_polygons(wl, i)
        if b == a or len(po) < 2:
            continue
        p = params[i]
        opi, otree = O.quadtree_on_points(wl.x[a:b], wl.y[a:b], p["x_min"], p["x_max"],
                                          p["y_min"], p["y_max"], p["scale"], p["max_depth"],
                                          p["max_size"])
        np.testing.assert_array_equal(u32(plan.point_indices(i)), opi)
        boxes = O.polygon_bounding_boxes(po, rg, px, py)
        scale = max(p["scale"], max(p["x_max"] - p["x_min"], p["y_max"] - p["y_min"]) /
                    ((1 << p["max_depth"]) + 2))
        pairs = O.join_quadtree_and_bounding_boxes(otree, boxes, p["x_min"], p["x_max"],
                                                   p["y_min"], p["y_max"], scale,
                                                   p["max_depth"])
        r = O.quadtree_point_in_polygon(pairs, otree, opi, wl.x[a:b], wl.y[a:b], po, rg, px, py)
        np.testing.assert_array_equal(pidx[ro[i]:ro[i + 1]], r["polygon_index"])
        np.testing.assert_array_equal(qidx[ro[i]:ro[i + 1]], r["point_index"])
        checked += 1
    assert checked >= 6
    plan.close()


def test_batched_autotuned_params_and_refinement():
    from cuspatial_gb300 import autotune
    wl = D.batched_instances(32, points_range=(1e3, 2e4), polygons_range=(1, 200),
                             seed_offset=3)
    params = autotune.batch_params(wl)
    plan = BatchedPointInPolygon(torch.from_numpy(wl.x).cuda(), torch.from_numpy(wl.y).cuda(),
                                 wl.point_offsets, _polygons(wl), wl.polygon_offsets, params,
                                 method="filtered", block_threads=128)
    plan.run(graph=True)
    torch.cuda.synchronize()
    ro = plan.rows()[0].cpu().numpy()
    for i in (0, 7, 31):
        _, _, rows = _single(wl, i, params[i], "exact")
        got = plan.instance_result(i)
        assert ro[i + 1] - ro[i] == len(rows[0])
        np.testing.assert_array_equal(u32(got["polygon_index"]), rows[0])
        np.testing.assert_array_equal(u32(got["point_index"]), rows[1])
    assert plan.refined_count() >= 0
    plan.close()


def test_batched_validation():
    wl, params = _workload(8, seed=4)
    x = torch.from_numpy(wl.x).cuda()
    y = torch.from_numpy(wl.y).cuda()
    bad = [dict(p) for p in params]
    bad[1]["max_depth"] = 0
    with pytest.raises(RuntimeError, match="maximum depth"):
        BatchedPointInPolygon(x, y, wl.point_offsets, _polygons(wl), wl.polygon_offsets, bad)
    bad = [dict(p) for p in params]
    bad[2]["x_max"] = bad[2]["x_min"]
    with pytest.raises(RuntimeError, match="invalid bounding box"):
        BatchedPointInPolygon(x, y, wl.point_offsets, _polygons(wl), wl.polygon_offsets, bad)
    with pytest.raises(TypeError):
        BatchedPointInPolygon(x.float(), y.float(), wl.point_offsets, _polygons(wl),
                              wl.polygon_offsets, params)


@pytest.mark.parametrize("method", ["exact", "filtered"])
def test_batched_boundary_points(method):
    """Points on polygon vertices and within 1e-9 of edges (half of them),
    through the ordered-slab index of the batched plan."""
    wl = D.batched_instances(12, points_range=(2000, 8000), polygons_range=(20, 120),
                             side_range=(200.0, 2000.0), vertices_range=(8, 200),
                             seed_offset=7)
    rng = np.random.default_rng(11)
    P = wl.polygons
    x, y = wl.x.copy(), wl.y.copy()
    po = wl.point_offsets.astype(np.int64)
    qo = wl.polygon_offsets.astype(np.int64)
    for i in range(wl.num_instances):
        a, b = po[i], po[i + 1]
        r0, r1 = int(P.part_offset[qo[i]]), int(P.part_offset[qo[i + 1]])
        sub = D.Polygons(P.x, P.y, P.ring_offset[r0:r1 + 1], P.part_offset, P.geometry_offset)
        k = (b - a) // 2
        bx, by = D._near_boundary(rng, sub, k)
        sel = rng.choice(np.arange(a, b), k, replace=False)
        x[sel], y[sel] = bx, by
    wl.x, wl.y = x, y
    params = autotune_free_params(wl)
    plan = BatchedPointInPolygon(torch.from_numpy(wl.x).cuda(), torch.from_numpy(wl.y).cuda(),
                                 wl.point_offsets, _polygons(wl), wl.polygon_offsets, params,
                                 method=method)
    plan.run(graph=True)
    torch.cuda.synchronize()
    # against the plain float64 single-instance calls, whatever the method
    out = _check_plan(plan, wl, params, "exact")
    assert sum(len(o[2][0]) for o in out if o is not None) > 5000
    plan.close()


def autotune_free_params(wl):
    params = []
    for i in range(wl.num_instances):
        x0, x1, y0, y1 = wl.boxes[i]
        params.append(dict(x_min=x0, x_max=x1, y_min=y0, y_max=y1,
                           scale=max(x1 - x0, y1 - y0) / 64.0, max_depth=6, max_size=40))
    return params
