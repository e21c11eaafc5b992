"""Serving form: every request's answer equals the single-instance calls
against the whole polygon set, and is the same alone and in a mix of
concurrent requests; admission by memory budget and per-request failures."""

import numpy as np
import pytest

import cuspatial_gb300 as cs
from cuspatial_gb300 import datasets as D
from cuspatial_gb300.serving import PolygonSet, Server, request_params, run_poisson
from oracle import oracle as O

from helpers import gpu_polygons, u32

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def polys():
    # 40 x 40 polygons over [0, 2000)^2: the serving shape at 1/156 scale
    P = D.serving_polygons(grid=40, extent=2000.0, vertices_range=(3, 60),
                           radius_range=(1.0, 40.0))
    return P


def _requests(n, seed):
    return D.serving_requests(n, points_range=(1, 4000), extent=2000.0, seed_offset=seed)


def _single(P, gpolys, r, p, method):
    """The drop-in pipeline for one request against the whole set."""
    pts = cs.GeoSeries.from_points(r.x, r.y)
    pi, tree = cs.quadtree_on_points(pts, p["x_min"], p["x_max"], p["y_min"], p["y_max"],
                                     p["scale"], p["max_depth"], p["max_size"])
    boxes = cs.polygon_bounding_boxes(gpolys)
    pairs = cs.join_quadtree_and_bounding_boxes(tree, boxes, p["x_min"], p["x_max"],
                                                p["y_min"], p["y_max"], p["scale"],
                                                p["max_depth"])
    res = cs.quadtree_point_in_polygon(pairs, tree, pi, pts, gpolys, method=method)
    return u32(pi), u32(res["polygon_index"]), u32(res["point_index"])


@pytest.mark.parametrize("method", ["exact", "filtered"])
def test_serving_matches_single_instance_calls(polys, method):
    gp = gpu_polygons(polys)
    pset = PolygonSet(gp)
    reqs = _requests(24, seed=1)
    params = [request_params(r.x, r.y) for r in reqs]
    with Server(pset, num_streams=2, method=method) as srv:
        for i, r in enumerate(reqs):
            srv.submit(i, r.x, r.y, params[i])
        got = srv.wait_all(range(len(reqs)))
    rows = 0
    for i, r in enumerate(reqs):
        pi, pp, pq = _single(polys, gp, r, params[i], method)
        g = got[i]
        assert g["status"] == 0, g["error"]
        np.testing.assert_array_equal(g["point_indices"], pi, err_msg=f"pi {i}")
        np.testing.assert_array_equal(g["polygon_index"], pp, err_msg=f"polygon_index {i}")
        np.testing.assert_array_equal(g["point_index"], pq, err_msg=f"point_index {i}")
        rows += len(pp)
    assert rows > 200
    pset.close()


def test_serving_alone_equals_mix(polys):
    gp = gpu_polygons(polys)
    pset = PolygonSet(gp)
    reqs = _requests(60, seed=2)
    params = [request_params(r.x, r.y) for r in reqs]
    alone = {}
    with Server(pset, num_streams=1, max_batch_requests=1) as srv:
        for i, r in enumerate(reqs):
            srv.submit(i, r.x, r.y, params[i])
            alone[i] = srv.wait_all([i])[i]
            assert alone[i]["batch_requests"] == 1
    # the mix: three streams, Poisson arrivals faster than a batch takes,
    # and a budget of a few requests so that admission has to wait
    with Server(pset, num_streams=3, memory_budget_bytes=24 << 20) as srv:
        s = run_poisson(srv, reqs, rate=20000.0, params=params, seed=5, keep_results=True)
        st = srv.stats()
    mixed = s["results"]
    assert s["failed"] == 0
    assert max(r["batch_requests"] for r in mixed.values()) > 1
    assert st["peak_device_bytes"] <= 24 << 20
    for i in range(len(reqs)):
        for k in ("polygon_index", "point_index", "point_indices"):
            np.testing.assert_array_equal(mixed[i][k], alone[i][k], err_msg=f"{k} {i}")
    pset.close()


def test_serving_against_oracle(polys):
    gp = gpu_polygons(polys)
    pset = PolygonSet(gp)
    reqs = _requests(6, seed=3)
    with Server(pset) as srv:
        for i, r in enumerate(reqs):
            srv.submit(i, r.x, r.y)
        got = srv.wait_all(range(len(reqs)))
    bb = O.polygon_bounding_boxes(polys.part_offset, polys.ring_offset, polys.x, polys.y)
    for i, r in enumerate(reqs):
        p = request_params(r.x, r.y)
        opi, otree = O.quadtree_on_points(r.x, r.y, p["x_min"], p["x_max"], p["y_min"],
                                          p["y_max"], p["scale"], p["max_depth"],
                                          p["max_size"])
        pairs = O.join_quadtree_and_bounding_boxes(otree, bb, p["x_min"], p["x_max"],
                                                   p["y_min"], p["y_max"], p["scale"],
                                                   p["max_depth"])
        res = O.quadtree_point_in_polygon(pairs, otree, opi, r.x, r.y, polys.part_offset,
                                          polys.ring_offset, polys.x, polys.y)
        np.testing.assert_array_equal(got[i]["point_indices"], opi)
        np.testing.assert_array_equal(got[i]["polygon_index"], res["polygon_index"])
        np.testing.assert_array_equal(got[i]["point_index"], res["point_index"])
    pset.close()


def test_serving_failures_stay_per_request(polys):
    gp = gpu_polygons(polys)
    pset = PolygonSet(gp)
    reqs = _requests(8, seed=4)
    with Server(pset, memory_budget_bytes=8 << 20) as srv:
        # invalid parameters are refused at submit, as the join refuses them
        bad = dict(request_params(reqs[0].x, reqs[0].y))
        bad["x_max"] = bad["x_min"]
        with pytest.raises(RuntimeError, match="invalid bounding box"):
            srv.submit(100, reqs[0].x, reqs[0].y, bad)
        # a request above the budget fails alone; the others complete
        big = np.random.default_rng(0).uniform(0, 2000, 200_000)
        srv.submit(101, big, big[::-1].copy())
        for i, r in enumerate(reqs):
            srv.submit(i, r.x, r.y)
        got = srv.wait_all(list(range(len(reqs))) + [101])
    assert got[101]["status"] != 0 and "memory budget" in got[101]["error"]
    assert all(got[i]["status"] == 0 for i in range(len(reqs)))
    # an empty request answers with no rows
    with Server(pset) as srv:
        srv.submit(7, np.zeros(0), np.zeros(0))
        e = srv.wait_all([7])[7]
    assert e["status"] == 0 and len(e["polygon_index"]) == 0
    pset.close()
