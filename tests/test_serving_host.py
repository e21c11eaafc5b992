"""Host-side parts of the serving form (no GPU): request parameters from the
request alone, arrival process, percentiles, synthetic request shapes."""

import numpy as np

from cuspatial_gb300 import datasets as D
from cuspatial_gb300 import serving as S


def test_request_params_cover_points():
    rng = np.random.default_rng(0)
    for n in (1, 2, 17, 5000):
        x = rng.uniform(-1e4, 1e4, n)
        y = rng.uniform(3.0, 4.0, n)
        p = S.request_params(x, y)
        assert p["x_min"] < x.min() and x.max() < p["x_max"]
        assert p["y_min"] < y.min() and y.max() < p["y_max"]
        assert 1 <= p["max_depth"] <= 15 and p["max_size"] >= 1
        span = max(p["x_max"] - p["x_min"], p["y_max"] - p["y_min"])
        # at or above the reference's minimum scale, so no clamping warning
        assert p["scale"] >= span / ((1 << p["max_depth"]) + 2)


def test_request_params_degenerate():
    # one point, identical points, empty request: the box still has area
    for x, y in ((np.array([5.0]), np.array([7.0])), (np.full(3, 1e6), np.full(3, -2.0)),
                 (np.zeros(0), np.zeros(0))):
        p = S.request_params(x, y)
        assert p["x_min"] < p["x_max"] and p["y_min"] < p["y_max"]


def test_request_params_depend_on_request_only():
    r = D.serving_requests(3, points_range=(10, 100), extent=100.0)
    a = S.request_params(r[0].x, r[0].y)
    b = S.request_params(r[0].x.copy(), r[0].y.copy())
    assert a == b


def test_poisson_arrivals():
    t = S.poisson_arrivals(20000, 2000.0, seed=1)
    assert np.all(np.diff(t) > 0)
    assert abs(len(t) / t[-1] - 2000.0) < 60.0
    assert S.percentile([1, 2, 3, 4], 0.5) == 2.5
    assert S.percentile([], 0.5) is None


def test_serving_workload_shapes():
    P = D.serving_polygons(grid=20, extent=800.0)
    assert P.num_polygons == 400
    k = np.diff(P.ring_offset) - 1
    assert k.min() >= 8 and k.max() <= 256
    reqs = D.serving_requests(50, points_range=(1, 1000), extent=800.0)
    sizes = np.array([len(r.x) for r in reqs])
    assert sizes.min() >= 1 and sizes.max() <= 1000
    assert {r.kind for r in reqs} == {"uniform", "cluster"}
    for r in reqs:
        assert np.all((r.x >= 0) & (r.x < 800.0) & (r.y >= 0) & (r.y < 800.0))
