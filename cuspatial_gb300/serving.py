"""Serving form: a device-resident polygon set answering point-in-polygon
requests as they arrive (no counterpart in cuSpatial).

A request is a set of float64 points; its answer is what

    quadtree_on_points(points, params) -> polygon_bounding_boxes(set) ->
    join_quadtree_and_bounding_boxes -> quadtree_point_in_polygon

returns for those points against the whole set (polygon_index into the set,
point_index = position in the request's point_indices).  `request_params`
derives the quadtree parameters from the request alone (its bounding box and
size), so an answer never depends on the other requests it was batched with.

`Server` wraps the native engine (cspt_server_*): requests queue on submit;
worker threads with one CUDA stream each take batches in arrival order while
the estimated device memory of the batches in flight stays within the budget.
`run_poisson` drives a server with a Poisson arrival process and reports
latency percentiles and throughput.
"""

import ctypes
import time

import numpy as np
import torch

from . import _lib
from .autotune import DEFAULT, TuningTable
from .geoseries import GeoSeries, contains_only_polygons

_METHODS = {"exact": _lib.METHOD_EXACT, "filtered": _lib.METHOD_FILTERED}

# quadtree parameters of a request by size (points): upper edge, max_depth, max_size
SERVING_TABLE = TuningTable([{"max_depth": 10, "max_size": 32} for _ in range(7)],
                            meta={"note": "serving defaults"})


def request_params(x, y, table=None):
    """Quadtree parameters of a request from its points alone: a box padded
    around the points, and the max_depth / max_size of its size bucket."""
    table = table or SERVING_TABLE
    n = len(x)
    if n == 0:
        xmin = xmax = ymin = ymax = 0.0
    else:
        xmin, xmax = float(np.min(x)), float(np.max(x))
        ymin, ymax = float(np.min(y)), float(np.max(y))
    mag = max(1.0, abs(xmin), abs(xmax), abs(ymin), abs(ymax))
    pad = 2.0 ** -20 * max(xmax - xmin, ymax - ymin) + 2.0 ** -30 * mag
    box = (xmin - pad, xmax + pad, ymin - pad, ymax + pad)
    c = table.choice(n) if table.buckets else DEFAULT
    d = int(c["max_depth"])
    scale = max(box[1] - box[0], box[3] - box[2]) / (1 << d)
    return {"x_min": box[0], "x_max": box[1], "y_min": box[2], "y_max": box[3],
            "scale": scale, "max_depth": d, "max_size": int(c["max_size"])}


def _params_struct(p):
    return _lib.CsptInstanceParams(float(p["x_min"]), float(p["x_max"]), float(p["y_min"]),
                                   float(p["y_max"]), float(p["scale"]), int(p["max_depth"]),
                                   int(p["max_size"]))


class PolygonSet:
    """Polygons copied to the device once, with their boxes, cell grid and
    point-in-polygon index."""

    def __init__(self, polygons: GeoSeries):
        if not contains_only_polygons(polygons):
            raise ValueError("`polygons` Geoseries must contains only polygons geometries.")
        self._lib = lib = _lib.load()
        poly = polygons.polygons
        if poly.x.dtype != torch.float64:
            raise TypeError("the serving form supports float64 coordinates")
        self._alloc = _lib.TorchAllocator(poly.x.device)
        h = ctypes.c_void_p()
        _lib.check(lib.cspt_polygon_set_create(
            _lib.ptr(poly.part_offset), int(poly.part_offset.numel()), _lib.ptr(poly.ring_offset),
            int(poly.ring_offset.numel()), _lib.ptr(poly.x), _lib.ptr(poly.y),
            int(poly.x.numel()), _lib.FLOAT64, self._alloc.ref, _lib.stream_ptr(),
            ctypes.byref(h)), lib)
        self._h = h
        self.num_polygons = int(poly.part_offset.numel()) - 1

    @property
    def device_bytes(self):
        return self._alloc.in_use

    def close(self):
        if getattr(self, "_h", None) is not None:
            torch.cuda.current_stream().synchronize()
            self._lib.cspt_polygon_set_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass


class Server:
    def __init__(self, polygon_set: PolygonSet, memory_budget_bytes=40 << 30, num_streams=2,
                 max_batch_points=4_000_000, max_batch_requests=512, method="filtered",
                 block_threads=256):
        self._lib = lib = _lib.load()
        self.set = polygon_set
        opt = _lib.CsptServerOptions(int(memory_budget_bytes), int(num_streams),
                                     int(max_batch_points), int(max_batch_requests),
                                     _METHODS[method], int(block_threads))
        h = ctypes.c_void_p()
        _lib.check(lib.cspt_server_create(polygon_set._h, ctypes.byref(opt), ctypes.byref(h)),
                   lib)
        self._h = h
        self._pending = {}  # request id -> host arrays kept alive until completion

    def now(self):
        return self._lib.cspt_server_now(self._h)

    def submit(self, request_id, x, y, params=None):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.ascontiguousarray(y, dtype=np.float64)
        if len(x) != len(y):
            raise RuntimeError("number of points must be the same for both x and y columns")
        params = params or request_params(x, y)
        ps = _params_struct(params)
        _lib.check(self._lib.cspt_server_submit(
            self._h, int(request_id), x.ctypes.data if len(x) else None,
            y.ctypes.data if len(y) else None, len(x), ctypes.byref(ps)), self._lib)
        self._pending[int(request_id)] = (x, y)

    def poll(self, timeout=0.0, max_ids=4096):
        ids = (ctypes.c_uint64 * max_ids)()
        k = self._lib.cspt_server_poll(self._h, ids, max_ids, float(timeout))
        return [int(ids[i]) for i in range(k)]

    def result(self, request_id, release=True):
        r = _lib.CsptRequestResult()
        _lib.check(self._lib.cspt_server_result(self._h, int(request_id), ctypes.byref(r)),
                   self._lib)

        def arr(p, n):
            if not p or n == 0:
                return np.zeros(0, np.uint32)
            return np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_uint32)),
                                         (n,)).copy()

        out = {"status": int(r.status),
               "error": r.error.decode() if r.error else "",
               "polygon_index": arr(r.polygon_index, r.num_rows),
               "point_index": arr(r.point_index, r.num_rows),
               "point_indices": arr(r.point_indices, r.num_points),
               "submit_s": r.submit_s, "admit_s": r.admit_s, "done_s": r.done_s,
               "batch": int(r.batch), "batch_requests": int(r.batch_requests)}
        if release:
            self._lib.cspt_server_release(self._h, int(request_id))
            self._pending.pop(int(request_id), None)
        return out

    def stats(self):
        s = _lib.CsptServerStats()
        _lib.check(self._lib.cspt_server_get_stats(self._h, ctypes.byref(s)), self._lib)
        return {k: getattr(s, k) for k, _ in s._fields_}

    def wait_all(self, ids, timeout=600.0):
        """Waits for the given request ids; returns {id: result}."""
        want = set(int(i) for i in ids)
        got = {}
        t_end = time.perf_counter() + timeout
        while want - set(got):
            if time.perf_counter() > t_end:
                raise TimeoutError("requests did not complete in time")
            for i in self.poll(timeout=0.01):
                got[i] = self.result(i)
        return got

    def close(self):
        if getattr(self, "_h", None) is not None:
            self._lib.cspt_server_free(self._h)
            self._h = None
            self._pending.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def poisson_arrivals(n, rate, seed=0):
    """Arrival times (seconds from 0) of a Poisson process of the given rate."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, n))


def percentile(v, q):
    v = np.sort(np.asarray(v, dtype=np.float64))
    if len(v) == 0:
        return None
    return float(np.quantile(v, q))


def run_poisson(server, requests, rate, params=None, seed=0, keep_results=False):
    """Submits requests at Poisson arrival times and collects them.

    Returns a summary: latency (completion - submission) percentiles in ms,
    queueing (admission - submission), throughput in points/s over the
    span from the first submission to the last completion, batch sizes."""
    params = params or [request_params(r.x, r.y) for r in requests]
    at = poisson_arrivals(len(requests), rate, seed) if rate else np.zeros(len(requests))
    results = {}
    start = time.perf_counter()
    for i, r in enumerate(requests):
        while True:
            wait = at[i] - (time.perf_counter() - start)
            if wait <= 0:
                break
            for j in server.poll(timeout=min(wait, 0.0005)):
                results[j] = server.result(j)
        server.submit(i, r.x, r.y, params[i])
    results.update(server.wait_all([i for i in range(len(requests)) if i not in results]))
    lat = [(results[i]["done_s"] - results[i]["submit_s"]) * 1e3 for i in range(len(requests))]
    que = [(results[i]["admit_s"] - results[i]["submit_s"]) * 1e3 for i in range(len(requests))]
    t0 = min(results[i]["submit_s"] for i in results)
    t1 = max(results[i]["done_s"] for i in results)
    pts = sum(len(r.x) for r in requests)
    batches = {}
    for res in results.values():
        batches[res["batch"]] = res["batch_requests"]
    summary = {
        "requests": len(requests), "points": int(pts),
        "offered_rate_per_s": rate, "span_s": t1 - t0,
        "points_per_s": pts / (t1 - t0) if t1 > t0 else None,
        "requests_per_s": len(requests) / (t1 - t0) if t1 > t0 else None,
        "p50_ms": percentile(lat, 0.5), "p99_ms": percentile(lat, 0.99),
        "max_ms": max(lat) if lat else None,
        "queue_p50_ms": percentile(que, 0.5), "queue_p99_ms": percentile(que, 0.99),
        "batches": len(batches),
        "mean_batch_requests": float(np.mean(list(batches.values()))) if batches else 0.0,
        "failed": sum(1 for r in results.values() if r["status"] != 0),
        "rows": int(sum(len(r["polygon_index"]) for r in results.values())),
    }
    if keep_results:
        summary["results"] = results
    return summary
