"""Autotuner for the batched point-in-polygon join.

Instances are grouped into size buckets by their point count.  For each
bucket the tuner plans and runs a sample batch of synthetic instances of
that size under every candidate (max_depth, max_size) and keeps the fastest;
then it picks the per-pair kernel block size (the tile of pairs one block
evaluates) for the whole batch.  Results are persisted as JSON and read back
by `instance_params`, which turns an instance's point count and box into the
quadtree_on_points arguments.

max_depth and max_size change the tree, hence which (polygon, quadrant)
pairs are generated and in which order rows come out, but never which
(polygon, point) pairs are found: every candidate is a valid reference
parameter set.
"""

import json
import math
import os
import time

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_TABLE = os.path.join(_HERE, "tuning", "batched_pip.json")

# bucket upper edges in points per instance (half-decades from 10^3 to 10^6)
BUCKET_EDGES = [10 ** (3 + 0.5 * k) for k in range(7)]
DEPTHS = (4, 5, 6, 7, 8, 10, 12)
MAX_SIZES = (32, 64, 128, 256, 512, 1024)
BLOCKS = (64, 128, 256)
DEFAULT = {"max_depth": 12, "max_size": 128}


def bucket_of(n_points, edges=BUCKET_EDGES):
    """Index of the bucket holding n_points (the last bucket is open-ended)."""
    for k, e in enumerate(edges):
        if n_points < e:
            return k
    return len(edges) - 1


class TuningTable:
    def __init__(self, buckets=None, block_threads=256, meta=None):
        self.buckets = buckets or [dict(DEFAULT) for _ in BUCKET_EDGES]
        self.block_threads = block_threads
        self.meta = meta or {}

    def choice(self, n_points):
        return self.buckets[bucket_of(n_points)]

    def to_json(self):
        return {"bucket_edges": BUCKET_EDGES, "buckets": self.buckets,
                "block_threads": self.block_threads, "meta": self.meta}

    @classmethod
    def from_json(cls, d):
        if [float(e) for e in d.get("bucket_edges", [])] != [float(e) for e in BUCKET_EDGES]:
            raise ValueError("tuning table was made for other bucket edges")
        return cls([dict(b) for b in d["buckets"]], int(d["block_threads"]), d.get("meta", {}))

    def save(self, path=DEFAULT_TABLE):
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        with open(path, "w") as f:
            json.dump(self.to_json(), f, indent=1, sort_keys=True)
            f.write("\n")

    @classmethod
    def load(cls, path=DEFAULT_TABLE):
        if not os.path.exists(path):
            return cls()
        with open(path) as f:
            return cls.from_json(json.load(f))


def instance_params(n_points, box, table=None):
    """quadtree_on_points arguments for one instance: the bucket's
    max_depth and max_size, and the finest scale the box allows."""
    table = table or TuningTable.load()
    c = table.choice(n_points)
    x_min, x_max, y_min, y_max = (float(v) for v in box)
    d = int(c["max_depth"])
    scale = max(x_max - x_min, y_max - y_min) / (1 << d)
    return {"x_min": x_min, "x_max": x_max, "y_min": y_min, "y_max": y_max,
            "scale": scale, "max_depth": d, "max_size": int(c["max_size"])}


def batch_params(workload, table=None):
    table = table or TuningTable.load()
    po = workload.point_offsets.astype(np.int64)
    return [instance_params(int(po[i + 1] - po[i]), workload.boxes[i], table)
            for i in range(workload.num_instances)]


def _time_once(wl, params, block, method, repeats, objective):
    import torch

    from .batched import BatchedPointInPolygon
    from .geoseries import GeoSeries
    x = torch.from_numpy(wl.x).cuda()
    y = torch.from_numpy(wl.y).cuda()
    p = wl.polygons
    polys = GeoSeries.from_polygons_xy(np.stack([p.x, p.y], 1).reshape(-1), p.ring_offset,
                                       p.part_offset, p.geometry_offset)
    best = math.inf
    for _ in range(repeats):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        plan = BatchedPointInPolygon(x, y, wl.point_offsets, polys, wl.polygon_offsets, params,
                                     method=method, block_threads=block)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        plan.run(graph=True)  # records the graph
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        plan.run(graph=True)
        torch.cuda.synchronize()
        t3 = time.perf_counter()
        step = t3 - t2
        best = min(best, step if objective == "step" else (t1 - t0) + step)
        plan.close()
    return best


def tune(n_instances=48, points_per_bucket=20_000_000, method="filtered", repeats=2,
         depths=DEPTHS, max_sizes=MAX_SIZES, blocks=BLOCKS, seed_offset=100, log=None,
         objective="plan+step"):
    """Measures every candidate per bucket on the current GPU; returns a TuningTable.

    objective "plan+step" times planning plus one evaluation (a batch used
    once); "step" times one evaluation replay (a plan evaluated repeatedly)."""
    import torch

    from . import datasets
    table = TuningTable()
    lo = 10 ** 3
    results = []
    for k, hi in enumerate(BUCKET_EDGES):
        mean = (hi - lo) / max(math.log(hi / lo), 1e-9)
        ni = int(max(4, min(n_instances, points_per_bucket // max(mean, 1))))
        wl = datasets.batched_instances(ni, points_range=(lo, hi), seed_offset=seed_offset + k)
        best = None
        for d in depths:
            for s in max_sizes:
                trial = TuningTable([{"max_depth": d, "max_size": s}] * len(BUCKET_EDGES))
                t = _time_once(wl, batch_params(wl, trial), 256, method, repeats, objective)
                pts = int(wl.point_offsets[-1])
                results.append({"bucket": k, "max_depth": d, "max_size": s, "seconds": t,
                                "points": pts})
                if log:
                    log(f"bucket {k} d={d} s={s}: {t * 1e3:.2f} ms ({pts / t / 1e9:.3f} Gpt/s)")
                if best is None or t < best[0]:
                    best = (t, d, s)
        table.buckets[k] = {"max_depth": best[1], "max_size": best[2]}
        lo = hi
    wl = datasets.batched_instances(n_instances, seed_offset=seed_offset + 50)
    params = batch_params(wl, table)
    block_t = {}
    for b in blocks:
        block_t[b] = _time_once(wl, params, b, method, repeats, objective)
        if log:
            log(f"block {b}: {block_t[b] * 1e3:.2f} ms")
    table.block_threads = min(block_t, key=block_t.get)
    table.meta = {"device": torch.cuda.get_device_name(), "method": method,
                  "objective": objective,
                  "trials": results, "block_seconds": {str(k): v for k, v in block_t.items()}}
    return table


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser(description="tune the batched point-in-polygon join")
    ap.add_argument("--out", default=DEFAULT_TABLE)
    ap.add_argument("--instances", type=int, default=48)
    ap.add_argument("--points-per-bucket", type=int, default=20_000_000)
    ap.add_argument("--repeats", type=int, default=2)
    ap.add_argument("--objective", choices=["plan+step", "step"], default="plan+step")
    a = ap.parse_args()
    t = tune(a.instances, a.points_per_bucket, repeats=a.repeats, log=print,
             objective=a.objective)
    t.save(a.out)
    print(json.dumps({"buckets": t.buckets, "block_threads": t.block_threads}))
