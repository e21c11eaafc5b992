"""Benchmark: quadtree point-in-polygon join throughput on one GB300.

Workload (default): 100,000,000 float64 points from a 64-component Gaussian
mixture (1% on polygon vertices or within 1e-9 of an edge) and 100,000
star-shaped polygons with 8-512 vertices, 10% with a hole; max_depth 15,
max_size 256 (cuspatial_gb300.datasets.precision_at_scale).

A step is one pass of the join over the resident point set:
polygon_bounding_boxes + join_quadtree_and_bounding_boxes +
quadtree_point_in_polygon (float32 filter + float64 refine).  The quadtree is
built once and reported separately (build_ms).  value = points / step time;
e2e repeats the whole chain through the public API from pinned host buffers
(host->device copies, quadtree build, join, device->host copy of the pairs).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("PiP join points/s: FP32-filter+FP64-refine vs plain FP64, exact pairs; p99 ms")


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--points", type=int, default=100_000_000)
    ap.add_argument("--polygons", type=int, default=100_000)
    ap.add_argument("--method", choices=["filtered", "exact"], default="filtered")
    ap.add_argument("--plain-steps", type=int, default=3)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-seconds", type=float, default=15.0,
                    help="target CPU time of the oracle baseline sample")
    ap.add_argument("--no-cpu", action="store_true")
    return ap.parse_args()


# --------------------------------------------------------------------------
# distributed plumbing: replicas only (the join has no exchange step)
# --------------------------------------------------------------------------
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None

    def init(self, backend):
        import torch.distributed as td
        if self.world > 1 and not td.is_initialized():
            td.init_process_group(backend=backend)
            self.pg = td

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v):
        if not self.pg:
            return v
        import torch
        t = torch.tensor([float(v)], device="cuda" if torch.cuda.is_available() else "cpu")
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())


# --------------------------------------------------------------------------
# clocks during the timed region
# --------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            import tempfile
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [c.strip() for c in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower() in ("active", "1", "yes"):
                    reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "power_w_max": max(power) if power else None, "samples": len(sm),
                "reasons": sorted(reasons)}


def percentile(v, q):
    v = sorted(v)
    k = (len(v) - 1) * q
    lo, hi = int(np.floor(k)), int(np.ceil(k))
    return v[lo] + (v[hi] - v[lo]) * (k - lo)


def measured_peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def make_workload(args):
    from cuspatial_gb300 import datasets as D
    return D.precision_at_scale(n_points=args.points, n_polygons=args.polygons)


def polygons_xy(P):
    xy = np.empty(2 * len(P.x))
    xy[0::2] = P.x
    xy[1::2] = P.y
    return xy


# --------------------------------------------------------------------------
# CPU oracle baseline on a polygon sample (and an at-scale parity check)
# --------------------------------------------------------------------------
def cpu_baseline(w, tree_np, pi_np, pairs_np, gpu_pip, target_s):
    from oracle import oracle as O
    P = w.polygons
    npoly = P.num_polygons
    qlen = tree_np["length"].astype(np.int64)
    cand_total = int(qlen[pairs_np["quad_offset"]].sum())
    # size the sample from a small probe: every stride-th polygon
    stride = max(1, npoly // 50)
    tried = []
    bb = O.polygon_bounding_boxes(P.part_offset, P.ring_offset, P.x, P.y)
    while True:
        sel = np.arange(0, npoly, stride)
        sbb = {k: np.ascontiguousarray(v[sel]) for k, v in bb.items()}
        t0 = time.perf_counter()
        sj = O.join_quadtree_and_bounding_boxes(tree_np, sbb, w.x_min, w.x_max, w.y_min, w.y_max,
                                                w.scale, w.max_depth)
        t1 = time.perf_counter()
        sj = dict(bbox_offset=sel[sj["bbox_offset"]].astype(np.uint32),
                  quad_offset=sj["quad_offset"])
        r = O.quadtree_point_in_polygon(sj, tree_np, pi_np, w.x, w.y, P.part_offset,
                                        P.ring_offset, P.x, P.y)
        t2 = time.perf_counter()
        tried.append((stride, t2 - t0))
        if t2 - t0 >= target_s / 4 or stride == 1:
            break
        stride = max(1, int(stride * (t2 - t0) / target_s))
        if stride == tried[-1][0]:
            break
    cand_s = int(qlen[sj["quad_offset"]].sum())
    t_join_full = (t1 - t0) * npoly / len(sel)
    t_pip_full = (t2 - t1) * cand_total / max(cand_s, 1)
    value = len(w.x) / (t_join_full + t_pip_full)
    # parity at scale: the GPU pairs of the sampled polygons, in order
    gp = gpu_pip["polygon_index"]
    keep = np.isin(gp, sel)
    parity = bool(np.array_equal(gp[keep], r["polygon_index"]) and
                  np.array_equal(gpu_pip["point_index"][keep], r["point_index"]))
    return {
        "value": value, "unit": "points/s", "cores": O.num_threads(), "kind": "port",
        "sample": ("every %d-th polygon (%d of %d, %.2f%% of candidates), full %d-point set; "
                   "oracle join %.2fs + PiP %.2fs scaled by polygons/candidates" %
                   (stride, len(sel), npoly, 100.0 * cand_s / max(cand_total, 1), len(w.x),
                    t1 - t0, t2 - t1)),
        "sample_pairs": int(len(r["polygon_index"])),
        "sample_parity_exact": parity,
    }


# --------------------------------------------------------------------------
# our arm
# --------------------------------------------------------------------------
def run_ours(args, dist):
    import torch

    import cuspatial_gb300 as cs
    from cuspatial_gb300 import _lib

    torch.cuda.set_device(dist.local)
    dist.init("nccl")
    lib = _lib.load()
    lib.cspt_launch_count.restype = ctypes.c_uint64
    lib.cspt_profile_read.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_double),
                                      ctypes.POINTER(ctypes.c_uint64)]
    lib.cspt_profile_enable.argtypes = [ctypes.c_int]

    t0 = time.time()
    w = make_workload(args)
    gen_s = time.time() - t0
    P = w.polygons
    n = len(w.x)
    pts = cs.GeoSeries.from_points(w.x, w.y)
    polys = cs.GeoSeries.from_polygons_xy(polygons_xy(P), P.ring_offset, P.part_offset,
                                          P.geometry_offset)
    stream = torch.cuda.current_stream()
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731

    # quadtree build (reported separately)
    build_ms = []
    for _ in range(3):
        a, b = ev(), ev()
        a.record(stream)
        pi, tree = cs.quadtree_on_points(pts, w.x_min, w.x_max, w.y_min, w.y_max, w.scale,
                                         w.max_depth, w.max_size)
        b.record(stream)
        b.synchronize()
        build_ms.append(a.elapsed_time(b))

    def step(method):
        bb = cs.polygon_bounding_boxes(polys)
        pairs = cs.join_quadtree_and_bounding_boxes(tree, bb, w.x_min, w.x_max, w.y_min,
                                                    w.y_max, w.scale, w.max_depth)
        res = cs.quadtree_point_in_polygon(pairs, tree, pi, pts, polys, method=method)
        return pairs, res

    for _ in range(args.warmup):
        pairs, res = step(args.method)
    torch.cuda.synchronize()

    # timed region
    clocks = ClockSampler(dist.local)
    clocks.start()
    lib.cspt_profile_enable(1)
    launches0 = lib.cspt_launch_count()
    dist.barrier()
    torch.cuda.synchronize()
    times = []
    g0, g1 = ev(), ev()
    g0.record(stream)
    for _ in range(args.steps):
        a, b = ev(), ev()
        a.record(stream)
        pairs, res = step(args.method)
        b.record(stream)
        times.append((a, b))
    g1.record(stream)
    torch.cuda.synchronize()
    dist.barrier()
    launches = int(lib.cspt_launch_count() - launches0)
    clock_info = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in times]
    total_ms = dist.max(g0.elapsed_time(g1))
    kern = {}
    for name in ("pip_bits", "pip_expand", "join_count", "join_write", "leaf_frames",
                 "polygon_index"):
        ms, cnt = ctypes.c_double(), ctypes.c_uint64()
        lib.cspt_profile_read(name.encode(), ctypes.byref(ms), ctypes.byref(cnt))
        kern[name] = (ms.value, int(cnt.value))
    lib.cspt_profile_enable(0)
    refined = cs.last_refined_count()

    ms_per_step = total_ms / args.steps
    value = n * args.gpus / (ms_per_step / 1e3)

    # plain float64 method for comparison (same pairs, identical output)
    plain = None
    if args.plain_steps > 0 and args.method == "filtered":
        pp, pr = step("exact")
        torch.cuda.synchronize()
        same = bool(torch.equal(pr["polygon_index"], res["polygon_index"]) and
                    torch.equal(pr["point_index"], res["point_index"]))
        pms = []
        for _ in range(args.plain_steps):
            a, b = ev(), ev()
            a.record(stream)
            step("exact")
            b.record(stream)
            b.synchronize()
            pms.append(a.elapsed_time(b))
        plain = {"points_per_s": n / (statistics.mean(pms) / 1e3),
                 "ms_per_step": statistics.mean(pms), "pairs_identical_to_filtered": same}

    # roofline of the dominant kernel (pip_bits)
    K = int(pairs["bbox_offset"].numel())
    M = int(res["polygon_index"].numel())
    qlen = tree["length"].long()
    cand = int(qlen[pairs["quad_offset"].long()].sum().item())
    words = int(((qlen[pairs["quad_offset"].long()] + 31) // 32).sum().item())
    V = len(P.x)
    bits_ms, bits_n = kern["pip_bits"]
    alg_bytes = 20 * n + 16 * V + 8 * K + 4 * K + 4 * words
    peak, peak_kind = measured_peak_hbm()
    achieved = alg_bytes / (bits_ms / max(bits_n, 1) / 1e3) / 1e9 if bits_n else None
    roofline = {"bound": "hbm", "kernel": "pip_bits_kernel", "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": (achieved / peak) if achieved else None,
                "peak_source": peak_kind, "traffic": None,
                "algorithmic_bytes_per_launch": alg_bytes,
                "kernel_ms_per_launch": bits_ms / max(bits_n, 1),
                "note": "traffic from ncu is recorded in profiles/"}

    # end to end through the public API from pinned host buffers
    e2e = None
    if args.e2e_steps > 0:
        hx = torch.from_numpy(w.x).pin_memory()
        hy = torch.from_numpy(w.y).pin_memory()
        hpxy = torch.from_numpy(polygons_xy(P)).pin_memory()
        hro = torch.from_numpy(P.ring_offset).pin_memory()
        hpo = torch.from_numpy(P.part_offset).pin_memory()
        hgo = torch.from_numpy(P.geometry_offset).pin_memory()
        ems, h2d, d2h = [], 0, 0
        for it in range(args.e2e_steps + 1):
            a, b = ev(), ev()
            a.record(stream)
            dx = hx.to("cuda", non_blocking=True)
            dy = hy.to("cuda", non_blocking=True)
            dxy = hpxy.to("cuda", non_blocking=True)
            epts = cs.GeoSeries.from_points(dx, dy)
            epolys = cs.GeoSeries.from_polygons_xy(dxy, hro.to("cuda", non_blocking=True),
                                                   hpo.to("cuda", non_blocking=True),
                                                   hgo.to("cuda", non_blocking=True))
            epi, etree = cs.quadtree_on_points(epts, w.x_min, w.x_max, w.y_min, w.y_max, w.scale,
                                               w.max_depth, w.max_size)
            ebb = cs.polygon_bounding_boxes(epolys)
            ej = cs.join_quadtree_and_bounding_boxes(etree, ebb, w.x_min, w.x_max, w.y_min,
                                                     w.y_max, w.scale, w.max_depth)
            er = cs.quadtree_point_in_polygon(ej, etree, epi, epts, epolys, method=args.method)
            o1 = torch.empty(er["polygon_index"].shape, dtype=torch.int32, pin_memory=True)
            o2 = torch.empty(er["point_index"].shape, dtype=torch.int32, pin_memory=True)
            o1.copy_(er["polygon_index"], non_blocking=True)
            o2.copy_(er["point_index"], non_blocking=True)
            b.record(stream)
            b.synchronize()
            if it > 0:  # first pass warms the allocator
                ems.append(a.elapsed_time(b))
            h2d = (hx.numel() + hy.numel() + hpxy.numel()) * 8 + (hro.numel() + hpo.numel() +
                                                                   hgo.numel()) * 4
            d2h = (o1.numel() + o2.numel()) * 4
        e2e_ms = dist.max(statistics.mean(ems))
        e2e = {"value": n * args.gpus / (e2e_ms / 1e3), "unit": "points/s",
               "ms_per_step": e2e_ms, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h),
               "pairs_identical": bool(torch.equal(er["polygon_index"], res["polygon_index"]))}

    cpu = None
    if dist.rank == 0 and args.gpus == 1 and not args.no_cpu:
        tree_np = {k: (v.cpu().numpy().view(np.uint32) if v.dtype == torch.int32 else
                       v.cpu().numpy()) for k, v in tree.items()}
        tree_np["is_internal_node"] = tree_np["is_internal_node"].astype(bool)
        pairs_np = {k: v.cpu().numpy().view(np.uint32) for k, v in pairs.items()}
        gpu_pip = {k: v.cpu().numpy().view(np.uint32) for k, v in res.items()}
        cpu = cpu_baseline(w, tree_np, pi.cpu().numpy().view(np.uint32), pairs_np, gpu_pip,
                           args.cpu_seconds)

    line = {
        "metric": METRIC, "value": value, "unit": "points/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "p50_ms": percentile(step_ms, 0.5), "p99_ms": percentile(step_ms, 0.99),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded numpy PCG64; shapes of the 100M-point precision config)",
        "config": {"workload": "precision_at_scale: 100M Gaussian-mixture points, 100k star "
                               "polygons (8-512 vertices, 10% holed), max_depth 15, "
                               "max_size 256" if args.points == 100_000_000 else
                   "precision_at_scale scaled to %d points / %d polygons" % (n, P.num_polygons),
                   "points": n, "polygons": P.num_polygons, "vertices": V,
                   "method": args.method, "step": "polygon_bounding_boxes + "
                   "join_quadtree_and_bounding_boxes + quadtree_point_in_polygon",
                   "l2": "inputs larger than L2 (%.1f GB of points resident)" % (16 * n / 1e9),
                   "parallelism": "replicas" if args.gpus > 1 else "single GPU"},
        "pairs": K, "candidates": cand, "hits": M,
        "refined_candidates": refined, "refine_fraction": refined / max(cand, 1),
        "build_ms": min(build_ms), "generation_s": gen_s,
        "kernels_ms_per_step": {k: v[0] / max(args.steps, 1) for k, v in kern.items()},
        "plain_fp64": plain,
        "speedup_vs_plain": (plain["ms_per_step"] / ms_per_step) if plain else None,
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
        "clocks": clock_info,
    }
    if dist.rank == 0:
        print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------
# reference arm: the oracle port on the host cores (the reference has no CPU
# implementation and its GPU build needs rmm and libcudf, which are absent)
# --------------------------------------------------------------------------
def run_reference(args, dist):
    if dist.rank != 0:
        return
    from oracle import oracle as O
    w = make_workload(args)
    P = w.polygons
    n = len(w.x)
    t0 = time.perf_counter()
    pi, tree = O.quadtree_on_points(w.x, w.y, w.x_min, w.x_max, w.y_min, w.y_max, w.scale,
                                    w.max_depth, w.max_size)
    build_s = time.perf_counter() - t0
    bb = O.polygon_bounding_boxes(P.part_offset, P.ring_offset, P.x, P.y)
    npoly = P.num_polygons
    qlen = tree["length"].astype(np.int64)
    # per step: every stride-th polygon, offset by the step number
    stride = max(1, npoly // 200)
    times, cand_frac = [], []
    full = O.join_quadtree_and_bounding_boxes(tree, bb, w.x_min, w.x_max, w.y_min, w.y_max,
                                              w.scale, w.max_depth)
    cand_total = int(qlen[full["quad_offset"]].sum())
    for it in range(args.warmup + args.steps):
        sel = np.arange(it % stride, npoly, stride)
        sbb = {k: np.ascontiguousarray(v[sel]) for k, v in bb.items()}
        t0 = time.perf_counter()
        sj = O.join_quadtree_and_bounding_boxes(tree, sbb, w.x_min, w.x_max, w.y_min, w.y_max,
                                                w.scale, w.max_depth)
        t1 = time.perf_counter()
        sj = dict(bbox_offset=sel[sj["bbox_offset"]].astype(np.uint32),
                  quad_offset=sj["quad_offset"])
        O.quadtree_point_in_polygon(sj, tree, pi, w.x, w.y, P.part_offset, P.ring_offset, P.x,
                                    P.y)
        t2 = time.perf_counter()
        if it >= args.warmup:
            cs_ = int(qlen[sj["quad_offset"]].sum())
            times.append((t1 - t0) * npoly / len(sel) + (t2 - t1) * cand_total / max(cs_, 1))
            cand_frac.append(cs_ / max(cand_total, 1))
    s_per_step = statistics.mean(times)
    value = n / s_per_step
    sample = ("per step every %d-th polygon (%.2f%% of candidates), full %d-point set; time "
              "scaled to the full join" % (stride, 100 * statistics.mean(cand_frac), n))
    line = {
        "metric": METRIC, "impl": "reference", "value": value, "unit": "points/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": s_per_step * 1e3, "p50_ms": percentile([t * 1e3 for t in times], 0.5),
        "p99_ms": percentile([t * 1e3 for t in times], 0.99), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "precision_at_scale", "points": n, "polygons": npoly,
                   "method": "reference crossing test (CPU oracle port)"},
        "cpu_baseline": {"value": value, "unit": "points/s", "cores": O.num_threads(),
                         "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "points/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "build_s": build_s,
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    dist = Dist()
    if args.impl == "reference":
        run_reference(args, dist)
    else:
        run_ours(args, dist)


if __name__ == "__main__":
    main()
