"""Benchmark: quadtree point-in-polygon join throughput on one GB300.

Workload (default): 100,000,000 float64 points from a 64-component Gaussian
mixture (1% on polygon vertices or within 1e-9 of an edge) and 100,000
star-shaped polygons with 8-512 vertices, 10% with a hole; max_depth 15,
max_size 256 (cuspatial_gb300.datasets.precision_at_scale).

A step is one pass of the join over the resident point set:
polygon_bounding_boxes + join_quadtree_and_bounding_boxes +
quadtree_point_in_polygon (float32 filter + float64 refine).  The quadtree and
the points in its order are built once and reported separately (build_ms).
value = points / step time; e2e repeats the whole chain through the public
API from pinned host buffers (host->device copies, quadtree build, join,
device->host copy of the pairs), beside the host link's measured rates.

The default run also measures the other configurations at their shapes
(other_configs: the 1M-point plain drop-in case against the CPU oracle in
full, the nearest-linestring join, the serving loop and the batched form),
each a short run; --no-configs skips them, --workload runs one alone.

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
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--points", type=int, default=100_000_000)
    ap.add_argument("--polygons", type=int, default=100_000)
    ap.add_argument("--method", choices=["filtered", "exact"], default="filtered")
    ap.add_argument("--plain-steps", type=int, default=3)
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the other configurations' sub-results in the default run")
    ap.add_argument("--workload", choices=["precision", "batched", "serving", "nearest",
                                           "unindexed"],
                    default="precision",
                    help="precision: the 100M-point join (default line); batched: 4096 "
                         "independent instances through the batched plan; serving: Poisson "
                         "requests against a resident 250k-polygon set; nearest: 50M points "
                         "to 200k linestrings; unindexed: 10M points against 31 polygons "
                         "without an index (the reference's point_in_polygon benchmark)")
    ap.add_argument("--requests", type=int, default=4000)
    ap.add_argument("--rate", type=float, default=2000.0)
    ap.add_argument("--streams", type=int, default=4)
    ap.add_argument("--nearest-points", type=int, default=50_000_000)
    ap.add_argument("--nearest-linestrings", type=int, default=200_000)
    ap.add_argument("--nearest-extent", type=float, default=10000.0,
                    help="side of the nearest-linestring domain (a smaller side with "
                         "proportionally fewer points and linestrings keeps the density)")
    ap.add_argument("--nearest-plain-every", type=int, default=64,
                    help="time the plain float64 nearest method on every k-th leaf "
                         "(0: skip)")
    ap.add_argument("--instances", type=int, default=4096)
    ap.add_argument("--sides", type=int, default=100,
                    help="polygon sides of the unindexed workload (reference: 4, 10, 100)")
    ap.add_argument("--unindexed-points", type=int, default=10_000_000)
    ap.add_argument("--single-sample", type=int, default=64,
                    help="instances timed through the single-instance calls (batched)")
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
# host link: where the GPU and the page-locked buffers sit, and what one
# plain copy of 1 GiB each way sustains (the e2e leg's copies are bounded by
# it)
# --------------------------------------------------------------------------
def gpu_numa(device_index):
    """NUMA node and local CPUs of the GPU's PCI device (Linux sysfs)."""
    import torch
    info = {}
    try:
        bus = torch.cuda.get_device_properties(device_index).pci_bus_id.lower()
    except Exception:  # noqa: BLE001 - older torch: no bus id
        return info
    for dom in (bus, bus.replace("00000000:", "0000:")):
        base = "/sys/bus/pci/devices/" + dom
        if os.path.isdir(base):
            for k in ("numa_node", "local_cpulist"):
                try:
                    info[k] = open(os.path.join(base, k)).read().strip()
                except OSError:
                    pass
            info["pci_bus_id"] = dom
            break
    return info


def pages_by_node(ptr, nbytes):
    """Resident pages of [ptr, ptr + nbytes) per NUMA node, from
    /proc/self/numa_maps of the mapping that holds ptr."""
    try:
        start = None
        for line in open("/proc/self/maps"):
            lo, hi = (int(v, 16) for v in line.split()[0].split("-"))
            if lo <= ptr < hi:
                start = lo
                break
        if start is None:
            return None
        for line in open("/proc/self/numa_maps"):
            f = line.split()
            if int(f[0], 16) == start:
                return {kv.split("=")[0]: int(kv.split("=")[1]) for kv in f[1:]
                        if kv.startswith("N") and "=" in kv}
    except (OSError, ValueError):
        return None
    return None


def measure_link(stream, nbytes=1 << 30, reps=3):
    """GB/s of one cudaMemcpyAsync of nbytes from page-locked host memory to
    the device and back, best of reps, with the pages' NUMA placement."""
    import torch
    h = torch.empty(nbytes // 8, dtype=torch.float64).pin_memory()
    h.fill_(1.0)
    d = torch.empty_like(h, device="cuda")
    out = {"bytes": nbytes, "host_pages_by_node": pages_by_node(h.data_ptr(), nbytes)}
    for name, dst, src in (("h2d_gbs", d, h), ("d2h_gbs", h, d)):
        best = None
        for _ in range(reps):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            dst.copy_(src, non_blocking=True)
            b.record(stream)
            b.synchronize()
            ms = a.elapsed_time(b)
            best = ms if best is None else min(best, ms)
        out[name] = nbytes / (best / 1e3) / 1e9
    del d, h
    return out


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
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        # the timed region starts once the sampler is producing rows
        t_end = time.time() + 5.0
        while time.time() < t_end and self.proc.poll() is None:
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.01)

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


TRAFFIC_PROFILE = "profiles/pip_pair_kernel_dram_precision_100M.md"


def recorded_traffic(args):
    """DRAM bytes per PiP launch from the committed ncu summary of the default
    workload (100M points, 100k polygons, filtered); None for other runs."""
    if args.points != 100_000_000 or args.polygons != 100_000 or args.method != "filtered":
        return None
    try:
        for line in open(os.path.join(ROOT, TRAFFIC_PROFILE)):
            if line.startswith("traffic_bytes_per_launch:"):
                return int(line.split(":")[1])
    except OSError:
        return None
    return None


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
# One sampling rule for both arms: the polygons i with i % CPU_STRIDE == offset
# (5% of them) against the full point set.  The sample's wall time is
# measured; the full join's time is estimated by scaling the join by the
# polygon fraction and the point-in-polygon tests by the candidate fraction.
CPU_STRIDE = 20


def cpu_sample(O, w, tree_np, pi_np, bb, qlen, cand_total, offset):
    P = w.polygons
    npoly = P.num_polygons
    sel = np.arange(offset % CPU_STRIDE, npoly, CPU_STRIDE)
    sbb = {k: np.ascontiguousarray(v[sel]) for k, v in bb.items()}
    t0 = time.perf_counter()
    sj = O.join_quadtree_and_bounding_boxes(tree_np, sbb, w.x_min, w.x_max, w.y_min, w.y_max,
                                            w.scale, w.max_depth)
    t1 = time.perf_counter()
    sj = dict(bbox_offset=sel[sj["bbox_offset"]].astype(np.uint32), quad_offset=sj["quad_offset"])
    r = O.quadtree_point_in_polygon(sj, tree_np, pi_np, w.x, w.y, P.part_offset, P.ring_offset,
                                    P.x, P.y)
    t2 = time.perf_counter()
    cand_s = int(qlen[sj["quad_offset"]].sum())
    full_s = (t1 - t0) * npoly / len(sel) + (t2 - t1) * cand_total / max(cand_s, 1)
    return {"sel": sel, "rows": r, "sample_s": t2 - t0, "full_s": full_s,
            "cand_fraction": cand_s / max(cand_total, 1), "polygons": len(sel),
            "value": len(w.x) / full_s}


def cpu_sample_text(res, n):
    return ("polygons i with i %% %d == offset (%d of %d, %.2f%% of candidates) against all "
            "%d points; sampled wall time %.2f s, scaled to the full join (join by polygons, "
            "point-in-polygon by candidates) %.1f s" %
            (CPU_STRIDE, res["polygons"], res["polygons"] * CPU_STRIDE, 100 * res["cand_fraction"],
             n, res["sample_s"], res["full_s"]))


# --------------------------------------------------------------------------
# CPU oracle baseline on a polygon sample (and an at-scale parity check)
# --------------------------------------------------------------------------
def cpu_baseline(w, tree_np, pi_np, pairs_np, gpu_pip):
    from oracle import oracle as O
    P = w.polygons
    qlen = tree_np["length"].astype(np.int64)
    cand_total = int(qlen[pairs_np["quad_offset"]].sum())
    bb = O.polygon_bounding_boxes(P.part_offset, P.ring_offset, P.x, P.y)
    res = cpu_sample(O, w, tree_np, pi_np, bb, qlen, cand_total, 0)
    r = res["rows"]
    # parity at scale: the GPU pairs of the sampled polygons, in order
    gp = gpu_pip["polygon_index"]
    keep = np.isin(gp, res["sel"])
    parity = bool(np.array_equal(gp[keep], r["polygon_index"]) and
                  np.array_equal(gpu_pip["point_index"][keep], r["point_index"]))
    return {
        "value": res["value"], "unit": "points/s", "cores": O.num_threads(), "kind": "port",
        "sample": cpu_sample_text(res, len(w.x)), "sample_s": res["sample_s"],
        "scale_to_full": res["full_s"] / res["sample_s"],
        "sample_pairs": int(len(r["polygon_index"])), "sample_parity_exact": parity,
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

    # point index build (reported separately): the quadtree and the points
    # in its order, built together; the tree alone for comparison
    build_ms, tree_ms = [], []
    for _ in range(3):
        a, b, c = ev(), ev(), ev()
        a.record(stream)
        pi, tree, xy = cs.quadtree_on_points_ordered(pts, w.x_min, w.x_max, w.y_min, w.y_max,
                                                     w.scale, w.max_depth, w.max_size)
        b.record(stream)
        cs.quadtree_on_points(pts, w.x_min, w.x_max, w.y_min, w.y_max, w.scale, w.max_depth,
                              w.max_size)
        c.record(stream)
        c.synchronize()
        build_ms.append(a.elapsed_time(b))
        tree_ms.append(b.elapsed_time(c))

    def step(method):
        bb = cs.polygon_bounding_boxes(polys)
        pairs = cs.join_quadtree_and_bounding_boxes(tree, bb, w.x_min, w.x_max, w.y_min,
                                                    w.y_max, w.scale, w.max_depth)
        res = cs.quadtree_point_in_polygon(pairs, tree, pi, pts, polys, method=method,
                                           ordered_points=xy)
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
    edge_free = cs.last_edge_free_pairs()

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
    traffic, traffic_src = recorded_traffic(args), None
    if traffic is not None:
        traffic_src = "ncu capture of this workload, " + TRAFFIC_PROFILE
    roofline = {"bound": "hbm", "kernel": "pip_pair_kernel", "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": (achieved / peak) if achieved else None,
                "peak_source": peak_kind, "traffic": traffic, "traffic_source": traffic_src,
                "algorithmic_bytes_per_launch": alg_bytes,
                "kernel_ms_per_launch": bits_ms / max(bits_n, 1)}

    # end to end through the public API from pinned host buffers: host->device
    # copies of polygons and points (the points' inside the quadtree build),
    # boxes, join, and PiP with its rows copied into page-locked host arrays
    # allocated once
    e2e = None
    if args.e2e_steps > 0:
        # page-locked buffers are first touched by this thread: run it on
        # the GPU's local CPUs (when sysfs names them) so the pages land on
        # the GPU's own NUMA node
        numa = gpu_numa(dist.local)
        old_aff = None
        if hasattr(os, "sched_setaffinity") and numa.get("local_cpulist"):
            cpus = set()
            for part in numa["local_cpulist"].split(","):
                lo, _, hi = part.partition("-")
                if lo.strip():
                    cpus.update(range(int(lo), int(hi or lo) + 1))
            try:
                old_aff = os.sched_getaffinity(0)
                os.sched_setaffinity(0, cpus & old_aff or old_aff)
            except (OSError, ValueError):
                old_aff = None
        link = measure_link(stream)
        link["gpu"] = numa
        hx = torch.from_numpy(w.x).pin_memory()
        hy = torch.from_numpy(w.y).pin_memory()
        hpxy = torch.from_numpy(polygons_xy(P)).pin_memory()
        hro = torch.from_numpy(P.ring_offset).pin_memory()
        hpo = torch.from_numpy(P.part_offset).pin_memory()
        hgo = torch.from_numpy(P.geometry_offset).pin_memory()
        # page-locked row arrays sized by the timed region's result; the
        # rows are written by quadtree_point_in_polygon_host, whose chunked
        # device->host copies overlap the evaluation
        M0 = int(res["polygon_index"].numel())
        o1 = torch.empty(M0, dtype=torch.int32, pin_memory=True)
        o2 = torch.empty(M0, dtype=torch.int32, pin_memory=True)
        link["points_pages_by_node"] = pages_by_node(hx.data_ptr(), hx.numel() * 8)
        if old_aff is not None:
            os.sched_setaffinity(0, old_aff)
        ems, phases, h2d, d2h = [], [], 0, 0
        e2e_warm = 2  # the first passes grow the allocators' pools
        for it in range(args.e2e_steps + e2e_warm):
            ph = [ev() for _ in range(5)]
            ph[0].record(stream)
            dxy = hpxy.to("cuda", non_blocking=True)
            epolys = cs.GeoSeries.from_polygons_xy(dxy, hro.to("cuda", non_blocking=True),
                                                   hpo.to("cuda", non_blocking=True),
                                                   hgo.to("cuda", non_blocking=True))
            ph[1].record(stream)
            # the points' copy overlaps their Morton keys, chunk by chunk
            epts, epi, etree, exy = cs.quadtree_on_points_host(
                hx, hy, w.x_min, w.x_max, w.y_min, w.y_max, w.scale, w.max_depth, w.max_size,
                ordered=True)
            ph[2].record(stream)
            ebb = cs.polygon_bounding_boxes(epolys)
            ej = cs.join_quadtree_and_bounding_boxes(etree, ebb, w.x_min, w.x_max, w.y_min,
                                                     w.y_max, w.scale, w.max_depth)
            ph[3].record(stream)
            m = cs.quadtree_point_in_polygon_host(ej, etree, epi, epts, epolys, o1, o2,
                                                  method=args.method, ordered_points=exy)
            ph[4].record(stream)
            ph[4].synchronize()
            if it >= e2e_warm:
                ems.append(ph[0].elapsed_time(ph[4]))
                phases.append([ph[k].elapsed_time(ph[k + 1]) for k in range(4)])
            h2d = (hx.numel() + hy.numel() + hpxy.numel()) * 8 + (hro.numel() + hpo.numel() +
                                                                   hgo.numel()) * 4
            d2h = 2 * m * 4
        sep_same = bool(m == M0 and torch.equal(o1[:m], res["polygon_index"].cpu()) and
                        torch.equal(o2[:m], res["point_index"].cpu()))
        # the same join through the one-call host entry point: the polygons'
        # copy, boxes and index run beside the quadtree build
        hpo32 = torch.from_numpy(P.part_offset.astype(np.int32)).pin_memory()
        hro32 = torch.from_numpy(P.ring_offset.astype(np.int32)).pin_memory()
        hpx = torch.from_numpy(np.ascontiguousarray(P.x)).pin_memory()
        hpy = torch.from_numpy(np.ascontiguousarray(P.y)).pin_memory()
        jms = []
        for it in range(args.e2e_steps + e2e_warm):
            a, b = ev(), ev()
            a.record(stream)
            mj = cs.point_in_polygon_join_host(hx, hy, w.x_min, w.x_max, w.y_min, w.y_max,
                                               w.scale, w.max_depth, w.max_size, hpo32, hro32,
                                               hpx, hpy, o1, o2, method=args.method)
            b.record(stream)
            b.synchronize()
            if it >= e2e_warm:
                jms.append(a.elapsed_time(b))
        # one more call with the library's stage timers on (per-stage device
        # time; stages on the second stream overlap the others)
        lib.cspt_profile_enable(1)
        cs.point_in_polygon_join_host(hx, hy, w.x_min, w.x_max, w.y_min, w.y_max, w.scale,
                                      w.max_depth, w.max_size, hpo32, hro32, hpx, hpy, o1, o2,
                                      method=args.method)
        torch.cuda.synchronize()
        one_call_stages = {}
        for name in ("quadtree_keys", "quadtree_sort", "quadtree_order", "quadtree_levels",
                     "bounding_boxes", "polygon_index", "join_count", "join_write",
                     "leaf_frames", "pip_bits", "pip_expand"):
            sms, cnt = ctypes.c_double(), ctypes.c_uint64()
            lib.cspt_profile_read(name.encode(), ctypes.byref(sms), ctypes.byref(cnt))
            one_call_stages[name] = sms.value
        lib.cspt_profile_enable(0)
        # its point column holds input point ids: point_indices[point_index]
        joined_same = bool(mj == M0 and torch.equal(o1[:mj], res["polygon_index"].cpu()) and
                           torch.equal(o2[:mj], pi.long()[res["point_index"].long()].int().cpu()))
        # median of the timed calls: on shared hosts single calls of either
        # form now and then take several times longer (host-side stalls
        # outside this library); the means and every call are in the line
        sep_ms = dist.max(statistics.median(ems))
        join_ms = dist.max(statistics.median(jms))
        e2e_ms = min(sep_ms, join_ms)
        if join_ms <= sep_ms:  # the one call's own copies
            h2d = (hx.numel() + hy.numel() + hpx.numel() + hpy.numel()) * 8 + (
                hpo32.numel() + hro32.numel()) * 4
            d2h = 2 * mj * 4
        # lower bounds of one e2e step: its copies at the link's measured
        # rates (the two directions do not overlap each other here), and its
        # device work (point index build + the step)
        link["copy_floor_ms"] = 1e3 * (h2d / (link["h2d_gbs"] * 1e9) +
                                       d2h / (link["d2h_gbs"] * 1e9))
        link["device_work_ms"] = min(build_ms) + ms_per_step
        e2e = {"value": n * args.gpus / (e2e_ms / 1e3), "unit": "points/s",
               "ms_per_step": e2e_ms, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "link": link,
               "api": ("point_in_polygon_join_host (one call)" if join_ms <= sep_ms else
                       "quadtree_on_points_host (ordered), polygon_bounding_boxes, "
                       "join_quadtree_and_bounding_boxes, quadtree_point_in_polygon_host"),
               "one_call_ms": join_ms, "one_call_ms_each": jms,
               "separate_calls_ms_each": ems, "statistic": "median of the timed calls",
               "one_call_ms_mean": statistics.mean(jms),
               "separate_calls_ms_mean": statistics.mean(ems),
               "one_call_rows_identical": joined_same,
               "one_call_stages_ms": one_call_stages,
               "separate_calls_ms": sep_ms,
               "separate_calls_phases_ms": dict(zip(
                   ["polygons_h2d", "points_h2d_and_quadtree_build", "boxes_join",
                    "pip_and_d2h"], [statistics.mean(p[k] for p in phases) for k in range(4)])),
               "pairs_identical": joined_same and sep_same}

    cpu = None
    if dist.rank == 0 and args.gpus == 1 and not args.no_cpu:
        tree_np = {k: (v.cpu().numpy().view(np.uint32) if v.dtype == torch.int32 else
                       v.cpu().numpy()) for k, v in tree.items()}
        tree_np["is_internal_node"] = tree_np["is_internal_node"].astype(bool)
        pairs_np = {k: v.cpu().numpy().view(np.uint32) for k, v in pairs.items()}
        gpu_pip = {k: v.cpu().numpy().view(np.uint32) for k, v in res.items()}
        cpu = cpu_baseline(w, tree_np, pi.cpu().numpy().view(np.uint32), pairs_np, gpu_pip)

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
                   "join_quadtree_and_bounding_boxes + quadtree_point_in_polygon (points "
                   "in quadtree order, gathered once with the quadtree build)",
                   "l2": "inputs larger than L2 (%.1f GB of points resident)" % (16 * n / 1e9),
                   "parallelism": "replicas" if args.gpus > 1 else "single GPU"},
        "pairs": K, "candidates": cand, "hits": M,
        "refined_candidates": refined, "refine_fraction": refined / max(cand, 1),
        "edge_free_pairs": edge_free,
        "build_ms": min(build_ms), "tree_only_build_ms": min(tree_ms),
        "generation_s": gen_s,
        "kernels_ms_per_step": {k: v[0] / max(args.steps, 1) for k, v in kern.items()},
        "plain_fp64": plain,
        "speedup_vs_plain": (plain["ms_per_step"] / ms_per_step) if plain else None,
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
        "clocks": clock_info,
    }
    return line


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
    full = O.join_quadtree_and_bounding_boxes(tree, bb, w.x_min, w.x_max, w.y_min, w.y_max,
                                              w.scale, w.max_depth)
    cand_total = int(qlen[full["quad_offset"]].sum())
    # per step: the shared sample rule, its offset moving with the step
    samples = []
    for it in range(args.warmup + args.steps):
        res = cpu_sample(O, w, tree, pi, bb, qlen, cand_total, it)
        if it >= args.warmup:
            samples.append(res)
    sample_s = [r["sample_s"] for r in samples]
    values = [r["value"] for r in samples]
    value = len(samples) / sum(1.0 / v for v in values)  # points over summed estimated time
    s_per_step = statistics.mean(sample_s)
    sample = cpu_sample_text(samples[0], n) + "; ms_per_step is the sampled wall time"
    line = {
        "metric": METRIC, "impl": "reference", "value": value, "unit": "points/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": s_per_step * 1e3, "p50_ms": percentile([t * 1e3 for t in sample_s], 0.5),
        "p99_ms": percentile([t * 1e3 for t in sample_s], 0.99), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "precision_at_scale", "points": n, "polygons": npoly,
                   "method": "reference crossing test (CPU oracle port)"},
        "cpu_baseline": {"value": value, "unit": "points/s", "cores": O.num_threads(),
                         "kind": "port", "sample": sample,
                         "scale_to_full": statistics.mean(r["full_s"] / r["sample_s"]
                                                          for r in samples),
                         "value_spread": {"min": min(values), "max": max(values),
                                          "stdev": statistics.pstdev(values)}},
        "e2e": {"value": value, "unit": "points/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "build_s": build_s,
    }
    return line


def run_plain_small(args, dist):
    """The plain drop-in configuration: 1,000,000 uniform points in
    [0,1000)^2, 256 star polygons (8-64 vertices), max_depth 7, scale
    1000/128, max_size 128.  A step is polygon_bounding_boxes +
    join_quadtree_and_bounding_boxes + quadtree_point_in_polygon; the whole
    configuration is small enough for the CPU oracle to run in full, so its
    pairs are compared with the GPU's exactly and its time is measured, not
    scaled."""
    import torch

    import cuspatial_gb300 as cs
    from cuspatial_gb300 import datasets
    from oracle import oracle as O

    torch.cuda.set_device(dist.local)
    dist.init("nccl")
    w = datasets.plain_small()
    P = w.polygons
    n = len(w.x)
    pts = cs.GeoSeries.from_points(w.x, w.y)
    polys = cs.GeoSeries.from_polygons_xy(polygons_xy(P), P.ring_offset, P.part_offset,
                                          P.geometry_offset)
    stream = torch.cuda.current_stream()
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    pi, tree, xy = cs.quadtree_on_points_ordered(pts, w.x_min, w.x_max, w.y_min, w.y_max,
                                                 w.scale, w.max_depth, w.max_size)

    def step(method):
        bb = cs.polygon_bounding_boxes(polys)
        pairs = cs.join_quadtree_and_bounding_boxes(tree, bb, w.x_min, w.x_max, w.y_min,
                                                    w.y_max, w.scale, w.max_depth)
        return cs.quadtree_point_in_polygon(pairs, tree, pi, pts, polys, method=method,
                                            ordered_points=xy)

    res, times = {}, {}
    for method in ("exact", "filtered"):
        for _ in range(max(3, args.warmup)):
            res[method] = step(method)
        torch.cuda.synchronize()
        ms = []
        for _ in range(max(10, args.steps)):
            a, b = ev(), ev()
            a.record(stream)
            step(method)
            b.record(stream)
            ms.append((a, b))
        torch.cuda.synchronize()
        times[method] = [a.elapsed_time(b) for a, b in ms]
    # the CPU oracle on the whole configuration (tree, boxes, join, PiP)
    t0 = time.perf_counter()
    opi, ot = O.quadtree_on_points(w.x, w.y, w.x_min, w.x_max, w.y_min, w.y_max, w.scale,
                                   w.max_depth, w.max_size)
    t1 = time.perf_counter()
    obb = O.polygon_bounding_boxes(P.part_offset, P.ring_offset, P.x, P.y)
    oj = O.join_quadtree_and_bounding_boxes(ot, obb, w.x_min, w.x_max, w.y_min, w.y_max,
                                            w.scale, w.max_depth)
    orr = O.quadtree_point_in_polygon(oj, ot, opi, w.x, w.y, P.part_offset, P.ring_offset,
                                      P.x, P.y)
    t2 = time.perf_counter()
    exact_ms = statistics.mean(times["exact"])
    filt_ms = statistics.mean(times["filtered"])
    # the join phase's algorithmic bytes: points, vertices, boxes, pairs, rows
    K, M, V = int(len(oj["bbox_offset"])), int(len(orr["polygon_index"])), int(len(P.x))
    alg_bytes = 20 * n + 16 * V + 32 * P.num_polygons + 8 * K + 8 * M
    peak, peak_kind = measured_peak_hbm()
    achieved = alg_bytes / (exact_ms / 1e3) / 1e9
    same = {m: bool(np.array_equal(r["polygon_index"].cpu().numpy().view(np.uint32),
                                   orr["polygon_index"]) and
                    np.array_equal(r["point_index"].cpu().numpy().view(np.uint32),
                                   orr["point_index"])) for m, r in res.items()}
    return {
        "workload": "plain_small: 1,000,000 uniform points in [0,1000)^2, 256 star polygons "
                    "(8-64 vertices), max_depth 7, scale 1000/128, max_size 128",
        "metric": METRIC, "unit": "points/s", "steps": max(10, args.steps),
        "value": n / (exact_ms / 1e3), "method": "exact (the drop-in)", "ms_per_step": exact_ms,
        "p50_ms": percentile(times["exact"], 0.5), "p99_ms": percentile(times["exact"], 0.99),
        "filtered": {"points_per_s": n / (filt_ms / 1e3), "ms_per_step": filt_ms,
                     "p99_ms": percentile(times["filtered"], 0.99)},
        "roofline": {"bound": "hbm", "kernel": "join step (boxes, join, point-in-polygon), "
                                               "exact method", "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": None,
                     "algorithmic_bytes": alg_bytes,
                     "note": "launch- and host-bound at this size: 1M points, 256 polygons"},
        "pairs_identical_to_oracle": same, "pairs": int(len(oj["bbox_offset"])),
        "hits": int(len(orr["polygon_index"])),
        "cpu_baseline": {"value": n / (t2 - t1), "unit": "points/s", "cores": O.num_threads(),
                         "kind": "port", "sample": "the whole configuration: boxes, join and "
                                                   "point-in-polygon timed (tree build %.2f s "
                                                   "apart)" % (t1 - t0)},
    }


def other_configs(args, dist):
    """The other configurations at their shapes, each a short run whose
    result rides in the default line (an error is recorded, not raised):
    the plain drop-in case (1M points), the nearest-linestring join (50M
    points, 200k linestrings), the serving form (250k resident polygons,
    4000 Poisson requests) and the batched form (4096 instances)."""
    import argparse
    import gc
    out = {}
    runs = [
        ("plain_small", run_plain_small, {}),
        ("nearest", run_nearest, {"steps": 3, "warmup": 1, "nearest_plain_every": 0,
                                  "nearest_points": 50_000_000,
                                  "nearest_linestrings": 200_000, "nearest_extent": 10000.0}),
        ("serving", run_serving, {}),
        ("batched", run_batched, {"steps": 5, "warmup": 2, "plain_steps": 1,
                                  "single_sample": 8, "e2e_steps": 1}),
    ]
    for name, fn, over in runs:
        sub = argparse.Namespace(**vars(args))
        for k, v in over.items():
            setattr(sub, k, v)
        t0 = time.time()
        try:
            out[name] = fn(sub, dist)
        except Exception as e:  # noqa: BLE001 - recorded in the line
            out[name] = {"error": "%s: %s" % (type(e).__name__, e)}
        if isinstance(out[name], dict):
            out[name]["wall_s"] = time.time() - t0
        gc.collect()
    return out


def batched_cpu_sample(wl, P, params, rows, ro_h, budget_s=8.0, max_instances=256):
    """The oracle's whole pipeline (quadtree, boxes, join, point-in-polygon)
    on instances taken in a seeded random order until about budget_s of CPU
    time; points/s over the sample and whether its rows equal the batched
    GPU rows of those instances."""
    from oracle import oracle as O
    order = np.random.default_rng(11).permutation(wl.num_instances)
    po = wl.point_offsets.astype(np.int64)
    qo = wl.polygon_offsets.astype(np.int64)
    gp = rows[0].cpu().numpy().view(np.uint32)
    gq = rows[1].cpu().numpy().view(np.uint32)
    spent, pts, used, same = 0.0, 0, 0, True
    for i in order:
        if spent >= budget_s or used >= max_instances:
            break
        a, b, pa, pb = po[i], po[i + 1], qo[i], qo[i + 1]
        if a == b or pa == pb:
            continue
        r0, r1 = int(P.part_offset[pa]), int(P.part_offset[pb])
        v0, v1 = int(P.ring_offset[r0]), int(P.ring_offset[r1])
        part = (P.part_offset[pa:pb + 1] - r0).astype(np.uint32)
        ring = (P.ring_offset[r0:r1 + 1] - v0).astype(np.uint32)
        vx, vy = np.ascontiguousarray(P.x[v0:v1]), np.ascontiguousarray(P.y[v0:v1])
        x, y = np.ascontiguousarray(wl.x[a:b]), np.ascontiguousarray(wl.y[a:b])
        p = params[i]
        box = (p["x_min"], p["x_max"], p["y_min"], p["y_max"])
        t = time.perf_counter()
        opi, ot = O.quadtree_on_points(x, y, *box, p["scale"], p["max_depth"], p["max_size"])
        obb = O.polygon_bounding_boxes(part, ring, vx, vy)
        oj = O.join_quadtree_and_bounding_boxes(ot, obb, *box, p["scale"], p["max_depth"])
        orr = O.quadtree_point_in_polygon(oj, ot, opi, x, y, part, ring, vx, vy)
        spent += time.perf_counter() - t
        pts += int(b - a)
        used += 1
        same = same and bool(np.array_equal(gp[ro_h[i]:ro_h[i + 1]], orr["polygon_index"]) and
                             np.array_equal(gq[ro_h[i]:ro_h[i + 1]], orr["point_index"]))
    return {"value": pts / spent if spent > 0 else None, "unit": "points/s",
            "cores": O.num_threads(), "kind": "port",
            "sample": "%d instances in a seeded random order (%d points), each through the "
                      "oracle's quadtree, boxes, join and point-in-polygon: %.2f s"
                      % (used, pts, spent),
            "sample_rows_identical_to_gpu": same}


def serving_cpu_sample(P, reqs, params, budget_s=8.0, max_requests=64):
    """The oracle answering requests taken in a seeded random order against
    the whole polygon set (its boxes computed once, untimed, as the resident
    set's are) until about budget_s of CPU time."""
    from oracle import oracle as O
    obb = O.polygon_bounding_boxes(P.part_offset, P.ring_offset, P.x, P.y)
    order = np.random.default_rng(12).permutation(len(reqs))
    spent, pts, used = 0.0, 0, 0
    for i in order:
        if spent >= budget_s or used >= max_requests:
            break
        r, p = reqs[i], params[i]
        if len(r.x) == 0:
            continue
        x, y = np.ascontiguousarray(r.x), np.ascontiguousarray(r.y)
        box = (p["x_min"], p["x_max"], p["y_min"], p["y_max"])
        t = time.perf_counter()
        opi, ot = O.quadtree_on_points(x, y, *box, p["scale"], p["max_depth"], p["max_size"])
        oj = O.join_quadtree_and_bounding_boxes(ot, obb, *box, p["scale"], p["max_depth"])
        O.quadtree_point_in_polygon(oj, ot, opi, x, y, P.part_offset, P.ring_offset, P.x, P.y)
        spent += time.perf_counter() - t
        pts += len(x)
        used += 1
    return {"value": pts / spent if spent > 0 else None, "unit": "points/s",
            "cores": O.num_threads(), "kind": "port",
            "sample": "%d requests in a seeded random order (%d points), each through the "
                      "oracle's quadtree, join against all %d polygons and point-in-polygon: "
                      "%.2f s" % (used, pts, P.num_polygons, spent)}


def run_batched(args, dist):
    """4096 uneven instances (points log-uniform in [1e3, 1e6], polygons
    log-uniform in [1, 2000]) planned together; a step is one replay of the
    captured evaluation graph over all instances."""
    import torch

    import cuspatial_gb300 as cs
    from cuspatial_gb300 import _lib, autotune, datasets
    from cuspatial_gb300.batched import BatchedPointInPolygon

    torch.cuda.set_device(dist.local)
    dist.init("nccl")
    lib = _lib.load()
    lib.cspt_launch_count.restype = ctypes.c_uint64
    t0 = time.time()
    wl = datasets.batched_instances(args.instances)
    gen_s = time.time() - t0
    table = autotune.TuningTable.load()
    params = autotune.batch_params(wl, table)
    P = wl.polygons
    n = len(wl.x)
    x = torch.from_numpy(wl.x).cuda()
    y = torch.from_numpy(wl.y).cuda()
    polys = cs.GeoSeries.from_polygons_xy(polygons_xy(P), P.ring_offset, P.part_offset,
                                          P.geometry_offset)
    stream = torch.cuda.current_stream()
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731

    def plan(method, ordered=True):
        """The plan (which evaluates once to size the rows) and its first
        run, which writes the rows from that evaluation; wall-clock ms."""
        torch.cuda.synchronize()
        t = time.perf_counter()
        pl = BatchedPointInPolygon(x, y, wl.point_offsets, polys, wl.polygon_offsets, params,
                                   method=method, block_threads=table.block_threads,
                                   ordered_index=ordered)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        pl.run(graph=False)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        return pl, (t1 - t) * 1e3, (t2 - t1) * 1e3

    def replays(pl, k, w, counted=None):
        for _ in range(w):
            pl.run(graph=True)
        torch.cuda.synchronize()
        if counted is not None:
            counted.append(lib.cspt_launch_count())
        out = []
        for _ in range(k):
            a, b = ev(), ev()
            a.record(stream)
            pl.run(graph=True)
            b.record(stream)
            out.append((a, b))
        torch.cuda.synchronize()
        return [a.elapsed_time(b) for a, b in out]

    pl, _, _ = plan(args.method)  # warms the allocator
    pl.close()
    lib.cspt_profile_read.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_double),
                                      ctypes.POINTER(ctypes.c_uint64)]
    lib.cspt_profile_enable.argtypes = [ctypes.c_int]
    lib.cspt_profile_enable(1)
    pl, plan_ms, first_ms = plan(args.method)
    plan_stages = {}
    for name in ("batched_tree", "batched_join", "polygon_index"):
        sms, cnt = ctypes.c_double(), ctypes.c_uint64()
        lib.cspt_profile_read(name.encode(), ctypes.byref(sms), ctypes.byref(cnt))
        plan_stages[name] = sms.value
    lib.cspt_profile_enable(0)
    clocks = ClockSampler(dist.local)
    clocks.start()
    counted = []
    dist.barrier()
    step_ms = replays(pl, args.steps, args.warmup, counted)
    dist.barrier()
    launches = int(lib.cspt_launch_count() - counted[0])
    inf = pl.info()
    clock_info = clocks.stop()
    ms = dist.max(statistics.mean(step_ms))
    value = n * args.gpus / (ms / 1e3)
    refined = pl.refined_count()
    ro, rp, rq = pl.rows()
    rows = (rp.clone(), rq.clone(), ro.clone())

    plain = None
    if args.plain_steps > 0 and args.method == "filtered":
        pe, pe_plan_ms, _ = plan("exact")
        pms = replays(pe, args.plain_steps, 1)
        er = pe.rows()
        plain = {"points_per_s": n / (statistics.mean(pms) / 1e3),
                 "ms_per_step": statistics.mean(pms), "plan_ms": pe_plan_ms,
                 "rows_identical_to_filtered": bool(
                     torch.equal(er[1], rows[0]) and torch.equal(er[2], rows[1]) and
                     torch.equal(er[0], rows[2]))}
        pe.close()

    # the one-shot index (no slab ordering): the shortest plan + one run
    pu, pu_plan_ms, pu_first_ms = plan(args.method, ordered=False)
    ur0 = [t.clone() for t in pu.rows()]
    ums = replays(pu, args.steps, args.warmup)
    ur = pu.rows()
    pu_ms = statistics.mean(ums)
    one_shot = {"plan_ms": pu_plan_ms, "ms_per_step": pu_ms, "first_run_ms": pu_first_ms,
                "plan_plus_first_run_points_per_s": n / ((pu_plan_ms + pu_first_ms) / 1e3),
                "first_run_rows_identical_to_replay": bool(
                    all(torch.equal(a, b) for a, b in zip(ur0, ur))),
                "plan_plus_step_points_per_s": n / ((pu_plan_ms + pu_ms) / 1e3),
                "rows_identical_to_ordered": bool(
                    torch.equal(ur[1], rows[0]) and torch.equal(ur[2], rows[1]) and
                    torch.equal(ur[0], rows[2]))}
    pu.close()

    # the same instances one by one through the single-instance calls
    # (sample, time scaled by points)
    rng = np.random.default_rng(7)
    sample = rng.choice(wl.num_instances, min(args.single_sample, wl.num_instances),
                        replace=False)
    po = wl.point_offsets.astype(np.int64)
    qo = wl.polygon_offsets.astype(np.int64)
    single_s, single_pts, mismatches = 0.0, 0, 0
    ro_h = rows[2].cpu().numpy()
    for it, i in enumerate(sample):
        a, b = po[i], po[i + 1]
        pa, pb = qo[i], qo[i + 1]
        r0, r1 = int(P.part_offset[pa]), int(P.part_offset[pb])
        v0, v1 = int(P.ring_offset[r0]), int(P.ring_offset[r1])
        ipts = cs.GeoSeries.from_points(x[a:b], y[a:b])
        xy = torch.empty(2 * (v1 - v0), dtype=torch.float64, device="cuda")
        xy[0::2] = polys.polygons.x[v0:v1]
        xy[1::2] = polys.polygons.y[v0:v1]
        ipolys = cs.GeoSeries.from_polygons_xy(xy, P.ring_offset[r0:r1 + 1] - v0,
                                               P.part_offset[pa:pb + 1] - r0,
                                               np.arange(pb - pa + 1))
        p = params[i]
        for rep in range(2):
            torch.cuda.synchronize()
            t = time.perf_counter()
            ipi, itree = cs.quadtree_on_points(ipts, p["x_min"], p["x_max"], p["y_min"],
                                               p["y_max"], p["scale"], p["max_depth"],
                                               p["max_size"])
            ibb = cs.polygon_bounding_boxes(ipolys)
            ij = cs.join_quadtree_and_bounding_boxes(itree, ibb, p["x_min"], p["x_max"],
                                                     p["y_min"], p["y_max"], p["scale"],
                                                     p["max_depth"])
            ir = cs.quadtree_point_in_polygon(ij, itree, ipi, ipts, ipolys, method=args.method)
            torch.cuda.synchronize()
            if rep == 1 or it == 0:
                el = time.perf_counter() - t
        single_s += el
        single_pts += b - a
        got_p = rows[0][ro_h[i]:ro_h[i + 1]]
        got_q = rows[1][ro_h[i]:ro_h[i + 1]]
        if not (torch.equal(got_p, ir["polygon_index"]) and torch.equal(got_q, ir["point_index"])):
            mismatches += 1
    single_pps = single_pts / single_s if single_s > 0 else None
    cpu = None
    if dist.rank == 0 and args.gpus == 1 and not args.no_cpu:
        cpu = batched_cpu_sample(wl, P, params, rows, ro_h)

    # end to end from pinned host buffers: copies, plan (one-shot index, one
    # evaluation), its first run (the rows), rows back
    e2e = None
    if args.e2e_steps > 0:
        hx = torch.from_numpy(wl.x).pin_memory()
        hy = torch.from_numpy(wl.y).pin_memory()
        hpxy = torch.from_numpy(polygons_xy(P)).pin_memory()
        ems = []
        for it in range(args.e2e_steps + 1):
            torch.cuda.synchronize()
            t = time.perf_counter()
            dx = hx.to("cuda", non_blocking=True)
            dy = hy.to("cuda", non_blocking=True)
            dxy = hpxy.to("cuda", non_blocking=True)
            epolys = cs.GeoSeries.from_polygons_xy(dxy, P.ring_offset, P.part_offset,
                                                   P.geometry_offset)
            ep = BatchedPointInPolygon(dx, dy, wl.point_offsets, epolys, wl.polygon_offsets,
                                       params, method=args.method,
                                       block_threads=table.block_threads, ordered_index=False)
            ep.run(graph=False)
            ero, erp, erq = ep.rows()
            if it == 0:  # pinned row buffers, sized by the untimed first pass
                h_ro = torch.empty(ero.shape, dtype=ero.dtype).pin_memory()
                h_p = torch.empty(erp.shape, dtype=erp.dtype).pin_memory()
                h_q = torch.empty(erq.shape, dtype=erq.dtype).pin_memory()
            h_ro.copy_(ero, non_blocking=True)
            h_p.copy_(erp, non_blocking=True)
            h_q.copy_(erq, non_blocking=True)
            torch.cuda.synchronize()
            if it > 0:
                ems.append((time.perf_counter() - t) * 1e3)
            ep.close()
        h2d = (hx.numel() + hy.numel() + hpxy.numel()) * 8 + (
            len(P.ring_offset) + len(P.part_offset) + len(P.geometry_offset)) * 4
        d2h = h_ro.numel() * 8 + (h_p.numel() + h_q.numel()) * 4
        e2e_ms = dist.max(statistics.mean(ems))
        e2e = {"value": n * args.gpus / (e2e_ms / 1e3), "unit": "points/s",
               "ms_per_step": e2e_ms, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h),
               "rows_identical": bool(torch.equal(h_p.cuda(), rows[0]) and
                                      torch.equal(h_q.cuda(), rows[1]))}

    V = len(P.x)
    alg_bytes = 20 * n + 16 * V + 12 * inf.num_pairs + 8 * inf.num_rows
    peak, peak_kind = measured_peak_hbm()
    achieved = alg_bytes / (ms / 1e3) / 1e9
    line = {
        "metric": METRIC, "workload": "batched", "value": value, "unit": "points/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "p50_ms": percentile(step_ms, 0.5), "p99_ms": percentile(step_ms, 0.99),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded numpy PCG64; shapes of the 4096-instance batched config)",
        "config": {"workload": "batched_instances: %d instances, points log-uniform "
                               "[1e3,1e6], polygons log-uniform [1,2000]" % wl.num_instances,
                   "points": n, "polygons": P.num_polygons, "vertices": V,
                   "method": args.method, "block_threads": table.block_threads,
                   "tuning": {"buckets": table.buckets,
                              "device": table.meta.get("device", "untuned defaults")},
                   "step": "one replay of the captured evaluation graph (all instances)",
                   "l2": "inputs larger than L2 (%.1f GB of points resident)" % (16 * n / 1e9)},
        "plan_ms": plan_ms, "plan_stages_ms": plan_stages,
        "plan_plus_step_points_per_s": n / ((plan_ms + ms) / 1e3),
        "first_run_ms": first_ms,
        "plan_plus_first_run_points_per_s": n / ((plan_ms + first_ms) / 1e3),
        "one_shot_index": one_shot,
        "nodes": inf.num_nodes, "pairs": inf.num_pairs, "rows": inf.num_rows,
        "refined_candidates": refined, "kernels_per_step": inf.kernels_per_run,
        "plain_fp64": plain,
        "speedup_vs_plain": (plain["ms_per_step"] / ms) if plain else None,
        "single_instance_calls": {"instances": len(sample), "points_per_s": single_pps,
                                  "rows_mismatching_batched": mismatches,
                                  "note": "quadtree + boxes + join + PiP per instance, "
                                          "timed one instance at a time"},
        "roofline": {"bound": "hbm", "kernel": "batched evaluation graph", "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": None},
        "e2e": e2e, "cpu_baseline": cpu, "gpu_launches": launches, "clocks": clock_info,
        "generation_s": gen_s,
    }
    pl.close()
    return line


def run_serving(args, dist):
    """A resident set of 250,000 star polygons over [0,20000)^2 and a Poisson
    stream of requests (log-uniform [1, 1e5] points, half uniform, half one
    Gaussian cluster); admission by a 40 GB device-memory budget."""
    import torch

    import cuspatial_gb300 as cs
    from cuspatial_gb300 import _lib, datasets
    from cuspatial_gb300.serving import PolygonSet, Server, request_params, run_poisson

    torch.cuda.set_device(dist.local)
    dist.init("nccl")
    lib = _lib.load()
    lib.cspt_launch_count.restype = ctypes.c_uint64
    lib.cspt_profile_read.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_double),
                                      ctypes.POINTER(ctypes.c_uint64)]
    lib.cspt_profile_enable.argtypes = [ctypes.c_int]
    t0 = time.time()
    P = datasets.serving_polygons()
    reqs = datasets.serving_requests(args.requests)
    warm = datasets.serving_requests(200, seed_offset=1)
    gen_s = time.time() - t0
    gp = cs.GeoSeries.from_polygons_xy(polygons_xy(P), P.ring_offset, P.part_offset,
                                       P.geometry_offset)
    torch.cuda.synchronize()
    t = time.perf_counter()
    pset = PolygonSet(gp)
    torch.cuda.synchronize()
    set_ms = (time.perf_counter() - t) * 1e3
    params = [request_params(r.x, r.y) for r in reqs]
    wparams = [request_params(r.x, r.y) for r in warm]
    budget = 40 << 30
    out = {}
    for method in (["filtered", "exact"] if args.method == "filtered" else [args.method]):
        with Server(pset, memory_budget_bytes=budget, num_streams=args.streams,
                    method=method) as srv:
            run_poisson(srv, warm, rate=0, params=wparams, seed=1)
            clocks = ClockSampler(dist.local)
            clocks.start()
            l0 = lib.cspt_launch_count()
            live = run_poisson(srv, reqs, rate=args.rate, params=params, seed=2)
            l1 = lib.cspt_launch_count()
            lib.cspt_profile_enable(1)
            sat = run_poisson(srv, reqs, rate=0, params=params, seed=3)
            stages = {}
            for name in ("forest_build", "serving_join", "serving_sort", "serving_pip"):
                ms_, cnt_ = ctypes.c_double(), ctypes.c_uint64()
                lib.cspt_profile_read(name.encode(), ctypes.byref(ms_), ctypes.byref(cnt_))
                stages[name] = {"ms": ms_.value, "launches": int(cnt_.value)}
            lib.cspt_profile_enable(0)
            clock_info = clocks.stop()
            st = srv.stats()
        out[method] = {"live": live, "saturated": sat, "stats": st, "clocks": clock_info,
                       "launches_live": int(l1 - l0), "stages_saturated": stages}
    f = out[args.method]
    value = f["saturated"]["points_per_s"] * args.gpus
    # algorithmic bytes at saturation: every request's points read (16 B)
    # and sorted-index read (4 B), every row written (8 B); the resident set
    # is not counted
    alg_bytes = 20 * f["saturated"]["points"] + 8 * f["saturated"]["rows"]
    peak, peak_kind = measured_peak_hbm()
    achieved = alg_bytes / f["saturated"]["span_s"] / 1e9
    cpu = None
    if dist.rank == 0 and args.gpus == 1 and not args.no_cpu:
        cpu = serving_cpu_sample(P, reqs, params)
    line = {
        "metric": METRIC, "workload": "serving", "value": value, "unit": "points/s",
        "n_gpus": args.gpus, "steps": args.requests, "warmup": len(warm),
        "ms_per_step": f["saturated"]["span_s"] * 1e3 / args.requests,
        "p50_ms": f["live"]["p50_ms"], "p99_ms": f["live"]["p99_ms"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded numpy PCG64; shapes of the serving config)",
        "config": {"workload": "serving: 250,000 resident star polygons (8-256 vertices, "
                               "radius U[1,30]) on a jittered 500x500 grid over [0,20000)^2; "
                               "%d Poisson requests at %.0f req/s, log-uniform [1,1e5] points"
                               % (args.requests, args.rate),
                   "polygons": P.num_polygons, "vertices": len(P.x),
                   "requests": args.requests, "points": f["live"]["points"],
                   "memory_budget_bytes": budget, "streams": args.streams,
                   "method": args.method,
                   "step": "one request (value: points/s with all requests queued at once; "
                           "p50/p99: latency at the offered Poisson rate)"},
        "polygon_set_ms": set_ms,
        "live": f["live"], "saturated": f["saturated"], "server_stats": f["stats"],
        "stages_saturated_ms": f["stages_saturated"],
        "plain_fp64": ({"live": out["exact"]["live"], "saturated": out["exact"]["saturated"]}
                       if "exact" in out and args.method != "exact" else None),
        "roofline": {"bound": "hbm", "kernel": "serving, all requests queued at once",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind, "traffic": None,
                     "algorithmic_bytes": alg_bytes},
        "cpu_baseline": cpu,
        "gpu_launches": f["launches_live"], "clocks": f["clocks"], "generation_s": gen_s,
    }
    pset.close()
    return line


def run_nearest(args, dist):
    """Points uniform in [0,10000)^2 (50,000,000 by default) and 200,000
    random-walk linestrings (2-256 segments); a step is
    linestring_bounding_boxes (radius 25) + join_quadtree_and_bounding_boxes +
    quadtree_point_to_nearest_linestring with the float32 filter.  The plain
    float64 method is timed on the pairs of every k-th leaf (about 5e11
    float64 segment distances per full step would take minutes on this
    part's float64 unit) and scaled by the candidate fraction; its rows are
    compared with the filtered rows of the same points.  The CPU oracle runs
    on every 4096th leaf: its rows are compared with the GPU's and its time,
    scaled by candidates, is the CPU baseline."""
    import torch

    import cuspatial_gb300 as cs
    from cuspatial_gb300 import _lib, datasets

    torch.cuda.set_device(dist.local)
    dist.init("nccl")
    lib = _lib.load()
    lib.cspt_launch_count.restype = ctypes.c_uint64
    lib.cspt_profile_read.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_double),
                                      ctypes.POINTER(ctypes.c_uint64)]
    lib.cspt_profile_enable.argtypes = [ctypes.c_int]
    t0 = time.time()
    w = datasets.nearest_linestring(n_points=args.nearest_points,
                                    n_linestrings=args.nearest_linestrings,
                                    extent=args.nearest_extent)
    gen_s = time.time() - t0
    L = w.linestrings
    n = len(w.x)
    nls = len(L.part_offset) - 1
    pts = cs.GeoSeries.from_points(w.x, w.y)
    xy = np.empty(2 * len(L.x))
    xy[0::2], xy[1::2] = L.x, L.y
    lines = cs.GeoSeries.from_linestrings_xy(xy, L.part_offset, L.geometry_offset)
    stream = torch.cuda.current_stream()
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    a, b = ev(), ev()
    a.record(stream)
    pi, tree, oxy = cs.quadtree_on_points_ordered(pts, w.x_min, w.x_max, w.y_min, w.y_max,
                                                  w.scale, w.max_depth, w.max_size)
    b.record(stream)
    b.synchronize()
    build_ms = a.elapsed_time(b)

    def step():
        bb = cs.linestring_bounding_boxes(lines, w.expansion_radius)
        pairs = cs.join_quadtree_and_bounding_boxes(tree, bb, w.x_min, w.x_max, w.y_min,
                                                    w.y_max, w.scale, w.max_depth)
        return pairs, cs.quadtree_point_to_nearest_linestring(pairs, tree, pi, pts, lines,
                                                              method="filtered",
                                                              ordered_points=oxy)

    for _ in range(args.warmup):
        pairs, res = step()
    torch.cuda.synchronize()
    clocks = ClockSampler(dist.local)
    clocks.start()
    lib.cspt_profile_enable(1)
    l0 = lib.cspt_launch_count()
    times = []
    for _ in range(args.steps):
        a, b = ev(), ev()
        a.record(stream)
        pairs, res = step()
        b.record(stream)
        times.append((a, b))
    torch.cuda.synchronize()
    kern = {}
    for name in ("bounding_boxes", "join_count", "join_write", "nearest_index", "leaf_frames",
                 "nearest"):
        kms, cnt = ctypes.c_double(), ctypes.c_uint64()
        lib.cspt_profile_read(name.encode(), ctypes.byref(kms), ctypes.byref(cnt))
        kern[name] = kms.value / max(args.steps, 1)
    lib.cspt_profile_enable(0)
    launches = int(lib.cspt_launch_count() - l0)
    clock_info = clocks.stop()
    ms = [x.elapsed_time(y) for x, y in times]
    f_ms = dist.max(statistics.mean(ms))
    paths = cs.last_nearest_stats()

    # plain float64 on every k-th leaf's pairs
    pq = pairs["quad_offset"].long()
    qlen = tree["length"].long()
    cand_all = int(qlen[pq].sum().item())
    plain = None
    if args.nearest_plain_every > 0:
        sel = (pq % args.nearest_plain_every) == 0
        sub = {"bbox_offset": pairs["bbox_offset"][sel].contiguous(),
               "quad_offset": pairs["quad_offset"][sel].contiguous()}
        cand_sub = int(qlen[pq[sel]].sum().item())
        a, b = ev(), ev()
        a.record(stream)
        ex = cs.quadtree_point_to_nearest_linestring(sub, tree, pi, pts, lines, method="exact")
        b.record(stream)
        b.synchronize()
        sub_ms = a.elapsed_time(b)
        fi = cs.quadtree_point_to_nearest_linestring(sub, tree, pi, pts, lines,
                                                     method="filtered")
        same = bool(torch.equal(fi["linestring_index"], ex["linestring_index"]) and
                    torch.equal(fi["distance"], ex["distance"]) and
                    torch.equal(fi["point_index"], ex["point_index"]))
        plain_ms = sub_ms * cand_all / max(cand_sub, 1)
        plain = {"leaves": "every %dth" % args.nearest_plain_every,
                 "candidate_fraction": cand_sub / max(cand_all, 1), "sample_ms": sub_ms,
                 "ms_per_step_scaled": plain_ms, "rows_identical_to_filtered": same}

    # the oracle on the pairs of every 4096th leaf (rows of those leaves' points)
    oracle_check = cpu = None
    if dist.rank == 0 and not args.no_cpu:
        from oracle import oracle as O
        osel = (pq % 4096) == 0
        osub = {"bbox_offset": pairs["bbox_offset"][osel].cpu().numpy().view(np.uint32),
                "quad_offset": pairs["quad_offset"][osel].cpu().numpy().view(np.uint32)}
        tree_np = {k: (v.cpu().numpy().view(np.uint32) if v.dtype == torch.int32 else
                       v.cpu().numpy()) for k, v in tree.items()}
        tree_np["is_internal_node"] = tree_np["is_internal_node"].astype(bool)
        t0 = time.perf_counter()
        orr = O.quadtree_point_to_nearest_linestring(osub, tree_np, pi.cpu().numpy().view(
            np.uint32), w.x, w.y, L.part_offset, L.x, L.y)
        o_s = time.perf_counter() - t0
        rows = orr["linestring_index"] != 0xFFFFFFFF
        g_ls = res["linestring_index"].cpu().numpy().view(np.uint32)
        g_d = res["distance"].cpu().numpy()
        o_cand = int(qlen[pq[osel]].sum().item())
        oracle_check = {"leaves": "every 4096th", "rows": int(rows.sum()),
                        "oracle_s": o_s, "cores": O.num_threads(),
                        "candidate_fraction": o_cand / max(cand_all, 1),
                        "rows_identical": bool(np.array_equal(g_ls[rows],
                                                              orr["linestring_index"][rows]) and
                                               np.array_equal(g_d[rows], orr["distance"][rows]))}
        full_s = o_s * cand_all / max(o_cand, 1)
        cpu = {"value": n / full_s, "unit": "points/s", "cores": O.num_threads(),
               "kind": "port",
               "sample": "the oracle on the pairs of every 4096th leaf (%.3f%% of candidates, "
                         "%d rows): %.2f s, scaled by candidates to %.0f s for the full join"
                         % (100.0 * o_cand / max(cand_all, 1), int(rows.sum()), o_s, full_s),
               "sample_s": o_s}
    # roofline of the nearest kernel: 20 N + 16 V + 32 L + 8 K + 16 N (points
    # and their index, linestring vertices and boxes, pairs, rows)
    nb_alg = 20 * n + 16 * len(L.x) + 32 * nls + 8 * int(pairs["bbox_offset"].numel()) + 16 * n
    peak, peak_kind = measured_peak_hbm()
    nk_ms = kern.get("nearest") or 0.0
    achieved = nb_alg / (nk_ms / 1e3) / 1e9 if nk_ms else None
    roofline = {"bound": "hbm", "kernel": "nearest_filtered_kernel", "achieved": achieved,
                "peak": peak, "unit": "GB/s", "frac": achieved / peak if achieved else None,
                "peak_source": peak_kind, "algorithmic_bytes_per_launch": nb_alg,
                "kernel_ms_per_launch": nk_ms,
                "note": "bound by instruction issue and the float64 pipe, not HBM "
                        "(profiles/nearest_filtered_kernel_5M_points_20k_linestrings.md)"}
    return {
        "metric": METRIC, "workload": "nearest", "value": n * args.gpus / (f_ms / 1e3),
        "unit": "points/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": f_ms, "p50_ms": percentile(ms, 0.5), "p99_ms": percentile(ms, 0.99),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded numpy PCG64; shapes of the nearest-linestring config)",
        "config": {"workload": "nearest_linestring: %d uniform points in [0,%g)^2, %d "
                               "random-walk linestrings (2-256 segments), max_depth 14, "
                               "max_size 256, expansion radius 25" % (n, args.nearest_extent, nls),
                   "points": n, "linestrings": nls, "vertices": len(L.x),
                   "step": "linestring_bounding_boxes + join_quadtree_and_bounding_boxes + "
                           "quadtree_point_to_nearest_linestring (float32 filter, points in "
                           "quadtree order built with the tree)"},
        "pairs": int(pairs["bbox_offset"].numel()), "candidates": cand_all,
        "build_ms": build_ms, "plain_fp64_sampled": plain,
        "speedup_vs_plain": plain["ms_per_step_scaled"] / f_ms if plain else None,
        "gpu_launches": launches, "clocks": clock_info, "generation_s": gen_s,
        "paths": paths, "oracle_sample": oracle_check, "kernels_ms_per_step": kern,
        "roofline": roofline, "cpu_baseline": cpu,
    }


def run_unindexed(args, dist):
    """The reference's point_in_polygon benchmark shape
    (cpp/benchmarks/point_in_polygon/point_in_polygon.cu): 10,000,000 points
    uniform in [-20,20]^2 against 31 regular polygons of 100 sides, radius 10,
    all centred on the origin; float64.  A step is one point_in_polygon call
    (polygon index + one thread per point through all 31 polygons); value is
    points per second.  e2e adds the host->device copies of the points and
    polygons and the device->host copy of the int32 bitmask."""
    import torch

    import cuspatial_gb300 as cs
    from cuspatial_gb300 import _lib, datasets
    from oracle import oracle as O

    torch.cuda.set_device(dist.local)
    dist.init("nccl")
    lib = _lib.load()
    lib.cspt_launch_count.restype = ctypes.c_uint64
    lib.cspt_profile_read.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_double),
                                      ctypes.POINTER(ctypes.c_uint64)]
    lib.cspt_profile_enable.argtypes = [ctypes.c_int]
    w = datasets.unindexed_pip(n_points=args.unindexed_points, sides=args.sides)
    P = w.polygons
    n = len(w.x)
    pts = cs.GeoSeries.from_points(w.x, w.y)
    polys = cs.GeoSeries.from_polygons_xy(polygons_xy(P), P.ring_offset, P.part_offset,
                                          P.geometry_offset)
    stream = torch.cuda.current_stream()
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731

    def timed(method, steps):
        for _ in range(args.warmup):
            cs.point_in_polygon_bitmask(pts, polys, method)
        torch.cuda.synchronize()
        times = []
        for _ in range(steps):
            a, b = ev(), ev()
            a.record(stream)
            r = cs.point_in_polygon_bitmask(pts, polys, method)
            b.record(stream)
            times.append((a, b))
        torch.cuda.synchronize()
        return r, [x.elapsed_time(y) for x, y in times]

    clocks = ClockSampler(dist.local)
    clocks.start()
    l0 = lib.cspt_launch_count()
    lib.cspt_profile_enable(1)
    res, ms = timed(args.method, args.steps)
    launches = int(lib.cspt_launch_count() - l0)
    clock_info = clocks.stop()
    refined = cs.last_refined_count()
    kern = {}
    for name in ("points_pip", "polygon_index"):
        t, c = ctypes.c_double(), ctypes.c_uint64()
        lib.cspt_profile_read(name.encode(), ctypes.byref(t), ctypes.byref(c))
        kern[name] = t.value / max(c.value, 1)
    lib.cspt_profile_enable(0)  # clears the totals
    f_ms = dist.max(statistics.mean(ms))
    ex_res, ex_ms = timed("exact", max(1, args.plain_steps))
    same = bool(torch.equal(res, ex_res))

    # e2e from pinned host buffers
    hx = torch.from_numpy(w.x).pin_memory()
    hy = torch.from_numpy(w.y).pin_memory()
    hpxy = torch.from_numpy(polygons_xy(P)).pin_memory()
    hoff = [torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
            for a in (P.ring_offset, P.part_offset, P.geometry_offset)]
    hout = torch.empty(n, dtype=torch.int32).pin_memory()
    h2d = n * 16 + hpxy.numel() * 8 + sum(a.numel() * 4 for a in hoff)
    e2e = []
    for i in range(args.warmup + args.e2e_steps):
        a, b = ev(), ev()
        a.record(stream)
        dx = hx.to("cuda", non_blocking=True)
        dy = hy.to("cuda", non_blocking=True)
        dxy = hpxy.to("cuda", non_blocking=True)
        doff = [t.to("cuda", non_blocking=True) for t in hoff]
        p2 = cs.GeoSeries.from_points(dx, dy)
        g2 = cs.GeoSeries.from_polygons_xy(dxy, *doff)
        m = cs.point_in_polygon_bitmask(p2, g2, args.method)
        hout.copy_(m, non_blocking=True)
        b.record(stream)
        b.synchronize()
        if i >= args.warmup:
            e2e.append(a.elapsed_time(b))
    e2e_ms = dist.max(statistics.mean(e2e))
    e2e_same = bool(torch.equal(hout, res.cpu()))

    # parity of a sample against the oracle, and the CPU baseline on it
    k = min(n, 200_000)
    t0 = time.time()
    want = O.point_in_polygon(w.x[:k], w.y[:k], P.part_offset, P.ring_offset, P.x, P.y)
    cpu_s = time.time() - t0
    parity = bool(np.array_equal(res[:k].cpu().numpy(), want))
    algo_bytes = n * (16 + 4) + len(P.x) * 16
    hbm, hbm_kind = measured_peak_hbm()
    pip_ms = kern["points_pip"]
    line = {
        "metric": "point_in_polygon points/s (31 polygons, unindexed)", "workload": "unindexed",
        "value": n * args.gpus / (f_ms / 1e3), "unit": "points/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": f_ms,
        "p50_ms": percentile(ms, 0.5), "p99_ms": percentile(ms, 0.99),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded numpy PCG64; the reference benchmark's shapes)",
        "config": {"workload": "point_in_polygon: %d points uniform in [-20,20]^2, 31 regular "
                               "%d-gons of radius 10 at the origin" % (n, args.sides),
                   "points": n, "polygons": 31, "sides": args.sides, "method": args.method,
                   "l2": "inputs (%.0f MB) larger than L2" % (n * 16 / 1e6)},
        "kernels_ms": kern, "exact_ms_per_step": statistics.mean(ex_ms),
        "filtered_equals_exact": same, "refined_tests": refined,
        "oracle_sample_identical": parity,
        "e2e": {"value": n * args.gpus / (e2e_ms / 1e3), "unit": "points/s",
                "ms_per_step": e2e_ms, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": n * 4, "result_identical": e2e_same},
        "roofline": {"bound": "hbm", "achieved": algo_bytes / (pip_ms / 1e3) / 1e9,
                     "peak": hbm, "unit": "GB/s",
                     "frac": algo_bytes / (pip_ms / 1e3) / 1e9 / hbm if hbm else None,
                     "traffic": None,
                     "peak_kind": hbm_kind,
                     "note": "points_pip kernel: 16 B read + 4 B written per point"},
        "cpu_baseline": {"value": k / cpu_s, "unit": "points/s", "cores": 1, "kind": "port",
                         "sample": "first %d points, all 31 polygons" % k},
        "gpu_launches": launches, "clocks": clock_info,
    }
    return line


def main():
    args = parse_args()
    dist = Dist()
    if args.impl == "reference":
        line = run_reference(args, dist)
    elif args.workload == "batched":
        line = run_batched(args, dist)
    elif args.workload == "serving":
        line = run_serving(args, dist)
    elif args.workload == "nearest":
        line = run_nearest(args, dist)
    elif args.workload == "unindexed":
        line = run_unindexed(args, dist)
    else:
        line = run_ours(args, dist)
        if not args.no_configs:
            line["other_configs"] = other_configs(args, dist)
    if line is not None and dist.rank == 0:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
