"""Batched quadtree point-in-polygon join (no counterpart in cuSpatial).

cuSpatial joins one point set with one polygon set per call
(python/cuspatial/cuspatial/core/spatial/join.py:177).  A workload of many
small, independent joins — one per tile, per customer, per time window —
would pay every stage's launches and host synchronisations once per
instance.  `BatchedPointInPolygon` plans all instances together (one tree
build, one box join, one polygon index) and evaluates every candidate pair of
every instance in the same kernels, optionally replayed from a CUDA graph.
Each instance's rows are exactly what

    quadtree_on_points -> polygon_bounding_boxes ->
    join_quadtree_and_bounding_boxes -> quadtree_point_in_polygon

return for that instance alone with its parameters.
"""

import ctypes

import numpy as np
import torch

from . import _lib
from .geoseries import GeoSeries, Table, as_device_tensor, contains_only_polygons

_METHODS = {"exact": _lib.METHOD_EXACT, "filtered": _lib.METHOD_FILTERED}
PARAM_FIELDS = ("x_min", "x_max", "y_min", "y_max", "scale", "max_depth", "max_size")


# cspt_instance_params as a numpy record: five doubles, two int32 (48 bytes)
_PARAMS_DTYPE = np.dtype([(k, "<f8") for k in PARAM_FIELDS[:5]] +
                         [(k, "<i4") for k in PARAM_FIELDS[5:]])
assert _PARAMS_DTYPE.itemsize == ctypes.sizeof(_lib.CsptInstanceParams)


def _params_array(params):
    """Sequence of dicts or tuples in PARAM_FIELDS order -> a contiguous
    array laid out as cspt_instance_params (filled column by column)."""
    rows = [[p[k] for k in PARAM_FIELDS] if isinstance(p, dict) else list(p) for p in params]
    arr = np.empty(len(rows), dtype=_PARAMS_DTYPE)
    if rows:
        for j, k in enumerate(PARAM_FIELDS):
            arr[k] = [r[j] for r in rows]
    return arr


class BatchedPointInPolygon:
    """A planned batched join.

    points_x, points_y: float64 coordinates of all instances' points.
    point_offsets: instance i owns points [point_offsets[i], point_offsets[i+1]).
    polygons: GeoSeries of all instances' polygons.
    polygon_offsets: instance i owns polygons [polygon_offsets[i], ...[i+1]).
    params: per instance x_min, x_max, y_min, y_max, scale, max_depth,
    max_size (dicts or tuples), the arguments of quadtree_on_points.
    method: "exact" (float64) or "filtered" (float32 filter, float64
    refinement; same rows).  ordered_index: sort each slab's crossing edges
    into per-(slab, x-bin) windows — a longer plan and faster runs, for plans
    run many times; False keeps the one-shot index (shortest plan + run).
    block_threads: block size of the per-pair kernels with the ordered index.
    budget_bytes: optional cap on the device memory the plan may take.
    """

    def __init__(self, points_x, points_y, point_offsets, polygons: GeoSeries, polygon_offsets,
                 params, method="filtered", block_threads=256, budget_bytes=None,
                 ordered_index=True):
        if len(polygons) and not contains_only_polygons(polygons):
            raise ValueError("`polygons` Geoseries must contains only polygons geometries.")
        self._lib = lib = _lib.load()
        x = as_device_tensor(points_x)
        y = as_device_tensor(points_y)
        if x.dtype != torch.float64 or y.dtype != torch.float64:
            raise TypeError("the batched form supports float64 coordinates")
        po = np.ascontiguousarray(np.asarray(point_offsets, dtype=np.uint64))
        qo = np.ascontiguousarray(np.asarray(polygon_offsets, dtype=np.uint64))
        ni = len(po) - 1
        if ni < 1 or len(qo) != ni + 1 or len(params) != ni:
            raise ValueError("offsets must have one more entry than params")
        poly = polygons.polygons
        self._alloc = _lib.TorchAllocator(x.device, budget_bytes)
        self._keep = (x, y, poly.part_offset, poly.ring_offset, poly.x, poly.y)
        self._params = _params_array(params)
        self.point_offsets = po
        self.polygon_offsets = qo
        u64p = ctypes.POINTER(ctypes.c_uint64)
        h = ctypes.c_void_p()
        _lib.check(lib.cspt_batched_pip_plan(
            ni, po.ctypes.data_as(u64p), _lib.ptr(x), _lib.ptr(y), qo.ctypes.data_as(u64p),
            _lib.ptr(poly.part_offset), int(poly.part_offset.numel()), _lib.ptr(poly.ring_offset),
            int(poly.ring_offset.numel()), _lib.ptr(poly.x), _lib.ptr(poly.y),
            int(poly.x.numel()),
            self._params.ctypes.data_as(ctypes.POINTER(_lib.CsptInstanceParams)), _lib.FLOAT64,
            _METHODS[method],
            1 if ordered_index else 0, int(block_threads), self._alloc.ref, _lib.stream_ptr(),
            ctypes.byref(h)), lib)
        self._h = h
        self._row_offsets_host = None

    # -- execution ---------------------------------------------------------
    def run(self, graph=True, stream=None):
        """Evaluates all instances (asynchronous on the current stream).  The
        first run after the plan writes the rows from the plan's sizing
        evaluation; later runs evaluate again (graph replays with
        ``graph=True``)."""
        _lib.check(self._lib.cspt_batched_pip_run(self._handle(), 1 if graph else 0,
                                                  _lib.stream_ptr(stream)), self._lib)
        self._row_offsets_host = None
        return self

    # -- results -----------------------------------------------------------
    def info(self):
        inf = _lib.CsptBatchedPipInfo()
        _lib.check(self._lib.cspt_batched_pip_get_info(self._handle(), ctypes.byref(inf)),
                   self._lib)
        return inf

    def _view(self, p, count, dtype):
        if not p or count == 0:
            return torch.empty(0, dtype=dtype, device=self._keep[0].device)
        t = self._alloc.blocks[p]
        nbytes = count * torch.empty(0, dtype=dtype).element_size()
        return t[:nbytes].view(dtype)

    def rows(self):
        """(row_offsets int64[num_instances+1], polygon_index int32, point_index int32)."""
        inf = self.info()
        ro = self._view(inf.row_offsets, inf.num_instances + 1, torch.int64)
        return (ro, self._view(inf.polygon_index, inf.num_rows, torch.int32),
                self._view(inf.point_index, inf.num_rows, torch.int32))

    def instance_result(self, i):
        """Table(polygon_index, point_index) of instance i (local indices)."""
        ro, pidx, qidx = self.rows()
        if self._row_offsets_host is None:
            self._row_offsets_host = ro.cpu().numpy()
        a, b = int(self._row_offsets_host[i]), int(self._row_offsets_host[i + 1])
        out = Table()
        out["polygon_index"] = pidx[a:b]
        out["point_index"] = qidx[a:b]
        return out

    def point_indices(self, i=None):
        inf = self.info()
        pi = self._view(inf.point_indices, inf.num_points, torch.int32)
        if i is None:
            return pi
        return pi[int(self.point_offsets[i]):int(self.point_offsets[i + 1])]

    def quadtree(self, i=None):
        """Table of the concatenated (or instance i's) quadtree columns."""
        inf = self.info()
        q = inf.num_nodes
        t = inf.tree
        cols = Table()
        cols["key"] = self._view(t.key, q, torch.int32)
        cols["level"] = self._view(t.level, q, torch.uint8)
        cols["is_internal_node"] = self._view(t.is_internal_node, q, torch.uint8).bool()
        cols["length"] = self._view(t.length, q, torch.int32)
        cols["offset"] = self._view(t.offset, q, torch.int32)
        if i is None:
            return cols
        no = self._view(inf.node_offsets, inf.num_instances + 1, torch.int64).cpu().numpy()
        a, b = int(no[i]), int(no[i + 1])
        out = Table()
        for k, v in cols.items():
            out[k] = v[a:b]
        return out

    def refined_count(self):
        v = ctypes.c_uint64()
        _lib.check(self._lib.cspt_batched_pip_refined_count(self._handle(), _lib.stream_ptr(),
                                                            ctypes.byref(v)), self._lib)
        return int(v.value)

    @property
    def device_bytes(self):
        return self._alloc.in_use

    # -- lifetime ----------------------------------------------------------
    def _handle(self):
        if self._h is None:
            raise RuntimeError("the batched plan has been closed")
        return self._h

    def close(self):
        if getattr(self, "_h", None) is not None:
            torch.cuda.current_stream().synchronize()
            self._lib.cspt_batched_pip_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
