"""ctypes binding of libcuspatial_gb300.so plus a torch-backed device allocator.

All device memory the library asks for (outputs and scratch) is taken from
torch's caching allocator on the current stream, so results come back as
torch tensors without a copy.  There is no CPU fallback: when the shared
library cannot be loaded or built, every call raises.
"""

import ctypes
import os
import threading

import torch

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libcuspatial_gb300.so")

OK, INVALID_ARGUMENT, OUT_OF_MEMORY, CUDA_ERROR, TIMEOUT, UNSUPPORTED = range(6)
FLOAT32, FLOAT64 = 0, 1
METHOD_EXACT, METHOD_FILTERED = 0, 1

_vp = ctypes.c_void_p
_sz = ctypes.c_size_t
_u32p = ctypes.POINTER(ctypes.c_uint32)

ALLOC_FN = ctypes.CFUNCTYPE(_vp, _vp, _sz, _vp)
FREE_FN = ctypes.CFUNCTYPE(None, _vp, _vp, _sz, _vp)


class CsptAllocator(ctypes.Structure):
    _fields_ = [("ctx", _vp), ("allocate", ALLOC_FN), ("deallocate", FREE_FN)]


class CsptQuadtree(ctypes.Structure):
    _fields_ = [("key", _vp), ("level", _vp), ("is_internal_node", _vp), ("length", _vp),
                ("offset", _vp), ("num_nodes", _sz)]


class CsptInstanceParams(ctypes.Structure):
    _fields_ = [("x_min", ctypes.c_double), ("x_max", ctypes.c_double),
                ("y_min", ctypes.c_double), ("y_max", ctypes.c_double),
                ("scale", ctypes.c_double), ("max_depth", ctypes.c_int32),
                ("max_size", ctypes.c_int32)]


class CsptBatchedPipInfo(ctypes.Structure):
    _fields_ = [("num_instances", _sz), ("num_points", _sz), ("num_polygons", _sz),
                ("num_nodes", _sz), ("num_pairs", _sz), ("num_rows", _sz),
                ("kernels_per_run", ctypes.c_uint64), ("polygon_index", _vp),
                ("point_index", _vp), ("row_offsets", _vp), ("point_indices", _vp),
                ("tree", CsptQuadtree), ("node_offsets", _vp)]


class CsptServerOptions(ctypes.Structure):
    _fields_ = [("memory_budget_bytes", _sz), ("num_streams", ctypes.c_int),
                ("max_batch_points", _sz), ("max_batch_requests", _sz),
                ("method", ctypes.c_int), ("block_threads", ctypes.c_int)]


class CsptServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64),
                ("failed", ctypes.c_uint64), ("batches", ctypes.c_uint64),
                ("split_batches", ctypes.c_uint64), ("queued", ctypes.c_uint64),
                ("reserved_bytes", _sz), ("peak_device_bytes", _sz),
                ("memory_budget_bytes", _sz), ("max_batch_requests_seen", ctypes.c_uint64)]


class CsptRequestResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("error", ctypes.c_char_p),
                ("polygon_index", _vp), ("point_index", _vp), ("num_rows", _sz),
                ("point_indices", _vp), ("num_points", _sz), ("submit_s", ctypes.c_double),
                ("admit_s", ctypes.c_double), ("done_s", ctypes.c_double),
                ("batch", ctypes.c_uint64), ("batch_requests", ctypes.c_uint32)]


class CuspatialError(RuntimeError):
    """Raised for CUDA, allocation and timeout failures reported by the library."""


_lib = None
_lock = threading.Lock()


def _declare(lib):
    lib.cspt_last_error_message.restype = ctypes.c_char_p
    lib.cspt_version.restype = ctypes.c_char_p
    lib.cspt_last_refined_count.restype = ctypes.c_uint64
    lib.cspt_last_edge_free_pairs.restype = ctypes.c_uint64
    lib.cspt_last_nearest_stats.argtypes = [ctypes.POINTER(ctypes.c_uint64),
                                            ctypes.POINTER(ctypes.c_uint64),
                                            ctypes.POINTER(ctypes.c_uint64)]
    lib.cspt_last_nearest_stats.restype = None
    lib.cspt_free.argtypes = [ctypes.POINTER(CsptAllocator), _vp, _sz, _vp]
    lib.cspt_pool_trim.argtypes = [_sz]
    lib.cspt_quadtree_free.argtypes = [ctypes.POINTER(CsptAllocator),
                                       ctypes.POINTER(CsptQuadtree), _vp]
    lib.cspt_quadtree_on_points.argtypes = [
        _vp, _vp, _sz, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
        ctypes.c_double, ctypes.c_double, ctypes.c_int8, ctypes.c_int32,
        ctypes.POINTER(CsptAllocator), _vp, ctypes.POINTER(_vp), ctypes.POINTER(CsptQuadtree)]
    lib.cspt_quadtree_on_points_host.argtypes = [
        _vp, _vp, _sz, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
        ctypes.c_double, ctypes.c_double, ctypes.c_int8, ctypes.c_int32, _vp, _vp,
        ctypes.POINTER(CsptAllocator), _vp, ctypes.POINTER(_vp), ctypes.POINTER(CsptQuadtree)]
    lib.cspt_polygon_bounding_boxes.argtypes = [
        _vp, _sz, _vp, _sz, _vp, _vp, _sz, ctypes.c_int, ctypes.c_double, _vp, _vp, _vp, _vp, _vp]
    lib.cspt_linestring_bounding_boxes.argtypes = [
        _vp, _sz, _vp, _vp, _sz, ctypes.c_int, ctypes.c_double, _vp, _vp, _vp, _vp, _vp]
    lib.cspt_join_quadtree_and_bounding_boxes.argtypes = [
        ctypes.POINTER(CsptQuadtree), _vp, _vp, _vp, _vp, _sz, ctypes.c_int, ctypes.c_double,
        ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int8,
        ctypes.POINTER(CsptAllocator), _vp, ctypes.POINTER(_vp), ctypes.POINTER(_vp),
        ctypes.POINTER(_sz)]
    lib.cspt_quadtree_point_in_polygon.argtypes = [
        _vp, _vp, _sz, ctypes.POINTER(CsptQuadtree), _vp, _sz, _vp, _vp, _sz, _vp, _sz, _vp, _sz,
        _vp, _vp, _sz, ctypes.c_int, ctypes.c_int, ctypes.POINTER(CsptAllocator), _vp,
        ctypes.POINTER(_vp), ctypes.POINTER(_vp), ctypes.POINTER(_sz)]
    lib.cspt_quadtree_point_in_polygon_host.argtypes = [
        _vp, _vp, _sz, ctypes.POINTER(CsptQuadtree), _vp, _sz, _vp, _vp, _sz, _vp, _sz, _vp, _sz,
        _vp, _vp, _sz, ctypes.c_int, ctypes.c_int, ctypes.POINTER(CsptAllocator), _vp, _vp, _vp,
        _sz, ctypes.POINTER(_sz)]
    lib.cspt_point_in_polygon_join_host.argtypes = [
        _vp, _vp, _sz, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
        ctypes.c_double, ctypes.c_double, ctypes.c_int8, ctypes.c_int32, _vp, _sz, _vp, _sz, _vp,
        _vp, _sz, ctypes.c_int, ctypes.POINTER(CsptAllocator), _vp, _vp, _vp, _sz,
        ctypes.POINTER(_sz)]
    lib.cspt_quadtree_point_to_nearest_linestring.argtypes = [
        _vp, _vp, _sz, ctypes.POINTER(CsptQuadtree), _vp, _sz, _vp, _vp, _sz, _vp, _sz, _vp, _vp,
        _sz, ctypes.c_int, ctypes.c_int, ctypes.POINTER(CsptAllocator), _vp, _vp, _vp, _vp,
        ctypes.POINTER(_sz)]
    lib.cspt_quadtree_on_points_ordered.argtypes = (lib.cspt_quadtree_on_points.argtypes +
                                                    [_vp])
    lib.cspt_quadtree_on_points_host_ordered.argtypes = (
        lib.cspt_quadtree_on_points_host.argtypes + [_vp])
    lib.cspt_points_in_quadtree_order.argtypes = [_vp, _sz, _vp, _vp, _sz, ctypes.c_int, _vp,
                                                  _vp]
    lib.cspt_quadtree_point_in_polygon_ordered.argtypes = [
        _vp, _vp, _sz, ctypes.POINTER(CsptQuadtree), _vp, _sz, _vp, _sz, _vp, _sz, _vp, _vp, _sz,
        ctypes.c_int, ctypes.c_int, ctypes.POINTER(CsptAllocator), _vp, ctypes.POINTER(_vp),
        ctypes.POINTER(_vp), ctypes.POINTER(_sz)]
    lib.cspt_quadtree_point_in_polygon_host_ordered.argtypes = [
        _vp, _vp, _sz, ctypes.POINTER(CsptQuadtree), _vp, _sz, _vp, _sz, _vp, _sz, _vp, _vp, _sz,
        ctypes.c_int, ctypes.c_int, ctypes.POINTER(CsptAllocator), _vp, _vp, _vp, _sz,
        ctypes.POINTER(_sz)]
    lib.cspt_quadtree_point_to_nearest_linestring_ordered.argtypes = [
        _vp, _vp, _sz, ctypes.POINTER(CsptQuadtree), _vp, _sz, _vp, _sz, _vp, _vp, _sz,
        ctypes.c_int, ctypes.c_int, ctypes.POINTER(CsptAllocator), _vp, _vp, _vp, _vp,
        ctypes.POINTER(_sz)]
    for name in ("cspt_point_in_polygon", "cspt_pairwise_point_in_polygon"):
        getattr(lib, name).argtypes = [
            _vp, _vp, _sz, _vp, _sz, _vp, _sz, _vp, _vp, _sz, ctypes.c_int, ctypes.c_int,
            ctypes.POINTER(CsptAllocator), _vp, _vp]
    lib.cspt_quadtree_contains_properly.argtypes = [
        _vp, _vp, _sz, _vp, _sz, _vp, _sz, _vp, _sz, _vp, _vp, _sz, ctypes.c_int, ctypes.c_int,
        ctypes.POINTER(CsptAllocator), _vp, ctypes.POINTER(_vp), ctypes.POINTER(_vp),
        ctypes.POINTER(_vp), ctypes.POINTER(_sz)]
    lib.cspt_pairwise_point_linestring_distance.argtypes = [
        _vp, _sz, _vp, _vp, _sz, _vp, _sz, _vp, _sz, _vp, _vp, _sz, ctypes.c_int, ctypes.c_int,
        _vp, _vp]
    lib.cspt_pairwise_point_linestring_nearest_points.argtypes = [
        _vp, _sz, _vp, _vp, _sz, _vp, _sz, _vp, _sz, _vp, _vp, _sz, ctypes.c_int, ctypes.c_int,
        _vp, _vp, _vp, _vp, _vp]
    _u64p = ctypes.POINTER(ctypes.c_uint64)
    lib.cspt_batched_pip_plan.argtypes = [
        _sz, _u64p, _vp, _vp, _u64p, _vp, _sz, _vp, _sz, _vp, _vp, _sz,
        ctypes.POINTER(CsptInstanceParams), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
        ctypes.POINTER(CsptAllocator), _vp, ctypes.POINTER(_vp)]
    lib.cspt_batched_pip_run.argtypes = [_vp, ctypes.c_int, _vp]
    lib.cspt_batched_pip_get_info.argtypes = [_vp, ctypes.POINTER(CsptBatchedPipInfo)]
    lib.cspt_batched_pip_refined_count.argtypes = [_vp, _vp, _u64p]
    lib.cspt_batched_pip_free.argtypes = [_vp]
    lib.cspt_batched_pip_free.restype = None
    lib.cspt_polygon_set_create.argtypes = [_vp, _sz, _vp, _sz, _vp, _vp, _sz, ctypes.c_int,
                                            ctypes.POINTER(CsptAllocator), _vp,
                                            ctypes.POINTER(_vp)]
    lib.cspt_polygon_set_free.argtypes = [_vp]
    lib.cspt_polygon_set_free.restype = None
    lib.cspt_server_create.argtypes = [_vp, ctypes.POINTER(CsptServerOptions),
                                       ctypes.POINTER(_vp)]
    lib.cspt_server_submit.argtypes = [_vp, ctypes.c_uint64, _vp, _vp, _sz,
                                       ctypes.POINTER(CsptInstanceParams)]
    lib.cspt_server_poll.argtypes = [_vp, ctypes.POINTER(ctypes.c_uint64), _sz, ctypes.c_double]
    lib.cspt_server_poll.restype = _sz
    lib.cspt_server_result.argtypes = [_vp, ctypes.c_uint64, ctypes.POINTER(CsptRequestResult)]
    lib.cspt_server_release.argtypes = [_vp, ctypes.c_uint64]
    lib.cspt_server_release.restype = None
    lib.cspt_server_now.argtypes = [_vp]
    lib.cspt_server_now.restype = ctypes.c_double
    lib.cspt_server_get_stats.argtypes = [_vp, ctypes.POINTER(CsptServerStats)]
    lib.cspt_server_free.argtypes = [_vp]
    lib.cspt_server_free.restype = None
    for name in ("cspt_polygon_set_create", "cspt_server_create", "cspt_server_submit",
                 "cspt_server_result", "cspt_server_get_stats"):
        getattr(lib, name).restype = ctypes.c_int
    for name in ("cspt_batched_pip_plan", "cspt_batched_pip_run", "cspt_batched_pip_get_info",
                 "cspt_batched_pip_refined_count"):
        getattr(lib, name).restype = ctypes.c_int
    for name in ("cspt_quadtree_on_points", "cspt_quadtree_on_points_host",
                 "cspt_polygon_bounding_boxes",
                 "cspt_linestring_bounding_boxes", "cspt_join_quadtree_and_bounding_boxes",
                 "cspt_quadtree_point_in_polygon", "cspt_quadtree_point_in_polygon_host",
                 "cspt_point_in_polygon_join_host",
                 "cspt_quadtree_point_to_nearest_linestring"):
        getattr(lib, name).restype = ctypes.c_int
    return lib


def load(build_if_missing=True):
    """Loads the shared library (building it in-tree first if needed)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        from . import build as _build
        if build_if_missing and not _build.up_to_date():
            _build.build()
        if not os.path.exists(LIB_PATH):
            raise CuspatialError("libcuspatial_gb300.so is not built (run cuspatial_gb300.build)")
        _lib = _declare(ctypes.CDLL(LIB_PATH))
        return _lib


def check(status, lib=None):
    if status == OK:
        return
    lib = lib or load()
    msg = lib.cspt_last_error_message().decode()
    if status == INVALID_ARGUMENT:
        # cuspatial::logic_error surfaces as RuntimeError through Cython
        raise RuntimeError(msg)
    if status == UNSUPPORTED:
        raise TypeError(msg)
    if status == OUT_OF_MEMORY:
        raise MemoryError(msg)
    raise CuspatialError(msg)


class TorchAllocator:
    """cspt_allocator whose memory comes from torch's caching allocator.

    Blocks handed to the library are kept alive in a dict until the library
    frees them or the caller adopts them as output tensors.  An optional byte
    budget makes allocations beyond it fail (the library then reports
    OUT_OF_MEMORY), which lets callers admit work by memory.
    """

    def __init__(self, device=None, budget_bytes=None):
        self.device = torch.device(device) if device is not None else torch.device(
            "cuda", torch.cuda.current_device())
        self.budget = budget_bytes
        self.in_use = 0
        self.peak = 0
        self.blocks = {}
        self._streams = {}  # library streams other than torch's current one
        self._alloc_cb = ALLOC_FN(self._allocate)
        self._free_cb = FREE_FN(self._deallocate)
        self.struct = CsptAllocator(None, self._alloc_cb, self._free_cb)
        self.ref = ctypes.byref(self.struct)

    def _allocate(self, ctx, nbytes, stream):
        try:
            if self.budget is not None and self.in_use + nbytes > self.budget:
                return None
            # the block belongs to the stream the library will use it on:
            # torch's caching allocator reuses a freed block only for later
            # work on that same stream
            cur = torch.cuda.current_stream(self.device)
            if stream and int(stream) != cur.cuda_stream:
                ext = self._streams.get(int(stream))
                if ext is None:
                    ext = torch.cuda.ExternalStream(int(stream), device=self.device)
                    self._streams[int(stream)] = ext
                with torch.cuda.stream(ext):
                    t = torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=self.device)
            else:
                t = torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=self.device)
        except Exception:  # noqa: BLE001 - out of memory: report NULL to the library
            return None
        p = t.data_ptr()
        self.blocks[p] = t
        self.in_use += int(nbytes)
        self.peak = max(self.peak, self.in_use)
        return p

    def _deallocate(self, ctx, ptr, nbytes, stream):
        t = self.blocks.pop(ptr, None)
        if t is not None:
            self.in_use -= int(nbytes)

    def adopt(self, ptr, count, dtype):
        """Takes ownership of a library-allocated block as a typed tensor."""
        if not ptr or count == 0:
            return torch.empty(0, dtype=dtype, device=self.device)
        t = self.blocks.pop(ptr)
        nbytes = count * torch.empty(0, dtype=dtype).element_size()
        self.in_use -= t.numel()
        return t[:nbytes].view(dtype)


def stream_ptr(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None and t.numel() else None
