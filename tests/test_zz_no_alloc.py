"""The no-allocation polygon-box entry point against the allocating one.

cspt_polygon_bounding_boxes_noalloc serves callers that must not allocate
device memory (stream capture, latency-bound loops, hosts that own all device
memory): it keeps its scratch in a fixed device array.  Two calls in a row
with different inputs must each equal cspt_polygon_bounding_boxes bit for bit
(each call reuses the array the previous one wrote), for float64 and float32
coordinates, and oversize inputs are refused before any GPU work.
"""

import ctypes

import numpy as np
import pytest
import torch

from cuspatial_gb300 import _lib
from cuspatial_gb300 import datasets as D

pytestmark = pytest.mark.gpu

_vp, _sz = ctypes.c_void_p, ctypes.c_size_t
ARGS = [_vp, _sz, _vp, _sz, _vp, _vp, _sz, ctypes.c_int, ctypes.c_double, _vp, _vp, _vp, _vp, _vp]


def _boxes(fn, po, ro, x, y, r):
    n = po.numel() - 1
    out = [torch.full((n,), -1.0, dtype=x.dtype, device="cuda") for _ in range(4)]
    status = fn(_lib.ptr(po), po.numel(), _lib.ptr(ro), ro.numel(), _lib.ptr(x), _lib.ptr(y),
                x.numel(), _lib.FLOAT64 if x.dtype == torch.float64 else _lib.FLOAT32, r,
                *[_lib.ptr(o) for o in out], _lib.stream_ptr())
    return status, out


def _polygon_set(n_polygons, seed, with_empty, dtype=torch.float64):
    w = D.precision_at_scale(n_points=1000, n_polygons=n_polygons, extent=5000.0,
                             max_vertices=200, seed_offset=seed)
    P = w.polygons
    po = P.part_offset.astype(np.int64)
    if with_empty:  # polygons without rings: rows move up, trailing rows are NaN
        po = np.insert(po, [3, 3, 10], [po[3], po[3], po[10]])
    dev = lambda a, t: torch.from_numpy(np.ascontiguousarray(a)).to(t).cuda()  # noqa: E731
    return (dev(po, torch.int32), dev(P.ring_offset, torch.int32), dev(P.x, dtype),
            dev(P.y, dtype))


def test_noalloc_matches_allocating_entry_point_twice():
    lib = _lib.load()
    lib.cspt_polygon_bounding_boxes.argtypes = ARGS
    lib.cspt_polygon_bounding_boxes_noalloc.argtypes = ARGS
    lib.cspt_polygon_bounding_boxes_noalloc.restype = ctypes.c_int
    # float64 and float32 coordinates (the float32 branch has its own box
    # kernel and NaN tail), with and without empty polygons and expansion
    inputs = [(_polygon_set(5000, 11, False), 0.0), (_polygon_set(700, 12, True), 0.25),
              (_polygon_set(3000, 13, True, torch.float32), 0.5),
              (_polygon_set(900, 14, False, torch.float32), 0.0)]
    for (po, ro, x, y), r in inputs:  # calls in a row
        s_ref, ref = _boxes(lib.cspt_polygon_bounding_boxes, po, ro, x, y, r)
        s_new, got = _boxes(lib.cspt_polygon_bounding_boxes_noalloc, po, ro, x, y, r)
        torch.cuda.synchronize()
        assert s_ref == _lib.OK and s_new == _lib.OK
        for a, b in zip(ref, got):
            assert torch.equal(torch.isnan(a), torch.isnan(b))
            assert torch.equal(a.nan_to_num(0.0), b.nan_to_num(0.0))


def test_noalloc_rejects_more_than_its_scratch_holds():
    lib = _lib.load()
    lib.cspt_polygon_bounding_boxes_noalloc.argtypes = ARGS
    lib.cspt_polygon_bounding_boxes_noalloc.restype = ctypes.c_int
    n = (1 << 20) + 1
    po = torch.zeros(n + 1, dtype=torch.int32, device="cuda")
    ro = torch.zeros(2, dtype=torch.int32, device="cuda")
    x = torch.zeros(4, dtype=torch.float64, device="cuda")
    status, _ = _boxes(lib.cspt_polygon_bounding_boxes_noalloc, po, ro, x, x, 0.0)
    assert status == _lib.INVALID_ARGUMENT
    assert b"at most 1048576 polygons" in lib.cspt_last_error_message()
