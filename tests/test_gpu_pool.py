"""Calls without a caller allocator draw on the library's own stream-ordered
pool: the results equal those of the torch-allocator path, the outputs go
back through cspt_free / cspt_quadtree_free, and the pool can be trimmed."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import cuspatial_gb300 as cs  # noqa: E402
from cuspatial_gb300 import _lib  # noqa: E402

pytestmark = pytest.mark.gpu


class _DeviceArray:
    """A raw device pointer seen through __cuda_array_interface__."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<i4",
                                         "data": (ptr, False), "version": 3}


def _copy_u32(ptr, n):
    if n == 0:
        return np.empty(0, dtype=np.uint32)
    t = torch.as_tensor(_DeviceArray(ptr, n), device="cuda")
    return t.cpu().numpy().view(np.uint32)


def test_quadtree_with_library_pool():
    lib = _lib.load()
    rng = np.random.default_rng(5)
    n = 200_000
    x = torch.from_numpy(rng.uniform(0, 1000, n)).cuda()
    y = torch.from_numpy(rng.uniform(0, 1000, n)).cuda()
    args = (0.0, 1000.0, 0.0, 1000.0, 1000.0 / 512, 9, 64)
    pi_ref, tree_ref = cs.quadtree_on_points(cs.GeoSeries.from_points(x, y), *args)
    for _ in range(3):  # repeated calls reuse the pool's memory
        out_pi = ctypes.c_void_p()
        tree = _lib.CsptQuadtree()
        st = lib.cspt_quadtree_on_points(
            ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), n, _lib.FLOAT64,
            *args, None, _lib.stream_ptr(), ctypes.byref(out_pi), ctypes.byref(tree))
        assert st == _lib.OK
        torch.cuda.synchronize()
        got_pi = _copy_u32(out_pi.value, n)
        np.testing.assert_array_equal(got_pi, pi_ref.cpu().numpy().view(np.uint32))
        assert tree.num_nodes == len(tree_ref["key"])
        got_key = _copy_u32(tree.key, tree.num_nodes)
        np.testing.assert_array_equal(got_key, tree_ref["key"].cpu().numpy().view(np.uint32))
        lib.cspt_free(None, out_pi, n * 4, _lib.stream_ptr())
        lib.cspt_quadtree_free(None, ctypes.byref(tree), _lib.stream_ptr())
    assert lib.cspt_pool_trim(0) == _lib.OK
