"""ctypes front end of the CPU oracle (oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and by
bench.py's CPU-baseline leg, always as the checker.  The product package
never imports this module.

Every function takes and returns numpy arrays and mirrors one libcuspatial
entry point (cpp/include/cuspatial/point_quadtree.hpp:68-78,
bounding_boxes.hpp:52-85, spatial_join.hpp:66-175).
"""

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

_vp = ctypes.c_void_p
_sz = ctypes.c_size_t


def build():
    """Compile liboracle.so with the Makefile beside this file."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def _load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH) or (
        os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "oracle.cpp"))
    ):
        build()
    lib = ctypes.CDLL(_LIB_PATH)
    lib.oracle_free.argtypes = [_vp]
    lib.oracle_num_threads.restype = ctypes.c_int
    lib.oracle_set_num_threads.argtypes = [ctypes.c_int]
    lib.oracle_quadtree_on_points.argtypes = [
        _vp, _vp, _sz, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
        ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int32,
        ctypes.POINTER(_vp), ctypes.POINTER(_vp), ctypes.POINTER(_vp), ctypes.POINTER(_vp),
        ctypes.POINTER(_vp), ctypes.POINTER(_vp), ctypes.POINTER(_sz)]
    lib.oracle_polygon_bounding_boxes.argtypes = [
        _vp, _sz, _vp, _sz, _vp, _vp, _sz, ctypes.c_int, ctypes.c_double, _vp, _vp, _vp, _vp]
    lib.oracle_linestring_bounding_boxes.argtypes = [
        _vp, _sz, _vp, _vp, _sz, ctypes.c_int, ctypes.c_double, _vp, _vp, _vp, _vp]
    lib.oracle_join_quadtree_and_bounding_boxes.argtypes = [
        _vp, _vp, _vp, _vp, _vp, _sz, _vp, _vp, _vp, _vp, _sz, ctypes.c_int, ctypes.c_double,
        ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int,
        ctypes.POINTER(_vp), ctypes.POINTER(_vp), ctypes.POINTER(_sz)]
    lib.oracle_quadtree_point_in_polygon.argtypes = [
        _vp, _vp, _sz, _vp, _vp, _vp, _sz, _vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_int,
        ctypes.POINTER(_vp), ctypes.POINTER(_vp), ctypes.POINTER(_sz)]
    lib.oracle_is_point_in_polygon.argtypes = [
        ctypes.c_double, ctypes.c_double, _vp, ctypes.c_int64, ctypes.c_int64, _vp, _vp]
    lib.oracle_pairwise_point_linestring.argtypes = [
        _sz, _vp, _vp, _vp, _vp, _vp, _sz, _vp, _vp, ctypes.c_int, _vp, _vp, _vp, _vp, _vp]
    lib.oracle_point_in_polygon.argtypes = [
        _vp, _vp, _sz, _vp, _sz, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int, _vp]
    lib.oracle_quadtree_point_to_nearest_linestring.argtypes = [
        _vp, _vp, _sz, _vp, _vp, _vp, _sz, _vp, _vp, _vp, _vp, _vp, ctypes.c_int, _vp, _vp, _vp]
    _lib = lib
    return lib


def _ptr(a):
    return a.ctypes.data_as(_vp) if a is not None and a.size else None


def _take(lib, p, n, dtype):
    if not p or n == 0:
        return np.zeros(0, dtype=dtype)
    buf = (ctypes.c_char * (n * np.dtype(dtype).itemsize)).from_address(p)
    out = np.frombuffer(buf, dtype=dtype).copy()
    lib.oracle_free(p)
    return out


def _dtype_code(a):
    return 1 if a.dtype == np.float64 else 0


def set_num_threads(n):
    _load().oracle_set_num_threads(int(n))


def num_threads():
    return _load().oracle_num_threads()


def quadtree_on_points(x, y, x_min, x_max, y_min, y_max, scale, max_depth, max_size):
    """Returns (point_indices, dict of the 5 quadtree columns)."""
    lib = _load()
    x = np.ascontiguousarray(x)
    y = np.ascontiguousarray(y, dtype=x.dtype)
    outs = [_vp() for _ in range(6)]
    nn = _sz()
    lib.oracle_quadtree_on_points(_ptr(x), _ptr(y), x.size, _dtype_code(x), x_min, x_max, y_min,
                                  y_max, scale, int(max_depth), int(max_size),
                                  *[ctypes.byref(o) for o in outs], ctypes.byref(nn))
    n = nn.value
    point_indices = _take(lib, outs[0].value, x.size, np.uint32)
    tree = dict(key=_take(lib, outs[1].value, n, np.uint32),
                level=_take(lib, outs[2].value, n, np.uint8),
                is_internal_node=_take(lib, outs[3].value, n, np.uint8).astype(bool),
                length=_take(lib, outs[4].value, n, np.uint32),
                offset=_take(lib, outs[5].value, n, np.uint32))
    return point_indices, tree


def polygon_bounding_boxes(poly_offsets, ring_offsets, x, y, expansion_radius=0.0):
    lib = _load()
    po = np.ascontiguousarray(poly_offsets, dtype=np.uint32)
    ro = np.ascontiguousarray(ring_offsets, dtype=np.uint32)
    x = np.ascontiguousarray(x)
    y = np.ascontiguousarray(y, dtype=x.dtype)
    n = max(po.size - 1, 0)
    outs = [np.empty(n, dtype=x.dtype) for _ in range(4)]
    lib.oracle_polygon_bounding_boxes(_ptr(po), po.size, _ptr(ro), ro.size, _ptr(x), _ptr(y),
                                      x.size, _dtype_code(x), expansion_radius,
                                      *[_ptr(o) for o in outs])
    return dict(zip(["minx", "miny", "maxx", "maxy"], outs))


def linestring_bounding_boxes(offsets, x, y, expansion_radius):
    lib = _load()
    lo = np.ascontiguousarray(offsets, dtype=np.uint32)
    x = np.ascontiguousarray(x)
    y = np.ascontiguousarray(y, dtype=x.dtype)
    n = max(lo.size - 1, 0)
    outs = [np.empty(n, dtype=x.dtype) for _ in range(4)]
    lib.oracle_linestring_bounding_boxes(_ptr(lo), lo.size, _ptr(x), _ptr(y), x.size,
                                         _dtype_code(x), expansion_radius,
                                         *[_ptr(o) for o in outs])
    return dict(zip(["minx", "miny", "maxx", "maxy"], outs))


def _tree_arrays(tree):
    return [np.ascontiguousarray(tree["key"], dtype=np.uint32),
            np.ascontiguousarray(tree["level"], dtype=np.uint8),
            np.ascontiguousarray(tree["is_internal_node"], dtype=np.uint8),
            np.ascontiguousarray(tree["length"], dtype=np.uint32),
            np.ascontiguousarray(tree["offset"], dtype=np.uint32)]


def join_quadtree_and_bounding_boxes(tree, bboxes, x_min, x_max, y_min, y_max, scale,
                                     max_depth):
    lib = _load()
    ta = _tree_arrays(tree)
    b = [np.ascontiguousarray(bboxes[k]) for k in ("minx", "miny", "maxx", "maxy")]
    ob, oq, nn = _vp(), _vp(), _sz()
    lib.oracle_join_quadtree_and_bounding_boxes(
        *[_ptr(a) for a in ta], ta[0].size, *[_ptr(a) for a in b], b[0].size,
        _dtype_code(b[0]), x_min, x_max, y_min, y_max, scale, int(max_depth),
        ctypes.byref(ob), ctypes.byref(oq), ctypes.byref(nn))
    n = nn.value
    return dict(bbox_offset=_take(lib, ob.value, n, np.uint32),
                quad_offset=_take(lib, oq.value, n, np.uint32))


def quadtree_point_in_polygon(pairs, tree, point_indices, x, y, poly_offsets, ring_offsets,
                              px, py):
    lib = _load()
    pp = np.ascontiguousarray(pairs["bbox_offset"], dtype=np.uint32)
    pq = np.ascontiguousarray(pairs["quad_offset"], dtype=np.uint32)
    ln = np.ascontiguousarray(tree["length"], dtype=np.uint32)
    of = np.ascontiguousarray(tree["offset"], dtype=np.uint32)
    pi = np.ascontiguousarray(point_indices, dtype=np.uint32)
    x = np.ascontiguousarray(x)
    y = np.ascontiguousarray(y, dtype=x.dtype)
    po = np.ascontiguousarray(poly_offsets, dtype=np.uint32)
    ro = np.ascontiguousarray(ring_offsets, dtype=np.uint32)
    px = np.ascontiguousarray(px, dtype=x.dtype)
    py = np.ascontiguousarray(py, dtype=x.dtype)
    op, oq, nn = _vp(), _vp(), _sz()
    lib.oracle_quadtree_point_in_polygon(_ptr(pp), _ptr(pq), pp.size, _ptr(ln), _ptr(of),
                                         _ptr(pi), pi.size, _ptr(x), _ptr(y), _ptr(po),
                                         _ptr(ro), _ptr(px), _ptr(py), _dtype_code(x),
                                         ctypes.byref(op), ctypes.byref(oq), ctypes.byref(nn))
    n = nn.value
    return dict(polygon_index=_take(lib, op.value, n, np.uint32),
                point_index=_take(lib, oq.value, n, np.uint32))


def is_point_in_polygon(px, py, ring_offsets, ring_begin, ring_end, vx, vy):
    lib = _load()
    ro = np.ascontiguousarray(ring_offsets, dtype=np.uint32)
    vx = np.ascontiguousarray(vx, dtype=np.float64)
    vy = np.ascontiguousarray(vy, dtype=np.float64)
    return bool(lib.oracle_is_point_in_polygon(float(px), float(py), _ptr(ro), int(ring_begin),
                                               int(ring_end), _ptr(vx), _ptr(vy)))


def point_in_polygon(x, y, poly_offsets, ring_offsets, px, py, pairwise=False):
    """Unindexed test: int32 bitmask per point over all polygons (bit p =
    inside polygon p), or with ``pairwise`` a uint8 per point for polygon i."""
    lib = _load()
    x = np.ascontiguousarray(x)
    y = np.ascontiguousarray(y, dtype=x.dtype)
    po = np.ascontiguousarray(poly_offsets, dtype=np.uint32)
    ro = np.ascontiguousarray(ring_offsets, dtype=np.uint32)
    px = np.ascontiguousarray(px, dtype=x.dtype)
    py = np.ascontiguousarray(py, dtype=x.dtype)
    npoly = max(po.size - 1, 0)
    if pairwise:
        assert x.size == npoly
    else:
        assert npoly <= 31
    out = np.zeros(x.size, dtype=np.uint8 if pairwise else np.int32)
    lib.oracle_point_in_polygon(_ptr(x), _ptr(y), x.size, _ptr(po), npoly, _ptr(ro), _ptr(px),
                                _ptr(py), _dtype_code(x), int(bool(pairwise)), _ptr(out))
    return out


def pairwise_point_linestring(x, y, part_offsets, lx, ly, point_geometry_offsets=None,
                              linestring_geometry_offsets=None):
    """Pairwise point-linestring distance and nearest points: a dict with
    distance, point_geometry_id, linestring_geometry_id, segment_id and the
    nearest points' x, y."""
    lib = _load()
    x = np.ascontiguousarray(x)
    y = np.ascontiguousarray(y, dtype=x.dtype)
    lx = np.ascontiguousarray(lx, dtype=x.dtype)
    ly = np.ascontiguousarray(ly, dtype=x.dtype)
    lpo = np.ascontiguousarray(part_offsets, dtype=np.uint32)
    pgo = (None if point_geometry_offsets is None
           else np.ascontiguousarray(point_geometry_offsets, dtype=np.uint32))
    lgo = (None if linestring_geometry_offsets is None
           else np.ascontiguousarray(linestring_geometry_offsets, dtype=np.uint32))
    n = (pgo.size - 1) if pgo is not None else x.size
    dist = np.zeros(n, dtype=x.dtype)
    opt = np.zeros(n, np.int32)
    ols = np.zeros(n, np.int32)
    oseg = np.zeros(n, np.int32)
    oxy = np.zeros(2 * n, dtype=x.dtype)
    lib.oracle_pairwise_point_linestring(n, _ptr(pgo), _ptr(x), _ptr(y), _ptr(lgo), _ptr(lpo),
                                         max(lpo.size - 1, 0), _ptr(lx), _ptr(ly),
                                         _dtype_code(x), _ptr(dist),
                                         _ptr(opt), _ptr(ols), _ptr(oseg), _ptr(oxy))
    return dict(distance=dist, point_geometry_id=opt, linestring_geometry_id=ols,
                segment_id=oseg, x=oxy[0::2].copy(), y=oxy[1::2].copy())


def quadtree_point_to_nearest_linestring(pairs, tree, point_indices, x, y, ls_offsets, lx, ly):
    lib = _load()
    pl = np.ascontiguousarray(pairs["bbox_offset"], dtype=np.uint32)
    pq = np.ascontiguousarray(pairs["quad_offset"], dtype=np.uint32)
    ln = np.ascontiguousarray(tree["length"], dtype=np.uint32)
    of = np.ascontiguousarray(tree["offset"], dtype=np.uint32)
    pi = np.ascontiguousarray(point_indices, dtype=np.uint32)
    x = np.ascontiguousarray(x)
    y = np.ascontiguousarray(y, dtype=x.dtype)
    lo = np.ascontiguousarray(ls_offsets, dtype=np.uint32)
    lx = np.ascontiguousarray(lx, dtype=x.dtype)
    ly = np.ascontiguousarray(ly, dtype=x.dtype)
    n = pi.size
    o_pt = np.empty(n, np.uint32)
    o_ls = np.empty(n, np.uint32)
    o_d = np.empty(n, x.dtype)
    lib.oracle_quadtree_point_to_nearest_linestring(
        _ptr(pl), _ptr(pq), pl.size, _ptr(ln), _ptr(of), _ptr(pi), n, _ptr(x), _ptr(y), _ptr(lo),
        _ptr(lx), _ptr(ly), _dtype_code(x), _ptr(o_pt), _ptr(o_ls), _ptr(o_d))
    return dict(point_index=o_pt, linestring_index=o_ls, distance=o_d)
