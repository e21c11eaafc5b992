"""cuSpatial-compatible Python API over the C ABI.

Signatures, argument handling (min/max swapping, scale clamping with a
warning, geometry-type checks) and column names follow
python/cuspatial/cuspatial/core/spatial/indexing.py:15-199,
join.py:105-355 and bounding.py:19-140.  The `method` keyword (exact or
filtered float32+float64 arithmetic) is an addition; it never changes results.
"""

import ctypes
import warnings

import torch

from . import _lib
from .geoseries import (MULTIPOINT, GeoSeries, Table, as_device_tensor,
                        contains_only_linestrings, contains_only_points,
                        contains_only_points_or_multipoints, contains_only_polygons)

_METHODS = {"exact": _lib.METHOD_EXACT, "filtered": _lib.METHOD_FILTERED}


def _dtype_code(t):
    if t.dtype == torch.float64:
        return _lib.FLOAT64
    if t.dtype == torch.float32:
        return _lib.FLOAT32
    raise TypeError("Only floating-point types are supported")


def _tree_struct(quadtree):
    """Table of the 5 quadtree columns -> (CsptQuadtree, tensors kept alive)."""
    cols = [quadtree["key"], quadtree["level"], quadtree["is_internal_node"],
            quadtree["length"], quadtree["offset"]]
    key = as_device_tensor(cols[0], dtype=torch.int32).view(torch.int32)
    lev = as_device_tensor(cols[1], dtype=torch.uint8)
    isi = as_device_tensor(cols[2]).to(torch.uint8).contiguous()
    ln = as_device_tensor(cols[3], dtype=torch.int32)
    of = as_device_tensor(cols[4], dtype=torch.int32)
    keep = (key, lev, isi, ln, of)
    st = _lib.CsptQuadtree(key.data_ptr() or None, lev.data_ptr() or None,
                           isi.data_ptr() or None, ln.data_ptr() or None,
                           of.data_ptr() or None, int(key.numel()))
    return st, keep


def quadtree_on_points(points: GeoSeries, x_min, x_max, y_min, y_max, scale, max_depth,
                       max_size):
    """Construct a quadtree on points (reference: core/spatial/indexing.py:15).

    Returns (point_indices, quadtree): point_indices maps sorted positions to
    input point indices; quadtree holds key, level, is_internal_node, length
    and offset.  uint32 columns are returned in int32 tensors (same bits).
    """
    return _quadtree_on_points(points, x_min, x_max, y_min, y_max, scale, max_depth, max_size,
                               False)


def quadtree_on_points_ordered(points: GeoSeries, x_min, x_max, y_min, y_max, scale, max_depth,
                               max_size):
    """quadtree_on_points that also returns the points in quadtree order.

    Returns (point_indices, quadtree, ordered_points); ordered_points equals
    points_in_quadtree_order(point_indices, points) and is built in the same
    pass (the key computation writes the points interleaved, the gather after
    the sort reads one row per point).  No counterpart in the reference.
    """
    return _quadtree_on_points(points, x_min, x_max, y_min, y_max, scale, max_depth, max_size,
                               True)


def _quadtree_on_points(points, x_min, x_max, y_min, y_max, scale, max_depth, max_size,
                        ordered):
    if not len(points) == 0 and not contains_only_points(points):
        raise ValueError("GeoSeries must contain only points.")
    lib = _lib.load()
    x_min, x_max, y_min, y_max = (min(x_min, x_max), max(x_min, x_max), min(y_min, y_max),
                                  max(y_min, y_max))
    min_scale = max(x_max - x_min, y_max - y_min) / ((1 << max_depth) + 2)
    if scale < min_scale:
        warnings.warn("scale {} is less than required minimum ".format(scale) +
                      "scale {}. Clamping to minimum scale".format(min_scale))
    xs = points.points.x if len(points) else torch.empty(0, dtype=torch.float64, device="cuda")
    ys = points.points.y if len(points) else xs
    alloc = _lib.TorchAllocator(xs.device)
    pi = ctypes.c_void_p()
    tree = _lib.CsptQuadtree()
    args = [_lib.ptr(xs), _lib.ptr(ys), int(xs.numel()), _dtype_code(xs), float(x_min),
            float(x_max), float(y_min), float(y_max), float(max(scale, min_scale)),
            int(max_depth), int(max_size), alloc.ref, _lib.stream_ptr(), ctypes.byref(pi),
            ctypes.byref(tree)]
    if not ordered:
        _lib.check(lib.cspt_quadtree_on_points(*args), lib)
        return _adopt_tree(alloc, pi, tree, int(xs.numel()))
    oxy = torch.empty((int(xs.numel()), 2), dtype=xs.dtype, device=xs.device)
    _lib.check(lib.cspt_quadtree_on_points_ordered(*args, _lib.ptr(oxy)), lib)
    return (*_adopt_tree(alloc, pi, tree, int(xs.numel())), oxy)


def _adopt_tree(alloc, pi, tree, n):
    q = int(tree.num_nodes)
    point_indices = alloc.adopt(pi.value, n, torch.int32)
    qt = Table()
    qt["key"] = alloc.adopt(tree.key, q, torch.int32)
    qt["level"] = alloc.adopt(tree.level, q, torch.uint8)
    qt["is_internal_node"] = alloc.adopt(tree.is_internal_node, q, torch.uint8).view(torch.bool)
    qt["length"] = alloc.adopt(tree.length, q, torch.int32)
    qt["offset"] = alloc.adopt(tree.offset, q, torch.int32)
    return point_indices, qt


def quadtree_on_points_host(x, y, x_min, x_max, y_min, y_max, scale, max_depth, max_size,
                            ordered=False):
    """quadtree_on_points for points in host memory.

    x and y are CPU tensors of one floating type (page-locked, for the copy to
    the device to overlap the Morton keys of the chunks already copied).
    Returns (points, point_indices, quadtree): points is a GeoSeries over the
    device copies of x and y, for the calls that follow.  ordered=True also
    returns the points in quadtree order, as quadtree_on_points_ordered does:
    (points, point_indices, quadtree, ordered_points).
    """
    for t in (x, y):
        if t.device.type != "cpu" or not t.is_contiguous():
            raise ValueError("x and y must be contiguous CPU tensors")
    if x.dtype != y.dtype or x.dtype not in (torch.float32, torch.float64):
        raise TypeError("Only floating-point types are supported")
    if x.numel() != y.numel():
        raise RuntimeError("x and y columns must have the same length")
    lib = _lib.load()
    x_min, x_max, y_min, y_max = (min(x_min, x_max), max(x_min, x_max), min(y_min, y_max),
                                  max(y_min, y_max))
    min_scale = max(x_max - x_min, y_max - y_min) / ((1 << max_depth) + 2)
    if scale < min_scale:
        warnings.warn("scale {} is less than required minimum ".format(scale) +
                      "scale {}. Clamping to minimum scale".format(min_scale))
    dx = torch.empty(x.numel(), dtype=x.dtype, device="cuda")
    dy = torch.empty(y.numel(), dtype=y.dtype, device="cuda")
    alloc = _lib.TorchAllocator(dx.device)
    pi = ctypes.c_void_p()
    tree = _lib.CsptQuadtree()
    args = [x.data_ptr() if x.numel() else None, y.data_ptr() if y.numel() else None,
            int(x.numel()), _dtype_code(x), float(x_min), float(x_max), float(y_min),
            float(y_max), float(max(scale, min_scale)), int(max_depth), int(max_size),
            _lib.ptr(dx), _lib.ptr(dy), alloc.ref, _lib.stream_ptr(), ctypes.byref(pi),
            ctypes.byref(tree)]
    if not ordered:
        _lib.check(lib.cspt_quadtree_on_points_host(*args), lib)
        point_indices, qt = _adopt_tree(alloc, pi, tree, int(x.numel()))
        return GeoSeries.from_points(dx, dy), point_indices, qt
    oxy = torch.empty((int(x.numel()), 2), dtype=x.dtype, device="cuda")
    _lib.check(lib.cspt_quadtree_on_points_host_ordered(*args, _lib.ptr(oxy)), lib)
    point_indices, qt = _adopt_tree(alloc, pi, tree, int(x.numel()))
    return GeoSeries.from_points(dx, dy), point_indices, qt, oxy


def _empty_boxes(dtype):
    t = Table()
    for k in ("minx", "miny", "maxx", "maxy"):
        t[k] = torch.empty(0, dtype=dtype, device="cuda")
    return t


def polygon_bounding_boxes(polygons: GeoSeries):
    """Per-polygon bounding boxes (reference: core/spatial/bounding.py:19)."""
    if len(polygons) == 0:
        return _empty_boxes(torch.float64)
    if not contains_only_polygons(polygons):
        raise ValueError("Geoseries must contain only polygons.")
    lib = _lib.load()
    p = polygons.polygons
    n = int(p.part_offset.numel()) - 1
    out = Table()
    for k in ("minx", "miny", "maxx", "maxy"):
        out[k] = torch.empty(n, dtype=p.x.dtype, device=p.x.device)
    _lib.check(lib.cspt_polygon_bounding_boxes(
        _lib.ptr(p.part_offset), int(p.part_offset.numel()), _lib.ptr(p.ring_offset),
        int(p.ring_offset.numel()), _lib.ptr(p.x), _lib.ptr(p.y), int(p.x.numel()),
        _dtype_code(p.x), 0.0, *[_lib.ptr(v) for v in out.values()], _lib.stream_ptr()), lib)
    return out


def linestring_bounding_boxes(linestrings: GeoSeries, expansion_radius: float):
    """Per-linestring bounding boxes expanded by a radius (bounding.py:89)."""
    if len(linestrings) == 0:
        return _empty_boxes(torch.float64)
    if not contains_only_linestrings(linestrings):
        raise ValueError("Geoseries must contain only linestrings.")
    lib = _lib.load()
    ls = linestrings.lines
    # part offsets of the first part of each geometry (bounding.py:125-127)
    offsets = ls.part_offset[ls.geometry_offset.long()].contiguous()
    n = int(offsets.numel()) - 1
    out = Table()
    for k in ("minx", "miny", "maxx", "maxy"):
        out[k] = torch.empty(n, dtype=ls.x.dtype, device=ls.x.device)
    _lib.check(lib.cspt_linestring_bounding_boxes(
        _lib.ptr(offsets), int(offsets.numel()), _lib.ptr(ls.x), _lib.ptr(ls.y),
        int(ls.x.numel()), _dtype_code(ls.x), float(expansion_radius),
        *[_lib.ptr(v) for v in out.values()], _lib.stream_ptr()), lib)
    return out


def join_quadtree_and_bounding_boxes(quadtree, bounding_boxes, x_min, x_max, y_min, y_max,
                                     scale, max_depth):
    """(bbox, leaf quadrant) pairs that intersect (reference: join.py:105)."""
    lib = _lib.load()
    x_min, x_max, y_min, y_max = (min(x_min, x_max), max(x_min, x_max), min(y_min, y_max),
                                  max(y_min, y_max))
    min_scale = max(x_max - x_min, y_max - y_min) / ((1 << max_depth) + 2)
    if scale < min_scale:
        warnings.warn("scale {} is less than required minimum ".format(scale) +
                      "scale {}. Clamping to minimum scale".format(min_scale))
    st, keep = _tree_struct(quadtree)
    b = [as_device_tensor(bounding_boxes[k]) for k in ("minx", "miny", "maxx", "maxy")]
    alloc = _lib.TorchAllocator(b[0].device)
    ob, oq, nn = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_size_t()
    _lib.check(lib.cspt_join_quadtree_and_bounding_boxes(
        ctypes.byref(st), *[_lib.ptr(v) for v in b], int(b[0].numel()), _dtype_code(b[0]),
        float(x_min), float(x_max), float(y_min), float(y_max), float(max(scale, min_scale)),
        int(max_depth), alloc.ref, _lib.stream_ptr(), ctypes.byref(ob), ctypes.byref(oq),
        ctypes.byref(nn)), lib)
    del keep
    n = int(nn.value)
    out = Table()
    out["bbox_offset"] = alloc.adopt(ob.value, n, torch.int32)
    out["quad_offset"] = alloc.adopt(oq.value, n, torch.int32)
    return out


def points_in_quadtree_order(point_indices, points: GeoSeries):
    """The points gathered into quadtree order: an (n, 2) tensor whose row i
    is (x, y) of point point_indices[i].

    No counterpart in the reference.  quadtree_point_in_polygon and
    quadtree_point_to_nearest_linestring take it as `ordered_points`, and then
    read each quadrant's points contiguously instead of through point_indices
    on every call; build it once per quadtree.
    """
    if not contains_only_points(points):
        raise ValueError("`point` Geoseries must contains only point geometries.")
    lib = _lib.load()
    pi = as_device_tensor(point_indices, dtype=torch.int32)
    pts = points.points
    out = torch.empty((int(pi.numel()), 2), dtype=pts.x.dtype, device=pts.x.device)
    _lib.check(lib.cspt_points_in_quadtree_order(
        _lib.ptr(pi), int(pi.numel()), _lib.ptr(pts.x), _lib.ptr(pts.y), int(pts.x.numel()),
        _dtype_code(pts.x), _lib.ptr(out), _lib.stream_ptr()), lib)
    return out


def _check_ordered(ordered_points, point_indices, points):
    """ordered_points must be points_in_quadtree_order(point_indices, points)."""
    t = ordered_points
    if not isinstance(t, torch.Tensor) or t.dim() != 2 or t.shape[1] != 2 or \
            not t.is_contiguous() or t.device.type != "cuda":
        raise ValueError("ordered_points must be the contiguous (n, 2) CUDA tensor that "
                         "points_in_quadtree_order returns")
    if int(t.shape[0]) != int(point_indices.numel()) or t.dtype != points.points.x.dtype:
        raise ValueError("ordered_points must hold one row per point index, in the points' "
                         "dtype")


def quadtree_point_in_polygon(poly_quad_pairs, quadtree, point_indices, points: GeoSeries,
                              polygons: GeoSeries, method="exact", ordered_points=None):
    """Points inside polygons, using (polygon, quadrant) pairs (join.py:177).

    point_index in the result is a position in point_indices (an index to an
    index), as in the reference.  method="filtered" runs the float32 filter
    with float64 refinement; the pairs are identical to method="exact".
    ordered_points (optional): points_in_quadtree_order(point_indices, points);
    the result is the same, the points are read in order.
    """
    if not contains_only_points(points):
        raise ValueError("`point` Geoseries must contains only point geometries.")
    if not contains_only_polygons(polygons):
        raise ValueError("`polygons` Geoseries must contains only polygons geometries.")
    lib = _lib.load()
    st, keep = _tree_struct(quadtree)
    pp = as_device_tensor(poly_quad_pairs["bbox_offset"] if "bbox_offset" in poly_quad_pairs
                          else poly_quad_pairs["polygon_index"], dtype=torch.int32)
    pq = as_device_tensor(poly_quad_pairs["quad_offset"], dtype=torch.int32)
    pi = as_device_tensor(point_indices, dtype=torch.int32)
    pts = points.points
    poly = polygons.polygons
    alloc = _lib.TorchAllocator(pts.x.device)
    op, oq, nn = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_size_t()
    if ordered_points is not None:
        _check_ordered(ordered_points, pi, points)
        _lib.check(lib.cspt_quadtree_point_in_polygon_ordered(
            _lib.ptr(pp), _lib.ptr(pq), int(pp.numel()), ctypes.byref(st),
            _lib.ptr(ordered_points), int(pi.numel()), _lib.ptr(poly.part_offset),
            int(poly.part_offset.numel()), _lib.ptr(poly.ring_offset),
            int(poly.ring_offset.numel()), _lib.ptr(poly.x), _lib.ptr(poly.y),
            int(poly.x.numel()), _dtype_code(pts.x), _METHODS[method], alloc.ref,
            _lib.stream_ptr(), ctypes.byref(op), ctypes.byref(oq), ctypes.byref(nn)), lib)
    else:
        _lib.check(lib.cspt_quadtree_point_in_polygon(
            _lib.ptr(pp), _lib.ptr(pq), int(pp.numel()), ctypes.byref(st), _lib.ptr(pi),
            int(pi.numel()), _lib.ptr(pts.x), _lib.ptr(pts.y), int(pts.x.numel()),
            _lib.ptr(poly.part_offset), int(poly.part_offset.numel()),
            _lib.ptr(poly.ring_offset), int(poly.ring_offset.numel()), _lib.ptr(poly.x),
            _lib.ptr(poly.y), int(poly.x.numel()), _dtype_code(pts.x), _METHODS[method],
            alloc.ref, _lib.stream_ptr(), ctypes.byref(op), ctypes.byref(oq),
            ctypes.byref(nn)), lib)
    del keep
    n = int(nn.value)
    out = Table()
    out["polygon_index"] = alloc.adopt(op.value, n, torch.int32)
    out["point_index"] = alloc.adopt(oq.value, n, torch.int32)
    return out


class HostRowsTooFew(RuntimeError):
    """The host arrays given to quadtree_point_in_polygon_host hold fewer rows
    than the result; `rows` is the result's row count."""

    def __init__(self, msg, rows):
        super().__init__(msg)
        self.rows = rows


def quadtree_point_in_polygon_host(poly_quad_pairs, quadtree, point_indices, points: GeoSeries,
                                   polygons: GeoSeries, polygon_index_out, point_index_out,
                                   method="exact", ordered_points=None):
    """quadtree_point_in_polygon with the rows written into host tensors.

    polygon_index_out and point_index_out are int32 CPU tensors of equal
    length (page-locked, for the device-to-host copies to overlap the
    evaluation, which runs in chunks of pairs).  Returns the number of rows
    written, in the order of quadtree_point_in_polygon.  Raises HostRowsTooFew
    (with the row count) when the tensors are too short.  ordered_points as in
    quadtree_point_in_polygon.
    """
    if not contains_only_points(points):
        raise ValueError("`point` Geoseries must contains only point geometries.")
    if not contains_only_polygons(polygons):
        raise ValueError("`polygons` Geoseries must contains only polygons geometries.")
    for t in (polygon_index_out, point_index_out):
        if t.device.type != "cpu" or t.dtype != torch.int32 or not t.is_contiguous():
            raise ValueError("host outputs must be contiguous int32 CPU tensors")
    cap = min(int(polygon_index_out.numel()), int(point_index_out.numel()))
    lib = _lib.load()
    st, keep = _tree_struct(quadtree)
    pp = as_device_tensor(poly_quad_pairs["bbox_offset"] if "bbox_offset" in poly_quad_pairs
                          else poly_quad_pairs["polygon_index"], dtype=torch.int32)
    pq = as_device_tensor(poly_quad_pairs["quad_offset"], dtype=torch.int32)
    pi = as_device_tensor(point_indices, dtype=torch.int32)
    pts = points.points
    poly = polygons.polygons
    alloc = _lib.TorchAllocator(pts.x.device)
    nn = ctypes.c_size_t()
    host_p = polygon_index_out.data_ptr() if cap else None
    host_q = point_index_out.data_ptr() if cap else None
    if ordered_points is not None:
        _check_ordered(ordered_points, pi, points)
        status = lib.cspt_quadtree_point_in_polygon_host_ordered(
            _lib.ptr(pp), _lib.ptr(pq), int(pp.numel()), ctypes.byref(st),
            _lib.ptr(ordered_points), int(pi.numel()), _lib.ptr(poly.part_offset),
            int(poly.part_offset.numel()), _lib.ptr(poly.ring_offset),
            int(poly.ring_offset.numel()), _lib.ptr(poly.x), _lib.ptr(poly.y),
            int(poly.x.numel()), _dtype_code(pts.x), _METHODS[method], alloc.ref,
            _lib.stream_ptr(), host_p, host_q, cap, ctypes.byref(nn))
    else:
        status = lib.cspt_quadtree_point_in_polygon_host(
            _lib.ptr(pp), _lib.ptr(pq), int(pp.numel()), ctypes.byref(st), _lib.ptr(pi),
            int(pi.numel()), _lib.ptr(pts.x), _lib.ptr(pts.y), int(pts.x.numel()),
            _lib.ptr(poly.part_offset), int(poly.part_offset.numel()),
            _lib.ptr(poly.ring_offset), int(poly.ring_offset.numel()), _lib.ptr(poly.x),
            _lib.ptr(poly.y), int(poly.x.numel()), _dtype_code(pts.x), _METHODS[method],
            alloc.ref, _lib.stream_ptr(), host_p, host_q, cap, ctypes.byref(nn))
    del keep
    if status != _lib.OK and int(nn.value) > cap:
        raise HostRowsTooFew(lib.cspt_last_error_message().decode(), int(nn.value))
    _lib.check(status, lib)
    return int(nn.value)


def point_in_polygon_join_host(x, y, x_min, x_max, y_min, y_max, scale, max_depth, max_size,
                               poly_offsets, ring_offsets, poly_x, poly_y, polygon_index_out,
                               point_index_out, method="exact"):
    """The whole quadtree point-in-polygon join from host columns to host rows
    in one call (no counterpart in cuSpatial).

    x, y: the points (float64 or float32 CPU tensors); poly_offsets,
    ring_offsets (int32), poly_x, poly_y: single-ring-list polygons in the
    layout quadtree_point_in_polygon reads (part and ring offsets), all on
    the host, page-locked for the copies to overlap the work.  The rows are
    those of quadtree_on_points -> polygon_bounding_boxes ->
    join_quadtree_and_bounding_boxes -> quadtree_point_in_polygon, in that
    order, with the point column holding each point's index in x / y
    (point_indices[point_index] of the separate calls).  Corners are ordered
    and the scale clamped as join_quadtree_and_bounding_boxes does.  Returns
    the number of rows written; raises HostRowsTooFew when the outputs are
    too short.
    """
    cols = (x, y, poly_offsets, ring_offsets, poly_x, poly_y, polygon_index_out,
            point_index_out)
    for t in cols:
        if not isinstance(t, torch.Tensor) or t.device.type != "cpu" or not t.is_contiguous():
            raise ValueError("inputs and outputs must be contiguous CPU tensors")
    if x.dtype != y.dtype or poly_x.dtype != x.dtype or poly_y.dtype != x.dtype:
        raise TypeError("point and polygon coordinates must share one floating-point dtype")
    if x.numel() != y.numel() or poly_x.numel() != poly_y.numel():
        raise ValueError("x and y columns must have the same length")
    for t in (poly_offsets, ring_offsets, polygon_index_out, point_index_out):
        if t.dtype != torch.int32:
            raise TypeError("offsets and outputs must be int32")
    x_min, x_max = min(x_min, x_max), max(x_min, x_max)
    y_min, y_max = min(y_min, y_max), max(y_min, y_max)
    min_scale = max(x_max - x_min, y_max - y_min) / ((1 << max_depth) + 2)
    if scale < min_scale:
        warnings.warn("scale {} is less than required minimum ".format(scale) +
                      "scale {}. Clamping to minimum scale".format(min_scale))
    cap = min(int(polygon_index_out.numel()), int(point_index_out.numel()))
    lib = _lib.load()
    alloc = _lib.TorchAllocator(torch.device("cuda", torch.cuda.current_device()))
    nn = ctypes.c_size_t()
    status = lib.cspt_point_in_polygon_join_host(
        x.data_ptr(), y.data_ptr(), int(x.numel()), _dtype_code(x), float(x_min), float(x_max),
        float(y_min), float(y_max), float(scale), int(max_depth), int(max_size),
        poly_offsets.data_ptr(), int(poly_offsets.numel()), ring_offsets.data_ptr(),
        int(ring_offsets.numel()), poly_x.data_ptr(), poly_y.data_ptr(), int(poly_x.numel()),
        _METHODS[method], alloc.ref, _lib.stream_ptr(),
        polygon_index_out.data_ptr() if cap else None,
        point_index_out.data_ptr() if cap else None, cap, ctypes.byref(nn))
    if status != _lib.OK and int(nn.value) > cap:
        raise HostRowsTooFew(lib.cspt_last_error_message().decode(), int(nn.value))
    _lib.check(status, lib)
    return int(nn.value)


def quadtree_point_to_nearest_linestring(linestring_quad_pairs, quadtree, point_indices,
                                         points: GeoSeries, linestrings: GeoSeries,
                                         method="exact", ordered_points=None):
    """Nearest linestring of each point in the paired quadrants (join.py:265).

    ordered_points (optional): points_in_quadtree_order(point_indices, points);
    the rows are the same, the points are read in order.
    """
    if not contains_only_points(points):
        raise ValueError("`point` Geoseries must contains only point geometries.")
    if not contains_only_linestrings(linestrings):
        raise ValueError("`linestrings` Geoseries must contains only linestring geometries.")
    ls = linestrings.lines
    if int(ls.part_offset.numel()) != int(ls.geometry_offset.numel()):
        raise ValueError("GeoSeries cannot contain multilinestrings.")
    lib = _lib.load()
    st, keep = _tree_struct(quadtree)
    pl = as_device_tensor(linestring_quad_pairs["bbox_offset"] if "bbox_offset" in
                          linestring_quad_pairs else linestring_quad_pairs["linestring_index"],
                          dtype=torch.int32)
    pq = as_device_tensor(linestring_quad_pairs["quad_offset"], dtype=torch.int32)
    pi = as_device_tensor(point_indices, dtype=torch.int32)
    pts = points.points
    n = int(pi.numel())
    o_pt = torch.empty(n, dtype=torch.int32, device=pts.x.device)
    o_ls = torch.empty(n, dtype=torch.int32, device=pts.x.device)
    o_d = torch.empty(n, dtype=pts.x.dtype, device=pts.x.device)
    alloc = _lib.TorchAllocator(pts.x.device)
    rows = ctypes.c_size_t()
    if ordered_points is not None:
        _check_ordered(ordered_points, pi, points)
        _lib.check(lib.cspt_quadtree_point_to_nearest_linestring_ordered(
            _lib.ptr(pl), _lib.ptr(pq), int(pl.numel()), ctypes.byref(st),
            _lib.ptr(ordered_points), n, _lib.ptr(ls.part_offset), int(ls.part_offset.numel()),
            _lib.ptr(ls.x), _lib.ptr(ls.y), int(ls.x.numel()), _dtype_code(pts.x),
            _METHODS[method], alloc.ref, _lib.stream_ptr(), _lib.ptr(o_pt), _lib.ptr(o_ls),
            _lib.ptr(o_d), ctypes.byref(rows)), lib)
    else:
        _lib.check(lib.cspt_quadtree_point_to_nearest_linestring(
            _lib.ptr(pl), _lib.ptr(pq), int(pl.numel()), ctypes.byref(st), _lib.ptr(pi), n,
            _lib.ptr(pts.x), _lib.ptr(pts.y), int(pts.x.numel()), _lib.ptr(ls.part_offset),
            int(ls.part_offset.numel()), _lib.ptr(ls.x), _lib.ptr(ls.y), int(ls.x.numel()),
            _dtype_code(pts.x), _METHODS[method], alloc.ref, _lib.stream_ptr(), _lib.ptr(o_pt),
            _lib.ptr(o_ls), _lib.ptr(o_d), ctypes.byref(rows)), lib)
    del keep
    r = int(rows.value)
    out = Table()
    out["point_index"] = o_pt[:r]
    out["linestring_index"] = o_ls[:r]
    out["distance"] = o_d[:r]
    return out


def _single_polygons(polygons):
    poly = polygons.polygons
    # the C++ API takes single polygons only (join.py:69-74)
    if int(poly.part_offset.numel()) != int(poly.geometry_offset.numel()):
        raise ValueError("GeoSeries cannot contain multipolygon.")
    return poly


def point_in_polygon(points: GeoSeries, polygons: GeoSeries, method="exact"):
    """Which points fall in which of at most 31 polygons (join.py:23-102).

    Returns a Table with one bool column per polygon, named by the polygon's
    position (the reference names them by the GeoSeries index, 0..n-1 by
    default); an empty Table when there are no polygons.
    """
    if len(polygons) == 0:
        return Table()
    if not contains_only_points(points):
        raise ValueError("`point` Geoseries must contains only point geometries.")
    if not contains_only_polygons(polygons):
        raise ValueError("`polygons` Geoseries must contains only polygons geometries.")
    poly = _single_polygons(polygons)
    mask = point_in_polygon_bitmask(points, polygons, method)
    out = Table()
    for p in range(int(poly.part_offset.numel()) - 1):
        out[p] = ((mask >> p) & 1).bool()
    return out


def point_in_polygon_bitmask(points: GeoSeries, polygons: GeoSeries, method="exact"):
    """The C++ API's int32 column (point_in_polygon.hpp:75): bit p of row i
    is point i inside polygon p."""
    poly = polygons.polygons
    pts = points.points
    n = int(pts.x.numel())
    mask = torch.empty(n, dtype=torch.int32, device=pts.x.device)
    lib = _lib.load()
    alloc = _lib.TorchAllocator(pts.x.device)
    _lib.check(lib.cspt_point_in_polygon(
        _lib.ptr(pts.x), _lib.ptr(pts.y), n, _lib.ptr(poly.part_offset),
        int(poly.part_offset.numel()), _lib.ptr(poly.ring_offset), int(poly.ring_offset.numel()),
        _lib.ptr(poly.x), _lib.ptr(poly.y), int(poly.x.numel()), _dtype_code(pts.x),
        _METHODS[method], alloc.ref, _lib.stream_ptr(), _lib.ptr(mask)), lib)
    return mask


def pairwise_point_in_polygon(points: GeoSeries, polygons: GeoSeries, method="exact"):
    """Point i against polygon i (point_in_polygon.hpp:124; the binding
    used by core/binpreds/contains.py:146): a uint8 column, 1 inside."""
    if not contains_only_points(points):
        raise ValueError("`point` Geoseries must contains only point geometries.")
    if not contains_only_polygons(polygons):
        raise ValueError("`polygons` Geoseries must contains only polygons geometries.")
    poly = _single_polygons(polygons)
    lib = _lib.load()
    pts = points.points
    n = int(pts.x.numel())
    out = torch.empty(n, dtype=torch.uint8, device=pts.x.device)
    alloc = _lib.TorchAllocator(pts.x.device)
    _lib.check(lib.cspt_pairwise_point_in_polygon(
        _lib.ptr(pts.x), _lib.ptr(pts.y), n, _lib.ptr(poly.part_offset),
        int(poly.part_offset.numel()), _lib.ptr(poly.ring_offset), int(poly.ring_offset.numel()),
        _lib.ptr(poly.x), _lib.ptr(poly.y), int(poly.x.numel()), _dtype_code(pts.x),
        _METHODS[method], alloc.ref, _lib.stream_ptr(), _lib.ptr(out)), lib)
    return out


def _point_linestring_args(points, linestrings):
    """C-ABI arguments shared by the pairwise point-linestring calls."""
    if points.kind == MULTIPOINT:
        mp = points.multipoints
        pgo, px, py = mp.geometry_offset, mp.x, mp.y
    else:
        pgo, px, py = None, points.points.x, points.points.y
    ls = linestrings.lines
    n = len(points)
    args = (_lib.ptr(pgo) if pgo is not None else None,
            int(pgo.numel()) if pgo is not None else 0, _lib.ptr(px), _lib.ptr(py),
            int(px.numel()), _lib.ptr(ls.geometry_offset), int(ls.geometry_offset.numel()),
            _lib.ptr(ls.part_offset), int(ls.part_offset.numel()), _lib.ptr(ls.x),
            _lib.ptr(ls.y), int(ls.x.numel()), _dtype_code(px))
    return n, px, args


def pairwise_point_linestring_distance(points: GeoSeries, linestrings: GeoSeries,
                                       method="exact"):
    """Distance of (multi)point i to (multi)linestring i (distance.py:317):
    the smallest distance between any of its points and any segment."""
    if not contains_only_points_or_multipoints(points):
        raise ValueError("`points` array must contain only points")
    if not contains_only_linestrings(linestrings):
        raise ValueError("`linestrings` array must contain only linestrings")
    lib = _lib.load()
    n, px, args = _point_linestring_args(points, linestrings)
    out = torch.empty(n, dtype=px.dtype, device=px.device)
    _lib.check(lib.cspt_pairwise_point_linestring_distance(
        *args, _METHODS[method], _lib.stream_ptr(), _lib.ptr(out)), lib)
    return out


def pairwise_point_linestring_nearest_points(points: GeoSeries, linestrings: GeoSeries,
                                             method="exact"):
    """Nearest points between (multi)point i and (multi)linestring i
    (nearest_points.py:16-124): a Table with point_geometry_id (0 for
    single points), linestring_geometry_id, segment_id and geometry (the
    nearest points on the linestrings, a point GeoSeries)."""
    if not contains_only_points_or_multipoints(points):
        raise ValueError("`points` must contain only point geometries.")
    if not contains_only_linestrings(linestrings):
        raise ValueError("`linestrings` must contain only linestring geometries.")
    lib = _lib.load()
    n, px, args = _point_linestring_args(points, linestrings)
    dev = px.device
    opt = torch.zeros(n, dtype=torch.int32, device=dev)
    ols = torch.empty(n, dtype=torch.int32, device=dev)
    oseg = torch.empty(n, dtype=torch.int32, device=dev)
    oxy = torch.empty(2 * n, dtype=px.dtype, device=dev)
    _lib.check(lib.cspt_pairwise_point_linestring_nearest_points(
        *args, _METHODS[method], _lib.stream_ptr(),
        _lib.ptr(opt) if points.kind == MULTIPOINT else None, _lib.ptr(ols), _lib.ptr(oseg),
        _lib.ptr(oxy)), lib)
    out = Table()
    out["point_geometry_id"] = opt
    out["linestring_geometry_id"] = ols
    out["segment_id"] = oseg
    out["geometry"] = GeoSeries.from_points_xy(oxy)
    return out


def last_refined_count():
    """Candidates re-evaluated in float64 by the last filtered PiP call."""
    return int(_lib.load().cspt_last_refined_count())


def last_edge_free_pairs():
    """(polygon, quadrant) pairs the last filtered PiP call decided whole
    (no edge near the quadrant's points)."""
    return int(_lib.load().cspt_last_edge_free_pairs())


def last_nearest_stats():
    """Paths of the last filtered float64 nearest-linestring call on this
    thread: {"points_folded_whole": points folded over every candidate in
    float64, "groups_scanned": quadrant groups scanned point by point instead
    of through their segment list, "float64_segments": listed segments whose
    distance was evaluated in float64}."""
    a, b, c = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
    _lib.load().cspt_last_nearest_stats(ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
    return {"points_folded_whole": int(a.value), "groups_scanned": int(b.value),
            "float64_segments": int(c.value)}
