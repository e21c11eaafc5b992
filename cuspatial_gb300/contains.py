"""contains_properly for polygons against points: the three modes of
python/cuspatial/cuspatial/core/binpreds/contains.py:19-183 and the
polygon-contains-point predicate built on them
(core/binpreds/feature_contains_properly.py:66-135 with
contains_geometry_processor.py:72-152 and 250-271).

The quadtree mode runs natively (cspt_quadtree_contains_properly: the whole
chain with the reference's parameters, the point-index remap and the
part -> multipolygon map in one call); pairwise and brute-force modes run the
pairwise and bitmask kernels.  Tables are column name -> tensor mappings.
"""

import ctypes

import torch

from . import _lib
from .api import _METHODS, _dtype_code
from .geoseries import GeoSeries, Table, contains_only_points, contains_only_polygons


def _parts(polygons):
    return polygons.polygons


def _quadtree_rows(points, polygons, method="exact"):
    """(point_index, part_index, polygon_index) rows of the native chain."""
    lib = _lib.load()
    pts = points.points
    poly = _parts(polygons)
    alloc = _lib.TorchAllocator(pts.x.device)
    op, oa, og, nn = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_size_t()
    _lib.check(lib.cspt_quadtree_contains_properly(
        _lib.ptr(pts.x), _lib.ptr(pts.y), int(pts.x.numel()), _lib.ptr(poly.geometry_offset),
        int(poly.geometry_offset.numel()), _lib.ptr(poly.part_offset),
        int(poly.part_offset.numel()), _lib.ptr(poly.ring_offset), int(poly.ring_offset.numel()),
        _lib.ptr(poly.x), _lib.ptr(poly.y), int(poly.x.numel()), _dtype_code(pts.x),
        _METHODS[method], alloc.ref, _lib.stream_ptr(), ctypes.byref(op), ctypes.byref(oa),
        ctypes.byref(og), ctypes.byref(nn)), lib)
    n = int(nn.value)
    return (alloc.adopt(op.value, n, torch.int32), alloc.adopt(oa.value, n, torch.int32),
            alloc.adopt(og.value, n, torch.int32))


def _quadtree_contains_properly(points, polygons, method="exact"):
    """contains.py:19-74: (point_index, part_index) rows, point_index an
    index into `points`, in the join's row order."""
    out = Table()
    if len(polygons) == 0:
        return out
    point, part, _ = _quadtree_rows(points, polygons, method)
    out["point_index"] = point
    out["part_index"] = part
    return out


def _pairwise_flags(points, polygons, method="exact"):
    """The pairwise kernel over the parts (the binding used by
    contains.py:146), multipolygons included."""
    lib = _lib.load()
    pts = points.points
    poly = _parts(polygons)
    n = int(pts.x.numel())
    out = torch.empty(n, dtype=torch.uint8, device=pts.x.device)
    alloc = _lib.TorchAllocator(pts.x.device)
    _lib.check(lib.cspt_pairwise_point_in_polygon(
        _lib.ptr(pts.x), _lib.ptr(pts.y), n, _lib.ptr(poly.part_offset),
        int(poly.part_offset.numel()), _lib.ptr(poly.ring_offset), int(poly.ring_offset.numel()),
        _lib.ptr(poly.x), _lib.ptr(poly.y), int(poly.x.numel()), _dtype_code(pts.x),
        _METHODS[method], alloc.ref, _lib.stream_ptr(), _lib.ptr(out)), lib)
    return out


def _pairwise_contains_properly(points, polygons, method="exact"):
    """contains.py:118-168: (pairwise_index, point_index, result) of the
    pairs whose point is inside."""
    hit = _pairwise_flags(points, polygons, method)
    trues = torch.nonzero(hit, as_tuple=False).reshape(-1).to(torch.int32)
    out = Table()
    out["pairwise_index"] = trues
    out["point_index"] = trues.clone()
    out["result"] = torch.ones(trues.numel(), dtype=torch.bool, device=trues.device)
    return out


def _bitmask(points, polygons, method="exact"):
    lib = _lib.load()
    pts = points.points
    poly = _parts(polygons)
    n = int(pts.x.numel())
    mask = torch.empty(n, dtype=torch.int32, device=pts.x.device)
    alloc = _lib.TorchAllocator(pts.x.device)
    _lib.check(lib.cspt_point_in_polygon(
        _lib.ptr(pts.x), _lib.ptr(pts.y), n, _lib.ptr(poly.part_offset),
        int(poly.part_offset.numel()), _lib.ptr(poly.ring_offset), int(poly.ring_offset.numel()),
        _lib.ptr(poly.x), _lib.ptr(poly.y), int(poly.x.numel()), _dtype_code(pts.x),
        _METHODS[method], alloc.ref, _lib.stream_ptr(), _lib.ptr(mask)), lib)
    return mask


def _brute_force_contains_properly(points, polygons, method="exact"):
    """contains.py:77-115 then the stack at :176-183: (point_index,
    part_index, result) of every true cell, point-major."""
    nparts = int(_parts(polygons).part_offset.numel()) - 1
    mask = _bitmask(points, polygons, method)
    bits = torch.arange(max(nparts, 0), device=mask.device, dtype=torch.int32)
    cells = ((mask.unsqueeze(1) >> bits) & 1).bool()
    pt, pa = torch.nonzero(cells, as_tuple=True)
    out = Table()
    out["point_index"] = pt.to(torch.int32)
    out["part_index"] = pa.to(torch.int32)
    out["result"] = torch.ones(pt.numel(), dtype=torch.bool, device=mask.device)
    return out


def contains_properly(polygons: GeoSeries, points: GeoSeries, mode="pairwise",
                      method="exact"):
    """contains.py:171-183."""
    if mode == "quadtree":
        return _quadtree_contains_properly(points, polygons, method)
    if mode == "pairwise":
        return _pairwise_contains_properly(points, polygons, method)
    return _brute_force_contains_properly(points, polygons, method)


def _has_multipolygons(polygons):
    p = _parts(polygons)
    return int(p.geometry_offset.numel()) != int(p.part_offset.numel())


def pip_mode(polygons, allpairs=False):
    """feature_contains_properly.py:66-90."""
    if len(polygons) <= 31:
        return "brute_force"
    if allpairs or _has_multipolygons(polygons):
        return "quadtree"
    return "pairwise"


def _part_geometry(polygons, part):
    """contains_geometry_processor.py:72-116: each part's multipolygon."""
    go = _parts(polygons).geometry_offset.long()
    return (torch.searchsorted(go[1:], part.long(), right=True)).to(torch.int32)


def polygons_contains_properly(polygons: GeoSeries, points: GeoSeries, allpairs=False,
                               method="exact"):
    """Polygon-contains-point predicate (GeoSeries.contains_properly with a
    point right-hand side, feature_contains_properly.py:92-135 and
    contains_geometry_processor.py:118-152, 250-271).

    allpairs=True: a Table (polygon_index, point_index) of every multipolygon
    that properly contains a point, without repeats, sorted by
    (polygon_index, point_index).  Otherwise a bool tensor over the points:
    with as many polygons as points, entry i says whether polygon i contains
    point i.
    """
    if not contains_only_polygons(polygons):
        raise TypeError("`.contains` can only be called with polygon series.")
    if not contains_only_points(points):
        raise TypeError("the right-hand side must contain only points")
    mode = pip_mode(polygons, allpairs)
    npts = len(points)
    if mode == "pairwise":
        # lhs[point_indices] with point_indices = 0..n-1 (one point per row)
        if len(polygons) < npts:
            raise IndexError("fewer polygons than points in pairwise mode")
        r = _pairwise_contains_properly(points, _take_geometries(polygons, npts), method)
        point, part = r["point_index"], r["pairwise_index"]
    elif mode == "quadtree":
        r = _quadtree_contains_properly(points, polygons, method)
        point = r.get("point_index", torch.zeros(0, dtype=torch.int32, device="cuda"))
        part = r.get("part_index", torch.zeros(0, dtype=torch.int32, device="cuda"))
    else:
        r = _brute_force_contains_properly(points, polygons, method)
        point, part = r["point_index"], r["part_index"]
    geom = _part_geometry(polygons, part) if part.numel() else part
    # drop repeats: a point inside several parts of one multipolygon
    if point.numel():
        key = torch.unique(geom.long() * (1 << 32) + point.long())
        geom = (key >> 32).to(torch.int32)
        point = (key & 0xFFFFFFFF).to(torch.int32)
    if allpairs:
        out = Table()
        out["polygon_index"] = geom
        out["point_index"] = point
        return out
    result = torch.zeros(npts, dtype=torch.bool, device=points.points.x.device)
    if len(polygons) == npts:
        match = geom == point
        result[point[match].long()] = True
    else:
        # contains_geometry_processor.py:265-267: rows named by polygon
        sel = geom.long()
        result[sel[sel < npts]] = True
    return result


def _take_geometries(polygons, n):
    """The first n multipolygons (polygons[0..n-1]) as a GeoSeries."""
    p = _parts(polygons)
    if len(polygons) == n:
        return polygons
    go = p.geometry_offset[: n + 1]
    po = p.part_offset[: int(go[-1].item()) + 1]
    ro = p.ring_offset[: int(po[-1].item()) + 1]
    nv = int(ro[-1].item())
    xy = torch.stack([p.x[:nv], p.y[:nv]], 1).reshape(-1)
    return GeoSeries.from_polygons_xy(xy, ro, po, go)
