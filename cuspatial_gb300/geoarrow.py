"""GeoArrow in and out.

Ingestion goes through the Arrow C data interface into the library
(cspt_geoarrow_import): the reference's dense union of points /
multipoints / (multi)linestrings / (multi)polygons
(python/cuspatial/cuspatial/io/pygeoarrow.py:9-70, GeoSeries.from_arrow in
core/geoseries.py:427-440) and native GeoArrow arrays (interleaved or struct
points, nested lists, the type from the "ARROW:extension:name" metadata or a
`kind` argument) become a device GeoSeries with one host->device copy per
buffer.  Export builds pyarrow arrays from the device buffers: the
reference's union layout (GeoSeries.to_arrow, core/geoseries.py:536-627) or
native GeoArrow with its extension name.

pyarrow is needed only by from_geoarrow / to_arrow / to_geoarrow; any other
Arrow producer can hand its C structures to from_arrow_c.
"""

import ctypes

import numpy as np
import torch

from . import _lib
from .geoseries import (LINESTRING, MULTIPOINT, POINT, POLYGON, GeoSeries, _Coords,
                        as_device_tensor)

_vp = ctypes.c_void_p
_sz = ctypes.c_size_t


class ArrowSchema(ctypes.Structure):
    pass


ArrowSchema._fields_ = [
    ("format", ctypes.c_char_p), ("name", ctypes.c_char_p), ("metadata", _vp),
    ("flags", ctypes.c_int64), ("n_children", ctypes.c_int64),
    ("children", ctypes.POINTER(ctypes.POINTER(ArrowSchema))),
    ("dictionary", ctypes.POINTER(ArrowSchema)), ("release", _vp), ("private_data", _vp)]


class ArrowArray(ctypes.Structure):
    pass


ArrowArray._fields_ = [
    ("length", ctypes.c_int64), ("null_count", ctypes.c_int64), ("offset", ctypes.c_int64),
    ("n_buffers", ctypes.c_int64), ("n_children", ctypes.c_int64),
    ("buffers", ctypes.POINTER(_vp)), ("children", ctypes.POINTER(ctypes.POINTER(ArrowArray))),
    ("dictionary", ctypes.POINTER(ArrowArray)), ("release", _vp), ("private_data", _vp)]


class Layout(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("multi", ctypes.c_int), ("interleaved", ctypes.c_int),
                ("dtype", ctypes.c_int), ("num_geometries", _sz),
                ("num_geometry_offsets", _sz), ("num_part_offsets", _sz),
                ("num_ring_offsets", _sz), ("num_points", _sz)]


class GeometryColumn(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("dtype", ctypes.c_int), ("num_geometries", _sz),
                ("geometry_offsets", _vp), ("num_geometry_offsets", _sz),
                ("part_offsets", _vp), ("num_part_offsets", _sz),
                ("ring_offsets", _vp), ("num_ring_offsets", _sz),
                ("x", _vp), ("y", _vp), ("num_points", _sz)]


KINDS = {None: -1, "point": 0, "multipoint": 1, "linestring": 2, "multilinestring": 2,
         "polygon": 3, "multipolygon": 3}
_SERIES_KIND = {0: POINT, 1: MULTIPOINT, 2: LINESTRING, 3: POLYGON}


def _bind(lib):
    if getattr(lib, "_geoarrow_bound", False):
        return lib
    sp, ap = ctypes.POINTER(ArrowSchema), ctypes.POINTER(ArrowArray)
    lib.cspt_geoarrow_describe.argtypes = [sp, ap, ctypes.c_int, ctypes.POINTER(Layout)]
    lib.cspt_geoarrow_read_host.argtypes = [sp, ap, ctypes.c_int, _vp, _vp, _vp, _vp, _vp]
    lib.cspt_geoarrow_import.argtypes = [sp, ap, ctypes.c_int, ctypes.POINTER(_lib.CsptAllocator),
                                         _vp, ctypes.POINTER(GeometryColumn)]
    lib._geoarrow_bound = True
    return lib


def describe_c(schema, array, kind=None):
    """Layout of an Arrow C array (host only)."""
    lib = _bind(_lib.load())
    out = Layout()
    _lib.check(lib.cspt_geoarrow_describe(ctypes.byref(schema), ctypes.byref(array),
                                          KINDS[kind], ctypes.byref(out)), lib)
    return {k: getattr(out, k) for k, _ in Layout._fields_}


def read_host_c(schema, array, kind=None):
    """The columns as numpy arrays (host only): geometry_offset,
    part_offset, ring_offset (None where absent), x, y."""
    lib = _bind(_lib.load())
    lay = describe_c(schema, array, kind)
    dt = np.float64 if lay["dtype"] == _lib.FLOAT64 else np.float32
    go = np.zeros(lay["num_geometry_offsets"], np.uint32)
    po = np.zeros(lay["num_part_offsets"], np.uint32)
    ro = np.zeros(lay["num_ring_offsets"], np.uint32)
    x = np.zeros(lay["num_points"], dt)
    y = np.zeros(lay["num_points"], dt)
    p = lambda a: a.ctypes.data_as(_vp) if a.size else None  # noqa: E731
    _lib.check(lib.cspt_geoarrow_read_host(ctypes.byref(schema), ctypes.byref(array),
                                           KINDS[kind], p(go), p(po), p(ro), p(x), p(y)), lib)
    return dict(kind=lay["kind"], geometry_offset=go if go.size else None,
                part_offset=po if po.size else None, ring_offset=ro if ro.size else None,
                x=x, y=y)


def from_arrow_c(schema, array, kind=None, device=None):
    """A GeoSeries on the device from Arrow C structures (ArrowSchema and
    ArrowArray instances of this module, or anything laid out like them)."""
    lib = _bind(_lib.load())
    dev = torch.device(device) if device is not None else torch.device(
        "cuda", torch.cuda.current_device())
    alloc = _lib.TorchAllocator(dev)
    col = GeometryColumn()
    _lib.check(lib.cspt_geoarrow_import(ctypes.byref(schema), ctypes.byref(array), KINDS[kind],
                                        alloc.ref, _lib.stream_ptr(), ctypes.byref(col)), lib)
    ct = torch.float64 if col.dtype == _lib.FLOAT64 else torch.float32
    x = alloc.adopt(col.x, col.num_points, ct)
    y = alloc.adopt(col.y, col.num_points, ct)
    offs = {}
    for name, ptr, cnt in (("geometry_offset", col.geometry_offsets, col.num_geometry_offsets),
                           ("part_offset", col.part_offsets, col.num_part_offsets),
                           ("ring_offset", col.ring_offsets, col.num_ring_offsets)):
        if cnt:
            offs[name] = alloc.adopt(ptr, cnt, torch.int32)
    kind_s = _SERIES_KIND[col.kind]
    if kind_s == MULTIPOINT and "geometry_offset" not in offs:
        offs["geometry_offset"] = torch.zeros(1, dtype=torch.int32, device=dev)
    if kind_s in (LINESTRING, POLYGON):
        offs.setdefault("geometry_offset", torch.zeros(1, dtype=torch.int32, device=dev))
        offs.setdefault("part_offset", torch.zeros(1, dtype=torch.int32, device=dev))
    if kind_s == POLYGON:
        offs.setdefault("ring_offset", torch.zeros(1, dtype=torch.int32, device=dev))
    return GeoSeries(kind_s, _Coords(x, y, **offs), int(col.num_geometries))


_release_schema = ctypes.CFUNCTYPE(None, ctypes.POINTER(ArrowSchema))
_release_array = ctypes.CFUNCTYPE(None, ctypes.POINTER(ArrowArray))


def _exported(arr, field=None):
    """(ArrowSchema, ArrowArray) exported by pyarrow; the caller releases."""
    schema, array = ArrowSchema(), ArrowArray()
    (field if field is not None else arr.type)._export_to_c(ctypes.addressof(schema))
    arr._export_to_c(ctypes.addressof(array))
    return schema, array


def _release(schema, array):
    if array.release:
        _release_array(array.release)(ctypes.byref(array))
    if schema.release:
        _release_schema(schema.release)(ctypes.byref(schema))


def from_geoarrow(arr, kind=None, field=None, device=None):
    """A GeoSeries on the device from a pyarrow array: the reference's union
    (GeoSeries.to_arrow's layout) or native GeoArrow.  `field` carries the
    geoarrow extension metadata when the array itself does not; otherwise
    give `kind` ("point", "multipoint", "linestring", "multilinestring",
    "polygon", "multipolygon")."""
    schema, array = _exported(arr, field)
    try:
        return from_arrow_c(schema, array, kind, device)
    finally:
        _release(schema, array)


def _host(gs):
    c = gs._coords
    get = lambda n: getattr(c, n).cpu().numpy() if hasattr(c, n) else None  # noqa: E731
    return (c.x.cpu().numpy(), c.y.cpu().numpy(), get("geometry_offset"), get("part_offset"),
            get("ring_offset"))


def _native(pa, kind, x, y, go, po, ro, interleaved=True):
    """Native GeoArrow array from host buffers."""
    ft = pa.float64() if x.dtype == np.float64 else pa.float32()
    if interleaved:
        xy = np.empty(2 * len(x), x.dtype)
        xy[0::2], xy[1::2] = x, y
        pts = pa.FixedSizeListArray.from_arrays(pa.array(xy, type=ft), 2)
    else:
        pts = pa.StructArray.from_arrays([pa.array(x, type=ft), pa.array(y, type=ft)],
                                         names=["x", "y"])
    i32 = lambda a: pa.array(a.astype(np.int32), type=pa.int32())  # noqa: E731
    if kind == POINT:
        return pts, "geoarrow.point"
    if kind == MULTIPOINT:
        return pa.ListArray.from_arrays(i32(go), pts), "geoarrow.multipoint"
    if kind == LINESTRING:
        lines = pa.ListArray.from_arrays(i32(po), pts)
        return pa.ListArray.from_arrays(i32(go), lines), "geoarrow.multilinestring"
    rings = pa.ListArray.from_arrays(i32(ro), pts)
    polys = pa.ListArray.from_arrays(i32(po), rings)
    return pa.ListArray.from_arrays(i32(go), polys), "geoarrow.multipolygon"


def to_geoarrow(gs, interleaved=True):
    """(pyarrow field, array) in native GeoArrow: linestrings and polygons as
    their multi types (this library's columns always carry geometry
    offsets), the extension name in the field's metadata."""
    import pyarrow as pa
    arr, name = _native(pa, gs.kind, *_host(gs), interleaved=interleaved)
    field = pa.field("geometry", arr.type, metadata={"ARROW:extension:name": name})
    return field, arr


def to_arrow(gs):
    """The reference's union layout (GeoSeries.to_arrow,
    core/geoseries.py:536-627): one child filled, points as list<double>."""
    import pyarrow as pa
    x, y, go, po, ro = _host(gs)
    f64 = pa.float64()
    xy = np.empty(2 * len(x), np.float64)
    xy[0::2], xy[1::2] = x, y
    coords = pa.ListArray.from_arrays(pa.array(np.arange(0, 2 * len(x) + 1, 2, dtype=np.int32)),
                                      pa.array(xy, type=f64))
    i32 = lambda a: pa.array(a.astype(np.int32), type=pa.int32())  # noqa: E731
    types = [pa.list_(f64), pa.list_(pa.list_(f64)), pa.list_(pa.list_(pa.list_(f64))),
             pa.list_(pa.list_(pa.list_(pa.list_(f64))))]
    children = [pa.array([], type=t) for t in types]
    if gs.kind == POINT:
        code, children[0] = 0, coords
    elif gs.kind == MULTIPOINT:
        code, children[1] = 1, pa.ListArray.from_arrays(i32(go), coords)
    elif gs.kind == LINESTRING:
        code = 2
        children[2] = pa.ListArray.from_arrays(i32(go), pa.ListArray.from_arrays(i32(po), coords))
    else:
        code = 3
        rings = pa.ListArray.from_arrays(i32(ro), coords)
        children[3] = pa.ListArray.from_arrays(i32(go), pa.ListArray.from_arrays(i32(po), rings))
    n = len(gs)
    return pa.UnionArray.from_dense(pa.array(np.full(n, code, np.int8), type=pa.int8()),
                                    pa.array(np.arange(n, dtype=np.int32), type=pa.int32()),
                                    children, ["points", "mpoints", "lines", "polygons"])


def geoseries_from_host(kind, x, y, geometry_offset=None, part_offset=None, ring_offset=None):
    """GeoSeries from host buffers as read_host_c returns them."""
    offs = {k: as_device_tensor(np.asarray(v).astype(np.int32)) for k, v in
            (("geometry_offset", geometry_offset), ("part_offset", part_offset),
             ("ring_offset", ring_offset)) if v is not None}
    kind_s = _SERIES_KIND[kind]
    n = (len(x) if kind_s == POINT else int(offs["geometry_offset"].numel()) - 1)
    return GeoSeries(kind_s, _Coords(x, y, **offs), n)
