"""Minimal GeoSeries and table stand-ins for the quadtree join API.

cuSpatial's GeoSeries (python/cuspatial/cuspatial/core/geoseries.py) is a
cuDF container of GeoArrow columns.  The join functions only read
`points.points.{x,y}`, `polygons.polygons.{part_offset,ring_offset,x,y}`
and `linestrings.lines.{part_offset,geometry_offset,x,y}`, so this stand-in
stores exactly those GeoArrow buffers as torch CUDA tensors and offers the
reference's `from_points_xy`, `from_multipoints_xy`, `from_linestrings_xy`
and `from_polygons_xy` constructors.  Results are returned as `Table`, an ordered mapping of column
name to tensor in place of cudf.DataFrame.
"""

from collections import OrderedDict

import numpy as np
import torch

POINT, MULTIPOINT, LINESTRING, POLYGON = "point", "multipoint", "linestring", "polygon"


def as_device_tensor(a, dtype=None, device=None):
    """Array-like -> contiguous CUDA tensor (no copy when already suitable)."""
    dev = torch.device(device) if device is not None else torch.device(
        "cuda", torch.cuda.current_device())
    if isinstance(a, torch.Tensor):
        t = a
    else:
        t = torch.from_numpy(np.ascontiguousarray(a))
    if dtype is not None and t.dtype != dtype:
        t = t.to(dtype)
    if t.device != dev:
        t = t.to(dev, non_blocking=False)
    return t.contiguous()


def _xy_split(xy):
    if isinstance(xy, torch.Tensor):
        t = xy.reshape(-1)
        return t[0::2].contiguous(), t[1::2].contiguous()
    a = np.asarray(xy).reshape(-1)
    return np.ascontiguousarray(a[0::2]), np.ascontiguousarray(a[1::2])


class _Coords:
    def __init__(self, x, y, **offsets):
        self.x = as_device_tensor(x)
        self.y = as_device_tensor(y, dtype=self.x.dtype)
        for k, v in offsets.items():
            setattr(self, k, as_device_tensor(v, dtype=torch.int32))


class GeoSeries:
    """Homogeneous series of points, linestrings or polygons."""

    def __init__(self, kind, coords, length):
        self.kind = kind
        self._coords = coords
        self._len = length

    def __len__(self):
        return self._len

    @property
    def points(self):
        if self.kind != POINT:
            raise ValueError("GeoSeries must contain only points.")
        return self._coords

    @property
    def multipoints(self):
        if self.kind != MULTIPOINT:
            raise ValueError("GeoSeries must contain only multipoints.")
        return self._coords

    @property
    def lines(self):
        if self.kind != LINESTRING:
            raise ValueError("GeoSeries must contain only linestrings.")
        return self._coords

    @property
    def polygons(self):
        if self.kind != POLYGON:
            raise ValueError("GeoSeries must contain only polygons.")
        return self._coords

    @classmethod
    def from_points_xy(cls, points_xy):
        x, y = _xy_split(points_xy)
        return cls(POINT, _Coords(x, y), len(x))

    @classmethod
    def from_points(cls, x, y):
        c = _Coords(x, y)
        return cls(POINT, c, int(c.x.numel()))

    @classmethod
    def from_multipoints_xy(cls, multipoints_xy, geometry_offset):
        x, y = _xy_split(multipoints_xy)
        c = _Coords(x, y, geometry_offset=geometry_offset)
        return cls(MULTIPOINT, c, int(c.geometry_offset.numel()) - 1)

    @classmethod
    def from_linestrings_xy(cls, linestrings_xy, part_offset, geometry_offset):
        x, y = _xy_split(linestrings_xy)
        c = _Coords(x, y, part_offset=part_offset, geometry_offset=geometry_offset)
        return cls(LINESTRING, c, int(c.geometry_offset.numel()) - 1)

    @classmethod
    def from_polygons_xy(cls, polygons_xy, ring_offset, part_offset, geometry_offset):
        x, y = _xy_split(polygons_xy)
        c = _Coords(x, y, ring_offset=ring_offset, part_offset=part_offset,
                    geometry_offset=geometry_offset)
        return cls(POLYGON, c, int(c.geometry_offset.numel()) - 1)


def contains_only_points(gs):
    return isinstance(gs, GeoSeries) and gs.kind == POINT


def contains_only_points_or_multipoints(gs):
    return isinstance(gs, GeoSeries) and gs.kind in (POINT, MULTIPOINT)


def contains_only_linestrings(gs):
    return isinstance(gs, GeoSeries) and gs.kind == LINESTRING


def contains_only_polygons(gs):
    return isinstance(gs, GeoSeries) and gs.kind == POLYGON


class Table(OrderedDict):
    """Ordered column name -> tensor mapping (the cudf.DataFrame stand-in)."""

    @property
    def columns(self):
        return list(self.keys())

    def __len__(self):
        for v in self.values():
            return int(v.numel())
        return 0

    def num_rows(self):
        return len(self)

    def to_numpy(self):
        return {k: v.cpu().numpy() for k, v in self.items() if isinstance(v, torch.Tensor)}
