"""A minimal Arrow C data interface producer for tests (no pyarrow): builds
ArrowSchema / ArrowArray trees over numpy buffers for the GeoArrow layouts
the library reads.  Every object is kept alive by the returned `Arrow`
handle; release callbacks are left NULL (the library never calls them)."""

import ctypes
import struct

import numpy as np

from cuspatial_gb300.geoarrow import ArrowArray, ArrowSchema


class Arrow:
    """Owns a schema/array tree and everything it points to."""

    def __init__(self, schema, array, keep):
        self.schema, self.array, self._keep = schema, array, keep


def _node(fmt, n_children, children_s, children_a, buffers, length, offset, keep, meta=None,
          name=b""):
    s = ArrowSchema()
    fb = ctypes.c_char_p(fmt)
    s.format = fb
    s.name = ctypes.c_char_p(name)
    if meta is not None:
        mb = ctypes.create_string_buffer(meta, len(meta))
        s.metadata = ctypes.cast(mb, ctypes.c_void_p)
        keep.append(mb)
    s.n_children = n_children
    cs = (ctypes.POINTER(ArrowSchema) * max(n_children, 1))(
        *[ctypes.pointer(c) for c in children_s])
    s.children = ctypes.cast(cs, ctypes.POINTER(ctypes.POINTER(ArrowSchema)))
    a = ArrowArray()
    a.length, a.null_count, a.offset = length, 0, offset
    a.n_buffers = len(buffers)
    bufs = (ctypes.c_void_p * max(len(buffers), 1))(
        *[b.ctypes.data if b is not None else None for b in buffers])
    a.buffers = ctypes.cast(bufs, ctypes.POINTER(ctypes.c_void_p))
    a.n_children = n_children
    ca = (ctypes.POINTER(ArrowArray) * max(n_children, 1))(
        *[ctypes.pointer(c) for c in children_a])
    a.children = ctypes.cast(ca, ctypes.POINTER(ctypes.POINTER(ArrowArray)))
    keep += [fb, cs, bufs, ca, buffers, children_s, children_a]
    return s, a


def _fmt(dtype):
    return b"g" if np.dtype(dtype) == np.float64 else b"f"


def points(x, y, layout="interleaved", keep=None, offset=0):
    """Point array: 'interleaved' (fixed_size_list[2]), 'struct' (x, y) or
    'list' (the reference's list<double> of length 2)."""
    keep = [] if keep is None else keep
    x = np.ascontiguousarray(x)
    y = np.ascontiguousarray(y, dtype=x.dtype)
    n = len(x) - offset
    f = _fmt(x.dtype)
    if layout == "struct":
        sx, ax = _node(f, 0, [], [], [None, x], len(x), 0, keep, name=b"x")
        sy, ay = _node(f, 0, [], [], [None, y], len(y), 0, keep, name=b"y")
        return _node(b"+s", 2, [sx, sy], [ax, ay], [None], n, offset, keep)
    xy = np.empty(2 * len(x), x.dtype)
    xy[0::2], xy[1::2] = x, y
    sv, av = _node(f, 0, [], [], [None, xy], len(xy), 0, keep)
    if layout == "interleaved":
        return _node(b"+w:2", 1, [sv], [av], [None], n, offset, keep)
    offs = np.arange(0, 2 * len(x) + 1, 2, dtype=np.int32)
    return _node(b"+l", 1, [sv], [av], [None, offs], n, offset, keep)


def lists(offsets, child, keep, offset=0, meta=None):
    offs = np.ascontiguousarray(offsets, dtype=np.int32)
    return _node(b"+l", 1, [child[0]], [child[1]], [None, offs], len(offs) - 1 - offset, offset,
                 keep, meta=meta)


def extension(name):
    """Arrow metadata blob with ARROW:extension:name."""
    k, v = b"ARROW:extension:name", name.encode()
    return struct.pack("<i", 1) + struct.pack("<i", len(k)) + k + struct.pack("<i", len(v)) + v


def union(child_index, n, children, keep):
    """The reference's dense union; children = 4 (schema, array) pairs."""
    types = np.full(n, child_index, np.int8)
    offs = np.arange(n, dtype=np.int32)
    return _node(b"+ud:0,1,2,3", 4, [c[0] for c in children], [c[1] for c in children],
                 [types, offs], n, 0, keep)


def empty_child(depth, keep, dtype=np.float64):
    """An empty child of the union at the given list depth above list<double>."""
    node = points(np.zeros(0, dtype), np.zeros(0, dtype), "list", keep)
    for _ in range(depth):
        node = lists(np.zeros(1, np.int32), node, keep)
    return node


def geometry(kind, x, y, geometry_offset=None, part_offset=None, ring_offset=None,
             layout="interleaved", with_extension=True, as_union=False):
    """A full GeoArrow array for `kind` ('point', 'multipoint', 'linestring',
    'multilinestring', 'polygon', 'multipolygon')."""
    keep = []
    lay = "list" if as_union else layout
    node = points(x, y, lay, keep)
    if kind in ("polygon", "multipolygon"):
        node = lists(ring_offset, node, keep)
    if kind in ("linestring", "multilinestring", "polygon", "multipolygon"):
        node = lists(part_offset, node, keep)
    if kind in ("multipoint", "multilinestring", "multipolygon"):
        node = lists(geometry_offset, node, keep)
    if as_union:
        index = {"point": 0, "multipoint": 1, "multilinestring": 2, "multipolygon": 3}[kind]
        depth = {0: 0, 1: 1, 2: 2, 3: 3}
        children = [node if i == index else empty_child(depth[i], keep) for i in range(4)]
        n = node[1].length
        s, a = union(index, n, children, keep)
        return Arrow(s, a, keep)
    if with_extension:
        meta = extension("geoarrow." + kind)
        mb = ctypes.create_string_buffer(meta, len(meta))
        node[0].metadata = ctypes.cast(mb, ctypes.c_void_p)
        keep.append(mb)
    return Arrow(node[0], node[1], keep)


KINDS = ["point", "multipoint", "linestring", "multilinestring", "polygon", "multipolygon"]


def sample(kind, rng, dtype=np.float64):
    """Host buffers of a small geometry column of `kind`."""
    n = 7
    if kind == "point":
        x = rng.uniform(-10, 10, n).astype(dtype)
        return dict(x=x, y=(x * 2).astype(dtype))
    parts = rng.integers(1, 4, n)
    if kind in ("multipoint",):
        go = np.concatenate([[0], np.cumsum(parts)]).astype(np.int32)
        m = int(go[-1])
        x = rng.uniform(-10, 10, m).astype(dtype)
        return dict(x=x, y=(x + 1).astype(dtype), geometry_offset=go)
    if kind in ("linestring", "multilinestring"):
        go = (np.concatenate([[0], np.cumsum(parts)]) if kind == "multilinestring"
              else np.arange(n + 1)).astype(np.int32)
        nparts = int(go[-1])
        po = np.concatenate([[0], np.cumsum(rng.integers(2, 6, nparts))]).astype(np.int32)
        x = rng.uniform(-10, 10, int(po[-1])).astype(dtype)
        return dict(x=x, y=(x - 3).astype(dtype), geometry_offset=go, part_offset=po)
    go = (np.concatenate([[0], np.cumsum(parts)]) if kind == "multipolygon"
          else np.arange(n + 1)).astype(np.int32)
    npoly = int(go[-1])
    po = np.concatenate([[0], np.cumsum(rng.integers(1, 3, npoly))]).astype(np.int32)
    ro = np.concatenate([[0], np.cumsum(rng.integers(4, 9, int(po[-1])))]).astype(np.int32)
    x = rng.uniform(-10, 10, int(ro[-1])).astype(dtype)
    return dict(x=x, y=(x * 0.5).astype(dtype), geometry_offset=go, part_offset=po,
                ring_offset=ro)
