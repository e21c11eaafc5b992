"""Shared helpers: run the GPU path and the oracle on the same workload."""

import numpy as np
import torch

import cuspatial_gb300 as cs
from oracle import oracle as O


def to_np(t):
    return t.detach().cpu().numpy()


def u32(t):
    return to_np(t).view(np.uint32) if t.dtype == torch.int32 else to_np(t).astype(np.uint32)


def gpu_points(w, dtype=np.float64):
    return cs.GeoSeries.from_points(w.x.astype(dtype), w.y.astype(dtype))


def gpu_polygons(p, dtype=np.float64):
    xy = np.empty(2 * len(p.x), dtype)
    xy[0::2] = p.x
    xy[1::2] = p.y
    return cs.GeoSeries.from_polygons_xy(xy, p.ring_offset, p.part_offset, p.geometry_offset)


def gpu_linestrings(ls, dtype=np.float64):
    xy = np.empty(2 * len(ls.x), dtype)
    xy[0::2] = ls.x
    xy[1::2] = ls.y
    return cs.GeoSeries.from_linestrings_xy(xy, ls.part_offset, ls.geometry_offset)


def tree_np(t):
    return dict(key=u32(t["key"]), level=to_np(t["level"]),
                is_internal_node=to_np(t["is_internal_node"]).astype(bool),
                length=u32(t["length"]), offset=u32(t["offset"]))


def oracle_tree(w, dtype=np.float64):
    return O.quadtree_on_points(w.x.astype(dtype), w.y.astype(dtype), w.x_min, w.x_max, w.y_min,
                                w.y_max, w.scale, w.max_depth, w.max_size)


def assert_tree_equal(gpu_pi, gpu_tree, ora_pi, ora_tree):
    np.testing.assert_array_equal(u32(gpu_pi), ora_pi)
    g = tree_np(gpu_tree)
    for k in ("key", "level", "is_internal_node", "length", "offset"):
        np.testing.assert_array_equal(g[k], ora_tree[k], err_msg=k)
