"""GeoArrow ingestion onto the GPU (Arrow C data from the test producer, so
no pyarrow is needed): device columns equal the host parse, and imported
columns run through the join and distance entry points with the same
results as columns built from numpy.  Export back to pyarrow where pyarrow
is installed."""

import numpy as np
import pytest
import torch

import cuspatial_gb300 as cs
from cuspatial_gb300 import datasets as D
from cuspatial_gb300 import geoarrow as GA

import arrow_c as AC
from helpers import gpu_polygons, to_np
from arrow_c import KINDS
from arrow_c import sample as _sample

pytestmark = pytest.mark.gpu


def _device_equals_host(gs, a):
    h = GA.read_host_c(a.schema, a.array)
    c = gs._coords
    np.testing.assert_array_equal(to_np(c.x), h["x"])
    np.testing.assert_array_equal(to_np(c.y), h["y"])
    for k in ("geometry_offset", "part_offset", "ring_offset"):
        if h[k] is not None:
            np.testing.assert_array_equal(to_np(getattr(c, k)).view(np.uint32), h[k], err_msg=k)


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("layout", ["interleaved", "struct", "list"])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_import_layouts(kind, layout, dtype):
    b = _sample(kind, np.random.default_rng(len(kind) + len(layout)), dtype)
    a = AC.geometry(kind, layout=layout, **b)
    gs = GA.from_arrow_c(a.schema, a.array)
    assert len(gs) == 7
    assert gs._coords.x.dtype == (torch.float64 if dtype == np.float64 else torch.float32)
    _device_equals_host(gs, a)


def test_imported_polygons_join():
    # polygons and points arriving as GeoArrow give the same join rows
    w = D.plain_small(n_points=200_000, n_polygons=64)
    P = w.polygons
    a = AC.geometry("multipolygon", P.x, P.y, geometry_offset=P.geometry_offset,
                    part_offset=P.part_offset, ring_offset=P.ring_offset)
    pa_ = AC.geometry("point", w.x, w.y, layout="struct")
    polys = GA.from_arrow_c(a.schema, a.array)
    pts = GA.from_arrow_c(pa_.schema, pa_.array)

    def rows(points, polygons):
        pi, tree = cs.quadtree_on_points(points, w.x_min, w.x_max, w.y_min, w.y_max, w.scale,
                                         w.max_depth, w.max_size)
        bb = cs.polygon_bounding_boxes(polygons)
        pairs = cs.join_quadtree_and_bounding_boxes(tree, bb, w.x_min, w.x_max, w.y_min,
                                                    w.y_max, w.scale, w.max_depth)
        r = cs.quadtree_point_in_polygon(pairs, tree, pi, points, polygons, method="filtered")
        return to_np(r["polygon_index"]), to_np(r["point_index"])

    got = rows(pts, polys)
    want = rows(cs.GeoSeries.from_points(w.x, w.y), gpu_polygons(P))
    assert len(want[0]) > 1000
    for g, e in zip(got, want):
        np.testing.assert_array_equal(g, e)


def test_imported_reference_union_distance():
    # multipoints and multilinestrings in the reference's union layout
    rng = np.random.default_rng(5)
    mp = _sample("multipoint", rng)
    ml = _sample("multilinestring", rng)
    a = AC.geometry("multipoint", as_union=True, **mp)
    b = AC.geometry("multilinestring", as_union=True, **ml)
    pts = GA.from_arrow_c(a.schema, a.array)
    lines = GA.from_arrow_c(b.schema, b.array)
    got = to_np(cs.pairwise_point_linestring_distance(pts, lines))
    xy = np.empty(2 * len(mp["x"]))
    xy[0::2], xy[1::2] = mp["x"], mp["y"]
    lxy = np.empty(2 * len(ml["x"]))
    lxy[0::2], lxy[1::2] = ml["x"], ml["y"]
    want = to_np(cs.pairwise_point_linestring_distance(
        cs.GeoSeries.from_multipoints_xy(xy, mp["geometry_offset"]),
        cs.GeoSeries.from_linestrings_xy(lxy, ml["part_offset"], ml["geometry_offset"])))
    np.testing.assert_array_equal(got, want)


def test_export_round_trip():
    pa = pytest.importorskip("pyarrow")
    b = _sample("multipolygon", np.random.default_rng(9))
    a = AC.geometry("multipolygon", **b)
    gs = GA.from_arrow_c(a.schema, a.array)
    field, arr = GA.to_geoarrow(gs)
    assert field.metadata[b"ARROW:extension:name"] == b"geoarrow.multipolygon"
    back = GA.from_geoarrow(arr, field=field)
    for k in ("x", "y"):
        np.testing.assert_array_equal(to_np(getattr(back._coords, k)), b[k])
    u = GA.to_arrow(gs)
    assert isinstance(u, pa.UnionArray)
    again = GA.from_geoarrow(u)
    np.testing.assert_array_equal(to_np(again._coords.ring_offset), b["ring_offset"])
