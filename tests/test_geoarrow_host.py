"""GeoArrow parsing on the host (no GPU): every layout the library reads,
from pyarrow's own export and from the test producer, sliced arrays and the
refusals (mixed unions, nulls, wrong nesting)."""

import numpy as np
import pytest

from cuspatial_gb300 import geoarrow as GA

import arrow_c as AC
from arrow_c import KINDS
from arrow_c import sample as _sample


def _check(got, b, kind):
    np.testing.assert_array_equal(got["x"], b["x"])
    np.testing.assert_array_equal(got["y"], b["y"])
    for k in ("geometry_offset", "part_offset", "ring_offset"):
        if k in b:
            np.testing.assert_array_equal(got[k], b[k].astype(np.uint32), err_msg=k)
        else:
            assert got[k] is None, k




@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("layout", ["interleaved", "struct", "list"])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_producer_layouts(kind, layout, dtype):
    rng = np.random.default_rng(len(kind))
    b = _sample(kind, rng, dtype)
    a = AC.geometry(kind, layout=layout, **b)
    got = GA.read_host_c(a.schema, a.array)
    lay = GA.describe_c(a.schema, a.array)
    assert lay["kind"] == GA.KINDS[kind]
    assert lay["interleaved"] == (layout != "struct")
    _check(got, b, kind)


@pytest.mark.parametrize("kind", ["point", "multipoint", "multilinestring", "multipolygon"])
def test_reference_union(kind):
    rng = np.random.default_rng(3)
    b = _sample(kind, rng)
    a = AC.geometry(kind, as_union=True, **b)
    got = GA.read_host_c(a.schema, a.array)
    assert got["kind"] == GA.KINDS[kind]
    _check(got, b, kind)


def test_kind_argument_and_refusals():
    rng = np.random.default_rng(4)
    b = _sample("linestring", rng)
    a = AC.geometry("linestring", with_extension=False, **b)
    with pytest.raises(RuntimeError, match="unknown geometry type"):
        GA.read_host_c(a.schema, a.array)
    _check(GA.read_host_c(a.schema, a.array, kind="linestring"), b, "linestring")
    # the nesting must fit the kind
    with pytest.raises(RuntimeError, match="nesting"):
        GA.read_host_c(a.schema, a.array, kind="polygon")
    # points must be 2-D
    keep = []
    s, arr = AC._node(b"+w:3", 1, [AC._node(b"g", 0, [], [], [None, np.zeros(6)], 6, 0, keep)[0]],
                      [AC._node(b"g", 0, [], [], [None, np.zeros(6)], 6, 0, keep)[1]], [None], 2,
                      0, keep)
    with pytest.raises(RuntimeError, match="2 coordinates"):
        GA.read_host_c(s, arr, kind="point")


@pytest.fixture
def pa():
    return pytest.importorskip("pyarrow")


def _pa_native(pa, kind, b, layout="interleaved"):
    ft = pa.float64() if b["x"].dtype == np.float64 else pa.float32()
    if layout == "struct":
        pts = pa.StructArray.from_arrays([pa.array(b["x"], type=ft), pa.array(b["y"], type=ft)],
                                         names=["x", "y"])
    else:
        xy = np.empty(2 * len(b["x"]), b["x"].dtype)
        xy[0::2], xy[1::2] = b["x"], b["y"]
        pts = pa.FixedSizeListArray.from_arrays(pa.array(xy, type=ft), 2)
    node = pts
    if "ring_offset" in b:
        node = pa.ListArray.from_arrays(pa.array(b["ring_offset"]), node)
    if "part_offset" in b:
        node = pa.ListArray.from_arrays(pa.array(b["part_offset"]), node)
    if kind.startswith("multi"):
        node = pa.ListArray.from_arrays(pa.array(b["geometry_offset"]), node)
    return node


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("layout", ["interleaved", "struct"])
def test_pyarrow_export(pa, kind, layout):
    rng = np.random.default_rng(10 + len(kind))
    b = _sample(kind, rng)
    arr = _pa_native(pa, kind, b, layout)
    field = pa.field("geometry", arr.type, metadata={"ARROW:extension:name": "geoarrow." + kind})
    schema, array = GA._exported(arr, field)
    try:
        _check(GA.read_host_c(schema, array), b, kind)
    finally:
        GA._release(schema, array)


def test_pyarrow_slices_and_nulls(pa):
    rng = np.random.default_rng(11)
    b = _sample("multipolygon", rng)
    arr = _pa_native(pa, "multipolygon", b)
    sl = arr.slice(2, 3)
    schema, array = GA._exported(sl)
    try:
        got = GA.read_host_c(schema, array, kind="multipolygon")
    finally:
        GA._release(schema, array)
    # the slice's own geometries, offsets rebased to 0
    go = b["geometry_offset"]
    p0, p1 = go[2], go[5]
    po = b["part_offset"][p0:p1 + 1]
    ro = b["ring_offset"][po[0]:po[-1] + 1]
    np.testing.assert_array_equal(got["geometry_offset"], go[2:6] - go[2])
    np.testing.assert_array_equal(got["part_offset"], po - po[0])
    np.testing.assert_array_equal(got["ring_offset"], ro - ro[0])
    np.testing.assert_array_equal(got["x"], b["x"][ro[0]:ro[-1]])
    # null geometries are refused
    withnull = pa.array([[[1.0, 2.0]], None], type=pa.list_(pa.list_(pa.float64())))
    schema, array = GA._exported(withnull)
    try:
        with pytest.raises(RuntimeError, match="null"):
            GA.read_host_c(schema, array, kind="multipoint")
    finally:
        GA._release(schema, array)


def test_pyarrow_union_matches_reference_layout(pa):
    # the union GeoSeries.to_arrow builds (pygeoarrow.py:22-31)
    f64 = pa.float64()
    t = [pa.list_(f64), pa.list_(pa.list_(f64)), pa.list_(pa.list_(pa.list_(f64))),
         pa.list_(pa.list_(pa.list_(pa.list_(f64))))]
    lines = pa.array([[[[0.0, 0.0], [1.0, 1.0]], [[2.0, 2.0], [3.0, 3.0], [4.0, 4.0]]]], type=t[2])
    u = pa.UnionArray.from_dense(pa.array([2], type=pa.int8()), pa.array([0], type=pa.int32()),
                                 [pa.array([], type=t[0]), pa.array([], type=t[1]), lines,
                                  pa.array([], type=t[3])], ["points", "mpoints", "lines",
                                                             "polygons"])
    schema, array = GA._exported(u)
    try:
        got = GA.read_host_c(schema, array)
    finally:
        GA._release(schema, array)
    assert got["kind"] == 2
    np.testing.assert_array_equal(got["geometry_offset"], [0, 2])
    np.testing.assert_array_equal(got["part_offset"], [0, 2, 5])
    np.testing.assert_array_equal(got["x"], [0, 1, 2, 3, 4])
    # a column mixing types is refused
    mixed = pa.UnionArray.from_dense(
        pa.array([0, 2], type=pa.int8()), pa.array([0, 0], type=pa.int32()),
        [pa.array([[5.0, 6.0]], type=t[0]), pa.array([], type=t[1]), lines,
         pa.array([], type=t[3])], ["points", "mpoints", "lines", "polygons"])
    schema, array = GA._exported(mixed)
    try:
        with pytest.raises(TypeError, match="mixed geometry types"):
            GA.read_host_c(schema, array)
    finally:
        GA._release(schema, array)
