"""Host-side logic of the batched-join autotuner (no GPU)."""

import json

import numpy as np

from cuspatial_gb300 import autotune as A
from cuspatial_gb300 import datasets as D


def test_buckets():
    assert A.bucket_of(1) == 0
    assert A.bucket_of(999) == 0
    assert A.bucket_of(1000) == 1
    assert A.bucket_of(3162) == 1
    assert A.bucket_of(3163) == 2
    assert A.bucket_of(10 ** 7) == len(A.BUCKET_EDGES) - 1


def test_table_round_trip(tmp_path):
    t = A.TuningTable([{"max_depth": 8 + k, "max_size": 32 << k} for k in
                       range(len(A.BUCKET_EDGES))], block_threads=128, meta={"x": 1})
    p = tmp_path / "t.json"
    t.save(str(p))
    u = A.TuningTable.load(str(p))
    assert u.buckets == t.buckets and u.block_threads == 128 and u.meta == {"x": 1}
    d = json.loads(p.read_text())
    d["bucket_edges"] = [1, 2]
    try:
        A.TuningTable.from_json(d)
        raise AssertionError("other bucket edges must be refused")
    except ValueError:
        pass


def test_default_table_is_valid():
    t = A.TuningTable.load()
    assert len(t.buckets) == len(A.BUCKET_EDGES)
    for b in t.buckets:
        assert 1 <= b["max_depth"] <= 15 and b["max_size"] >= 1
    assert t.block_threads % 32 == 0 and 32 <= t.block_threads <= 256


def test_instance_params_cover_box():
    t = A.TuningTable([{"max_depth": 10, "max_size": 64}] * len(A.BUCKET_EDGES))
    p = A.instance_params(5000, (10.0, 110.0, -5.0, 45.0), t)
    assert p["max_depth"] == 10 and p["max_size"] == 64
    # the finest scale the reference's clamp allows is below this one
    assert p["scale"] == 100.0 / 1024
    assert p["scale"] >= 100.0 / ((1 << 10) + 2)


def test_batched_workload_shape():
    wl = D.batched_instances(16, points_range=(10, 1000), polygons_range=(1, 20))
    assert wl.num_instances == 16
    assert int(wl.point_offsets[-1]) == len(wl.x)
    assert int(wl.polygon_offsets[-1]) == wl.polygons.num_polygons
    po = wl.point_offsets.astype(np.int64)
    for i in range(16):
        x = wl.x[po[i]:po[i + 1]]
        y = wl.y[po[i]:po[i + 1]]
        x0, x1, y0, y1 = wl.boxes[i]
        assert np.all((x >= x0) & (x < x1) & (y >= y0) & (y < y1))
    params = A.batch_params(wl)
    assert len(params) == 16
