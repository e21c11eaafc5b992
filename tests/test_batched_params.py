"""The batched form's per-instance parameters are packed column by column
into a numpy record array that the C ABI reads as cspt_instance_params[]:
its bytes must equal those of the ctypes structs, field by field."""
import ctypes

import numpy as np

from cuspatial_gb300 import _lib
from cuspatial_gb300.batched import PARAM_FIELDS, _params_array


def _ctypes_bytes(rows):
    arr = (_lib.CsptInstanceParams * len(rows))()
    for i, r in enumerate(rows):
        arr[i] = _lib.CsptInstanceParams(*(float(v) for v in r[:5]), int(r[5]), int(r[6]))
    return bytes(arr)


def test_record_layout_matches_the_c_struct():
    rng = np.random.default_rng(3)
    rows = [(float(a), float(a) + 10.0, float(b), float(b) + 7.5, 0.25 * (i + 1), i % 15 + 1,
             int(rng.integers(1, 5000)))
            for i, (a, b) in enumerate(rng.uniform(-1e6, 1e6, (37, 2)))]
    dicts = [dict(zip(PARAM_FIELDS, r)) for r in rows]
    expect = _ctypes_bytes(rows)
    for params in (rows, dicts, rows[:1], dicts[:1]):
        got = _params_array(params)
        assert got.dtype.itemsize == ctypes.sizeof(_lib.CsptInstanceParams)
        assert got.tobytes() == expect[:len(params) * got.dtype.itemsize]


def test_empty_parameter_list():
    assert _params_array([]).size == 0
