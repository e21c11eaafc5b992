"""The reference's Python tests for the join path, replayed from
tests/golden/python_tests.json (made by tests/golden/make_golden.py from
python/cuspatial/cuspatial/tests/spatial/indexing/test_indexing.py,
tests/spatial/join/test_spatial_join.py and
tests/spatial/join/test_point_in_polygon.py): first the oracle, then this
library's public API on the GPU, each against the frame the reference test
expects."""

import json
import os

import numpy as np
import pytest

import python_kats as K

_CASES = json.load(open(os.path.join(os.path.dirname(__file__), "golden",
                                     "python_tests.json")))["cases"]
_IDS = ["%s-%s-%s" % (os.path.basename(c["source"].split(":")[0])[:-3], c["test"], c["dtype"])
        for c in _CASES]


def test_fixture_covers_the_reference_tests():
    names = {(c["source"].split(":")[0].rsplit("/", 1)[1], c["test"]) for c in _CASES}
    assert len(_CASES) == 27 and len(names) == 21


@pytest.mark.parametrize("case", _CASES, ids=_IDS)
def test_oracle(case):
    K.check(case, K.run(case["actual"], np.dtype(case["dtype"]).type, "oracle"))


@pytest.mark.gpu
@pytest.mark.parametrize("case", _CASES, ids=_IDS)
def test_gpu(case):
    K.check(case, K.run(case["actual"], np.dtype(case["dtype"]).type, "gpu"))
