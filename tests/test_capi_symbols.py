"""The C-ABI library builds for sm_103a, loads without a GPU and exports every
function include/cuspatial_gb300.h declares (no compute calls here)."""

import os
import re

from conftest import ROOT


def declared_functions():
    text = open(os.path.join(ROOT, "include", "cuspatial_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cspt_\w+)\s*\(", text)))


def test_header_declares_reference_entry_points():
    names = declared_functions()
    for f in ("cspt_quadtree_on_points", "cspt_polygon_bounding_boxes",
              "cspt_linestring_bounding_boxes", "cspt_join_quadtree_and_bounding_boxes",
              "cspt_quadtree_point_in_polygon", "cspt_quadtree_point_to_nearest_linestring",
              "cspt_point_in_polygon", "cspt_pairwise_point_in_polygon"):
        assert f in names


def test_library_exports_every_declared_symbol():
    from cuspatial_gb300 import _lib
    lib = _lib.load()  # builds in-tree with nvcc when missing
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert b"sm_103a" in lib.cspt_version()


def test_last_error_empty_on_fresh_thread():
    from cuspatial_gb300 import _lib
    lib = _lib.load()
    assert lib.cspt_last_error_message() == b""


def test_point_in_polygon_argument_checks_on_host():
    # the reference's checks run before any device work, so they can be
    # exercised without a GPU (point_in_polygon.cu:118-136 and
    # detail/point_in_polygon.cuh:93-94)
    import ctypes

    import numpy as np

    from cuspatial_gb300 import _lib
    lib = _lib.load()
    po = np.arange(33, dtype=np.uint32)
    ro = np.arange(33, dtype=np.uint32) * 4
    p = po.ctypes.data_as(ctypes.c_void_p)
    r = ro.ctypes.data_as(ctypes.c_void_p)
    st = lib.cspt_point_in_polygon(None, None, 5, p, 33, r, 33, None, None, 128, _lib.FLOAT64,
                                   _lib.METHOD_EXACT, None, None, None)
    assert st == _lib.INVALID_ARGUMENT
    assert lib.cspt_last_error_message() == b"Number of polygons cannot exceed 31"
    # an empty point column returns before the polygon count is checked
    assert lib.cspt_point_in_polygon(None, None, 0, p, 33, r, 33, None, None, 128, _lib.FLOAT64,
                                     _lib.METHOD_EXACT, None, None, None) == _lib.OK
    st = lib.cspt_pairwise_point_in_polygon(None, None, 5, p, 33, r, 33, None, None, 128,
                                            _lib.FLOAT64, _lib.METHOD_EXACT, None, None, None)
    assert st == _lib.INVALID_ARGUMENT
    assert lib.cspt_last_error_message() == b"Must pass in the same number of points as polygons."
    st = lib.cspt_pairwise_point_in_polygon(None, None, 5, p, 6, r, 6, None, None, 20, 7,
                                            _lib.METHOD_EXACT, None, None, None)
    assert st == _lib.UNSUPPORTED


def test_host_buffer_entry_points_argument_checks_on_host():
    # the host-buffer entry points check their arguments before any device work
    import ctypes

    import pytest
    import torch

    import cuspatial_gb300 as cs
    from cuspatial_gb300 import _lib
    lib = _lib.load()
    pi, tree = ctypes.c_void_p(), _lib.CsptQuadtree()
    args = (0.0, 1.0, 0.0, 1.0, 0.1, 3, 8)
    assert lib.cspt_quadtree_on_points_host(None, None, 0, _lib.FLOAT64, *args, None, None, None,
                                            None, ctypes.byref(pi), ctypes.byref(tree)) == _lib.OK
    assert tree.num_nodes == 0 and not pi.value
    assert lib.cspt_quadtree_on_points_host(None, None, 5, 7, *args, None, None, None, None,
                                            ctypes.byref(pi), ctypes.byref(tree)) == _lib.UNSUPPORTED
    assert lib.cspt_quadtree_on_points_host(None, None, 5, _lib.FLOAT64, *args, None, None, None,
                                            None, ctypes.byref(pi),
                                            ctypes.byref(tree)) == _lib.INVALID_ARGUMENT
    assert lib.cspt_last_error_message() == b"x and y columns must have the same length"

    n = ctypes.c_size_t(7)
    common = (None, None, 0, ctypes.byref(tree), None, 0, None, None, 0, None, 1, None, 1, None,
              None, 0, _lib.FLOAT64, _lib.METHOD_FILTERED, None, None)
    assert lib.cspt_quadtree_point_in_polygon_host(*common, None, None, 0,
                                                   None) == _lib.INVALID_ARGUMENT
    assert lib.cspt_last_error_message() == b"output pointers must not be null"
    assert lib.cspt_quadtree_point_in_polygon_host(*common, None, None, 4,
                                                   ctypes.byref(n)) == _lib.INVALID_ARGUMENT
    assert lib.cspt_last_error_message() == b"host output arrays must not be null"
    # no pairs: nothing to write
    assert lib.cspt_quadtree_point_in_polygon_host(*common, None, None, 0,
                                                   ctypes.byref(n)) == _lib.OK
    assert n.value == 0

    with pytest.raises(TypeError):
        cs.quadtree_on_points_host(torch.zeros(3, dtype=torch.int32),
                                   torch.zeros(3, dtype=torch.int32), *args)
    with pytest.raises(RuntimeError):
        cs.quadtree_on_points_host(torch.zeros(3, dtype=torch.float64),
                                   torch.zeros(2, dtype=torch.float64), *args)
