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
              "cspt_quadtree_point_in_polygon", "cspt_quadtree_point_to_nearest_linestring"):
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
