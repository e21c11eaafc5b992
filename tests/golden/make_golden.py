"""Extract known-answer vectors from cuSpatial's own tests into JSON fixtures.

Run from the repository root with the cuSpatial sources available:

    python tests/golden/make_golden.py /path/to/cuspatial

It reads the reference test files as text (it never imports or runs them) and
writes one JSON file per source test file next to this script.  The fixtures
are committed; the tests read only the JSON files.

Sources:
  cpp/tests/index/point_quadtree_test.cu                        (quadtree KATs)
  cpp/tests/join/quadtree_point_in_polygon_test_small.cu        (join + PiP KAT)
  cpp/tests/join/quadtree_point_to_nearest_linestring_test_small.cu
  cpp/tests/point_in_polygon/point_in_polygon_test.cu           (boundary rule)
  python/cuspatial/cuspatial/tests/spatial/bounding/test_linestring_bounding_boxes.py
  cpp/tests/distance/point_linestring_distance_test.cu          (pairwise distance)
  cpp/tests/nearest_points/point_linestring_nearest_points_test.cu
  python/cuspatial/cuspatial/tests/spatial/indexing/test_indexing.py
  python/cuspatial/cuspatial/tests/spatial/join/test_spatial_join.py
  python/cuspatial/cuspatial/tests/spatial/join/test_point_in_polygon.py

The Python tests are parsed with the ast module and followed by a small
evaluator (python_test_kats below); they are not imported or executed either.
"""

import ast
import json
import os
import re
import sys


def strip_comments(text):
    text = re.sub(r"//[^\n]*", "", text)
    return re.sub(r"/\*.*?\*/", "", text, flags=re.S)


def parse_number(tok):
    tok = tok.strip()
    if tok in ("true", "false"):
        return tok == "true"
    if tok.startswith(("0b", "0B")):
        return int(tok[2:], 2)
    tok = tok.rstrip("fFuUlL") if not tok.startswith(("0x", "0X")) else tok
    if tok.startswith(("0x", "0X")):
        return int(tok, 16)
    if re.fullmatch(r"[-+]?\d+", tok):
        return int(tok)
    return float(tok)


def parse_braces(text, pos):
    """Parse a C++ brace initializer starting at text[pos] == '{'.

    Returns (value, next_pos).  Scalars become numbers, braces become lists.
    """
    assert text[pos] == "{", text[pos:pos + 40]
    pos += 1
    out = []
    tok = ""
    while True:
        c = text[pos]
        if c == "{":
            val, pos = parse_braces(text, pos)
            out.append(val)
            continue
        if c in ",}":
            if tok.strip():
                out.append(parse_number(tok))
            tok = ""
            pos += 1
            if c == "}":
                return out, pos
            continue
        tok += c
        pos += 1


def matching_paren(text, pos):
    assert text[pos] == "("
    depth = 0
    for i in range(pos, len(text)):
        if text[i] in "({":
            depth += 1
        elif text[i] in ")}":
            depth -= 1
            if depth == 0:
                return i
    raise ValueError("unbalanced")


def split_top_level(args):
    parts, depth, cur = [], 0, ""
    for c in args:
        if c in "({<" and not (c == "<" and depth == 0 and False):
            depth += 1 if c != "<" else 0
        if c in ")}":
            depth -= 1
        if c == "," and depth == 0:
            parts.append(cur.strip())
            cur = ""
        else:
            cur += c
    if cur.strip():
        parts.append(cur.strip())
    return parts


def first_braces(text):
    i = text.index("{")
    return parse_braces(text, i)[0]


def test_bodies(text, fixture):
    pat = re.compile(r"TYPED_TEST\(\s*%s\s*,\s*(\w+)\s*\)\s*\{" % fixture)
    out = {}
    for m in pat.finditer(text):
        start = m.end() - 1
        depth = 0
        for i in range(start, len(text)):
            if text[i] == "{":
                depth += 1
            elif text[i] == "}":
                depth -= 1
                if depth == 0:
                    out[m.group(1)] = text[start:i + 1]
                    break
    return out


def run_test_args(body, fn):
    m = re.search(r"CUSPATIAL_RUN_TEST\(\s*this->%s\s*," % fn, body)
    if not m:
        return None
    open_pos = body.index("(", m.start())
    close = matching_paren(body, open_pos)
    return split_top_level(body[m.end():close])


def quadtree_kats(root):
    path = os.path.join(root, "cpp/tests/index/point_quadtree_test.cu")
    text = strip_comments(open(path).read())
    cases = []
    for name, body in test_bodies(text, "QuadtreeOnPointIndexingTest").items():
        args = run_test_args(body, "test")
        env = {}
        for var in ("vertex_1", "vertex_2"):
            m = re.search(r"%s\s*(\{[^}]*\})" % var, body)
            env[var] = first_braces(m.group(1))
        for var in ("max_depth", "max_size", "scale"):
            m = re.search(r"%s\s*=\s*([-+0-9.eE]+)" % var, body)
            if m:
                env[var] = parse_number(m.group(1))

        def val(a):
            a = a.strip()
            if a in env:
                return env[a]
            wrapped = a.startswith("thrust::host_vector")
            a = re.sub(r"^thrust::host_vector\s*", "", a)
            if a.startswith("{"):
                v = first_braces(a)
                # thrust::host_vector{{...}} wraps the list once more
                if wrapped and len(v) == 1 and isinstance(v[0], list):
                    v = v[0]
                return v
            return parse_number(a)

        vals = [val(a) for a in args]
        points, v1, v2, scale, max_depth, max_size = vals[:6]
        key, level, internal, length, offset = vals[6:11]
        cases.append(
            dict(name=name, x=[p[0] for p in points], y=[p[1] for p in points],
                 x_min=v1[0], y_min=v1[1], x_max=v2[0], y_max=v2[1], scale=scale,
                 max_depth=max_depth, max_size=max_size, key=key, level=level,
                 is_internal_node=[int(b) for b in internal], length=length,
                 offset=offset))
    return dict(source="cpp/tests/index/point_quadtree_test.cu", cases=cases)


def device_vectors(body):
    """All make_device_vector<...>( {...} ) literals in order."""
    out = []
    for m in re.finditer(r"make_device_vector<[^(]*>\(\s*\{", body):
        out.append(parse_braces(body, m.end() - 1)[0])
    return out


def small_params(body):
    env = {}
    for var in ("v_min", "v_max"):
        m = re.search(r"%s\s*(\{[^}]*\})" % var, body)
        env[var] = first_braces(m.group(1))
    for var in ("scale", "max_depth", "max_size", "expansion_radius"):
        m = re.search(r"%s\s*\{\s*([-+0-9.eE]+)\s*\}" % var, body)
        if m:
            env[var] = parse_number(m.group(1))
    return env


def pip_small_kat(root):
    rel = "cpp/tests/join/quadtree_point_in_polygon_test_small.cu"
    text = strip_comments(open(os.path.join(root, rel)).read())
    body = test_bodies(text, "PIPRefineTestSmall")["TestSmall"]
    env = small_params(body)
    vecs = device_vectors(body)
    points = vecs[0]
    m = re.search(r"make_multipolygon_array<T>\(", body)
    open_pos = body.index("(", m.start())
    args = split_top_level(body[open_pos + 1:matching_paren(body, open_pos)])
    geom, part, ring, verts = [first_braces(a) for a in args]
    exp_poly_join, exp_quad_join, exp_poly, exp_point = vecs[1:5]
    return dict(source=rel, x=[p[0] for p in points], y=[p[1] for p in points],
                x_min=env["v_min"][0], y_min=env["v_min"][1], x_max=env["v_max"][0],
                y_max=env["v_max"][1], scale=env["scale"], max_depth=env["max_depth"],
                max_size=env["max_size"], geometry_offset=geom, part_offset=part,
                ring_offset=ring, px=[v[0] for v in verts], py=[v[1] for v in verts],
                join_bbox_offset=exp_poly_join, join_quad_offset=exp_quad_join,
                polygon_index=exp_poly, point_index=exp_point)


def nearest_small_kat(root):
    rel = "cpp/tests/join/quadtree_point_to_nearest_linestring_test_small.cu"
    text = strip_comments(open(os.path.join(root, rel)).read())
    body = test_bodies(text, "QuadtreePointToLinestringTestSmall")["TestSmall"]
    env = small_params(body)
    vecs = device_vectors(body)
    points = vecs[0]
    m = re.search(r"make_multilinestring_array<T>\(", body)
    open_pos = body.index("(", m.start())
    args = split_top_level(body[open_pos + 1:matching_paren(body, open_pos)])
    geom, part, verts = [first_braces(a) for a in args]
    join_ls, join_quad = vecs[1], vecs[2]
    dist_f32, dist_f64 = vecs[3], vecs[4]
    exp_point, exp_ls = vecs[5], vecs[6]
    return dict(source=rel, x=[p[0] for p in points], y=[p[1] for p in points],
                x_min=env["v_min"][0], y_min=env["v_min"][1], x_max=env["v_max"][0],
                y_max=env["v_max"][1], scale=env["scale"], max_depth=env["max_depth"],
                max_size=env["max_size"], expansion_radius=env["expansion_radius"],
                geometry_offset=geom, part_offset=part, lx=[v[0] for v in verts],
                ly=[v[1] for v in verts], join_bbox_offset=join_ls,
                join_quad_offset=join_quad, point_index=exp_point,
                linestring_index=exp_ls, distance_f32=dist_f32, distance_f64=dist_f64)


def point_in_polygon_kats(root):
    rel = "cpp/tests/point_in_polygon/point_in_polygon_test.cu"
    text = strip_comments(open(os.path.join(root, rel)).read())
    cases = []
    for name, body in test_bodies(text, "PointInPolygonTest").items():
        args = run_test_args(body, "run_test")
        if args is None or len(args) != 5:
            continue
        points, poly_off, ring_off, verts, expected = [first_braces(a) for a in args]
        cases.append(dict(name=name, x=[p[0] for p in points], y=[p[1] for p in points],
                          poly_offsets=poly_off, ring_offsets=ring_off,
                          px=[v[0] for v in verts], py=[v[1] for v in verts],
                          expected=expected))
    return dict(source=rel, note="expected[i] bit j = point i inside polygon j", cases=cases)


def linestring_bbox_kat(root):
    rel = "python/cuspatial/cuspatial/tests/spatial/bounding/test_linestring_bounding_boxes.py"
    text = open(os.path.join(root, rel)).read()
    m = re.search(r"def test_linestring_bounding_boxes_small\(dtype\):(.*?)\ndef ", text, re.S)
    body = m.group(1)
    series = re.findall(r"cudf\.Series\(\s*\[([^\]]*)\]", body)
    nums = [[parse_number(t) for t in s.replace("\n", " ").split(",") if t.strip()]
            for s in series]
    xy, part, geom = nums[0], nums[1], nums[2]
    radius = parse_number(re.search(r"s,\s*([0-9.]+),\s*#\s*expansion_radius", body).group(1))
    minx, miny, maxx, maxy = nums[3:7]
    return dict(source=rel, lx=xy[0::2], ly=xy[1::2], part_offset=part, geometry_offset=geom,
                expansion_radius=radius, minx=minx, miny=miny, maxx=maxx, maxy=maxy)


def cpp_expr(tok):
    """A number or the tests' std::sqrt(T{a}) [/ b] expressions."""
    tok = " ".join(tok.split())
    m = re.fullmatch(r"std::sqrt\(T\{([-+0-9.eE]+)\}\)(?:\s*/\s*([-+0-9.eE]+))?", tok)
    if m:
        v = parse_number(m.group(1)) ** 0.5
        return v / parse_number(m.group(2)) if m.group(2) else v
    return parse_number(tok)


def braces_after(body, pattern):
    """The brace list that follows the first match of `pattern` (None if absent)."""
    m = re.search(pattern, body, re.S)
    if not m:
        return None
    return parse_braces(body, body.index("{", m.end() - 1))[0]


def expr_list_after(body, pattern):
    m = re.search(pattern, body, re.S)
    if not m:
        return None
    start = body.index("{", m.end() - 1)
    depth, i = 0, start
    while True:
        if body[i] == "{":
            depth += 1
        elif body[i] == "}":
            depth -= 1
            if depth == 0:
                break
        i += 1
    inner = body[start + 1:i]
    parts, depth, tok = [], 0, ""
    for c in inner:
        if c in "({":
            depth += 1
        elif c in ")}":
            depth -= 1
        if c == "," and depth == 0:
            parts.append(tok)
            tok = ""
        else:
            tok += c
    if tok.strip():
        parts.append(tok)
    return [cpp_expr(t) for t in parts]


def point_linestring_distance_kats(root):
    rel = "cpp/tests/distance/point_linestring_distance_test.cu"
    text = strip_comments(open(os.path.join(root, rel)).read())
    cases = []
    for name, body in test_bodies(text, "PairwisePointLinestringDistanceTest").items():
        c = dict(name=name)
        if name == "ManyPairsFromIteratorsSingleComponent":
            # built from counting iterators in the test: linestring i has the
            # vertices (3i, 1), (3i+1, 1), (3i+2, 1); point i is (3i, 0)
            n = 100
            c.update(x=[3.0 * i for i in range(n)], y=[0.0] * n,
                     point_geometry_offsets=None, linestring_geometry_offsets=None,
                     part_offsets=[3 * i for i in range(n + 1)],
                     lx=[float(i) for i in range(3 * n)], ly=[1.0] * (3 * n),
                     expected=[1.0] * n)
            cases.append(c)
            continue
        if "d_points_x" in body:
            px = braces_after(body, r"d_points_x\s*=\s*rmm::device_vector<T>\(\s*std::vector<T>")
            py = braces_after(body, r"d_points_y\s*=\s*rmm::device_vector<T>\(\s*std::vector<T>")
            lx = braces_after(body, r"d_linestring_points_x\s*=\s*rmm::device_vector<T>\(\s*std::vector<T>")
            ly = braces_after(body, r"d_linestring_points_y\s*=\s*rmm::device_vector<T>\(\s*std::vector<T>")
            n = len(px)
            c.update(x=px, y=py, point_geometry_offsets=None, linestring_geometry_offsets=None,
                     part_offsets=[3 * i for i in range(n + 1)], lx=lx, ly=ly,
                     expected=expr_list_after(body, r"expect\s*=\s*std::vector<T>"))
            cases.append(c)
            continue
        pts = braces_after(body, r"CartVec points")
        lpts = braces_after(body, r"CartVec linestring_points")
        c.update(x=[float(p[0]) for p in pts], y=[float(p[1]) for p in pts],
                 point_geometry_offsets=braces_after(body, r"point_geometry_offsets"),
                 linestring_geometry_offsets=braces_after(body, r"linestring_geometry_offsets"),
                 part_offsets=braces_after(body, r"linestring_part_offsets"),
                 lx=[float(p[0]) for p in lpts], ly=[float(p[1]) for p in lpts],
                 expected=expr_list_after(body, r"expect\(std::vector<T>"))
        if c["expected"] is None:
            c["expected"] = []
        cases.append(c)
    return dict(source=rel, note="expected distances; the reference compares them "
                "with CUSPATIAL_EXPECT_VECTORS_EQUIVALENT (float tolerance)", cases=cases)


def nearest_points_kats(root):
    rel = "cpp/tests/nearest_points/point_linestring_nearest_points_test.cu"
    text = strip_comments(open(os.path.join(root, rel)).read())
    cases = []
    for name, body in test_bodies(text, "PairwisePointLinestringNearestPointsTest").items():
        n = int(re.search(r"num_pairs\s*=\s*(\d+)", body).group(1))
        pts = braces_after(body, r"\bpoints(?:_it)?\s*=\s*rmm::device_vector<vec_2d<T>>\(\s*CartVec")
        lpts = braces_after(body, r"\blinestring_points(?:_it)?\s*=\s*rmm::device_vector<vec_2d<T>>\(\s*CartVec")
        pgo = braces_after(body, r"points_geometry_offsets\s*=\s*rmm::device_vector<int32_t>\(\s*std::vector<int>")
        lgo = braces_after(body, r"linestring_geometry_offsets\s*=\s*rmm::device_vector<int32_t>\(\s*std::vector<int>")
        lpo = braces_after(body, r"linestring_part_offsets\s*=\s*rmm::device_vector<int32_t>\(\s*std::vector<int32_t>")

        def ids(var):
            m = re.search(r"EXPECT_EQ\((?:thrust::host_vector<int32_t>\()?%s\)?\s*,\s*"
                          r"std::vector<int32_t>\(?" % var, body)
            if not m:
                return None
            return parse_braces(body, body.index("{", m.end() - 1))[0]

        coords = braces_after(body, r"expected_coordinate\s*=\s*CartVec")
        if coords is None:
            coords = braces_after(body, r"CUSPATIAL_EXPECT_VECTORS_EQUIVALENT\(\s*neartest_point_coordinate\s*,\s*CartVec")
        cases.append(dict(
            name=name, num_pairs=n, x=[float(p[0]) for p in pts], y=[float(p[1]) for p in pts],
            point_geometry_offsets=pgo, linestring_geometry_offsets=lgo, part_offsets=lpo,
            lx=[float(p[0]) for p in lpts], ly=[float(p[1]) for p in lpts],
            point_geometry_id=ids("nearest_point_id"),
            linestring_geometry_id=ids(r"nearest_linestring_(?:linestring_|parts_)?id"),
            segment_id=ids(r"nearest_(?:linestring_)?segment_id"),
            nearest_x=[float(p[0]) for p in (coords or [])],
            nearest_y=[float(p[1]) for p in (coords or [])]))
    return dict(source=rel, note="ids exact; coordinates compared with float tolerance in "
                "the reference", cases=cases)


# ---------------------------------------------------------------------------
# The reference's Python tests.  Each test body is parsed (ast) and followed by
# a small evaluator over the forms these tests use: literals, cudf.Series and
# DataFrame become lists and dicts, GeoSeries constructors become geometry
# records, every cuspatial.* call becomes an op record over its evaluated
# arguments, and cudf.testing.assert_frame_equal pairs an op record (the
# value under test) with its expected frame.  Tests parametrised by dtype are
# followed once per dtype.  Anything outside those forms skips the test, and
# the skipped tests are listed in the fixture.
# ---------------------------------------------------------------------------
_NP_NAMES = {"np.float32": "float32", "np.float64": "float64", "np.uint32": "uint32",
             "np.uint8": "uint8", "np.bool_": "bool", "np.int8": "int8"}


def _dotted(node):
    if isinstance(node, ast.Name):
        return node.id
    if isinstance(node, ast.Attribute):
        base = _dotted(node.value)
        return base + "." + node.attr if base else None
    return None


class _Unsupported(Exception):
    pass


class _Eval:
    def __init__(self, env, helpers):
        self.env = dict(env)
        self.helpers = helpers
        self.checks = []

    def ev(self, n):
        if isinstance(n, ast.Constant):
            return n.value
        if isinstance(n, (ast.List, ast.Tuple)):
            out = []
            for e in n.elts:
                if isinstance(e, ast.Starred):
                    out.extend(self.ev(e.value))
                else:
                    out.append(self.ev(e))
            return out
        if isinstance(n, ast.Dict):
            return {self.ev(k): self.ev(v) for k, v in zip(n.keys, n.values)}
        if isinstance(n, ast.UnaryOp) and isinstance(n.op, ast.USub):
            return -self.ev(n.operand)
        if isinstance(n, ast.Compare) and len(n.ops) == 1 and isinstance(n.ops[0], ast.Eq):
            return self.ev(n.left) == self.ev(n.comparators[0])
        if isinstance(n, ast.Name):
            if n.id in self.env:
                return self.env[n.id]
            raise _Unsupported("name " + n.id)
        if isinstance(n, ast.Attribute) and _dotted(n) in _NP_NAMES:
            return _NP_NAMES[_dotted(n)]
        if isinstance(n, ast.Call):
            return self.call(n)
        raise _Unsupported(type(n).__name__)

    def call(self, n):
        f = n.func
        if isinstance(f, ast.Attribute) and f.attr == "astype":
            return self.ev(f.value)
        if isinstance(f, ast.Attribute) and f.attr == "interleave_columns":
            df = self.ev(f.value)
            out = []
            for a, b in zip(df["x"], df["y"]):
                out += [a, b]
            return out
        name = _dotted(f)
        args = []
        for a in n.args:
            if isinstance(a, ast.Starred):
                args.extend(self.ev(a.value))
            else:
                args.append(self.ev(a))
        kw = {k.arg: self.ev(k.value) for k in n.keywords}
        if name == "cudf.Series":
            return list(args[0]) if args else []
        if name == "cudf.DataFrame":
            return dict(args[0]) if args else {}
        if name == "Point":
            return [args[0], args[1]]
        if name == "len":
            return len(args[0])
        if name in ("cp.arange", "np.arange"):
            return list(range(args[0]))
        if name == "cuspatial.GeoSeries":
            if not args[0]:
                return {"geometry": "empty"}
            return {"geometry": "points", "xy": [c for p in args[0] for c in p]}
        if name == "cuspatial.GeoSeries.from_points_xy":
            return {"geometry": "points", "xy": args[0]}
        if name == "cuspatial.GeoSeries.from_polygons_xy":
            return {"geometry": "polygons", "xy": args[0], "ring_offset": args[1],
                    "part_offset": args[2], "geometry_offset": args[3]}
        if name == "cuspatial.GeoSeries.from_linestrings_xy":
            return {"geometry": "linestrings", "xy": args[0], "part_offset": args[1],
                    "geometry_offset": args[2]}
        if name == "cudf.testing.assert_frame_equal":
            self.checks.append((args[0], args[1]))
            return None
        if name and name.startswith("cuspatial."):
            return {"op": name.split(".", 1)[1], "args": args}
        if name in self.helpers:
            fdef = self.helpers[name]
            saved = dict(self.env)
            for p, v in zip([a.arg for a in fdef.args.args], args):
                self.env[p] = v
            self.env.update(kw)
            self.run(fdef.body)
            self.env = saved
            return None
        raise _Unsupported("call " + str(name))

    def run(self, body):
        for st in body:
            if isinstance(st, ast.Assign):
                v = self.ev(st.value)
                for t in st.targets:
                    self.assign(t, v)
            elif isinstance(st, ast.Expr):
                if not isinstance(st.value, ast.Constant):  # docstrings
                    self.ev(st.value)
            elif isinstance(st, ast.If):
                self.run(st.body if self.ev(st.test) else st.orelse)
            else:
                raise _Unsupported(type(st).__name__)

    def assign(self, t, v):
        if isinstance(t, ast.Name):
            self.env[t.id] = v
        elif isinstance(t, ast.Tuple) and isinstance(v, dict) and "op" in v:
            for i, e in enumerate(t.elts):  # an op returning a pair
                self.env[e.id] = dict(v, out=i)
        elif isinstance(t, ast.Subscript):
            self.ev(t.value)[self.ev(t.slice)] = v
        else:
            raise _Unsupported("assignment")


def _dtype_params(fdef):
    for d in fdef.decorator_list:
        if (isinstance(d, ast.Call) and _dotted(d.func) == "pytest.mark.parametrize" and
                isinstance(d.args[0], ast.Constant) and d.args[0].value == "dtype"):
            return [_NP_NAMES.get(_dotted(e), getattr(e, "value", None)) for e in d.args[1].elts]
    return None


def kats_from_python_source(rel, text):
    """The cases and skipped tests of one Python test file's source text."""
    cases, skipped = [], []
    tree = ast.parse(text)
    env, helpers, tests = {}, {}, []
    for st in tree.body:
        if isinstance(st, ast.Assign):
            try:
                v = _Eval(env, helpers).ev(st.value)
            except _Unsupported:
                continue
            for t in st.targets:
                if isinstance(t, ast.Name):
                    env[t.id] = v
        elif isinstance(st, ast.FunctionDef):
            if st.name.startswith("test_"):
                tests.append(st)
            else:
                helpers[st.name] = st
    for fdef in tests:
        dtypes = _dtype_params(fdef) or [None]
        for dt in dtypes:
            e = _Eval(env, helpers)
            if dt is not None:
                e.env["dtype"] = dt
            try:
                e.run(fdef.body)
            except (_Unsupported, KeyError, IndexError, TypeError) as exc:
                skipped.append(dict(source=rel, test=fdef.name, reason=str(exc)))
                break
            for actual, expected in e.checks:
                if isinstance(expected, dict) and "op" in expected:
                    actual, expected = expected, actual
                cases.append(dict(source="%s:%d" % (rel, fdef.lineno), test=fdef.name,
                                  dtype=dt or "float64", actual=actual,
                                  expected={str(k): v for k, v in expected.items()}))
    return cases, skipped


def python_test_kats(root):
    files = ["python/cuspatial/cuspatial/tests/spatial/indexing/test_indexing.py",
             "python/cuspatial/cuspatial/tests/spatial/join/test_spatial_join.py",
             "python/cuspatial/cuspatial/tests/spatial/join/test_point_in_polygon.py"]
    cases, skipped = [], []
    for rel in files:
        c, sk = kats_from_python_source(rel, open(os.path.join(root, rel)).read())
        cases += c
        skipped += sk
    return dict(note="each case: an op record (the value under test, built from the "
                     "reference's Python API calls) and the frame the test expects",
                cases=cases, skipped=skipped)


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    here = os.path.dirname(os.path.abspath(__file__))
    outputs = {
        "point_quadtree.json": quadtree_kats(root),
        "quadtree_point_in_polygon_small.json": pip_small_kat(root),
        "quadtree_point_to_nearest_linestring_small.json": nearest_small_kat(root),
        "point_in_polygon.json": point_in_polygon_kats(root),
        "linestring_bounding_boxes_small.json": linestring_bbox_kat(root),
        "point_linestring_distance.json": point_linestring_distance_kats(root),
        "point_linestring_nearest_points.json": nearest_points_kats(root),
        "python_tests.json": python_test_kats(root),
    }
    for name, data in outputs.items():
        with open(os.path.join(here, name), "w") as f:
            json.dump(data, f, indent=1)
        print("wrote", name)


if __name__ == "__main__":
    main()
