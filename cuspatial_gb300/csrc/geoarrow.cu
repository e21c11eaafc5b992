// GeoArrow ingestion through the Arrow C data interface.
//
// Reference: python/cuspatial/cuspatial/io/pygeoarrow.py:9-70 (the union of
// points / multipoints / (multi)linestrings / (multi)polygons the reference
// builds its GeoColumn from, points as list<double> of length 2) and
// core/_column/geocolumn.py (its offsets geometry -> part -> ring -> xy).
// Native GeoArrow layouts are read too: points as fixed_size_list<double>[2]
// (interleaved) or struct<x, y> (separated), nested in lists, the geometry
// type taken from the "ARROW:extension:name" field metadata or from the
// union child.
//
// The parse runs on the host over the Arrow buffers (no copy of the
// coordinates); each offset level is rebased to start at 0 on the host
// (sliced arrays) and copied, the coordinates are copied once as they are
// and split into x / y by a kernel when interleaved.
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"

namespace cspt {
namespace {

constexpr unsigned kArrowBlock = 256;

bool starts_with(char const* s, char const* p)
{
  return s && std::strncmp(s, p, std::strlen(p)) == 0;
}

// "ARROW:extension:name" from an Arrow metadata blob (int32 pair count, then
// int32 key length, key, int32 value length, value for each pair)
std::string extension_name(char const* md)
{
  if (!md) return "";
  int32_t n;
  std::memcpy(&n, md, 4);
  char const* p = md + 4;
  for (int32_t i = 0; i < n; ++i) {
    int32_t kl, vl;
    std::memcpy(&kl, p, 4);
    std::string const key(p + 4, static_cast<size_t>(kl));
    p += 4 + kl;
    std::memcpy(&vl, p, 4);
    std::string const val(p + 4, static_cast<size_t>(vl));
    p += 4 + vl;
    if (key == "ARROW:extension:name") return val;
  }
  return "";
}

bool has_nulls(ArrowArray const* a, int64_t start, int64_t len)
{
  if (a->null_count == 0 || a->n_buffers < 1 || !a->buffers[0]) return false;
  uint8_t const* bits = static_cast<uint8_t const*>(a->buffers[0]);
  for (int64_t i = start; i < start + len; ++i)
    if (!((bits[i >> 3] >> (i & 7)) & 1)) return true;
  return false;
}

// one list level: the logical rows [start, start + len) of `a`; returns the
// rebased offsets (host) and the child's logical row range
struct Level {
  std::vector<uint32_t> offsets;
  int64_t child_start = 0, child_len = 0;
};

Level list_level(ArrowSchema const* s, ArrowArray const* a, int64_t start, int64_t len)
{
  Level l;
  CSPT_EXPECTS(!has_nulls(a, a->offset + start, len), "null geometries are not supported");
  int64_t const first = a->offset + start;
  l.offsets.resize(static_cast<size_t>(len) + 1);
  if (std::strcmp(s->format, "+l") == 0) {
    int32_t const* o = static_cast<int32_t const*>(a->buffers[1]);
    for (int64_t i = 0; i <= len; ++i) {
      CSPT_EXPECTS(o[first + i] >= o[first], "list offsets must not decrease");
      l.offsets[static_cast<size_t>(i)] = static_cast<uint32_t>(o[first + i] - o[first]);
    }
    l.child_start = o[first];
    l.child_len   = o[first + len] - o[first];
  } else {
    int64_t const* o = static_cast<int64_t const*>(a->buffers[1]);
    CSPT_EXPECTS(o[first + len] - o[first] < (int64_t{1} << 32),
                 "more than 2^32 elements below one list level");
    for (int64_t i = 0; i <= len; ++i) {
      CSPT_EXPECTS(o[first + i] >= o[first], "list offsets must not decrease");
      l.offsets[static_cast<size_t>(i)] = static_cast<uint32_t>(o[first + i] - o[first]);
    }
    l.child_start = o[first];
    l.child_len   = o[first + len] - o[first];
  }
  return l;
}

bool is_list(ArrowSchema const* s) { return s && (!std::strcmp(s->format, "+l") || !std::strcmp(s->format, "+L")); }

// A point array: its coordinate layout and where the rows' values start.
struct PointLayout {
  bool interleaved = true;
  cspt_dtype dtype = CSPT_FLOAT64;
  void const* xy = nullptr;  // interleaved: 2 values per point from here
  void const* x  = nullptr;  // separated
  void const* y  = nullptr;
};

cspt_dtype coord_type(char const* f)
{
  if (!std::strcmp(f, "g")) return CSPT_FLOAT64;
  if (!std::strcmp(f, "f")) return CSPT_FLOAT32;
  throw Error{CSPT_UNSUPPORTED, std::string("coordinates must be float64 or float32, not ") + f};
}

PointLayout point_level(ArrowSchema const* s, ArrowArray const* a, int64_t start, int64_t len)
{
  PointLayout p;
  CSPT_EXPECTS(!has_nulls(a, a->offset + start, len), "null geometries are not supported");
  int64_t const first = a->offset + start;
  if (starts_with(s->format, "+w:")) {
    CSPT_EXPECTS(std::strcmp(s->format, "+w:2") == 0, "points must have 2 coordinates (xy)");
    ArrowArray const* c = a->children[0];
    p.dtype             = coord_type(s->children[0]->format);
    size_t const es     = p.dtype == CSPT_FLOAT64 ? 8 : 4;
    CSPT_EXPECTS(!has_nulls(c, c->offset + 2 * first, 2 * len), "null coordinates");
    p.xy = static_cast<char const*>(c->buffers[1]) + (c->offset + 2 * first) * es;
  } else if (!std::strcmp(s->format, "+s")) {
    CSPT_EXPECTS(s->n_children >= 2, "struct points need x and y children");
    p.interleaved   = false;
    p.dtype         = coord_type(s->children[0]->format);
    CSPT_EXPECTS(coord_type(s->children[1]->format) == p.dtype, "x and y types differ");
    size_t const es = p.dtype == CSPT_FLOAT64 ? 8 : 4;
    ArrowArray const* cx = a->children[0];
    ArrowArray const* cy = a->children[1];
    CSPT_EXPECTS(!has_nulls(cx, cx->offset + first, len) && !has_nulls(cy, cy->offset + first, len),
                 "null coordinates");
    p.x = static_cast<char const*>(cx->buffers[1]) + (cx->offset + first) * es;
    p.y = static_cast<char const*>(cy->buffers[1]) + (cy->offset + first) * es;
  } else if (is_list(s)) {
    // the reference's layout: list<double> of length 2 per point
    Level const l = list_level(s, a, start, len);
    for (int64_t i = 0; i < len; ++i)
      CSPT_EXPECTS(l.offsets[static_cast<size_t>(i) + 1] - l.offsets[static_cast<size_t>(i)] == 2,
                   "points must have 2 coordinates (xy)");
    ArrowArray const* c = a->children[0];
    p.dtype             = coord_type(s->children[0]->format);
    size_t const es     = p.dtype == CSPT_FLOAT64 ? 8 : 4;
    p.xy = static_cast<char const*>(c->buffers[1]) + (c->offset + l.child_start) * es;
  } else {
    throw Error{CSPT_UNSUPPORTED, std::string("unsupported point layout ") + s->format};
  }
  return p;
}

// nesting depth above the point level
int list_depth(ArrowSchema const* s)
{
  int d = 0;
  while (is_list(s)) {
    // a list whose child is a float is the reference's point itself
    if (s->n_children == 1 && (!std::strcmp(s->children[0]->format, "g") ||
                               !std::strcmp(s->children[0]->format, "f")))
      break;
    ++d;
    s = s->children[0];
  }
  return d;
}

__global__ void __launch_bounds__(kArrowBlock)
  split_xy_kernel(char const* __restrict__ xy, size_t n, size_t es, char* __restrict__ x,
                  char* __restrict__ y)
{
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    if (es == 8) {
      double2 const v = reinterpret_cast<double2 const*>(xy)[i];
      reinterpret_cast<double*>(x)[i] = v.x;
      reinterpret_cast<double*>(y)[i] = v.y;
    } else {
      float2 const v = reinterpret_cast<float2 const*>(xy)[i];
      reinterpret_cast<float*>(x)[i] = v.x;
      reinterpret_cast<float*>(y)[i] = v.y;
    }
  }
}

uint32_t* to_device(std::vector<uint32_t> const& h, Allocator const& alloc)
{
  auto* d = static_cast<uint32_t*>(alloc.allocate(h.size() * 4));
  if (!h.empty())
    CSPT_CUDA_TRY(cudaMemcpyAsync(d, h.data(), h.size() * 4, cudaMemcpyHostToDevice,
                                  alloc.stream()));
  return d;
}

// The whole parse: the geometry kind, the rebased offsets of every level
// and where the points' coordinates are.
struct Parsed {
  cspt_geoarrow_layout layout{};
  std::vector<uint32_t> geom, part, ring;
  PointLayout points;
};

Parsed parse(ArrowSchema const* schema, ArrowArray const* array, int kind)
{
  Parsed r;
  ArrowSchema const* s = schema;
  ArrowArray const* a  = array;
  int64_t start = 0, len = a->length;
  // the reference's dense union of four children (pygeoarrow.py:22-31)
  if (starts_with(s->format, "+ud:")) {
    CSPT_EXPECTS(s->n_children == 4, "the geometry union has four children");
    // unions carry no validity buffer: type ids and value offsets (a
    // leading validity slot is tolerated)
    CSPT_EXPECTS(a->n_buffers == 2 || a->n_buffers == 3, "a dense union has two buffers");
    int const b0           = a->n_buffers == 3 ? 1 : 0;
    int8_t const* types    = static_cast<int8_t const*>(a->buffers[b0]);
    int32_t const* offsets = static_cast<int32_t const*>(a->buffers[b0 + 1]);
    int8_t const t         = len > 0 ? types[a->offset] : 0;
    int32_t const o0       = len > 0 ? offsets[a->offset] : 0;
    for (int64_t i = 0; i < len; ++i) {
      if (types[a->offset + i] != t || offsets[a->offset + i] != o0 + i)
        throw Error{CSPT_UNSUPPORTED,
                    "mixed geometry types in one column are not supported; split the column by "
                    "type"};
    }
    // type ids to children: the codes listed after "+ud:" (0,1,2,3 in the
    // reference's union)
    int child = -1, idx = 0;
    for (char const* c = s->format + 4; *c; ++idx) {
      char* end      = nullptr;
      int const code = static_cast<int>(std::strtol(c, &end, 10));
      if (end == c) break;  // not a number: stop
      if (code == t) child = idx;
      c = *end == ',' ? end + 1 : end;
    }
    CSPT_EXPECTS(child >= 0 && child < 4, "unknown union child");
    kind  = child;  // 0 points, 1 multipoints, 2 (multi)linestrings, 3 (multi)polygons
    s     = s->children[child];
    a     = a->children[child];
    start = o0;
  } else if (kind < 0) {
    std::string const ext = extension_name(s->metadata);
    if (ext == "geoarrow.point")
      kind = CSPT_GEOM_POINT;
    else if (ext == "geoarrow.multipoint")
      kind = CSPT_GEOM_MULTIPOINT;
    else if (ext == "geoarrow.linestring" || ext == "geoarrow.multilinestring")
      kind = CSPT_GEOM_LINESTRING;
    else if (ext == "geoarrow.polygon" || ext == "geoarrow.multipolygon")
      kind = CSPT_GEOM_POLYGON;
    else
      throw Error{CSPT_INVALID_ARGUMENT,
                  "unknown geometry type: give a geoarrow extension name or a kind"};
  }
  CSPT_EXPECTS(kind >= CSPT_GEOM_POINT && kind <= CSPT_GEOM_POLYGON, "unknown geometry kind");
  int const depth = list_depth(s);
  // list levels each kind has above its points; one more = multi
  int const base = kind == CSPT_GEOM_POINT ? 0 : kind == CSPT_GEOM_POLYGON ? 2 : 1;
  CSPT_EXPECTS(depth == base || (depth == base + 1 && kind != CSPT_GEOM_POINT &&
                                 kind != CSPT_GEOM_MULTIPOINT),
               "list nesting does not match the geometry type");
  bool const multi = depth > base;
  size_t const n   = static_cast<size_t>(len);
  for (int lvl = 0; lvl < depth; ++lvl) {
    Level l = list_level(s, a, start, len);
    if (lvl == 0 && (multi || kind == CSPT_GEOM_MULTIPOINT))
      r.geom = std::move(l.offsets);
    else if (kind == CSPT_GEOM_POLYGON && lvl == depth - 1)
      r.ring = std::move(l.offsets);
    else
      r.part = std::move(l.offsets);
    s     = s->children[0];
    a     = a->children[0];
    start = l.child_start;
    len   = l.child_len;
  }
  // single linestrings / polygons: one part per geometry
  if ((kind == CSPT_GEOM_LINESTRING || kind == CSPT_GEOM_POLYGON) && !multi) {
    r.geom.resize(n + 1);
    for (size_t i = 0; i <= n; ++i) r.geom[i] = static_cast<uint32_t>(i);
  }
  r.points                          = point_level(s, a, start, len);
  r.layout.kind                     = kind;
  r.layout.multi                    = multi ? 1 : 0;
  r.layout.interleaved              = r.points.interleaved ? 1 : 0;
  r.layout.dtype                    = r.points.dtype;
  r.layout.num_geometries           = n;
  r.layout.num_geometry_offsets     = r.geom.size();
  r.layout.num_part_offsets         = r.part.size();
  r.layout.num_ring_offsets         = r.ring.size();
  r.layout.num_points               = static_cast<size_t>(len);
  return r;
}

}  // namespace

void geoarrow_import(ArrowSchema const* schema, ArrowArray const* array, int kind_hint,
                     cspt_allocator const* mr, cudaStream_t st, cspt_geometry_column* out)
{
  Allocator const alloc(mr, st);
  Parsed const r      = parse(schema, array, kind_hint);
  PointLayout const& p = r.points;
  size_t const np     = r.layout.num_points;
  size_t const es     = p.dtype == CSPT_FLOAT64 ? 8 : 4;
  *out                = cspt_geometry_column{};
  out->kind           = r.layout.kind;
  out->dtype          = p.dtype;
  out->num_geometries = r.layout.num_geometries;
  try {
    if (!r.geom.empty()) {
      out->geometry_offsets     = to_device(r.geom, alloc);
      out->num_geometry_offsets = r.geom.size();
    }
    if (!r.part.empty()) {
      out->part_offsets     = to_device(r.part, alloc);
      out->num_part_offsets = r.part.size();
    }
    if (!r.ring.empty()) {
      out->ring_offsets     = to_device(r.ring, alloc);
      out->num_ring_offsets = r.ring.size();
    }
    out->num_points = np;
    out->x          = alloc.allocate(np * es);
    out->y          = alloc.allocate(np * es);
    if (np > 0) {
      if (p.interleaved) {
        Buffer<char> xy(alloc, 2 * np * es);
        CSPT_CUDA_TRY(cudaMemcpyAsync(xy.data(), p.xy, 2 * np * es, cudaMemcpyHostToDevice, st));
        split_xy_kernel<<<grid_for(np, kArrowBlock, static_cast<unsigned>(num_sms()) * 8u),
                          kArrowBlock, 0, st>>>(xy.data(), np, es, static_cast<char*>(out->x),
                                                static_cast<char*>(out->y));
        CSPT_CHECK_LAUNCH();
        CSPT_CUDA_TRY(cudaStreamSynchronize(st));  // before the staging buffer is released
      } else {
        CSPT_CUDA_TRY(cudaMemcpyAsync(out->x, p.x, np * es, cudaMemcpyHostToDevice, st));
        CSPT_CUDA_TRY(cudaMemcpyAsync(out->y, p.y, np * es, cudaMemcpyHostToDevice, st));
      }
    }
    // the offset vectors are pageable host memory owned here
    CSPT_CUDA_TRY(cudaStreamSynchronize(st));
  } catch (...) {
    cspt_geometry_column_free(mr, out, st);
    throw;
  }
}

}  // namespace cspt

extern "C" {

cspt_status cspt_geoarrow_describe(const struct ArrowSchema* schema,
                                   const struct ArrowArray* array, int kind,
                                   cspt_geoarrow_layout* out)
{
  return cspt::guarded([&] {
    CSPT_EXPECTS(schema && array && out, "arguments must not be null");
    *out = cspt::parse(schema, array, kind).layout;
  });
}

cspt_status cspt_geoarrow_read_host(const struct ArrowSchema* schema,
                                    const struct ArrowArray* array, int kind,
                                    uint32_t* geometry_offsets, uint32_t* part_offsets,
                                    uint32_t* ring_offsets, void* x, void* y)
{
  return cspt::guarded([&] {
    CSPT_EXPECTS(schema && array, "arguments must not be null");
    cspt::Parsed const r = cspt::parse(schema, array, kind);
    auto put = [](std::vector<uint32_t> const& v, uint32_t* dst) {
      if (!v.empty()) {
        CSPT_EXPECTS(dst, "output pointers must not be null");
        std::memcpy(dst, v.data(), v.size() * 4);
      }
    };
    put(r.geom, geometry_offsets);
    put(r.part, part_offsets);
    put(r.ring, ring_offsets);
    size_t const np = r.layout.num_points;
    size_t const es = r.points.dtype == CSPT_FLOAT64 ? 8 : 4;
    if (np == 0) return;
    CSPT_EXPECTS(x && y, "output pointers must not be null");
    if (r.points.interleaved) {
      char const* xy = static_cast<char const*>(r.points.xy);
      for (size_t i = 0; i < np; ++i) {
        std::memcpy(static_cast<char*>(x) + i * es, xy + 2 * i * es, es);
        std::memcpy(static_cast<char*>(y) + i * es, xy + (2 * i + 1) * es, es);
      }
    } else {
      std::memcpy(x, r.points.x, np * es);
      std::memcpy(y, r.points.y, np * es);
    }
  });
}

cspt_status cspt_geoarrow_import(const struct ArrowSchema* schema, const struct ArrowArray* array,
                                 int kind, const cspt_allocator* mr, void* stream,
                                 cspt_geometry_column* out)
{
  return cspt::guarded([&] {
    CSPT_EXPECTS(schema && array && out, "arguments must not be null");
    *out = cspt_geometry_column{};
    cspt::geoarrow_import(schema, array, kind, mr, static_cast<cudaStream_t>(stream), out);
  });
}

void cspt_geometry_column_free(const cspt_allocator* mr, cspt_geometry_column* col, void* stream)
{
  if (!col) return;
  cspt::Allocator const a(mr, static_cast<cudaStream_t>(stream));
  size_t const es = col->dtype == CSPT_FLOAT64 ? 8 : 4;
  a.deallocate(col->geometry_offsets, col->num_geometry_offsets * 4);
  a.deallocate(col->part_offsets, col->num_part_offsets * 4);
  a.deallocate(col->ring_offsets, col->num_ring_offsets * 4);
  a.deallocate(col->x, col->num_points * es);
  a.deallocate(col->y, col->num_points * es);
  *col = cspt_geometry_column{};
}

}  // extern "C"
