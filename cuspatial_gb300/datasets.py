"""Seeded synthetic inputs with the shapes of the benchmark configurations.

No public dataset is involved; every array is drawn from numpy's PCG64 with
seed 20261203 + config id, so the same call gives the same bytes on any
machine.  All sizes can be scaled down (same distributions) for tests.

  plain_small          1,000,000 uniform points in [0,1000)^2, 256 star
                       polygons (8-64 vertices, per-vertex radius U[5,40]).
  precision_at_scale   100,000,000 points from a 64-component Gaussian
                       mixture, 1% of them on polygon vertices or within 1e-9
                       of an edge; 100,000 star polygons (8-512 vertices,
                       radius U[2,60] per polygon with per-vertex factor
                       U[0.5,1]), 10% with a reversed hole at 0.4 scale.
  batched_instances    4096 independent instances: points per instance
                       log-uniform in [1e3, 1e6], uniform in a box of side
                       U[100, 10000] at a random origin; polygons per
                       instance log-uniform in [1, 2000], star-shaped with
                       4-256 vertices and radius 0.5%-5% of the box side.
  serving_polygons     250,000 star polygons (8-256 vertices, radius U[1,30])
                       centred on a jittered 500 x 500 grid over [0,20000)^2.
  serving_requests     request point sets of log-uniform [1, 1e5] points,
                       half uniform over the domain, half one Gaussian cluster
                       (sigma U[5,500]).
  nearest_linestring   50,000,000 uniform points in [0,10000)^2, 200,000
                       random-walk linestrings (2-256 segments, step U[1,20],
                       heading change N(0, 0.3 rad)).
  unindexed_pip        10,000,000 uniform points in [-20,20]^2 against 31
                       regular polygons of 100 sides, radius 10, all centred
                       on the origin (one closed ring each), as in the
                       reference's point-in-polygon benchmark
                       (cpp/benchmarks/point_in_polygon/point_in_polygon.cu).
  pairwise_pip         one point per star polygon: 4-400 vertices, 10% with
                       a hole, points inside, outside and on the boundary.
"""

import math
from dataclasses import dataclass, field

import numpy as np

SEED = 20261203


@dataclass
class Polygons:
    x: np.ndarray
    y: np.ndarray
    ring_offset: np.ndarray    # ring -> first vertex
    part_offset: np.ndarray    # polygon -> first ring
    geometry_offset: np.ndarray  # multipolygon -> first polygon (identity)

    @property
    def num_polygons(self):
        return len(self.part_offset) - 1


@dataclass
class Linestrings:
    x: np.ndarray
    y: np.ndarray
    part_offset: np.ndarray
    geometry_offset: np.ndarray


@dataclass
class Workload:
    name: str
    x: np.ndarray
    y: np.ndarray
    x_min: float
    x_max: float
    y_min: float
    y_max: float
    scale: float
    max_depth: int
    max_size: int
    polygons: Polygons = None
    linestrings: Linestrings = None
    expansion_radius: float = 0.0
    extra: dict = field(default_factory=dict)


def star_polygons(rng, centers, nverts, radius_fn, hole_fraction=0.0, hole_scale=0.4):
    """Star-shaped single-ring polygons (optionally with one reversed hole).

    Vertex angles are the sorted order statistics of nverts uniforms on
    [0, 2pi) plus a random rotation; rings are closed by repeating vertex 0.
    radius_fn(rng, polygon_ids) returns one radius per vertex.
    """
    p = len(centers)
    nverts = np.asarray(nverts, dtype=np.int64)
    pid = np.repeat(np.arange(p), nverts)
    # sorted uniforms via normalised cumulative exponential spacings
    e = rng.exponential(size=len(pid) + p)
    starts = np.concatenate([[0], np.cumsum(nverts + 1)])
    cs = np.cumsum(e)
    base = np.concatenate([[0.0], cs[starts[1:-1] - 1]])
    tot = cs[starts[1:] - 1] - base
    local = np.arange(len(pid)) - np.repeat(np.cumsum(nverts) - nverts, nverts)
    idx = np.repeat(starts[:-1], nverts) + local
    ang = (cs[idx] - np.repeat(base, nverts)) / np.repeat(tot, nverts) * 2 * math.pi
    ang += np.repeat(rng.uniform(0, 2 * math.pi, p), nverts)
    r = radius_fn(rng, pid)
    vx = np.repeat(centers[:, 0], nverts) + r * np.cos(ang)
    vy = np.repeat(centers[:, 1], nverts) + r * np.sin(ang)
    has_hole = rng.random(p) < hole_fraction
    # rings: outer closed by repeating its first vertex, then (optionally) the
    # hole: the closed outer ring scaled about the centre and reversed
    ring_len = nverts + 1
    rings_per_poly = np.where(has_hole, 2, 1)
    poly_len = ring_len * rings_per_poly
    pstart = np.concatenate([[0], np.cumsum(poly_len)])
    vstart = np.concatenate([[0], np.cumsum(nverts)])
    total = int(pstart[-1])
    x = np.empty(total)
    y = np.empty(total)
    # outer ring: position pstart + j (j < k) takes vertex j, j = k closes
    pos = np.repeat(pstart[:-1], nverts) + local
    x[pos] = vx
    y[pos] = vy
    x[pstart[:-1] + nverts] = vx[vstart[:-1]]
    y[pstart[:-1] + nverts] = vy[vstart[:-1]]
    hp = np.nonzero(has_hole)[0]
    if len(hp):
        hk = ring_len[hp]
        hpos = np.repeat(pstart[hp] + hk, hk) + (np.arange(hk.sum()) -
                                                  np.repeat(np.cumsum(hk) - hk, hk))
        j = hpos - np.repeat(pstart[hp] + hk, hk)          # 0..k within the hole
        src = np.repeat(pstart[hp], hk) + (np.repeat(hk, hk) - 1 - j)  # reversed outer
        cx = np.repeat(centers[hp, 0], hk)
        cy = np.repeat(centers[hp, 1], hk)
        x[hpos] = cx + hole_scale * (x[src] - cx)
        y[hpos] = cy + hole_scale * (y[src] - cy)
    ring_sizes = np.repeat(ring_len, rings_per_poly)
    ring_offset = np.concatenate([[0], np.cumsum(ring_sizes)]).astype(np.int32)
    part_offset = np.concatenate([[0], np.cumsum(rings_per_poly)]).astype(np.int32)
    geometry_offset = np.arange(p + 1, dtype=np.int32)
    return Polygons(x, y, ring_offset, part_offset, geometry_offset)


def plain_small(n_points=1_000_000, n_polygons=256, seed_offset=0):
    rng = np.random.Generator(np.random.PCG64(SEED + 0 + seed_offset))
    x = rng.uniform(0, 1000, n_points)
    y = rng.uniform(0, 1000, n_points)
    centers = rng.uniform(50, 950, (n_polygons, 2))
    k = rng.integers(8, 65, n_polygons)
    polys = star_polygons(rng, centers, k, lambda g, pid: g.uniform(5, 40, len(pid)))
    return Workload("plain_small", x, y, 0.0, 1000.0, 0.0, 1000.0, 1000.0 / 128, 7, 128,
                    polygons=polys)


def _near_boundary(rng, polys, count):
    """Points on polygon vertices (half) or within 1e-9 of an edge (half)."""
    nring = len(polys.ring_offset) - 1
    ring = rng.integers(0, nring, count)
    rb = polys.ring_offset[ring].astype(np.int64)
    rl = polys.ring_offset[ring + 1].astype(np.int64) - rb
    j = rb + (rng.random(count) * (rl - 1)).astype(np.int64)  # edge j -> j+1 (closed ring)
    ax, ay = polys.x[j], polys.y[j]
    bx, by = polys.x[j + 1], polys.y[j + 1]
    on_vertex = rng.random(count) < 0.5
    t = rng.random(count)
    dx, dy = bx - ax, by - ay
    ln = np.hypot(dx, dy)
    ln[ln == 0] = 1.0
    off = rng.uniform(-1e-9, 1e-9, count)
    px = ax + t * dx - dy / ln * off
    py = ay + t * dy + dx / ln * off
    px = np.where(on_vertex, ax, px)
    py = np.where(on_vertex, ay, py)
    return px, py


def precision_at_scale(n_points=100_000_000, n_polygons=100_000, n_components=64,
                       boundary_fraction=0.01, extent=10000.0, max_vertices=512,
                       seed_offset=0):
    rng = np.random.Generator(np.random.PCG64(SEED + 1 + seed_offset))
    centers = rng.uniform(0, extent, (n_components, 2))
    sigma = rng.uniform(10, 200, n_components)
    comp = rng.integers(0, n_components, n_points)
    x = centers[comp, 0] + sigma[comp] * rng.standard_normal(n_points)
    y = centers[comp, 1] + sigma[comp] * rng.standard_normal(n_points)
    del comp
    hi = np.nextafter(extent, 0.0)
    np.clip(x, 0.0, hi, out=x)
    np.clip(y, 0.0, hi, out=y)
    pc = rng.uniform(0, extent, (n_polygons, 2))
    k = rng.integers(8, max_vertices + 1, n_polygons)
    prad = rng.uniform(2, 60, n_polygons)
    polys = star_polygons(rng, pc, k, lambda g, pid: prad[pid] * g.uniform(0.5, 1.0, len(pid)),
                          hole_fraction=0.10)
    nb = int(round(boundary_fraction * n_points))
    if nb:
        sel = rng.choice(n_points, nb, replace=False)
        bx, by = _near_boundary(rng, polys, nb)
        x[sel] = bx
        y[sel] = by
    # cells stay below 2^15 for points in [0, extent)
    return Workload("precision_at_scale", x, y, 0.0, extent, 0.0, extent, extent / 32768, 15,
                    256, polygons=polys, extra=dict(boundary_points=nb))


def nearest_linestring(n_points=50_000_000, n_linestrings=200_000, extent=10000.0,
                       seed_offset=0):
    rng = np.random.Generator(np.random.PCG64(SEED + 4 + seed_offset))
    x = rng.uniform(0, extent, n_points)
    y = rng.uniform(0, extent, n_points)
    nseg = rng.integers(2, 257, n_linestrings)
    nv = nseg + 1
    start = rng.uniform(0, extent, (n_linestrings, 2))
    lid = np.repeat(np.arange(n_linestrings), nseg)
    step = rng.uniform(1, 20, len(lid))
    dtheta = rng.normal(0, 0.3, len(lid))
    h0 = rng.uniform(0, 2 * math.pi, n_linestrings)
    # heading = initial heading + cumulative turn within each linestring
    cum = np.cumsum(dtheta)
    seg_start = np.concatenate([[0], np.cumsum(nseg)[:-1]])
    base = np.where(seg_start > 0, cum[seg_start - 1], 0.0)
    heading = np.repeat(h0, nseg) + cum - np.repeat(base, nseg)
    sx = np.cumsum(step * np.cos(heading))
    sy = np.cumsum(step * np.sin(heading))
    bx = np.where(seg_start > 0, sx[seg_start - 1], 0.0)
    by = np.where(seg_start > 0, sy[seg_start - 1], 0.0)
    rel_x = sx - np.repeat(bx, nseg)
    rel_y = sy - np.repeat(by, nseg)
    # vertices: start point, then the walk
    voff = np.concatenate([[0], np.cumsum(nv)])
    lx = np.empty(voff[-1])
    ly = np.empty(voff[-1])
    first = voff[:-1]
    lx[first] = start[:, 0]
    ly[first] = start[:, 1]
    rest = np.ones(voff[-1], bool)
    rest[first] = False
    lx[rest] = np.repeat(start[:, 0], nseg) + rel_x
    ly[rest] = np.repeat(start[:, 1], nseg) + rel_y
    ls = Linestrings(lx, ly, voff.astype(np.int32), np.arange(n_linestrings + 1, dtype=np.int32))
    return Workload("nearest_linestring", x, y, 0.0, extent, 0.0, extent, extent / 16384, 14,
                    256, linestrings=ls, expansion_radius=25.0)


@dataclass
class BatchedWorkload:
    """Concatenated instances: instance i owns points
    [point_offsets[i], point_offsets[i+1]) and polygons
    [polygon_offsets[i], polygon_offsets[i+1]) of `polygons` (global ring and
    vertex offsets); box[i] = (x_min, x_max, y_min, y_max)."""
    x: np.ndarray
    y: np.ndarray
    point_offsets: np.ndarray
    polygons: Polygons
    polygon_offsets: np.ndarray
    boxes: np.ndarray

    @property
    def num_instances(self):
        return len(self.point_offsets) - 1


def _log_uniform_int(rng, lo, hi, n):
    return np.floor(np.exp(rng.uniform(math.log(lo), math.log(hi), n))).astype(np.int64)


def batched_instances(n_instances=4096, points_range=(1e3, 1e6), polygons_range=(1, 2000),
                      side_range=(100.0, 10000.0), vertices_range=(4, 256), seed_offset=0):
    rng = np.random.Generator(np.random.PCG64(SEED + 2 + seed_offset))
    npts = _log_uniform_int(rng, points_range[0], points_range[1], n_instances)
    npoly = _log_uniform_int(rng, polygons_range[0], polygons_range[1], n_instances)
    side = rng.uniform(side_range[0], side_range[1], n_instances)
    origin = rng.uniform(-50000.0, 50000.0, (n_instances, 2))
    boxes = np.stack([origin[:, 0], origin[:, 0] + side, origin[:, 1], origin[:, 1] + side], 1)
    point_offsets = np.concatenate([[0], np.cumsum(npts)]).astype(np.uint64)
    total = int(point_offsets[-1])
    x = np.empty(total)
    y = np.empty(total)
    for i in range(n_instances):
        a, b = int(point_offsets[i]), int(point_offsets[i + 1])
        u = rng.random((2, b - a))
        np.minimum(origin[i, 0] + side[i] * u[0], np.nextafter(boxes[i, 1], -np.inf), out=x[a:b])
        np.minimum(origin[i, 1] + side[i] * u[1], np.nextafter(boxes[i, 3], -np.inf), out=y[a:b])
    pinst = np.repeat(np.arange(n_instances), npoly)
    u = rng.uniform(0.05, 0.95, (len(pinst), 2))
    centers = origin[pinst] + u * side[pinst, None]
    k = rng.integers(vertices_range[0], vertices_range[1] + 1, len(pinst))
    prad = side[pinst] * rng.uniform(0.005, 0.05, len(pinst))
    polys = star_polygons(rng, centers, k,
                          lambda g, pid: prad[pid] * g.uniform(0.5, 1.0, len(pid)))
    polygon_offsets = np.concatenate([[0], np.cumsum(npoly)]).astype(np.uint64)
    return BatchedWorkload(x, y, point_offsets, polys, polygon_offsets, boxes)


def serving_polygons(grid=500, extent=20000.0, vertices_range=(8, 256), radius_range=(1.0, 30.0),
                     seed_offset=0):
    rng = np.random.Generator(np.random.PCG64(SEED + 3 + seed_offset))
    step = extent / grid
    gx, gy = np.meshgrid(np.arange(grid), np.arange(grid))
    centers = np.stack([(gx.ravel() + rng.uniform(0.25, 0.75, grid * grid)) * step,
                        (gy.ravel() + rng.uniform(0.25, 0.75, grid * grid)) * step], 1)
    k = rng.integers(vertices_range[0], vertices_range[1] + 1, grid * grid)
    prad = rng.uniform(radius_range[0], radius_range[1], grid * grid)
    return star_polygons(rng, centers, k,
                         lambda g, pid: prad[pid] * g.uniform(0.5, 1.0, len(pid)))


@dataclass
class Request:
    x: np.ndarray
    y: np.ndarray
    kind: str


def serving_requests(n_requests, points_range=(1, 100_000), extent=20000.0, seed_offset=0):
    rng = np.random.Generator(np.random.PCG64(SEED + 13 + seed_offset))
    sizes = _log_uniform_int(rng, points_range[0], points_range[1] + 1, n_requests)
    hi = np.nextafter(extent, 0.0)
    out = []
    for i, n in enumerate(sizes):
        if rng.random() < 0.5:
            x = rng.uniform(0.0, extent, n)
            y = rng.uniform(0.0, extent, n)
            kind = "uniform"
        else:
            c = rng.uniform(0.0, extent, 2)
            sig = rng.uniform(5.0, 500.0)
            x = np.clip(c[0] + sig * rng.standard_normal(n), 0.0, hi)
            y = np.clip(c[1] + sig * rng.standard_normal(n), 0.0, hi)
            kind = "cluster"
        out.append(Request(x, y, kind))
    return out


@dataclass
class PointsPolygons:
    x: np.ndarray
    y: np.ndarray
    polygons: Polygons


def regular_polygons(n_polygons, sides, radius=10.0, center=(0.0, 0.0)):
    """n identical closed regular polygons (sides + 1 vertices per ring)."""
    k = np.arange(sides + 1)
    ang = 2.0 * math.pi * (k % sides) / sides
    rx = center[0] + radius * np.cos(ang)
    ry = center[1] + radius * np.sin(ang)
    x = np.tile(rx, n_polygons)
    y = np.tile(ry, n_polygons)
    ring_offset = np.arange(n_polygons + 1, dtype=np.int32) * (sides + 1)
    part_offset = np.arange(n_polygons + 1, dtype=np.int32)
    return Polygons(x, y, ring_offset, part_offset, part_offset.copy())


def unindexed_pip(n_points=10_000_000, n_polygons=31, sides=100, radius=10.0, seed_offset=0):
    rng = np.random.Generator(np.random.PCG64(SEED + 7 + seed_offset))
    x = rng.uniform(-2 * radius, 2 * radius, n_points)
    y = rng.uniform(-2 * radius, 2 * radius, n_points)
    return PointsPolygons(x, y, regular_polygons(n_polygons, sides, radius))


def pairwise_pip(n=100_000, vertices_range=(4, 400), boundary_fraction=0.2, seed_offset=0):
    """Point i paired with star polygon i: inside, outside or on the boundary."""
    rng = np.random.Generator(np.random.PCG64(SEED + 8 + seed_offset))
    centers = rng.uniform(-1000, 1000, (n, 2))
    k = _log_uniform_int(rng, vertices_range[0], vertices_range[1], n)
    polys = star_polygons(rng, centers, k, lambda g, pid: g.uniform(1, 20, len(pid)),
                          hole_fraction=0.1)
    # a point at a random offset from the centre, radius U[0, 25]
    ang = rng.uniform(0, 2 * math.pi, n)
    rad = rng.uniform(0, 25, n)
    x = centers[:, 0] + rad * np.cos(ang)
    y = centers[:, 1] + rad * np.sin(ang)
    # some points moved onto a vertex or next to an edge of their own polygon
    b = np.nonzero(rng.random(n) < boundary_fraction)[0]
    if len(b):
        ring = polys.part_offset[b]  # the outer ring of polygon b
        rb = polys.ring_offset[ring].astype(np.int64)
        rl = polys.ring_offset[ring + 1].astype(np.int64) - rb
        j = rb + (rng.random(len(b)) * (rl - 1)).astype(np.int64)
        t = np.where(rng.random(len(b)) < 0.5, 0.0, rng.random(len(b)))
        dx, dy = polys.x[j + 1] - polys.x[j], polys.y[j + 1] - polys.y[j]
        ln = np.hypot(dx, dy)
        ln[ln == 0] = 1.0
        off = np.where(t == 0.0, 0.0, rng.uniform(-1e-9, 1e-9, len(b)))
        x[b] = polys.x[j] + t * dx - dy / ln * off
        y[b] = polys.y[j] + t * dy + dx / ln * off
    return PointsPolygons(x, y, polys)
