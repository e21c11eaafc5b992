"""Properties of the oracle on seeded random inputs, checked by independent
means: the point-in-polygon test against a convex-polygon half-plane test for
points away from the boundary, the quadtree against the invariants of
cpp/include/cuspatial/detail/index/construction/phase_2.cuh (a permutation,
leaves that partition the sorted points, internal nodes above max_size), and
the box join against a brute-force overlap of every leaf's cell with every
box (pairs clearly overlapping must be there, pairs clearly apart must not),
and the pairwise and nearest-linestring distances against a numpy
point-segment distance."""

import numpy as np
import pytest

from oracle import oracle as O


def _convex_polygons(rng, n, dtype):
    """n convex polygons (regular k-gons, random centre, radius, rotation),
    closed rings; returns offsets, vertices and each polygon's own vertices."""
    xs, ys, ro, po, shapes = [], [], [0], [0], []
    for _ in range(n):
        k = int(rng.integers(3, 12))
        c = rng.uniform(-50, 50, 2)
        r = rng.uniform(1, 20)
        ph = rng.uniform(0, 2 * np.pi)
        a = ph + 2 * np.pi * np.arange(k) / k
        vx, vy = c[0] + r * np.cos(a), c[1] + r * np.sin(a)
        xs += list(vx) + [vx[0]]
        ys += list(vy) + [vy[0]]
        ro.append(len(xs))
        po.append(len(ro) - 1)
        shapes.append((vx.astype(dtype), vy.astype(dtype)))
    return (np.array(po, np.uint32), np.array(ro, np.uint32), np.array(xs, dtype),
            np.array(ys, dtype), shapes)


def _inside_convex(px, py, vx, vy):
    """Signed distance of each point to each edge line of a counter-clockwise
    convex polygon (positive inside), in float64."""
    vx = vx.astype(np.float64)
    vy = vy.astype(np.float64)
    ax, ay = vx, vy
    bx, by = np.roll(vx, -1), np.roll(vy, -1)
    ex, ey = bx - ax, by - ay
    ln = np.hypot(ex, ey)
    d = (ex[None, :] * (py[:, None] - ay[None, :]) - ey[None, :] * (px[:, None] - ax[None, :]))
    return d / ln[None, :]


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_point_in_polygon_matches_half_planes(dtype):
    rng = np.random.default_rng(11)
    po, ro, vx, vy, shapes = _convex_polygons(rng, 31, dtype)
    px = rng.uniform(-75, 75, 20000).astype(dtype)
    py = rng.uniform(-75, 75, 20000).astype(dtype)
    mask = O.point_in_polygon(px, py, po, ro, vx, vy)
    checked = 0
    for p, (sx, sy) in enumerate(shapes):
        d = _inside_convex(px.astype(np.float64), py.astype(np.float64), sx, sy)
        clear = np.all(np.abs(d) > 1e-3, axis=1)  # away from every edge line
        want = np.all(d > 0, axis=1)
        got = ((mask >> p) & 1).astype(bool)
        np.testing.assert_array_equal(got[clear], want[clear], err_msg=str(p))
        checked += int(clear.sum())
    assert checked > 500000


@pytest.mark.parametrize("max_depth,max_size", [(3, 8), (7, 16), (10, 64)])
def test_quadtree_invariants(max_depth, max_size):
    rng = np.random.default_rng(max_depth)
    n = 20000
    x = np.concatenate([rng.normal(300, 40, n // 2), rng.uniform(0, 1000, n - n // 2)])
    y = np.concatenate([rng.normal(700, 40, n // 2), rng.uniform(0, 1000, n - n // 2)])
    x, y = np.clip(x, 0, 1000), np.clip(y, 0, 1000)
    scale = 1000.0 / (1 << max_depth)
    pi, t = O.quadtree_on_points(x, y, 0.0, 1000.0, 0.0, 1000.0, scale, max_depth, max_size)
    assert sorted(pi.tolist()) == list(range(n))  # a permutation
    key, level = t["key"].astype(np.int64), t["level"].astype(np.int64)
    internal = t["is_internal_node"].astype(bool)
    length, offset = t["length"].astype(np.int64), t["offset"].astype(np.int64)
    leaves = ~internal
    # leaves partition the sorted positions
    cover = np.zeros(n, np.int64)
    for o, ln in zip(offset[leaves], length[leaves]):
        cover[o:o + ln] += 1
    assert np.all(cover == 1)
    # every point of a leaf lies in the leaf's cell
    for k, lv, o, ln in zip(key[leaves], level[leaves], offset[leaves], length[leaves]):
        s = scale * (1 << (max_depth - 1 - lv))
        cx = sum(((k >> (2 * b)) & 1) << b for b in range(16))
        cy = sum(((k >> (2 * b + 1)) & 1) << b for b in range(16))
        idx = pi[o:o + ln]
        assert np.all((x[idx] >= cx * s - 1e-9) & (x[idx] <= (cx + 1) * s + 1e-9))
        assert np.all((y[idx] >= cy * s - 1e-9) & (y[idx] <= (cy + 1) * s + 1e-9))
    # internal nodes hold more than max_size points; children are in range
    q = len(key)
    for i in np.nonzero(internal)[0]:
        kids = range(offset[i], offset[i] + length[i])
        assert all(0 <= c < q and level[c] == level[i] + 1 for c in kids)
        total = 0
        stack = list(kids)
        while stack:
            c = stack.pop()
            if internal[c]:
                stack.extend(range(offset[c], offset[c] + length[c]))
            else:
                total += length[c]
        assert total > max_size
    # a leaf above the last level holds at most max_size points
    assert np.all(length[leaves & (level < max_depth - 1)] <= max_size)


def test_join_matches_brute_force_overlap():
    rng = np.random.default_rng(5)
    d, n = 6, 30000
    x = rng.uniform(0, 1000, n)
    y = rng.uniform(0, 1000, n)
    scale = 1000.0 / (1 << d)
    pi, t = O.quadtree_on_points(x, y, 0.0, 1000.0, 0.0, 1000.0, scale, d, 32)
    nb = 300
    cx, cy = rng.uniform(0, 1000, nb), rng.uniform(0, 1000, nb)
    w, h = rng.uniform(1, 80, nb), rng.uniform(1, 80, nb)
    bb = dict(minx=cx - w, miny=cy - h, maxx=cx + w, maxy=cy + h)
    j = O.join_quadtree_and_bounding_boxes(t, bb, 0.0, 1000.0, 0.0, 1000.0, scale, d)
    got = set(zip(j["bbox_offset"].tolist(), j["quad_offset"].tolist()))
    assert len(got) == len(j["bbox_offset"])  # no repeats
    key, level = t["key"].astype(np.int64), t["level"].astype(np.int64)
    leaves = np.nonzero(~t["is_internal_node"].astype(bool))[0]
    clear_in = clear_out = 0
    for q in leaves:
        s = scale * (1 << (d - 1 - level[q]))
        kx = sum(((key[q] >> (2 * b)) & 1) << b for b in range(16))
        ky = sum(((key[q] >> (2 * b + 1)) & 1) << b for b in range(16))
        x0, x1, y0, y1 = kx * s, (kx + 1) * s, ky * s, (ky + 1) * s
        gap = np.maximum.reduce([bb["minx"] - x1, x0 - bb["maxx"], bb["miny"] - y1,
                                 y0 - bb["maxy"]])
        for b in np.nonzero(gap < -1e-6)[0]:  # clearly overlapping
            assert (int(b), int(q)) in got
            clear_in += 1
        for b in np.nonzero(gap > 1e-6)[0]:  # clearly apart
            assert (int(b), int(q)) not in got
            clear_out += 1
    assert clear_in > 1000 and clear_out > 100000
    # the reference's order: leaf first point, then box
    order = list(zip(t["offset"][j["quad_offset"]].tolist(), j["bbox_offset"].tolist()))
    assert order == sorted(order)


def _segment_distances(px, py, lx, ly):
    """Distance from each point to each segment (float64, numpy)."""
    ax, ay, bx, by = lx[:-1], ly[:-1], lx[1:], ly[1:]
    ex, ey = bx - ax, by - ay
    l2 = ex * ex + ey * ey
    t = ((px[:, None] - ax) * ex + (py[:, None] - ay) * ey) / np.where(l2 > 0, l2, 1.0)
    t = np.clip(np.where(l2 > 0, t, 0.0), 0.0, 1.0)
    dx = px[:, None] - (ax + t * ex)
    dy = py[:, None] - (ay + t * ey)
    return np.hypot(dx, dy)


def test_pairwise_distance_matches_brute_force():
    rng = np.random.default_rng(17)
    n = 400
    nv = rng.integers(2, 30, n)
    start = np.concatenate([[0], np.cumsum(nv)])
    lx = np.concatenate([c + np.cumsum(rng.normal(0, 3, k)) for c, k in
                         zip(rng.uniform(-100, 100, n), nv)])
    ly = np.concatenate([c + np.cumsum(rng.normal(0, 3, k)) for c, k in
                         zip(rng.uniform(-100, 100, n), nv)])
    x = lx[start[:-1]] + rng.normal(0, 10, n)
    y = ly[start[:-1]] + rng.normal(0, 10, n)
    o = O.pairwise_point_linestring(x, y, start, lx, ly)
    for i in range(n):
        s = slice(start[i], start[i + 1])
        d = _segment_distances(x[i:i + 1], y[i:i + 1], lx[s], ly[s])[0]
        assert abs(o["distance"][i] - d.min()) <= 1e-9 * max(1.0, d.min())
        seg = int(o["segment_id"][i])
        assert abs(d[seg] - d.min()) <= 1e-9 * max(1.0, d.min())
        assert abs(np.hypot(o["x"][i] - x[i], o["y"][i] - y[i]) - d.min()) <= 1e-9 * max(1.0,
                                                                                         d.min())


def test_nearest_linestring_matches_brute_force():
    rng = np.random.default_rng(23)
    d, n, L = 5, 5000, 60
    x = rng.uniform(0, 1000, n)
    y = rng.uniform(0, 1000, n)
    scale = 1000.0 / (1 << d)
    pi, t = O.quadtree_on_points(x, y, 0.0, 1000.0, 0.0, 1000.0, scale, d, 64)
    nv = rng.integers(2, 20, L)
    lo = np.concatenate([[0], np.cumsum(nv)]).astype(np.uint32)
    lx = np.concatenate([c + np.cumsum(rng.normal(0, 15, k)) for c, k in
                         zip(rng.uniform(0, 1000, L), nv)])
    ly = np.concatenate([c + np.cumsum(rng.normal(0, 15, k)) for c, k in
                         zip(rng.uniform(0, 1000, L), nv)])
    bb = O.linestring_bounding_boxes(lo, lx, ly, 60.0)
    j = O.join_quadtree_and_bounding_boxes(t, bb, 0.0, 1000.0, 0.0, 1000.0, scale, d)
    r = O.quadtree_point_to_nearest_linestring(j, t, pi, x, y, lo, lx, ly)
    # candidates of each sorted position: the linestrings paired with its leaf
    cand = {}
    off, ln = t["offset"], t["length"]
    for b, q in zip(j["bbox_offset"], j["quad_offset"]):
        for pos in range(int(off[q]), int(off[q] + ln[q])):
            cand.setdefault(pos, []).append(int(b))
    checked = 0
    for row, (pos, ls, dist) in enumerate(zip(r["point_index"], r["linestring_index"],
                                              r["distance"])):
        if int(pos) not in cand:
            continue
        p = int(pi[pos])
        best = [(_segment_distances(x[p:p + 1], y[p:p + 1], lx[lo[c]:lo[c + 1]],
                                    ly[lo[c]:lo[c + 1]])[0].min(), c) for c in cand[int(pos)]]
        dmin = min(b[0] for b in best)
        assert abs(dist - dmin) <= 1e-9 * max(1.0, dmin)
        # ties (equal distances) go to the lower id; a clear winner must be it
        clear = sorted(b[0] for b in best)
        if len(clear) == 1 or clear[1] - clear[0] > 1e-6:
            assert int(ls) == min(best)[1]
        checked += 1
    assert checked > 2000
