"""The CPU oracle pinned against the reference's own known answers and against
independent restatements (CPU only, no GPU)."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests import phr_py
from tests.helpers import canonical_equal, first_mismatch
from trace_gb300 import scenes

GOLD = os.path.join(os.path.dirname(__file__), "golden")
TABLES = json.load(open(os.path.join(GOLD, "morton256.json")))["tables"]


def spread_by_tables(v, axis="x"):
    """splitBy3 built from the reference's byte tables (morton.go:23-129)."""
    t = np.asarray(TABLES[axis], np.uint64)
    v = np.asarray(v, np.uint64) & np.uint64(0x1FFFFF)
    return (t[v & np.uint64(255)] | (t[(v >> np.uint64(8)) & np.uint64(255)] << np.uint64(24))
            | (t[(v >> np.uint64(16)) & np.uint64(255)] << np.uint64(48)))


def test_split_by3_matches_reference_tables():
    for b in range(256):
        assert O.split_by3(b) == TABLES["x"][b]
        assert O.split_by3(b) << 1 == TABLES["y"][b]
        assert O.split_by3(b) << 2 == TABLES["z"][b]


def test_encode_matches_table_composition():
    rng = np.random.default_rng(0)
    for _ in range(2000):
        x, y, z = (int(v) for v in rng.integers(0, 1 << 21, 3))
        want = int(spread_by_tables(x, "x")) | int(spread_by_tables(y, "y")) | int(spread_by_tables(z, "z"))
        assert O.lib().orc_encode(x, y, z) == want
    # bits above 21 are masked (morton.go:13)
    assert O.split_by3((1 << 21) | 5) == O.split_by3(5)
    assert O.lib().orc_encode((1 << 21) - 1, (1 << 21) - 1, (1 << 21) - 1) == (1 << 63) - 1


def numpy_morton(verts):
    """float64 restatement of lbvh.go:64-73 with table-based interleave."""
    v = verts.astype(np.float64).reshape(-1, 3, 3)
    lo, hi = v.min(axis=1), v.max(axis=1)
    c = (lo + hi) * 0.5
    elo, ehi = lo.min(axis=0), hi.max(axis=0)
    step = (ehi - elo) / float(2097151)
    with np.errstate(invalid="ignore", divide="ignore"):
        q = np.abs(elo - c) / step
    q = np.where(np.isfinite(q), q, 0.0)
    qi = np.floor(q).astype(np.uint64)
    return (spread_by_tables(qi[:, 0], "x") | spread_by_tables(qi[:, 1], "y") | spread_by_tables(qi[:, 2], "z"))


@pytest.mark.parametrize("n", [1, 7, 1000, 20000])
def test_morton_codes_numpy_restatement(n):
    s = scenes.soup(n, seed=11)
    boxes = O.prim_boxes(s["verts"])
    codes = O.morton(boxes, O.enclosing(boxes))
    assert np.array_equal(codes, numpy_morton(s["verts"]))


def test_morton_zero_extent_axis():
    """A flat scene has a zero-width axis: 0/0 is NaN and quantises to 0 (lbvh.go:69-71)."""
    s = scenes.terrain_tris(9, seed=2)
    s[:, 1::3] = 0.25
    boxes = O.prim_boxes(s)
    codes = O.morton(boxes, O.enclosing(boxes))
    assert np.all((codes & np.uint64(0x2492492492492492)) == 0)  # no y bit set
    assert np.array_equal(codes, numpy_morton(s))


def test_sort_is_stable_and_matches_numpy():
    rng = np.random.default_rng(5)
    codes = rng.integers(0, 1 << 20, 50000).astype(np.uint64) << np.uint64(40)
    sc, si = O.sort_pairs(codes, threads=4)
    order = np.argsort(codes, kind="stable")
    assert np.array_equal(sc, codes[order])
    assert np.array_equal(si, order.astype(np.int32))


def test_sort_bucket_4096_is_an_error():
    """Codes >= 4096*bucketSize land in bucket 4096 and the Go builder panics (lbvh.go:240-245)."""
    codes = np.array([1, (1 << 63) - 1], np.uint64)
    with pytest.raises(RuntimeError):
        O.sort_pairs(codes)


def radix_tree_export(codes, idx, boxes):
    """Independent binary radix tree: split each range at the highest bit of
    first^last (a different formulation of lbvh.go:133-203)."""
    kind, count, box, prims = [], [], [], []

    def rec(a, b):
        if codes[a] == codes[b - 1]:
            p = idx[a:b]
            bx = boxes[p]
            kind.append(1)
            count.append(b - a)
            box.append(np.concatenate([bx[:, :3].min(0), bx[:, 3:].max(0)]))
            prims.extend(p.tolist())
            return box[-1]
        bit = int(codes[a] ^ codes[b - 1]).bit_length() - 1
        mask = np.uint64(1 << bit)
        s = a + int(np.searchsorted((codes[a:b] & mask) != 0, True))
        me = len(kind)
        kind.append(0)
        count.append(2)
        box.append(None)
        l = rec(a, s)
        r = rec(s, b)
        box[me] = np.concatenate([np.minimum(l[:3], r[:3]), np.maximum(l[3:], r[3:])])
        return box[me]

    rec(0, len(codes))
    return (np.asarray(kind, np.int8), np.asarray(count, np.int32), np.asarray(box, np.float64),
            np.asarray(prims, np.int32))


@pytest.mark.parametrize("n,seed", [(2, 1), (100, 2), (3000, 3)])
def test_lbvh_topology_independent(n, seed):
    s = scenes.soup(n, seed=seed)
    b = O.lbvh(s["verts"], threads=3)
    codes, idx = b.sorted_pairs(n)
    want = radix_tree_export(codes, idx, O.prim_boxes(s["verts"]))
    got = b.export()
    assert canonical_equal(got, want), first_mismatch(got, want)
    assert b.size() == 2 * len(np.unique(codes)) - 1


def test_lbvh_duplicates_make_multi_prim_leaves():
    """Equal codes become one leaf with all their primitives (lbvh.go:134-145)."""
    s = scenes.soup(200, seed=4)["verts"]
    v = np.concatenate([s, s, s[:50]])
    b = O.lbvh(v)
    kind, count, box, prims = b.export()
    assert count[kind == 1].max() >= 2
    assert sorted(prims.tolist()) == list(range(len(v)))


def test_lbvh_root_leaf():
    """All centroids equal: the root is one leaf (the Go refit would panic, bvh.go:202)."""
    t = np.tile(np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0]], np.float32), (5, 1))
    b = O.lbvh(t)
    kind, count, box, prims = b.export()
    assert kind.tolist() == [1] and count.tolist() == [5] and prims.tolist() == [0, 1, 2, 3, 4]


def test_cost_hand_computed():
    """bvh.go:226-239 on a two-leaf tree: 2 + A(l)/A(root)*1 + A(r)/A(root)*1."""
    t = np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0], [3, 0, 0, 4, 0, 0, 3, 1, 0]], np.float32)
    t[:, 2::3] += np.array([[0, 0, 1], [0, 0, 1]], np.float32)  # give both a z extent of 1
    b = O.lbvh(t)
    a_leaf = 2 * (1 * 1 + 1 * 1 + 1 * 1)
    a_root = 2 * (4 * 1 + 4 * 1 + 1 * 1)
    assert b.cost() == pytest.approx(2 + 2 * a_leaf / a_root, rel=1e-15)


def brute_force_closest(verts, rays):
    """Moeller-Trumbore over every triangle in float64 (vectorised)."""
    v = verts.astype(np.float64).reshape(-1, 3, 3)
    v0, e1, e2 = v[:, 0], v[:, 1] - v[:, 0], v[:, 2] - v[:, 0]
    out_p, out_t = [], []
    for r in rays.astype(np.float64):
        o, d, tmin, tmax = r[0:3], r[4:7], r[3], r[7]
        pv = np.cross(d, e2)
        det = np.einsum("ij,ij->i", e1, pv)
        with np.errstate(divide="ignore", invalid="ignore"):
            inv = 1 / det
            tv = o - v0
            u = np.einsum("ij,ij->i", tv, pv) * inv
            qv = np.cross(tv, e1)
            vv = (qv @ d) * inv
            t = np.einsum("ij,ij->i", e2, qv) * inv
        ok = (np.abs(det) > 1e-7) & (u >= 0) & (u <= 1) & (vv >= 0) & (u + vv <= 1) & (t >= tmin) & (t <= tmax)
        if ok.any():
            tt = np.where(ok, t, np.inf)
            out_p.append(int(np.argmin(tt)))
            out_t.append(tt.min())
        else:
            out_p.append(-1)
            out_t.append(np.inf)
    return np.asarray(out_p), np.asarray(out_t)


def test_trace_matches_brute_force():
    s = scenes.soup(40000, seed=7)
    b = O.lbvh(s["verts"])
    rays = scenes.camera_rays(s["camera"], 32, 18, jitter_seed=3)
    p, t, _, _ = b.trace(rays)
    bp, bt = brute_force_closest(s["verts"], rays)
    assert (p >= 0).mean() > 0.1
    np.testing.assert_allclose(t[p >= 0], bt[p >= 0], rtol=1e-12)
    assert np.array_equal(p >= 0, bp >= 0)
    assert (p == bp).mean() > 0.999


def test_trace_lbvh_equals_phr_closest_distance():
    s = scenes.cornell()
    b = O.lbvh(s["verts"])
    ph = b.phr(0.5, 6, 2)
    rays = scenes.camera_rays(s["camera"], 64, 64)
    p1, t1, _, _ = b.trace(rays)
    p2, t2, _, _ = ph.trace(rays)
    np.testing.assert_array_equal(t1, t2)


@pytest.mark.parametrize("n,alpha,delta,bf", [(300, 0.5, 6, 2), (2000, 0.5, 6, 2), (2000, 0.55, 9, 4),
                                              (1500, 0.5, 3, 3), (972, 0.5, 6, 2)])
def test_phr_matches_python_restatement(n, alpha, delta, bf):
    s = scenes.cornell() if n == 972 else scenes.soup(n, seed=n)
    b = O.lbvh(s["verts"])
    aux_tree = phr_py.parse(*b.export())
    st = {}
    want = phr_py.export(phr_py.phr(aux_tree, alpha, delta, bf, st))
    ph = b.phr(alpha, delta, bf)
    got = ph.export()
    assert canonical_equal(got, want), first_mismatch(got, want)
    assert ph.stats["build_cost"] == st["build_cost"]  # BuildWithCost's count


def test_phr_invariants():
    s = scenes.soup(5000, seed=9)
    b = O.lbvh(s["verts"])
    for bf in (2, 3, 4):
        ph = b.phr(0.5, 6, bf)
        kind, count, box, prims = ph.export()
        assert sorted(prims.tolist()) == list(range(5000))
        assert count[kind == 0].max() <= bf
        assert ph.cost() < b.cost()  # the refinement lowers the SAH cost on a random soup


def test_render_light_only_sees_emission():
    """A camera looking straight at an emitter of radiance 10 with MaxDepth 0 sees 10 (Light, material.go:13-23)."""
    quad = np.array([[-1, -1, 0, 1, -1, 0, 1, 1, 0], [-1, -1, 0, 1, 1, 0, -1, 1, 0]], np.float32)
    b = O.lbvh(quad)
    sc = dict(prim_mat=np.array([0, 0], np.int32), mat_type=np.array([1], np.int32),
              mat_color=np.array([[10.0, 10.0, 10.0]]),
              camera=dict(look_from=(0, 0, 2), look_at=(0, 0, 0), up=(0, 1, 0), fov=20.0, aspect=1.0),
              render=dict(width=8, height=8, spp=2, max_depth=0, miss_mode=0, miss_color=(0, 0, 0)))
    img = b.render(sc)
    np.testing.assert_allclose(img, 10.0)


def test_heatmap_matches_python_restatement():
    """The oracle's heat map (render.go:137-197, bvh.go:21-44) against tests/heat_py.py on the
    Cornell box, LBVH and PHR trees: identical step counts and colours."""
    from tests import heat_py

    s = scenes.cornell()
    w, h, thr = 24, 18, 20
    cam = dict(s["camera"], aspect=w / h)
    tris = [tuple(float(x) for x in t) for t in s["verts"]]
    b = O.lbvh(s["verts"])
    for tree in (b, b.phr(0.5, 6, 2), b.phr(0.55, 9, 4)):
        root = phr_py.parse(*tree.export())
        want_c, want_rgb = heat_py.heatmap(root, tris, cam, w, h, thr)
        rgb, counts = tree.heatmap(cam, w, h, thr)
        assert counts.ravel().tolist() == want_c
        np.testing.assert_array_equal(rgb.reshape(-1, 3), np.array(want_rgb))
        assert counts.max() > 0


@pytest.mark.parametrize("kind", ["mirror", "glass"])
def test_render_reflective_and_refractive_exact(kind):
    """Reflective (material.go:44-57) and Refractive (:59-106) in the oracle renderer on
    scenes whose every path is known: albedo * Le after a mirror, albedo^2 * Le through a
    ratio-1 slab."""
    from tests.helpers import clear_glass_scene, mirror_scene

    s = mirror_scene() if kind == "mirror" else clear_glass_scene()
    s["render"] = dict(width=16, height=16, spp=4, max_depth=3, miss_mode=0, miss_color=(0.0, 0.0, 0.0))
    img = O.lbvh(s["verts"]).render(s)
    a, le = np.asarray(s["mat_color"][0]), s["mat_color"][1][0]
    want = a * le if kind == "mirror" else a * a * le
    np.testing.assert_allclose(img.reshape(-1, 3), np.broadcast_to(want, (256, 3)), rtol=1e-9)


def _to_image_py(rgb):
    """buffer.go:60-69 with math.go:20-25, written out pixel by pixel: the row of buffer
    index i is height - i // width (row 0 falls outside the image); each channel is
    uint8(Clamp(sqrt(c), 0, 1) * 255) with Go's truncation (NaN -> 0)."""
    import math

    h, w, _ = rgb.shape
    out = np.zeros((h, w, 4), np.uint8)
    flat = rgb.reshape(-1, 3)
    for i in range(w * h):
        x, y = i % w, h - i // w
        if not (0 <= y < h):
            continue
        px = []
        for c in flat[i]:
            s = math.sqrt(float(c)) if float(c) >= 0 else float("nan")
            s = 0.0 if s < 0.0 else (1.0 if s > 1.0 else s)
            v = s * 255.0
            px.append(0 if v != v else int(v))
        out[y, x] = px + [255]
    return out


def test_oracle_to_image_matches_python_restatement():
    rng = np.random.default_rng(3)
    h, w = 7, 5
    rgb = rng.uniform(-0.2, 1.3, (h, w, 3)).astype(np.float32)
    # exact squares of k/255 and their neighbours, where the truncation turns
    k = np.arange(0, 256, dtype=np.float64) / 255.0
    sq = (k * k).astype(np.float32)
    edge = np.concatenate([sq, np.nextafter(sq, np.float32(-1)), np.nextafter(sq, np.float32(2)),
                           np.array([np.nan, np.inf, -np.inf, -0.0, 0.0, 1.0, 4.0], np.float32)])
    rgb2 = np.resize(edge, 16 * 17 * 3).reshape(16, 17, 3)
    for img in (rgb, rgb2):
        got = O.to_image(img)
        assert np.array_equal(got, _to_image_py(img))
        assert np.all(got[0] == 0)  # image row 0 is never written
