"""Comparison helpers shared by the parity tests."""
import numpy as np

EPS32 = 2.0 ** -24  # unit roundoff of float32
COND_C = 4.0        # rounding steps allowed in the bound of a float32 barycentric coordinate


def mt_float32_margin_bound(verts, prim, ray):
    """Bound on the float32 rounding error of Moeller-Trumbore's u and v (primitive.go:172-208)
    for one triangle and ray, from float64: u = (tv . pv) / det and v = (d . qv) / det lose
    about EPS32 * (|tv| |pv|) / |det| and EPS32 * (|d| |qv|) / |det|, which is large when the
    ray grazes the triangle's plane (|det| near the reference's 1e-7 cut-off)."""
    v = np.asarray(verts[prim], np.float64).reshape(3, 3)
    o = np.asarray(ray[0:3], np.float64)
    d = np.asarray(ray[4:7], np.float64)
    e1, e2 = v[1] - v[0], v[2] - v[0]
    pv = np.cross(d, e2)
    det = float(np.dot(e1, pv))
    if det == 0.0:
        return np.inf
    tv = o - v[0]
    qv = np.cross(tv, e1)
    cu = np.linalg.norm(tv) * np.linalg.norm(pv) / abs(det)
    cv = np.linalg.norm(d) * np.linalg.norm(qv) / abs(det)
    return COND_C * EPS32 * max(cu, cv, 1.0)


def classify_disagreements(orc_bvh, rays, gpu_prim, gpu_t, orc_prim, orc_t, rel_tie=1e-5, edge=1e-4, verts=None):
    """Split hit-ID disagreements into near-ties and hard mismatches.

    near-tie: both primitives are hit in float64 at distances within rel_tie
    (an equal-distance tie whose winner depends on traversal order), or the
    primitive one side reports lies within `edge` of a barycentric or
    distance boundary in float64 (float32 rounding decides it).  With `verts`
    (the scene's triangles), the barycentric margin is also compared with the
    float32 rounding bound of that triangle and ray (mt_float32_margin_bound),
    which covers grazing rays whose float32 u, v are off by more than `edge`.
    """
    bad = np.nonzero(gpu_prim != orc_prim)[0]
    near, hard = [], []
    n_tri = None if verts is None else len(verts)
    for i in bad:
        r = rays[i]
        gp, op = int(gpu_prim[i]), int(orc_prim[i])
        tie = False
        if gp >= 0 and op >= 0:
            ok, t, u, v, det = orc_bvh.prim_intersect(gp, r)
            if ok and abs(t - orc_t[i]) <= rel_tie * max(1.0, abs(orc_t[i])):
                tie = True
        for p in (gp, op):
            if tie or p < 0:
                continue
            ok, t, u, v, det = orc_bvh.prim_intersect(p, r)
            margin = min(abs(u), abs(1 - u), abs(v), abs(1 - u - v))
            if margin <= edge or abs(abs(det) - 1e-7) <= 1e-7 * 0.5 or abs(t - r[3]) <= edge * max(1.0, abs(t)):
                tie = True
            elif n_tri is not None and p < n_tri and margin <= mt_float32_margin_bound(verts, p, r):
                tie = True
            if p == gp and op >= 0 and not ok:
                # the GPU's primitive is not hit in float64 but the closest is: compare distances
                ok2, t2, *_ = orc_bvh.prim_intersect(op, r)
                if ok2 and np.isfinite(t) and abs(t - t2) <= 1e-4 * max(1.0, abs(t2)):
                    tie = True
        (near if tie else hard).append(int(i))
    return np.asarray(near, np.int64), np.asarray(hard, np.int64)


def canonical_equal(a, b):
    """Exact equality of two pre-order exports (kind, count, box, prims)."""
    ka, ca, ba, pa = a
    kb, cb, bb, pb = b
    return (ka.shape == kb.shape and np.array_equal(ka, kb) and np.array_equal(ca, cb)
            and np.array_equal(pa, pb) and np.array_equal(ba, bb))


def first_mismatch(a, b):
    ka, ca, ba, pa = a
    kb, cb, bb, pb = b
    n = min(len(ka), len(kb))
    for i in range(n):
        if ka[i] != kb[i] or ca[i] != cb[i]:
            return "node %d kind/count %s/%s vs %s/%s" % (i, ka[i], ca[i], kb[i], cb[i])
        if not np.array_equal(ba[i], bb[i]):
            return "node %d box %s vs %s" % (i, ba[i], bb[i])
    if len(ka) != len(kb):
        return "node count %d vs %d" % (len(ka), len(kb))
    m = np.nonzero(pa != pb)[0]
    return "prims differ at %s" % m[:5] if len(m) else "equal"


def _quad(c, a, b):
    c, a, b = (np.asarray(x, np.float64) for x in (c, a, b))
    p0, p1, p2, p3 = c, c + a, c + a + b, c + b
    return [np.concatenate([p0, p1, p2]), np.concatenate([p0, p2, p3])]


def mirror_scene(albedo=(0.8, 0.6, 0.4), le=5.0):
    """A Reflective mirror (diffusion 0) at z = -1 facing a camera at the origin; a Light
    plane at z = +1 behind the camera: every camera ray reflects into the light, so each
    pixel is albedo * Le exactly (MaxDepth >= 1)."""
    tris = _quad([-10, -10, -1], [20, 0, 0], [0, 20, 0]) + _quad([-10, -10, 1], [0, 20, 0], [20, 0, 0])
    return dict(verts=np.asarray(tris, np.float32), spheres=np.zeros((0, 4), np.float32),
                prim_mat=np.array([0, 0, 1, 1], np.int32), mat_type=np.array([2, 1], np.int32),
                mat_color=np.array([albedo, [le, le, le]]), mat_param=np.array([0.0, 0.0]),
                camera=dict(look_from=(0, 0, 0), look_at=(0, 0, -1), up=(0, 1, 0), fov=10.0, aspect=1.0))


def clear_glass_scene(albedo=(0.9, 0.8, 0.7), le=5.0):
    """A Refractive slab of ratio 1 (faces at z = -1 and z = -1.2) in front of a Light plane
    at z = -3: near-normal rays pass straight through both faces (Schlick reflectance
    (1 - cos)^5 ~ 0), so each pixel is albedo^2 * Le (MaxDepth >= 2)."""
    tris = (_quad([-10, -10, -1], [20, 0, 0], [0, 20, 0]) + _quad([-10, -10, -1.2], [0, 20, 0], [20, 0, 0])
            + _quad([-10, -10, -3], [20, 0, 0], [0, 20, 0]))
    return dict(verts=np.asarray(tris, np.float32), spheres=np.zeros((0, 4), np.float32),
                prim_mat=np.array([0, 0, 0, 0, 1, 1], np.int32), mat_type=np.array([3, 1], np.int32),
                mat_color=np.array([albedo, [le, le, le]]), mat_param=np.array([1.0, 0.0]),
                camera=dict(look_from=(0, 0, 0), look_at=(0, 0, -1), up=(0, 1, 0), fov=10.0, aspect=1.0))
