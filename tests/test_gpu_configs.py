"""Parity at the full sizes of the benchmarked workloads, against the oracle.

  terrain   2048x2048 fBm heightfield (8,380,418 triangles) plus its sun sphere:
            Morton codes, sorted pairs and the LBVH (pre-order topology and
            boxes) bit-exact (lbvh.go:17-25); the PHR trees at (0.5, 6, 2) and
            at the grid optimiser's choice equal to the oracle's (phr.go:47-84)
  soup      1M triangles, PHR(0.5, 6, 2): closest-hit IDs on the full 1920x1080
            camera-ray set plus one deterministic diffuse bounce per hit
            (bvh.go:179-199); >= 99.99% agreement, no hard mismatch, near-ties
            counted and printed
  cornell   ~1k triangles, 256x256, 16 spp, MaxDepth 5 (render.go:91-129):
            per-channel RMSE against a converged oracle image within the
            renderer tests' ratio of the oracle's own at equal spp
  adjoint   the Cornell box with a 256x128 UV sphere (65,036 triangles):
            central differences (h = 1e-3) on the 12 largest gradients within
            1e-3 relative
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import canonical_equal, classify_disagreements, first_mismatch
from tests.test_gpu_render import run as render_parity
from tests.test_gpu_trace import T_REL, bounce_rays
from trace_gb300 import pt, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def terrain_full(ctx):
    s = scenes.terrain(2048)
    ds = pt.DeviceScene.from_dict(ctx, s)
    g = pt.DefaultLBVH(ds)
    o = O.lbvh(s["verts"], s["spheres"])
    yield s, ds, g, o
    g.close()
    ds.close()


def test_terrain_full_lbvh_bit_exact(terrain_full):
    s, ds, g, o = terrain_full
    n = s["verts"].shape[0] + s["spheres"].shape[0]
    assert n == 8_380_419
    gc, gi = g.sorted_pairs()
    oc, oi = o.sorted_pairs(n)
    assert np.array_equal(gc, oc), "Morton code sequence differs"
    assert np.array_equal(gi, oi), "sorted primitive order differs"
    del gc, gi, oc, oi
    gk, gn, gb, gp = g.export()
    ok, on, ob, op = o.export()
    assert np.array_equal(gk, ok) and np.array_equal(gn, on), "topology differs"
    assert np.array_equal(gp, op), "leaf primitives differ"
    assert g.Size() == o.size()
    # triangle boxes are exact; the boxes enclosing the sun sphere (its leaf and that leaf's
    # ancestors) are the float64 box rounded outward to float32
    diff = np.nonzero(np.any(gb != ob, axis=1))[0]
    print("terrain LBVH: %d nodes, %d boxes holding the sphere" % (len(gk), len(diff)))
    assert len(diff) <= 64
    assert np.all(gb[diff, :3] <= ob[diff, :3]) and np.all(gb[diff, 3:] >= ob[diff, 3:])
    np.testing.assert_allclose(gb[diff], ob[diff], rtol=1e-6, atol=1e-6)


@pytest.mark.parametrize("alpha,delta", [(0.5, 6.0), (0.55, 12.0)])
def test_terrain_full_phr_tree_equals_oracle(terrain_full, alpha, delta):
    s, ds, g, o = terrain_full
    ph = pt.NewPHRBuilder(alpha, delta, 2).BuildFromAuxilary(g)
    oph = o.phr(alpha, delta, 2)
    ge, oe = ph.export(), oph.export()
    assert canonical_equal(ge, oe), first_mismatch(ge, oe)
    assert ph.Cost() == oph.cost()
    print("terrain PHR(%g, %g, 2): %d nodes, SAH %.4f" % (alpha, delta, len(ge[0]), oph.cost()))
    ph.close()


def test_terrain_full_grid_choice_equals_oracle(terrain_full):
    """The grid optimiser's pick for the 1920x1080 frame (the grid the terrain render uses):
    the chosen candidate's SAH and build cost and its tree equal the oracle's."""
    s, ds, g, o = terrain_full
    rd = s["render"]
    opt = pt.NewGridOptimizer([0.4, 0.5, 0.55], [6, 8, 10, 12], rd["width"], rd["height"])
    alpha, delta = opt.OptimizedPHRparams(g, 2)
    k = [(e[0], e[1]) for e in opt.evaluations].index((alpha, delta))
    _, _, sah, build = opt.evaluations[k]
    oph = o.phr(alpha, delta, 2)
    print("terrain grid choice (%g, %g): SAH %.4f build cost %d" % (alpha, delta, sah, build))
    assert build == oph.stats["build_cost"]
    assert sah == pytest.approx(oph.cost(), rel=1e-12)
    ph = pt.NewPHRBuilder(alpha, delta, 2).BuildFromAuxilary(g)
    ge, oe = ph.export(), oph.export()
    assert canonical_equal(ge, oe), first_mismatch(ge, oe)
    ph.close()


def _check_hits(g, o, rays, label, verts):
    """Closest hits against the float64 oracle.  Disagreements are near-ties when float32
    rounding decides them: equal distances, or a barycentric margin within the float32
    rounding bound of Moeller-Trumbore for that triangle and ray (grazing rays, whose
    determinant is near the reference's absolute 1e-7 cut-off, lose the most)."""
    gp, gt, _, _ = g.trace(rays)
    op, ot, _, _ = o.trace(rays)
    agree = (gp == op).mean()
    near, hard = classify_disagreements(o, rays, gp, gt, op, ot, verts=verts)
    both = (gp == op) & (op >= 0)
    rel = np.abs(gt[both] - ot[both]) / np.maximum(np.abs(ot[both]), 1e-30)
    print("%s: rays=%d hit=%.4f agree=%.6f near_ties=%d (%.2e of rays) hard=%d t_rel_max=%.2e" % (
        label, len(rays), (op >= 0).mean(), agree, len(near), len(near) / max(1, len(rays)), len(hard),
        rel.max() if rel.size else 0.0))
    assert len(hard) == 0, "hard hit-ID mismatches at rays %s" % hard[:10]
    assert agree >= 0.9999
    assert len(near) <= 1e-4 * len(rays)
    assert (rel <= T_REL).mean() >= 0.9999
    return gp, gt


def test_soup_full_frame_hit_ids_on_phr(ctx):
    s = scenes.soup(1_000_000, seed=1)
    ds = pt.DeviceScene.from_dict(ctx, s)
    g = pt.NewPHRBuilder(0.5, 6.0, 2).BuildFromAuxilary(pt.DefaultLBVH(ds))
    o = O.lbvh(s["verts"]).phr(0.5, 6.0, 2)
    rays = scenes.camera_rays(s["camera"], 1920, 1080, jitter_seed=6)
    assert rays.shape[0] == 1920 * 1080
    gp, gt = _check_hits(g, o, rays, "soup1M PHR camera 1920x1080", s["verts"])
    b = bounce_rays(s["verts"], rays, gp, gt, seed=10)
    _check_hits(g, o, b, "soup1M PHR bounce", s["verts"])


def test_cornell_full_render(ctx):
    """256x256, 16 spp, MaxDepth 5, black miss."""
    s = scenes.cornell()
    assert (s["render"]["width"], s["render"]["height"], s["render"]["spp"], s["render"]["max_depth"]) == (
        256, 256, 16, 5)
    st = render_parity(ctx, s, 256, 256, spp_eq=16, spp_conv=512, spp_hi=4096)
    assert st["rays_traced"] >= 256 * 256 * 16


def test_adjoint_65k_central_differences(ctx):
    H, REL = 1e-3, 1e-3
    s = scenes.cornell(sphere_u=256, sphere_v=128)
    n = s["verts"].shape[0]
    assert n == 65_036
    w, h = 128, 128
    ds = pt.DeviceScene.from_dict(ctx, s)
    g = pt.DefaultLBVH(ds)
    r4, r5 = np.random.default_rng(4), np.random.default_rng(5)
    a0, e0 = r4.uniform(0.2, 0.8, (n, 3)).astype(np.float32), r4.uniform(0.2, 0.8, n).astype(np.float32)
    a1, e1 = r5.uniform(0.2, 0.8, (n, 3)).astype(np.float32), r5.uniform(0.2, 0.8, n).astype(np.float32)
    cam = dict(s["camera"], aspect=w / h)
    f = pt.RenderFunction(g, cam, dict(width=w, height=h, spp=16, max_depth=5, miss_mode=0, seed=7))
    try:
        f.set_target(f.Forward(a1, e1))
        loss, ga, ge = f.loss_and_grad(a0, e0)
        assert np.isfinite(ga).all() and np.isfinite(ge).all() and loss > 0
        flat = np.concatenate([np.abs(ga).ravel(), np.abs(ge)])
        worst = 0.0
        for k in np.argsort(-flat)[:12]:
            a_p, a_m, e_p, e_m = a0.copy(), a0.copy(), e0.copy(), e0.copy()
            if k < 3 * n:
                t, c = divmod(int(k), 3)
                a_p[t, c] += H
                a_m[t, c] -= H
                step, gk = float(a_p[t, c]) - float(a_m[t, c]), float(ga[t, c])
                label = "albedo[%d,%d]" % (t, c)
            else:
                t = int(k) - 3 * n
                e_p[t] += H
                e_m[t] -= H
                step, gk = float(e_p[t]) - float(e_m[t]), float(ge[t])
                label = "emission[%d]" % t
            fd = (f.loss(a_p, e_p) - f.loss(a_m, e_m)) / step
            rel = abs(fd - gk) / max(abs(fd), 1e-12)
            print("%s adjoint %.6e fd %.6e rel %.2e" % (label, gk, fd, rel))
            worst = max(worst, rel)
        assert worst <= REL, worst
    finally:
        f.close()
