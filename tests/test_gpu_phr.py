"""GPU PHR vs the oracle's PHR: the same tree (splits, tie orders, leaves),
hence the same SAH cost (bar: within 1%) and the same closest hits."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import canonical_equal, classify_disagreements, first_mismatch
from trace_gb300 import pt, scenes

pytestmark = pytest.mark.gpu

CASES = [
    ("cornell_a0.5_d6_bf2", lambda: scenes.cornell()["verts"], 0.5, 6.0, 2),
    ("cornell_a0.55_d9_bf4", lambda: scenes.cornell()["verts"], 0.55, 9.0, 4),
    ("soup2k_bf3", lambda: scenes.soup(2000, seed=2000)["verts"], 0.5, 3.0, 3),
    ("soup50k_bf2", lambda: scenes.soup(50_000, seed=5)["verts"], 0.5, 6.0, 2),
    ("soup50k_hq_bf2", lambda: scenes.soup(50_000, seed=5)["verts"], 0.55, 9.0, 2),
    ("soup50k_bf4", lambda: scenes.soup(50_000, seed=5)["verts"], 0.5, 6.0, 4),
    ("terrain129_bf2", lambda: scenes.terrain_tris(129, seed=2), 0.5, 6.0, 2),
    ("dups_bf2", lambda: np.concatenate([scenes.soup(3000, seed=7)["verts"]] * 2), 0.5, 6.0, 2),
    ("one_point", lambda: np.tile(np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0]], np.float32), (64, 1)), 0.5, 6.0, 2),
]


@pytest.mark.parametrize("name,make,alpha,delta,bf", CASES, ids=[c[0] for c in CASES])
def test_phr_matches_oracle_tree(ctx, name, make, alpha, delta, bf):
    verts = np.ascontiguousarray(make(), np.float32)
    ds = pt.DeviceScene(ctx, verts)
    aux = pt.DefaultLBVH(ds)
    g = pt.NewPHRBuilder(alpha, delta, bf).BuildFromAuxilary(aux)
    o = O.lbvh(verts).phr(alpha, delta, bf)
    ge, oe = g.export(), o.export()
    assert canonical_equal(ge, oe), first_mismatch(ge, oe)
    oc = o.cost()
    assert abs(g.Cost() - oc) <= 0.01 * oc  # the stated bar; the trees are identical so it is ~1e-12
    assert g.Cost() == oc  # the device evaluates the recursion's float64 operations in its order


@pytest.mark.parametrize("small_cut", [4, 16, 64])
def test_phr_level_batches_and_relaunches_give_the_same_tree(ctx, small_cut):
    """With a low threshold for one-warp levels, batched launches meet levels
    with larger cuts, flag a stall and are relaunched with wider blocks; the
    tree stays the oracle's (branching 2 and 4)."""
    verts = scenes.soup(50_000, seed=5)["verts"]
    aux = pt.DefaultLBVH(pt.DeviceScene(ctx, verts))
    try:
        ctx.set_option("phr_small_cut", small_cut)
        for bf in (2, 4):
            g = pt.NewPHRBuilder(0.5, 6.0, bf).BuildFromAuxilary(aux)
            ge, oe = g.export(), O.lbvh(verts).phr(0.5, 6.0, bf).export()
            assert canonical_equal(ge, oe), first_mismatch(ge, oe)
    finally:
        ctx.set_option("phr_small_cut", 256)


def test_phr_workspace_kept_or_released_gives_the_same_tree(ctx):
    """Refinements that reuse the context's workspace (default), grow it, and
    free it after every build (GBT_OPT_KEEP_WORKSPACE 0) give the same tree."""
    big = scenes.soup(50_000, seed=5)["verts"]
    small = scenes.soup(3000, seed=7)["verts"]
    aux_big = pt.DefaultLBVH(pt.DeviceScene(ctx, big))
    aux_small = pt.DefaultLBVH(pt.DeviceScene(ctx, small))
    ref_small = O.lbvh(small).phr(0.5, 6.0, 2).export()
    ref_big = O.lbvh(big).phr(0.5, 6.0, 2).export()
    try:
        for keep in (1, 0):
            ctx.set_option("keep_workspace", keep)
            for aux, ref in ((aux_small, ref_small), (aux_big, ref_big), (aux_small, ref_small)):
                g = pt.NewPHRBuilder(0.5, 6.0, 2).BuildFromAuxilary(aux)
                ge = g.export()
                assert canonical_equal(ge, ref), first_mismatch(ge, ref)
    finally:
        ctx.set_option("keep_workspace", 1)


@pytest.mark.parametrize("coord", [1e-12, 3e9])
def test_phr_outside_the_screening_range_matches_oracle(ctx, coord):
    """A box coordinate outside [2^-30, 2^30] in magnitude (other than 0) turns
    the float32 screening off for the whole refinement, which then decides every
    comparison in float64: the tree is still the oracle's."""
    verts = np.array(scenes.soup(3000, seed=11)["verts"], np.float32)
    verts[0, 0] = coord
    aux = pt.DefaultLBVH(pt.DeviceScene(ctx, verts))
    g = pt.NewPHRBuilder(0.5, 6.0, 2).BuildFromAuxilary(aux)
    o = O.lbvh(verts).phr(0.5, 6.0, 2)
    ge, oe = g.export(), o.export()
    assert canonical_equal(ge, oe), first_mismatch(ge, oe)
    assert g.Cost() == o.cost()


def test_reused_tree_blocks_give_the_same_tree_and_hits(ctx):
    """A destroyed tree's device blocks (its arrays and its 4-wide view) stay on
    the context for the next trees: a tree built into the blocks of a larger
    one, with that tree's contents still in them, exports the oracle's tree and
    gives the same hits as the same tree built into fresh blocks."""
    small_s = scenes.soup(30_000, seed=9)
    small, big = small_s["verts"], scenes.soup(50_000, seed=5)["verts"]
    aux_small = pt.DefaultLBVH(pt.DeviceScene(ctx, small))
    aux_big = pt.DefaultLBVH(pt.DeviceScene(ctx, big))
    rays = scenes.camera_rays(small_s["camera"], 96, 64, jitter_seed=3)
    ref = O.lbvh(small).phr(0.5, 6.0, 2).export()
    fresh = pt.NewPHRBuilder(0.5, 6.0, 2).BuildFromAuxilary(aux_small)  # kept: its blocks stay in use
    want = fresh.trace(rays)
    other = pt.NewPHRBuilder(0.5, 6.0, 2).BuildFromAuxilary(aux_big)
    other.trace(rays)
    other.close()  # its blocks go to the context's cache, the only ones there of these sizes
    g = pt.NewPHRBuilder(0.5, 6.0, 2).BuildFromAuxilary(aux_small)
    ge = g.export()
    assert canonical_equal(ge, ref), first_mismatch(ge, ref)
    got = g.trace(rays)
    for a, b in zip(got, want):
        assert np.array_equal(a, b)
    fresh.close()


@pytest.mark.parametrize("alpha,delta,bf", [(0.5, 6.0, 2), (0.55, 9.0, 2), (0.5, 6.0, 4)])
def test_phr_1m_soup(ctx, alpha, delta, bf):
    s = scenes.soup(1_000_000, seed=1)
    ds = pt.DeviceScene.from_dict(ctx, s)
    aux = pt.DefaultLBVH(ds)
    g = pt.NewPHRBuilder(alpha, delta, bf).BuildFromAuxilary(aux)
    o = O.lbvh(s["verts"]).phr(alpha, delta, bf)
    ge, oe = g.export(), o.export()
    assert canonical_equal(ge, oe), first_mismatch(ge, oe)
    # the same closest hits on a fixed ray set
    rays = scenes.camera_rays(s["camera"], 480, 270, jitter_seed=5)
    gp, gt, _, _ = g.trace(rays)
    op, ot, _, _ = o.trace(rays)
    near, hard = classify_disagreements(o, rays, gp, gt, op, ot)
    print("phr 1M a=%g d=%g bf=%d cost %.4f agree %.6f near %d hard %d" % (
        alpha, delta, bf, o.cost(), (gp == op).mean(), len(near), len(hard)))
    assert len(hard) == 0
    assert (gp == op).mean() >= 0.9999 or len(near) <= 1e-4 * len(rays) + 2


def oracle_grid(verts, spheres, alphas, deltas, bf, pixels):
    """optimizer.go:44-94 (OptimizedPHRparams, omega, evalPHR) over oracle PHR builds."""
    o = O.lbvh(verts, spheres)
    evs = []
    for a in alphas:
        for d in deltas:
            ph = o.phr(a, d, bf)
            evs.append((ph.cost(), ph.stats["build_cost"], a, d))
    max_b = max(e[1] for e in evs)
    max_s = max(e[0] for e in evs)
    n = verts.shape[0] + (0 if spheres is None else spheres.shape[0])
    q = n / 2e6
    om = (q * q) * (pixels / 2e5)
    best, pick = float("inf"), None
    for e in evs:
        c = e[1] / max_b + (om * om) * (e[0] / max_s)
        if c < best:
            best, pick = c, (e[2], e[3])
    return pick, evs


GRID_CASES = [
    ("soup20k_default_grid", lambda: (scenes.soup(20_000, seed=11)["verts"], None), None, None, 2, (1920, 1080)),
    ("soup5k_bf4", lambda: (scenes.soup(5000, seed=12)["verts"], None), [0.4, 0.5], [3, 6, 9], 4, (640, 480)),
    ("terrain129_sun_deep_grid", lambda: (scenes.terrain(129)["verts"], scenes.terrain(129)["spheres"]),
     [0.4, 0.55], [6, 8, 10, 12], 2, (1920, 1080)),
    # omega large enough for the SAH term to decide
    ("terrain257_large_frame", lambda: (scenes.terrain_tris(257, seed=2), None), [0.45, 0.55], [6, 9], 2,
     (40000, 40000)),
]


@pytest.mark.parametrize("name,make,alphas,deltas,bf,frame", GRID_CASES, ids=[c[0] for c in GRID_CASES])
def test_grid_optimizer_matches_oracle(ctx, name, make, alphas, deltas, bf, frame):
    verts, spheres = make()
    verts = np.ascontiguousarray(verts, np.float32)
    ds = pt.DeviceScene(ctx, verts, spheres=spheres)
    aux = pt.DefaultLBVH(ds)
    opt = pt.NewDefaultGridOptimizer(*frame) if alphas is None else pt.NewGridOptimizer(alphas, deltas, *frame)
    got = opt.OptimizedPHRparams(aux, bf)
    want, evs = oracle_grid(verts, spheres, opt.Alphas, opt.Deltas, bf, frame[0] * frame[1])
    for (a, d, sah, build), (osah, obuild, oa, od) in zip(opt.evaluations, evs):
        assert (a, d) == (oa, od)
        assert build == obuild, (a, d, build, obuild)
        assert sah == pytest.approx(osah, rel=1e-12), (a, d)
    assert got == want, (got, want, opt.evaluations)
    # BuildWithCost on the chosen parameters reports the same build cost
    tree, cost = pt.NewPHRBuilder(got[0], got[1], bf).BuildWithCost(aux)
    k = [(e[0], e[1]) for e in opt.evaluations].index(got)
    assert cost == opt.evaluations[k][3] and tree.Cost() == pytest.approx(opt.evaluations[k][2], rel=1e-12)


@pytest.mark.parametrize("alpha,delta,bf", [(0.5, 9.0, 3), (0.55, 9.0, 4), (0.5, 12.0, 3)])
def test_phr_terrain_with_sun_matches_oracle(ctx, alpha, delta, bf):
    """Branching 3 and 4 split refined cuts of a job again inside the same block: those cuts
    can be up to 2^(bf-2) times the job's own cut, which the per-block scratch must hold."""
    s = scenes.terrain(129)
    ds = pt.DeviceScene.from_dict(ctx, s)
    g = pt.NewPHRBuilder(alpha, delta, bf).BuildFromAuxilary(pt.DefaultLBVH(ds))
    o = O.lbvh(s["verts"], s["spheres"]).phr(alpha, delta, bf)
    ge, oe = g.export(), o.export()
    assert canonical_equal(ge, oe), first_mismatch(ge, oe)
    assert g.Cost() == o.cost()  # the same float64 operations in the same order
