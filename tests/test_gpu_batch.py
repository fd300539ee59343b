"""Batched persistent rendering vs the per-scene wavefront loop.

Both trace the same paths (same Philox counters per scene), so the images
agree up to the order of float additions into the accumulators; the batched
form must therefore have the same image RMSE against a converged image.
"""
import numpy as np
import pytest

from trace_gb300 import pt, scenes

pytestmark = pytest.mark.gpu


def make_batch(ctx, count=6, lo=1_000, hi=60_000, w=96, h=64, spp=4, depth=3):
    ss = scenes.batch(count=count, lo=lo, hi=hi, seed=3, width=w, height=h, spp=spp, max_depth=depth)
    bvhs, cams, params = [], [], []
    for k, s in enumerate(ss):
        ds = pt.DeviceScene.from_dict(ctx, s)
        bvhs.append(pt.DefaultLBVH(ds))
        cams.append(s["camera"])
        p = dict(s["render"])
        p["seed"] = 100 + k
        params.append(p)
    return ss, pt.Batch(ctx, bvhs, cams, params)


def test_batched_equals_plain(ctx):
    ss, b = make_batch(ctx)
    try:
        b.render("plain")
        plain = [b.read(i) for i in range(b.n)]
        b.render("batched")
        batched = [b.read(i) for i in range(b.n)]
        for p, q in zip(plain, batched):
            assert np.all(np.isfinite(q))
            np.testing.assert_allclose(q, p, rtol=1e-4, atol=1e-5)
        # the autotuner returns one of the supported configurations and it renders the same
        cfg, ms = b.autotune()
        assert cfg.block in (64, 128, 256) and cfg.fetch_min in (0, 16) and cfg.stack in (0, 1) and ms > 0
        b.render("batched", cfg)
        for i, p in enumerate(plain):
            np.testing.assert_allclose(b.read(i), p, rtol=1e-4, atol=1e-5)
    finally:
        b.close()


def test_batch_graph_with_rebuild(ctx):
    ss, b = make_batch(ctx, count=4)
    try:
        b.make_graph(rebuild=True)
        b.render("graph")
        g1 = [b.read(i) for i in range(b.n)]
        b.render("graph")  # a replay rebuilds and renders again: same result
        g2 = [b.read(i) for i in range(b.n)]
        b.render("plain")
        plain = [b.read(i) for i in range(b.n)]
        for x, y, p in zip(g1, g2, plain):
            np.testing.assert_allclose(x, y, rtol=1e-4, atol=1e-5)
            np.testing.assert_allclose(x, p, rtol=1e-4, atol=1e-5)
    finally:
        b.close()
