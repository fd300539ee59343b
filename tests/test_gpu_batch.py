"""Batched persistent rendering vs the per-scene wavefront loop.

Both trace the same paths (same Philox counters per scene), so the images
agree up to the order of float additions into the accumulators; the batched
form must therefore have the same image RMSE against a converged image.
"""
import numpy as np
import pytest

from trace_gb300 import _lib, pt, scenes

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


MEGA = _lib.BatchConfig(128, 16, 0, _lib.BATCH_MEGAKERNEL, 0)
WAVE = _lib.BatchConfig(128, 16, 0, _lib.BATCH_WAVEFRONT, 0)
WAVE_PACKETS = _lib.BatchConfig(128, 16, 0, _lib.BATCH_WAVEFRONT, 1)


@pytest.mark.parametrize("cfg", [None, MEGA, WAVE, WAVE_PACKETS, _lib.BatchConfig(256, 0, 1, _lib.BATCH_MEGAKERNEL, 0)],
                         ids=["default", "megakernel", "wavefront", "wavefront_packets", "megakernel_b256_shared"])
def test_batched_equals_plain(ctx, cfg):
    ss, b = make_batch(ctx)
    try:
        b.render("plain")
        plain = [b.read(i) for i in range(b.n)]
        b.render("batched", cfg)
        batched = [b.read(i) for i in range(b.n)]
        for p, q in zip(plain, batched):
            assert np.all(np.isfinite(q))
            np.testing.assert_allclose(q, p, rtol=1e-4, atol=1e-5)
    finally:
        b.close()


def test_autotune_choice_renders_the_same(ctx):
    ss, b = make_batch(ctx)
    try:
        b.render("plain")
        plain = [b.read(i) for i in range(b.n)]
        cfg, ms = b.autotune()
        assert ms > 0 and cfg.mode in (_lib.BATCH_MEGAKERNEL, _lib.BATCH_WAVEFRONT)
        if cfg.mode == _lib.BATCH_MEGAKERNEL:
            assert cfg.block in (64, 128, 256) and cfg.fetch_min in (0, 16) and cfg.stack in (0, 1)
        b.render("batched", cfg)
        for i, p in enumerate(plain):
            np.testing.assert_allclose(b.read(i), p, rtol=1e-4, atol=1e-5)
        b.render("batched")  # the tuned choice is now the context's default
        for i, p in enumerate(plain):
            np.testing.assert_allclose(b.read(i), p, rtol=1e-4, atol=1e-5)
    finally:
        b.close()


def test_mixed_depths_and_sizes(ctx):
    """Items of different depth, size and spp in one frame: the wavefront runs the deepest
    item's levels, and shallower items' paths end at their own depth."""
    ss = scenes.batch(count=3, lo=2_000, hi=20_000, seed=5, width=64, height=48, spp=2, max_depth=1)
    bvhs, cams, params = [], [], []
    for k, s in enumerate(ss):
        bvhs.append(pt.DefaultLBVH(pt.DeviceScene.from_dict(ctx, s)))
        cams.append(s["camera"])
        p = dict(s["render"])
        p.update(seed=7 + k, max_depth=[0, 5, 2][k], width=[64, 40, 33][k], height=[48, 30, 17][k], spp=[2, 3, 1][k])
        params.append(p)
    b = pt.Batch(ctx, bvhs, cams, params)
    try:
        b.render("plain")
        plain = [b.read(i) for i in range(b.n)]
        for cfg in (WAVE, WAVE_PACKETS, MEGA):
            b.render("batched", cfg)
            for i, p in enumerate(plain):
                np.testing.assert_allclose(b.read(i), p, rtol=1e-4, atol=1e-5)
    finally:
        b.close()


def test_bad_config_is_rejected(ctx):
    ss, b = make_batch(ctx, count=2)
    try:
        with pytest.raises(pt.GbtError):
            b.render("batched", _lib.BatchConfig(96, 16, 0, _lib.BATCH_MEGAKERNEL))
        with pytest.raises(pt.GbtError):
            b.render("batched", _lib.BatchConfig(128, 16, 0, 7, 0))
        with pytest.raises(pt.GbtError):
            b.render("batched", _lib.BatchConfig(128, 16, 0, _lib.BATCH_WAVEFRONT, 2))
    finally:
        b.close()


@pytest.mark.parametrize("cfg", [WAVE, WAVE_PACKETS, MEGA], ids=["wavefront", "wavefront_packets", "megakernel"])
def test_batch_graph_with_rebuild(ctx, cfg):
    ss, b = make_batch(ctx, count=4)
    try:
        b.make_graph(rebuild=True, cfg=cfg)
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


def test_graph_owns_its_buffers(ctx):
    """A plain render after graph creation reuses and may regrow the context's path buffers;
    the graph's replays must not be affected."""
    ss, b = make_batch(ctx, count=2)
    try:
        b.make_graph(rebuild=False, cfg=WAVE_PACKETS)
        b.render("graph")
        g1 = [b.read(i) for i in range(b.n)]
        s = scenes.batch(count=1, lo=2_000, hi=2_001, seed=9, width=256, height=256, spp=8, max_depth=2)[0]
        big = pt.DefaultLBVH(pt.DeviceScene.from_dict(ctx, s))
        big.render(s["camera"], 256, 256, 8, 2)
        b.render("graph")
        g2 = [b.read(i) for i in range(b.n)]
        for x, y in zip(g1, g2):
            np.testing.assert_allclose(x, y, rtol=1e-4, atol=1e-5)
    finally:
        b.close()


def test_packet_and_single_ray_items_in_one_wave(ctx):
    """Items whose trees take camera rays as packets lead the queue; a wave splits into a
    packet range and a one-ray-per-lane range (here inside the first of two waves)."""
    ss = scenes.batch(count=3, lo=2_000, hi=8_000, seed=6, width=1024, height=1024, spp=3, max_depth=2)
    bvhs, cams, params = [], [], []
    for k, s in enumerate(ss):
        g = pt.DefaultLBVH(pt.DeviceScene.from_dict(ctx, s))
        g.set_packets([2, 1, 1][k])  # the single-ray item first in the caller's order
        bvhs.append(g)
        cams.append(s["camera"])
        p = dict(s["render"])
        p["seed"] = 40 + k
        params.append(p)
    b = pt.Batch(ctx, bvhs, cams, params)
    try:
        assert b.paths > (1 << 23)  # two waves
        b.render("plain")
        plain = [b.read(i) for i in range(b.n)]
        b.render("batched", WAVE_PACKETS)
        for i, p in enumerate(plain):
            np.testing.assert_allclose(b.read(i), p, rtol=1e-4, atol=1e-5)
        b.make_graph(cfg=WAVE_PACKETS)
        b.render("graph")
        for i, p in enumerate(plain):
            np.testing.assert_allclose(b.read(i), p, rtol=1e-4, atol=1e-5)
    finally:
        b.close()


def test_forced_packets_option(ctx):
    """GBT_OPT_PRIMARY_PACKETS 1 takes every item's camera rays as packets, 0 none; the
    images are the same."""
    ss, b = make_batch(ctx, count=3)
    try:
        b.render("plain")
        plain = [b.read(i) for i in range(b.n)]
        for opt in (1, 0):
            ctx.set_option("primary_packets", opt)
            b.render("batched", WAVE_PACKETS)
            for i, p in enumerate(plain):
                np.testing.assert_allclose(b.read(i), p, rtol=1e-4, atol=1e-5)
    finally:
        ctx.set_option("primary_packets", 2)
        b.close()


@pytest.mark.parametrize("layout", [4, 2])
def test_graph_rebuild_follows_moved_vertices(ctx, layout):
    """A graph with rebuilds renders the scenes as they are at replay: after the vertices move
    (gbt_scene_update_async), one replay gives the images of freshly built trees.  In the
    4-wide layout the replay also collapses each rebuilt tree (a conditional graph node)."""
    ss = scenes.batch(count=3, lo=3_000, hi=30_000, seed=8, width=96, height=64, spp=4, max_depth=3)
    dss, bvhs, cams, params = [], [], [], []
    for k, s in enumerate(ss):
        ds = pt.DeviceScene.from_dict(ctx, s)
        g = pt.DefaultLBVH(ds)
        g.set_layout(layout)
        dss.append(ds)
        bvhs.append(g)
        cams.append(s["camera"])
        p = dict(s["render"])
        p["seed"] = 60 + k
        params.append(p)
    b = pt.Batch(ctx, bvhs, cams, params)
    bufs = []
    try:
        b.make_graph(rebuild=True, cfg=WAVE)
        b.render("graph")
        before = [b.read(i) for i in range(b.n)]
        rng = np.random.default_rng(1)
        moved = []
        for ds, s in zip(dss, ss):
            v = (s["verts"] + rng.normal(0, 0.01, s["verts"].shape)).astype(np.float32)
            d = ctx.alloc(v.nbytes)
            ctx.h2d(d, v)
            bufs.append(d)
            ctx.check(ctx.L.gbt_scene_update_async(ctx.h, ds.h, d), "scene_update")
            moved.append(v)
        b.render("graph")
        after = [b.read(i) for i in range(b.n)]
        assert any(np.max(np.abs(x - y)) > 1e-3 for x, y in zip(before, after))
        # fresh trees over the moved vertices, rendered one by one
        for i, (s, v) in enumerate(zip(ss, moved)):
            s2 = dict(s)
            s2["verts"] = v
            g = pt.DefaultLBVH(pt.DeviceScene.from_dict(ctx, s2))
            g.set_layout(layout)
            p = params[i]
            img, _ = g.render(s["camera"], p["width"], p["height"], p["spp"], p["max_depth"], p["miss_mode"],
                              p.get("miss_color", (0, 0, 0)), p["seed"])
            np.testing.assert_allclose(after[i], img, rtol=1e-4, atol=1e-5)
    finally:
        b.close()
        for d in bufs:
            ctx.free(d)
