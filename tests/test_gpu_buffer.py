"""Render targets of pkg/pt/buffer.go on the device: PixelBuffer's running mean
across RenderToBuffer calls (buffer.go:19-26), FrameBuffer's last write
(buffer.go:91-93) and ToImage (buffer.go:60-69 with math.go:20-25)."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from tests.test_gpu_render import MEAN_REL, RMSE_RATIO, rmse
from trace_gb300 import _lib, pt, scenes

pytestmark = pytest.mark.gpu

GOLDEN = 0x9E3779B97F4A7C15  # seed step between calls on one buffer


def _renderer(ctx, s, spp, seed=5):
    g = pt.DefaultLBVH(pt.DeviceScene.from_dict(ctx, s))
    cam = s["camera"]
    r = pt.ImageRenderer(g, pt.NewCamera(cam["aspect"], cam["fov"], pt.CameraTransformation(
        cam["look_from"], cam["look_at"], cam["up"])), MaxDepth=s["render"]["max_depth"], Spp=spp,
        Miss=s["render"]["miss_mode"], MissColor=s["render"]["miss_color"], Seed=seed)
    return g, r


def test_pixel_buffer_accumulates_across_calls(ctx):
    """Two RenderToBuffer calls of S samples into one PixelBuffer hold the mean of 2S
    samples: the first call equals gbt_render's image, the second adds new samples, and
    the result matches the oracle at 2S spp as closely as the oracle's own image does.
    The frame is large enough (128x128) for the per-channel RMSE, which the light's few
    bright samples dominate, to be a stable estimate."""
    w = h = 128
    S = 16
    s = scenes.cornell(width=w, height=h)
    g, r = _renderer(ctx, s, S)
    buf = pt.NewPxlBuffer(w, h)
    r.RenderToBuffer(buf)
    first = buf.data.copy()
    assert buf.samples == S
    one, _ = g.render(s["camera"], w, h, S, s["render"]["max_depth"], seed=5)
    # the same paths; the per-pixel sums of S deposits are taken in atomic order
    np.testing.assert_allclose(first, one, rtol=1e-5, atol=1e-6)
    r.RenderToBuffer(buf)
    assert buf.samples == 2 * S
    assert not np.array_equal(buf.data, first)
    o = O.lbvh(s["verts"])
    conv = o.render(s, width=w, height=h, spp=512, seed=11)
    orc = o.render(s, width=w, height=h, spp=2 * S, seed=12)
    r_b, r_o, r_1 = rmse(buf.data, conv), rmse(orc, conv), rmse(first, conv)
    print("pixel buffer rmse after 2 calls", r_b, "oracle at 2S", r_o, "after 1 call", r_1)
    assert np.all(r_b <= RMSE_RATIO * r_o + 1e-6)
    assert np.all(r_b < r_1)  # twice the samples: lower error than one call
    m_b, m_c = buf.data.mean(axis=(0, 1)), conv.mean(axis=(0, 1))
    assert np.all(np.abs(m_b - m_c) <= 5 * MEAN_REL * np.maximum(m_c, 1e-3))
    buf.close()


def test_pixel_buffer_mean_weights(ctx):
    """Blending is weighted by sample counts: 2 calls of 4 spp then 1 call of 8 spp equal the
    mean of the three images with weights 4, 4, 8 (float32 rounding and atomic summation
    order apart)."""
    w = h = 32
    s = scenes.cornell(width=w, height=h)
    g = pt.DefaultLBVH(pt.DeviceScene.from_dict(ctx, s))
    buf = pt.NewPxlBuffer(w, h, ctx)
    imgs = []
    for k, spp in enumerate((4, 4, 8)):
        p = _lib.RenderParams(w, h, spp, 5, 0, (C.c_float * 3)(0, 0, 0), 3)
        cam = pt.make_camera(s["camera"])
        buf._render(g, cam, p)
        one, _ = g.render(s["camera"], w, h, spp, 5, seed=(3 + k * GOLDEN) % (1 << 64))
        imgs.append(one.astype(np.float64))
    want = (4 * imgs[0] + 4 * imgs[1] + 8 * imgs[2]) / 16
    assert buf.samples == 16
    np.testing.assert_allclose(buf.data, want, rtol=1e-5, atol=1e-5)
    buf.close()


def test_frame_buffer_keeps_the_last_sample(ctx):
    """A FrameBuffer holds one sample per pixel, from the last call: the image of the
    second call's seed at 1 spp, whatever the call's spp (one deposit per pixel, so
    bitwise equal)."""
    w = h = 48
    s = scenes.cornell(width=w, height=h)
    g, r = _renderer(ctx, s, 16, seed=9)
    fb = pt.NewFrameBuffer(w, h)
    r.RenderToBuffer(fb)
    r.RenderToBuffer(fb)
    assert fb.samples == 1
    last, _ = g.render(s["camera"], w, h, 1, s["render"]["max_depth"], seed=(9 + GOLDEN) % (1 << 64))
    assert np.array_equal(fb.data, last)
    first, _ = g.render(s["camera"], w, h, 1, s["render"]["max_depth"], seed=9)
    assert not np.array_equal(fb.data, first)
    fb.close()


@pytest.mark.parametrize("kind", ["pixel", "frame"])
def test_to_image_bit_exact(ctx, kind):
    """ToImage bytes equal the oracle's restatement, on a rendered image and on a buffer
    holding edge values (exact squares of k/255 and their float32 neighbours, negatives,
    values above 1, NaN, inf) added through gbt_buffer_add_async."""
    w, h = 40, 30
    s = scenes.cornell(width=w, height=h)
    g, r = _renderer(ctx, s, 4)
    b = pt.NewPxlBuffer(w, h) if kind == "pixel" else pt.NewFrameBuffer(w, h)
    r.RenderToBuffer(b)
    got = b.ToImage()
    assert got.shape == (h, w, 4) and got.dtype == np.uint8
    assert np.array_equal(got, O.to_image(b.data))
    assert np.all(got[0] == 0) and np.all(got[1:, :, 3] == 255)
    k = np.arange(256, dtype=np.float64) / 255.0
    sq = (k * k).astype(np.float32)
    edge = np.concatenate([sq, np.nextafter(sq, np.float32(-1)), np.nextafter(sq, np.float32(2)),
                           np.array([np.nan, np.inf, -np.inf, -0.0, -1.0, 1.0, 3.0], np.float32)])
    img = np.resize(edge, h * w * 3).reshape(h, w, 3).astype(np.float32)
    fb = pt.NewFrameBuffer(w, h, ctx)
    d = ctx.alloc(img.nbytes)
    try:
        ctx.h2d(d, img)
        ctx.check(ctx.L.gbt_buffer_add_async(ctx.h, fb.h, C.c_void_p(d), 1), "buffer_add")
        ctx.sync()
    finally:
        ctx.free(d)
    got = fb.ToImage()
    assert np.array_equal(got, O.to_image(img))
    b.close()
    fb.close()


def test_buffer_rejects_a_frame_of_another_size(ctx):
    s = scenes.cornell(width=32, height=32)
    g, r = _renderer(ctx, s, 1)
    b = pt.NewPxlBuffer(32, 16)
    r.RenderToBuffer(b)  # the renderer takes the buffer's size
    assert b.samples == 1
    cam = pt.make_camera(s["camera"])
    p = _lib.RenderParams(32, 32, 1, 5, 0, (C.c_float * 3)(0, 0, 0), 1)
    with pytest.raises(_lib.GbtError):
        b._render(g, cam, p)
    b.close()
