"""GPU wavefront path tracer vs the oracle's path tracer (statistical parity).

Both sides sample with their own random numbers (the reference seeds from the
clock), so images are compared through their error against a converged
oracle image: at equal spp the GPU image's per-channel RMSE must be within
RMSE_RATIO of the oracle's own, and the converged means must agree.
"""
import numpy as np
import pytest

from oracle import oracle as O
from trace_gb300 import pt, scenes

pytestmark = pytest.mark.gpu

RMSE_RATIO = 1.15   # GPU RMSE / oracle RMSE at equal spp, per channel
MEAN_REL = 0.01     # relative difference of the image means at high spp
BLOCK_REL = 0.03    # relative RMSE of 8x8 block means at high spp


def rmse(a, b):
    return np.sqrt(np.mean((a - b) ** 2, axis=(0, 1)))


def blocks(img, k=8):
    h, w, _ = img.shape
    return img[: h // k * k, : w // k * k].reshape(h // k, k, w // k, k, 3).mean(axis=(1, 3))


def run(ctx, s, w, h, spp_eq, spp_conv, spp_hi, max_depth=None):
    rd = s["render"]
    md = rd["max_depth"] if max_depth is None else max_depth
    cam = dict(s["camera"], aspect=w / h)
    s2 = dict(s, camera=cam)
    o = O.lbvh(s["verts"], s.get("spheres"))
    conv = o.render(s2, width=w, height=h, spp=spp_conv, max_depth=md, seed=101)
    orc = o.render(s2, width=w, height=h, spp=spp_eq, max_depth=md, seed=202)
    ds = pt.DeviceScene.from_dict(ctx, s)
    g = pt.DefaultLBVH(ds)
    gpu, st = g.render(cam, w, h, spp_eq, md, rd["miss_mode"], rd["miss_color"], seed=303)
    gpu_hi, st_hi = g.render(cam, w, h, spp_hi, md, rd["miss_mode"], rd["miss_color"], seed=404)
    r_g, r_o = rmse(gpu, conv), rmse(orc, conv)
    print("rmse gpu", r_g, "oracle", r_o, "means", gpu_hi.mean(axis=(0, 1)), conv.mean(axis=(0, 1)),
          "rays", st["rays_traced"])
    assert np.all(r_g <= RMSE_RATIO * r_o + 1e-6), (r_g, r_o)
    m_g, m_c = gpu_hi.mean(axis=(0, 1)), conv.mean(axis=(0, 1))
    assert np.all(np.abs(m_g - m_c) <= MEAN_REL * np.maximum(m_c, 1e-3)), (m_g, m_c)
    bg, bc = blocks(gpu_hi), blocks(conv)
    brel = np.sqrt(np.mean((bg - bc) ** 2)) / max(bc.mean(), 1e-3)
    assert brel <= BLOCK_REL, brel
    return st


def test_render_cornell(ctx):
    st = run(ctx, scenes.cornell(), 96, 96, spp_eq=16, spp_conv=512, spp_hi=1024)
    assert st["rays_traced"] >= 96 * 96 * 16


def test_render_soup_primary_plus_bounce(ctx):
    s = scenes.soup(200_000, seed=1)
    st = run(ctx, s, 160, 90, spp_eq=4, spp_conv=256, spp_hi=512)
    # MaxDepth 0: one primary ray per path plus one bounce per primary hit
    assert 160 * 90 * 4 <= st["rays_traced"] <= 2 * 160 * 90 * 4


def test_render_terrain_sun_constant_sky(ctx):
    s = scenes.terrain(g=129)
    run(ctx, s, 96, 54, spp_eq=16, spp_conv=512, spp_hi=1024)


def test_render_emitter_exact(ctx):
    """Looking straight at a Light quad with MaxDepth 0 gives exactly its colour."""
    quad = np.array([[-1, -1, 0, 1, -1, 0, 1, 1, 0], [-1, -1, 0, 1, 1, 0, -1, 1, 0]], np.float32)
    ds = pt.DeviceScene(ctx, quad, prim_mat=np.array([0, 0]), mat_type=[1], mat_color=[[10.0, 10.0, 10.0]])
    g = pt.DefaultLBVH(ds)
    cam = dict(look_from=(0, 0, 2), look_at=(0, 0, 0), up=(0, 1, 0), fov=20.0, aspect=1.0)
    img, st = g.render(cam, 8, 8, 2, 0)
    np.testing.assert_allclose(img, 10.0)


@pytest.mark.parametrize("kind", ["cornell", "soup"])
def test_execution_options_leave_images_identical(ctx, kind):
    """Any-hit past MaxDepth, tiled camera rays, packet tracing and the traversal kernel change the
    order of work only: with spp 2 (two deposits per pixel add commutatively) the
    images and ray counts are bitwise equal under every setting.  The frame size is
    no multiple of the 8x4 tile, so the right and bottom strips are covered too."""
    s = scenes.cornell() if kind == "cornell" else scenes.soup(100_000, seed=3)
    rd = s["render"]
    w, h, spp, md = 83, 61, 2, (3 if kind == "cornell" else 0)
    cam = dict(s["camera"], aspect=w / h)
    g = pt.DefaultLBVH(pt.DeviceScene.from_dict(ctx, s))
    ref = None
    try:
        for trav in (0, 1, 2):
            for anyhit in (0, 1):
                for tiles, packets in ((0, 0), (1, 0), (1, 1), (1, 2)):
                    ctx.set_option("traversal", trav)
                    ctx.set_option("anyhit_last", anyhit)
                    ctx.set_option("primary_tiles", tiles)
                    ctx.set_option("primary_packets", packets)
                    img, st = g.render(cam, w, h, spp, md, rd["miss_mode"], rd["miss_color"], seed=5)
                    if ref is None:
                        ref = (img, st["rays_traced"])
                        assert img.mean() > 0
                    else:
                        assert st["rays_traced"] == ref[1], (trav, anyhit, tiles, packets)
                        assert np.array_equal(img, ref[0]), (trav, anyhit, tiles, packets, np.abs(img - ref[0]).max())
    finally:
        ctx.set_option("traversal", 0)
        ctx.set_option("anyhit_last", 1)
        ctx.set_option("primary_tiles", 1)
        ctx.set_option("primary_packets", 2)


def test_render_cornell_reflective_refractive(ctx):
    """Glass UV sphere (Refractive, triangles) and a brushed-metal sphere primitive
    (Reflective): statistical parity with the oracle's renderer."""
    # caustics through the glass are noisy: more samples for the converged and high-spp images
    run(ctx, scenes.cornell_materials(), 96, 96, spp_eq=16, spp_conv=2048, spp_hi=2048)


@pytest.mark.parametrize("kind", ["mirror", "glass"])
def test_render_reflective_and_refractive_exact(ctx, kind):
    from tests.helpers import clear_glass_scene, mirror_scene

    s = mirror_scene() if kind == "mirror" else clear_glass_scene()
    g = pt.DefaultLBVH(pt.DeviceScene.from_dict(ctx, s))
    img, st = g.render(s["camera"], 16, 16, 4, 3)
    a, le = np.asarray(s["mat_color"][0]), s["mat_color"][1][0]
    want = a * le if kind == "mirror" else a * a * le
    np.testing.assert_allclose(img.reshape(-1, 3), np.broadcast_to(want, (256, 3)), rtol=1e-5)
    # mirror: camera ray + reflected ray; glass: camera ray + two refracted rays
    assert st["rays_traced"] == 16 * 16 * 4 * (2 if kind == "mirror" else 3)


def test_measured_packet_choice_keeps_the_image(ctx):
    """GBT_OPT_PRIMARY_PACKETS = 2: the first render on a tree traces its camera rays with both
    kernels and keeps the faster; the image equals the one without packets, then and after."""
    s = scenes.cornell()
    rd = s["render"]
    cam = dict(s["camera"], aspect=1.0)
    g = pt.DefaultLBVH(pt.DeviceScene.from_dict(ctx, s))
    try:
        ctx.set_option("primary_packets", 0)
        ref, st0 = g.render(cam, 256, 256, 1, 3, rd["miss_mode"], rd["miss_color"], seed=9)
        ctx.set_option("primary_packets", 2)
        first, st1 = g.render(cam, 256, 256, 1, 3, rd["miss_mode"], rd["miss_color"], seed=9)  # measures
        again, st2 = g.render(cam, 256, 256, 1, 3, rd["miss_mode"], rd["miss_color"], seed=9)  # uses the choice
        assert np.array_equal(first, ref) and np.array_equal(again, ref)
        assert st0["rays_traced"] == st1["rays_traced"] == st2["rays_traced"]
    finally:
        ctx.set_option("primary_packets", 2)


def test_render_into_page_locked_image_equals_copy(ctx):
    """gbt_render writes a page-locked host image from the frame's last kernel and
    copies into other host memory; the same seed gives the same image bits (spp 1:
    one path per pixel, so each shading launch adds at most once to a pixel)."""
    import ctypes as C

    from trace_gb300 import _lib

    s = scenes.cornell()
    w, h = 64, 48
    rd = s["render"]
    cam = dict(s["camera"], aspect=w / h)
    ds = pt.DeviceScene.from_dict(ctx, s)
    g = pt.DefaultLBVH(ds)
    ref, _ = g.render(cam, w, h, 1, rd["max_depth"], rd["miss_mode"], rd["miss_color"], seed=7)
    hp = C.c_void_p()
    ctx.check(ctx.L.gbt_host_alloc(ctx.h, w * h * 3 * 4, C.byref(hp)), "host_alloc")
    try:
        img = np.ctypeslib.as_array(C.cast(hp, C.POINTER(C.c_float)), shape=(h, w, 3))
        img[...] = -1.0
        p = _lib.RenderParams(w, h, 1, rd["max_depth"], rd["miss_mode"], (C.c_float * 3)(*rd["miss_color"]), 7)
        st = _lib.RenderStats()
        ctx.check(ctx.L.gbt_render(ctx.h, g.h, C.byref(pt.make_camera(cam)), C.byref(p), hp, C.byref(st)), "render")
        assert np.array_equal(img.view(np.uint32), ref.view(np.uint32))
    finally:
        ctx.check(ctx.L.gbt_host_free(ctx.h, hp), "host_free")
