"""Device heat map (HeatMapRenderer, render.go:137-197) vs the oracle's.

Both count BVH.traversalSteps (bvh.go:21-44) on the same tree for the same
pixel-centre rays; the device traces in float32, the oracle in float64, so a
count may differ where a ray grazes a box or a hit distance decides a cull.
Bar: >= 99% of pixels with equal counts, mean count within 0.5%, and where the
counts agree the colour is the oracle's rounded to float32."""
import numpy as np
import pytest

from oracle import oracle as O
from trace_gb300 import pt, scenes

pytestmark = pytest.mark.gpu

EQUAL_FRAC = 0.99
MEAN_REL = 0.005

CASES = [
    ("cornell_lbvh", lambda: scenes.cornell(), None, 64, 48, 20),
    ("cornell_phr_bf2", lambda: scenes.cornell(), (0.5, 6.0, 2), 64, 48, 20),
    ("cornell_phr_bf4", lambda: scenes.cornell(), (0.55, 9.0, 4), 64, 48, 20),
    ("soup50k_lbvh", lambda: scenes.soup(50_000, seed=4), None, 160, 90, 40),
    ("soup50k_phr", lambda: scenes.soup(50_000, seed=4), (0.5, 6.0, 2), 160, 90, 40),
    ("terrain129_sun_phr_bf3", lambda: scenes.terrain(129), (0.5, 9.0, 3), 128, 72, 30),
]


@pytest.mark.parametrize("name,make,phr,w,h,thr", CASES, ids=[c[0] for c in CASES])
def test_heatmap_matches_oracle(ctx, name, make, phr, w, h, thr):
    s = make()
    cam = dict(s["camera"], aspect=w / h)
    ds = pt.DeviceScene.from_dict(ctx, s)
    g = pt.DefaultLBVH(ds)
    o = O.lbvh(s["verts"], s.get("spheres"))
    if phr is not None:
        g = pt.NewPHRBuilder(*phr).BuildFromAuxilary(g)
        o = o.phr(*phr)
    r = pt.NewHeatMapRenderer(g, pt.NewCamera(cam["aspect"], cam["fov"], pt.CameraTransformation(
        cam["look_from"], cam["look_at"], cam["up"])), thr)
    buf = r.RenderToBuffer(pt.NewPxlBuffer(w, h))
    got_c = r.last_counts
    want_rgb, want_c = o.heatmap(cam, w, h, thr)
    eq = got_c == want_c
    print("%s: equal %.5f mean %.3f vs %.3f max %d" % (name, eq.mean(), got_c.mean(), want_c.mean(), want_c.max()))
    assert eq.mean() >= EQUAL_FRAC
    assert abs(got_c.mean() - want_c.mean()) <= MEAN_REL * want_c.mean()
    assert want_c.max() > thr or name.startswith("cornell")  # both shader branches are exercised somewhere
    np.testing.assert_array_equal(buf.data[eq], want_rgb[eq].astype(np.float32))


def test_heatmap_rejects_bad_arguments(ctx):
    s = scenes.cornell()
    g = pt.DefaultLBVH(pt.DeviceScene.from_dict(ctx, s))
    cam = pt.make_camera(dict(s["camera"], aspect=1.0))
    rgb = np.empty((8, 8, 3), np.float32)
    L = ctx.L
    import ctypes as C
    assert L.gbt_heatmap(ctx.h, g.h, C.byref(cam), 8, 8, 0, rgb.ctypes.data_as(C.c_void_p), None) != 0
    assert L.gbt_heatmap(ctx.h, g.h, C.byref(cam), 1, 8, 5, rgb.ctypes.data_as(C.c_void_p), None) != 0
    assert L.gbt_heatmap(ctx.h, g.h, C.byref(cam), 8, 8, 5, rgb.ctypes.data_as(C.c_void_p), None) == 0
