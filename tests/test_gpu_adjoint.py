"""Path-replay adjoint vs central finite differences (h = 1e-3).

The sampled paths do not depend on albedo or emission and the forward image
is bitwise reproducible, so the loss is a deterministic polynomial in the
parameters and central differences check the adjoint directly.  Bar: 1e-3
relative on the parameters with the largest gradients.
"""
import numpy as np
import pytest

from trace_gb300 import pt, scenes

pytestmark = pytest.mark.gpu

H = 1e-3      # finite-difference step
REL = 1e-3    # relative agreement bar


def setup(ctx, w=64, h=64, spp=8, depth=5):
    s = scenes.cornell()
    n = s["verts"].shape[0]
    ds = pt.DeviceScene.from_dict(ctx, s)
    g = pt.DefaultLBVH(ds)
    rng4, rng5 = np.random.default_rng(4), np.random.default_rng(5)
    a0, e0 = rng4.uniform(0.2, 0.8, (n, 3)), rng4.uniform(0.2, 0.8, n)
    a1, e1 = rng5.uniform(0.2, 0.8, (n, 3)), rng5.uniform(0.2, 0.8, n)
    cam = dict(s["camera"], aspect=w / h)
    f = pt.RenderFunction(g, cam, dict(width=w, height=h, spp=spp, max_depth=depth, miss_mode=0, seed=11))
    target = f.Forward(a1, e1)
    f.set_target(target)
    return f, a0.astype(np.float32), e0.astype(np.float32)


def test_forward_is_reproducible(ctx):
    f, a, e = setup(ctx)
    try:
        i1, i2 = f.Forward(a, e), f.Forward(a, e)
        assert np.array_equal(i1, i2) and i1.mean() > 0
    finally:
        f.close()


def test_adjoint_matches_central_differences(ctx):
    f, a, e = setup(ctx)
    try:
        loss, ga, ge = f.loss_and_grad(a, e)
        assert np.isfinite(ga).all() and np.isfinite(ge).all() and loss > 0
        # the parameters with the largest gradients: albedo channels and emissions
        checks = []
        for idx in np.argsort(-np.abs(ge))[:6]:
            checks.append(("e", int(idx), 0, float(ge[idx])))
        flat = np.argsort(-np.abs(ga).ravel())[:6]
        for k in flat:
            checks.append(("a", int(k // 3), int(k % 3), float(ga.ravel()[k])))
        worst = 0.0
        for kind, t, c, g in checks:
            a1, a2, e1, e2 = a.copy(), a.copy(), e.copy(), e.copy()
            if kind == "e":
                e1[t] += H
                e2[t] -= H
            else:
                a1[t, c] += H
                a2[t, c] -= H
            # parameters are float32 on the device: use the step that was actually taken
            step = (float(e1[t]) - float(e2[t])) if kind == "e" else (float(a1[t, c]) - float(a2[t, c]))
            fd = (f.loss(a1, e1) - f.loss(a2, e2)) / step
            rel = abs(fd - g) / max(abs(fd), 1e-12)
            print("%s[%d,%d] adjoint %.6e fd %.6e rel %.2e" % (kind, t, c, g, fd, rel))
            worst = max(worst, rel)
        assert worst <= REL, worst
    finally:
        f.close()


def test_adjoint_matches_float64_cpu_adjoint(ctx):
    """The float64 CPU adjoint (oracle, same random numbers, so the same paths up to
    rounding) on the ~1k-triangle Cornell scene: images and gradients agree."""
    from oracle import oracle as O

    w, h, spp = 32, 32, 4
    s = scenes.cornell()
    n = s["verts"].shape[0]
    ds = pt.DeviceScene.from_dict(ctx, s)
    g = pt.DefaultLBVH(ds)
    rng = np.random.default_rng(4)
    a = rng.uniform(0.2, 0.8, (n, 3)).astype(np.float32)
    e = rng.uniform(0.2, 0.8, n).astype(np.float32)
    cam = dict(s["camera"], aspect=w / h)
    f = pt.RenderFunction(g, cam, dict(width=w, height=h, spp=spp, max_depth=5, miss_mode=0, seed=11))
    try:
        img = f.Forward(a, e)
        dimg = (2.0 * (img - 0.5)).astype(np.float32)  # a fixed upstream gradient, the same for both
        ga, ge = f.Backward(dimg)
        o = O.lbvh(s["verts"])
        oimg, oga, oge = o.adjoint(cam, w, h, spp, 5, a, e, dimg, seed=11)
        assert np.abs(img - oimg).max() <= 1e-3 * np.abs(oimg).max()
        rel_a = np.linalg.norm(ga - oga) / np.linalg.norm(oga)
        rel_e = np.linalg.norm(ge - oge) / np.linalg.norm(oge)
        print("cpu float64 adjoint: relative L2 gap albedo %.2e emission %.2e" % (rel_a, rel_e))
        assert rel_a <= 1e-3 and rel_e <= 1e-3
    finally:
        f.close()


def test_gradient_descent_reduces_loss(ctx):
    f, a, e = setup(ctx, spp=4)
    try:
        l0, ga, ge = f.loss_and_grad(a, e)
        lr = 0.5 / max(np.abs(ga).max(), np.abs(ge).max())
        a2 = np.clip(a - lr * ga, 0.0, 1.0)
        e2 = np.clip(e - lr * ge, 0.0, None)
        assert f.loss(a2, e2) < l0
    finally:
        f.close()
