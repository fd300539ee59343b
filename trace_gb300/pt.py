"""Host-side mirror of ChSchmidt99/trace pkg/pt over the C ABI (include/gbtrace.h).

The names follow the Go package so a caller of the reference finds the same
entry points:

  Go (pkg/pt)                                   here
  ------------------------------------------    -----------------------------------------
  ParseFromPath (obj.go:10-17)                  ParseFromPath(path) -> Geometry
  NewScene / NewSceneNode / NewMesh (scene.go)  the same names; node transforms of transformation.go
  Scene.CompileLBVH (scene.go:27-30)            Scene.CompileLBVH(ctx) / DefaultLBVH(scene)
  Scene.Compile / CompilePHR (scene.go:21-36)   Scene.Compile(ctx) / Scene.CompilePHR(ctx, a, d, bf)
  HeatMapRenderer (render.go:137-197)           NewHeatMapRenderer(bvh, camera, threshold)
  gridOptimizer (optimizer.go:19-94)            NewGridOptimizer(...).OptimizedPHRparams(aux, bf)
  NewPHRBuilder + BuildFromAuxilary (phr.go)    NewPHRBuilder(alpha, delta, bf).BuildFromAuxilary(aux)
  BVH.Cost / BVH.Size (bvh.go:46-52)            BVH.Cost() / BVH.Size()
  NewCamera (camera.go:53-59)                   NewCamera(aspect, fov, CameraTransformation)
  ImageRenderer.RenderToBuffer (render.go:91)   ImageRenderer(...).RenderToBuffer(buffer)
  NewPxlBuffer / NewFrameBuffer (buffer.go)     NewPxlBuffer(w, h) / NewFrameBuffer(w, h)

Errors: the Go code panics; here every failing call raises GbtError with the
library's message.  Everything runs on the GPU through libgbtrace.so; there
is no CPU path.
"""
from __future__ import annotations

import ctypes as C
import weakref
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import GbtError
from .scenegraph import (Diffuse, Geometry, IdentityMatrix, Light, Mesh, NewColor, NewMesh,  # noqa: F401
                         NewSceneNode, NewSphere, NewTriangle, NewTriangleWithoutNormals, NewVector3, Reflective,
                         Refractive, Rotate, Scale, ScaleUniform, SceneNode, Translate)
from .scenegraph import flatten as _flatten

DIFFUSE, LIGHT, REFLECTIVE, REFRACTIVE = 0, 1, 2, 3
MISS_BLACK, MISS_WHITE, MISS_SKY, MISS_CONSTANT = 0, 1, 2, 3


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Context:
    """A CUDA stream plus grow-only device scratch on one GPU (gbt_ctx)."""

    def __init__(self, device=0):
        self.L = _lib.load()
        h = C.c_void_p()
        rc = self.L.gbt_ctx_create(device, C.byref(h))
        if rc != 0:
            raise GbtError(rc, "gbt_ctx_create(device=%d) failed" % device)
        self.h = h
        # scenes and BVHs refer to the context: they are destroyed before it
        self._children = weakref.WeakSet()

    def _adopt(self, obj):
        self._children.add(obj)

    def check(self, rc, what=""):
        if rc != 0:
            msg = self.L.gbt_last_error(self.h)
            raise GbtError(rc, (what + ": " if what else "") + (msg.decode() if msg else ""))

    @property
    def stream(self):
        return self.L.gbt_ctx_stream(self.h)

    def sync(self):
        self.check(self.L.gbt_ctx_sync(self.h), "sync")

    OPTIONS = {"traversal": 0, "anyhit_last": 1, "primary_tiles": 2, "primary_packets": 3, "keep_workspace": 4,
               "phr_small_cut": 5, "spin_limit": 6, "test_withhold_tile": 7, "test_collapse_cap": 8}

    def set_option(self, name, value):
        """Execution option of later calls (gbt_ctx_set_option); results do not depend on it."""
        self.check(self.L.gbt_ctx_set_option(self.h, self.OPTIONS[name], int(value)), "set_option")

    def close(self):
        if getattr(self, "h", None):
            kids = list(getattr(self, "_children", ()))
            for k in kids:  # BVHs first, then the scenes they were built from
                if isinstance(k, BVH):
                    k.close()
            for k in kids:
                k.close()
            self.L.gbt_ctx_destroy(self.h)
            self.h = None

    @property
    def alive(self):
        return getattr(self, "h", None) is not None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # raw device buffers for callers without a CUDA runtime of their own
    def alloc(self, nbytes):
        p = C.c_void_p()
        self.check(self.L.gbt_device_alloc(self.h, nbytes, C.byref(p)), "device_alloc")
        return p.value

    def free(self, ptr):
        self.check(self.L.gbt_device_free(self.h, C.c_void_p(ptr)), "device_free")

    def h2d(self, dptr, arr):
        arr = np.ascontiguousarray(arr)
        self.check(self.L.gbt_copy_h2d_async(self.h, C.c_void_p(dptr), _p(arr), arr.nbytes), "h2d")

    def d2h(self, arr, dptr):
        self.check(self.L.gbt_copy_d2h_async(self.h, _p(arr), C.c_void_p(dptr), arr.nbytes), "d2h")


class DeviceScene:
    """Flattened primitives resident on the device (gbt_scene)."""

    def __init__(self, ctx, verts, normals=None, spheres=None, prim_mat=None, mat_type=None, mat_color=None,
                 mat_param=None):
        self.ctx = ctx
        self.verts = np.ascontiguousarray(verts, np.float32).reshape(-1, 9)
        self.normals = None if normals is None else np.ascontiguousarray(normals, np.float32).reshape(-1, 9)
        sph = np.zeros((0, 4), np.float32) if spheres is None else np.ascontiguousarray(spheres, np.float32).reshape(-1, 4)
        self.spheres = sph
        n = self.verts.shape[0] + sph.shape[0]
        pm = np.zeros(n, np.uint32) if prim_mat is None else np.ascontiguousarray(prim_mat, np.uint32)
        mt = np.array([DIFFUSE], np.int32) if mat_type is None else np.asarray(mat_type, np.int32)
        mc = np.array([[0.5, 0.5, 0.5]]) if mat_color is None else np.asarray(mat_color, np.float64).reshape(-1, 3)
        mats = (_lib.Material * len(mt))()
        mp = np.zeros(len(mt)) if mat_param is None else np.asarray(mat_param, np.float64).reshape(-1)
        for i in range(len(mt)):
            mats[i].type = int(mt[i])
            mats[i].color[:] = [float(x) for x in mc[i]]
            mats[i].param = float(mp[i])
        sarr = (_lib.Sphere * max(1, sph.shape[0]))()
        for i in range(sph.shape[0]):
            sarr[i].center[:] = [float(x) for x in sph[i, :3]]
            sarr[i].radius = float(sph[i, 3])
        h = C.c_void_p()
        ctx.check(ctx.L.gbt_scene_upload(ctx.h, _p(self.verts), _p(self.normals), self.verts.shape[0],
                                         C.cast(sarr, C.c_void_p), sph.shape[0], _p(pm), C.cast(mats, C.c_void_p),
                                         len(mt), C.byref(h)), "scene_upload")
        self.h = h
        self.n_prim = n
        ctx._adopt(self)

    @classmethod
    def from_dict(cls, ctx, s):
        return cls(ctx, s["verts"], s.get("normals"), s.get("spheres"), s.get("prim_mat"), s.get("mat_type"),
                   s.get("mat_color"), s.get("mat_param"))

    def close(self):
        if getattr(self, "h", None):
            if self.ctx.alive:  # a closed context has already destroyed this scene
                self.ctx.L.gbt_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BVH:
    """A device BVH (gbt_bvh) with the queries of pkg/pt/bvh.go."""

    def __init__(self, ctx, h, scene, kind):
        self.ctx, self.h, self.scene, self.kind = ctx, h, scene, kind
        ctx._adopt(self)

    def close(self):
        if getattr(self, "h", None):
            if self.ctx.alive:
                self.ctx.L.gbt_bvh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def Cost(self):
        c = C.c_double()
        self.ctx.check(self.ctx.L.gbt_bvh_cost(self.ctx.h, self.h, C.byref(c)), "bvh_cost")
        return c.value

    def Size(self):
        c = C.c_int64()
        self.ctx.check(self.ctx.L.gbt_bvh_size(self.ctx.h, self.h, C.byref(c)), "bvh_size")
        return c.value

    def set_layout(self, width):
        """Traversal layout: 4 (a 4-wide view collapsed from the binary tree) or 2 (the binary nodes)."""
        self.ctx.check(self.ctx.L.gbt_bvh_set_layout(self.ctx.h, self.h, int(width)), "bvh_set_layout")

    def set_packets(self, choice):
        """Camera rays of a 4-wide tree: 0 measure on the next render, 1 packets, 2 one ray per lane."""
        self.ctx.check(self.ctx.L.gbt_bvh_set_packets(self.ctx.h, self.h, int(choice)), "bvh_set_packets")

    def packets(self):
        c = C.c_int32()
        self.ctx.check(self.ctx.L.gbt_bvh_get_packets(self.ctx.h, self.h, C.byref(c)), "bvh_get_packets")
        return c.value

    def counts(self):
        out = np.zeros(4, np.int64)
        self.ctx.check(self.ctx.L.gbt_bvh_counts(self.ctx.h, self.h, _p(out)), "bvh_counts")
        return out

    def export(self):
        n_nodes, _, n_refs, _ = self.counts()
        kind = np.empty(n_nodes, np.int8)
        count = np.empty(n_nodes, np.int32)
        box = np.empty((n_nodes, 6), np.float64)
        prims = np.empty(max(1, n_refs), np.int32)
        self.ctx.check(self.ctx.L.gbt_bvh_export(self.ctx.h, self.h, _p(kind), _p(count), _p(box), _p(prims)), "export")
        return kind, count, box, prims[:n_refs]

    def sorted_pairs(self):
        n = self.scene.n_prim
        codes = np.empty(n, np.uint64)
        idx = np.empty(n, np.int32)
        self.ctx.check(self.ctx.L.gbt_lbvh_sorted(self.ctx.h, self.h, _p(codes), _p(idx)), "lbvh_sorted")
        return codes, idx

    def trace(self, rays):
        """rays: (n, 8) float32 (origin, tmin, dir, tmax) -> (prim, t, u, v)."""
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        n = rays.shape[0]
        hits = np.empty((n, 4), np.float32)
        self.ctx.check(self.ctx.L.gbt_trace(self.ctx.h, self.h, _p(rays), n, _p(hits)), "trace")
        return hits[:, 0].view(np.int32).copy(), hits[:, 1].copy(), hits[:, 2].copy(), hits[:, 3].copy()

    def render(self, camera, width, height, spp, max_depth, miss_mode=MISS_BLACK, miss_color=(0, 0, 0), seed=1):
        cam = camera if isinstance(camera, _lib.Camera) else make_camera(camera)
        p = _lib.RenderParams(width, height, spp, max_depth, miss_mode, (C.c_float * 3)(*miss_color), seed)
        img = np.empty((height, width, 3), np.float32)
        st = _lib.RenderStats()
        self.ctx.check(self.ctx.L.gbt_render(self.ctx.h, self.h, C.byref(cam), C.byref(p), _p(img), C.byref(st)),
                       "render")
        return img, dict(rays_traced=st.rays_traced, paths=st.paths, ms=st.ms_total)


class Batch:
    """Many renders in one call (gbt_render_batch_async): items of (BVH, camera, params)."""

    def __init__(self, ctx, bvhs, cameras, params):
        self.ctx = ctx
        n = len(bvhs)
        self.items = (_lib.BatchItem * n)()
        self.images = []
        self.bvhs = list(bvhs)  # kept alive with the batch
        self.paths = 0
        for i, (b, cam, p) in enumerate(zip(bvhs, cameras, params)):
            it = self.items[i]
            it.bvh = b.h
            it.camera = cam if isinstance(cam, _lib.Camera) else make_camera(cam)
            w, h = int(p["width"]), int(p["height"])
            it.params = _lib.RenderParams(w, h, int(p["spp"]), int(p["max_depth"]), int(p.get("miss_mode", 0)),
                                          (C.c_float * 3)(*p.get("miss_color", (0, 0, 0))), int(p.get("seed", 1)))
            d = ctx.alloc(w * h * 3 * 4)
            it.d_rgb = d
            self.images.append((d, h, w))
            self.paths += w * h * int(p["spp"])
        self.n = n
        self.graph = None

    def render(self, mode="batched", cfg=None):
        L, h = self.ctx.L, self.ctx.h
        if mode == "batched":
            self.ctx.check(L.gbt_render_batch_async(h, self.items, self.n, C.byref(cfg) if cfg else None), "batch")
        elif mode == "plain":
            self.ctx.check(L.gbt_render_batch_plain_async(h, self.items, self.n), "batch plain")
        elif mode == "graph":
            self.ctx.check(L.gbt_graph_launch(h, self.graph), "graph launch")
        else:
            raise ValueError(mode)

    def autotune(self):
        best = _lib.BatchConfig()
        ms = C.c_double()
        self.ctx.check(self.ctx.L.gbt_batch_autotune(self.ctx.h, self.items, self.n, C.byref(best), C.byref(ms)),
                       "autotune")
        return best, ms.value

    def make_graph(self, rebuild=False, cfg=None):
        self.close_graph()
        g = C.c_void_p()
        self.ctx.check(self.ctx.L.gbt_batch_graph_create(self.ctx.h, self.items, self.n, C.byref(cfg) if cfg else None,
                                                         1 if rebuild else 0, C.byref(g)), "graph create")
        self.graph = g

    def close_graph(self):
        if self.graph:
            self.ctx.L.gbt_graph_destroy(self.graph)
            self.graph = None

    def read(self, i):
        d, h, w = self.images[i]
        img = np.empty((h, w, 3), np.float32)
        self.ctx.d2h(img, d)
        self.ctx.sync()
        return img

    def close(self):
        if self.graph:
            self.ctx.L.gbt_graph_destroy(self.graph)
            self.graph = None
        for d, _, _ in self.images:
            self.ctx.free(d)
        self.images = []


class RenderFunction:
    """Differentiable render with Forward/Backward in the manner of
    torch.autograd.Function (gbt_adjoint_*): per-triangle albedo (n, 3) and
    emission (n,) in, image out; Backward maps dLoss/dImage to the parameter
    gradients by path replay."""

    def __init__(self, bvh, camera, params):
        self.ctx, self.bvh = bvh.ctx, bvh
        self.cam = camera if isinstance(camera, _lib.Camera) else make_camera(camera)
        p = params
        self.w, self.h = int(p["width"]), int(p["height"])
        self.params = _lib.RenderParams(self.w, self.h, int(p["spp"]), int(p["max_depth"]), int(p.get("miss_mode", 0)),
                                        (C.c_float * 3)(*p.get("miss_color", (0, 0, 0))), int(p.get("seed", 1)))
        n = bvh.scene.verts.shape[0]
        self.n = n
        c = self.ctx
        npx = self.w * self.h * 3
        self.d_alb, self.d_emi = c.alloc(n * 12), c.alloc(n * 4)
        self.d_img, self.d_tgt, self.d_dimg = c.alloc(npx * 4), c.alloc(npx * 4), c.alloc(npx * 4)
        self.d_ga, self.d_ge, self.d_loss = c.alloc(n * 12), c.alloc(n * 4), c.alloc(8)

    def _set(self, albedo, emission):
        self.ctx.h2d(self.d_alb, np.ascontiguousarray(albedo, np.float32).reshape(self.n, 3))
        self.ctx.h2d(self.d_emi, np.ascontiguousarray(emission, np.float32).reshape(self.n))

    def Forward(self, albedo, emission):
        self._set(albedo, emission)
        L, h = self.ctx.L, self.ctx.h
        self.ctx.check(L.gbt_adjoint_forward_async(h, self.bvh.h, C.byref(self.cam), C.byref(self.params),
                                                   C.c_void_p(self.d_alb), C.c_void_p(self.d_emi),
                                                   C.c_void_p(self.d_img)), "adjoint forward")
        img = np.empty((self.h, self.w, 3), np.float32)
        self.ctx.d2h(img, self.d_img)
        self.ctx.sync()
        return img

    def Backward(self, dimage):
        """dLoss/dImage (h, w, 3) -> (dLoss/dalbedo (n, 3), dLoss/demission (n,)) at the last Forward's parameters."""
        self.ctx.h2d(self.d_dimg, np.ascontiguousarray(dimage, np.float32))
        return self._backward()

    def _backward(self):
        L, h = self.ctx.L, self.ctx.h
        self.ctx.check(L.gbt_adjoint_backward_async(h, self.bvh.h, C.byref(self.cam), C.byref(self.params),
                                                    C.c_void_p(self.d_alb), C.c_void_p(self.d_emi),
                                                    C.c_void_p(self.d_dimg), C.c_void_p(self.d_ga),
                                                    C.c_void_p(self.d_ge)), "adjoint backward")
        ga = np.empty((self.n, 3), np.float32)
        ge = np.empty(self.n, np.float32)
        self.ctx.d2h(ga, self.d_ga)
        self.ctx.d2h(ge, self.d_ge)
        self.ctx.sync()
        return ga, ge

    def set_target(self, target):
        self.ctx.h2d(self.d_tgt, np.ascontiguousarray(target, np.float32))
        self.ctx.sync()

    def loss(self, albedo, emission):
        """L2 loss of the image at these parameters against the target (float64)."""
        self.Forward(albedo, emission)
        L, h = self.ctx.L, self.ctx.h
        self.ctx.check(L.gbt_l2_loss_async(h, C.c_void_p(self.d_img), C.c_void_p(self.d_tgt), self.w * self.h * 3,
                                           C.c_void_p(self.d_dimg), C.c_void_p(self.d_loss)), "l2")
        out = np.zeros(1, np.float64)
        self.ctx.d2h(out, self.d_loss)
        self.ctx.sync()
        return float(out[0])

    def loss_and_grad(self, albedo, emission):
        """One optimisation step's worth: forward, loss, backward (dLoss/dImage stays on the device)."""
        loss = self.loss(albedo, emission)
        ga, ge = self._backward()
        return loss, ga, ge

    def close(self):
        for p in (self.d_alb, self.d_emi, self.d_img, self.d_tgt, self.d_dimg, self.d_ga, self.d_ge, self.d_loss):
            self.ctx.free(p)


def make_camera(cam):
    c = _lib.Camera()
    c.look_from[:] = [float(x) for x in cam["look_from"]]
    c.look_at[:] = [float(x) for x in cam["look_at"]]
    c.up[:] = [float(x) for x in cam["up"]]
    c.aspect = float(cam["aspect"])
    c.fov_deg = float(cam["fov"])
    return c


# ---------------------------------------------------------------------------
# Go-named entry points
# ---------------------------------------------------------------------------
def DefaultLBVH(scene: DeviceScene) -> BVH:
    """pkg/pt/lbvh.go:13-15."""
    ctx = scene.ctx
    h = C.c_void_p()
    ctx.check(ctx.L.gbt_lbvh_build(ctx.h, scene.h, C.byref(h)), "lbvh_build")
    return BVH(ctx, h, scene, "lbvh")


@dataclass
class PhrBuilder:
    """pkg/pt/phr.go:13-24 (Threshold = DefaultThreshold, Split = SweepSAH)."""
    Alpha: float = 0.5
    Delta: float = 6.0
    BranchingFactor: int = 2

    def BuildFromAuxilary(self, aux: BVH) -> BVH:
        ctx = aux.ctx
        h = C.c_void_p()
        ctx.check(ctx.L.gbt_phr_build(ctx.h, aux.h, float(self.Alpha), float(self.Delta), int(self.BranchingFactor),
                                      C.byref(h)), "phr_build")
        return BVH(ctx, h, aux.scene, "phr")

    def Build(self, scene: DeviceScene) -> BVH:
        aux = DefaultLBVH(scene)
        out = self.BuildFromAuxilary(aux)
        out.aux = aux
        return out

    def BuildWithCost(self, aux: BVH):
        """phr.go:154-192: (tree, build cost = initial cut size + sizes of the cuts split)."""
        ctx = aux.ctx
        h = C.c_void_p()
        cost = C.c_int64()
        ctx.check(ctx.L.gbt_phr_build_with_cost(ctx.h, aux.h, float(self.Alpha), float(self.Delta),
                                                int(self.BranchingFactor), C.byref(h), C.byref(cost)),
                  "phr_build_with_cost")
        return BVH(ctx, h, aux.scene, "phr"), int(cost.value)


def NewPHRBuilder(alpha, delta, branching_factor):
    return PhrBuilder(alpha, delta, branching_factor)


@dataclass
class GridOptimizer:
    """optimizer.go:19-94: exhaustive (alpha, delta) search scored by build cost and SAH cost."""
    Alphas: list
    Deltas: list
    pixels: int
    width: int = 0
    height: int = 0

    def OptimizedPHRparams(self, aux: BVH, branching: int = 2, threads: int = 0):
        """(alpha, delta) of the best candidate; self.evaluations holds (alpha, delta, sah, build) per
        candidate in grid order.  `threads` is accepted for the reference's signature."""
        ctx = aux.ctx
        al = np.ascontiguousarray(self.Alphas, np.float64)
        de = np.ascontiguousarray(self.Deltas, np.float64)
        ev = np.zeros((al.size * de.size, 2), np.float64)
        a, d = C.c_double(), C.c_double()
        w, h = (self.width, self.height) if self.width * self.height == self.pixels else (self.pixels, 1)
        ctx.check(ctx.L.gbt_phr_optimize_grid(ctx.h, aux.h, int(branching), _p(al), al.size, _p(de), de.size, w, h,
                                              C.byref(a), C.byref(d), _p(ev)), "phr_optimize_grid")
        self.evaluations = [(float(x), float(y), float(ev[k, 0]), int(ev[k, 1]))
                            for k, (x, y) in enumerate((x, y) for x in al for y in de)]
        return a.value, d.value


def NewGridOptimizer(alphas, deltas, frameWidth, frameHeight):
    return GridOptimizer(list(alphas), list(deltas), frameWidth * frameHeight, frameWidth, frameHeight)


def NewDefaultGridOptimizer(frameWidth, frameHeight):
    return NewGridOptimizer([0.4, 0.45, 0.5, 0.55], [6, 7, 8, 9], frameWidth, frameHeight)  # optimizer.go:25-27


def NewDefaultBuilder():
    return PhrBuilder(0.5, 6.0, 2)  # phr.go:26-28


@dataclass
class CameraTransformation:
    LookFrom: tuple
    LookAt: tuple
    Up: tuple = (0.0, 1.0, 0.0)


@dataclass
class Camera:
    aspect: float
    fov: float
    transform: CameraTransformation

    def SetTransformation(self, t):
        self.transform = t

    def desc(self):
        return dict(look_from=self.transform.LookFrom, look_at=self.transform.LookAt, up=self.transform.Up,
                    aspect=self.aspect, fov=self.fov)


def NewCamera(aspect, fov, transform):
    return Camera(aspect, fov, transform)


def NewDefaultCamera(aspect, fov):
    return Camera(aspect, fov, CameraTransformation((0, 0, 0), (1, 0, 0), (0, 1, 0)))


class _Buffer:
    """A device-resident render target (gbt_buffer).  The device side is created on the first
    RenderToBuffer, on the BVH's context, unless a context is given here.  `data` is the
    host copy of the colours (height, width, 3), row y = 0 first (buffer.go:47-49),
    refreshed after every RenderToBuffer."""

    KIND = 0

    def __init__(self, width, height, ctx=None):
        self.width, self.height = int(width), int(height)
        self.data = np.zeros((self.height, self.width, 3), np.float32)
        self.samples = 0
        self.ctx = None
        self.h = None
        if ctx is not None:
            self._bind(ctx)

    def _bind(self, ctx):
        if self.h is not None:
            if ctx is not self.ctx:
                raise GbtError(-1, "buffer belongs to another context")
            return
        h = C.c_void_p()
        ctx.check(ctx.L.gbt_buffer_create(ctx.h, self.KIND, self.width, self.height, C.byref(h)), "buffer_create")
        self.ctx, self.h = ctx, h
        ctx._adopt(self)

    def Width(self):
        return self.width

    def Height(self):
        return self.height

    def _render(self, bvh, cam, params):
        self._bind(bvh.ctx)
        st = _lib.RenderStats()
        c = self.ctx
        c.check(c.L.gbt_render_to_buffer(c.h, bvh.h, C.byref(cam), C.byref(params), self.h, C.byref(st)),
                "render_to_buffer")
        n = C.c_uint64()
        c.check(c.L.gbt_buffer_read(c.h, self.h, _p(self.data), C.byref(n)), "buffer_read")
        self.samples = int(n.value)
        return st

    def ToImage(self):
        """buffer.go:60-69 / 104-116: (height, width, 4) uint8 RGBA, image row 0 first."""
        if self.h is None:
            raise GbtError(-1, "ToImage: the buffer has no device side yet (give NewPxlBuffer a context or render "
                               "into it first)")
        out = np.empty((self.height, self.width, 4), np.uint8)
        self.ctx.check(self.ctx.L.gbt_buffer_to_image(self.ctx.h, self.h, _p(out)), "buffer_to_image")
        return out

    def close(self):
        if getattr(self, "h", None):
            if self.ctx.alive:
                self.ctx.L.gbt_buffer_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PixelBuffer(_Buffer):
    """buffer.go:28-58: each pixel is the running mean of every sample added, across calls."""
    KIND = 0


class FrameBuffer(_Buffer):
    """buffer.go:71-116: each pixel holds the last sample written."""
    KIND = 1


def NewPxlBuffer(width, height, ctx=None):
    return PixelBuffer(width, height, ctx)  # buffer.go:39-45


def NewPxlBufferAR(height, aspect, ctx=None):
    return PixelBuffer(int(float(height) * aspect), height, ctx)  # buffer.go:34-37


def NewFrameBuffer(width, height, ctx=None):
    return FrameBuffer(width, height, ctx)  # buffer.go:83-89


def NewFrameBufferAR(height, aspect, ctx=None):
    return FrameBuffer(int(float(height) * aspect), height, ctx)  # buffer.go:78-81


@dataclass
class ImageRenderer:
    """pkg/pt/render.go:20-30; only the built-in shaders run on the device."""
    Bvh: BVH
    Camera: Camera
    MaxDepth: int = 5
    Spp: int = 300
    Miss: int = MISS_BLACK
    MissColor: tuple = (0.0, 0.0, 0.0)
    Seed: int = 1
    Verbose: bool = False
    last_stats: dict = None

    def RenderToBuffer(self, buff):
        """Adds Spp samples per pixel to buff (a PixelBuffer keeps the running mean of all of
        them, a FrameBuffer the last one)."""
        cam = make_camera(self.Camera.desc())
        p = _lib.RenderParams(buff.width, buff.height, int(self.Spp), int(self.MaxDepth), int(self.Miss),
                              (C.c_float * 3)(*self.MissColor), int(self.Seed))
        st = buff._render(self.Bvh, cam, p)
        self.last_stats = dict(rays_traced=st.rays_traced, paths=st.paths, ms=st.ms_total)
        return buff

    def GetBvh(self):
        return self.Bvh

    def SetBvh(self, bvh):
        self.Bvh = bvh

    def GetCamera(self):
        return self.Camera


def NewDefaultRenderer(bvh, camera):
    return ImageRenderer(bvh, camera, MaxDepth=5, Spp=300, Miss=MISS_BLACK)  # render.go:32-44


def NewBenchmarkRenderer(bvh, camera):
    return ImageRenderer(bvh, camera, MaxDepth=5, Spp=1, Miss=MISS_WHITE)  # render.go:60-72


@dataclass
class HeatMapRenderer:
    """pkg/pt/render.go:137-197: per pixel the traversal-step count of the pixel-centre ray,
    coloured by DefaultTraversalCountShader (render.go:250-257)."""
    Bvh: BVH
    Camera: Camera
    Threshold: int
    last_counts: np.ndarray = field(default=None, repr=False)

    def RenderToBuffer(self, buff):
        """One sample per pixel added to buff (render.go:155-197 calls addSample once per pixel)."""
        ctx = self.Bvh.ctx
        cam = make_camera(self.Camera.desc() if isinstance(self.Camera, Camera) else self.Camera)
        w, h = buff.width, buff.height
        counts = np.empty((h, w), np.int32)
        buff._bind(ctx)
        d_rgb, d_cnt = ctx.alloc(w * h * 3 * 4), ctx.alloc(w * h * 4)
        try:
            ctx.check(ctx.L.gbt_heatmap_async(ctx.h, self.Bvh.h, C.byref(cam), w, h, int(self.Threshold),
                                              C.c_void_p(d_rgb), C.c_void_p(d_cnt)), "heatmap")
            ctx.check(ctx.L.gbt_buffer_add_async(ctx.h, buff.h, C.c_void_p(d_rgb), 1), "buffer_add")
            ctx.d2h(counts, d_cnt)
            n = C.c_uint64()
            ctx.check(ctx.L.gbt_buffer_read(ctx.h, buff.h, _p(buff.data), C.byref(n)), "buffer_read")
            buff.samples = int(n.value)
        finally:
            ctx.free(d_rgb)
            ctx.free(d_cnt)
        self.last_counts = counts
        return buff

    def GetBvh(self):
        return self.Bvh

    def SetBvh(self, bvh):
        self.Bvh = bvh

    def GetCamera(self):
        return self.Camera


def NewHeatMapRenderer(bvh, camera, threshold):
    return HeatMapRenderer(bvh, camera, threshold)  # render.go:145-153


def ParseFromPath(path):
    """pkg/pt/obj.go:10-17 -> Geometry: triangles (n, 9) with per-vertex normals (n, 9); faces
    without normal indices get calcNormal normals (obj.go:93-110).  has_normals tells whether
    the file gave any."""
    L = _lib.load()
    n = C.c_uint32(0)
    hn = C.c_int32(0)
    rc = L.gbt_obj_parse(str(path).encode(), None, None, C.byref(n), C.byref(hn))
    if rc != 0:
        raise GbtError(rc, "ParseFromPath(%s)" % path)
    verts = np.empty((n.value, 9), np.float32)
    normals = np.empty((n.value, 9), np.float32)
    rc = L.gbt_obj_parse(str(path).encode(), _p(verts), _p(normals), C.byref(n), C.byref(hn))
    if rc != 0:
        raise GbtError(rc, "ParseFromPath(%s)" % path)
    g = Geometry(verts.astype(np.float64), normals.astype(np.float64), np.zeros((0, 4)))
    g.has_normals = bool(hn.value)
    return g


class Scene:
    """pkg/pt/scene.go:7-36: a scene graph compiled into a device scene and a BVH."""

    def __init__(self):
        self.root = NewSceneNode(None)

    def Add(self, node):
        self.root.Add(node)

    def tracables(self):
        """collectTracables from the identity (scene.go:21-36), flattened for upload."""
        return _flatten(self.root.collect(IdentityMatrix(), []))

    def UntransformedTracables(self):
        return _flatten(self.root.collect_raw([]))

    def upload(self, ctx):
        d = self.tracables()
        return DeviceScene(ctx, d["verts"], d["normals"] if d["verts"].shape[0] else None, d["spheres"],
                           d["prim_mat"], d["mat_type"], d["mat_color"], d["mat_param"])

    def Compile(self, ctx):
        return NewDefaultBuilder().Build(self.upload(ctx))

    def CompileLBVH(self, ctx):
        return DefaultLBVH(self.upload(ctx))

    def CompilePHR(self, ctx, alpha, delta, branchingFactor):
        return NewPHRBuilder(alpha, delta, branchingFactor).Build(self.upload(ctx))


def NewScene():
    return Scene()
