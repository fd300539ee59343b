"""ctypes wrapper over the CPU oracle (oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker.  The product package never
imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_lib = None


def build(force=False):
    if force or not os.path.exists(LIB_PATH) or \
            os.path.getmtime(LIB_PATH) < max(os.path.getmtime(os.path.join(HERE, f)) for f in ("oracle.c", "oracle.h")):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        i64, i32, d = C.c_int64, C.c_int32, C.c_double
        L.orc_split_by3.restype = C.c_uint64
        L.orc_split_by3.argtypes = [C.c_uint64]
        L.orc_encode.restype = C.c_uint64
        L.orc_encode.argtypes = [C.c_uint64] * 3
        L.orc_prim_boxes.argtypes = [P, i64, P, i64, P]
        L.orc_enclosing.argtypes = [P, i64, P]
        L.orc_surface.restype = d
        L.orc_surface.argtypes = [P]
        L.orc_morton.argtypes = [P, i64, P, P]
        L.orc_sort_pairs.restype = C.c_int
        L.orc_sort_pairs.argtypes = [P, i64, C.c_int, P, P]
        L.orc_lbvh_build.restype = C.c_int
        L.orc_lbvh_build.argtypes = [P, i64, P, i64, C.c_int, C.POINTER(P)]
        L.orc_bvh_free.argtypes = [P]
        L.orc_bvh_counts.argtypes = [P, P]
        L.orc_bvh_export.argtypes = [P, P, P, P, P]
        L.orc_bvh_cost.restype = d
        L.orc_bvh_cost.argtypes = [P]
        L.orc_bvh_size.restype = i64
        L.orc_bvh_size.argtypes = [P]
        L.orc_bvh_sorted.argtypes = [P, P, P]
        L.orc_trace.argtypes = [P, P, i64, C.c_int, P, P, P, P]
        L.orc_prim_intersect.restype = C.c_int
        L.orc_prim_intersect.argtypes = [P, i32, P, P, P, P, P]
        L.orc_traversal_steps.argtypes = [P, P, i64, C.c_int, P]
        L.orc_render.restype = C.c_int
        L.orc_render.argtypes = [P, P, P, P, P, P, P, P]
        L.orc_adjoint.restype = C.c_int
        L.orc_adjoint.argtypes = [P, P, P, P, P, P, P, P, P]
        L.orc_heatmap.argtypes = [P, P, i32, i32, i32, C.c_int, P, P]
        L.orc_to_image.argtypes = [P, i32, i32, P]
        L.orc_phr_build.restype = C.c_int
        L.orc_phr_build.argtypes = [P, d, d, C.c_int, C.POINTER(P), P]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


class CameraDesc(C.Structure):
    _fields_ = [("look_from", C.c_double * 3), ("look_at", C.c_double * 3), ("up", C.c_double * 3),
                ("aspect", C.c_double), ("fov_deg", C.c_double)]


class RenderDesc(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("spp", C.c_int32), ("max_depth", C.c_int32),
                ("miss_mode", C.c_int32), ("miss_color", C.c_double * 3), ("seed", C.c_uint64),
                ("threads", C.c_int32), ("rays_traced", C.c_int64)]


def split_by3(a):
    return lib().orc_split_by3(int(a))


def prim_boxes(verts, spheres=None):
    verts = np.ascontiguousarray(verts, np.float32)
    sph = np.ascontiguousarray(spheres if spheres is not None else np.zeros((0, 4)), np.float32)
    n = verts.shape[0] + sph.shape[0]
    out = np.empty((n, 6), np.float64)
    lib().orc_prim_boxes(_p(verts), verts.shape[0], _p(sph), sph.shape[0], _p(out))
    return out


def enclosing(boxes):
    out = np.empty(6, np.float64)
    lib().orc_enclosing(_p(np.ascontiguousarray(boxes)), boxes.shape[0], _p(out))
    return out


def morton(boxes, encl):
    boxes = np.ascontiguousarray(boxes, np.float64)
    codes = np.empty(boxes.shape[0], np.uint64)
    lib().orc_morton(_p(boxes), boxes.shape[0], _p(np.ascontiguousarray(encl, np.float64)), _p(codes))
    return codes


def sort_pairs(codes, threads=1):
    codes = np.ascontiguousarray(codes, np.uint64)
    sc = np.empty_like(codes)
    si = np.empty(codes.shape[0], np.int32)
    rc = lib().orc_sort_pairs(_p(codes), codes.shape[0], threads, _p(sc), _p(si))
    if rc != 0:
        raise RuntimeError("oracle sort failed: %d" % rc)
    return sc, si


class BVH:
    """An oracle BVH (LBVH or PHR) owned by the C library."""

    def __init__(self, handle):
        self.h = handle

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_bvh_free(self.h)
            self.h = None

    def counts(self):
        out = np.zeros(4, np.int64)
        lib().orc_bvh_counts(self.h, _p(out))
        return out

    def export(self):
        """(kind, count, box, prims) in depth-first pre-order."""
        n_nodes, _, n_refs, _ = self.counts()
        kind = np.empty(n_nodes, np.int8)
        count = np.empty(n_nodes, np.int32)
        box = np.empty((n_nodes, 6), np.float64)
        prims = np.empty(max(n_refs, 1), np.int32)[:n_refs]
        lib().orc_bvh_export(self.h, _p(kind), _p(count), _p(box), _p(prims))
        return kind, count, box, prims

    def cost(self):
        return lib().orc_bvh_cost(self.h)

    def size(self):
        return lib().orc_bvh_size(self.h)

    def sorted_pairs(self, n):
        c = np.empty(n, np.uint64)
        i = np.empty(n, np.int32)
        lib().orc_bvh_sorted(self.h, _p(c), _p(i))
        return c, i

    def trace(self, rays, threads=os.cpu_count() or 1):
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        prim = np.empty(n, np.int32)
        t, u, v = (np.empty(n, np.float64) for _ in range(3))
        lib().orc_trace(self.h, _p(rays), n, threads, _p(prim), _p(t), _p(u), _p(v))
        return prim, t, u, v

    def prim_intersect(self, prim, ray8):
        ray8 = np.ascontiguousarray(ray8, np.float32)
        t, u, v, det = (C.c_double() for _ in range(4))
        ok = lib().orc_prim_intersect(self.h, int(prim), _p(ray8), C.byref(t), C.byref(u), C.byref(v), C.byref(det))
        return bool(ok), t.value, u.value, v.value, det.value

    def traversal_steps(self, rays, threads=os.cpu_count() or 1):
        rays = np.ascontiguousarray(rays, np.float32)
        out = np.empty(rays.shape[0], np.int32)
        lib().orc_traversal_steps(self.h, _p(rays), rays.shape[0], threads, _p(out))
        return out

    def render(self, scene, width=None, height=None, spp=None, max_depth=None, seed=1, threads=None):
        cam, rd = scene["camera"], scene["render"]
        cd = CameraDesc()
        cd.look_from[:] = cam["look_from"]
        cd.look_at[:] = cam["look_at"]
        cd.up[:] = cam["up"]
        cd.aspect = cam["aspect"]
        cd.fov_deg = cam["fov"]
        r = RenderDesc()
        r.width = width or rd["width"]
        r.height = height or rd["height"]
        r.spp = spp or rd["spp"]
        r.max_depth = rd["max_depth"] if max_depth is None else max_depth
        r.miss_mode = rd["miss_mode"]
        r.miss_color[:] = rd["miss_color"]
        r.seed = seed
        r.threads = threads or (os.cpu_count() or 1)
        img = np.empty((r.height, r.width, 3), np.float64)
        pm = np.ascontiguousarray(scene["prim_mat"], np.int32)
        mt = np.ascontiguousarray(scene["mat_type"], np.int32)
        mc = np.ascontiguousarray(scene["mat_color"], np.float64)
        mp = scene.get("mat_param")
        mp = np.ascontiguousarray(mp if mp is not None else np.zeros(len(mt)), np.float64)
        rc = lib().orc_render(self.h, _p(pm), _p(mt), _p(mc), _p(mp), C.byref(cd), C.byref(r), _p(img))
        if rc != 0:
            raise RuntimeError("oracle render failed: %d" % rc)
        self.last_rays = int(r.rays_traced)
        return img

    def adjoint(self, camera, width, height, spp, max_depth, albedo, emission, dimg=None, seed=1, miss_mode=0,
                threads=None):
        """float64 image and (if dimg is given) dLoss/d(albedo, emission) with the GPU's random numbers."""
        cd = CameraDesc()
        cd.look_from[:] = camera["look_from"]
        cd.look_at[:] = camera["look_at"]
        cd.up[:] = camera["up"]
        cd.aspect = camera["aspect"]
        cd.fov_deg = camera["fov"]
        r = RenderDesc()
        r.width, r.height, r.spp, r.max_depth, r.miss_mode = width, height, spp, max_depth, miss_mode
        r.seed = seed
        r.threads = threads or (os.cpu_count() or 1)
        n = len(emission)
        alb = np.ascontiguousarray(albedo, np.float32).reshape(n, 3)
        emi = np.ascontiguousarray(emission, np.float32).reshape(n)
        img = np.empty((height, width, 3), np.float64)
        ga = np.zeros((n, 3), np.float64)
        ge = np.zeros(n, np.float64)
        d = None if dimg is None else np.ascontiguousarray(dimg, np.float32)
        rc = lib().orc_adjoint(self.h, C.byref(cd), C.byref(r), _p(alb), _p(emi), _p(d), _p(img), _p(ga), _p(ge))
        if rc != 0:
            raise RuntimeError("oracle adjoint failed: %d" % rc)
        return img, ga, ge

    def heatmap(self, camera, width, height, threshold, threads=None):
        """(rgb float64 (h, w, 3), counts int32 (h, w)) of the reference's heat-map renderer."""
        cd = CameraDesc()
        cd.look_from[:] = camera["look_from"]
        cd.look_at[:] = camera["look_at"]
        cd.up[:] = camera["up"]
        cd.aspect = camera["aspect"]
        cd.fov_deg = camera["fov"]
        rgb = np.empty((height, width, 3), np.float64)
        counts = np.empty((height, width), np.int32)
        lib().orc_heatmap(self.h, C.byref(cd), width, height, threshold, threads or (os.cpu_count() or 1), _p(rgb),
                          _p(counts))
        return rgb, counts

    def phr(self, alpha=0.5, delta=6.0, bf=2):
        h = C.c_void_p()
        stats = np.zeros(5, np.int64)
        rc = lib().orc_phr_build(self.h, float(alpha), float(delta), int(bf), C.byref(h), _p(stats))
        if rc != 0:
            raise RuntimeError("oracle PHR failed: %d" % rc)
        b = BVH(h)
        b.stats = dict(initial_cut=int(stats[0]), max_cut=int(stats[1]), nodes=int(stats[2]), leaves=int(stats[3]),
                       build_cost=int(stats[4]))
        return b


def to_image(rgb):
    """ToImage (buffer.go:60-69) of a (height, width, 3) float32 buffer: (height, width, 4) uint8."""
    rgb = np.ascontiguousarray(rgb, np.float32)
    h, w, _ = rgb.shape
    out = np.empty((h, w, 4), np.uint8)
    lib().orc_to_image(_p(rgb), w, h, _p(out))
    return out


def lbvh(verts, spheres=None, threads=os.cpu_count() or 1):
    verts = np.ascontiguousarray(verts, np.float32)
    sph = np.ascontiguousarray(spheres if spheres is not None else np.zeros((0, 4)), np.float32)
    h = C.c_void_p()
    rc = lib().orc_lbvh_build(_p(verts), verts.shape[0], _p(sph), sph.shape[0], threads, C.byref(h))
    if rc != 0:
        raise RuntimeError("oracle LBVH failed: %d" % rc)
    return BVH(h)
