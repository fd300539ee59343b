"""Seeded synthetic scenes.

The reference renders external meshes (pkg/demoscenes/*.go, loading
assets/local/*.obj, which are not distributed).  These generators stand in
for them with deterministic float32 geometry of the sizes the benchmark
configurations name:

* ``cornell``  -- five unit quads, a 0.3x0.3 emissive ceiling quad and a UV
  sphere (r=0.3 at (0,0.3,0)), like pkg/demoscenes/cornellbox.go but built from
  triangles only; 256x256, 16 spp, depth 5.
* ``soup``     -- N random triangles, centroids U[0,1]^3, vertices offset by
  U[-0.005,0.005] per axis; 1920x1080 primary rays plus one diffuse bounce.
* ``terrain``  -- a GxG height-field grid with 6-octave fBm heights over
  [0,1]^2, a sun-sized emissive sphere and a constant sky of 0.5.
* ``batch``    -- many soups / terrain patches with log-uniform sizes.

Every scene is a plain dict of numpy arrays:
  verts (N,9) float32  v0 v1 v2 per triangle
  spheres (S,4) float32 cx cy cz r
  prim_mat (N+S,) int32 material per primitive (triangles first)
  mat_type (M,) int32   0 = Diffuse(albedo), 1 = Light(color)  (material.go:13-42)
  mat_color (M,3) float64
  camera dict(look_from, look_at, up, fov, aspect)
  render dict(width, height, spp, max_depth, miss_mode, miss_color)
"""
from __future__ import annotations

import numpy as np

DIFFUSE, LIGHT, REFLECTIVE, REFRACTIVE = 0, 1, 2, 3
MISS_BLACK, MISS_WHITE, MISS_SKY, MISS_CONSTANT = 0, 1, 2, 3


def _quad(p, e1, e2):
    """Two triangles spanning the parallelogram p, p+e1, p+e1+e2, p+e2."""
    p, e1, e2 = (np.asarray(a, np.float64) for a in (p, e1, e2))
    a, b, c, d = p, p + e1, p + e1 + e2, p + e2
    return [np.concatenate([a, b, c]), np.concatenate([a, c, d])]


def uv_sphere(center, radius, seg_u, seg_v):
    """Triangles of a UV sphere with pole fans: 2*seg_u + 2*seg_u*(seg_v-2)."""
    c = np.asarray(center, np.float64)
    th = np.linspace(0.0, np.pi, seg_v + 1)
    ph = np.linspace(0.0, 2.0 * np.pi, seg_u + 1)
    st, ct = np.sin(th), np.cos(th)
    sp, cp = np.sin(ph), np.cos(ph)
    # points[i, j]: latitude i (0 = north pole), longitude j
    pts = np.stack([st[:, None] * cp[None, :], ct[:, None] * np.ones_like(cp)[None, :],
                    st[:, None] * sp[None, :]], axis=-1) * radius + c
    tris = []
    for i in range(seg_v):
        for j in range(seg_u):
            p00, p01 = pts[i, j], pts[i, j + 1]
            p10, p11 = pts[i + 1, j], pts[i + 1, j + 1]
            if i == 0:
                tris.append(np.concatenate([p00, p11, p10]))
            elif i == seg_v - 1:
                tris.append(np.concatenate([p00, p01, p10]))
            else:
                tris.append(np.concatenate([p00, p01, p11]))
                tris.append(np.concatenate([p00, p11, p10]))
    return np.asarray(tris)


def cornell(sphere_u=32, sphere_v=16, width=256, height=256, spp=16, max_depth=5):
    """Cornell-box-style scene (the small plain configuration)."""
    tris, mats = [], []

    def add(ts, m):
        tris.extend(ts)
        mats.extend([m] * len(ts))

    # materials: 0 grey, 1 red, 2 green, 3 light
    add(_quad([-0.5, 0.0, -0.5], [0, 0, 1], [1, 0, 0]), 0)      # floor y=0
    add(_quad([-0.5, 1.0, -0.5], [1, 0, 0], [0, 0, 1]), 0)      # ceiling y=1
    add(_quad([-0.5, 0.0, -0.5], [1, 0, 0], [0, 1, 0]), 0)      # back z=-0.5
    add(_quad([-0.5, 0.0, -0.5], [0, 1, 0], [0, 0, 1]), 1)      # left x=-0.5 (red)
    add(_quad([0.5, 0.0, -0.5], [0, 0, 1], [0, 1, 0]), 2)       # right x=+0.5 (green)
    add(_quad([-0.15, 0.999, -0.15], [0.3, 0, 0], [0, 0, 0.3]), 3)  # light 0.3x0.3
    sph = uv_sphere([0.0, 0.3, 0.0], 0.3, sphere_u, sphere_v)
    add(list(sph), 0)
    verts = np.asarray(tris, np.float64).astype(np.float32)
    return dict(
        name="cornell_%dx%d" % (sphere_u, sphere_v),
        verts=verts,
        spheres=np.zeros((0, 4), np.float32),
        prim_mat=np.asarray(mats, np.int32),
        mat_type=np.array([DIFFUSE, DIFFUSE, DIFFUSE, LIGHT], np.int32),
        mat_color=np.array([[0.7, 0.7, 0.7], [0.7, 0.1, 0.1], [0.1, 0.7, 0.1], [10.0, 10.0, 10.0]]),
        camera=dict(look_from=(0.0, 0.5, 2.2), look_at=(0.0, 0.5, 0.0), up=(0.0, 1.0, 0.0),
                    fov=40.0, aspect=width / height),
        render=dict(width=width, height=height, spp=spp, max_depth=max_depth,
                    miss_mode=MISS_BLACK, miss_color=(0.0, 0.0, 0.0)),
    )


def cornell_materials(width=256, height=256, spp=16, max_depth=5):
    """The Cornell box with a glass UV sphere (Refractive, ratio 1.5) and a small
    brushed-metal analytic sphere (Reflective, diffusion 0.15): the materials of
    material.go:44-106 on triangles and on a sphere primitive."""
    s = cornell(width=width, height=height, spp=spp, max_depth=max_depth)
    n = s["verts"].shape[0]
    pm = s["prim_mat"].copy()
    pm[n - len(list(uv_sphere([0.0, 0.3, 0.0], 0.3, 32, 16))):] = 4  # the UV sphere's triangles (added last)
    s.update(
        name="cornell_materials",
        spheres=np.array([[-0.28, 0.14, 0.22, 0.14]], np.float32),
        prim_mat=np.concatenate([pm, np.array([5], np.int32)]),
        mat_type=np.array([DIFFUSE, DIFFUSE, DIFFUSE, LIGHT, REFRACTIVE, REFLECTIVE], np.int32),
        mat_color=np.array([[0.7, 0.7, 0.7], [0.7, 0.1, 0.1], [0.1, 0.7, 0.1], [10.0, 10.0, 10.0],
                            [0.95, 0.95, 0.95], [0.8, 0.8, 0.8]]),
        mat_param=np.array([0.0, 0.0, 0.0, 0.0, 1.5, 0.15]),
    )
    return s


def soup(n=1_000_000, seed=1, width=1920, height=1080, spp=1, max_depth=0):
    """Random triangle soup (the 1M-triangle configuration)."""
    rng = np.random.default_rng(seed)
    c = rng.random((n, 1, 3))
    off = rng.uniform(-0.005, 0.005, size=(n, 3, 3))
    verts = (c + off).reshape(n, 9).astype(np.float32)
    return dict(
        name="soup_%d" % n,
        verts=verts,
        spheres=np.zeros((0, 4), np.float32),
        prim_mat=np.zeros(n, np.int32),
        mat_type=np.array([DIFFUSE], np.int32),
        mat_color=np.array([[0.7, 0.7, 0.7]]),
        camera=dict(look_from=(0.5, 0.5, 2.0), look_at=(0.5, 0.5, 0.5), up=(0.0, 1.0, 0.0),
                    fov=40.0, aspect=width / height),
        render=dict(width=width, height=height, spp=spp, max_depth=max_depth,
                    miss_mode=MISS_WHITE, miss_color=(1.0, 1.0, 1.0)),
    )


def fbm_heights(g, seed=2, octaves=6, amplitude=0.2, lacunarity=2.0, gain=0.5, base_cells=4):
    """6-octave value-noise fBm sampled on a g x g grid over [0,1]^2."""
    rng = np.random.default_rng(seed)
    x = np.linspace(0.0, 1.0, g)
    h = np.zeros((g, g), np.float64)
    amp, cells = amplitude, float(base_cells)
    for _ in range(octaves):
        nc = int(round(cells))
        lattice = rng.random((nc + 2, nc + 2)) * 2.0 - 1.0
        f = x * nc
        i = np.minimum(f.astype(np.int64), nc - 1)
        t = f - i
        s = t * t * (3.0 - 2.0 * t)
        i0, i1 = i[:, None], i[None, :]
        s0, s1 = s[:, None], s[None, :]
        v00 = lattice[i0, i1]
        v10 = lattice[i0 + 1, i1]
        v01 = lattice[i0, i1 + 1]
        v11 = lattice[i0 + 1, i1 + 1]
        a = v00 + (v10 - v00) * s0
        b = v01 + (v11 - v01) * s0
        h += amp * (a + (b - a) * s1)
        amp *= gain
        cells *= lacunarity
    return h


def terrain_tris(g, seed=2, x0=0.0, z0=0.0, size=1.0):
    """2*(g-1)^2 triangles of an fBm height field over [x0,x0+size]x[z0,z0+size]."""
    h = fbm_heights(g, seed=seed)
    xs = x0 + np.linspace(0.0, size, g)
    zs = z0 + np.linspace(0.0, size, g)
    X, Z = np.meshgrid(xs, zs, indexing="ij")
    P = np.stack([X, h * size, Z], axis=-1).astype(np.float32)
    p00 = P[:-1, :-1].reshape(-1, 3)
    p10 = P[1:, :-1].reshape(-1, 3)
    p01 = P[:-1, 1:].reshape(-1, 3)
    p11 = P[1:, 1:].reshape(-1, 3)
    n = p00.shape[0]
    verts = np.empty((2 * n, 9), np.float32)
    verts[0::2, 0:3], verts[0::2, 3:6], verts[0::2, 6:9] = p00, p01, p11
    verts[1::2, 0:3], verts[1::2, 3:6], verts[1::2, 6:9] = p00, p11, p10
    return verts


def terrain(g=2048, seed=2, width=1920, height=1080, spp=64, max_depth=4):
    """Procedural fBm terrain with a sun-sized spherical light (the 8.4M-triangle configuration)."""
    verts = terrain_tris(g, seed=seed)
    sun = np.array([[1.6, 2.2, -1.2, 0.25]], np.float32)
    n = verts.shape[0]
    prim_mat = np.zeros(n + 1, np.int32)
    prim_mat[n] = 1
    return dict(
        name="terrain_%d" % g,
        verts=verts,
        spheres=sun,
        prim_mat=prim_mat,
        mat_type=np.array([DIFFUSE, LIGHT], np.int32),
        mat_color=np.array([[0.5, 0.5, 0.5], [40.0, 38.0, 32.0]]),
        camera=dict(look_from=(0.5, 0.55, 1.6), look_at=(0.5, 0.0, 0.4), up=(0.0, 1.0, 0.0),
                    fov=50.0, aspect=width / height),
        render=dict(width=width, height=height, spp=spp, max_depth=max_depth,
                    miss_mode=MISS_CONSTANT, miss_color=(0.5, 0.5, 0.5)),
    )


def batch_sizes(count=64, lo=1_000, hi=2_000_000, seed=3):
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(np.log(lo), np.log(hi), size=count)).astype(np.int64)


def batch(count=64, lo=1_000, hi=2_000_000, seed=3, width=512, height=512, spp=16, max_depth=4):
    """Many independent scenes of log-uniform size: soups or terrain patches."""
    rng = np.random.default_rng(seed + 1000)
    sizes = batch_sizes(count, lo, hi, seed)
    scenes = []
    for k, n in enumerate(sizes):
        if rng.random() < 0.5:
            s = soup(int(n), seed=seed * 1000 + k, width=width, height=height, spp=spp, max_depth=max_depth)
            s["render"]["miss_mode"] = MISS_SKY
        else:
            g = max(2, int(np.sqrt(n / 2.0)) + 1)
            verts = terrain_tris(g, seed=seed * 1000 + k)
            s = dict(
                name="patch_%d" % verts.shape[0], verts=verts, spheres=np.zeros((0, 4), np.float32),
                prim_mat=np.zeros(verts.shape[0], np.int32), mat_type=np.array([DIFFUSE], np.int32),
                mat_color=np.array([[0.5, 0.5, 0.5]]),
                camera=dict(look_from=(0.5, 0.6, 1.6), look_at=(0.5, 0.0, 0.4), up=(0.0, 1.0, 0.0),
                            fov=50.0, aspect=width / height),
                render=dict(width=width, height=height, spp=spp, max_depth=max_depth,
                            miss_mode=MISS_SKY, miss_color=(0.0, 0.0, 0.0)))
        scenes.append(s)
    return scenes


def camera_basis(cam):
    """Pinhole camera of pkg/pt/camera.go:53-66 in float64: origin, lower-left corner, horizontal, vertical."""
    lf = np.asarray(cam["look_from"], np.float64)
    la = np.asarray(cam["look_at"], np.float64)
    up = np.asarray(cam["up"], np.float64)
    vh = 2.0 * np.tan(cam["fov"] * (np.pi / 180) / 2)
    vw = cam["aspect"] * vh
    w = lf - la
    w = w / np.sqrt(np.sum(w * w))
    u = np.cross(up, w)
    u = u / np.sqrt(np.sum(u * u))
    v = np.cross(w, u)
    hor, ver = u * vw, v * vh
    llc = lf - hor * 0.5 - ver * 0.5 - w
    return lf, llc, hor, ver


def camera_rays(cam, width, height, jitter_seed=None, tmin=0.001, tmax=np.inf, stride=1):
    """Deterministic primary rays (float32, 8 per ray: o, tmin, d, tmax) through
    pixel sample points u=(x+j)/(w-1), v=(y+j)/(h-1) (render.go:201-205), j=0.5 or seeded."""
    o, llc, hor, ver = camera_basis(cam)
    ys, xs = np.meshgrid(np.arange(0, height, stride), np.arange(0, width, stride), indexing="ij")
    xs, ys = xs.ravel().astype(np.float64), ys.ravel().astype(np.float64)
    if jitter_seed is None:
        jx = jy = 0.5
    else:
        rng = np.random.default_rng(jitter_seed)
        jx, jy = rng.random(xs.shape), rng.random(xs.shape)
    s = (xs + jx) / (width - 1)
    t = (ys + jy) / (height - 1)
    d = llc[None, :] + hor[None, :] * s[:, None] + ver[None, :] * t[:, None] - o[None, :]
    rays = np.empty((xs.shape[0], 8), np.float32)
    rays[:, 0:3] = o
    rays[:, 3] = tmin
    rays[:, 4:7] = d
    rays[:, 7] = tmax
    return rays
