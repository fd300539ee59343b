"""Scene graph of pkg/pt (scene.go, primitive.go, transformation.go, math.go,
material.go) flattened into the arrays gbt_scene_upload takes.

The arithmetic follows the reference in float64 and in its operand order:
Matrix4.Multiply and MultiplyMatrix sum their four products left to right
(math.go:155-162, 299-325), a node's transformation composes as node x parent
(scene.go:101), Rotate builds the quaternion matrix (transformation.go:27-33,
math.go:341-352).  Quirks kept on purpose:
  - a node whose own transformation is the identity contributes its mesh
    untransformed, whatever its parents hold (scene.go:104-105);
  - normals are transformed as points (w = 1) by the inverse transpose and are
    not renormalised (primitive.go:152-170);
  - a sphere's centre is transformed, its radius is kept (primitive.go:42-50).
The upload puts all triangles first, then all spheres (primitive ids follow
that order); geometry is kept in arrays so that meshes of millions of
triangles flatten in vectorised numpy.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

DIFFUSE, LIGHT, REFLECTIVE, REFRACTIVE = 0, 1, 2, 3


# ---------------------------------------------------------------------------
# math.go / transformation.go
# ---------------------------------------------------------------------------
def NewVector3(x, y, z):
    return np.array([x, y, z], np.float64)


def NewColor(r, g, b):
    return (float(r), float(g), float(b))


def IdentityMatrix():
    return np.eye(4)


def Scale(x, y, z):
    return np.diag([float(x), float(y), float(z), 1.0])


def ScaleUniform(factor):
    return Scale(factor, factor, factor)


def Translate(x, y, z):
    m = np.eye(4)
    m[0, 3], m[1, 3], m[2, 3] = x, y, z
    return m


def Rotate(direction, angle):
    """Rotation by `angle` radians about `direction` through the unit quaternion."""
    d = np.asarray(direction, np.float64)
    u = d / math.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
    c, s = math.cos(angle / 2), math.sin(angle / 2)
    w, x, y, z = c, s * u[0], s * u[1], s * u[2]
    return np.array([
        [1 - 2 * y * y - 2 * z * z, 2 * x * y - 2 * z * w, 2 * x * z + 2 * y * w, 0],
        [2 * x * y + 2 * z * w, 1 - 2 * x * x - 2 * z * z, 2 * y * z - 2 * x * w, 0],
        [2 * x * z - 2 * y * w, 2 * y * z + 2 * x * w, 1 - 2 * x * x - 2 * y * y, 0],
        [0, 0, 0, 1]], np.float64)


def multiply_matrix(a, b):
    """a x b with each entry summed left to right."""
    out = np.empty((4, 4))
    for i in range(4):
        for j in range(4):
            out[i, j] = ((a[i, 0] * b[0, j] + a[i, 1] * b[1, j]) + a[i, 2] * b[2, j]) + a[i, 3] * b[3, j]
    return out


def transform_points(m, p, w=1.0):
    """Rows of p (n, 3) as (x, y, z, w) through m; the x, y, z of the result."""
    x, y, z = p[:, 0], p[:, 1], p[:, 2]
    return np.stack([((m[r, 0] * x + m[r, 1] * y) + m[r, 2] * z) + m[r, 3] * w for r in range(3)], axis=1)


# ---------------------------------------------------------------------------
# materials (material.go)
# ---------------------------------------------------------------------------
@dataclass(frozen=True)
class Diffuse:
    Albedo: tuple


@dataclass(frozen=True)
class Light:
    Color: tuple


@dataclass(frozen=True)
class Reflective:
    Albedo: tuple
    Diffusion: float = 0.0


@dataclass(frozen=True)
class Refractive:
    Albedo: tuple
    Ratio: float = 1.5


def _material_record(m):
    if isinstance(m, Diffuse):
        return DIFFUSE, m.Albedo, 0.0
    if isinstance(m, Light):
        return LIGHT, m.Color, 0.0
    if isinstance(m, Reflective):
        return REFLECTIVE, m.Albedo, float(m.Diffusion)
    if isinstance(m, Refractive):
        return REFRACTIVE, m.Albedo, float(m.Ratio)
    raise TypeError("only Diffuse, Light, Reflective and Refractive materials run on the device: %r" % (m,))


# ---------------------------------------------------------------------------
# primitives (primitive.go) and geometry
# ---------------------------------------------------------------------------
def _unit_rows(v):
    return v / np.sqrt(np.sum(v * v, axis=1, keepdims=True))


@dataclass
class Geometry:
    """A list of primitives held as arrays: triangle vertices (n, 9), per-vertex normals
    (n, 9) and spheres (m, 4) (center, radius)."""
    verts: np.ndarray = field(default_factory=lambda: np.zeros((0, 9)))
    normals: np.ndarray = field(default_factory=lambda: np.zeros((0, 9)))
    spheres: np.ndarray = field(default_factory=lambda: np.zeros((0, 4)))

    def __len__(self):
        return self.verts.shape[0] + self.spheres.shape[0]

    def append(self, prim):
        g = prim if isinstance(prim, Geometry) else prim.geometry()
        self.verts = np.concatenate([self.verts, g.verts])
        self.normals = np.concatenate([self.normals, g.normals])
        self.spheres = np.concatenate([self.spheres, g.spheres])
        return self

    def __add__(self, other):
        return Geometry(self.verts, self.normals, self.spheres).append(other)


def triangles_without_normals(verts):
    """NewTriangleWithoutNormals (primitive.go:116-132) over rows of (v0, v1, v2):
    each vertex normal is (right - p) x (left - p), normalised (calcNormal)."""
    v = np.asarray(verts, np.float64).reshape(-1, 3, 3)
    out = np.empty_like(v)
    for k in range(3):
        p, right, left = v[:, k], v[:, (k + 1) % 3], v[:, (k + 2) % 3]
        out[:, k] = _unit_rows(np.cross(right - p, left - p))
    return Geometry(v.reshape(-1, 9), out.reshape(-1, 9), np.zeros((0, 4)))


def NewTriangleWithoutNormals(v0, v1, v2):
    return triangles_without_normals(np.concatenate([v0, v1, v2]).reshape(1, 9))


def NewTriangle(positions, normals):
    """NewTriangle (primitive.go:102-114) from three positions and three vertex normals."""
    return Geometry(np.asarray(positions, np.float64).reshape(1, 9), np.asarray(normals, np.float64).reshape(1, 9),
                    np.zeros((0, 4)))


def NewSphere(center, radius):
    c = np.asarray(center, np.float64)
    return Geometry(np.zeros((0, 9)), np.zeros((0, 9)), np.array([[c[0], c[1], c[2], float(radius)]]))


# ---------------------------------------------------------------------------
# scene graph (scene.go)
# ---------------------------------------------------------------------------
@dataclass
class Mesh:
    geometry: Geometry
    material: object

    def raw(self):
        return self.geometry

    def Transformed(self, t):
        g = self.geometry
        tinv = np.linalg.inv(t.T)
        v = transform_points(t, g.verts.reshape(-1, 3)).reshape(-1, 9)
        n = transform_points(tinv, g.normals.reshape(-1, 3)).reshape(-1, 9)
        s = g.spheres.copy()
        if s.shape[0]:
            s[:, :3] = transform_points(t, g.spheres[:, :3])
        return Geometry(v, n, s)


def NewMesh(geometry, material):
    return Mesh(geometry, material)


class SceneNode:
    def __init__(self, mesh=None):
        self.transformation = IdentityMatrix()
        self.children = []
        self.mesh = mesh

    def Add(self, node):
        self.children.append(node)

    def transform(self, t):
        self.transformation = multiply_matrix(self.transformation, t)

    def ScaleUniform(self, factor):
        self.transform(ScaleUniform(factor))

    def Scale(self, x, y, z):
        self.transform(Scale(x, y, z))

    def Translate(self, x, y, z):
        self.transform(Translate(x, y, z))

    def Rotate(self, direction, angle):
        self.transform(Rotate(direction, angle))

    def SetTransformation(self, t):
        self.transformation = np.asarray(t, np.float64).reshape(4, 4)

    def ResetTransformation(self):
        self.transformation = IdentityMatrix()

    def collect(self, t, out):
        """collectTracables (scene.go:99-114): (geometry, material) pairs in scene order."""
        t = multiply_matrix(self.transformation, t)
        if self.mesh is not None:
            if np.array_equal(self.transformation, IdentityMatrix()):
                out.append((self.mesh.raw(), self.mesh.material))
            else:
                out.append((self.mesh.Transformed(t), self.mesh.material))
        for c in self.children:
            c.collect(t, out)
        return out

    def collect_raw(self, out):
        if self.mesh is not None:
            out.append((self.mesh.raw(), self.mesh.material))
        for c in self.children:
            c.collect_raw(out)
        return out


def NewSceneNode(mesh=None):
    return SceneNode(mesh)


def flatten(parts):
    """(geometry, material) pairs -> the arrays of gbt_scene_upload: triangles of every part
    first, then spheres; one material entry per distinct material."""
    mats, index = [], {}
    verts, normals, spheres, tri_mat, sph_mat = [], [], [], [], []
    for g, m in parts:
        if m not in index:
            index[m] = len(mats)
            mats.append(_material_record(m))
        k = index[m]
        verts.append(g.verts)
        normals.append(g.normals)
        spheres.append(g.spheres)
        tri_mat.append(np.full(g.verts.shape[0], k, np.int32))
        sph_mat.append(np.full(g.spheres.shape[0], k, np.int32))
    cat = lambda a, shape: np.concatenate(a) if a else np.zeros(shape)
    return dict(
        verts=cat(verts, (0, 9)).astype(np.float32),
        normals=cat(normals, (0, 9)).astype(np.float32),
        spheres=cat(spheres, (0, 4)).astype(np.float32),
        prim_mat=np.concatenate(tri_mat + sph_mat).astype(np.int32) if parts else np.zeros(0, np.int32),
        mat_type=np.array([r[0] for r in mats], np.int32),
        mat_color=np.array([r[1] for r in mats], np.float64).reshape(-1, 3),
        mat_param=np.array([r[2] for r in mats], np.float64),
    )
