"""Scene graph (scene.go, transformation.go, primitive.go:102-170) flattened for upload:
composition order, the identity-node and w = 1 normal quirks, spheres, material table."""
import math

import numpy as np

from trace_gb300 import pt
from trace_gb300 import scenegraph as sg


def tri():
    return pt.NewTriangleWithoutNormals(pt.NewVector3(0, 0, 0), pt.NewVector3(1, 0, 0), pt.NewVector3(0, 1, 0))


def test_without_normals_is_calc_normal():
    g = tri()
    np.testing.assert_array_equal(g.normals, [[0, 0, 1] * 3])
    g2 = sg.triangles_without_normals(np.array([[0, 0, 0, 0, 0, 2, 0, 3, 0]], np.float64))
    np.testing.assert_allclose(g2.normals, [[-1, 0, 0] * 3])


def test_translate_then_scale_composes_node_times_parent():
    s = pt.NewScene()
    parent = pt.NewSceneNode(None)
    parent.Translate(10, 0, 0)
    child = pt.NewSceneNode(pt.NewMesh(tri(), pt.Diffuse((0.5, 0.5, 0.5))))
    child.ScaleUniform(2.0)
    parent.Add(child)
    s.Add(parent)
    d = s.tracables()
    # t = child x parent: a point is scaled by 2 first... in the row-vector reading of
    # Multiply(child x parent) the parent's translation is applied to the scaled point
    want = sg.multiply_matrix(sg.ScaleUniform(2.0), sg.Translate(10, 0, 0))
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float64)
    np.testing.assert_allclose(d["verts"].reshape(3, 3), sg.transform_points(want, v))
    np.testing.assert_allclose(d["verts"].reshape(3, 3), [[20, 0, 0], [22, 0, 0], [20, 2, 0]])
    # normals through the inverse transpose as points: scale 2 halves them (not renormalised)
    np.testing.assert_allclose(d["normals"].reshape(3, 3), [[0, 0, 0.5]] * 3)


def test_identity_node_ignores_parent_transform():
    """scene.go:104-105: a mesh on a node whose own transformation is the identity is added raw."""
    s = pt.NewScene()
    parent = pt.NewSceneNode(pt.NewMesh(tri(), pt.Diffuse((0.5, 0.5, 0.5))))
    parent.Translate(0, 0, 5)
    child = pt.NewSceneNode(pt.NewMesh(tri(), pt.Light((4.0, 4.0, 4.0))))
    parent.Add(child)
    s.Add(parent)
    d = s.tracables()
    np.testing.assert_allclose(d["verts"][0].reshape(3, 3)[:, 2], [5, 5, 5])  # parent's mesh moved
    np.testing.assert_allclose(d["verts"][1].reshape(3, 3)[:, 2], [0, 0, 0])  # child's mesh raw
    assert d["prim_mat"].tolist() == [0, 1] and d["mat_type"].tolist() == [pt.DIFFUSE, pt.LIGHT]


def test_rotation_quaternion_and_spheres_last():
    s = pt.NewScene()
    n = pt.NewSceneNode(pt.NewMesh(pt.NewSphere(pt.NewVector3(1, 0, 0), 0.25) + tri(), pt.Reflective((0.8,) * 3, 0.1)))
    n.Rotate(pt.NewVector3(0, 0, 1), math.pi / 2)  # x -> y
    s.Add(n)
    s.Add(pt.NewSceneNode(pt.NewMesh(tri(), pt.Reflective((0.8,) * 3, 0.1))))  # same material: one entry
    d = s.tracables()
    assert d["verts"].shape == (2, 9) and d["spheres"].shape == (1, 4)
    np.testing.assert_allclose(d["spheres"][0], [0, 1, 0, 0.25], atol=1e-7)
    np.testing.assert_allclose(d["verts"][0].reshape(3, 3), [[0, 0, 0], [0, 1, 0], [-1, 0, 0]], atol=1e-7)
    assert d["prim_mat"].tolist() == [0, 0, 0] and d["mat_param"].tolist() == [0.1]
    raw = s.UntransformedTracables()
    np.testing.assert_allclose(raw["spheres"][0], [1, 0, 0, 0.25])


def test_translation_leaves_normals():
    s = pt.NewScene()
    n = pt.NewSceneNode(pt.NewMesh(tri(), pt.Diffuse((0.5,) * 3)))
    n.Translate(3, -2, 7)
    s.Add(n)
    d = s.tracables()
    np.testing.assert_allclose(d["normals"].reshape(3, 3), [[0, 0, 1]] * 3)
    np.testing.assert_allclose(d["verts"].reshape(3, 3)[0], [3, -2, 7])
