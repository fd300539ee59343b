"""A scene graph (scene.go) compiled on the device: Compile / CompileLBVH / CompilePHR trace
the flattened, transformed geometry."""
import math

import numpy as np
import pytest

from trace_gb300 import pt, scenes
from trace_gb300 import scenegraph as sg

pytestmark = pytest.mark.gpu


def build_scene():
    s = pt.NewScene()
    quad = pt.NewTriangleWithoutNormals(pt.NewVector3(-1, -1, 0), pt.NewVector3(1, -1, 0), pt.NewVector3(1, 1, 0)) + \
        pt.NewTriangleWithoutNormals(pt.NewVector3(-1, -1, 0), pt.NewVector3(1, 1, 0), pt.NewVector3(-1, 1, 0))
    wall = pt.NewSceneNode(pt.NewMesh(quad, pt.Diffuse((0.7, 0.7, 0.7))))
    wall.Translate(0, 0, -5)            # a quad at z = -5
    ball = pt.NewSceneNode(pt.NewMesh(pt.NewSphere(pt.NewVector3(0, 0, 0), 0.5), pt.Light((3.0, 3.0, 3.0))))
    ball.Translate(2, 0, -3)            # a sphere centred at (2, 0, -3)
    tilted = pt.NewSceneNode(pt.NewMesh(sg.triangles_without_normals(scenes.uv_sphere([0, 0, 0], 0.4, 16, 8)),
                                        pt.Refractive((0.9, 0.9, 0.9), 1.5)))
    # node x t composition: the transform added last acts on the points first (rotate, then move)
    tilted.Translate(-2, 0, -3)
    tilted.Rotate(pt.NewVector3(1, 0, 0), math.pi / 3)   # a tilted glass ball at (-2, 0, -3)
    for n in (wall, ball, tilted):
        s.Add(n)
    return s


@pytest.mark.parametrize("how", ["lbvh", "default", "phr4"])
def test_compiled_scene_traces_transformed_geometry(ctx, how):
    s = build_scene()
    g = s.CompileLBVH(ctx) if how == "lbvh" else (s.Compile(ctx) if how == "default" else s.CompilePHR(ctx, 0.55, 9, 4))
    rays = np.array([[0, 0, 0, 1e-3, 0, 0, -1, np.inf],      # the quad at t = 5
                     [2, 0, 0, 1e-3, 0, 0, -1, np.inf],      # the sphere's near side at t = 2.5
                     [-2, 0, 0, 1e-3, 0, 0, -1, np.inf],     # the glass ball at about t = 2.6
                     [0, 5, 0, 1e-3, 0, 1, 0, np.inf]], np.float32)  # nothing
    prim, t, _, _ = g.trace(rays)
    d = s.tracables()
    n_tri = d["verts"].shape[0]
    assert t[0] == pytest.approx(5.0, rel=1e-6) and prim[0] in (0, 1)
    assert prim[1] == n_tri and t[1] == pytest.approx(2.5, rel=1e-6)   # spheres come after the triangles
    assert 2 <= prim[2] < n_tri and 2.55 < t[2] < 2.65
    assert prim[3] == -1
