"""Host-side checks of the C-ABI library (no GPU calls)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from trace_gb300 import _lib, pt, scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    hdr = open(os.path.join(ROOT, "include", "gbtrace.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    return sorted(set(re.findall(r"\b(gbt_[a-z0-9_]+)\s*\(", hdr)))


def test_library_exports_every_declared_symbol():
    L = C.CDLL(_lib.LIB_PATH)
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(L, s), s
    assert sorted(_lib.EXPORTS) == syms


CUBE = """# unit cube written for this test: quads with v/vt/vn and negative indices
v -0.5 -0.5 0.5
v 0.5 -0.5 0.5
v -0.5 0.5 0.5
v 0.5 0.5 0.5
v -0.5 0.5 -0.5
v 0.5 0.5 -0.5
v -0.5 -0.5 -0.5
v 0.5 -0.5 -0.5
vt 0 0
vn 0 0 1
vn 0 1 0
vn 0 0 -1
vn 0 -1 0
vn 1 0 0
vn -1 0 0
f 1/1/1 2/1/1 4/1/1 3/1/1
f 3/1/2 4/1/2 6/1/2 5/1/2
f 5/1/3 6/1/3 8/1/3 7/1/3
f -1/1/4 -2/1/4 2/1/4 1/1/4
f 2/1/5 8/1/5 6/1/5 4/1/5
f 7/1/6 1/1/6 3/1/6 5/1/6
"""


def test_obj_parse_fan_triangulation_and_negative_indices(tmp_path):
    p = tmp_path / "cube.obj"
    p.write_text(CUBE)
    g = pt.ParseFromPath(p)
    verts, normals = g.verts, (g.normals if g.has_normals else None)
    assert verts.shape == (12, 9)  # 6 quads, fan-triangulated (obj.go:193-203)
    assert normals is not None
    # first face: (v1, v2, v4), (v1, v4, v3)
    np.testing.assert_array_equal(verts[0], [-0.5, -0.5, 0.5, 0.5, -0.5, 0.5, 0.5, 0.5, 0.5])
    np.testing.assert_array_equal(verts[1], [-0.5, -0.5, 0.5, 0.5, 0.5, 0.5, -0.5, 0.5, 0.5])
    # -1 is the last vertex (8), -2 the one before (7) (obj.go:176-178)
    np.testing.assert_array_equal(verts[6, 0:3], [0.5, -0.5, -0.5])
    np.testing.assert_array_equal(verts[6, 3:6], [-0.5, -0.5, -0.5])
    np.testing.assert_array_equal(normals[0], [0, 0, 1] * 3)
    # every vertex on the unit cube
    assert np.all(np.abs(np.abs(verts) - 0.5) < 1e-7)


def test_reference_cube_obj():
    """The reference's own fixture (assets/cube.obj, copied to tests/golden/): 12 triangles
    with per-face normals (obj.go:19-140), checked against a direct reading of the file."""
    path = os.path.join(ROOT, "tests", "golden", "cube.obj")
    g = pt.ParseFromPath(path)
    assert g.has_normals
    v, vn, want_v, want_n = [None], [None], [], []
    for line in open(path):
        f = line.split()
        if not f:
            continue
        if f[0] == "v":
            v.append([float(x) for x in f[1:4]])
        elif f[0] == "vn":
            vn.append([float(x) for x in f[1:4]])
        elif f[0] == "f":
            idx = [tuple(int(k) for k in a.split("/")) for a in f[1:]]
            assert len(idx) == 3  # the fixture is all triangles
            want_v.append(sum((v[i[0]] for i in idx), []))
            want_n.append(sum((vn[i[2]] for i in idx), []))
    assert g.verts.shape == (12, 9)
    np.testing.assert_array_equal(g.verts, np.asarray(want_v, np.float32))
    np.testing.assert_array_equal(g.normals, np.asarray(want_n, np.float32))
    # each face's three normals agree and are axis-aligned unit vectors
    n3 = g.normals.reshape(12, 3, 3)
    assert np.all(n3 == n3[:, :1]) and np.all(np.abs(n3).sum(axis=2) == 1)


def test_obj_parse_without_normals_and_errors(tmp_path):
    p = tmp_path / "tri.obj"
    p.write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    g = pt.ParseFromPath(p)
    verts, normals = g.verts, (g.normals if g.has_normals else None)
    assert verts.shape == (1, 9) and normals is None
    bad = tmp_path / "bad.obj"
    bad.write_text("v 0 0 x\n")
    with pytest.raises(_lib.GbtError):
        pt.ParseFromPath(bad)
    with pytest.raises(_lib.GbtError):
        pt.ParseFromPath(tmp_path / "missing.obj")
    oob = tmp_path / "oob.obj"
    oob.write_text("v 0 0 0\nf 1 2 3\n")
    with pytest.raises(_lib.GbtError):
        pt.ParseFromPath(oob)


def test_scene_generators_sizes_and_determinism():
    c = scenes.cornell()
    assert c["verts"].shape == (972, 9)  # 10 walls + 2 light + 960 sphere
    assert scenes.cornell(256, 128)["verts"].shape[0] == 12 + 2 * 256 + 2 * 256 * 126
    a, b = scenes.soup(1000, seed=1), scenes.soup(1000, seed=1)
    assert np.array_equal(a["verts"], b["verts"])
    assert scenes.terrain_tris(9).shape == (2 * 8 * 8, 9)
    sz = scenes.batch_sizes()
    assert len(sz) == 64 and sz.min() >= 1000 and sz.max() <= 2_000_000


def test_header_compiles_as_c99(tmp_path):
    """include/gbtrace.h is what a cgo binding includes: it must be plain C."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "hdr.c"
    src.write_text('#include "gbtrace.h"\nint main(void) { gbt_ctx *c = 0; (void)c; return GBT_OK; }\n')
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
                        "-c", str(src), "-o", str(tmp_path / "hdr.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
