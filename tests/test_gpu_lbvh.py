"""GPU LBVH vs the oracle: Morton codes, sorted order and topology bit-exact."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import canonical_equal, first_mismatch
from trace_gb300 import pt, scenes

pytestmark = pytest.mark.gpu


def build_both(ctx, verts, spheres=None):
    ds = pt.DeviceScene(ctx, verts, spheres=spheres)
    g = pt.DefaultLBVH(ds)
    o = O.lbvh(verts, spheres)
    return ds, g, o


CASES = [
    ("cornell", lambda: scenes.cornell()["verts"]),
    ("soup_1", lambda: scenes.soup(1, seed=1)["verts"]),
    ("soup_2", lambda: scenes.soup(2, seed=1)["verts"]),
    ("soup_4095", lambda: scenes.soup(4095, seed=2)["verts"]),
    ("soup_4097", lambda: scenes.soup(4097, seed=3)["verts"]),
    ("soup_100k", lambda: scenes.soup(100_000, seed=4)["verts"]),
    ("terrain_257", lambda: scenes.terrain_tris(257, seed=2)),
    ("dups", lambda: np.concatenate([scenes.soup(3000, seed=5)["verts"]] * 3)),
    ("same_point", lambda: np.tile(np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0]], np.float32), (1000, 1))),
    ("flat", lambda: np.concatenate([scenes.terrain_tris(65, seed=3)[:, :]]) * np.array([1, 0, 1] * 3, np.float32)),
]


@pytest.mark.parametrize("name,make", CASES, ids=[c[0] for c in CASES])
def test_lbvh_bit_exact(ctx, name, make):
    verts = np.ascontiguousarray(make(), np.float32)
    ds, g, o = build_both(ctx, verts)
    n = verts.shape[0]
    gc, gi = g.sorted_pairs()
    oc, oi = o.sorted_pairs(n)
    assert np.array_equal(gc, oc), "Morton code sequence differs"
    assert np.array_equal(gi, oi), "sorted primitive order differs"
    ge, oe = g.export(), o.export()
    assert canonical_equal(ge, oe), first_mismatch(ge, oe)
    assert g.Size() == o.size()
    assert g.Cost() == o.cost()  # the same float64 operations in the same order


def test_lbvh_with_sphere(ctx):
    s = scenes.terrain(g=129, width=64, height=36)
    ds, g, o = build_both(ctx, s["verts"], s["spheres"])
    n = s["verts"].shape[0] + 1
    gc, gi = g.sorted_pairs()
    oc, oi = o.sorted_pairs(n)
    assert np.array_equal(gc, oc) and np.array_equal(gi, oi)
    gk, gn, gb, gp = g.export()
    ok, on, ob, op = o.export()
    assert np.array_equal(gk, ok) and np.array_equal(gn, on) and np.array_equal(gp, op)
    # boxes holding the sphere are float32-rounded outward from the float64 box
    assert np.all(gb[:, :3] <= ob[:, :3]) and np.all(gb[:, 3:] >= ob[:, 3:])
    np.testing.assert_allclose(gb, ob, rtol=1e-6, atol=1e-6)


def test_lbvh_1m_soup_properties(ctx):
    """Full-size soup: codes bit-exact vs the oracle, tree covers every primitive once."""
    s = scenes.soup(1_000_000, seed=1)
    ds, g, o = build_both(ctx, s["verts"])
    gc, gi = g.sorted_pairs()
    oc, oi = o.sorted_pairs(1_000_000)
    assert np.array_equal(gc, oc) and np.array_equal(gi, oi)
    ge, oe = g.export(), o.export()
    assert canonical_equal(ge, oe), first_mismatch(ge, oe)


def test_rebuild_in_place_is_identical(ctx):
    s = scenes.soup(50_000, seed=8)
    ds = pt.DeviceScene(ctx, s["verts"])
    g = pt.DefaultLBVH(ds)
    e1 = g.export()
    ctx.check(ctx.L.gbt_lbvh_rebuild_async(ctx.h, g.h), "rebuild")
    ctx.sync()
    assert canonical_equal(e1, g.export())


def test_context_closed_before_its_objects():
    """Closing a context first destroys its scenes and BVHs; later deletes are no-ops."""
    c = pt.Context(0)
    s = scenes.soup(1000, seed=2)
    ds = pt.DeviceScene.from_dict(c, s)
    g = pt.DefaultLBVH(ds)
    c.close()
    del g, ds
    import gc

    gc.collect()
