"""Failure paths with no GPU fault: a bounded wait that runs out, and a work list
that is full.  The reference panics on bad input (obj.go:13); here a call returns
an error code, nothing is written out of range, and the context stays usable.

  wait      GBT_OPT_TEST_WITHHOLD_TILE keeps one tile of the LBVH sort's first pass
            from publishing its digit counts: the tiles after it wait for a status
            nothing sets, give up after GBT_OPT_SPIN_LIMIT polls, and gbt_lbvh_build
            returns GBT_ETIMEOUT; the kernels after the sort do nothing.
  capacity  GBT_OPT_TEST_COLLAPSE_CAP caps the 4-wide collapse's work list: the
            children past it are dropped (never written), and gbt_lbvh_build
            returns GBT_EDEVICE with "work list full".
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import canonical_equal, first_mismatch
from trace_gb300 import _lib, pt, scenes

pytestmark = pytest.mark.gpu


def _expect_oracle_tree(ctx, verts):
    g = pt.DefaultLBVH(pt.DeviceScene(ctx, verts))
    ge, oe = g.export(), O.lbvh(verts).export()
    assert canonical_equal(ge, oe), first_mismatch(ge, oe)
    g.close()


def test_sort_wait_runs_out_and_reports_timeout():
    ctx = pt.Context(0)
    try:
        verts = scenes.soup(100_000, seed=31)["verts"]  # 25 tiles of 4096 keys per pass
        ds = pt.DeviceScene(ctx, verts)
        ctx.set_option("spin_limit", 256)
        ctx.set_option("test_withhold_tile", 3)
        with pytest.raises(_lib.GbtError) as e:
            pt.DefaultLBVH(ds)
        assert e.value.code == -4, e.value  # GBT_ETIMEOUT
        assert "bounded wait ran out" in str(e.value)
        # a lower limit than the default (about 4 ms of polling), with every tile
        # publishing, changes nothing
        ctx.set_option("test_withhold_tile", -1)
        ctx.set_option("spin_limit", 1 << 16)
        _expect_oracle_tree(ctx, verts)
        # and the context goes on: a second failure and a recovery
        ctx.set_option("spin_limit", 64)
        ctx.set_option("test_withhold_tile", 0)
        with pytest.raises(_lib.GbtError) as e:
            pt.DefaultLBVH(ds)
        assert e.value.code == -4
        ctx.set_option("test_withhold_tile", -1)
        ctx.set_option("spin_limit", 1 << 22)
        _expect_oracle_tree(ctx, verts)
    finally:
        ctx.close()


def test_collapse_work_list_full_reports_capacity():
    ctx = pt.Context(0)
    try:
        verts = scenes.soup(20_000, seed=32)["verts"]
        ds = pt.DeviceScene(ctx, verts)
        ctx.set_option("test_collapse_cap", 16)
        with pytest.raises(_lib.GbtError) as e:
            pt.DefaultLBVH(ds)
        assert e.value.code == -5, e.value  # GBT_EDEVICE
        assert "work list full" in str(e.value)
        ctx.set_option("test_collapse_cap", 0)
        _expect_oracle_tree(ctx, verts)
        # the 4-wide view built after the failure traces like the binary tree
        g = pt.DefaultLBVH(ds)
        rays = scenes.camera_rays(scenes.soup(20_000, seed=32)["camera"], 64, 64, jitter_seed=1)
        p4, t4, _, _ = g.trace(rays)
        g.set_layout(2)
        p2, t2, _, _ = g.trace(rays)
        assert np.array_equal(t4, t2)
    finally:
        ctx.close()


def test_option_ranges_are_checked(ctx):
    for name, bad in (("spin_limit", 0), ("spin_limit", (1 << 22) + 1), ("test_withhold_tile", -2),
                      ("test_collapse_cap", -1)):
        with pytest.raises(_lib.GbtError):
            ctx.set_option(name, bad)
