"""The pair sort that allocates nothing (gbt_sort_morton_pairs_noalloc).

It serves callers that may not call cudaMalloc, such as a plugin whose host
application owns all device memory, or a per-frame loop that cannot take
cudaMalloc's implicit synchronisation.  Its output must equal the sorted
(Morton code, primitive index) pairs that gbt_lbvh_build produces, on two
calls in a row on the same static scratch.  This file is collected last (its
name sorts last) so that a failure here cannot hide earlier tests.
"""
import ctypes as C

import numpy as np
import pytest

from trace_gb300 import _lib, pt, scenes

pytestmark = pytest.mark.gpu

MAX_PAIRS = 262144  # GBT_NOALLOC_MAX_PAIRS in include/gbtrace.h


def reference_pairs(c, verts):
    """Sorted pairs from the allocating entry points, and the unsorted codes they came from."""
    ds = pt.DeviceScene(c, verts)
    g = pt.DefaultLBVH(ds)
    codes, idx = g.sorted_pairs()
    unsorted = np.empty_like(codes)
    unsorted[idx] = codes
    return codes, idx, unsorted


def run_noalloc(c, codes_in, stream=None):
    """One call on `stream` (a cudaStream_t handle; None is the default stream), or on the
    context's own non-blocking stream when stream is "ctx"."""
    n = codes_in.shape[0]
    d_in, d_out, d_idx = c.alloc(n * 8), c.alloc(n * 8), c.alloc(n * 4)
    try:
        c.h2d(d_in, codes_in)
        c.sync()
        st = c.stream if stream == "ctx" else stream
        rc = c.L.gbt_sort_morton_pairs_noalloc(st, C.c_void_p(d_in), C.c_void_p(d_out), C.c_void_p(d_idx), n)
        assert rc == 0, _lib.ERRORS.get(rc, rc)
        out = np.empty(n, np.uint64)
        idx = np.empty(n, np.int32)
        c.d2h(out, d_out)
        c.d2h(idx, d_idx)
        c.sync()
        return out, idx
    finally:
        for p in (d_in, d_out, d_idx):
            c.free(p)


def test_noalloc_sort_matches_lbvh_pairs_twice():
    c = pt.Context(0)
    try:
        # first call: 200k soup triangles (with duplicate codes to exercise the stable order)
        v1 = scenes.soup(150_000, seed=21)["verts"]
        v1 = np.concatenate([v1, v1[:50_000]])
        codes, idx, unsorted = reference_pairs(c, v1)
        got_c, got_i = run_noalloc(c, unsorted, "ctx")
        assert np.array_equal(got_c, codes)
        assert np.array_equal(got_i, idx)
        # second call in a row, a different and larger input (the maximum size): the
        # state the first call left in the shared scratch must not leak into this one
        v2 = scenes.terrain_tris(364, seed=5)[:MAX_PAIRS]
        codes2, idx2, unsorted2 = reference_pairs(c, v2)
        assert unsorted2.shape[0] == MAX_PAIRS
        got_c2, got_i2 = run_noalloc(c, unsorted2, "ctx")
        assert np.array_equal(got_c2, codes2)
        assert np.array_equal(got_i2, idx2)
        # the same input again on the default stream (NULL), and on the stream of a second
        # context (another non-blocking stream of this device)
        got_c3, got_i3 = run_noalloc(c, unsorted, None)
        assert np.array_equal(got_c3, codes) and np.array_equal(got_i3, idx)
        c2 = pt.Context(0)
        try:
            got_c4, got_i4 = run_noalloc(c2, unsorted2, "ctx")
            assert np.array_equal(got_c4, codes2) and np.array_equal(got_i4, idx2)
        finally:
            c2.close()
        # sizes beyond the static scratch are refused, not truncated
        d = c.alloc(8)
        try:
            rc = c.L.gbt_sort_morton_pairs_noalloc(c.stream, C.c_void_p(d), C.c_void_p(d), C.c_void_p(d), MAX_PAIRS + 1)
            assert rc == -1  # GBT_EINVAL
        finally:
            c.free(d)
    finally:
        c.close()
