"""gg_active_edges_noalloc against gg_active_edges.

The no-allocation entry point serves callers that cannot let a library call
cudaMalloc (a serving process that owns all of HBM through its own pool, a
latency-critical caller that cannot take cudaMalloc's device
synchronisation): the caller passes device inputs and a device output, and
the only scratch is a fixed device array inside the library.  This file runs
last so that a failure here leaves every other test already run.
"""
import ctypes

import numpy as np
import pytest

import geminigraph_gb300 as gg

pytestmark = pytest.mark.gpu

GG_ERR_LIMIT = 8
MAX_VERTICES = 268435456


def _dev(torch, a):
    return torch.from_numpy(a).cuda()


def test_noalloc_matches_active_edges_on_two_calls():
    torch = pytest.importorskip("torch")
    L = gg.library()
    V = 200_003                      # several 65,536-vertex slices, not a multiple of 64
    rng = np.random.default_rng(5)
    src = rng.integers(0, V, 3 * V).astype(np.uint32)
    dst = rng.integers(0, V, 3 * V).astype(np.uint32)
    g = gg.Graph.from_edges(V, src, dst)
    deg = g.out_degree()
    d_deg = _dev(torch, deg.view(np.int32))
    words = V // 64 + 1
    for trial in range(2):           # two calls in a row share the scratch array
        bm = rng.integers(0, 2 ** 63, words, dtype=np.uint64)
        if trial == 1:
            bm |= np.uint64(1) << np.uint64(63)   # bits past V must be ignored
        expected = g.active_edges(bm)
        d_bm = _dev(torch, bm.view(np.int64))
        d_out = torch.full((1,), -1, dtype=torch.int64, device="cuda")
        rc = L.gg_active_edges_noalloc(ctypes.c_void_p(d_bm.data_ptr()), ctypes.c_void_p(d_deg.data_ptr()), V,
                                       ctypes.c_void_p(d_out.data_ptr()), None)
        assert rc == 0, L.gg_last_error()
        assert int(d_out.item()) == expected
    g.close()


def test_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    L = gg.library()
    d = torch.zeros(4, dtype=torch.int64, device="cuda")
    p = ctypes.c_void_p(d.data_ptr())
    assert L.gg_active_edges_noalloc(p, p, MAX_VERTICES + 1, p, None) == GG_ERR_LIMIT
    assert b"exceed" in L.gg_last_error()
