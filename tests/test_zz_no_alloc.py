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
SLICE = 65536


def _dev(torch, a):
    return torch.from_numpy(a).cuda()


def _call(L, d_bm, d_deg, V, d_out, stream=None):
    return L.gg_active_edges_noalloc(ctypes.c_void_p(d_bm.data_ptr()), ctypes.c_void_p(d_deg.data_ptr()), V,
                                     ctypes.c_void_p(d_out.data_ptr()), stream)


# several slices, not a multiple of 64; exactly one and two slices; one past a slice
@pytest.mark.parametrize("V", [200_003, SLICE, 2 * SLICE, 2 * SLICE + 1])
def test_noalloc_matches_active_edges_on_two_calls(V):
    torch = pytest.importorskip("torch")
    L = gg.library()
    rng = np.random.default_rng(V)
    src = rng.integers(0, V, 3 * V).astype(np.uint32)
    dst = rng.integers(0, V, 3 * V).astype(np.uint32)
    g = gg.Graph.from_edges(V, src, dst)
    deg = g.out_degree()
    d_deg = _dev(torch, deg.view(np.int32))
    words = V // 64 + 1
    side = torch.cuda.Stream()
    for trial in range(2):           # two calls in a row share the scratch array
        bm = rng.integers(0, 2 ** 63, words, dtype=np.uint64)
        if trial == 1:
            bm |= np.uint64(1) << np.uint64(63)   # bits past V must be ignored
        expected = g.active_edges(bm)
        d_bm = _dev(torch, bm.view(np.int64))
        d_out = torch.full((1,), -1, dtype=torch.int64, device="cuda")
        rc = _call(L, d_bm, d_deg, V, d_out)
        assert rc == 0, L.gg_last_error()
        assert int(d_out.item()) == expected
        # the same on a stream of the caller's (the call returns once it has finished)
        d_out2 = torch.full((1,), -1, dtype=torch.int64, device="cuda")
        torch.cuda.synchronize()
        rc = _call(L, d_bm, d_deg, V, d_out2, ctypes.c_void_p(side.cuda_stream))
        assert rc == 0, L.gg_last_error()
        assert int(d_out2.item()) == expected
    g.close()


def test_noalloc_zero_vertices_gives_zero():
    torch = pytest.importorskip("torch")
    L = gg.library()
    d_bm = torch.zeros(1, dtype=torch.int64, device="cuda")
    d_deg = torch.zeros(1, dtype=torch.int32, device="cuda")
    d_out = torch.full((1,), -1, dtype=torch.int64, device="cuda")
    assert _call(L, d_bm, d_deg, 0, d_out) == 0, L.gg_last_error()
    assert int(d_out.item()) == 0


def test_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    L = gg.library()
    d = torch.zeros(4, dtype=torch.int64, device="cuda")
    p = ctypes.c_void_p(d.data_ptr())
    assert L.gg_active_edges_noalloc(p, p, MAX_VERTICES + 1, p, None) == GG_ERR_LIMIT
    assert b"exceed" in L.gg_last_error()
