"""Batched multi-source BFS / SSSP: every lane must equal the single-root
toolkit run on the same root (BFS levels identical, parents a valid tree and
the same TEPS numerator; SSSP distances bit-identical)."""
import numpy as np
import pytest

import geminigraph_gb300 as gg
import graphgen
from golden_util import Fixture
from oracle.oracle import bfs_levels

pytestmark = pytest.mark.gpu


def graphs():
    s, d, w = graphgen.rmat(15, 16, 21, weighted=True)
    yield "rmat15", 1 << 15, s, d, w
    s, d, w = graphgen.grid(64, seed=3, weighted=True)
    yield "grid64", 64 * 64, s, d, w
    fx = Fixture("edgecase")
    yield "edgecase", fx.V, fx.src, fx.dst, fx.w


@pytest.fixture(scope="module", params=list(graphs()), ids=lambda p: p[0])
def case(request):
    name, V, s, d, w = request.param
    return V, s, d, w, gg.Graph.from_edges(V, s, d, w)


def roots_for(V, s, n, seed):
    deg = np.bincount(s, minlength=V)
    roots = gg.pick_roots(deg, n, seed)
    roots[1] = roots[0]                              # a duplicated root
    zero = np.nonzero(deg == 0)[0]
    if len(zero):
        roots[2] = int(zero[0])                      # a root with no out-edges
    return roots


@pytest.mark.parametrize("n", [1, 7, 64])
def test_bfs_batched_lanes_equal_single_runs(case, n):
    V, s, d, w, g = case
    roots = roots_for(V, s, max(n, 3), seed=n)[:n]
    lv, pa, reached, edges, st = gg.bfs_batched(g, roots, levels=True, parents=True)
    for i, r in enumerate(roots):
        parent, single = g.bfs(r)
        ref = bfs_levels(parent, r)
        assert np.array_equal(lv[i], ref), f"lane {i} root {r}"
        assert np.array_equal(bfs_levels(pa[i], r), ref)
        ok = pa[i] < V
        ok[r] = False
        src = pa[i][ok].astype(np.int64)
        dst = np.nonzero(ok)[0]
        have = set(zip(s.tolist(), d.tolist()))
        assert all((int(a), int(b)) in have for a, b in zip(src, dst))
        assert int(reached[i]) == int((parent < V).sum())
        assert int(edges[i]) == single.active_edges_total


@pytest.mark.parametrize("n", [1, 13, 64])
def test_sssp_batched_lanes_equal_single_runs(case, n):
    V, s, d, w, g = case
    roots = roots_for(V, s, max(n, 3), seed=100 + n)[:n]
    dist, reached, st = gg.sssp_batched(g, roots)
    for i, r in enumerate(roots):
        single, _ = g.sssp(r)
        assert np.array_equal(dist[i].view(np.uint32), single.view(np.uint32)), f"lane {i} root {r}"
        assert int(reached[i]) == int((single < np.float32(1e9)).sum())


@pytest.mark.parametrize("thread_lanes", [0, 64])
def test_sssp_batched_push_forms_agree(case, thread_lanes):
    """Warp-per-edge (0) and thread-per-edge (64: every step) relaxation give
    every lane the single-root distances bit for bit."""
    V, s, d, w, g = case
    g.set_batched_thread_lanes(thread_lanes)
    try:
        roots = roots_for(V, s, 20, seed=70)
        dist, reached, st = gg.sssp_batched(g, roots)
    finally:
        g.set_batched_thread_lanes(16)
    for i, r in enumerate(roots):
        single, _ = g.sssp(r)
        assert np.array_equal(dist[i].view(np.uint32), single.view(np.uint32)), f"lane {i} root {r}"
    with pytest.raises(gg.GeminiError):
        g.set_batched_thread_lanes(65)


def test_batched_argument_errors(case):
    V, s, d, w, g = case
    with pytest.raises(ValueError):
        gg.bfs_batched(g, list(range(65)))
    with pytest.raises(gg.GeminiError):
        gg.bfs_batched(g, [V])
    gu = gg.Graph.from_edges(V, s, d)
    with pytest.raises(gg.GeminiError):
        gg.sssp_batched(gu, [0])


@pytest.mark.parametrize("n", [1, 5, 64])
def test_bc_batched_lanes_equal_single_runs(case, n):
    """Every lane's dependencies and 1/num_paths equal the single-root BC
    (gg_bc) of its root: NaN / inf in the same places, path counts exact,
    dependencies within relative L1 1e-10 (sums in another order)."""
    V, s, d, w, g = case
    roots = roots_for(V, s, max(n, 3), seed=100 + n)[:n]
    dep, inv, reached, st = gg.bc_batched(g, roots)
    for i, r in enumerate(roots):
        sdep, sinv, _ = g.bc(r)
        assert np.array_equal(np.isnan(dep[i]), np.isnan(sdep)), f"lane {i} root {r}"
        assert np.array_equal(inv[i], sinv)
        ok = ~np.isnan(sdep)
        den = max(np.abs(sdep[ok]).sum(), 1e-300)
        assert np.abs(dep[i][ok] - sdep[ok]).sum() / den < 1e-10
        assert int(reached[i]) == int(np.isfinite(sinv).sum())
    assert st.calls >= 2


def test_bc_batched_rejects_bad_arguments(case):
    V, s, d, w, g = case
    with pytest.raises(gg.GeminiError):
        gg.bc_batched(g, [V])
    with pytest.raises((gg.GeminiError, ValueError)):
        gg.bc_batched(g, list(range(65)))


@pytest.mark.parametrize("delta", [0.0, 0.03, 0.5])
def test_sssp_batched_bucket_width_does_not_change_distances(case, delta):
    """Plain rounds (0) and distance buckets of any width reach the same
    distances, bit for bit, as the single-root SSSP."""
    V, s, d, w, g = case
    g.set_sssp_delta(delta)
    roots = roots_for(V, s, 9, seed=50)
    dist, reached, st = gg.sssp_batched(g, roots)
    for i, r in enumerate(roots):
        single, _ = g.sssp(r)
        assert np.array_equal(dist[i].view(np.uint32), single.view(np.uint32)), f"lane {i} root {r}"
    g.set_sssp_delta(0.0)
    with pytest.raises(gg.GeminiError):
        g.set_sssp_delta(-1.0)


@pytest.mark.parametrize("n", [3, 64])
def test_bfs_batched_levels_without_parents(case, n):
    """Without parents the dense steps write levels in a separate pass; every
    lane's levels still equal the single-root run's."""
    V, s, d, w, g = case
    roots = roots_for(V, s, max(n, 3), seed=200 + n)[:n]
    lv, pa, reached, edges, st = gg.bfs_batched(g, roots, levels=True, parents=False)
    assert pa is None
    for i, r in enumerate(roots):
        parent, single = g.bfs(r)
        assert np.array_equal(lv[i], bfs_levels(parent, r)), f"lane {i} root {r}"
        assert int(edges[i]) == single.active_edges_total


@pytest.mark.parametrize("divisor", [2, 160])
def test_bfs_batched_switch_point_keeps_levels(case, divisor):
    """Moving the batched sparse/dense switch changes which kernels run, not
    the levels or the reached counts."""
    V, s, d, w, g = case
    roots = roots_for(V, s, 16, seed=300 + divisor)
    ref = gg.bfs_batched(g, roots, levels=True, parents=False)
    g.set_batched_switch(divisor)
    try:
        lv, _, reached, _, _ = gg.bfs_batched(g, roots, levels=True, parents=True)
    finally:
        g.set_batched_switch(0)
    assert np.array_equal(lv, ref[0])
    assert np.array_equal(reached, ref[2])
