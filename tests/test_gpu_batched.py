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


def device_driven(g, fn):
    """fn() with the batched steps device-driven (one CUDA-graph launch)."""
    g.set_batched_graph(True)
    try:
        return fn()
    finally:
        g.set_batched_graph(False)


@pytest.mark.parametrize("parents", [False, True])
def test_bfs_batched_device_driven_equals_host_steps(case, parents):
    """Device-driven steps (one CUDA-graph launch per batch, push or pull
    picked on the device) give the levels, per-lane counts and per-step trace
    of host-driven steps; parents stay valid trees with the same levels."""
    V, s, d, w, g = case
    roots = roots_for(V, s, 64, seed=400)
    dev = device_driven(g, lambda: gg.bfs_batched(g, roots, levels=True, parents=parents))
    host = gg.bfs_batched(g, roots, levels=True, parents=parents)
    # asked for per-step kernel times, the steps run from the host
    timed = device_driven(g, lambda: gg.bfs_batched(g, roots, levels=True, parents=parents, timing=True))
    for other in (host, timed):
        assert np.array_equal(dev[0], other[0])
        assert np.array_equal(dev[2], other[2])
        assert np.array_equal(dev[3], other[3])
        assert dev[4].rows() == other[4].rows()
    if parents:
        for i, r in enumerate(roots):
            assert np.array_equal(bfs_levels(dev[1][i], r), dev[0][i])
    assert dev[4].kernel_launches > 0


@pytest.mark.parametrize("thread_lanes", [0, 16, 64])
def test_sssp_batched_device_driven_equals_host_steps(case, thread_lanes):
    """The same distances and reached counts for batched SSSP, with each
    relaxation form (thread per edge up to thread_lanes lanes in flight, warp
    per edge above)."""
    V, s, d, w, g = case
    g.set_batched_thread_lanes(thread_lanes)
    try:
        roots = roots_for(V, s, 40, seed=500 + thread_lanes)
        dev = device_driven(g, lambda: gg.sssp_batched(g, roots))
        host = gg.sssp_batched(g, roots)
    finally:
        g.set_batched_thread_lanes(16)
    assert np.array_equal(dev[0].view(np.uint32), host[0].view(np.uint32))
    assert np.array_equal(dev[1], host[1])
    # a step relaxes from distances as other threads of the same step leave
    # them, so how many vertices each step lowers varies from run to run (the
    # fixpoint does not); the first step's row is fixed by the roots
    assert dev[2].rows()[0] == host[2].rows()[0]


def test_batched_device_driven_over_many_launches():
    """On the 1024 x 1024 grid a corner root is 2,046 levels deep: the
    device-driven loop runs 1,024 steps per launch, so the batch takes several
    launches, the state carried between them through the host."""
    g = gg.Graph.generate(gg.GRID, 1024, 0, 1, weighted=True)
    try:
        n = 1024
        roots = [0, n * n - 1, n * (n // 2) + n // 2, 5]
        dev = device_driven(g, lambda: gg.bfs_batched(g, roots, levels=True))
        host = gg.bfs_batched(g, roots, levels=True)
        assert np.array_equal(dev[0], host[0])
        assert dev[4].rows() == host[4].rows()
        assert len(dev[4].rows()) == 2 * (n - 1) + 1 > 1024
        assert int(dev[0][0].max()) == 2 * (n - 1)
        ddist = device_driven(g, lambda: gg.sssp_batched(g, roots))
        hdist = gg.sssp_batched(g, roots)
        assert np.array_equal(ddist[0].view(np.uint32), hdist[0].view(np.uint32))
        assert ddist[2].calls > 1024
    finally:
        g.close()


@pytest.mark.parametrize("n", [5, 64])
def test_bfs_batched_level_lists_equal_rows(case, n):
    """Levels kept as level lists (the default without parents) and as
    per-vertex rows give the same levels, reached counts, TEPS numerators
    and per-step trace.  On graphs this small a step's worst-case room (two
    entries per vertex plus a slot range per warp) exceeds 16 entries per
    vertex, so the lists move into the rows at the first step: this covers
    that hand-over; test_gpu_configs.py covers lists kept to the end."""
    V, s, d, w, g = case
    roots = roots_for(V, s, max(n, 3), seed=600 + n)[:n]
    lists = gg.bfs_batched(g, roots, levels=True)
    g.set_batched_lists(False)
    try:
        rows = gg.bfs_batched(g, roots, levels=True)
    finally:
        g.set_batched_lists(True)
    assert np.array_equal(lists[0], rows[0])
    assert np.array_equal(lists[2], rows[2]) and np.array_equal(lists[3], rows[3])
    assert lists[4].rows() == rows[4].rows()
    # without levels asked for, the counts come from the lists alone
    bare = gg.bfs_batched(g, roots, levels=False)
    assert np.array_equal(bare[2], rows[2]) and np.array_equal(bare[3], rows[3])


def test_bfs_batched_level_lists_move_into_rows():
    """On a path with 64 roots spread along it, lanes reach most vertices at
    up to 64 different steps; the lists move into the rows and every lane
    still has its single-root levels over the 2,000-odd steps."""
    V = 4000
    a = np.arange(V - 1, dtype=np.uint32)
    s = np.concatenate([a, a + 1])
    d = np.concatenate([a + 1, a])
    g = gg.Graph.from_edges(V, s, d)
    try:
        roots = [int(x) for x in np.linspace(0, V - 1, 64).astype(np.int64)]
        lv, _, reached, edges, st = gg.bfs_batched(g, roots, levels=True)
        for i, r in enumerate(roots):
            parent, single = g.bfs(r)
            assert np.array_equal(lv[i], bfs_levels(parent, r)), f"lane {i} root {r}"
            assert int(reached[i]) == V and int(edges[i]) == single.active_edges_total
        assert st.calls > 2000
    finally:
        g.close()
