"""GPU parity: the CUDA engine against the CPU oracle (itself pinned to the
reference's outputs) and against the reference fixtures directly.

Bars (the reference's own determinism, measured): CC labels, SSSP float
distances and BFS levels bit-exact; BFS parents a valid tree; PageRank and BC
(double) within relative L1 1e-10 of the oracle (the tolerance the
comparison states; the float PageRank variant within 1e-5).  The per-call
trace -- mode, active_edges, activated -- must equal the oracle's exactly:
that pins the sparse/dense switch (core/graph.hpp:1503-1509).
"""
import os
import tempfile

import numpy as np
import pytest

import geminigraph_gb300 as gg
import graphgen
from golden_util import Fixture, names
from oracle.oracle import OracleGraph, bfs_levels

pytestmark = pytest.mark.gpu

PR_TOL = 1e-10
PR_F32_TOL = 1e-5
BC_TOL = 1e-10


def rel_l1(a, b):
    return float(np.abs(a - b).sum() / max(np.abs(b).sum(), 1e-300))


def check_parent_tree(parent, root, V, src, dst):
    lv = bfs_levels(parent, root)
    reached = np.nonzero(parent < V)[0]
    edges = set(zip(src.tolist(), dst.tolist()))
    for v in reached:
        if v != root:
            assert (int(parent[v]), int(v)) in edges
    return lv


def random_graph(V, E, seed, selfloops=True):
    rng = np.random.default_rng(seed)
    s = rng.integers(0, V, E).astype(np.uint32)
    d = rng.integers(0, V, E).astype(np.uint32)
    if not selfloops:
        d = np.where(d == s, (d + 1) % V, d).astype(np.uint32)
    w = graphgen.weights(seed, np.arange(E, dtype=np.uint64))
    return s, d, w


CASES = {}


def case(name):
    if name in CASES:
        return CASES[name]
    if name.startswith("golden:"):
        fx = Fixture(name.split(":")[1])
        c = (fx.V, fx.src, fx.dst, fx.w, fx.root)
    elif name == "rmat16":
        s, d, w = graphgen.rmat(16, 16, 3, weighted=True)
        c = (1 << 16, s, d, w, None)
    elif name == "grid128":
        s, d, w = graphgen.grid(128, seed=2, weighted=True)
        c = (128 * 128, s, d, w, 0)
    elif name == "random_odd":
        s, d, w = random_graph(777, 5000, 11)
        c = (777, s, d, w, None)
    elif name == "chain":
        V = 300
        s = np.arange(V - 1, dtype=np.uint32)
        d = s + 1
        w = np.full(V - 1, 0.5, np.float32)
        c = (V, s, d, w, 0)
    elif name == "star":
        V = 5000
        s = np.zeros(V - 1, np.uint32)
        d = np.arange(1, V, dtype=np.uint32)
        s = np.concatenate([s, d[:100]])
        d = np.concatenate([d, np.zeros(100, np.uint32)])
        w = graphgen.weights(4, np.arange(len(s), dtype=np.uint64))
        c = (V, s.astype(np.uint32), d.astype(np.uint32), w, 0)
    else:
        raise KeyError(name)
    V, s, d, w, root = c
    if root is None:
        root = graphgen.pick_root(s, V, seed=V)
    CASES[name] = (V, s, d, w, root)
    return CASES[name]


ALL = ["golden:" + n for n in names()] + ["rmat16", "grid128", "random_odd", "chain", "star"]


@pytest.fixture(scope="module", params=ALL)
def gcase(request):
    return request.param, case(request.param)


def test_adjacency_matches_oracle(gcase):
    _, (V, s, d, w, _) = gcase
    for symmetric in (False, True):
        g = gg.Graph.from_edges(V, s, d, w, symmetric=symmetric)
        o = OracleGraph(V, s, d, w, symmetric=symmetric)
        for incoming in (False, True):
            go, gn, gw, gd = g.adjacency(incoming)
            oo, on, ow, od = o.adjacency(incoming)
            assert np.array_equal(go, oo)
            assert np.array_equal(gn, on)
            assert np.array_equal(gw.view(np.uint32), ow.view(np.uint32))
            assert np.array_equal(gd, od)
        info = g.info()
        assert info["edges"] == len(s)
        assert info["adj_entries"] == (2 if symmetric else 1) * len(s)


def test_bfs(gcase):
    name, (V, s, d, w, root) = gcase
    g = gg.Graph.from_edges(V, s, d)
    parent, st = g.bfs(root)
    o = OracleGraph(V, s, d)
    oparent, otrace = o.bfs(root)
    assert st.rows() == otrace
    lv = check_parent_tree(parent, root, V, s, d)
    assert np.array_equal(lv, bfs_levels(oparent, root))
    assert st.active_edges_total == sum(r[1] for r in otrace)
    if name.startswith("golden:"):
        fx = Fixture(name.split(":")[1])
        assert np.array_equal(lv, bfs_levels(fx["bfs_parent"], root))


def test_pagerank(gcase):
    name, (V, s, d, w, _) = gcase
    g = gg.Graph.from_edges(V, s, d)
    ranks, deltas, st = g.pagerank(20)
    o = OracleGraph(V, s, d)
    oranks, odeltas, otrace = o.pagerank(20)
    assert rel_l1(ranks, oranks) < PR_TOL
    assert np.allclose(deltas, odeltas, rtol=1e-9, atol=1e-15)
    assert st.rows() == otrace
    r32, _, _ = g.pagerank(20, f32=True)
    assert rel_l1(r32.astype(np.float64), oranks) < PR_F32_TOL
    if name.startswith("golden:"):
        fx = Fixture(name.split(":")[1])
        assert rel_l1(ranks, fx["pr_ranks"]) < PR_TOL


def test_cc(gcase):
    name, (V, s, d, w, _) = gcase
    g = gg.Graph.from_edges(V, s, d, symmetric=True)
    label, st = g.cc()
    o = OracleGraph(V, s, d, symmetric=True)
    olabel, otrace = o.cc()
    assert np.array_equal(label, olabel)
    assert st.rows() == otrace
    if name.startswith("golden:"):
        assert np.array_equal(label, Fixture(name.split(":")[1])["cc_label"])


def test_sssp(gcase):
    name, (V, s, d, w, root) = gcase
    g = gg.Graph.from_edges(V, s, d, w)
    dist, st = g.sssp(root)
    o = OracleGraph(V, s, d, w)
    odist, otrace = o.sssp(root)
    assert np.array_equal(dist.view(np.uint32), odist.view(np.uint32))
    assert st.rows() == otrace
    if name.startswith("golden:"):
        ref = Fixture(name.split(":")[1])["sssp_dist"]
        assert np.array_equal(dist.view(np.uint32), ref.view(np.uint32))


def test_bc(gcase):
    name, (V, s, d, w, root) = gcase
    g = gg.Graph.from_edges(V, s, d)
    dep, inv, st = g.bc(root)
    o = OracleGraph(V, s, d)
    odep, oinv, otrace = o.bc(root)
    assert np.array_equal(np.isnan(dep), np.isnan(odep))
    assert np.array_equal(inv, oinv)
    ok = ~np.isnan(odep)
    assert rel_l1(dep[ok], odep[ok]) < BC_TOL
    assert [r[:2] for r in st.rows()] == [r[:2] for r in otrace]
    if name.startswith("golden:"):
        fx = Fixture(name.split(":")[1])
        assert np.array_equal(np.isnan(dep), np.isnan(fx["bc_dep"]))
        assert rel_l1(dep[ok], fx["bc_dep"][ok]) < BC_TOL


def test_file_load_matches_records(tmp_path):
    V, s, d, w, root = case("golden:edgecase")
    rec = graphgen.to_records(s, d, w) + b"\x01\x02\x03"   # trailing partial record ignored
    p = tmp_path / "g.wbin"
    p.write_bytes(rec)
    g1 = gg.Graph.load(str(p), V, weighted=True)
    g2 = gg.Graph.from_edges(V, s, d, w)
    assert g1.info()["edges"] == len(s)
    for incoming in (False, True):
        a, b = g1.adjacency(incoming), g2.adjacency(incoming)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


def test_device_generator_matches_host():
    for kind, p1, p2, wtd in ((gg.RMAT, 12, 8, True), (gg.GRID, 40, 0, True), (gg.RMAT, 10, 16, False)):
        gd = gg.Graph.generate(kind, p1, p2, 9, weighted=wtd)
        rec = gg.generate_records(kind, p1, p2, 9, weighted=wtd)
        V = (1 << p1) if kind == gg.RMAT else p1 * p1
        gh = gg.Graph.from_records(rec, V, weighted=wtd)
        for incoming in (False, True):
            a, b = gd.adjacency(incoming), gh.adjacency(incoming)
            for x, y in zip(a, b):
                if x is not None:
                    assert np.array_equal(x, y)


def test_errors():
    with pytest.raises(gg.GeminiError) as e:
        gg.Graph.from_edges(10, np.array([1, 12], np.uint32), np.array([2, 3], np.uint32))
    assert e.value.code == 3
    g = gg.Graph.from_edges(10, np.array([1, 2], np.uint32), np.array([2, 3], np.uint32))
    with pytest.raises(gg.GeminiError) as e:
        g.bfs(10)
    assert e.value.code == 1
    with pytest.raises(gg.GeminiError) as e:
        g.sssp(0)
    assert e.value.code == 6
    with pytest.raises(gg.GeminiError) as e:
        gg.Graph.load("/nonexistent/g.bin", 10)
    assert e.value.code == 2


def test_empty_and_isolated():
    # no edges at all: every toolkit terminates after one call
    g = gg.Graph.from_edges(70, np.zeros(0, np.uint32), np.zeros(0, np.uint32), np.zeros(0, np.float32))
    parent, st = g.bfs(5)
    assert parent[5] == 5 and (parent == 70).sum() == 69
    assert st.calls == 1
    dist, _ = g.sssp(3)
    assert dist[3] == 0 and (dist == np.float32(1e9)).sum() == 69
    ranks, _, _ = g.pagerank(3)
    assert np.allclose(ranks, 0.15)
    dep, inv, _ = g.bc(1)
    assert inv[1] == 1.0 and np.isinf(inv).sum() == 69
    gs = gg.Graph.from_edges(70, np.zeros(0, np.uint32), np.zeros(0, np.uint32), symmetric=True)
    label, _ = gs.cc()
    assert np.array_equal(label, np.arange(70))


def test_transpose_roundtrip():
    V, s, d, w, root = case("rmat16")
    g = gg.Graph.from_edges(V, s, d)
    out0 = g.adjacency(False)
    g.transpose()
    assert np.array_equal(g.adjacency(True)[1], out0[1])
    # BFS on the transposed graph follows in-edges
    parent, _ = g.bfs(root)
    o = OracleGraph(V, d, s)
    op, _ = o.bfs(root)
    assert np.array_equal(bfs_levels(parent, root), bfs_levels(op, root))
    g.transpose()
    assert g.info()["transposed"] == 0


def test_active_edges_primitive():
    V, s, d, w, _ = case("random_odd")
    g = gg.Graph.from_edges(V, s, d)
    rng = np.random.default_rng(0)
    words = V // 64 + 1
    bm = rng.integers(0, 2 ** 63, words, dtype=np.uint64) | (rng.integers(0, 2, words, dtype=np.uint64) << 63)
    bits = np.unpackbits(bm.view(np.uint8), bitorder="little")[:V].astype(bool)
    deg = np.bincount(s, minlength=V)
    assert g.active_edges(bm) == int(deg[bits].sum())


def test_repeated_runs_are_stable():
    V, s, d, w, root = case("rmat16")
    g = gg.Graph.from_edges(V, s, d, w)
    d1, _ = g.sssp(root)
    g.bfs(root)
    d2, _ = g.sssp(root)
    assert np.array_equal(d1.view(np.uint32), d2.view(np.uint32))


def test_bfs_dense_parent_is_first_active_in_csc_order():
    # hub 0 has in-edges from every other vertex (5 heavy chunks); the dense
    # call must pick the smallest active in-neighbour (bfs.cpp:63-66 with the
    # CSC sorted by source id), which sits in the third chunk
    V = 10000
    s = list(range(1, V - 1)) + [9999] * 1000 + list(range(5000, 6000))
    d = [0] * (V - 2) + list(range(5000, 6000)) + [0] * 1000
    s, d = np.array(s, np.uint32), np.array(d, np.uint32)
    g = gg.Graph.from_edges(V, s, d)
    parent, st = g.bfs(9999)
    o = OracleGraph(V, s, d)
    op, otrace = o.bfs(9999)
    assert st.rows() == otrace
    assert otrace[1][0] == 1          # the call that reaches the hub is dense
    assert parent[0] == op[0] == 5000
    assert g.info()["adj_entries"] == len(s)


def test_pull_bins_cover_all_degrees():
    # one vertex in each bin, including a heavy list that is not a multiple
    # of the chunk size, for every reduction toolkit
    V = 7000
    s, d = [], []
    for hub, deg in ((0, 6001), (1, 2049), (2, 2048), (3, 33), (4, 32), (5, 1)):
        src = np.arange(100, 100 + deg) % V
        s += src.tolist()
        d += [hub] * deg
        s += [hub]
        d += [int(src[0])]
    s, d = np.array(s, np.uint32), np.array(d, np.uint32)
    w = graphgen.weights(8, np.arange(len(s), dtype=np.uint64))
    g = gg.Graph.from_edges(V, s, d, w)
    o = OracleGraph(V, s, d, w)
    r, _, _ = g.pagerank(10)
    orr, _, _ = o.pagerank(10)
    assert rel_l1(r, orr) < PR_TOL
    dist, _ = g.sssp(100)
    odist, _ = o.sssp(100)
    assert np.array_equal(dist.view(np.uint32), odist.view(np.uint32))
    dep, inv, _ = g.bc(100)
    odep, oinv, _ = o.bc(100)
    ok = ~np.isnan(odep)
    assert np.array_equal(np.isnan(dep), np.isnan(odep)) and rel_l1(dep[ok], odep[ok]) < BC_TOL
    gs = gg.Graph.from_edges(V, s, d, symmetric=True)
    lab, _ = gs.cc()
    olab, _ = OracleGraph(V, s, d, symmetric=True).cc()
    assert np.array_equal(lab, olab)


@pytest.mark.parametrize("light,chunk,vec", [(16, 128, 1), (64, 512, 0), (1, 256, 0), (32, 256, 0)])
def test_results_do_not_depend_on_bins(light, chunk, vec):
    V, s, d, w, root = case("rmat16")
    g = gg.Graph.from_edges(V, s, d, w)
    g.set_bins(light, chunk, vec)
    o = OracleGraph(V, s, d, w)
    parent, st = g.bfs(root)
    op, otr = o.bfs(root)
    assert st.rows() == otr and np.array_equal(bfs_levels(parent, root), bfs_levels(op, root))
    ranks, _, _ = g.pagerank(10)
    assert rel_l1(ranks, o.pagerank(10)[0]) < PR_TOL
    dist, _ = g.sssp(root)
    assert np.array_equal(dist.view(np.uint32), o.sssp(root)[0].view(np.uint32))
    dep, inv, _ = g.bc(root)
    odep, oinv, _ = o.bc(root)
    ok = ~np.isnan(odep)
    assert rel_l1(dep[ok], odep[ok]) < BC_TOL
    lv, _, _, _, _ = gg.bfs_batched(g, [root, 0, 5])
    assert np.array_equal(lv[0], bfs_levels(op, root))
    gs = gg.Graph.from_edges(V, s, d, symmetric=True)
    gs.set_bins(light, chunk, vec)
    assert np.array_equal(gs.cc()[0], OracleGraph(V, s, d, symmetric=True).cc()[0])


@pytest.mark.parametrize("name", ["rmat16", "golden:edgecase", "star", "random_odd"])
@pytest.mark.parametrize("light", [4, 32, 512])
def test_l1_policy_matches_oracle(name, light):
    """The L1 gather policy changes how loads are cached, not the results:
    CC labels and SSSP distances bit-exact, per-call traces equal, PageRank
    and BC within tolerance."""
    V, s, d, w, root = case(name)
    o = OracleGraph(V, s, d, w)
    for hot in (0, 1 << 12, 0xffffffff):
        g = gg.Graph.from_edges(V, s, d, w)
        g.set_bins(light, 256, 0)
        g.set_l1_hot(hot)
        for layout in (True, False):
            g.set_pr_layout(layout)
            ranks, _, st = g.pagerank(10)
            oranks, _, otr = o.pagerank(10)
            assert rel_l1(ranks, oranks) < PR_TOL and st.rows() == otr
            r32, _, _ = g.pagerank(10, f32=True)
            assert rel_l1(r32.astype(np.float64), oranks) < PR_F32_TOL
            dist, st = g.sssp(root)
            odist, otr = o.sssp(root)
            assert np.array_equal(dist.view(np.uint32), odist.view(np.uint32)) and st.rows() == otr
            dep, inv, _ = g.bc(root)
            odep, oinv, _ = o.bc(root)
            assert np.array_equal(np.isnan(dep), np.isnan(odep)) and np.array_equal(inv, oinv)
            ok = ~np.isnan(odep)
            assert rel_l1(dep[ok], odep[ok]) < BC_TOL
        g.close()
        gs = gg.Graph.from_edges(V, s, d, symmetric=True)
        gs.set_bins(light, 256, 1)
        gs.set_l1_hot(hot)
        label, st = gs.cc()
        olabel, otr = OracleGraph(V, s, d, symmetric=True).cc()
        assert np.array_equal(label, olabel) and st.rows() == otr
        gs.close()


@pytest.mark.parametrize("name", ["rmat16", "grid128", "golden:edgecase", "star", "chain"])
@pytest.mark.parametrize("div", [1, 4])
def test_dense_push_matches_oracle(name, div):
    """Dense CC / SSSP calls run as a push over the frontier (div = 1: every
    one of them) give the oracle's labels and distances bit for bit and the
    same per-call trace, on both layouts."""
    V, s, d, w, root = case(name)
    o = OracleGraph(V, s, d, w)
    odist, otr = o.sssp(root)
    olabel, octr = OracleGraph(V, s, d, symmetric=True).cc()
    for layout in (True, False):
        g = gg.Graph.from_edges(V, s, d, w)
        g.set_pr_layout(layout)
        g.set_dense_push(div)
        dist, st = g.sssp(root)
        assert np.array_equal(dist.view(np.uint32), odist.view(np.uint32)) and st.rows() == otr
        g.close()
        gs = gg.Graph.from_edges(V, s, d, symmetric=True)
        gs.set_pr_layout(layout)
        gs.set_dense_push(div)
        label, st = gs.cc()
        assert np.array_equal(label, olabel) and st.rows() == octr
        gs.close()


@pytest.mark.parametrize("name", ["rmat16", "golden:edgecase", "star"])
def test_light_windows_keep_results(name):
    """Light lists read by 32-byte windows (pull_vector bit 1) combine the
    same entries in the same order: PageRank ranks, CC labels and SSSP
    distances are bit-identical to the scalar loads', at every light bound;
    BC dependencies (whose push steps add atomically, in no fixed order)
    agree within 1e-12."""
    V, s, d, w, root = case(name)
    g = gg.Graph.from_edges(V, s, d, w)
    gs = gg.Graph.from_edges(V, s, d, symmetric=True)
    for light in (4, 37, 512):
        got = []
        for vec in (0, 2, 3, 1):
            g.set_bins(light, 128, vec)
            gs.set_bins(light, 128, vec)
            got.append((g.pagerank(8)[0], g.pagerank(8, f32=True)[0], g.sssp(root)[0], gs.cc()[0], g.bc(root)[0]))
        for x, y in ((got[0], got[1]), (got[3], got[2])):
            for a, b in zip(x[:4], y[:4]):
                assert np.array_equal(a.view(np.uint8), b.view(np.uint8))
            assert np.array_equal(np.isnan(x[4]), np.isnan(y[4]))
            ok = ~np.isnan(x[4])
            assert rel_l1(y[4][ok], x[4][ok]) < 1e-12
    assert np.array_equal(got[1][2].view(np.uint32), OracleGraph(V, s, d, w).sssp(root)[0].view(np.uint32))
    with pytest.raises(gg.GeminiError):
        g.set_bins(32, 128, 4)
    g.close()
    gs.close()


@pytest.mark.parametrize("name", ["rmat16", "grid128", "golden:edgecase", "star", "chain"])
@pytest.mark.parametrize("div", [1, 5, 80, 100000])
def test_bfs_pull_switch_keeps_levels(name, div):
    """The BFS kernel switch (pull at active out-edges >= edges / div) moves
    which kernels run, not the levels, the tree's validity or the recorded
    per-call trace, which stays the reference's."""
    V, s, d, w, root = case(name)
    oparent, otrace = OracleGraph(V, s, d).bfs(root)
    g = gg.Graph.from_edges(V, s, d)
    g.set_bfs_pull(div)
    parent, st = g.bfs(root)
    assert np.array_equal(bfs_levels(parent, root), bfs_levels(oparent, root))
    assert st.rows() == otrace
    ok = parent < V
    ok[root] = False
    have = set(zip(s.tolist(), d.tolist()))
    assert all((int(p), int(v)) in have for v, p in zip(np.nonzero(ok)[0], parent[ok]))
    with pytest.raises(gg.GeminiError):
        g.set_bfs_pull(0)
    g.close()


@pytest.mark.parametrize("split", [1, 4, 7])
def test_pull_split_keeps_results(split):
    """The light and chunk kernels sharing every SM (gg_graph_set_pull_split)
    change only the launch shapes: PageRank ranks, CC labels and SSSP
    distances are bit-identical to the unsplit launches', and the oracle's."""
    V, s, d, w, root = case("rmat16")
    g = gg.Graph.from_edges(V, s, d, w)
    gs = gg.Graph.from_edges(V, s, d, symmetric=True)
    g.set_bins(16, 128, 0)
    gs.set_bins(16, 128, 0)
    base = (g.pagerank(8)[0], g.pagerank(8, f32=True)[0], g.sssp(root)[0], gs.cc()[0])
    g.set_pull_split(split)
    gs.set_pull_split(split)
    got = (g.pagerank(8)[0], g.pagerank(8, f32=True)[0], g.sssp(root)[0], gs.cc()[0])
    for a, b in zip(base, got):
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8))
    assert np.array_equal(got[2].view(np.uint32), OracleGraph(V, s, d, w).sssp(root)[0].view(np.uint32))
    assert np.array_equal(got[3], OracleGraph(V, s, d, symmetric=True).cc()[0])
    with pytest.raises(gg.GeminiError):
        g.set_pull_split(8)
    g.close()
    gs.close()


def test_pagerank_graph_replay():
    """PageRank runs are captured once as a CUDA graph and replayed while
    their arguments are unchanged: replays give bit-identical ranks, per-call
    timing works inside the graph, and a change of bins or precision
    recaptures."""
    V, s, d, w, _ = case("rmat16")
    g = gg.Graph.from_edges(V, s, d)
    oranks = OracleGraph(V, s, d).pagerank(12)[0]
    first, _, _ = g.pagerank(12)
    f32, _, _ = g.pagerank(12, f32=True)
    for _ in range(2):
        again, _, st = g.pagerank(12)
        assert np.array_equal(again, first)
        assert np.array_equal(g.pagerank(12, f32=True)[0], f32)
    st = gg.RunStats()
    st.enable_call_timing()
    import ctypes
    ranks = np.empty(V, np.float64)
    gg._check(gg.library().gg_pagerank(g.h, 12, gg._ptr(ranks), None, ctypes.byref(st.s)))
    assert np.array_equal(ranks, first)
    assert st.calls == 12 and all(float(st.call_ms[i]) > 0 for i in range(12))
    g.set_bins(16, 128, 0)
    moved, _, _ = g.pagerank(12)
    assert rel_l1(moved, oranks) < PR_TOL
    assert rel_l1(g.pagerank(7)[0], OracleGraph(V, s, d).pagerank(7)[0]) < PR_TOL


@pytest.mark.parametrize("name", ["rmat16", "grid128"])
def test_call_timing(name):
    """Per-call CUDA-event timing (the benchmark's roofline pass) works for
    host-driven runs and leaves results unchanged."""
    import ctypes
    V, s, d, w, root = case(name)
    g = gg.Graph.from_edges(V, s, d, w)
    ref_parent, _ = g.bfs(root)
    ref_dist, _ = g.sssp(root)
    for fn, out in ((gg.library().gg_bfs, np.empty(V, np.uint32)),
                    (gg.library().gg_sssp, np.empty(V, np.float32))):
        st = gg.RunStats()
        st.enable_call_timing()
        gg._check(fn(g.h, root, gg._ptr(out), ctypes.byref(st.s)))
        assert st.calls > 0
        # calls that a cooperative small run executes on the device have no
        # events of their own; the R-MAT runs have host-launched calls
        if name == "rmat16":
            assert float(np.sum(st.call_ms[:st.calls])) > 0
    assert np.array_equal(out.view(np.uint32), ref_dist.view(np.uint32))
    cc_st = gg.RunStats()
    cc_st.enable_call_timing()
    gs = gg.Graph.from_edges(V, s, d, symmetric=True)
    gg._check(gg.library().gg_cc(gs.h, None, ctypes.byref(cc_st.s)))
    assert cc_st.calls > 0


def test_autotune_picks_and_caches(tmp_path):
    V, s, d, w, root = case("rmat16")
    g = gg.Graph.from_edges(V, s, d, w)
    r1 = g.autotune(str(tmp_path))
    # 36 bin candidates, then the light windows (once or twice), the L1
    # policy and the pull split (the default objective includes PageRank)
    assert 39 <= r1["candidates"] <= 40 and r1["from_cache"] == 0
    assert r1["bfs_pull"] == 20
    assert r1["light_deg"] in (16, 32, 64, 128, 256, 512) and r1["pull_chunk"] in (128, 256, 512)
    assert r1["l1_hot_bytes"] in (160 << 10, 0xffffffff)
    assert r1["pull_split"] in (0, 4)
    assert r1["best_ms"] <= r1["default_ms"]
    g2 = gg.Graph.from_edges(V, s, d, w)
    r2 = g2.autotune(str(tmp_path))
    key = ("light_deg", "pull_chunk", "pull_vector", "l1_hot_bytes", "pull_split", "bfs_pull")
    assert r2["from_cache"] == 1 and [r2[k] for k in key] == [r1[k] for k in key]
    parent, st = g2.bfs(root)
    assert st.rows() == OracleGraph(V, s, d).bfs(root)[1]
    with pytest.raises(gg.GeminiError):
        g2.set_bins(32, 300)


@pytest.mark.parametrize("name", ["rmat16", "grid128", "random_odd"])
def test_cc_layouts_agree(name):
    """CC on a symmetric graph runs on the hot-source layout by default (labels
    stay vertex ids, mapped back to vertex order); the plain adjacency gives
    the same labels and the same per-call trace, both equal to the oracle's."""
    V, s, d, w, _ = case(name)
    g = gg.Graph.from_edges(V, s, d, symmetric=True)
    olabel, otrace = OracleGraph(V, s, d, symmetric=True).cc()
    hot, st = g.cc()
    g.set_pr_layout(False)
    plain, st2 = g.cc()
    assert np.array_equal(hot, olabel) and np.array_equal(plain, olabel)
    assert st.rows() == otrace and st2.rows() == otrace
    g.set_pr_layout(True)
    ranks_hot = g.pagerank(5)[0]
    again, _ = g.cc()
    assert np.array_equal(again, olabel)
    assert rel_l1(ranks_hot, OracleGraph(V, s, d, symmetric=True).pagerank(5)[0]) < PR_TOL


@pytest.mark.parametrize("name", ["rmat16", "grid128", "random_odd"])
def test_pagerank_layouts_agree(name):
    """The hot-source layout (default) and the plain incoming adjacency give
    the same ranks up to summation order, both within tolerance of the
    oracle; the layout is rebuilt after a transpose and freed on request."""
    V, s, d, w, _ = case(name)
    g = gg.Graph.from_edges(V, s, d)
    oranks = OracleGraph(V, s, d).pagerank(20)[0]
    hot, _, st = g.pagerank(20)
    bytes_hot = g.info()["device_bytes"]
    g.set_pr_layout(False)
    plain, _, st2 = g.pagerank(20)
    assert g.info()["device_bytes"] < bytes_hot
    assert st.rows() == st2.rows()
    assert rel_l1(hot, oranks) < PR_TOL and rel_l1(plain, oranks) < PR_TOL
    assert rel_l1(hot, plain) < 1e-13
    f_plain, _, _ = g.pagerank(20, f32=True)
    g.set_pr_layout(True)
    f_hot, _, _ = g.pagerank(20, f32=True)
    assert rel_l1(f_hot.astype(np.float64), oranks) < PR_F32_TOL
    assert rel_l1(f_hot.astype(np.float64), f_plain.astype(np.float64)) < 1e-5
    g.transpose()
    g.transpose()
    again, _, _ = g.pagerank(20)
    assert np.array_equal(again, hot)


def test_autotune_objectives(tmp_path):
    V, s, d, w, root = case("rmat16")
    g = gg.Graph.from_edges(V, s, d, w)
    seen = set()
    for obj in (("pagerank",), ("bfs",), ("batched",)):
        r = g.autotune(str(tmp_path), objective=obj)
        assert (39 <= r["candidates"] <= 40 if obj == ("pagerank",) else r["candidates"] == 36)
        assert r["from_cache"] == 0 and r["best_ms"] > 0
        seen.add(obj)
    # double PageRank: windows, L1 policy, split; BC: windows, split
    r = g.autotune(str(tmp_path), objective=("pagerank_f64",))
    assert 39 <= r["candidates"] <= 40 and r["best_ms"] > 0
    r = g.autotune(str(tmp_path), objective=("bc",))
    assert 38 <= r["candidates"] <= 39 and r["best_ms"] > 0
    dep, inv, _ = g.bc(root)
    odep, oinv, _ = OracleGraph(V, s, d, w).bc(root)
    assert np.array_equal(inv, oinv)
    assert g.autotune(str(tmp_path), objective=("batched",))["from_cache"] == 1
    lv, _, _, _, _ = gg.bfs_batched(g, [root, 1, 2])
    o = OracleGraph(V, s, d, w)
    assert np.array_equal(lv[0], bfs_levels(o.bfs(root)[0], root))
    with pytest.raises(gg.GeminiError):
        g.autotune(str(tmp_path), objective=())


def test_dump_vertex_array_from_device(tmp_path):
    """A device result array (the last call's, gg_result_device_ptr) dumps
    to the same bytes as its host copy, and restores into device memory."""
    import ctypes
    V, s, d, w, root = case("rmat16")
    g = gg.Graph.from_edges(V, s, d, w)
    dist, _ = g.sssp(root)
    dev = gg.library().gg_result_device_ptr(g.h, 0)
    assert dev
    p = tmp_path / "dist.bin"
    assert gg.library().gg_dump_vertex_array(ctypes.c_void_p(dev), 4, V, str(p).encode()) == 0
    assert p.read_bytes() == dist.tobytes()
    assert gg.library().gg_restore_vertex_array(ctypes.c_void_p(dev), 4, V, str(p).encode()) == 0
    assert gg.library().gg_dump_vertex_array(ctypes.c_void_p(dev), 4, V, str(tmp_path / "again.bin").encode()) == 0
    assert (tmp_path / "again.bin").read_bytes() == dist.tobytes()


def test_bfs_many_equals_single_runs():
    """gg_bfs_many: each run's parent tree lands in its host array and equals
    gg_bfs on the same root; a NULL output skips the copy."""
    V, s, d, w, root = case("rmat16")
    g = gg.Graph.from_edges(V, s, d)
    deg = np.bincount(s, minlength=V)
    roots = gg.pick_roots(deg, 5, 31)
    outs = [np.empty(V, np.uint32) for _ in roots]
    outs[3] = None
    st = g.bfs_many(roots, outs)
    total = 0
    for r, o in zip(roots, outs):
        parent, single = g.bfs(r)
        total += single.active_edges_total
        if o is not None:
            assert np.array_equal(bfs_levels(o, r), bfs_levels(parent, r))
    assert st.active_edges_total == total
    with pytest.raises(gg.GeminiError):
        g.bfs_many([V], [None])
