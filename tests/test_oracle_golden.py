"""Pins the CPU oracle to the reference: every fixture in tests/golden/ holds
the outputs of the unmodified reference toolkits (see golden/make_golden.py)."""
import numpy as np
import pytest

from golden_util import Fixture, names
from oracle.oracle import OracleGraph, bfs_levels, bfs_reference_levels

FIXTURES = names()


@pytest.fixture(scope="module", params=FIXTURES)
def fx(request):
    return Fixture(request.param)


def rel_l1(a, b):
    return float(np.abs(a - b).sum() / max(np.abs(b).sum(), 1e-300))


def test_fixtures_present():
    assert {"rmat10", "rmat12", "grid32", "edgecase"} <= set(FIXTURES)


def test_degrees(fx):
    g = OracleGraph(fx.V, fx.src, fx.dst)
    _, _, _, deg = g.adjacency(incoming=False)
    assert np.array_equal(deg, fx["out_degree"])
    s = OracleGraph(fx.V, fx.src, fx.dst, symmetric=True)
    _, _, _, sdeg = s.adjacency()
    assert np.array_equal(sdeg, fx["sym_degree"])


def test_bfs_levels_and_counts(fx):
    g = OracleGraph(fx.V, fx.src, fx.dst)
    parent, trace = g.bfs(fx.root)
    ref_levels = bfs_levels(fx["bfs_parent"], fx.root)
    assert np.array_equal(bfs_levels(parent, fx.root), ref_levels)
    assert np.array_equal(ref_levels, bfs_reference_levels(fx.V, fx.src, fx.dst, fx.root))
    # active(i) printed = popcount of the frontier entering iteration i
    printed = fx.printed_active("bfs")
    assert printed == [1] + [row[2] for row in trace[:-1]]
    found = int((parent < fx.V).sum())
    assert fx.summary("bfs").strip() == f"found_vertices = {found}"


def test_pagerank(fx):
    g = OracleGraph(fx.V, fx.src, fx.dst)
    ranks, deltas, trace = g.pagerank(20)
    ref = fx["pr_ranks"]
    assert rel_l1(ranks, ref) < 1e-12
    assert ["%f" % d for d in deltas] == ["%f" % d for d in fx.printed_deltas()]
    assert all(mode == 1 for mode, _, _ in trace)
    amax = int(np.argmax(ranks))
    assert fx.summary("pr").splitlines()[1] == "pr[%d]=%f" % (amax, ranks[amax])


def test_cc_bit_exact(fx):
    g = OracleGraph(fx.V, fx.src, fx.dst, symmetric=True)
    label, trace = g.cc()
    assert np.array_equal(label, fx["cc_label"])
    printed = fx.printed_active("cc")
    assert printed[0] == fx.V
    # dense calls return one activation per changed vertex; sparse calls count
    # racing activations (>= the number of distinct vertices)
    for (mode, _, act), p in zip(trace[:-1], printed[1:]):
        assert p == act if mode == 1 else p >= act > 0
    assert len(printed) == len(trace)
    assert fx.summary("cc").strip() == f"components = {len(np.unique(label))}"


def test_sssp_bit_exact(fx):
    g = OracleGraph(fx.V, fx.src, fx.dst, fx.w)
    dist, trace = g.sssp(fx.root)
    assert np.array_equal(dist.view(np.uint32), fx["sssp_dist"].view(np.uint32))
    printed = fx.printed_active("sssp")
    for (mode, _, act), p in zip(trace[:-1], printed[1:]):
        assert p == act if mode == 1 else p >= act > 0
    assert len(printed) == len(trace)


def test_bc(fx):
    g = OracleGraph(fx.V, fx.src, fx.dst)
    dep, inv, trace = g.bc(fx.root)
    ref_dep, ref_inv = fx["bc_dep"], fx["bc_inv"]
    assert np.array_equal(np.isnan(dep), np.isnan(ref_dep))
    assert np.array_equal(inv, ref_inv)            # 1 / path counts: exact integers
    ok = ~np.isnan(ref_dep)
    assert rel_l1(dep[ok], ref_dep[ok]) < 1e-12
    fwd = fx.printed_active("bc")
    nfwd = len(fwd)
    assert fwd == [1] + [row[2] for row in trace[: nfwd - 1]]
    lines = fx.summary("bc").strip().splitlines()
    assert lines == ["%f %f" % (dep[v], 1 / inv[v]) for v in range(20)]
