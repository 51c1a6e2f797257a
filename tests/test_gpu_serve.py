"""Serving loop: continuous batching over resident graphs.  Every served
query must report the same reached count and result checksum as the same
root run alone through the single-root toolkit (gg_bfs / gg_sssp), whatever
else was on the device with it."""
import time

import numpy as np
import pytest

import geminigraph_gb300 as gg
import graphgen

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def graphs():
    out = []
    for kind, p1, seed in ((gg.RMAT, 12, 4), (gg.RMAT, 14, 5), (gg.GRID, 48, 6)):
        rec = gg.generate_records(kind, p1, 16, seed, weighted=True)
        V = (1 << p1) if kind == gg.RMAT else p1 * p1
        g = gg.Graph.from_records(rec, V, weighted=True)
        src = rec.view(np.uint32).reshape(-1, 3)[:, 0]
        out.append((g, V, np.bincount(src, minlength=V)))
    return out


def expected(g, kind, root):
    if kind == 0:
        parent, _ = g.bfs(root)
        lv = gg.levels_from_parents(parent, root)
        return int((lv >= 0).sum()), gg.result_checksum(lv, 0)
    dist, _ = g.sssp(root)
    return int((dist < np.float32(1e9)).sum()), gg.result_checksum(dist, 1)


def run_queries(server, queries, burst=37, pause=0.002):
    done = {}
    tickets = {}
    for i in range(0, len(queries), burst):
        for (gid, kind, root) in queries[i:i + burst]:
            tickets[server.submit(gid, kind, root)] = (gid, kind, root)
        time.sleep(pause)
        for r in server.wait(timeout_ms=0):
            done[r["ticket"]] = r
    t0 = time.time()
    while len(done) < len(tickets) and time.time() - t0 < 120:
        for r in server.wait(timeout_ms=100):
            done[r["ticket"]] = r
    assert len(done) == len(tickets)
    return tickets, done


@pytest.mark.parametrize("solo", [0, 16, 64])
def test_served_results_equal_single_root_runs(graphs, solo):
    """solo = 0: every SSSP query in a batch; 16 (default) / 64: an idle SSSP
    pool with fewer waiting queries runs them alone through gg_sssp."""
    rng = np.random.default_rng(3)
    server = gg.Server()
    server.set_solo(solo)
    ids = [server.add_graph(g) for g, _, _ in graphs]
    queries = []
    for _ in range(400):
        j = int(rng.integers(0, len(graphs)))
        g, V, deg = graphs[j]
        kind = int(rng.integers(0, 2))
        root = int(rng.integers(0, V)) if rng.random() < 0.1 else gg.pick_roots(deg, 1, int(rng.integers(1 << 30)))[0]
        queries.append((ids[j], kind, root))
    tickets, done = run_queries(server, queries)
    cache = {}
    for t, (gid, kind, root) in tickets.items():
        key = (gid, kind, root)
        if key not in cache:
            cache[key] = expected(graphs[gid][0], kind, root)
        r = done[t]
        assert r["status"] == 0
        assert (r["reached"], r["checksum"]) == cache[key], (gid, kind, root)
        assert r["graph"] == gid and r["kind"] == kind and r["root"] == root
    st = server.stats()
    assert st["completed"] == len(queries)
    assert (st["solo_runs"] > 0) == (solo > 0)
    assert st["max_lanes_in_use"] > 1         # queries shared the device
    assert st["max_busy_pools"] > 1           # pools of different graphs/kinds overlapped
    server.close()


def test_batch_window_keeps_results(graphs):
    """Idle pools that hold their first queries for a batch window start them
    together; every result still equals the query's single-root run."""
    rng = np.random.default_rng(9)
    server = gg.Server()
    server.set_window(gg.Server.SSSP, 4.0)
    server.set_window(gg.Server.BFS, 1.0)
    ids = [server.add_graph(g) for g, _, _ in graphs]
    queries = []
    for _ in range(150):
        j = int(rng.integers(0, len(graphs)))
        g, V, deg = graphs[j]
        queries.append((ids[j], int(rng.integers(0, 2)), gg.pick_roots(deg, 1, int(rng.integers(1 << 30)))[0]))
    tickets, done = run_queries(server, queries, burst=5, pause=0.003)
    for t, (gid, kind, root) in tickets.items():
        assert (done[t]["reached"], done[t]["checksum"]) == expected(graphs[gid][0], kind, root)
    assert server.stats()["max_lanes_in_use"] > 1
    with pytest.raises(gg.GeminiError):
        server.set_window(2, 1.0)
    with pytest.raises(gg.GeminiError):
        server.set_window(0, -1.0)
    server.close()


def test_admission_waits_for_memory(graphs):
    # a budget that holds one pool at a time: pools must close when idle and
    # queries of the other graphs wait for their memory
    g0, V0, deg0 = graphs[0]
    g1, V1, deg1 = graphs[1]
    need = max(gg.Server.pool_bytes(g0, 0), gg.Server.pool_bytes(g1, 0))
    server = gg.Server(hbm_budget=need + 1)
    a, b = server.add_graph(g0), server.add_graph(g1)
    qs = [(a, 0, r) for r in gg.pick_roots(deg0, 20, 1)] + [(b, 0, r) for r in gg.pick_roots(deg1, 20, 2)]
    tickets, done = run_queries(server, qs, burst=40)
    for t, (gid, kind, root) in tickets.items():
        g = (g0, g1)[gid]
        assert (done[t]["reached"], done[t]["checksum"]) == expected(g, kind, root)
    st = server.stats()
    assert st["admission_waits"] > 0
    assert st["pools_closed"] >= 1
    assert st["bytes_in_use"] <= st["budget"]
    server.close()


def test_submit_errors(graphs):
    g, V, _ = graphs[0]
    server = gg.Server()
    gid = server.add_graph(g)
    with pytest.raises(gg.GeminiError):
        server.submit(gid, 0, V)
    with pytest.raises(gg.GeminiError):
        server.submit(gid + 5, 0, 0)
    gu = gg.Graph.from_edges(10, np.array([1, 2], np.uint32), np.array([2, 3], np.uint32))
    uid = server.add_graph(gu)
    with pytest.raises(gg.GeminiError):
        server.submit(uid, 1, 1)
    server.close()
