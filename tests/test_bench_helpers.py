"""CPU checks of the arithmetic bench.py reports with: the algorithmic bytes
behind the roofline fraction, the committed DRAM-traffic lookup, the peak
source and the latency percentiles."""
import json
import os
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)

import bench  # noqa: E402


def test_algorithmic_bytes_pull_and_push():
    V, ae = 1 << 20, 16 << 20
    # float PageRank pull: 8 B per counted edge (neighbour id + gathered rank),
    # per vertex 8 B offset + 4 B rank write, plus three bitmaps of V bits
    assert bench.algorithmic_bytes(1, ae, V, 0, "pagerank") == 8 * ae + V * 12 + 3 * (V // 8)
    # SSSP pull: neighbour id + weight + distance per edge, 4 B distance per vertex
    assert bench.algorithmic_bytes(1, ae, V, 0, "sssp") == 12 * ae + V * 12 + 3 * (V // 8)
    # double BC pull: 8 B state
    assert bench.algorithmic_bytes(1, ae, V, 0, "bc") == 12 * ae + V * 16 + 3 * (V // 8)
    # BFS push over a frontier of 1000 vertices: offset, degree and queue entry each
    assert bench.algorithmic_bytes(0, ae, V, 1000, "bfs") == 8 * ae + 1000 * 16


def test_committed_traffic_matches_scale():
    d = json.load(open(os.path.join(REPO, "profiles", "traffic.json")))
    e = d["bfs"]["bfs_pull"]
    assert bench.committed_traffic("bfs_pull", "bfs", e["scale"]) == float(e["bytes_per_launch"])
    assert bench.committed_traffic("bfs_pull", "bfs", int(e["scale"]) - 2) is None
    assert bench.committed_traffic("no_such_kernel", "bfs", 26) is None


def test_peak_source():
    peak, kind = bench.peaks()
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        assert kind == "measured" and peak == float(json.load(open(p))["hbm_gbs"])
    else:
        assert kind == "fallback" and peak == bench.FALLBACK_HBM_GBS


def test_percentiles():
    xs = list(range(1, 101))
    assert bench.pct(xs, 50) == 51 and bench.pct(xs, 99) == 99 and bench.pct(xs, 100) == 100
    assert bench.pct([], 50) is None
