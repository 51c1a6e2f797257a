"""CPU checks of the inputs the reference arm builds without the product
library: the oracle's generator gives the product generator's bytes, its root
rule draws the product's roots, its tree check agrees with the Python one,
and the reference arm of bench.py loads no product code."""
import hashlib
import os
import subprocess
import sys

import numpy as np
import pytest

import geminigraph_gb300 as gg
import graphgen
from oracle import oracle

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("kind,p1,p2,seed,weighted", [
    (oracle.RMAT, 12, 16, 1, False), (oracle.RMAT, 11, 16, 5, True), (oracle.RMAT, 9, 3, 77, False),
    (oracle.GRID, 2, 0, 0, False), (oracle.GRID, 17, 0, 3, True), (oracle.GRID, 64, 0, 5, False)])
def test_oracle_generator_is_byte_identical(kind, p1, p2, seed, weighted):
    mine = oracle.records(kind, p1, p2, seed, weighted, threads=3).tobytes()
    prod = gg.generate_records(kind, p1, p2, seed, weighted=weighted).tobytes()
    assert hashlib.sha256(mine).hexdigest() == hashlib.sha256(prod).hexdigest()
    if kind == oracle.RMAT:
        s, d, w = graphgen.rmat(p1, p2, seed, weighted=weighted)
    else:
        s, d, w = graphgen.grid(p1, seed=seed, weighted=weighted)
    assert mine == graphgen.to_records(s, d, w)


def test_generator_ranges_and_file(tmp_path):
    full = oracle.records(oracle.RMAT, 10, 16, 3, True)
    part = oracle.records(oracle.RMAT, 10, 16, 3, True, first=1000, count=5000, threads=4)
    assert np.array_equal(full.reshape(-1, 3)[1000:6000].ravel(), part)
    path = str(tmp_path / "g.bin")
    V, n, deg = oracle.write_records_file(path, oracle.RMAT, 10, 16, 3, weighted=True, threads=2, chunk=4096)
    assert (V, n) == (1024, 16384)
    assert open(path, "rb").read() == full.tobytes()
    assert np.array_equal(deg, np.bincount(full.reshape(-1, 3)[:, 0], minlength=V))


def test_root_rule_matches_product_and_prefix():
    rng = np.random.default_rng(4)
    deg = rng.integers(0, 3, 5000).astype(np.uint32)
    for seed in (1, 1001, 2001):
        a = oracle.pick_roots(deg, 40, seed)
        assert a == gg.pick_roots(deg, 40, seed)
        # a shorter draw is a prefix of a longer one: the reference arm's
        # roots are the GPU arm's roots
        assert oracle.pick_roots(deg, 25, seed) == a[:25]
        assert all(deg[r] > 0 for r in a)


def test_tree_levels():
    parent = np.array([0, 0, 1, 1, 9, 3], np.uint32)   # vertex 4 unreached (parent = V... > V)
    parent[4] = 6
    lv = oracle.tree_levels(parent, 0)
    assert lv.tolist() == [0, 1, 2, 2, -1, 3]
    assert np.array_equal(lv, oracle.bfs_levels(parent, 0))
    bad = parent.copy()
    bad[1], bad[3] = 3, 1          # a cycle 1 -> 3 -> 1
    with pytest.raises(AssertionError):
        oracle.tree_levels(bad, 0)
    with pytest.raises(AssertionError):
        oracle.tree_levels(parent, 1)   # root is not its own parent


@pytest.mark.skipif(not os.path.exists(os.path.join(REPO, "oracle", "_ref", "bin", "ref_bfs")),
                    reason="reference toolkits not built here")
def test_reference_arm_loads_no_product_code():
    code = (
        "import sys, json; sys.path.insert(0, %r); import bench\n"
        "bench.WORKLOADS['bfs'] = dict(bench.WORKLOADS['bfs'], scale=12)\n"
        "r = bench.cpu_reference('bfs', 2, 1)\n"
        "maps = open('/proc/self/maps').read()\n"
        "print(json.dumps({'kind': r['kind'], 'edges': r['edges'], 'mod': 'geminigraph_gb300' in sys.modules,\n"
        "                  'so': 'libgemini_gb300' in maps}))\n" % REPO)
    p = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    import json
    out = json.loads(p.stdout.strip().splitlines()[-1])
    assert out["kind"] == "reference"
    assert not out["mod"] and not out["so"]
    # the reference's own traversed-edge count equals the oracle's trace sum
    rec = oracle.records(oracle.RMAT, 12, 16, 1)
    s, d = rec[0::2].copy(), rec[1::2].copy()
    roots = oracle.pick_roots(np.bincount(s, minlength=4096), 3, seed=1001)
    og = oracle.OracleGraph(4096, s, d)
    assert out["edges"] == [sum(r[1] for r in og.bfs(x)[1]) for x in roots[1:]]
