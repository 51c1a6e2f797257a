"""The bounds-checked build (libgemini_gb300_check.so, GG_CHECK): every
adjacency entry index and neighbour id a kernel reads is checked before use
(gg_common.cuh), standing in for compute-sanitizer on the device.  The
toolkits, the batched runs and the partitioned build run through it on
several graphs in a child process (GG_LIBRARY=check), with results equal to
the oracle's and no check failing."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r'''
import sys
sys.path.insert(0, REPO); sys.path.insert(0, REPO + "/tests")
import numpy as np
import geminigraph_gb300 as gg
import graphgen
from golden_util import Fixture
from oracle.oracle import OracleGraph, bfs_levels
assert gg.LIB_PATH.endswith("libgemini_gb300_check.so"), gg.LIB_PATH

def rel(a, b):
    return float(np.abs(a - b).sum() / max(np.abs(b).sum(), 1e-300))

cases = []
s, d, w = graphgen.rmat(15, 16, 3, weighted=True); cases.append((1 << 15, s, d, w))
s, d, w = graphgen.grid(64, seed=2, weighted=True); cases.append((64 * 64, s, d, w))
fx = Fixture("edgecase"); cases.append((fx.V, fx.src, fx.dst, fx.w))
for V, s, d, w in cases:
    root = graphgen.pick_root(s, V, seed=V)
    o = OracleGraph(V, s, d, w)
    for kw in ({}, {"force_partitions": 3}):
        g = gg.Graph.from_edges(V, s, d, w, **kw)
        parent, _ = g.bfs(root)
        assert np.array_equal(bfs_levels(parent, root), bfs_levels(o.bfs(root)[0], root))
        ranks, _, _ = g.pagerank(10)
        assert rel(ranks, o.pagerank(10)[0]) < 1e-10
        dist, _ = g.sssp(root)
        assert np.array_equal(dist.view(np.uint32), o.sssp(root)[0].view(np.uint32))
        dep, inv, _ = g.bc(root)
        odep = o.bc(root)[0]
        ok = ~np.isnan(odep)
        assert np.array_equal(np.isnan(dep), np.isnan(odep)) and rel(dep[ok], odep[ok]) < 1e-10
        roots = gg.pick_roots(np.bincount(s, minlength=V), 9, seed=4)
        lv = gg.bfs_batched(g, roots)[0]
        bd = gg.sssp_batched(g, roots)[0]
        bdep = gg.bc_batched(g, roots)[0]
        for i, r in enumerate(roots):
            assert np.array_equal(lv[i], bfs_levels(o.bfs(r)[0], r))
            assert np.array_equal(bd[i].view(np.uint32), o.sssp(r)[0].view(np.uint32))
        g.close()
    gs = gg.Graph.from_edges(V, s, d, symmetric=True)
    assert np.array_equal(gs.cc()[0], OracleGraph(V, s, d, symmetric=True).cc()[0])
    gs.close()
maps = open("/proc/self/maps").read()
assert "libgemini_gb300_check.so" in maps and "libgemini_gb300.so" not in maps
print("CHECKED OK")
'''


def test_checked_build_runs_clean():
    lib = os.path.join(REPO, "geminigraph_gb300", "libgemini_gb300_check.so")
    assert os.path.exists(lib), "build() makes the checked library beside the plain one"
    env = dict(os.environ, GG_LIBRARY="check")
    p = subprocess.run([sys.executable, "-c", "REPO = %r\n" % REPO + SCRIPT], capture_output=True, text=True,
                       env=env, timeout=900)
    assert p.returncode == 0, p.stdout[-2000:] + p.stderr[-4000:]
    assert "CHECKED OK" in p.stdout
