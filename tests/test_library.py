"""CPU checks of the C-ABI library: it loads, exports every entry point the
header declares, its host generator matches the numpy restatement, and
device calls without a GPU fail with a status instead of crashing."""
import os
import re

import numpy as np
import pytest

import geminigraph_gb300 as gg
import graphgen

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in sorted(os.listdir(os.path.join(REPO, "include"))):
        if h.endswith(".h"):
            text = open(os.path.join(REPO, "include", h)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names += re.findall(r"\b(gg_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    L = gg.library()
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_checked_library_exports_the_same_symbols():
    """libgemini_gb300_check.so (device bounds checks) is a drop-in for the
    plain library."""
    import ctypes
    path = os.path.join(REPO, "geminigraph_gb300", "libgemini_gb300_check.so")
    if not os.path.exists(path):
        pytest.skip("checked library not built")
    C = ctypes.CDLL(path)
    missing = [n for n in declared_functions() if not hasattr(C, n)]
    assert not missing, missing


@pytest.mark.parametrize("kind,p1,p2,seed,weighted", [
    (gg.RMAT, 8, 16, 1, False), (gg.RMAT, 11, 16, 5, True), (gg.RMAT, 14, 4, 99, True),
    (gg.GRID, 2, 0, 0, False), (gg.GRID, 17, 0, 3, True), (gg.GRID, 64, 0, 5, False)])
def test_host_generator_matches_restatement(kind, p1, p2, seed, weighted):
    buf = gg.generate_records(kind, p1, p2, seed, weighted=weighted, threads=3)
    if kind == gg.RMAT:
        s, d, w = graphgen.rmat(p1, p2, seed, weighted=weighted)
    else:
        s, d, w = graphgen.grid(p1, seed=seed, weighted=weighted)
    assert buf.tobytes() == graphgen.to_records(s, d, w)


def test_grid_counts_and_symmetry():
    s, d, _ = graphgen.grid(9)
    assert len(s) == 4 * 9 * 8
    pairs = set(zip(s.tolist(), d.tolist()))
    assert all((b, a) in pairs for a, b in pairs)
    assert gg.library().gg_generate_count(gg.GRID, 8192, 0) == 268402688
    assert gg.library().gg_generate_count(gg.RMAT, 26, 16) == 1073741824


def test_switch_rule():
    L = gg.library()
    # core/graph.hpp:1509: sparse iff active_edges < edges / 20 (integer division)
    assert L.gg_is_sparse(0, 19) == 0
    assert L.gg_is_sparse(0, 20) == 1
    assert L.gg_is_sparse(49, 1000) == 1
    assert L.gg_is_sparse(50, 1000) == 0


def test_bad_arguments_return_status():
    L = gg.library()
    import ctypes
    h = ctypes.c_void_p()
    assert L.gg_graph_generate(0, 40, 16, 1, 0, 0, 0, ctypes.byref(h)) == 1
    assert L.gg_graph_load(b"/nonexistent/graph.bin", 10, 0, 0, 0, ctypes.byref(h)) == 2
    assert L.gg_bfs(None, 0, None, None) == 1


@pytest.mark.skipif(os.path.exists("/dev/nvidia0"), reason="a GPU is present")
def test_device_call_without_gpu_fails_loudly():
    with pytest.raises(gg.GeminiError):
        gg.Graph.generate(gg.RMAT, 8, 4, 1)


def test_dump_and_restore_vertex_array(tmp_path):
    """core/graph.hpp:253-307 with one partition: the file is the array's
    bytes; a restore of a file of another length is an error, not an assert."""
    a = np.arange(1000, dtype=np.float64) * 0.5
    p = tmp_path / "ranks.bin"
    gg.dump_vertex_array(a, str(p))
    assert p.read_bytes() == a.tobytes()
    b = gg.restore_vertex_array(str(p), 1000, np.float64)
    assert np.array_equal(a, b)
    with pytest.raises(gg.GeminiError):
        gg.restore_vertex_array(str(p), 999, np.float64)
    with pytest.raises(gg.GeminiError):
        gg.restore_vertex_array(str(tmp_path / "missing.bin"), 10, np.uint32)
