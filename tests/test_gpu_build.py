"""GPU checks of the partitioned (out-of-core) build and of host-resident
adjacency.

The reference streams the edge file in CHUNKSIZE pieces
(core/graph.hpp:805-821) so the edge list is never resident at once.  Here the
bound is on device memory: the partitioned build leaves the records in host
memory and builds each direction range by range.  Its adjacency must be
bit-identical to the in-core build's (neighbours, weights, offsets, degrees),
and graphs whose adjacency lives in host memory must give the same results
as device-resident ones.
"""
import os

import numpy as np
import pytest

import geminigraph_gb300 as gg

pytestmark = pytest.mark.gpu

RMAT = 0


def records(scale, seed, weighted, ef=16):
    return gg.generate_records(RMAT, scale, ef, seed, weighted=weighted)


def same_adjacency(a, b):
    ia, ib = a.info(), b.info()
    assert ia["adj_entries"] == ib["adj_entries"] and ia["edges"] == ib["edges"]
    for incoming in (False, True):
        oa, na, wa, da = a.adjacency(incoming)
        ob, nb, wb, db = b.adjacency(incoming)
        assert np.array_equal(oa, ob)
        assert np.array_equal(na, nb)
        assert np.array_equal(da, db)
        if wa is not None:
            assert np.array_equal(wa.view(np.uint32), wb.view(np.uint32))


@pytest.mark.parametrize("weighted", [False, True])
@pytest.mark.parametrize("symmetric", [False, True])
@pytest.mark.parametrize("parts", [2, 7, 256])
def test_partitioned_equals_in_core(weighted, symmetric, parts):
    rec = records(13, 5 + parts, weighted)
    V = 1 << 13
    a = gg.Graph.from_records(rec, V, weighted=weighted, symmetric=symmetric)
    b = gg.Graph.from_records(rec, V, weighted=weighted, symmetric=symmetric, force_partitions=parts)
    assert a.build["partitions"] == 1
    assert b.build["partitions"] > 1
    same_adjacency(a, b)


def test_partitioned_by_budget_scale_20():
    """A 100 MB build budget cannot hold the in-core working set of 16.8 M
    records (~420 MB): the build cuts each direction into ranges."""
    rec = records(20, 11, True)
    V = 1 << 20
    a = gg.Graph.from_records(rec, V, weighted=True)
    b = gg.Graph.from_records(rec, V, weighted=True, build_budget=100 << 20)
    assert a.build["partitions"] == 1
    assert b.build["partitions"] >= 4
    same_adjacency(a, b)
    pa, _ = a.bfs(0)
    pb, _ = b.bfs(0)
    assert np.array_equal(gg.levels_from_parents(pa, 0), gg.levels_from_parents(pb, 0))


def test_budget_too_small_is_an_error():
    rec = records(16, 3, False)
    with pytest.raises(gg.GeminiError) as e:
        gg.Graph.from_records(rec, 1 << 16, build_budget=1 << 20)
    assert e.value.code == 5  # GG_ERR_NOMEM


def test_partitioned_range_error():
    rec = np.array([[0, 1], [1, 2], [2, 9]], np.uint32)
    with pytest.raises(gg.GeminiError) as e:
        gg.Graph.from_records(rec, 4, force_partitions=2)
    assert e.value.code == 3  # GG_ERR_RANGE


def test_partitioned_empty_and_tiny():
    g = gg.Graph.from_records(np.zeros((0, 2), np.uint32), 5, force_partitions=3)
    off, nbr, _, deg = g.adjacency(True)
    assert (off == 0).all() and len(nbr) == 0 and (deg == 0).all()
    rec = np.array([[3, 0], [0, 3], [3, 0], [1, 1]], np.uint32)
    a = gg.Graph.from_records(rec, 4)
    b = gg.Graph.from_records(rec, 4, force_partitions=256)
    same_adjacency(a, b)


def test_partitioned_from_pinned_records():
    """Records already in pinned host memory are read in place."""
    rec = records(12, 9, True)
    p = gg.library()
    import ctypes
    ptr = ctypes.c_void_p()
    gg._check(p.gg_host_alloc(rec.nbytes, ctypes.byref(ptr)))
    try:
        pinned = np.ctypeslib.as_array((ctypes.c_uint8 * rec.nbytes).from_address(ptr.value))
        pinned[:] = rec
        a = gg.Graph.from_records(rec, 1 << 12, weighted=True)
        b = gg.Graph.from_records(pinned, 1 << 12, weighted=True, force_partitions=5)
        same_adjacency(a, b)
        del b
    finally:
        p.gg_host_free(ptr)


def test_load_file_partitioned(tmp_path):
    rec = records(14, 21, True)
    path = os.path.join(tmp_path, "rmat14.bin")
    rec.tofile(path)
    a = gg.Graph.load(path, 1 << 14, weighted=True)
    b = gg.Graph.load(path, 1 << 14, weighted=True, force_partitions=6)
    c = gg.Graph.load(path, 1 << 14, weighted=True, symmetric=True, force_partitions=3)
    d = gg.Graph.load(path, 1 << 14, weighted=True, symmetric=True)
    assert b.build["partitions"] > 1 and b.build["build_ms"] > 0
    same_adjacency(a, b)
    same_adjacency(c, d)


@pytest.mark.parametrize("partitioned", [False, True])
def test_host_adjacency_toolkits(partitioned):
    """Neighbour and weight arrays in mapped host memory: every toolkit gives
    the device-resident graph's results."""
    rec = records(14, 31, True)
    V = 1 << 14
    kw = {"force_partitions": 4} if partitioned else {}
    dev = gg.Graph.from_records(rec, V, weighted=True)
    host = gg.Graph.from_records(rec, V, weighted=True, adjacency_host=True, **kw)
    ih, idv = host.info(), dev.info()
    assert ih["host_bytes"] >= 8 * ih["adj_entries"]
    assert ih["device_bytes"] < idv["device_bytes"]
    same_adjacency(dev, host)
    dev.set_pr_layout(0)
    out_deg = dev.out_degree()
    roots = [int(r) for r in np.nonzero(out_deg)[0][:3]]
    for r in roots:
        pd, _ = dev.bfs(r)
        ph, _ = host.bfs(r)
        assert np.array_equal(gg.levels_from_parents(pd, r), gg.levels_from_parents(ph, r))
        dd, _ = dev.sssp(r)
        dh, _ = host.sssp(r)
        assert np.array_equal(dd.view(np.uint32), dh.view(np.uint32))
        bd = dev.bc(r)
        bh = host.bc(r)
        np.testing.assert_allclose(bh[0], bd[0], rtol=1e-12, atol=0, equal_nan=True)
    rd = dev.pagerank(20)[0]
    rh = host.pagerank(20)[0]
    assert np.array_equal(rd, rh)
    lv_d = gg.bfs_batched(dev, roots)[0]
    lv_h = gg.bfs_batched(host, roots)[0]
    assert np.array_equal(lv_d, lv_h)


def test_host_adjacency_cc_symmetric():
    rec = records(14, 41, False)
    V = 1 << 14
    dev = gg.Graph.from_records(rec, V, symmetric=True)
    host = gg.Graph.from_records(rec, V, symmetric=True, adjacency_host=True, force_partitions=3)
    same_adjacency(dev, host)
    assert np.array_equal(dev.cc()[0], host.cc()[0])
