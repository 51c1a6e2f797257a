"""CPU model of the partitioned build's index arithmetic (gg_partition.cu).

Restates, in numpy, what the kernels compute: greedy ranges over the offsets
(oc_bounds), per (range, tile) counts and their range-major scan (oc_count),
groups of consecutive ranges, and the stable compaction order of oc_scatter
(warp w of a 4096-entry tile owns entries [w*512, +512), 16 rounds of 32
lanes, peers of one range ranked in lane order).  The model must reproduce
the in-core build's stable sort on (major, minor) exactly, weights included,
and every write must land on a distinct slot inside its group buffer.
"""
import numpy as np
import pytest

TILE, WARPS, WARP_ENTRIES, ROUNDS, GROUP, MAX_PARTS = 4096, 8, 512, 16, 32, 1024


def entries(rec, mode):
    s, d = rec[:, 0], rec[:, 1]
    w = rec[:, 2] if rec.shape[1] == 3 else np.zeros(len(rec), np.uint32)
    if mode == 0:
        return s, d, w
    if mode == 1:
        return d, s, w
    return np.concatenate([s, d]), np.concatenate([d, s]), np.concatenate([w, w])


def bits_for(V):
    b = 1
    while b < 32 and (1 << b) < V:
        b += 1
    return b


def in_core(rec, V, mode):
    maj, mnr, w = entries(rec, mode)
    keys = (maj.astype(np.uint64) << np.uint64(bits_for(V))) | mnr.astype(np.uint64)
    order = np.argsort(keys, kind="stable")
    off = np.zeros(V + 1, np.uint64)
    off[1:] = np.cumsum(np.bincount(maj, minlength=V)[:V])
    return off, mnr[order], w[order]


def greedy_bounds(off, V, cap):
    a, bounds = 0, [0]
    while a < V:
        assert len(bounds) <= MAX_PARTS
        lim = int(off[a]) + cap
        b = a + 1 if off[a + 1] > lim else int(np.searchsorted(off, lim, side="right")) - 1
        bounds.append(max(b, a + 1))
        a = bounds[-1]
    return bounds


def partitioned(rec, V, mode, force):
    maj, mnr, w = entries(rec, mode)
    n, bits = len(maj), bits_for(V)
    off = np.zeros(V + 1, np.uint64)
    off[1:] = np.cumsum(np.bincount(maj, minlength=V)[:V])
    cap = max((n + force - 1) // force, 1)
    gcap = 4 * cap
    bounds = greedy_bounds(off, V, cap)
    base = [int(off[b]) for b in bounds]
    nparts = len(bounds) - 1
    ntiles = (n + TILE - 1) // TILE
    part = np.searchsorted(np.array(bounds[:-1]), maj, side="right") - 1
    counts = np.zeros(nparts * ntiles, np.int64)
    np.add.at(counts, part * ntiles + np.arange(n) // TILE, 1)
    scanned = np.concatenate([[0], np.cumsum(counts)])
    groups, gsum = [0], 0
    for p in range(nparts):
        np_ = base[p + 1] - base[p]
        if p > groups[-1] and (p - groups[-1] == GROUP or gsum + np_ > gcap):
            groups.append(p)
            gsum = 0
        gsum += np_
    groups.append(nparts)
    nbr = np.zeros(n, np.uint32)
    wout = np.zeros(n, np.uint32)
    # build order inside a tile: warp-major, then round, then lane
    lane_order = np.arange(TILE).reshape(WARPS, ROUNDS, 32).reshape(-1)
    for g0, g1 in zip(groups[:-1], groups[1:]):
        gn = base[g1] - base[g0]
        if gn == 0:
            continue
        keys = np.zeros(gn, np.uint64)
        vals = np.zeros(gn, np.uint32)
        written = np.zeros(gn, bool)
        for t in range(ntiles):
            js = t * TILE + lane_order
            js = js[js < n]
            inside = (part[js] >= g0) & (part[js] < g1)
            for p in range(g0, g1):
                sel = js[inside & (part[js] == p)]
                at = (base[p] - base[g0]) + (scanned[p * ntiles + t] - scanned[p * ntiles]) + np.arange(len(sel))
                assert np.all(at < gn) and not written[at].any()
                written[at] = True
                keys[at] = ((maj[sel] - bounds[p]).astype(np.uint64) << np.uint64(bits)) | mnr[sel].astype(np.uint64)
                vals[at] = w[sel]
        assert written.all()
        for p in range(g0, g1):
            lo, hi = base[p] - base[g0], base[p + 1] - base[g0]
            k, v = keys[lo:hi], vals[lo:hi]
            o = np.argsort(k, kind="stable")
            nbr[base[p]:base[p + 1]] = (k[o] & np.uint64((1 << bits) - 1)).astype(np.uint32)
            wout[base[p]:base[p + 1]] = v[o]
    return off, nbr, wout, nparts, len(groups) - 1


def skewed_records(V, E, weighted, seed):
    rng = np.random.default_rng(seed)
    s = rng.integers(0, V, E, dtype=np.uint32)
    d = rng.integers(0, V, E, dtype=np.uint32)
    s[: E // 3] = rng.integers(0, 3, E // 3)   # hub lists longer than a range
    d[: E // 4] = rng.integers(0, 2, E // 4)   # duplicate edges with other weights
    cols = [s, d]
    if weighted:
        cols.append(rng.integers(0, 2 ** 32, E, dtype=np.uint64).astype(np.uint32))
    return np.stack(cols, 1)


@pytest.mark.parametrize("V,E,weighted,mode,force", [
    (50, 9000, True, 0, 5), (50, 9000, True, 1, 40), (37, 5000, True, 2, 3),
    (1000, 12000, False, 0, 100), (7, 300, True, 2, 256), (3000, 4096, True, 1, 2), (64, 0, True, 0, 4)])
def test_partitioned_model_equals_in_core(V, E, weighted, mode, force):
    rec = skewed_records(V, E, weighted, seed=V + E) if E else np.zeros((0, 3 if weighted else 2), np.uint32)
    off, nbr, w = in_core(rec, V, mode)
    off2, nbr2, w2, nparts, ngroups = partitioned(rec, V, mode, force)
    assert np.array_equal(off, off2) and np.array_equal(nbr, nbr2) and np.array_equal(w, w2)
    assert 1 <= ngroups <= nparts <= MAX_PARTS


def plan(V, n, weighted, budget, tile=4096, max_parts=1024):
    """build_plan's sizing arithmetic (gg_partition.cu): the (range, tile)
    count table sized for `ranges`, a group buffer of gcap entries, one
    range's sort buffer and digit counts of cap = gcap / 4 entries."""
    tiles = (n + tile - 1) // tile
    kv = 8 + (4 if weighted else 0)
    ranges = 64
    while True:
        fixed = V * 8 + tiles * 8 * ranges + (64 << 20)
        avail = budget - fixed if budget > fixed else 0
        gcap = avail * 4 // (4 * kv + kv + 1)
        cap = gcap // 4
        if cap == 0:
            return cap, gcap, ranges, fixed
        need = min(2 * n // cap + 1, max_parts)
        if need <= ranges:
            return cap, gcap, ranges, fixed
        ranges = need


@pytest.mark.parametrize("weighted", [False, True])
@pytest.mark.parametrize("V,n", [(1 << 20, 1 << 24), (1 << 24, 1 << 28), (1 << 26, 1 << 30), (1 << 26, 1 << 31)])
@pytest.mark.parametrize("budget_mb", [200, 300, 600, 1000, 4000, 16000])
def test_build_plan_stays_within_budget(V, n, weighted, budget_mb):
    budget = budget_mb << 20
    cap, gcap, ranges, fixed = plan(V, n, weighted, budget)
    if cap < (1 << 16) and cap < n:
        return                                        # refused: GG_ERR_NOMEM
    kv = 8 + (4 if weighted else 0)
    planned = fixed + gcap * kv + cap * kv + cap      # group buffer, sort buffer, digit counts
    assert planned <= budget
    # the count table holds every range that cap implies (capped at the kernel's maximum)
    assert min(2 * n // cap + 1, 1024) <= ranges
