"""The level-list room rule of the batched BFS (gg_batched.cu), restated in
numpy and checked on the CPU: in a pull step every warp of the two pull
kernels appends the entries of its vertex groups (at most 32 per group)
through a cursor that takes LIST_CHUNK slots from the step's counter when the
group does not fit in what it holds, blanks what it leaves, and blanks its
tail at the end.  The host makes room for 2 V + 2 * SMs * 64 * LIST_CHUNK
slots before the step; the slots a step takes must never exceed that."""
import numpy as np
import pytest

LIST_CHUNK = 256
WARPS_PER_SM = 64  # 8 blocks of 256 threads


def slots_taken(counts, warps):
    """Slots taken when `warps` warps walk the vertex groups grid-strided,
    group i holding counts[i] entries (the ListCursor rule)."""
    total = 0
    for w in range(min(warps, len(counts))):
        nxt = end = 0
        for c in counts[w::warps]:
            if c == 0:
                continue
            if end - nxt < c:
                nxt = total
                end = total + LIST_CHUNK
                total += LIST_CHUNK
            nxt += c
    return total


def room(V, sms):
    return 2 * V + 2 * sms * WARPS_PER_SM * LIST_CHUNK


@pytest.mark.parametrize("V", [1, 31, 4000, 100_000, 1 << 20])
@pytest.mark.parametrize("pattern", ["full", "one", "thirtyone", "random", "sparse"])
def test_pull_step_stays_in_room(V, pattern):
    sms = 152
    groups = (V + 31) // 32
    rng = np.random.default_rng(V)
    last = V - 32 * (groups - 1)
    if pattern == "full":
        counts = np.full(groups, 32)
    elif pattern == "one":
        counts = np.ones(groups, np.int64)
    elif pattern == "thirtyone":
        counts = np.full(groups, 31)
    elif pattern == "random":
        counts = rng.integers(0, 33, groups)
    else:
        counts = (rng.random(groups) < 0.01).astype(np.int64) * rng.integers(1, 33, groups)
    counts[-1] = min(counts[-1], last)
    warps = sms * WARPS_PER_SM
    # the light-list kernel over all vertices, then the long-list finish
    # over a tenth of them, in the same step
    big = counts[: max(1, groups // 10)]
    taken = slots_taken(counts.tolist(), warps) + slots_taken(big.tolist(), warps)
    assert counts.sum() + big.sum() <= 2 * V
    assert taken <= room(V, sms)


def test_room_outgrows_sixteen_per_vertex_on_small_graphs():
    """Below a few hundred thousand vertices the worst-case room is more than
    16 entries per vertex, so the lists move into the rows at the first step
    (what the small-graph GPU tests exercise); at a million vertices they stay."""
    sms = 152
    assert room(4000, sms) > 16 * 4000 + 64
    assert room(1 << 15, sms) > 16 * (1 << 15) + 64
    assert room(1 << 20, sms) <= 16 * (1 << 20) + 64
