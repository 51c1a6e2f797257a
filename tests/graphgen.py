"""Seeded synthetic edge lists (numpy restatement used by the tests).

The product library generates the same edge lists in C++ (host) and CUDA
(device); tests/test_generator.py checks all three agree bit for bit.

R-MAT (Chakrabarti, Zhan, Faloutsos 2004): each edge picks one quadrant per
level, most significant bit first, with probabilities a=0.57, b=0.19, c=0.19,
d=0.05 (b sets the destination bit, c the source bit).  Draws are
counter-based so any edge can be generated independently:

    key          = mix64(seed ^ 0x5851F42D4C957F2D)
    draw64(e, j) = mix64(key + (e * 64 + j) * 0x9E3779B97F4A7C15)      (mod 2**64)

where mix64 is the SplitMix64 finaliser (Steele, Lea, Flood 2014).  Level l
uses the low (l even) or high (l odd) 32 bits of draw64(e, l // 2), compared
against integer thresholds floor(p * 2**32).  The float32 weight of edge e is
(low32(draw64(e, 16)) >> 8) * 2**-24, uniform on [0, 1) and exact in float32.

Records are the reference's binary edge list (core/type.hpp:27-41,
README.md:24-26): packed {uint32 src, uint32 dst} or {uint32 src, uint32 dst,
float32 weight}.
"""
import numpy as np

GOLDEN = np.uint64(0x9E3779B97F4A7C15)
SEED_XOR = np.uint64(0x5851F42D4C957F2D)
T_A = np.uint64(2448131358)    # floor(0.57 * 2**32)
T_AB = np.uint64(3264175144)   # floor(0.76 * 2**32)
T_ABC = np.uint64(4080218931)  # floor(0.95 * 2**32)
WEIGHT_DRAW = 16


def mix64(z):
    z = np.asarray(z, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def _key(seed):
    return mix64(np.uint64(seed) ^ SEED_XOR)


def draw64(seed, e, j):
    e = np.asarray(e, dtype=np.uint64)
    with np.errstate(over="ignore"):
        return mix64(_key(seed) + (e * np.uint64(64) + np.uint64(j)) * GOLDEN)


def weights(seed, e):
    lo = draw64(seed, e, WEIGHT_DRAW) & np.uint64(0xFFFFFFFF)
    return (lo >> np.uint64(8)).astype(np.float32) * np.float32(2.0 ** -24)


def rmat(scale, edge_factor, seed, weighted=False):
    n = (1 << scale) * edge_factor
    e = np.arange(n, dtype=np.uint64)
    src = np.zeros(n, dtype=np.uint64)
    dst = np.zeros(n, dtype=np.uint64)
    for level in range(scale):
        d = draw64(seed, e, level // 2)
        u = (d >> np.uint64(32)) if (level & 1) else (d & np.uint64(0xFFFFFFFF))
        bit = np.uint64(scale - 1 - level)
        sbit = (u >= T_AB).astype(np.uint64)
        dbit = (((u >= T_A) & (u < T_AB)) | (u >= T_ABC)).astype(np.uint64)
        src |= sbit << bit
        dst |= dbit << bit
    src = src.astype(np.uint32)
    dst = dst.astype(np.uint32)
    w = weights(seed, e) if weighted else None
    return src, dst, w


def grid(n, seed=0, weighted=False):
    """n x n 4-neighbour grid, both directions; vertex id = r * n + c.

    Records in row-major vertex order: (v, v+1), (v+1, v) when c+1 < n, then
    (v, v+n), (v+n, v) when r+1 < n.  4 n (n-1) records in all.
    """
    r, c = np.meshgrid(np.arange(n, dtype=np.int64), np.arange(n, dtype=np.int64), indexing="ij")
    v = (r * n + c).ravel()
    has_right = (c + 1 < n).ravel()
    has_down = (r + 1 < n).ravel()
    cnt = 2 * has_right.astype(np.int64) + 2 * has_down.astype(np.int64)
    start = np.concatenate([[0], np.cumsum(cnt)[:-1]])
    total = int(cnt.sum())
    src = np.empty(total, dtype=np.uint32)
    dst = np.empty(total, dtype=np.uint32)
    vr = v[has_right]
    sr = start[has_right]
    src[sr], dst[sr] = vr, vr + 1
    src[sr + 1], dst[sr + 1] = vr + 1, vr
    vd = v[has_down]
    sd = start[has_down] + 2 * has_right[has_down].astype(np.int64)
    src[sd], dst[sd] = vd, vd + n
    src[sd + 1], dst[sd + 1] = vd + n, vd
    w = weights(seed, np.arange(total, dtype=np.uint64)) if weighted else None
    return src, dst, w


def to_records(src, dst, w=None):
    """Packs the reference's on-disk records (8 B, or 12 B with a weight)."""
    if w is None:
        rec = np.empty(len(src), dtype=[("s", "<u4"), ("d", "<u4")])
    else:
        rec = np.empty(len(src), dtype=[("s", "<u4"), ("d", "<u4"), ("w", "<f4")])
        rec["w"] = w
    rec["s"] = src
    rec["d"] = dst
    return rec.tobytes()


def from_records(buf, weighted):
    unit = 12 if weighted else 8
    n = len(buf) // unit
    buf = buf[: n * unit]
    if weighted:
        rec = np.frombuffer(buf, dtype=[("s", "<u4"), ("d", "<u4"), ("w", "<f4")])
        return rec["s"].copy(), rec["d"].copy(), rec["w"].copy()
    rec = np.frombuffer(buf, dtype=[("s", "<u4"), ("d", "<u4")])
    return rec["s"].copy(), rec["d"].copy(), None


def pick_root(src, V, seed):
    """Seeded uniform draw of a root with out-degree > 0."""
    outdeg = np.bincount(src, minlength=V)
    rng = np.random.default_rng(seed)
    for _ in range(100000):
        r = int(rng.integers(0, V))
        if outdeg[r] > 0:
            return r
    raise ValueError("no vertex with out-degree > 0")
