"""ctypes front end of the CPU oracle (oracle/gg_oracle.c) -- TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
import this module, and only as the checker.  `build()` compiles the oracle
with gcc into oracle/liboracle.so.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
_lib = None


def build(force=False):
    src = os.path.join(HERE, "gg_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-O2", "-std=c99", "-shared", "-fPIC", "-o", LIB_PATH, src, "-lm"])
    return LIB_PATH


class _Trace(ctypes.Structure):
    _fields_ = [("capacity", ctypes.c_int), ("count", ctypes.c_int),
                ("mode", ctypes.c_void_p), ("active_edges", ctypes.c_void_p),
                ("activated", ctypes.c_void_p)]


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        vp, u32, u64, i32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
        L.orc_build.argtypes = [u32, u64, vp, vp, vp, i32, ctypes.POINTER(vp)]
        L.orc_build.restype = i32
        L.orc_free.argtypes = [vp]
        L.orc_num_adj.argtypes = [vp]
        L.orc_num_adj.restype = u64
        L.orc_get_adj.argtypes = [vp, i32, vp, vp, vp, vp]
        L.orc_rmat_records.argtypes = [u32, u64, i32, u64, u64, vp]
        L.orc_grid_records.argtypes = [u32, u64, i32, u64, u64, vp]
        L.orc_grid_count.argtypes = [u32]
        L.orc_grid_count.restype = u64
        L.orc_count_out_degree.argtypes = [vp, u64, i32, vp]
        L.orc_tree_levels.argtypes = [vp, u32, u32, vp]
        L.orc_tree_levels.restype = i32
        L.orc_tree_bad_edges.argtypes = [vp, vp, u32]
        L.orc_tree_bad_edges.restype = u64
        for name, extra in (("orc_bfs", [u32, vp]), ("orc_pagerank", [i32, vp, vp]), ("orc_cc", [vp]),
                            ("orc_sssp", [u32, vp]), ("orc_bc", [u32, vp, vp])):
            f = getattr(L, name)
            f.argtypes = [vp] + extra + [ctypes.POINTER(_Trace)]
            f.restype = i32
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class Trace:
    """Per-process_edges record: mode (0 sparse / 1 dense), active_edges, activated."""

    def __init__(self, capacity=1 << 16):
        self.mode = np.zeros(capacity, np.int32)
        self.active_edges = np.zeros(capacity, np.uint64)
        self.activated = np.zeros(capacity, np.uint64)
        self.t = _Trace(capacity, 0, self.mode.ctypes.data, self.active_edges.ctypes.data,
                        self.activated.ctypes.data)

    def rows(self):
        n = min(self.t.count, len(self.mode))
        return [(int(self.mode[i]), int(self.active_edges[i]), int(self.activated[i])) for i in range(n)]


class OracleGraph:
    def __init__(self, V, src, dst, w=None, symmetric=False):
        L = lib()
        self.V = int(V)
        self.src = np.ascontiguousarray(src, np.uint32)
        self.dst = np.ascontiguousarray(dst, np.uint32)
        self.w = None if w is None else np.ascontiguousarray(w, np.float32)
        self.E = len(self.src)
        self.symmetric = bool(symmetric)
        h = ctypes.c_void_p()
        rc = L.orc_build(self.V, self.E, _ptr(self.src), _ptr(self.dst), _ptr(self.w), int(symmetric),
                         ctypes.byref(h))
        if rc != 0:
            raise ValueError("vertex id out of range")
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_free(self.h)
            self.h = None

    def adjacency(self, incoming=False):
        n = int(lib().orc_num_adj(self.h))
        off = np.zeros(self.V + 1, np.uint64)
        nbr = np.zeros(max(n, 1), np.uint32)
        w = np.zeros(max(n, 1), np.float32) if self.w is not None else None
        deg = np.zeros(self.V, np.uint32)
        lib().orc_get_adj(self.h, int(incoming), _ptr(off), _ptr(nbr), _ptr(w), _ptr(deg))
        return off, nbr[:n], (None if w is None else w[:n]), deg

    def bfs(self, root):
        parent = np.zeros(self.V, np.uint32)
        tr = Trace()
        rc = lib().orc_bfs(self.h, root, _ptr(parent), ctypes.byref(tr.t))
        if rc < 0:
            raise ValueError("bad root")
        return parent, tr.rows()

    def pagerank(self, iterations):
        ranks = np.zeros(self.V, np.float64)
        deltas = np.zeros(max(iterations, 1), np.float64)
        tr = Trace()
        lib().orc_pagerank(self.h, iterations, _ptr(ranks), _ptr(deltas), ctypes.byref(tr.t))
        return ranks, deltas[:iterations], tr.rows()

    def cc(self):
        label = np.zeros(self.V, np.uint32)
        tr = Trace()
        lib().orc_cc(self.h, _ptr(label), ctypes.byref(tr.t))
        return label, tr.rows()

    def sssp(self, root):
        dist = np.zeros(self.V, np.float32)
        tr = Trace()
        rc = lib().orc_sssp(self.h, root, _ptr(dist), ctypes.byref(tr.t))
        if rc < 0:
            raise ValueError("bad root or unweighted graph")
        return dist, tr.rows()

    def tree_bad_edges(self, parent, root):
        """Reached vertices whose parent edge is not an edge of this graph."""
        parent = np.ascontiguousarray(parent, np.uint32)
        return int(lib().orc_tree_bad_edges(self.h, _ptr(parent), int(root)))

    def bc(self, root):
        dep = np.zeros(self.V, np.float64)
        inv = np.zeros(self.V, np.float64)
        tr = Trace()
        rc = lib().orc_bc(self.h, root, _ptr(dep), _ptr(inv), ctypes.byref(tr.t))
        if rc < 0:
            raise ValueError("bad root")
        return dep, inv, tr.rows()


def bfs_levels(parent, root):
    """Level of every vertex in a parent tree (-1 when unreached); raises if
    the array is not a tree rooted at `root`."""
    V = len(parent)
    parent = parent.astype(np.int64)
    level = np.full(V, -1, np.int64)
    if parent[root] != root:
        raise AssertionError("root is not its own parent")
    level[root] = 0
    reached = np.nonzero(parent < V)[0]
    order = [root]
    children = {}
    for v in reached:
        if v != root:
            children.setdefault(int(parent[v]), []).append(int(v))
    i = 0
    while i < len(order):
        u = order[i]
        for c in children.get(u, ()):
            level[c] = level[u] + 1
            order.append(c)
        i += 1
    if len(order) != len(reached):
        raise AssertionError("parent array has a cycle or a dangling parent")
    return level


def bfs_reference_levels(V, src, dst, root):
    """Plain queue BFS over out-edges: the level of every vertex (-1 unreached)."""
    order = np.argsort(src, kind="stable")
    s = np.asarray(src)[order]
    d = np.asarray(dst)[order].astype(np.int64)
    off = np.zeros(V + 1, np.int64)
    np.add.at(off, s.astype(np.int64) + 1, 1)
    off = np.cumsum(off)
    level = np.full(V, -1, np.int64)
    level[root] = 0
    frontier = np.array([root], np.int64)
    k = 0
    while len(frontier):
        k += 1
        nb = np.concatenate([d[off[u]:off[u + 1]] for u in frontier]) if len(frontier) else np.array([], np.int64)
        nb = np.unique(nb)
        nb = nb[level[nb] < 0]
        level[nb] = k
        frontier = nb
    return level


# ---------------------------------------------------------------- inputs
RMAT, GRID = 0, 1


def record_count(kind, p1, p2):
    """Records of R-MAT (p1 = scale, p2 = edge factor) or of the p1 x p1 grid."""
    return (1 << p1) * p2 if kind == RMAT else int(lib().orc_grid_count(p1))


def records(kind, p1, p2, seed, weighted=False, first=0, count=None, threads=1):
    """Packed edge-list records [first, first + count) as a uint32 array of
    2 (3 when weighted) words per record, from the oracle's own restatement of
    the benchmark generator (orc_rmat_records / orc_grid_records).  Threads
    split the range; ctypes releases the GIL during each call."""
    n = record_count(kind, p1, p2)
    count = n - first if count is None else count
    words = 3 if weighted else 2
    out = np.empty(count * words, np.uint32)
    fn = lib().orc_rmat_records if kind == RMAT else lib().orc_grid_records

    def part(lo, hi):
        if hi > lo:
            fn(p1, seed, int(weighted), first + lo, hi - lo,
               ctypes.c_void_p(out.ctypes.data + lo * words * 4))

    threads = max(1, int(threads))
    if threads == 1 or count < (1 << 16):
        part(0, count)
    else:
        from concurrent.futures import ThreadPoolExecutor
        step = (count + threads - 1) // threads
        with ThreadPoolExecutor(threads) as ex:
            list(ex.map(lambda i: part(i * step, min(count, (i + 1) * step)), range(threads)))
    return out


def write_records_file(path, kind, p1, p2, seed, weighted=False, threads=1, chunk=1 << 26):
    """Writes the whole edge list to `path` chunk by chunk and returns
    (vertices, records, out_degree uint32[V]) without holding the list."""
    n = record_count(kind, p1, p2)
    V = (1 << p1) if kind == RMAT else p1 * p1
    words = 3 if weighted else 2
    deg = np.zeros(V, np.uint32)
    with open(path, "wb") as f:
        for first in range(0, n, chunk):
            c = min(chunk, n - first)
            rec = records(kind, p1, p2, seed, weighted, first, c, threads)
            lib().orc_count_out_degree(_ptr(rec), c, words, _ptr(deg))
            rec.tofile(f)
    return V, n, deg


def pick_roots(out_degree, count, seed):
    """Seeded uniform draws among the vertices with out-degree > 0: the
    benchmark's root rule, restated so that the CPU baseline draws the GPU
    run's roots without the product library."""
    rng = np.random.default_rng(seed)
    cand = np.nonzero(np.asarray(out_degree) > 0)[0]
    if len(cand) == 0:
        raise ValueError("no vertex with out-degree > 0")
    return [int(x) for x in cand[rng.integers(0, len(cand), count)]]


def tree_levels(parent, root):
    """bfs_levels in C for large graphs: levels of the parent tree (-1
    unreached); raises if the array is not a tree rooted at `root`."""
    parent = np.ascontiguousarray(parent, np.uint32)
    level = np.empty(len(parent), np.int32)
    if lib().orc_tree_levels(_ptr(parent), len(parent), int(root), _ptr(level)) != 0:
        raise AssertionError("parent array is not a tree rooted at %d" % root)
    return level
