"""GB300-native edge-processing engine for Gemini graphs (Python front end).

A thin ctypes layer over the C ABI in include/gemini_gb300.h
(libgemini_gb300.so, built in-tree by geminigraph_gb300/build.py).  There is
no CPU fallback: if the library is missing or no GPU is present, calls raise.

    g = Graph.load("graph.bin", vertices)            # Graph::load_directed
    g = Graph.load("graph.bin", vertices, symmetric=True)
    parent, stats = g.bfs(root)                      # toolkits/bfs.cpp
"""
import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
# GG_LIBRARY=check selects libgemini_gb300_check.so, the build with device
# bounds checks (a failed check makes the call return GG_ERR_CHECK)
LIB_PATH = os.path.join(PKG, "libgemini_gb300_check.so" if os.environ.get("GG_LIBRARY") == "check"
                        else "libgemini_gb300.so")

GG_OK = 0
STATUS = {1: "invalid argument", 2: "I/O error", 3: "vertex id out of range", 4: "CUDA error",
          5: "out of memory", 6: "graph is unweighted", 7: "graph too large", 8: "capacity exceeded",
          9: "device bounds check failed"}

RMAT, GRID = 0, 1

_lib = None


class GeminiError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class _Info(ctypes.Structure):
    _fields_ = [("vertices", ctypes.c_uint32), ("edges", ctypes.c_uint64), ("adj_entries", ctypes.c_uint64),
                ("weighted", ctypes.c_int32), ("symmetric", ctypes.c_int32), ("transposed", ctypes.c_int32),
                ("device", ctypes.c_int32), ("device_bytes", ctypes.c_uint64), ("host_bytes", ctypes.c_uint64)]


class _BuildOptions(ctypes.Structure):
    _fields_ = [("build_budget", ctypes.c_uint64), ("adjacency_host", ctypes.c_int32),
                ("force_partitions", ctypes.c_int32), ("partitions", ctypes.c_uint32),
                ("record_passes", ctypes.c_uint32), ("build_ms", ctypes.c_double)]


class _Stats(ctypes.Structure):
    _fields_ = [("trace_capacity", ctypes.c_int32), ("calls", ctypes.c_int32),
                ("mode", ctypes.c_void_p), ("active_edges", ctypes.c_void_p), ("activated", ctypes.c_void_p),
                ("call_ms", ctypes.c_void_p), ("active_edges_total", ctypes.c_uint64), ("device_ms", ctypes.c_double),
                ("kernel_launches", ctypes.c_int32)]


def library():
    """Loads libgemini_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: run python -c 'import __graft_entry__ as g; g.build()'")
    L = ctypes.CDLL(LIB_PATH)
    vp, u32, u64, i32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
    pg = ctypes.POINTER(vp)
    sig = {
        "gg_last_error": ([], ctypes.c_char_p),
        "gg_host_alloc": ([u64, ctypes.POINTER(vp)], i32),
        "gg_host_free": ([vp], i32),
        "gg_graph_load": ([ctypes.c_char_p, u32, i32, i32, i32, pg], i32),
        "gg_graph_from_records": ([vp, u64, u32, i32, i32, i32, pg], i32),
        "gg_graph_from_device_records": ([vp, u64, u32, i32, i32, i32, pg], i32),
        "gg_graph_load_ex": ([ctypes.c_char_p, u32, i32, i32, i32, ctypes.POINTER(_BuildOptions), pg], i32),
        "gg_graph_from_records_ex": ([vp, u64, u32, i32, i32, i32, ctypes.POINTER(_BuildOptions), pg], i32),
        "gg_graph_generate_ex": ([i32, u32, u32, u64, i32, i32, i32, ctypes.POINTER(_BuildOptions), pg], i32),
        "gg_graph_generate": ([i32, u32, u32, u64, i32, i32, i32, pg], i32),
        "gg_generate_count": ([i32, u32, u32], u64),
        "gg_generate_records": ([i32, u32, u32, u64, i32, vp, i32], i32),
        "gg_graph_free": ([vp], i32),
        "gg_graph_info_get": ([vp, ctypes.POINTER(_Info)], i32),
        "gg_graph_transpose": ([vp], i32),
        "gg_graph_adjacency": ([vp, i32, vp, vp, vp, vp], i32),
        "gg_bfs": ([vp, u32, vp, ctypes.POINTER(_Stats)], i32),
        "gg_pagerank": ([vp, i32, vp, vp, ctypes.POINTER(_Stats)], i32),
        "gg_pagerank_f32": ([vp, i32, vp, vp, ctypes.POINTER(_Stats)], i32),
        "gg_cc": ([vp, vp, ctypes.POINTER(_Stats)], i32),
        "gg_sssp": ([vp, u32, vp, ctypes.POINTER(_Stats)], i32),
        "gg_bc": ([vp, u32, vp, vp, ctypes.POINTER(_Stats)], i32),
        "gg_result_device_ptr": ([vp, i32], vp),
        "gg_active_edges": ([vp, vp, ctypes.POINTER(u64)], i32),
        "gg_is_sparse": ([u64, u64], i32),
        "gg_active_edges_noalloc": ([vp, vp, u32, vp, vp], i32),
        "gg_bfs_batched": ([vp, vp, i32, vp, vp, vp, vp, ctypes.POINTER(_Stats)], i32),
        "gg_result_checksum": ([vp, u32, i32], u64),
        "gg_levels_from_parents": ([vp, u32, u32, vp], i32),
        "gg_server_create": ([i32, u64, pg], i32),
        "gg_server_add_graph": ([vp, vp, ctypes.POINTER(i32)], i32),
        "gg_server_submit": ([vp, i32, i32, u32, ctypes.POINTER(u64)], i32),
        "gg_server_wait": ([vp, ctypes.POINTER(_QueryResult), i32, i32, ctypes.POINTER(i32)], i32),
        "gg_server_stats_get": ([vp, ctypes.POINTER(_ServerStats)], i32),
        "gg_server_free": ([vp], i32),
        "gg_server_set_window": ([vp, i32, ctypes.c_double], i32),
        "gg_server_set_solo": ([vp, i32], i32),
        "gg_pool_bytes": ([vp, i32], u64),
        "gg_graph_set_bins": ([vp, u32, u32, u32], i32),
        "gg_bfs_many": ([vp, vp, i32, vp, ctypes.POINTER(_Stats)], i32),
        "gg_graph_set_sssp_delta": ([vp, ctypes.c_float], i32),
        "gg_graph_set_batched_switch": ([vp, u32], i32),
        "gg_graph_set_batched_thread_lanes": ([vp, u32], i32),
        "gg_graph_set_batched_graph": ([vp, i32], i32),
        "gg_graph_set_batched_lists": ([vp, i32], i32),
        "gg_dump_vertex_array": ([vp, u64, u32, ctypes.c_char_p], i32),
        "gg_restore_vertex_array": ([vp, u64, u32, ctypes.c_char_p], i32),
        "gg_bc_batched": ([vp, vp, i32, vp, vp, vp, ctypes.POINTER(_Stats)], i32),
        "gg_graph_set_pr_layout": ([vp, i32], i32),
        "gg_graph_set_l1_hot": ([vp, u32], i32),
        "gg_graph_set_dense_push": ([vp, u32], i32),
        "gg_graph_set_pull_split": ([vp, u32], i32),
        "gg_graph_set_bfs_pull": ([vp, u32], i32),
        "gg_autotune": ([vp, u32, ctypes.c_char_p, ctypes.POINTER(_TuneResult)], i32),
        "gg_sssp_batched": ([vp, vp, i32, vp, vp, ctypes.POINTER(_Stats)], i32),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def _check(rc):
    if rc != GG_OK:
        raise GeminiError(rc, library().gg_last_error().decode())


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class _QueryResult(ctypes.Structure):
    _fields_ = [("ticket", ctypes.c_uint64), ("graph", ctypes.c_int32), ("kind", ctypes.c_int32),
                ("root", ctypes.c_uint32), ("status", ctypes.c_int32), ("reached", ctypes.c_uint64),
                ("checksum", ctypes.c_uint64), ("active_edges", ctypes.c_uint64), ("latency_ms", ctypes.c_double)]


class _ServerStats(ctypes.Structure):
    _fields_ = [("completed", ctypes.c_uint64), ("pending", ctypes.c_uint64), ("pools_open", ctypes.c_uint64),
                ("pools_opened", ctypes.c_uint64), ("pools_closed", ctypes.c_uint64),
                ("admission_waits", ctypes.c_uint64), ("bytes_in_use", ctypes.c_uint64), ("budget", ctypes.c_uint64),
                ("max_busy_pools", ctypes.c_int32), ("max_lanes_in_use", ctypes.c_int32),
                ("solo_runs", ctypes.c_uint64)]


class _TuneResult(ctypes.Structure):
    _fields_ = [("light_deg", ctypes.c_uint32), ("pull_chunk", ctypes.c_uint32), ("pull_vector", ctypes.c_uint32),
                ("best_ms", ctypes.c_double),
                ("default_ms", ctypes.c_double), ("candidates", ctypes.c_int32), ("from_cache", ctypes.c_int32),
                ("l1_hot_bytes", ctypes.c_uint32), ("pull_split", ctypes.c_uint32), ("bfs_pull", ctypes.c_uint32)]


class RunStats:
    """Per-call trace of one toolkit run: mode (0 sparse, 1 dense),
    active_edges and activated per process_edges call."""

    def __init__(self, capacity=1 << 16):
        self.mode = np.zeros(capacity, np.int32)
        self.active_edges = np.zeros(capacity, np.uint64)
        self.activated = np.zeros(capacity, np.uint64)
        self.call_ms = None
        self.s = _Stats(capacity, 0, self.mode.ctypes.data, self.active_edges.ctypes.data,
                        self.activated.ctypes.data, None, 0, 0.0, 0)

    def enable_call_timing(self):
        """Ask for the device time of each call's edge kernel (CUDA events)."""
        self.call_ms = np.zeros(len(self.mode), np.float64)
        self.s.call_ms = self.call_ms.ctypes.data
        return self

    @property
    def calls(self):
        return self.s.calls

    @property
    def device_ms(self):
        return self.s.device_ms

    @property
    def active_edges_total(self):
        return int(self.s.active_edges_total)

    @property
    def kernel_launches(self):
        return self.s.kernel_launches

    def rows(self, with_ms=False):
        n = min(self.s.calls, len(self.mode))
        if with_ms and self.call_ms is not None:
            return [(int(self.mode[i]), int(self.active_edges[i]), int(self.activated[i]),
                     round(float(self.call_ms[i]), 4)) for i in range(n)]
        return [(int(self.mode[i]), int(self.active_edges[i]), int(self.activated[i])) for i in range(n)]


class PinnedArray:
    """A page-locked host array (gg_host_alloc) of n elements of dtype, and
    an optional second one of the same size (ptr2)."""

    def __init__(self, n, dtype, second=True):
        self.dtype = np.dtype(dtype)
        self.itemsize = self.dtype.itemsize
        self.n = n
        self._p = [ctypes.c_void_p(), ctypes.c_void_p()]
        for i in range(2 if second else 1):
            _check(library().gg_host_alloc(n * self.itemsize, ctypes.byref(self._p[i])))
        self.ptr = self._p[0]
        self.ptr2 = self._p[1] if second else None

    def array(self, which=0):
        buf = (ctypes.c_char * (self.n * self.itemsize)).from_address(self._p[which].value)
        return np.frombuffer(buf, self.dtype)

    def __del__(self):
        try:
            for p in self._p:
                if p:
                    library().gg_host_free(p)
        except Exception:
            pass


def generate_records(kind, p1, p2, seed, weighted=False, threads=0):
    """Host generator: the packed edge-list records of a seeded R-MAT
    (kind=RMAT, p1=scale, p2=edge factor) or grid (kind=GRID, p1=side)."""
    L = library()
    n = int(L.gg_generate_count(kind, p1, p2))
    unit = 12 if weighted else 8
    buf = np.empty(n * unit, np.uint8)
    _check(L.gg_generate_records(kind, p1, p2, seed, int(weighted), _ptr(buf), threads))
    return buf


class Graph:
    """One graph resident on one GPU (Graph<EdgeData>, core/graph.hpp:91)."""

    def __init__(self, handle, build=None):
        self.h = handle
        self._info = None
        # {"partitions": ranges per direction (1 = in-core), "build_ms": wall time}
        self.build = build

    # -- construction -------------------------------------------------------
    @staticmethod
    def _options(build_budget, adjacency_host, force_partitions):
        return _BuildOptions(build_budget=int(build_budget), adjacency_host=int(bool(adjacency_host)),
                             force_partitions=int(force_partitions))

    @classmethod
    def load(cls, path, vertices, weighted=False, symmetric=False, device=0, build_budget=0, adjacency_host=False,
             force_partitions=0):
        """Graph::load_directed / load_undirected_from_directed.  build_budget
        (device bytes beyond the graph, 0 = automatic), force_partitions and
        adjacency_host are the gg_build_options of gg_graph_load_ex."""
        h = ctypes.c_void_p()
        opt = cls._options(build_budget, adjacency_host, force_partitions)
        _check(library().gg_graph_load_ex(os.fsencode(path), vertices, int(weighted), int(symmetric), device,
                                          ctypes.byref(opt), ctypes.byref(h)))
        return cls(h, {"partitions": opt.partitions, "record_passes": opt.record_passes,
                       "build_ms": opt.build_ms})

    @classmethod
    def from_records(cls, records, vertices, weighted=False, symmetric=False, device=0, build_budget=0,
                     adjacency_host=False, force_partitions=0):
        buf = np.frombuffer(records, np.uint8) if isinstance(records, (bytes, bytearray)) else \
            np.ascontiguousarray(records).view(np.uint8)
        h = ctypes.c_void_p()
        opt = cls._options(build_budget, adjacency_host, force_partitions)
        _check(library().gg_graph_from_records_ex(_ptr(buf), buf.nbytes, vertices, int(weighted), int(symmetric),
                                                  device, ctypes.byref(opt), ctypes.byref(h)))
        return cls(h, {"partitions": opt.partitions, "record_passes": opt.record_passes,
                       "build_ms": opt.build_ms})

    @classmethod
    def from_edges(cls, vertices, src, dst, w=None, symmetric=False, device=0, **build):
        n = len(src)
        if w is None:
            rec = np.empty(n, dtype=[("s", "<u4"), ("d", "<u4")])
        else:
            rec = np.empty(n, dtype=[("s", "<u4"), ("d", "<u4"), ("w", "<f4")])
            rec["w"] = w
        rec["s"] = src
        rec["d"] = dst
        return cls.from_records(rec, vertices, weighted=w is not None, symmetric=symmetric, device=device, **build)

    @classmethod
    def generate(cls, kind, p1, p2, seed, weighted=False, symmetric=False, device=0, build_budget=0,
                 adjacency_host=False, force_partitions=0):
        h = ctypes.c_void_p()
        opt = cls._options(build_budget, adjacency_host, force_partitions)
        _check(library().gg_graph_generate_ex(kind, p1, p2, seed, int(weighted), int(symmetric), device,
                                              ctypes.byref(opt), ctypes.byref(h)))
        return cls(h, {"partitions": opt.partitions, "record_passes": opt.record_passes,
                       "build_ms": opt.build_ms})

    def close(self):
        if self.h:
            library().gg_graph_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- public fields ------------------------------------------------------
    def info(self):
        i = _Info()
        _check(library().gg_graph_info_get(self.h, ctypes.byref(i)))
        return {k: getattr(i, k) for k, _ in _Info._fields_}

    @property
    def vertices(self):
        return self.info()["vertices"]

    @property
    def edges(self):
        return self.info()["edges"]

    def set_bins(self, light_deg, pull_chunk, pull_vector=1):
        """Pull bins (gg_graph_set_bins): light-list bound, chunk size and the
        load flags (bit 0: chunk lanes read 16-byte windows; bit 1: light
        lanes read 32-byte windows)."""
        _check(library().gg_graph_set_bins(self.h, light_deg, pull_chunk, int(pull_vector)))

    def set_batched_switch(self, divisor):
        _check(library().gg_graph_set_batched_switch(self.h, int(divisor)))

    def set_batched_thread_lanes(self, lanes):
        """Batched SSSP steps with at most this many lanes in flight relax
        edges one thread per edge (gg_graph_set_batched_thread_lanes)."""
        _check(library().gg_graph_set_batched_thread_lanes(self.h, int(lanes)))

    def set_batched_graph(self, on):
        """Batched BFS / SSSP steps device-driven in one CUDA-graph launch per
        batch (True) or one host wait per step (False, the default;
        gg_graph_set_batched_graph)."""
        _check(library().gg_graph_set_batched_graph(self.h, 1 if on else 0))

    def set_batched_lists(self, on):
        """Batched BFS without parents keeps levels as per-step level lists
        (True, the default) or as per-vertex rows (gg_graph_set_batched_lists)."""
        _check(library().gg_graph_set_batched_lists(self.h, 1 if on else 0))

    def set_sssp_delta(self, delta):
        _check(library().gg_graph_set_sssp_delta(self.h, float(delta)))

    def bfs_many(self, roots, outputs):
        """Single-root BFS of each root in turn, result i copied into
        outputs[i] (a host array of V uint32, or None) while run i + 1
        computes; returns the summed RunStats."""
        r = np.ascontiguousarray(roots, np.uint32)
        ptrs = (ctypes.c_void_p * max(len(r), 1))(*[(o.ctypes.data if o is not None else None) for o in outputs])
        st = RunStats()
        _check(library().gg_bfs_many(self.h, _ptr(r), len(r), ctypes.cast(ptrs, ctypes.c_void_p), ctypes.byref(st.s)))
        return st

    def set_pr_layout(self, hot_sources):
        _check(library().gg_graph_set_pr_layout(self.h, 1 if hot_sources else 0))

    def set_l1_hot(self, l1_bytes):
        """Bytes of the most gathered sources' state the pulls cache in L1 on
        the hot-source layout (gg_graph_set_l1_hot)."""
        _check(library().gg_graph_set_l1_hot(self.h, int(l1_bytes)))

    def set_dense_push(self, divisor):
        """CC / SSSP dense calls with active out-edges below adjacency
        entries / divisor run as a push (0: always pull)."""
        _check(library().gg_graph_set_dense_push(self.h, int(divisor)))

    def set_bfs_pull(self, divisor):
        """BFS calls pull when active out-edges >= edges / divisor (default
        20, the reference's switch; gg_graph_set_bfs_pull)."""
        _check(library().gg_graph_set_bfs_pull(self.h, int(divisor)))

    def set_pull_split(self, light_blocks):
        """Light-list kernel blocks per SM beside the chunk kernel (1..7), or
        0 for both over the whole GPU (gg_graph_set_pull_split)."""
        _check(library().gg_graph_set_pull_split(self.h, int(light_blocks)))

    def autotune(self, cache_dir=None, objective=("pagerank", "bfs")):
        """Times the bin candidates on this graph for the named workloads
        ("pagerank", "pagerank_f64", "bfs", "batched", "sssp", "cc", "bc")
        and keeps the fastest; cached on disk."""
        names = {"pagerank": 1, "bfs": 2, "batched": 4, "sssp": 8, "cc": 16, "pagerank_f64": 32, "bc": 64}
        mask = 0
        for o in objective:
            mask |= names[o]
        r = _TuneResult()
        _check(library().gg_autotune(self.h, mask, os.fsencode(cache_dir) if cache_dir else None, ctypes.byref(r)))
        return {k: getattr(r, k) for k, _ in _TuneResult._fields_}

    def transpose(self):
        _check(library().gg_graph_transpose(self.h))

    def adjacency(self, incoming=False):
        inf = self.info()
        V, n = inf["vertices"], inf["adj_entries"]
        off = np.zeros(V + 1, np.uint64)
        nbr = np.zeros(max(n, 1), np.uint32)
        w = np.zeros(max(n, 1), np.float32) if inf["weighted"] else None
        deg = np.zeros(V, np.uint32)
        _check(library().gg_graph_adjacency(self.h, int(incoming), _ptr(off), _ptr(nbr), _ptr(w), _ptr(deg)))
        return off, nbr[:n], (None if w is None else w[:n]), deg

    def out_degree(self):
        deg = np.zeros(self.vertices, np.uint32)
        _check(library().gg_graph_adjacency(self.h, 0, None, None, None, _ptr(deg)))
        return deg

    def active_edges(self, bitmap64):
        out = ctypes.c_uint64()
        b = np.ascontiguousarray(bitmap64, np.uint64)
        _check(library().gg_active_edges(self.h, _ptr(b), ctypes.byref(out)))
        return int(out.value)

    # -- toolkits -------------------------------------------------------------
    def bfs(self, root, to_host=True):
        st = RunStats()
        parent = np.empty(self.vertices, np.uint32) if to_host else None
        _check(library().gg_bfs(self.h, root, _ptr(parent), ctypes.byref(st.s)))
        return parent, st

    def pagerank(self, iterations, to_host=True, f32=False):
        st = RunStats()
        V = self.vertices
        ranks = np.empty(V, np.float32 if f32 else np.float64) if to_host else None
        deltas = np.zeros(max(iterations, 1), np.float64)
        fn = library().gg_pagerank_f32 if f32 else library().gg_pagerank
        _check(fn(self.h, iterations, _ptr(ranks), _ptr(deltas), ctypes.byref(st.s)))
        return ranks, deltas[:iterations], st

    def cc(self, to_host=True):
        st = RunStats()
        label = np.empty(self.vertices, np.uint32) if to_host else None
        _check(library().gg_cc(self.h, _ptr(label), ctypes.byref(st.s)))
        return label, st

    def sssp(self, root, to_host=True):
        st = RunStats()
        dist = np.empty(self.vertices, np.float32) if to_host else None
        _check(library().gg_sssp(self.h, root, _ptr(dist), ctypes.byref(st.s)))
        return dist, st

    def bc(self, root, to_host=True):
        st = RunStats()
        V = self.vertices
        dep = np.empty(V, np.float64) if to_host else None
        inv = np.empty(V, np.float64) if to_host else None
        _check(library().gg_bc(self.h, root, _ptr(dep), _ptr(inv), ctypes.byref(st.s)))
        return dep, inv, st


def _roots_array(roots):
    r = np.ascontiguousarray(roots, np.uint32)
    if not 1 <= len(r) <= 64:
        raise ValueError("1..64 roots per batch")
    return r


def bfs_batched(g, roots, levels=True, parents=False, timing=False):
    """Multi-source BFS of up to 64 roots: (levels, parents, reached, lane_edges, stats);
    levels/parents are (len(roots), V) arrays or None."""
    r = _roots_array(roots)
    V = g.vertices
    lv = np.empty((len(r), V), np.int32) if levels else None
    pa = np.empty((len(r), V), np.uint32) if parents else None
    reached = np.zeros(len(r), np.uint64)
    edges = np.zeros(len(r), np.uint64)
    st = RunStats()
    if timing:
        st.enable_call_timing()
    _check(library().gg_bfs_batched(g.h, _ptr(r), len(r), _ptr(lv), _ptr(pa), _ptr(reached), _ptr(edges),
                                    ctypes.byref(st.s)))
    return lv, pa, reached, edges, st


def sssp_batched(g, roots, distances=True, timing=False):
    """Multi-source SSSP of up to 64 roots: (distances (len(roots), V) or None, reached, stats)."""
    r = _roots_array(roots)
    V = g.vertices
    dist = np.empty((len(r), V), np.float32) if distances else None
    reached = np.zeros(len(r), np.uint64)
    st = RunStats()
    if timing:
        st.enable_call_timing()
    _check(library().gg_sssp_batched(g.h, _ptr(r), len(r), _ptr(dist), _ptr(reached), ctypes.byref(st.s)))
    return dist, reached, st


def bc_batched(g, roots, outputs=True, timing=False):
    """Batched BC of up to 64 roots: (dependencies (len(roots), V), 1/num_paths
    (len(roots), V), reached, stats); the arrays are None when outputs=False."""
    r = _roots_array(roots)
    V = g.vertices
    dep = np.empty((len(r), V), np.float64) if outputs else None
    inv = np.empty((len(r), V), np.float64) if outputs else None
    reached = np.zeros(len(r), np.uint64)
    st = RunStats()
    if timing:
        st.enable_call_timing()
    _check(library().gg_bc_batched(g.h, _ptr(r), len(r), _ptr(dep), _ptr(inv), _ptr(reached), ctypes.byref(st.s)))
    return dep, inv, reached, st


def dump_vertex_array(array, path):
    """core/graph.hpp:253 with one partition: the array's bytes in `path`."""
    a = np.ascontiguousarray(array)
    _check(library().gg_dump_vertex_array(_ptr(a), a.itemsize, len(a), os.fsencode(path)))


def restore_vertex_array(path, vertices, dtype):
    """core/graph.hpp:289: a vertex array back from `path` (its length must match)."""
    a = np.empty(vertices, dtype)
    _check(library().gg_restore_vertex_array(_ptr(a), a.itemsize, vertices, os.fsencode(path)))
    return a


def result_checksum(values, kind):
    """gg_result_checksum of a level (kind 0, int32) or distance (kind 1, float32) array."""
    a = np.ascontiguousarray(values, np.int32 if kind == 0 else np.float32)
    return int(library().gg_result_checksum(_ptr(a), len(a), kind))


def levels_from_parents(parent, root):
    p = np.ascontiguousarray(parent, np.uint32)
    lv = np.empty(len(p), np.int32)
    _check(library().gg_levels_from_parents(_ptr(p), len(p), root, _ptr(lv)))
    return lv


class Server:
    """Continuous-batching BFS/SSSP server over resident graphs (gg_server_*)."""
    BFS, SSSP = 0, 1

    def __init__(self, device=0, hbm_budget=0):
        h = ctypes.c_void_p()
        _check(library().gg_server_create(device, hbm_budget, ctypes.byref(h)))
        self.h = h
        self.graphs = []

    @staticmethod
    def pool_bytes(graph, kind):
        return int(library().gg_pool_bytes(graph.h, kind))

    def set_solo(self, below):
        """Idle SSSP pools with fewer waiting queries run them alone (gg_server_set_solo)."""
        _check(library().gg_server_set_solo(self.h, int(below)))

    def set_window(self, kind, window_ms):
        """Batch window of the kind's pools (gg_server_set_window)."""
        _check(library().gg_server_set_window(self.h, kind, float(window_ms)))

    def add_graph(self, graph):
        gid = ctypes.c_int32()
        _check(library().gg_server_add_graph(self.h, graph.h, ctypes.byref(gid)))
        self.graphs.append(graph)
        return gid.value

    def submit(self, graph_id, kind, root):
        t = ctypes.c_uint64()
        _check(library().gg_server_submit(self.h, graph_id, kind, root, ctypes.byref(t)))
        return t.value

    def wait(self, max_results=256, timeout_ms=100):
        buf = (_QueryResult * max_results)()
        n = ctypes.c_int32()
        _check(library().gg_server_wait(self.h, buf, max_results, timeout_ms, ctypes.byref(n)))
        return [{k: getattr(buf[i], k) for k, _ in _QueryResult._fields_} for i in range(n.value)]

    def stats(self):
        st = _ServerStats()
        _check(library().gg_server_stats_get(self.h, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in _ServerStats._fields_}

    def close(self):
        if self.h:
            library().gg_server_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def pick_roots(out_degree, count, seed):
    """Seeded uniform draws of vertices with out-degree > 0 (the benchmark's
    "non-isolated" roots)."""
    rng = np.random.default_rng(seed)
    cand = np.nonzero(np.asarray(out_degree) > 0)[0]
    if len(cand) == 0:
        raise ValueError("no vertex with out-degree > 0")
    return [int(x) for x in cand[rng.integers(0, len(cand), count)]]
