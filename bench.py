#!/usr/bin/env python3
"""Benchmark of the GB300 edge-processing engine (one JSON line on stdout).

Default workload: BFS (toolkits/bfs.cpp semantics) from seeded non-isolated
roots on a directed R-MAT graph of scale 26, edge factor 16 (67,108,864
vertices, 1,073,741,824 edges, a=.57 b=.19 c=.19 d=.05), generated on the
device from a seed -- synthetic data of the benchmark's shape.  One step =
one BFS from the next root.  GTEPS = sum over process_edges calls of
active_edges (core/graph.hpp:1503-1508, identical for the reference and this
engine) / time.

  value      graph and root resident in HBM; device time of each BFS
             (CUDA events on the library's stream), results left on device
  e2e        the same roots through the C ABI with every parent array copied
             back to pinned host memory inside the timed region (wall clock):
             gg_bfs_many (each copy overlaps the next root's BFS); the
             one-gg_bfs-call-per-root figure is e2e.sync_value
  roofline   the dominant edge kernel's algorithmic bytes / its event time,
             from a second pass over the first timed roots with CUDA events
             around every process_edges call (the timed steps carry none)
  cpu_baseline  the reference's own BFS (oracle/_ref, built from the
             reference sources) on this host's cores, on the benchmark's own
             R-MAT 26 graph and roots (the reference arm's result when it ran
             on this host first, else one warm-up and three timed roots)

--impl reference runs the reference arm: the reference's own CPU BFS
(mpirun -np 1 equivalent, every host core) on the same graph and the same
roots, its edge file written by the oracle's restatement of the generator, so
that no product code is loaded; printed with impl=reference.  Workloads other
than BFS time the reference on a smaller R-MAT sample whose TEPS numerators
come from the oracle's trace.  Multi-GPU (torchrun): replicas -- each rank
runs its own BFSes on its own GPU; value = all ranks' edges / the slowest
rank's time.  --check checks the first timed run against the oracle on the
full-size graph after timing.

Other workloads (--workload): cc, pagerank, pagerank_f64, sssp, bc, bfs_grid
(GTEPS as above); bfs_batched, sssp_batched, bc_batched (queries/s of
64-root batches beside the same roots run one at a time); serve (continuous
batching over four resident graphs: capacity under a stream offered above it,
then p50/p99 latency at 50% and 90% of that capacity, each beside a plain
FIFO replay of the same arrivals; --mix adds plain vs full-batch costs per
graph and kind); build (the partitioned graph build from records in pinned
host memory under --build-budget-gb, Medges/s, beside the in-core build).
--adjacency host keeps the neighbour arrays in mapped host memory (read over
NVLink-C2C) and adds the link rate to the roofline; --bins default skips the
autotuner, which otherwise tunes each workload for its own kernels (bins, light
windows, L1 policy, pull split: config.bins).  The batched BFS keeps its
levels as level lists during the timed batches (every lane's levels stay on
the device) and extracts lane-major level arrays in the e2e batches.
"""
import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

METRIC = "GTEPS at RMAT-26 vs HBM roofline; batched BFS/SSSP queries/s, p99 vs plain"
SEED = 1
FALLBACK_HBM_GBS = 6800.0

WORKLOADS = {
    "bfs": dict(kind="rmat", scale=26, ef=16, weighted=False, symmetric=False,
                desc="BFS from seeded non-isolated roots on directed R-MAT scale 26, edge factor 16"),
    "cc": dict(kind="rmat", scale=26, ef=16, weighted=False, symmetric=True,
               desc="CC (min-label, symmetrised edges) on R-MAT scale 26, edge factor 16"),
    "pagerank": dict(kind="rmat", scale=20, ef=16, weighted=False, symmetric=False,
                     desc="PageRank 20 iterations, float ranks (d=0.85), on directed R-MAT scale 20, edge factor 16"),
    "pagerank_f64": dict(kind="rmat", scale=20, ef=16, weighted=False, symmetric=False,
                         desc="PageRank 20 iterations, double ranks as the reference, on directed R-MAT scale 20, "
                              "edge factor 16"),
    "sssp": dict(kind="rmat", scale=25, ef=16, weighted=True, symmetric=False,
                 desc="SSSP (float weights in [0,1)) from seeded roots on R-MAT scale 25, edge factor 16"),
    "bc": dict(kind="rmat", scale=25, ef=16, weighted=False, symmetric=False,
               desc="BC (double) from seeded roots on R-MAT scale 25, edge factor 16"),
    "bfs_grid": dict(kind="grid", scale=8192, ef=0, weighted=False, symmetric=False,
                     desc="BFS on the 8192 x 8192 4-neighbour grid (both directions)"),
    "bfs_batched": dict(kind="rmat", scale=24, ef=16, weighted=False, symmetric=False,
                        desc="batched BFS, 64 seeded roots per launch, on directed R-MAT scale 24, edge factor 16"),
    "serve": dict(kind="rmat", scale=26, ef=16, weighted=True, symmetric=False,
                  desc="serving: 4 resident weighted R-MAT graphs (scales 20, 22, 24, 26, edge factor 16), Poisson "
                       "arrivals at 5000 queries/s, graph drawn with p = 0.4/0.3/0.2/0.1, 75% BFS / 25% SSSP, "
                       "seeded uniform non-isolated roots"),
    "bc_batched": dict(kind="rmat", scale=24, ef=16, weighted=False, symmetric=False,
                       desc="batched BC (double), 64 seeded roots per launch, on directed R-MAT scale 24, "
                            "edge factor 16"),
    "sssp_batched": dict(kind="rmat", scale=24, ef=16, weighted=True, symmetric=False,
                         desc="batched SSSP, 64 seeded roots per launch, on R-MAT scale 24, edge factor 16, "
                              "float weights in [0,1)"),
    "build": dict(kind="rmat", scale=26, ef=16, weighted=False, symmetric=False,
                  desc="graph build (CSR + CSC) of directed R-MAT scale 26, edge factor 16, from records in pinned "
                       "host memory, partitioned under a device-memory budget"),
}
REF_APP = {"bfs": "bfs", "cc": "cc", "pagerank": "pagerank", "pagerank_f64": "pagerank", "sssp": "sssp", "bc": "bc", "bfs_grid": "bfs",
           "bfs_batched": "bfs", "sssp_batched": "sssp", "bc_batched": "bc", "serve": "bfs"}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ----------------------------------------------------------------- distributed
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as td
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, x):
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x):
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


# ----------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples (every 20 ms) of SM clock and throttle reasons."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "20",
                 "-i", str(self.device)], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        # the timed region starts only once samples are flowing
        t0 = time.time()
        while time.time() - t0 < 5.0:
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.01)

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append(dict(sm=float(parts[1]), sm_max=float(parts[2]), power=float(parts[3]),
                                 hw=parts[5], hwt=parts[6], swt=parts[7], swp=parts[8]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return None
        reasons = []
        for key, name in (("hw", "hw_slowdown"), ("hwt", "hw_thermal_slowdown"), ("swt", "sw_thermal_slowdown"),
                          ("swp", "sw_power_cap")):
            if any(r[key].lower().startswith("active") for r in rows):
                reasons.append(name)
        load = [r["sm"] for r in rows]
        return {"sm_mhz": statistics.median(load), "sm_max_mhz": max(r["sm_max"] for r in rows),
                "reasons": reasons, "samples": len(rows), "power_w_max": max(r["power"] for r in rows)}


# ----------------------------------------------------------------- helpers
def peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def committed_traffic(kernel, workload, scale):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary, if
    one was captured on this workload at this scale."""
    p = os.path.join(REPO, "profiles", "traffic.json")
    try:
        d = json.load(open(p))
        e = d[workload][kernel]
        if int(e["scale"]) != int(scale):
            return None
        return float(e["bytes_per_launch"])
    except (OSError, KeyError, ValueError, TypeError):
        return None


def algorithmic_bytes(mode, ae, V, n_frontier, workload):
    """Bytes a call must move (per counted edge: neighbour id + the value it
    gathers or scatters; per vertex: offsets, degree, state; bitmaps)."""
    per_edge = {"bfs": 8, "bfs_grid": 8, "cc": 8, "sssp": 12, "bc": 12, "pagerank": 8, "pagerank_f64": 12}[workload]
    state = {"bfs": 4, "bfs_grid": 4, "cc": 4, "sssp": 4, "bc": 8, "pagerank": 4, "pagerank_f64": 8}[workload]
    if mode == 1:   # pull: every vertex's offsets, its state write, three bitmaps
        return per_edge * ae + V * (8 + state) + 3 * (V // 8)
    return per_edge * ae + n_frontier * (8 + 4 + 4)   # push: frontier offsets, degree, queue entry


def make_graph(gg, w, device, **build):
    """build: build_budget / adjacency_host / force_partitions (gg_build_options)."""
    if w["kind"] == "rmat":
        return gg.Graph.generate(gg.RMAT, w["scale"], w["ef"], SEED, weighted=w["weighted"],
                                 symmetric=w["symmetric"], device=device, **build)
    return gg.Graph.generate(gg.GRID, w["scale"], 0, SEED, weighted=w["weighted"], symmetric=w["symmetric"],
                             device=device, **build)


def link_h2d_gbs(device, nbytes=1 << 30, reps=5):
    """Pinned host -> device copy rate (NVLink-C2C on GB300), CUDA events."""
    import torch
    src = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    dst = torch.empty(nbytes, dtype=torch.uint8, device=f"cuda:{device}")
    dst.copy_(src, non_blocking=True)
    torch.cuda.synchronize(device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        dst.copy_(src, non_blocking=True)
    e1.record()
    torch.cuda.synchronize(device)
    gbs = nbytes * reps / (e0.elapsed_time(e1) / 1000.0) / 1e9
    del src, dst
    torch.cuda.empty_cache()
    return gbs


def run_once(gg, g, workload, arg, to_host, stats_cls):
    if workload in ("bfs", "bfs_grid"):
        _, st = g.bfs(arg, to_host=to_host)
    elif workload == "cc":
        _, st = g.cc(to_host=to_host)
    elif workload == "pagerank":
        _, _, st = g.pagerank(arg, to_host=to_host, f32=True)
    elif workload == "pagerank_f64":
        _, _, st = g.pagerank(arg, to_host=to_host)
    elif workload == "sssp":
        _, st = g.sssp(arg, to_host=to_host)
    else:
        _, _, st = g.bc(arg, to_host=to_host)
    return st


def step_args(gg, g, workload, count):
    if workload in ("pagerank", "pagerank_f64"):
        return [20] * count
    if workload == "cc":
        return [None] * count
    if workload == "bfs_grid":
        return [0] * count
    return gg.pick_roots(g.out_degree(), count, seed=root_seed(workload))


# ----------------------------------------------------------------- CPU side
# Workloads whose reference run is timed on the benchmark's own graph and
# roots: the reference's BFS driver reports each run's traversed edges itself
# (teps_edges, read from its parent array), so no oracle trace is needed.
FULL_SCALE_REFERENCE = ("bfs",)


def ref_sample_scale(workload):
    """Graph the reference is timed on: the workload's own scale where the
    reference reports its TEPS numerator, else a bounded sample whose
    numerator the oracle's per-call trace gives."""
    if workload in FULL_SCALE_REFERENCE:
        return WORKLOADS[workload]["scale"]
    return {"cc": 21, "pagerank": 20, "pagerank_f64": 20, "sssp": 21, "bc": 21, "bfs_grid": 1024,
            "bfs_batched": 22, "sssp_batched": 21, "bc_batched": 21, "serve": 22}[workload]


def root_seed(workload):
    """Seed of the workload's root sequence; the GPU arm draws the same one."""
    return SEED + 1000 if workload in ("bfs", "sssp", "bc") else SEED + 2000


def scratch_dir(nbytes):
    """RAM-backed /dev/shm when it has room for the edge file, else the default temp dir."""
    try:
        st = os.statvfs("/dev/shm")
        if st.f_bavail * st.f_frsize > 2 * nbytes:
            return "/dev/shm"
    except OSError:
        pass
    return None


def cpu_reference(workload, nsteps, warmup, first_root=0):
    """Times the reference's own compute() (oracle/_ref/bin/ref_<app>, the
    reference's sources built on this host) with every host core; falls back
    to the oracle port.  The edge file and the roots come from the oracle's
    restatement of the benchmark generator and root rule, so this leg loads no
    product code.  For FULL_SCALE_REFERENCE workloads the graph is the
    benchmark's own and the roots are the GPU arm's roots first_root,
    first_root + 1, ... (warm-up roots first)."""
    from oracle import oracle
    w = WORKLOADS[workload]
    s = ref_sample_scale(workload)
    cores = os.cpu_count() or 1
    n = warmup + nsteps
    kind = oracle.RMAT if w["kind"] == "rmat" else oracle.GRID
    V = (1 << s) if kind == oracle.RMAT else s * s
    unit = 12 if w["weighted"] else 8
    nrec = oracle.record_count(kind, s, w["ef"])
    sample = (f"R-MAT scale {s}, edge factor {w['ef']}, seed {SEED}" if kind == oracle.RMAT else f"{s} x {s} grid")
    if s == w["scale"]:
        sample += " (the benchmark's graph)"
    fd, path = tempfile.mkstemp(suffix=".bin", dir=scratch_dir(nrec * unit))
    os.close(fd)
    try:
        t0 = time.perf_counter()
        V, nrec, deg = oracle.write_records_file(path, kind, s, w["ef"], SEED, weighted=w["weighted"],
                                                 threads=cores)
        gen_s = time.perf_counter() - t0
        if workload in ("bfs", "sssp", "bc", "bfs_batched", "sssp_batched", "bc_batched", "serve"):
            args = oracle.pick_roots(deg, first_root + n, seed=root_seed(workload))[first_root:]
            if s == w["scale"]:
                sample += f"; roots {first_root}..{first_root + n - 1} of the benchmark's root sequence"
        elif workload == "bfs_grid":
            args = [0] * n
        elif workload in ("pagerank", "pagerank_f64"):
            args = [20] * n
        else:
            args = [0] * n
        numer = None
        if workload not in FULL_SCALE_REFERENCE:
            # TEPS numerators from the oracle's trace (the quantity the reference counts)
            rec = np.fromfile(path, dtype=np.uint32).reshape(-1, unit // 4)
            og = oracle.OracleGraph(V, rec[:, 0].copy(), rec[:, 1].copy(),
                                    rec[:, 2].copy().view(np.float32) if w["weighted"] else None,
                                    symmetric=w["symmetric"])
            del rec
            numer = [sum(r[1] for r in oracle_trace(og, workload, a)) for a in args]
        exe = os.path.join(REPO, "oracle", "_ref", "bin", "ref_" + REF_APP[workload])
        if os.path.exists(exe):
            env = dict(os.environ, OMP_NUM_THREADS=str(cores), GG_REF_THREADS=str(cores))
            p = subprocess.run([exe, path, str(V)] + [str(a) for a in args], capture_output=True, text=True,
                               env=env, timeout=1500)
            times = [float(x) for x in re.findall(r"exec_time=([0-9.]+)", p.stdout)]
            counted = [int(x) for x in re.findall(r"teps_edges=([0-9]+)", p.stdout)]
            load = re.findall(r"load_time=([0-9.]+)", p.stdout)
            if numer is None and len(counted) == n:
                numer = counted
            if p.returncode == 0 and len(times) == n and numer is not None:
                t = times[warmup:]
                e = numer[warmup:]
                return dict(value=sum(e) / sum(t) / 1e9, unit="GTEPS", cores=cores, kind="reference",
                            sample=f"{sample}; {nsteps} timed runs after {warmup} warm-up; reference compute() "
                                   f"exec_time, {cores} OpenMP threads", times=t, edges=e,
                            load_s=float(load[0]) if load else None, generate_s=round(gen_s, 1))
            log("reference driver failed:", p.returncode, p.stderr[-500:])
        if numer is None:
            raise RuntimeError("the reference driver did not run and the oracle port has no numerators")
        # oracle port: serial C restatement
        rec = np.fromfile(path, dtype=np.uint32).reshape(-1, unit // 4)
        og = oracle.OracleGraph(V, rec[:, 0].copy(), rec[:, 1].copy(),
                                rec[:, 2].copy().view(np.float32) if w["weighted"] else None,
                                symmetric=w["symmetric"])
        del rec
    finally:
        os.unlink(path)
    t, e = [], []
    for i, a in enumerate(args):
        t0 = time.perf_counter()
        oracle_trace(og, workload, a)
        if i >= warmup:
            t.append(time.perf_counter() - t0)
            e.append(numer[i])
    return dict(value=sum(e) / sum(t) / 1e9, unit="GTEPS", cores=1, kind="port",
                sample=f"{sample}; {nsteps} timed runs after {warmup} warm-up; oracle port, 1 thread",
                times=t, edges=e)


def check_against_oracle(g, workload, arg):
    """Checks one run of the timed workload, on its full-size graph, against
    the oracle (bench.py --check; outside every timed region): BFS levels and
    tree edges, CC labels and SSSP distances bit-exact, float PageRank within
    1e-5 relative L1 of the oracle's double ranks, BC within 1e-10."""
    from oracle import oracle
    w = WORKLOADS[workload]
    t0 = time.perf_counter()
    kind = oracle.RMAT if w["kind"] == "rmat" else oracle.GRID
    V = (1 << w["scale"]) if kind == oracle.RMAT else w["scale"] * w["scale"]
    rec = oracle.records(kind, w["scale"], w["ef"], SEED, w["weighted"], threads=os.cpu_count() or 1)
    rec = rec.reshape(-1, 3 if w["weighted"] else 2)
    og = oracle.OracleGraph(V, rec[:, 0].copy(), rec[:, 1].copy(),
                            rec[:, 2].copy().view(np.float32) if w["weighted"] else None, symmetric=w["symmetric"])
    del rec

    def rel(a, b):
        return float(np.abs(a - b).sum() / max(np.abs(b).sum(), 1e-300))

    out = {"workload": workload, "arg": arg}
    if workload in ("bfs", "bfs_grid"):
        parent, _ = g.bfs(arg)
        oparent, otrace = og.bfs(arg)
        out["levels_equal"] = bool(np.array_equal(oracle.tree_levels(parent, arg), oracle.tree_levels(oparent, arg)))
        out["bad_tree_edges"] = og.tree_bad_edges(parent, arg)
        out["passed"] = out["levels_equal"] and out["bad_tree_edges"] == 0
    elif workload in ("pagerank", "pagerank_f64"):
        ranks, _, _ = g.pagerank(arg, f32=workload == "pagerank")
        oranks = og.pagerank(arg)[0]
        out["rel_l1_vs_fp64"] = rel(ranks.astype(np.float64), oranks)
        out["passed"] = out["rel_l1_vs_fp64"] < (1e-5 if workload == "pagerank" else 1e-10)
    elif workload == "sssp":
        dist, _ = g.sssp(arg)
        out["passed"] = bool(np.array_equal(dist.view(np.uint32), og.sssp(arg)[0].view(np.uint32)))
    elif workload == "cc":
        label, _ = g.cc()
        out["passed"] = bool(np.array_equal(label, og.cc()[0]))
    else:
        dep, _, _ = g.bc(arg)
        odep = og.bc(arg)[0]
        ok = ~np.isnan(odep)
        out["rel_l1"] = rel(dep[ok], odep[ok])
        out["passed"] = bool(np.array_equal(np.isnan(dep), np.isnan(odep))) and out["rel_l1"] < 1e-10
    out["seconds"] = round(time.perf_counter() - t0, 1)
    return out


def _boot_id():
    try:
        return open("/proc/sys/kernel/random/boot_id").read().strip()
    except OSError:
        return None


def _reference_cache_path(workload):
    return os.path.join(tempfile.gettempdir(), f"gg_reference_{workload}_s{ref_sample_scale(workload)}.json")


def save_reference_result(workload, r):
    """Keeps the reference arm's result for this host's later GPU run (the
    reference's own load of an R-MAT 26 file takes minutes)."""
    try:
        with open(_reference_cache_path(workload), "w") as f:
            json.dump(dict(r, boot_id=_boot_id(), when=time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime())), f)
    except OSError:
        pass


def cached_reference_result(workload):
    """The reference arm's result from this boot of this host, if any."""
    try:
        r = json.load(open(_reference_cache_path(workload)))
    except (OSError, ValueError):
        return None
    if r.get("boot_id") != _boot_id() or r.get("boot_id") is None or r.get("kind") != "reference":
        return None
    return r


def oracle_trace(og, workload, a):
    if workload in ("bfs", "bfs_grid", "bfs_batched", "serve"):
        return og.bfs(a)[1]
    if workload in ("sssp", "sssp_batched"):
        return og.sssp(a)[1]
    if workload in ("bc", "bc_batched"):
        return og.bc(a)[2]
    if workload in ("pagerank", "pagerank_f64"):
        return og.pagerank(a)[2]
    return og.cc()[1]


# ----------------------------------------------------------------- arms
def reference_arm(args, dist):
    if dist.rank != 0:
        return 0
    if args.workload == "build":
        print(json.dumps({"impl": "reference", "unavailable": "the reference's loader reports no load time of its "
                          "own (its toolkits time compute() only)"}), flush=True)
        return 0
    w = WORKLOADS[args.workload]
    r = cpu_reference(args.workload, args.steps, args.warmup)
    save_reference_result(args.workload, r)
    if args.workload.endswith("_batched") or args.workload == "serve":
        # the reference has no batching: its queries/s is one root at a time
        r["value"], r["unit"] = len(r["times"]) / sum(r["times"]), "queries/s"
    line = {
        "impl": "reference", "metric": METRIC, "value": round(r["value"], 4), "unit": r["unit"],
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000 * sum(r["times"]) / len(r["times"]), 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": {"sssp": "f32", "bc": "f64", "pagerank": "f32", "pagerank_f64": "f64", "sssp_batched": "f32",
                                                     "bc_batched": "f64"}.get(args.workload, "u32"),
        "data": "synthetic", "config": {"workload": w["desc"], "sample": r["sample"]},
        "cpu_baseline": {k: r[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": round(r["value"], 4), "unit": r["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def tune_bins(g, args):
    """Degree bins for this graph: the library defaults, or the autotuner's
    pick for the workload's kernels (timed on the graph, cached on disk)."""
    if args.bins == "default":
        return {"source": "default", "light_deg": 32, "pull_chunk": 256, "pull_vector": 1, "l1_hot_bytes": None,
                "pull_split": 0, "bfs_pull": 20}
    objective = ("pagerank_f64",) if args.workload == "pagerank_f64" else \
        ("pagerank",) if args.workload.startswith("pagerank") else \
        ("bc",) if args.workload == "bc" else \
        ("batched",) if args.workload in ("bfs_batched", "sssp_batched", "bc_batched", "serve") else \
        ("bfs",) if args.workload.startswith("bfs") else ("sssp",) if args.workload == "sssp" else \
        ("cc",) if args.workload == "cc" else ("pagerank", "bfs")
    t0 = time.perf_counter()
    r = g.autotune(objective=objective)
    return {"source": "autotune(%s)" % "+".join(objective), "light_deg": r["light_deg"],
            "pull_chunk": r["pull_chunk"], "pull_vector": r["pull_vector"],
            "l1_hot_bytes": None if r["l1_hot_bytes"] == 0xffffffff else r["l1_hot_bytes"],
            "pull_split": r["pull_split"], "bfs_pull": r["bfs_pull"], "from_cache": bool(r["from_cache"]),
            "tune_s": round(time.perf_counter() - t0, 2),
            "objective_ms_default": round(r["default_ms"], 3), "objective_ms_chosen": round(r["best_ms"], 3)}


def gpu_arm(args, dist):
    import geminigraph_gb300 as gg
    w = WORKLOADS[args.workload]
    device = dist.local_rank
    t0 = time.perf_counter()
    g = make_graph(gg, w, device, build_budget=int(args.build_budget_gb * 1e9),
                   adjacency_host=args.adjacency == "host")
    build_s = time.perf_counter() - t0
    bins = tune_bins(g, args)
    info = g.info()
    V = info["vertices"]
    n = args.warmup + args.steps
    step_in = step_args(gg, g, args.workload, n + args.steps)
    for a in step_in[:args.warmup]:
        run_once(gg, g, args.workload, a, False, None)
    # ---- value: resident inputs, results on device, device time per step
    clocks = ClockSampler(device)
    clocks.start()
    dist.barrier()
    stats = []
    wall0 = time.perf_counter()
    for a in step_in[args.warmup:n]:
        st = gg.RunStats()
        stats.append(run_once_stats(gg, g, args.workload, a, st))
    wall = time.perf_counter() - wall0
    dist.barrier()
    clk = clocks.stop()
    dev_ms = sum(s.device_ms for s in stats)
    edges = sum(s.active_edges_total for s in stats)
    launches = sum(s.kernel_launches for s in stats)
    t_max = dist.max(dev_ms / 1000.0)
    edges_all = dist.sum(edges)
    value = edges_all / t_max / 1e9
    # ---- dominant kernel roofline: the first timed steps again, with CUDA
    # events around every process_edges call (events between the kernels
    # would slow the timed steps above, and break up PageRank's captured graph)
    tstats = []
    for a in step_in[args.warmup:n][:5]:
        st = gg.RunStats()
        st.enable_call_timing()
        tstats.append(run_once_stats(gg, g, args.workload, a, st))
    per_mode = {0: [0.0, 0.0, 0, 0], 1: [0.0, 0.0, 0, 0]}   # ms, bytes, launches, adjacency bytes
    adj_per_edge = 8 if w["weighted"] else 4
    for s in tstats:
        prev_act = 1
        for i, (mode, ae, act) in enumerate(s.rows()):
            ms = float(s.call_ms[i])
            frontier = prev_act if i else 1
            per_mode[mode][0] += ms
            per_mode[mode][1] += algorithmic_bytes(mode, ae, V, frontier, args.workload)
            per_mode[mode][2] += 1
            per_mode[mode][3] += adj_per_edge * ae
            prev_act = act
    dom = 1 if per_mode[1][0] >= per_mode[0][0] else 0
    kname = {0: "push_lb", 1: "bfs_pull" if args.workload.startswith("bfs") else "pull_reduce"}[dom]
    timed_in = ("per-call CUDA events on the library's stream, a second pass over the first "
                f"{len(tstats)} timed roots")
    if per_mode[0][0] + per_mode[1][0] < 0.5 * sum(s.device_ms for s in tstats):
        # most calls ran inside cooperative small-run launches, which have no
        # per-call events: the whole runs' bytes over their device time
        dom = 0 if per_mode[0][1] >= per_mode[1][1] else 1
        kname = "push_small_coop + push_lb" if dom == 0 else kname
        for m in (0, 1):
            per_mode[m][0] = sum(s.device_ms for s in tstats) * (per_mode[m][1] / max(per_mode[0][1] + per_mode[1][1], 1))
        timed_in = ("whole runs (CUDA events around each run; the calls inside cooperative launches have no "
                    f"events of their own), a second pass over the first {len(tstats)} timed roots")
    peak, peak_kind = peaks()
    ach = per_mode[dom][1] / (per_mode[dom][0] / 1000.0) / 1e9 if per_mode[dom][0] > 0 else 0.0
    traffic = committed_traffic(kname, args.workload, w["scale"])
    total_kernel_ms = per_mode[0][0] + per_mode[1][0]
    avg_ms = per_mode[dom][0] / max(per_mode[dom][2], 1)
    roofline = {"bound": "hbm", "kernel": kname, "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
                "frac": round(ach / peak, 4), "peak_source": f"{peak_kind} hbm_gbs",
                "traffic": traffic,
                # DRAM bytes the kernel class really moves (committed ncu capture) over its time:
                # below frac where pull-mode BFS skips counted edges
                "dram_frac": round(traffic / (avg_ms / 1000.0) / 1e9 / peak, 4) if traffic and avg_ms > 0 else None,
                "launches": per_mode[dom][2],
                "timed_in": timed_in,
                "avg_launch_ms": round(per_mode[dom][0] / max(per_mode[dom][2], 1), 4),
                "share_of_edge_kernel_time": round(per_mode[dom][0] / total_kernel_ms, 4) if total_kernel_ms else None}
    # ---- e2e through the C ABI with host buffers
    host_out = gg.PinnedArray(V, np.uint32 if args.workload in ("bfs", "bfs_grid", "cc") else
                              (np.float32 if args.workload in ("sssp", "pagerank") else np.float64))
    dist.barrier()
    e_edges, e_wall = 0, 0.0
    for a in step_in[n:n + args.steps]:
        t1 = time.perf_counter()
        st = run_e2e(gg, g, args.workload, a, host_out)
        e_wall += time.perf_counter() - t1
        e_edges += st.active_edges_total
    e_max = dist.max(e_wall)
    e_value = dist.sum(e_edges) / e_max / 1e9
    e2e_extra = {}
    if args.workload in ("bfs", "bfs_grid"):
        # the same roots through gg_bfs_many: each parent tree still lands in
        # pinned host memory, copied while the next root's BFS computes
        outs = gg.PinnedArray(V, np.uint32)
        bufs = [outs.array(0), outs.array(1)]
        roots = list(step_in[n:n + args.steps])
        warm = list(step_in[:max(args.warmup, 2)])
        g.bfs_many(warm, [bufs[i % 2] for i in range(len(warm))])   # allocates the second result buffer
        dist.barrier()
        t1 = time.perf_counter()
        st = g.bfs_many(roots, [bufs[i % 2] for i in range(len(roots))])
        p_wall = time.perf_counter() - t1
        p_max = dist.max(p_wall)
        e2e_extra = {"sync_value": round(e_value, 3), "sync_ms_per_step": round(e_max * 1000 / args.steps, 3),
                     "mode": "gg_bfs_many: result i copied to pinned host memory while root i+1 computes "
                             "(sync_value: one gg_bfs call per root)"}
        e_value = dist.sum(st.active_edges_total) / p_max / 1e9
        e_max = p_max
    d2h = V * host_out.itemsize * (2 if args.workload == "bc" else 1)
    h2d = 4 if args.workload in ("bfs", "bfs_grid", "sssp", "bc") else 0
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "GTEPS", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(t_max * 1000 / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": {"sssp": "f32", "bc": "f64", "pagerank": "f32", "pagerank_f64": "f64"}.get(args.workload, "u32"),
        "data": "synthetic (seeded R-MAT / grid generated on the device)",
        "config": {"workload": w["desc"], "vertices": V, "edges": info["edges"],
                   "l2": "inputs larger than L2 (graph %.1f GB)" % (info["device_bytes"] / 1e9),
                   "parallelism": f"replicas x{args.gpus}", "graph_build_s": round(build_s, 2),
                   "adjacency": args.adjacency, "build_partitions": g.build["partitions"],
                   "host_adjacency_gb": round(info["host_bytes"] / 1e9, 2),
                   "active_edges_per_step": edges // max(len(stats), 1), "bins": bins},
        "e2e": dict({"value": round(e_value, 3), "unit": "GTEPS", "h2d_bytes_per_step": h2d,
                     "d2h_bytes_per_step": d2h, "ms_per_step": round(e_max * 1000 / args.steps, 3)}, **e2e_extra),
        "roofline": roofline,
        "gpu_launches": launches,
        "trace_first_step": [[m, ae, act, round(float(tstats[0].call_ms[i]), 4)]
                             for i, (m, ae, act) in enumerate(tstats[0].rows()[:40])] if tstats else [],
        "wall_s": round(wall, 3),
        "clocks": clk,
    }
    if args.adjacency == "host":
        # the adjacency reads cross NVLink-C2C: the same achieved rate against the link
        # only the neighbour (and weight) arrays cross the link
        link = link_h2d_gbs(device)
        adj_rate = per_mode[dom][3] / (per_mode[dom][0] / 1000.0) / 1e9 if per_mode[dom][0] > 0 else 0.0
        line["roofline"]["link"] = {"achieved": round(adj_rate, 1), "peak": round(link, 1), "unit": "GB/s",
                                    "frac": round(adj_rate / link, 4),
                                    "bytes": "adjacency bytes of the counted edges (pull-mode BFS reads fewer)",
                                    "peak_source": "measured pinned host->device copy (torch, CUDA events)"}
    if args.check and dist.rank == 0:
        line["check"] = check_against_oracle(g, args.workload, step_in[args.warmup])
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        try:
            r = cached_reference_result(args.workload)
            if r is not None:
                r["sample"] += f"; measured by this host's reference arm (bench.py --impl reference) at {r['when']}"
            else:
                # bounded: one warm-up and three timed roots, the first of the sequence timed above
                r = cpu_reference(args.workload, 3, 1, first_root=max(args.warmup - 1, 0))
            line["cpu_baseline"] = {k: (round(r[k], 4) if k == "value" else r[k])
                                    for k in ("value", "unit", "cores", "kind", "sample")}
            line["cpu_baseline"]["reference_load_s"] = r.get("load_s")
        except Exception as e:  # the baseline is reported, never required
            line["cpu_baseline"] = {"value": None, "error": str(e)[:200]}
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    g.close()
    return 0


def gpu_arm_batched(args, dist):
    """One step = one batch of 64 roots.  value = queries/s of the batched
    kernel; plain = the same roots one at a time through gg_bfs / gg_sssp."""
    import geminigraph_gb300 as gg
    w = WORKLOADS[args.workload]
    device = dist.local_rank
    t0 = time.perf_counter()
    g = make_graph(gg, w, device, build_budget=int(args.build_budget_gb * 1e9),
                   adjacency_host=args.adjacency == "host")
    build_s = time.perf_counter() - t0
    bins = tune_bins(g, args)
    info = g.info()
    V = info["vertices"]
    bfs = args.workload == "bfs_batched"
    lanes = 64
    roots = gg.pick_roots(g.out_degree(), lanes * (args.warmup + 2 * args.steps), seed=SEED + 3000)
    batches = [roots[i * lanes:(i + 1) * lanes] for i in range(args.warmup + 2 * args.steps)]

    bc = args.workload == "bc_batched"

    def run_batch(rs, host, timing=False):
        if bfs:
            _, _, _, edges, st = gg.bfs_batched(g, rs, levels=host, parents=False, timing=timing)
            return st, int(edges.sum())
        if bc:
            _, _, _, st = gg.bc_batched(g, rs, outputs=host, timing=timing)
            return st, 0
        _, _, st = gg.sssp_batched(g, rs, distances=host, timing=timing)
        return st, 0

    for b in batches[:args.warmup]:
        run_batch(b, False)
    clocks = ClockSampler(device)
    clocks.start()
    dist.barrier()
    dev_ms, edges, launches = 0.0, 0, 0
    first = None
    for b in batches[args.warmup:args.warmup + args.steps]:
        st, e = run_batch(b, False)
        dev_ms += st.device_ms
        edges += e
        launches += st.kernel_launches
    dist.barrier()
    clk = clocks.stop()
    # per-step kernel times of the first batch, in a pass of its own
    first = run_batch(batches[args.warmup], False, timing=True)[0]
    t_max = dist.max(dev_ms / 1000.0)
    q_all = dist.sum(lanes * args.steps)
    value = q_all / t_max
    # plain: the same number of roots one at a time (device time)
    plain_ms = 0.0
    plain_roots = [r for b in batches[args.warmup:args.warmup + args.steps] for r in b][:lanes]
    for r in plain_roots:
        if bfs:
            _, st = g.bfs(r, to_host=False)
        elif bc:
            _, _, st = g.bc(r, to_host=False)
        else:
            _, st = g.sssp(r, to_host=False)
        plain_ms += st.device_ms
    plain_qps = len(plain_roots) / (plain_ms / 1000.0)
    # e2e: per-lane results copied to host memory
    dist.barrier()
    e_wall = 0.0
    for b in batches[args.warmup + args.steps:]:
        t1 = time.perf_counter()
        run_batch(b, True)
        e_wall += time.perf_counter() - t1
    e_max = dist.max(e_wall)
    line = {
        "metric": METRIC, "value": round(value, 1), "unit": "queries/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(t_max * 1000 / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64 lane masks" if bfs else ("f64" if bc else "f32"),
        "data": "synthetic (seeded R-MAT generated on the device)",
        "config": {"workload": w["desc"], "vertices": V, "edges": info["edges"], "lanes": lanes,
                   "parallelism": f"replicas x{args.gpus}", "graph_build_s": round(build_s, 2),
                   "adjacency": args.adjacency, "build_partitions": g.build["partitions"],
                   "host_adjacency_gb": round(info["host_bytes"] / 1e9, 2),
                   "l2": "inputs larger than L2", "bins": bins},
        "plain": {"value": round(plain_qps, 1), "unit": "queries/s",
                  "what": f"{len(plain_roots)} roots one at a time through the single-root kernels (device time)"},
        "speedup_vs_plain": round(value / plain_qps, 2),
        "e2e": {"value": round(dist.sum(lanes * args.steps) / e_max, 1), "unit": "queries/s",
                "h2d_bytes_per_step": 4 * lanes, "d2h_bytes_per_step": (16 if bc else 4) * lanes * V,
                "ms_per_step": round(e_max * 1000 / args.steps, 3)},
        "gpu_launches": launches, "clocks": clk,
        "trace_first_step": [list(r) for r in first.rows(with_ms=True)[:60]] if first else [],
    }
    if bfs:
        line["lane_gteps"] = round(dist.sum(edges) / t_max / 1e9, 2)
    if bc and first is not None:
        # level storage of the first batch: a 12-byte list entry per (vertex,
        # level) pair occurring in some lane plus two dense u64 mask arrays,
        # against one u64 mask per vertex per level
        rows = first.rows()
        fwd = rows[:len(rows) // 2]
        pairs = len(set(batches[args.warmup])) + sum(r[2] for r in fwd)
        line["level_storage"] = {"levels": len(fwd), "pairs": pairs,
                                 "bytes_per_vertex": round((12 * pairs + 16 * V) / V, 2),
                                 "per_level_masks_bytes_per_vertex": 8 * len(fwd)}
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    g.close()
    return 0


def gpu_arm_build(args, dist):
    """Partitioned build from host records (the out-of-core load) against the
    in-core build of the same records.  A step is one whole build."""
    import ctypes
    import geminigraph_gb300 as gg
    w = WORKLOADS["build"]
    device = dist.local_rank
    L = gg.library()
    rec_host = gg.generate_records(gg.RMAT, w["scale"], w["ef"], SEED + dist.rank, weighted=w["weighted"])
    ptr = ctypes.c_void_p()
    gg._check(L.gg_host_alloc(rec_host.nbytes, ctypes.byref(ptr)))
    rec = np.ctypeslib.as_array((ctypes.c_uint8 * rec_host.nbytes).from_address(ptr.value))
    rec[:] = rec_host
    del rec_host
    V = 1 << w["scale"]
    E = rec.nbytes // (12 if w["weighted"] else 8)
    budget = int((args.build_budget_gb or 4.0) * 1e9)

    def build(**kw):
        t0 = time.perf_counter()
        g = gg.Graph.from_records(rec, V, weighted=w["weighted"], symmetric=w["symmetric"], device=device, **kw)
        dt = time.perf_counter() - t0
        b = dict(g.build)
        info = g.info()
        g.close()
        return dt, b, info

    for _ in range(args.warmup):
        build(build_budget=budget)
    dist.barrier()
    times, parts, info = [], 0, None
    for _ in range(args.steps):
        dt, b, info = build(build_budget=budget)
        times.append(dt)
        parts = b["partitions"]
    t_max = dist.max(sum(times))
    value = dist.sum(E * len(times)) / t_max / 1e6
    ic = [build()[0] for _ in range(2)]
    in_core = E / min(ic) / 1e6
    # the partitioned build reads the records over the link: degrees, range
    # counts, and one compaction pass per group of ranges, for each direction
    passes = b["record_passes"]
    read_gbs = passes * rec.nbytes / (sum(times) / len(times)) / 1e9
    link = link_h2d_gbs(device)
    line = {
        "metric": "graph build rate", "value": round(value, 1), "unit": "Medges/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t_max * 1000 / args.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic (seeded R-MAT records generated on the host)",
        "config": {"workload": w["desc"], "vertices": V, "edges": E, "records_gb": round(rec.nbytes / 1e9, 2),
                   "build_budget_gb": round(budget / 1e9, 2), "partitions_per_direction": parts,
                   "record_passes": passes,
                   "graph_device_gb": round(info["device_bytes"] / 1e9, 2),
                   "in_core_rate_medges_s": round(in_core, 1), "in_core_s": round(min(ic), 3),
                   "l2": "records and graph larger than L2", "parallelism": f"replicas x{args.gpus}"},
        "e2e": {"value": round(value, 1), "unit": "Medges/s", "h2d_bytes_per_step": passes * rec.nbytes,
                "d2h_bytes_per_step": 0},
        "roofline": {"bound": "link", "kernel": "oc_scatter / oc_count / oc_degree (records read in place)",
                     "achieved": round(read_gbs, 1), "peak": round(link, 1), "unit": "GB/s",
                     "frac": round(read_gbs / link, 4),
                     "peak_source": "measured pinned host->device copy (torch, CUDA events)", "traffic": None},
        "gpu_launches": None,
        "cpu_baseline": {"value": None, "note": "the reference's loader reports no load time of its own"},
    }
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    L.gg_host_free(ptr)
    return 0


def pct(xs, q):
    xs = sorted(xs)
    return xs[min(len(xs) - 1, int(round(q / 100.0 * (len(xs) - 1))))] if xs else None


def fifo_replay(arrivals, service):
    """One-at-a-time FIFO service of queries arriving at `arrivals` (s) with
    service times `service` (s): (latencies in ms, served queries/s)."""
    done, lat = 0.0, []
    for a, sv in zip(arrivals, service):
        done = max(a, done) + sv
        lat.append((done - a) * 1000.0)
    return lat, len(lat) / (done - arrivals[0]) if len(lat) else None


def serve_stream(gg, server, ids, queries, arrivals):
    """Submits queries[i] at arrivals[i] (s after the start) from a client
    thread and collects the results: (results by query index, span in s)."""
    import threading
    results, tickets = {}, {}

    def client():
        start = time.perf_counter()
        for i, (j, k, r) in enumerate(queries):
            due = start + arrivals[i]
            while True:
                now = time.perf_counter()
                if now >= due:
                    break
                time.sleep(min(due - now, 0.0005))
            tickets[server.submit(ids[j], k, r)] = i

    wall0 = time.perf_counter()
    th = threading.Thread(target=client)
    th.start()
    while len(results) < len(queries):
        for r in server.wait(max_results=1024, timeout_ms=50):
            results[r["ticket"]] = r
    th.join()
    span = time.perf_counter() - wall0
    return {tickets[t]: r for t, r in results.items()}, span


def gpu_arm_serve(args, dist):
    """One step = one query of the stream.  value = completed queries / the
    span from the first arrival to the last completion of a stream offered at
    args.rate (the server's capacity when that rate is above it).  The same
    query mix is then offered at 50% and 90% of that capacity, with and
    without a batch window on the SSSP pools, for p50/p99 service latency.
    plain = the first args.plain queries run one at a time through gg_bfs /
    gg_sssp (device time as service time), replayed FIFO on each stream's
    arrival times."""
    import geminigraph_gb300 as gg
    device = dist.local_rank
    rng = np.random.default_rng(SEED + 77)
    scales, probs = (20, 22, 24, 26), (0.4, 0.3, 0.2, 0.1)
    t0 = time.perf_counter()
    graphs = [gg.Graph.generate(gg.RMAT, sc, 16, SEED + i, weighted=True, device=device) for i, sc in enumerate(scales)]
    build_s = time.perf_counter() - t0
    bins = [tune_bins(g, args) for g in graphs]
    degs = [g.out_degree() for g in graphs]
    n = args.queries
    unit = rng.exponential(1.0, n)          # arrival gaps at rate 1, scaled per stream
    gsel = rng.choice(len(scales), size=n, p=probs)
    kinds = (rng.random(n) < 0.25).astype(int)
    roots = [gg.pick_roots(degs[j], 1, int(rng.integers(1 << 30)))[0] for j in gsel]
    queries = list(zip(gsel.tolist(), kinds.tolist(), roots))
    # plain service times and checksums of the first queries, one at a time
    m = min(args.plain, n)
    plain_svc, plain_chk = [], []
    for i in range(m):
        j, k, r = queries[i]
        g = graphs[j]
        if k == 0:
            parent, s1 = g.bfs(r)
            chk = gg.result_checksum(gg.levels_from_parents(parent, r), 0)
        else:
            d1, s1 = g.sssp(r)
            chk = gg.result_checksum(d1, 1)
        plain_svc.append(s1.device_ms / 1000.0)
        plain_chk.append(chk)

    def new_server(window_ms=0.0):
        server = gg.Server(device=device)
        server.set_solo(args.solo)
        ids = [server.add_graph(g) for g in graphs]
        if window_ms:
            server.set_window(gg.Server.SSSP, window_ms)
        # warm-up: one query per (graph, kind) opens the pools' code paths
        for j in range(len(graphs)):
            for k in (0, 1):
                server.submit(ids[j], k, gg.pick_roots(degs[j], 1, 5)[0])
        got = 0
        while got < 2 * len(graphs):
            got += len(server.wait(timeout_ms=1000))
        return server, ids

    def run(rate, count, window_ms=0.0):
        server, ids = new_server(window_ms)
        arr = np.cumsum(unit[:count]) / rate
        served, span = serve_stream(gg, server, ids, queries[:count], arr)
        st = server.stats()
        server.close()
        lat = [served[i]["latency_ms"] for i in range(count)]
        mism = sum(int(plain_chk[i] != served[i]["checksum"]) for i in range(min(m, count)))
        plat, pqps = fifo_replay(arr[:m], plain_svc[:count])
        return {"offered_qps": round(rate, 1), "queries": count, "served_qps": round(count / span, 1),
                "p50_ms": round(pct(lat, 50), 3), "p99_ms": round(pct(lat, 99), 3),
                "window_ms": window_ms, "checksum_mismatches": mism,
                "plain": {"served_qps": round(pqps, 1) if pqps else None, "p50_ms": round(pct(plat, 50), 3),
                          "p99_ms": round(pct(plat, 99), 3), "queries": min(m, count)},
                "server": {k: st[k] for k in ("pools_opened", "pools_closed", "admission_waits", "max_busy_pools",
                                              "max_lanes_in_use", "solo_runs")}}

    clocks = ClockSampler(device)
    clocks.start()
    over = run(args.rate, n)
    capacity = over["served_qps"]
    loads = [run(f * capacity, min(n, args.load_queries), w) for f in (0.5, 0.9) for w in (0.0, args.window)]
    clk = clocks.stop()
    value = capacity
    line = {
        "metric": METRIC, "value": round(value, 1), "unit": "queries/s", "n_gpus": args.gpus, "steps": n,
        "warmup": 2 * len(graphs), "ms_per_step": round(1000.0 / value, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64 lane masks / f32",
        "data": "synthetic (seeded R-MAT generated on the device; Poisson query stream)",
        "config": {"workload": WORKLOADS["serve"]["desc"], "queries": n, "rate_qps": args.rate,
                   "sssp_solo_below": args.solo,
                   "graph_build_s": round(build_s, 2), "parallelism": f"replicas x{args.gpus}",
                   "bins": [{k: b[k] for k in ("source", "light_deg", "pull_chunk", "pull_vector", "l1_hot_bytes")}
                            for b in bins]},
        "latency_ms": {"p50": over["p50_ms"], "p99": over["p99_ms"],
                       "note": "offered above capacity: queueing time"},
        "plain": dict(over["plain"], what=f"first {m} queries one at a time through gg_bfs / gg_sssp (device "
                                          "time), FIFO on the same arrivals"),
        "speedup_vs_plain": round(value / over["plain"]["served_qps"], 2) if over["plain"]["served_qps"] else None,
        "checksum_mismatches": over["checksum_mismatches"], "checked": min(m, n),
        "server": over["server"],
        "loads": loads,
        "e2e": {"value": round(value, 1), "unit": "queries/s", "h2d_bytes_per_step": 4,
                "d2h_bytes_per_step": 16, "note": "per query the root in and reached count + checksum out"},
        "clocks": clk,
    }
    if args.mix:
        line["mix_ceiling"] = serve_mix_ceiling(gg, graphs, degs, scales, probs)
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    for g in graphs:
        g.close()
    return 0


def serve_mix_ceiling(gg, graphs, degs, scales, probs):
    """Per graph and kind: plain per-query wall time (one gg_bfs / gg_sssp per
    root) against full 64-root batches, and the serving mix's speed-up if
    every batch were full (75% BFS / 25% SSSP, the stream's graph weights)."""
    rows, pl, ba = [], 0.0, 0.0
    for g, deg, sc, p in zip(graphs, degs, scales, probs):
        roots = gg.pick_roots(deg, 3 * 64, seed=SEED + 9000 + sc)
        cost = {}
        for kind in ("bfs", "sssp"):
            one = g.bfs if kind == "bfs" else g.sssp
            for r in roots[:2]:
                one(int(r), to_host=False)
            k = 16 if kind == "bfs" or sc < 26 else 6
            t0 = time.perf_counter()
            for r in roots[:k]:
                one(int(r), to_host=False)
            plain = (time.perf_counter() - t0) / k * 1000
            batch = (lambda rs: gg.bfs_batched(g, rs, levels=False, parents=False)) if kind == "bfs" else \
                (lambda rs: gg.sssp_batched(g, rs, distances=False))
            batch(roots[:64])
            t0 = time.perf_counter()
            batch(roots[64:128])
            batch(roots[128:192])
            batched = (time.perf_counter() - t0) / 128 * 1000
            cost[kind] = (plain, batched)
            rows.append({"scale": sc, "kind": kind, "plain_ms_per_query": round(plain, 3),
                         "batched_ms_per_query": round(batched, 3), "x": round(plain / batched, 2)})
        pl += p * (0.75 * cost["bfs"][0] + 0.25 * cost["sssp"][0])
        ba += p * (0.75 * cost["bfs"][1] + 0.25 * cost["sssp"][1])
    return {"rows": rows, "plain_ms_per_query": round(pl, 3), "full_batch_ms_per_query": round(ba, 3),
            "speedup_if_full": round(pl / ba, 2)}


def run_once_stats(gg, g, workload, a, st):
    L = gg.library()
    import ctypes
    if workload in ("bfs", "bfs_grid"):
        gg._check(L.gg_bfs(g.h, a, None, ctypes.byref(st.s)))
    elif workload == "cc":
        gg._check(L.gg_cc(g.h, None, ctypes.byref(st.s)))
    elif workload == "pagerank":
        gg._check(L.gg_pagerank_f32(g.h, a, None, None, ctypes.byref(st.s)))
    elif workload == "pagerank_f64":
        gg._check(L.gg_pagerank(g.h, a, None, None, ctypes.byref(st.s)))
    elif workload == "sssp":
        gg._check(L.gg_sssp(g.h, a, None, ctypes.byref(st.s)))
    else:
        gg._check(L.gg_bc(g.h, a, None, None, ctypes.byref(st.s)))
    return st


def run_e2e(gg, g, workload, a, out):
    L = gg.library()
    import ctypes
    st = gg.RunStats()
    p = out.ptr
    if workload in ("bfs", "bfs_grid"):
        gg._check(L.gg_bfs(g.h, a, p, ctypes.byref(st.s)))
    elif workload == "cc":
        gg._check(L.gg_cc(g.h, p, ctypes.byref(st.s)))
    elif workload == "pagerank":
        gg._check(L.gg_pagerank_f32(g.h, a, p, None, ctypes.byref(st.s)))
    elif workload == "pagerank_f64":
        gg._check(L.gg_pagerank(g.h, a, p, None, ctypes.byref(st.s)))
    elif workload == "sssp":
        gg._check(L.gg_sssp(g.h, a, p, ctypes.byref(st.s)))
    else:
        gg._check(L.gg_bc(g.h, a, p, out.ptr2, ctypes.byref(st.s)))
    return st


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=64)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="bfs", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--check", action="store_true",
                    help="after timing, check the first timed run against the oracle on the full-size graph")
    ap.add_argument("--bins", default="autotune", choices=["autotune", "default"],
                    help="degree bins: the autotuner's pick for this graph, or the library defaults")
    ap.add_argument("--scale", type=int, default=None, help="override the workload's R-MAT scale / grid side")
    ap.add_argument("--adjacency", default="device", choices=["device", "host"],
                    help="neighbour / weight arrays in device memory or in mapped host memory (NVLink-C2C)")
    ap.add_argument("--build-budget-gb", type=float, default=0.0,
                    help="device GB the graph build may use beyond the graph (0 = free memory); "
                         "a smaller budget selects the partitioned build")
    ap.add_argument("--queries", type=int, default=2000, help="serve: queries in the stream")
    ap.add_argument("--rate", type=float, default=5000.0, help="serve: mean arrival rate (queries/s)")
    ap.add_argument("--plain", type=int, default=300, help="serve: queries replayed one at a time")
    ap.add_argument("--load-queries", type=int, default=1000,
                    help="serve: queries per stream offered at 50%% and 90%% of the measured capacity")
    ap.add_argument("--solo", type=int, default=16,
                    help="serve: idle SSSP pools with fewer waiting queries run them one at a time (0: always batch)")
    ap.add_argument("--window", type=float, default=5.0,
                    help="serve: SSSP batch window (ms) of the second stream at each offered load")
    ap.add_argument("--mix", action="store_true",
                    help="serve: also time plain and full-batch queries per graph and kind (the mix's ceiling)")
    args = ap.parse_args()
    if args.warmup < 3:
        log("warmup raised to 3 (timing rule)")
        args.warmup = 3
    if args.scale is not None:
        WORKLOADS[args.workload] = dict(WORKLOADS[args.workload], scale=args.scale)
        w = WORKLOADS[args.workload]
        WORKLOADS[args.workload]["desc"] = re.sub(r"scale \d+", f"scale {args.scale}", w["desc"])
    dist = Dist()
    try:
        if args.impl == "reference":
            return reference_arm(args, dist)
        if args.workload.endswith("_batched"):
            return gpu_arm_batched(args, dist)
        if args.workload == "serve":
            return gpu_arm_serve(args, dist)
        if args.workload == "build":
            return gpu_arm_build(args, dist)
        return gpu_arm(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    sys.exit(main())
