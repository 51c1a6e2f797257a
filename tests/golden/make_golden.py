"""Generates tests/golden/*.npz from the Gemini reference itself.

Runs the reference toolkits built from their own sources by
oracle/build_ref.sh (oracle/_ref/bin/{bfs,cc,pagerank,sssp,bc}) on small
seeded graphs and stores their full result arrays.  The toolkits print only
summaries, so the arrays are taken from the oracle/shim/numa.h dump hook: every
vertex array freed through numa_free is written out (GG_REF_DUMP_DIR).  Dump
order per toolkit (core/graph.hpp:488,912 free the load-time out_degree first):

    bfs       dump_000 out_degree, dump_001 parent               (bfs.cpp:105)
    pagerank  dump_000 out_degree, dump_001 curr (final ranks)   (pagerank.cpp:126)
    cc        dump_000 out_degree (both endpoints), dump_001 label (cc.cpp:106)
    sssp      dump_000 out_degree, dump_001 distance             (sssp.cpp:102)
    bc        dump_000 out_degree, dump_001 dependencies, dump_002 inv_num_paths
                                                                  (bc.cpp:192-193)

Only the first compute() of the six each toolkit runs is dumped
(GG_REF_DUMP_MAX).  The stdout of that run is kept too.

Usage: python tests/golden/make_golden.py   (needs the reference checkout to
have been staged and built: sh oracle/build_ref.sh)
"""
import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(HERE))
import graphgen  # noqa: E402

BIN = os.path.join(REPO, "oracle", "_ref", "bin")


def edgecase_graph():
    """V = 1000 (not a multiple of 64): self-loops, duplicate edges, isolated
    vertices, a hub, a long chain, and ids up to V-1."""
    rng = np.random.default_rng(7)
    V = 1000
    s = list(rng.integers(0, 600, 3000))
    d = list(rng.integers(0, 600, 3000))
    for v in range(600, 700):        # chain 600 -> 601 -> ... -> 699
        s.append(v)
        d.append(v + 1)
    s += [5] * 200                   # hub 5 with duplicates
    d += list(rng.integers(0, 1000, 100)) * 2
    s += [10, 10, 11, 999, 999]      # self-loops and a duplicated self-loop
    d += [10, 10, 11, 999, 0]
    # vertices 701..998 except 999's targets stay isolated
    src = np.array(s, dtype=np.uint32)
    dst = np.array(d, dtype=np.uint32)
    w = graphgen.weights(3, np.arange(len(src), dtype=np.uint64))
    return V, src, dst, w


def graphs():
    out = []
    for scale in (10, 12):
        s, d, w = graphgen.rmat(scale, 16, seed=scale, weighted=True)
        out.append(dict(name=f"rmat{scale}", V=1 << scale, src=s, dst=d, w=w,
                        gen=("rmat", scale, 16, scale), store_edges=False))
    s, d, w = graphgen.grid(32, seed=5, weighted=True)
    out.append(dict(name="grid32", V=32 * 32, src=s, dst=d, w=w, gen=("grid", 32, 0, 5),
                    store_edges=False))
    V, s, d, w = edgecase_graph()
    out.append(dict(name="edgecase", V=V, src=s, dst=d, w=w, gen=("explicit", 0, 0, 0),
                    store_edges=True))
    return out


def run_ref(app, path, V, arg, dumps, tmp):
    dump_dir = tempfile.mkdtemp(dir=tmp)
    env = dict(os.environ, GG_REF_DUMP_DIR=dump_dir, GG_REF_DUMP_MAX=str(dumps),
               GG_REF_THREADS="4", OMP_NUM_THREADS="4")
    cmd = [os.path.join(BIN, app), path, str(V)] + ([str(arg)] if arg is not None else [])
    p = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=600)
    if p.returncode != 0:
        raise RuntimeError(f"{cmd} failed: {p.returncode}\n{p.stdout}\n{p.stderr}")
    first_run = p.stdout.split("exec_time=")[0]
    rest = p.stdout.split("exec_time=")[1].split("\n", 1)[1]
    summary = rest.split("active(")[0].split("forward")[0].split("delta(")[0]
    files = [os.path.join(dump_dir, f"dump_{i:03d}.bin") for i in range(dumps)]
    return [open(f, "rb").read() for f in files], first_run, summary


def main():
    if not os.path.exists(os.path.join(BIN, "bfs")):
        sys.exit("reference toolkits not built: run sh oracle/build_ref.sh first")
    tmp = tempfile.mkdtemp()
    for g in graphs():
        V = g["V"]
        src, dst, w = g["src"], g["dst"], g["w"]
        root = graphgen.pick_root(src, V, seed=V + 11)
        unw = graphgen.to_records(src, dst)
        wtd = graphgen.to_records(src, dst, w)
        if g["name"] == "edgecase":
            unw += b"\x01\x02\x03"   # trailing partial record: ignored by the loader
            wtd += b"\x01\x02\x03\x04\x05"
        pu = os.path.join(tmp, g["name"] + ".bin")
        pw = os.path.join(tmp, g["name"] + ".wbin")
        open(pu, "wb").write(unw)
        open(pw, "wb").write(wtd)
        res = dict(V=np.uint32(V), root=np.uint32(root),
                   gen=np.array(g["gen"], dtype=object).astype(str),
                   edges_sha256=hashlib.sha256(wtd).hexdigest())
        if g["store_edges"]:
            res.update(src=src, dst=dst, w=w)
        (deg, parent), out, summ = run_ref("bfs", pu, V, root, 2, tmp)
        res.update(out_degree=np.frombuffer(deg, np.uint32), bfs_parent=np.frombuffer(parent, np.uint32),
                   bfs_stdout=out, bfs_summary=summ)
        (_, ranks), out, summ = run_ref("pagerank", pu, V, 20, 2, tmp)
        res.update(pr_ranks=np.frombuffer(ranks, np.float64), pr_stdout=out, pr_summary=summ)
        (sdeg, label), out, summ = run_ref("cc", pu, V, None, 2, tmp)
        res.update(sym_degree=np.frombuffer(sdeg, np.uint32), cc_label=np.frombuffer(label, np.uint32),
                   cc_stdout=out, cc_summary=summ)
        (_, dist), out, summ = run_ref("sssp", pw, V, root, 2, tmp)
        res.update(sssp_dist=np.frombuffer(dist, np.float32), sssp_stdout=out, sssp_summary=summ)
        (_, dep, inv), out, summ = run_ref("bc", pu, V, root, 3, tmp)
        res.update(bc_dep=np.frombuffer(dep, np.float64), bc_inv=np.frombuffer(inv, np.float64),
                   bc_stdout=out, bc_summary=summ)
        np.savez_compressed(os.path.join(HERE, g["name"] + ".npz"), **res)
        print(g["name"], "V", V, "E", len(src), "root", root)


if __name__ == "__main__":
    main()
