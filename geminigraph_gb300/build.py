"""Builds the CUDA library (libgemini_gb300.so, sm_103a) and the C++ command
lines in-tree.  Each translation unit compiles in its own nvcc process, in
parallel; nothing is rebuilt when its sources are older than its output."""
import glob
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libgemini_gb300.so")
INCLUDE = os.path.join(REPO, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
                     "--expt-relaxed-constexpr", "-I", INCLUDE]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


LIB_CHECK = os.path.join(PKG, "libgemini_gb300_check.so")


def build_library(verbose=False, check=False):
    """check=True builds libgemini_gb300_check.so: the same library with the
    device bounds checks of GG_CHECK compiled in (gg_common.cuh)."""
    build_dir = BUILD + ("_check" if check else "")
    lib = LIB_CHECK if check else LIB
    flags = NVCC_FLAGS + (["-DGG_CHECK"] if check else [])
    os.makedirs(build_dir, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    nvcc = _nvcc()
    objs = []
    jobs = []
    for src in sources:
        obj = os.path.join(build_dir, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append([nvcc] + flags + ["-c", src, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + p.stdout + p.stderr)
        return p.stderr

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for err in ex.map(run, jobs):
            if verbose and err:
                print(err)
    if _stale(lib, objs):
        run([nvcc] + ARCH + ["-shared", "-o", lib] + objs + ["-lpthread"])
    return lib


CPP = os.path.join(PKG, "cpp")
BIN = os.path.join(PKG, "bin")
TOOLKITS = ("bfs", "cc", "pagerank", "sssp", "bc")


def build_toolkits(verbose=False):
    """The five command lines (toolkits/*.cpp of the reference, same argv and
    output) against libgemini_gb300.so, with g++."""
    os.makedirs(BIN, exist_ok=True)
    headers = glob.glob(os.path.join(CPP, "*", "*.hpp")) + glob.glob(os.path.join(INCLUDE, "*.h"))
    jobs = []
    for app in TOOLKITS:
        src = os.path.join(CPP, "toolkits", app + ".cpp")
        out = os.path.join(BIN, app)
        if _stale(out, [src, LIB] + headers):
            jobs.append([os.environ.get("CXX", "g++"), "-O2", "-std=c++11", "-I", INCLUDE, "-I", CPP,
                         "-I", os.path.join(CPP, "toolkits"), src, "-o", out, "-L", PKG, "-lgemini_gb300",
                         "-Wl,-rpath,$ORIGIN/..", "-lpthread"])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("g++ failed:\n" + " ".join(cmd) + "\n" + p.stdout + p.stderr)

    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(run, jobs))
    return BIN


EXAMPLES = ("engine_toolkits",)


def build_examples(verbose=False):
    """Programs written against the header-only engine (gemini/engine.cuh):
    nvcc with extended lambdas, linked to libgemini_gb300.so."""
    os.makedirs(BIN, exist_ok=True)
    headers = glob.glob(os.path.join(CPP, "*", "*.hpp")) + glob.glob(os.path.join(CPP, "*", "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    for ex in EXAMPLES:
        src = os.path.join(CPP, "examples", ex + ".cu")
        out = os.path.join(BIN, ex)
        if not _stale(out, [src, LIB] + headers):
            continue
        cmd = [_nvcc()] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "--extended-lambda", "-I", INCLUDE, "-I", CPP,
                                  src, "-o", out, "-L", PKG, "-lgemini_gb300", "-Xlinker", "-rpath,$ORIGIN/.."]
        if verbose:
            print(" ".join(cmd), flush=True)
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + p.stdout + p.stderr)
    return BIN


def build(verbose=False):
    lib = build_library(verbose)
    with ThreadPoolExecutor(max_workers=3) as ex:
        jobs = [ex.submit(build_toolkits, verbose), ex.submit(build_examples, verbose),
                ex.submit(build_library, verbose, True)]
        for j in jobs:
            j.result()
    return lib


if __name__ == "__main__":
    print(build(verbose=True))
