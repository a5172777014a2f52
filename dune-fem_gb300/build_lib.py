"""Builds libgbfem.so (the CUDA kernels + C-ABI) in-tree for sm_103a.

Each translation unit under csrc/ is compiled by its own nvcc process, in
parallel, into _build/; they are linked into lib/libgbfem.so.  Rebuilds only
what changed (object older than any source or header).  bench_csrc/ (the
benchmark's FMA-peak microbenchmark, not part of the C-ABI) becomes
lib/libgbfem_bench.so.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BENCH_CSRC = os.path.join(HERE, "bench_csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libgbfem.so")
BENCH_LIB = os.path.join(LIBDIR, "libgbfem_bench.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I", INCLUDE, "-I", CSRC]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _deps_mtime():
    m = 0.0
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            if f.endswith((".cuh", ".hpp", ".h")):
                m = max(m, os.path.getmtime(os.path.join(d, f)))
    return m


def _compile(src, obj, extra):
    cmd = [_nvcc()] + ARCH + NVCC_FLAGS + extra + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return r.stderr


def build(verbose=False, extra_flags=()):
    """Compiles every csrc/*.cu and links lib/libgbfem.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    dep_m = _deps_mtime()
    jobs = []
    objs = []
    bench_objs = []
    for d, out in ((CSRC, objs), (BENCH_CSRC, bench_objs)):
        for f in sorted(f for f in os.listdir(d) if f.endswith(".cu")):
            src = os.path.join(d, f)
            obj = os.path.join(BUILD, ("bench_" if d == BENCH_CSRC else "") + f[:-3] + ".o")
            out.append(obj)
            if (not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), dep_m)):
                jobs.append((src, obj))
    if jobs:
        workers = min(len(jobs), max(2, os.cpu_count() or 2))
        with cf.ThreadPoolExecutor(workers) as ex:
            futs = {ex.submit(_compile, s, o, list(extra_flags)): s for s, o in jobs}
            for fut in cf.as_completed(futs):
                out = fut.result()
                if verbose and out:
                    sys.stderr.write(out)
    for lib, lobjs in ((LIB, objs), (BENCH_LIB, bench_objs)):
        if jobs or not os.path.exists(lib):
            cmd = [_nvcc()] + ARCH + ["-shared", "-o", lib] + lobjs + ["-lcudart"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
