"""Build libgcq.so (sm_103a) and the harness executables, in-tree.

Outputs (git-ignored) under gcq_gb300/_build/:
  libgcq.so                 C ABI of include/gcq.h (queues, harnesses, BFS, RT, roofline)
  tb, history, bfs, rt      harness executables with the reference's argv and
                            Makefile knobs, linked against libgcq.so
  rt_compact, rt_bench      the stream-compaction comparator and the
                            benchmark-scene ray tracer, same form

Every translation unit is compiled by nvcc for sm_103a only
(-gencode arch=compute_103a,code=sm_103a) in parallel, then linked with the
static CUDA runtime so the library loads without a CUDA runtime on the path.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HARNESS = os.path.join(HERE, "harness")
OUT = os.path.join(HERE, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(OUT, "libgcq.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code is compiled without floating-point contraction as well: on Arm the host
# compiler would otherwise fuse a*b+c in host-side setup (the ray tracer's scene),
# which then differs in the last bit from the CPU oracle built the same way.
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-I" + INCLUDE, "-I" + CSRC]
# Per-file extra flags: the ray tracer's device float math must round exactly like
# the CPU reference render, so it is compiled without FMA contraction.
EXTRA = {"gcq_rt.cu": ["--fmad=false"], "gcq_serve.cu": ["--fmad=false"]}


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgcq.so")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _deps():
    out = []
    for d in (CSRC, os.path.join(INCLUDE, "gcq")):
        out += [os.path.join(d, f) for f in os.listdir(d) if f.endswith((".cuh", ".h"))]
    out.append(os.path.join(INCLUDE, "gcq.h"))
    return out


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every CUDA translation unit for sm_103a and link libgcq.so."""
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()
    hdrs = _deps()
    srcs = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    jobs, objs = [], []
    for f in srcs:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT, f[:-3] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            jobs.append([cc] + ARCH + NVCC_FLAGS + EXTRA.get(f, []) + ["-Xptxas", "-v", "-c", src, "-o", obj])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            logs = list(ex.map(_run, jobs))
        if verbose:
            for l in logs:
                print(l)
        with open(os.path.join(OUT, "ptxas.log"), "w") as f:
            f.write("\n".join(logs))
    if force or jobs or _stale(LIB, objs):
        _run([cc] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs)
    _build_harness(force)
    return LIB


def _build_harness(force: bool):
    """Host-only C++ harness mains, linked against libgcq.so (rpath $ORIGIN)."""
    if not os.path.isdir(HARNESS):
        return
    cxx = os.environ.get("CXX", "g++")
    jobs = []
    for f in sorted(os.listdir(HARNESS)):
        if not f.endswith(".cpp"):
            continue
        src = os.path.join(HARNESS, f)
        exe = os.path.join(OUT, f[:-4])
        common = [os.path.join(HARNESS, h) for h in os.listdir(HARNESS) if h.endswith(".h")]
        if force or _stale(exe, [src, LIB, os.path.join(INCLUDE, "gcq.h")] + common):
            jobs.append([cxx, "-O2", "-std=c++17", "-I" + INCLUDE, "-I" + HARNESS, src, "-o", exe,
                         "-L" + OUT, "-lgcq", "-Wl,-rpath,$ORIGIN", "-pthread"])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(_run, jobs))


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
