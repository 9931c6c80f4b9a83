"""Build recipe for the oracle (test infrastructure: the checker, never the product).

Compiles the CPU restatements under oracle/ with the host C++ compiler into
oracle/_build/:

  liboracle.so   lincheck.cpp (FIFO linearizability checker), cpu_queues.cpp
                 (std::atomic restatements of the four queues), bfs_serial.cpp
                 (serial BFS), rt_cpu.cpp (serial ray tracer)
  lincheck       command-line checker with the reference checker's verdicts

The reference itself (HIP for AMD GPUs) cannot be compiled in this image: there
is no hipcc/ROCm, and its CUDA branch does not compile (missing return type at
gwf_ring.hpp:173, removed non-_sync shuffles at gwf_ring.hpp:931-932).  So there
is no oracle/_ref build; these restatements are the CPU side.

Usage:  python -m oracle.build        (or oracle.build.build() from Python)
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")

LIB_SOURCES = ["lincheck.cpp", "cpu_queues.cpp", "bfs_serial.cpp", "rt_cpu.cpp"]
CXX = os.environ.get("CXX", "g++")
# -ffp-contract=off keeps a*b+c as two rounded operations so the CPU ray tracer
# performs the same float operations as the device one (built with --fmad=false).
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-pthread", "-ffp-contract=off", "-Wall",
            "-Wno-unused-function"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, sanitize: str | None = None) -> str:
    """Compile liboracle.so and the lincheck CLI; returns the library path.

    sanitize="thread" builds a ThreadSanitizer copy (liboracle_tsan.so) of the
    same sources for the race tests.
    """
    os.makedirs(OUT, exist_ok=True)
    srcs = [os.path.join(HERE, s) for s in LIB_SOURCES if os.path.exists(os.path.join(HERE, s))]
    hdrs = [os.path.join(HERE, h) for h in os.listdir(HERE) if h.endswith((".h", ".hpp"))]
    suffix = "" if not sanitize else "_" + {"thread": "tsan", "address": "asan"}[sanitize]
    flags = list(CXXFLAGS)
    if sanitize:
        flags = [f for f in flags if not f.startswith("-O")] + ["-O1", "-g", "-fsanitize=" + sanitize]
    objs = []
    jobs = []
    for s in srcs:
        o = os.path.join(OUT, os.path.basename(s)[:-4] + suffix + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append([CXX] + flags + ["-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        list(ex.map(_run, jobs))
    lib = os.path.join(OUT, "liboracle%s.so" % suffix)
    if force or jobs or _stale(lib, objs):
        _run([CXX] + flags + ["-shared", "-o", lib] + objs)
    if not sanitize:
        cli = os.path.join(OUT, "lincheck")
        src = os.path.join(HERE, "lincheck.cpp")
        if force or _stale(cli, [src]):
            _run([CXX] + CXXFLAGS + ["-DGCQ_LINCHECK_MAIN", src, "-o", cli])
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv,
                sanitize="thread" if "--tsan" in sys.argv else None))
