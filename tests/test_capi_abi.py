"""The drop-in boundary: every function declared in include/gcq.h is exported by
libgcq.so and bound in gcq_gb300.SIGNATURES (no GPU calls are made here)."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    text = open(header).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gcq_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def built_lib():
    from gcq_gb300 import build
    return build.build()


def _exports(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    return {l.split()[-1] for l in out.splitlines() if l.strip()}


def test_header_symbols_exported(built_lib):
    declared = _declared(os.path.join(ROOT, "include", "gcq.h"))
    assert len(declared) >= 15
    exported = _exports(built_lib)
    missing = [d for d in declared if d not in exported]
    assert not missing, missing


def test_bindings_cover_header(built_lib):
    import gcq_gb300
    declared = _declared(os.path.join(ROOT, "include", "gcq.h"))
    missing = [d for d in declared if d not in gcq_gb300.SIGNATURES]
    assert not missing, missing


def test_library_loads_without_gpu(built_lib):
    import ctypes
    import gcq_gb300
    L = gcq_gb300.lib()
    # pure host functions are safe without a device
    assert L.gcq_strerror(0) == b"ok"
    assert L.gcq_strerror(-6).startswith(b"configuration")
    k = gcq_gb300.Knobs()
    L.gcq_default_knobs(ctypes.byref(k))
    assert (k.help_delay, k.enq_patience, k.deq_patience) == (64, 128, 256)
    assert k.ymc_patience == 16 and k.ymc_ops_per_thread == 512




def test_argument_checks_without_gpu(built_lib):
    """Argument checks that return before any CUDA call: invalid configurations are
    rejected with their status on a machine without a GPU."""
    import ctypes
    import gcq_gb300 as g
    L = g.lib()
    q = ctypes.c_void_p()
    # SCQ rings: Threshold = 3N - 1 is an int, so N <= 2^29
    assert L.gcq_create(g.KINDS["gwfq"], 30, 64, None, ctypes.byref(q)) == g.EINVAL
    assert L.gcq_create(g.KINDS["glfq"], 30, 64, None, ctypes.byref(q)) == g.EINVAL
    assert L.gcq_create(g.KINDS["gwfq"], 15, 0, None, ctypes.byref(q)) == g.EINVAL
    r = g.RtResult()
    img = None
    # benchmark-scene renderer: scene, size, queue kind, ring too small for a tile
    cases = [((g.KINDS["gwfq"], 2, 64, 64, 32, 64, 4, 15, 1), g.EINVAL),
             ((g.KINDS["gwfq"], 0, 0, 64, 32, 64, 4, 15, 1), g.EINVAL),
             ((g.KINDS["gwfq"], 0, 64, 64, 32, 64, -1, 15, 1), g.EINVAL),
             ((7, 0, 64, 64, 32, 64, 4, 15, 1), g.EUNSUPPORTED),
             ((g.KINDS["gwfq"], 0, 64, 64, 32, 64, 4, 9, 1), g.ECAPACITY)]
    for args, want in cases:
        assert L.gcq_rt_bounce_render(*args, img, ctypes.byref(r)) == want, args
    ctx = ctypes.c_void_p()
    assert L.gcq_rt_ctx_create(g.KINDS["sfq"], 1, 64, 64, 64, 32, 4, 10, 1, 0, ctypes.byref(ctx)) == g.ECAPACITY
    assert L.gcq_rt_ctx_render(None, None, 0, None, ctypes.byref(r)) == g.EINVAL
    # harness checks and bounded runs: a null queue or a missing result is rejected
    # before any device work
    tr = g.TbResult()
    assert L.gcq_tb_run_bounded(None, 0, 50, 1024, 256, 128, 10.0, 10.0, 0, ctypes.byref(tr)) == g.EINVAL
    fr = g.FifoResult()
    assert L.gcq_fifo_check_split(None, 1024, 256, 50, 32, ctypes.byref(fr)) == g.EINVAL
    n = ctypes.c_size_t()
    assert L.gcq_drain_host(None, 1024, 256, None, 0, ctypes.byref(n)) == g.EINVAL
    # served engine defaults
    cfg = g.ServeCfg()
    L.gcq_serve_default_cfg(ctypes.byref(cfg))
    assert cfg.budget_bytes == 150 << 30 and cfg.rt_scenes == 0
    assert (cfg.rt_width, cfg.rt_height, cfg.rt_tile_px, cfg.rt_max_bounces, cfg.rt_slots) == (1024, 1024, 32, 4, 1024)


C_CALLER = r"""
#include <stdio.h>
#include <string.h>
#include "gcq.h"
int main(void) {
    gcq_knobs k;
    gcq_serve_cfg c;
    gcq_rt_result r;
    gcq_queue* q = 0;
    gcq_default_knobs(&k);
    gcq_serve_default_cfg(&c);
    if (gcq_create(GCQ_GWFQ, 30, 64, &k, &q) != GCQ_EINVAL) return 2;
    if (gcq_rt_bounce_render(GCQ_WFQ, 2, 64, 64, 32, 64, 4, 15, 1, 0, &r) != GCQ_EINVAL) return 3;
    printf("%s|%u|%u\n", gcq_strerror(GCQ_EINVAL), k.help_delay, c.rt_tile_px);
    return 0;
}
"""


def test_header_is_plain_c(built_lib, tmp_path):
    """include/gcq.h compiles as strict C11 and a C caller links and runs against
    libgcq.so (host-only calls: no GPU needed)."""
    src = tmp_path / "caller.c"
    src.write_text(C_CALLER)
    exe = tmp_path / "caller"
    lib_dir = os.path.dirname(built_lib)
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I" + os.path.join(ROOT, "include"),
                    str(src), "-o", str(exe), "-L" + lib_dir, "-lgcq", "-Wl,-rpath," + lib_dir], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out
    assert out.stdout.strip() == "invalid argument|64|32"
