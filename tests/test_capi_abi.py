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


