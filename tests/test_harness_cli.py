"""The harness executables (gcq_gb300/harness/*.cpp): built, usage paths on the CPU;
on the GPU each one runs the reference harness's command line and its output is
checked against the oracle."""
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BUILD = os.path.join(ROOT, "gcq_gb300", "_build")
HARNESS = os.path.join(ROOT, "gcq_gb300", "harness")


@pytest.fixture(scope="module")
def built():
    from gcq_gb300 import build
    build.build()
    return BUILD


def _run(args, cwd, env=None, timeout=300):
    e = dict(os.environ)
    e.update(env or {})
    return subprocess.run(args, cwd=cwd, env=e, capture_output=True, text=True, timeout=timeout)


def _compile(name, out, defines):
    cmd = ["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), "-I" + HARNESS] + \
          ["-D" + d for d in defines] + [os.path.join(HARNESS, name + ".cpp"), "-o", out,
                                         "-L" + BUILD, "-lgcq", "-Wl,-rpath," + BUILD, "-pthread"]
    subprocess.run(cmd, check=True)
    return out


def test_harness_binaries_built(built):
    for exe in ["tb", "history", "bfs", "rt", "rt_compact", "rt_bench"]:
        assert os.access(os.path.join(built, exe), os.X_OK), exe


def test_bfs_usage_without_graph(built, tmp_path):
    r = _run([os.path.join(built, "bfs")], cwd=tmp_path)
    assert r.returncode == 1 and "Usage: --graph <path> | --grid R C" in r.stdout
    r = _run([os.path.join(built, "bfs"), "--bogus"], cwd=tmp_path)
    assert r.returncode == 1 and "Unknown: --bogus" in r.stdout


def test_unknown_queue_rejected(built, tmp_path):
    r = _run([os.path.join(built, "bfs")], cwd=tmp_path, env={"QUEUE": "bq"})
    assert r.returncode == 2 and "Unsupported QUEUE" in r.stderr


def test_rt_bench_rejections(built, tmp_path):
    # refused before any device work
    r = _run([os.path.join(built, "rt_bench"), "5"], cwd=tmp_path, env={"QUEUE": "gwfq", "GPU_NAME": "none"})
    assert r.returncode == 1 and "ERROR: invalid argument (scene 5" in r.stderr


def test_history_bad_args(built, tmp_path):
    r = _run([os.path.join(built, "history"), str(tmp_path / "h.jsonl"), "0"], cwd=tmp_path)
    assert r.returncode == 2


@pytest.mark.gpu
def test_tb_balanced_fifo(built, tmp_path):
    exe = _compile("tb", str(tmp_path / "tb_gwfq_fifo1"),
                   ["USE_GWFQ", "RUN_MS=60", "WARMUP_MS=10", "CHUNK_OPS=32", "ONLY_BALANCED=1", "MODE_FIFO=1",
                    'CSV_FILE="bench.csv"'])
    r = _run([exe], cwd=tmp_path, env={"TB_THREADS": "1024,4096"})
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if "balanced | threads=" in l]
    assert len(lines) == 2
    for l in lines:
        assert float(re.search(r"succ=\s*([\d.]+) Mops/s", l).group(1)) > 0
    assert r.stdout.count("FIFO verified: YES") == 2
    rows = open(tmp_path / "bench.csv").read().splitlines()
    assert rows[0].startswith("gpu_name,queue,mode,producer_percent,threads") and len(rows) == 3
    assert rows[1].split(",")[1:5] == ["gWFQ", "balanced", "-1", "1024"]


@pytest.mark.gpu
@pytest.mark.parametrize("queue", ["gwfq", "sfq"])
def test_history_cli_linearizable(built, oracle_lib, tmp_path, queue):
    out = tmp_path / "h.jsonl"
    r = _run([os.path.join(built, "history"), str(out), "64", "16", "0", "50"], cwd=tmp_path,
             env={"QUEUE": queue, "HIST_KEEP_BUSY": "1"})
    assert r.returncode == 0, r.stderr
    recs = oracle_lib.load_jsonl(str(out))
    assert len(recs) == 64 * 16 * 2
    assert oracle_lib.check(recs) == "Linearizable (FIFO)"


@pytest.mark.gpu
def test_bfs_cli_grid_and_mtx(built, oracle_lib, tmp_path):
    import gcq_gb300 as g
    r = _run([os.path.join(built, "bfs"), "--grid", "212", "212", "--keep", "0.6", "--diag", "0.01", "--seed", "2",
              "--iters", "2", "--warmup", "1", "--threads", "2048"], cwd=tmp_path, env={"QUEUE": "glfq"})
    assert r.returncode == 0, r.stderr
    off, idx = g.graph_grid(212, 212, 0.6, 0.01, 2)
    lv, ecc = oracle_lib.bfs(off, idx, 0)
    m = re.search(r"Reached: (\d+)/(\d+) Levels: (\d+)", r.stdout)
    assert (int(m.group(1)), int(m.group(2)), int(m.group(3))) == (int((lv >= 0).sum()), len(lv), ecc + 1)
    # the same graph as a MatrixMarket file, 1-based, each edge once
    mtx = tmp_path / "gridB.mtx"
    with open(mtx, "w") as f:
        src = np.repeat(np.arange(len(off) - 1), np.diff(off))
        keep = src < idx
        f.write("%%%%MatrixMarket matrix coordinate pattern symmetric\n%d %d %d\n" % (len(lv), len(lv), keep.sum()))
        for u, v in zip(src[keep], idx[keep]):
            f.write("%d %d\n" % (u + 1, v + 1))
    r = _run([os.path.join(built, "bfs"), "--graph", str(mtx), "--iters", "1", "--warmup", "0", "--persistent", "1"],
             cwd=tmp_path, env={"QUEUE": "gwfq", "CSV_NAME": "b.csv"})
    assert r.returncode == 0, r.stderr
    m2 = re.search(r"Reached: (\d+)/(\d+) Levels: (\d+)", r.stdout)
    assert m2.groups() == m.groups()
    assert open(tmp_path / "b.csv").read().startswith(r.stdout.split("GPU: ")[1].split("  CUs")[0])


@pytest.mark.gpu
def test_rt_cli_writes_image(built, oracle_lib, tmp_path):
    r = _run([os.path.join(built, "rt"), "1", "4", "256"], cwd=tmp_path, env={"QUEUE": "gwfq"})
    assert r.returncode == 0, r.stderr
    assert "=== RESULTS ===" in r.stdout and "Image saved: rt_gwfq_cornell.ppm" in r.stdout
    data = open(tmp_path / "rt_gwfq_cornell.ppm", "rb").read()
    assert data.startswith(b"P6\n1280 720\n255\n") and len(data) == len(b"P6\n1280 720\n255\n") + 1280 * 720 * 3
    # the image equals the oracle's render of the same scene, quantised as the file is
    img = np.zeros((720, 1280, 3), np.float32)
    oracle_lib.lib().oracle_rt_render(1, 1280, 720, 4, img.ctypes.data)
    want = np.clip(img * 255.0, 0, 255).astype(np.uint8)
    got = np.frombuffer(data[len(b"P6\n1280 720\n255\n"):], np.uint8).reshape(720, 1280, 3)
    assert np.array_equal(got, want)
    assert "GWFQ,cornell,256,4," in open(tmp_path / "rt_queue_perf.csv").read()


@pytest.mark.gpu
def test_rt_compact_cli(built, oracle_lib, tmp_path):
    r = _run([os.path.join(built, "rt_compact"), "2", "6"], cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    assert "Image saved: rt_COMPACT_mirror_tunnel.ppm" in r.stdout
    img = np.zeros((720, 1280, 3), np.float32)
    n = oracle_lib.lib().oracle_rt_compact_render(2, 1280, 720, 6, img.ctypes.data)
    assert "Total rays traced: %d" % n in r.stdout
    data = open(tmp_path / "rt_COMPACT_mirror_tunnel.ppm", "rb").read()
    got = np.frombuffer(data[len(b"P6\n1280 720\n255\n"):], np.uint8).reshape(720, 1280, 3)
    assert np.array_equal(got, np.clip(img * 255.0, 0, 255).astype(np.uint8))
    assert ",COMPACT,256,%d," % n in open(tmp_path / "rt_performance.csv").read()


@pytest.mark.gpu
def test_rt_bench_cli(built, oracle_lib, tmp_path):
    """The benchmark-scene harness: the 1024x1024 room with G-LFQ; the PPM equals the
    serial render quantised as the file is, and the ray count matches."""
    r = _run([os.path.join(built, "rt_bench"), "1", "4", "1024"], cwd=tmp_path, env={"QUEUE": "glfq"})
    assert r.returncode == 0, r.stderr
    assert "Image saved: rtb_glfq_room.ppm" in r.stdout
    img = np.zeros((1024, 1024, 3), np.float32)
    n = oracle_lib.lib().oracle_rt_bounce_render(1, 1024, 1024, 4, 1, 16, img.ctypes.data)
    assert "Total rays traced:  %d" % n in r.stdout
    data = open(tmp_path / "rtb_glfq_room.ppm", "rb").read()
    hdr = b"P6\n1024 1024\n255\n"
    assert data.startswith(hdr) and len(data) == len(hdr) + 1024 * 1024 * 3
    got = np.frombuffer(data[len(hdr):], np.uint8).reshape(1024, 1024, 3)
    assert np.array_equal(got, np.clip(img * 255.0, 0, 255).astype(np.uint8))
    assert "GLFQ,room,1024,4,1048576,%d," % n in open(tmp_path / "rt_bench_perf.csv").read()
