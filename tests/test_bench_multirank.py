"""The multi-GPU path of bench.py on the CPU: replicas over a gloo process group of
two ranks.  The whole-job value is all ranks' work over the slowest rank's time;
the reference arm runs on rank 0 only."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r took (r + 1) ms for 10 (r + 1) operations
        ms, ops = bench.whole_job(rank + 1.0, 10 * (rank + 1))
        r, w, local = bench._env_rank()
        out.put((rank, ms, ops, r, w, local))
    finally:
        dist.destroy_process_group()


def test_whole_job_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, ms, ops, r, w, local in got:
        assert (ms, ops) == (2.0, 30.0)          # max time, summed work
        assert (r, w, local) == (rank, 2, rank)


def test_whole_job_single_process():
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    assert bench.whole_job(3.5, 7) == (3.5, 7.0)


def test_reference_arm_other_ranks_exit(monkeypatch, capsys):
    """Under torchrun only rank 0 runs the CPU reference arm and prints its line."""
    import sys
    import types
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    args = types.SimpleNamespace(warmup=3, steps=2, gpus=2)
    assert bench.run_reference(args) == 0
    assert capsys.readouterr().out == ""
