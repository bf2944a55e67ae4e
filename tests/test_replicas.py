"""The multi-GPU path is replicas (one process per GPU, no data-path
collective): two gloo ranks on CPU check the max-over-ranks timing, the
whole-job value, and that only rank 0 runs the reference arm."""
import io
import os
import sys
from contextlib import redirect_stdout

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench.max_over_ranks(10.0 * (rank + 1), world, device="cpu")
    v = bench.job_value(1e9, 4, ms, world, 1e9)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, ms, v))


def test_two_gloo_ranks():
    import random

    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + random.randint(0, 2000)
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    # both ranks see the slowest rank's 20 ms; 2 ranks x 4 steps x 1e9 units / 20 ms
    assert [g[1] for g in got] == [20.0, 20.0]
    assert all(abs(g[2] - 2 * 4 / 0.020) < 1e-6 for g in got)


def test_reference_arm_runs_on_rank0_only(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    args = bench.argparse.Namespace(workload="radix", warmup=1, steps=1, cpu_sample_log=10, gpus=2)
    buf = io.StringIO()
    with redirect_stdout(buf):
        assert bench.run_reference(args) is None
    assert buf.getvalue() == ""
