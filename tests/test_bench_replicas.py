"""Multi-GPU form of the benchmark: independent replicas, max-over-ranks
timing (gloo, two CPU ranks; no GPU)."""

import io
import os
import socket
import sys
from contextlib import redirect_stdout

import torch.multiprocessing as mp

from conftest import ROOT

sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, world, "cpu")
    q.put((rank, ms, bench.replica_value(world, 300, ms)))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_replica_value_with_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [15.0, 15.0]
    assert all(abs(o[2] - 2 * 300 / 0.015) < 1e-6 for o in out)


def test_reference_arm_prints_only_on_rank_0(monkeypatch):
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    buf = io.StringIO()

    class A:
        gpus, steps, warmup = 2, 2, 3
    with redirect_stdout(buf):
        assert bench.run_reference(A) is None
    assert buf.getvalue() == ""
