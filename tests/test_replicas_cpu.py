"""Multi-GPU is replicas only: bench.py runs one independent replica per
rank and reduces the timing with a barrier and a max over ranks.  This runs
that host logic with the gloo backend, world size 2, on the CPU."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import importlib
    import torch.distributed as dist
    bench = importlib.import_module("bench")
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ws, r, local = bench._dist()
    bench._barrier(ws)
    mx = bench._barrier_max(float(10 * (rank + 1)), ws)
    q.put((r, ws, mx))
    dist.destroy_process_group()


def test_replica_timing_reduction_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    out = sorted(q.get() for _ in range(2))
    assert out == [(0, 2, 20.0), (1, 2, 20.0)]


def test_reference_arm_prints_only_on_rank0(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import importlib
    bench = importlib.import_module("bench")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class A:
        workload, steps, warmup, gpus = "tgv64", 1, 1, 2
    assert bench.run_reference(A()) == 0
    assert capsys.readouterr().out == ""
