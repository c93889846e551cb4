"""Multi-GPU form of the benchmark on CPU: independent replicas, gloo only for
the barrier and the max-over-ranks time (no data-path collective)."""
import importlib.util
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules[spec.name] = mod
    spec.loader.exec_module(mod)
    return mod


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench = _bench()
    dist.barrier()
    t = bench.max_over_ranks(dist, torch, 1.0 + rank)
    out[rank] = t
    dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    port = _free_port()
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert dict(out) == {0: 2.0, 1: 2.0}


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    bench = _bench()
    monkeypatch.setenv("RANK", "1")
    args = type("A", (), {"cpu_lg": 16, "warmup": 3, "steps": 2, "gpus": 2})()
    bench.reference_arm(args)        # rank 1: no work, no output
    assert capsys.readouterr().out == ""


def test_single_process_needs_no_collective():
    import torch
    assert _bench().max_over_ranks(None, torch, 3.5) == 3.5
