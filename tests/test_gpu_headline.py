"""The benchmark's timed launch, checked bit for bit.

bench.py times one batched plan: 16 communicators of 4..256 ranks (1024 rank
blocks in one persistent cooperative launch, replayed as a CUDA graph), each
running Bcast, Allreduce(SUM) and Alltoall on int32 and FP64 data, with the
schedules and threads per rank the autotuner picks.  These tests build that
plan with bench.build_plan and coll.autotune, give every buffer fresh data,
run the captured launch and compare every output of every rank with its
inputs: Bcast and Alltoall as copies, Allreduce against a NumPy rank-order
fold (acc = x_0; acc = x_q + acc, the order of the reference's MPI_Reduce,
gpu_libs/gpu_mpi/mpi.cu:209-225).  At 2^17 elements per rank every Allreduce
segment is larger than the bulk-staged fold's chunk, so the staged pipeline
(and the bulk copy engine of Bcast and Alltoall) runs under the contention of
the full launch; the schedules are also forced one by one.
"""
import importlib.util
import os
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _mod(name, path):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[spec.name] = mod
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="module")
def env(gpu_built):
    sys.path.insert(0, gpu_built.PKG)
    bench = _mod("bench_mod", os.path.join(ROOT, "bench.py"))
    coll = _mod("gpumpi_coll", os.path.join(gpu_built.PKG, "gpumpi_coll.py"))
    lib = coll.bind(gpu_built.load_library())
    return bench, coll, lib


def _run_checked(bench, coll, lib, lg, algo=None, tune_reps=1, sample=None):
    import torch

    n = 1 << lg
    plan, comms, keep, items, descs = bench.build_plan(coll, lib, torch, bench.COMM_SIZES, n, True, 128)
    plan.close()
    threads = 128
    if algo is None:
        threads, _, _ = coll.autotune(lib, descs, reps=tune_reps)
    else:
        for d in descs:
            d.algo = algo
    plan = coll.Plan(lib, descs, threads=threads, batched=True)
    stream = torch.cuda.Stream()
    plan.capture(stream.cuda_stream)
    try:
        g = torch.Generator(device="cuda").manual_seed(lg * 10 + (algo or 0))
        for it in items:
            bench.fill_random(torch, it.send if it.send is not None else it.recv, it.dt, g)
            if it.send is not None:
                it.recv.fill_(-7)
        torch.cuda.synchronize()
        plan.launch(stream.cuda_stream)
        torch.cuda.synchronize()
        assert coll.status(lib) is None
        bad = bench.verify_items(torch, items, sample=sample)
        assert not bad, bad
        # a second replay of the same graph leaves the same results
        plan.launch(stream.cuda_stream)
        torch.cuda.synchronize()
        assert not bench.verify_items(torch, items, sample=4096)
    finally:
        plan.close()
        for c in comms:
            c.close()
        del items
        torch.cuda.empty_cache()


def test_headline_plan_tuned_bitwise_2_17(env):
    bench, coll, lib = env
    _run_checked(bench, coll, lib, 17)


@pytest.mark.parametrize("algo", [1, 2, 3, 4])
def test_headline_plan_each_schedule_bitwise_2_17(env, algo):
    """algo 1/2/3/4 for every call: Allreduce every-rank fold / reduce-scatter
    + allgather / pushing bulk-staged fold (and 4 as 3); Alltoall whole-block /
    per-warp / bulk engine / vectors of all blocks over all threads; Bcast
    from the root / binomial tree (and 3, 4 as 1)."""
    bench, coll, lib = env
    _run_checked(bench, coll, lib, 17, algo=algo)


def test_headline_plan_tuned_bitwise_2_20(env):
    """The benchmark's own size: 2^20 elements per rank, about 64 GB of
    buffers; every element of every output is checked."""
    import torch

    free, _ = torch.cuda.mem_get_info()
    if free < 80 * (1 << 30):
        pytest.skip("needs about 70 GB of free device memory")
    bench, coll, lib = env
    _run_checked(bench, coll, lib, 20, tune_reps=1)
