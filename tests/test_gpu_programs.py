"""Converted programs on the GPU against the hostmpi oracle (parity gate)."""
import pytest

from kat_cases import KAT_CASES, check_all_ok

pytestmark = pytest.mark.gpu
GPU_OPTS = ["--timeout-ms", "20000", "--max-seconds", "120"]


@pytest.mark.parametrize("prog,scenario,nranks", KAT_CASES)
def test_gpu_known_answers(gpu_built, prog, scenario, nranks):
    args = [scenario] if scenario else []
    res = gpu_built.run_program(prog, args, nranks=nranks, extra=GPU_OPTS, timeout=180)
    check_all_ok(res, scenario, nranks)


@pytest.mark.parametrize("n,ranks", [(1000, 1), (100000, 3), (10000000, 8), (1000003, 64)])
def test_gpu_pi_bit_exact(gpu_built, n, ranks):
    """FP64 rank-order MPI_Reduce: GPU result equals the host MPI result bit for bit."""
    g = gpu_built.run_program("pi", [str(n)], nranks=ranks, extra=GPU_OPTS, timeout=180)
    c = gpu_built.run_oracle("pi", [str(n)], nranks=ranks, timeout=180)
    assert g.returncode == 0, g.stderr
    assert g.lines("pi bits") == c.lines("pi bits")
    assert g.lines("pi is approximately") == c.lines("pi is approximately")


@pytest.mark.parametrize("lg,iters,ranks", [(8, 2, 40), (12, 1, 1024), (14, 2, 256)])
def test_gpu_coll_bench_matches_oracle(gpu_built, lg, iters, ranks):
    """Batched-collectives program: every result checksum equals the host MPI run."""
    g = gpu_built.run_program("coll_bench", [str(lg), str(iters)], nranks=ranks,
                              extra=GPU_OPTS + ["-p", "4G"], timeout=300)
    c = gpu_built.run_oracle("coll_bench", [str(lg), str(iters)], nranks=ranks, timeout=300)
    assert g.returncode == 0, g.stderr[-2000:]
    assert c.returncode == 0, c.stderr[-2000:]
    assert g.lines("coll_bench checksum") == c.lines("coll_bench checksum")
