"""Converted programs on the GPU against the hostmpi oracle (parity gate)."""
import pytest

from conftest import run_oracle

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
    c = run_oracle("pi", [str(n)], nranks=ranks, timeout=180)
    assert g.returncode == 0, g.stderr
    assert g.lines("pi bits") == c.lines("pi bits")
    assert g.lines("pi is approximately") == c.lines("pi is approximately")


@pytest.mark.parametrize("lg,iters,ranks", [(8, 2, 40), (12, 1, 1024), (14, 2, 256)])
def test_gpu_coll_bench_matches_oracle(gpu_built, lg, iters, ranks):
    """Batched-collectives program: every result checksum equals the host MPI run."""
    g = gpu_built.run_program("coll_bench", [str(lg), str(iters)], nranks=ranks,
                              extra=GPU_OPTS + ["-p", "4G"], timeout=300)
    c = run_oracle("coll_bench", [str(lg), str(iters)], nranks=ranks, timeout=300)
    assert g.returncode == 0, g.stderr[-2000:]
    assert c.returncode == 0, c.stderr[-2000:]
    assert g.lines("coll_bench checksum") == c.lines("coll_bench checksum")


P2P_CASES = [
    ("pairs", "block", 3, 16, 10, 2, "1G", "world"),
    ("ring", "block", 3, 14, 10, 7, "1G", "world"),
    ("pairs", "nb", 3, 20, 5, 64, "1G", "world"),
    ("ring", "nb", 10, 22, 3, 256, "4G", "world"),
    ("ring", "block", 3, 12, 4, 1024, "1G", "world"),
    ("pairs", "nb", 24, 26, 2, 8, "2G", "world"),
    ("pairs", "block", 3, 20, 6, 4, "1G", "dup"),
    ("ring", "nb", 3, 18, 4, 33, "1G", "dup"),
]


@pytest.mark.parametrize("pattern,mode,lo,hi,iters,ranks,heap,comm", P2P_CASES)
def test_gpu_p2p_sweep_matches_oracle(gpu_built, pattern, mode, lo, hi, iters, ranks, heap, comm):
    """Point-to-point sweep: every payload arrives intact (errors 0) and the
    per-size checksums of the received bytes equal the host MPI run's, on
    MPI_COMM_WORLD and on a duplicate of it."""
    args = [pattern, mode, str(lo), str(hi), str(iters), comm]
    g = gpu_built.run_program("p2p_sweep", args, nranks=ranks, extra=GPU_OPTS + ["-p", heap], timeout=300)
    c = run_oracle("p2p_sweep", args, nranks=ranks, timeout=300)
    assert g.returncode == 0, g.stdout[-2000:] + g.stderr[-2000:]
    assert c.returncode == 0, c.stderr[-2000:]
    got = g.lines("p2p ")
    assert len(got) == hi - lo + 1
    assert all(" errors 0 " in ln for ln in got)
    assert got == c.lines("p2p ")


@pytest.mark.parametrize("args,ranks", [(["23", "10"], 64), (["14", "3"], 7), (["12", "2"], 1),
                                        (["20", "4", "19", "10"], 256), (["10", "2"], 64)])
def test_gpu_is_sort_matches_oracle(gpu_built, args, ranks):
    """IS-like bucket sort: globally sorted, and every per-iteration checksum and
    the sorted-key checksum equal the host MPI run's."""
    g = gpu_built.run_program("is_sort", args, nranks=ranks, extra=GPU_OPTS + ["-p", "2G"], timeout=300)
    c = run_oracle("is_sort", args, nranks=ranks, timeout=300)
    assert g.returncode == 0, g.stdout[-2000:] + g.stderr[-2000:]
    assert c.returncode == 0, c.stderr[-2000:]
    assert g.lines("is verify")[0].endswith("PASSED")
    assert g.lines("is ") == c.lines("is ")


def _pic_values(res):
    out = []
    for ln in res.lines("pic cycle"):
        w = ln.split()
        out.append((int(w[2]), int(w[4]), [float(w[i]) for i in (6, 8, 10, 12)]))
    return out


@pytest.mark.parametrize("args,ranks,heap", [(["10", "64", "32", "20", "5"], 16, "1G"),
                                             (["20", "32", "16", "20", "5"], 4, "1G"),
                                             (["6", "16", "8", "10", "3"], 1, "1G"),
                                             (["50", "256", "128", "125", "10"], 64, "4G")])
def test_gpu_pic_matches_oracle(gpu_built, args, ranks, heap):
    """PIC mini-app: energies within 1e-10 relative of the host MPI run (the
    stated tolerance; the arithmetic is + - * / only, so they agree bit for
    bit) and the same particle count and position checksum."""
    g = gpu_built.run_program("pic", args, nranks=ranks, extra=GPU_OPTS + ["-p", heap], timeout=600)
    c = run_oracle("pic", args, nranks=ranks, timeout=600)
    assert g.returncode == 0, g.stdout[-2000:] + g.stderr[-2000:]
    assert c.returncode == 0, c.stderr[-2000:]
    gv, cv = _pic_values(g), _pic_values(c)
    assert len(gv) == len(cv) > 0
    for (gc, gn, ge), (cc, cn, ce) in zip(gv, cv):
        assert gc == cc and gn == cn
        for a, b in zip(ge, ce):
            assert abs(a - b) <= 1e-10 * abs(b)
    assert g.lines("pic positions") == c.lines("pic positions")
    assert g.lines("pic cycle") == c.lines("pic cycle")


@pytest.mark.parametrize("ranks,heap", [(4, "1G"), (64, "4G"), (1, "64M")])
def test_gpu_allocator_known_answers(gpu_built, ranks, heap):
    """Device malloc: sizes 1 B .. 4 MiB aligned and disjoint, reuse after free,
    calloc zeros, realloc keeps the prefix.  With one rank and a 64 MiB heap
    the growing large blocks fit only if freed runs are merged."""
    g = gpu_built.run_program("kat_malloc", [], nranks=ranks, extra=GPU_OPTS + ["-p", heap], timeout=300)
    assert g.returncode == 0, g.stdout[-2000:] + g.stderr[-2000:]
    assert sorted(g.lines("kat_malloc")) == sorted(f"kat_malloc rank {r} ok" for r in range(ranks))


def _cpi_golden():
    import os
    rows = []
    for ln in open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "cpi_pi.txt")):
        if ln.startswith("#") or not ln.strip():
            continue
        key, line = ln.rstrip("\n").split(" | ")
        n, ranks = map(int, key.split())
        rows.append((n, ranks, line))
    return rows


@pytest.mark.parametrize("n,ranks,line", _cpi_golden())
def test_gpu_pi_matches_reference_program(gpu_built, n, ranks, line):
    """GPU run of the converted pi program prints exactly the result line of
    the reference's cpi.c on a host MPI (committed golden fixture)."""
    g = gpu_built.run_program("pi", [str(n)], nranks=ranks, extra=GPU_OPTS, timeout=180)
    assert g.returncode == 0, g.stderr
    assert g.lines("pi is approximately") == [line]


# ---------------------------------------------------------------- ranks as clusters of thread blocks

CLUSTER_KAT = [c for c in KAT_CASES if c[0] in ("kat_p2p", "kat_coll")]


@pytest.mark.parametrize("blocks", [2, 4])
@pytest.mark.parametrize("prog,scenario,nranks", CLUSTER_KAT)
def test_gpu_known_answers_with_cluster_ranks(gpu_built, prog, scenario, nranks, blocks):
    """Every known-answer scenario with each rank launched as a cluster of
    2 or 4 thread blocks (the helper blocks take shares of parallel loops)."""
    args = [scenario] if scenario else []
    res = gpu_built.run_program(prog, args, nranks=nranks, extra=GPU_OPTS + ["--blocks-per-rank", str(blocks)],
                                timeout=180)
    check_all_ok(res, scenario, nranks)


@pytest.mark.parametrize("blocks", [1, 2, 4, 8])
def test_gpu_parallel_loop_spans_the_cluster(gpu_built, blocks):
    """A parallel loop of a rank made of `blocks` thread blocks runs every
    iteration exactly once and runs iterations on all of the blocks."""
    res = gpu_built.run_program("kat_coll", ["parfor"], nranks=4,
                                extra=GPU_OPTS + ["--blocks-per-rank", str(blocks)], timeout=180)
    check_all_ok(res, "parfor", 4)
    got = sorted(ln for ln in res.lines("parfor rank") if " blocks " in ln)
    assert got == [f"parfor rank {r} blocks {blocks}" for r in range(4)]


def test_gpu_cluster_ranks_reject_bad_sizes(gpu_built):
    res = gpu_built.run_program("kat_coll", ["parfor"], nranks=2, extra=GPU_OPTS + ["--blocks-per-rank", "3"],
                                timeout=60)
    assert res.returncode != 0
    assert "blocks-per-rank" in res.stderr


@pytest.mark.parametrize("prog,args,ranks,heap,blocks", [
    ("pic", ["10", "64", "32", "20", "5"], 16, "1G", 2),
    ("pic", ["50", "256", "128", "125", "10"], 64, "4G", 2),
    ("is_sort", ["23", "10"], 64, "2G", 2),
    ("is_sort", ["14", "3"], 7, "1G", 4),
])
def test_gpu_apps_with_cluster_ranks_match_oracle(gpu_built, prog, args, ranks, heap, blocks):
    """PIC and the IS-like sort with every rank a cluster of thread blocks:
    the printed results (energies, checksums) equal the host MPI run's."""
    g = gpu_built.run_program(prog, args, nranks=ranks,
                              extra=GPU_OPTS + ["-p", heap, "--blocks-per-rank", str(blocks)], timeout=600)
    c = run_oracle(prog, args, nranks=ranks, timeout=600)
    assert g.returncode == 0, g.stdout[-2000:] + g.stderr[-2000:]
    assert c.returncode == 0, c.stderr[-2000:]
    key = "pic " if prog == "pic" else "is "
    strip = lambda lines: [ln for ln in lines if "-time" not in ln]
    assert strip(g.lines(key)) == strip(c.lines(key))


# ---------------------------------------------------------------- one-cluster jobs (mailboxes in shared memory)

ONE_CLUSTER_KAT = [c for c in KAT_CASES if c[0] in ("kat_p2p", "kat_coll") and c[2] <= 16]


@pytest.mark.parametrize("prog,scenario,nranks", ONE_CLUSTER_KAT)
def test_gpu_known_answers_in_one_cluster(gpu_built, prog, scenario, nranks):
    """Every known-answer scenario of at most 16 ranks with the whole job in
    one thread-block cluster: each rank's mailbox lives in its block's shared
    memory and senders write headers and small payloads through distributed
    shared memory."""
    args = [scenario] if scenario else []
    res = gpu_built.run_program(prog, args, nranks=nranks, extra=GPU_OPTS + ["--one-cluster"], timeout=180)
    check_all_ok(res, scenario, nranks)


@pytest.mark.parametrize("pattern,mode,lo,hi,iters,ranks,comm", [
    ("pairs", "block", 3, 16, 10, 2, "world"),
    ("pairs", "nb", 3, 20, 5, 8, "world"),
    ("ring", "block", 3, 14, 10, 7, "dup"),
    ("ring", "nb", 3, 12, 4, 16, "world"),
])
def test_gpu_p2p_sweep_in_one_cluster_matches_oracle(gpu_built, pattern, mode, lo, hi, iters, ranks, comm):
    """The point-to-point sweep with the job in one cluster: every payload
    intact and every checksum equal to the host MPI run's."""
    args = [pattern, mode, str(lo), str(hi), str(iters), comm]
    g = gpu_built.run_program("p2p_sweep", args, nranks=ranks, extra=GPU_OPTS + ["--one-cluster"], timeout=300)
    c = run_oracle("p2p_sweep", args, nranks=ranks, timeout=300)
    assert g.returncode == 0, g.stdout[-2000:] + g.stderr[-2000:]
    got = g.lines("p2p ")
    assert len(got) == hi - lo + 1 and all(" errors 0 " in ln for ln in got)
    assert got == c.lines("p2p ")


def test_gpu_pi_in_one_cluster_bit_exact(gpu_built):
    g = gpu_built.run_program("pi", ["10000000"], nranks=8, extra=GPU_OPTS + ["--one-cluster"], timeout=180)
    c = run_oracle("pi", ["10000000"], nranks=8, timeout=180)
    assert g.returncode == 0, g.stderr
    assert g.lines("pi bits") == c.lines("pi bits")


def test_gpu_one_cluster_rejects_too_many_ranks(gpu_built):
    res = gpu_built.run_program("pi", ["1000"], nranks=17, extra=GPU_OPTS + ["--one-cluster"], timeout=60)
    assert res.returncode != 0
    assert "one-cluster" in res.stderr


@pytest.mark.parametrize("runs,blocks", [(64, 1), (4096, 1), (4096, 4)])
def test_gpu_pi_parallel_runs_bit_exact(gpu_built, runs, blocks):
    """pi with each rank's intervals summed as `runs` consecutive runs in a
    parallel loop and the run sums added in order: the GPU (one or several
    blocks per rank) and the host MPI build print the same bits."""
    args = ["10000000", str(runs)]
    g = gpu_built.run_program("pi", args, nranks=8, extra=GPU_OPTS + ["--blocks-per-rank", str(blocks)], timeout=180)
    c = run_oracle("pi", args, nranks=8, timeout=180)
    assert g.returncode == 0, g.stderr
    assert g.lines("pi bits") == c.lines("pi bits")
    assert g.lines("pi is approximately") == c.lines("pi is approximately")
