"""Failure detection on the GPU without a GPU fault.

One rank of a job fails on purpose, in ways the host can see: a receive that
nobody serves (its wait runs out after --timeout-ms), exit() with a nonzero
status, MPI_Abort, a failed assert.  Every other rank must leave its wait
with an error code, the kernel must end by itself long before the launcher's
wall-clock limit, and the process must report the failure in its exit status
and on stderr.  Nothing here traps, faults or hangs the GPU: every device wait
is bounded by the job's timeout and polls the job's abort flag.
"""
import re
import time

import pytest

pytestmark = pytest.mark.gpu

ERR_TIMEOUT = 50
ERR_ABORTED = 51
OPTS = ["--timeout-ms", "400", "--max-seconds", "60"]


def run(host, scenario, ranks=4):
    t0 = time.time()
    res = host.run_program("kat_fail", [scenario], nranks=ranks, extra=OPTS, timeout=120)
    return res, time.time() - t0


def codes(res, what):
    out = {}
    for ln in res.stdout.splitlines():
        m = re.match(rf"rank (\d+) {what} rc (-?\d+)", ln)
        if m:
            out[int(m.group(1))] = int(m.group(2))
    return out


def test_control_run_succeeds(gpu_built):
    res, secs = run(gpu_built, "ok")
    assert res.returncode == 0, res.stderr
    assert codes(res, "barrier") == {r: 0 for r in range(4)}


def test_receive_nobody_serves_times_out(gpu_built):
    res, secs = run(gpu_built, "recv_timeout")
    assert res.returncode != 0
    assert codes(res, "recv") == {0: ERR_TIMEOUT}
    assert codes(res, "barrier") == {1: ERR_ABORTED, 2: ERR_ABORTED, 3: ERR_ABORTED}
    assert "timed out" in res.stderr
    assert secs < 30


def test_exit_of_one_rank_aborts_the_others(gpu_built):
    res, secs = run(gpu_built, "exit_rank")
    assert res.returncode != 0
    assert codes(res, "barrier") == {0: ERR_ABORTED, 2: ERR_ABORTED, 3: ERR_ABORTED}
    assert "exit()" in res.stderr
    assert secs < 30


def test_mpi_abort_ends_pending_receives(gpu_built):
    res, secs = run(gpu_built, "abort_rank")
    assert res.returncode != 0
    assert codes(res, "recv") == {0: ERR_ABORTED, 1: ERR_ABORTED, 3: ERR_ABORTED}
    assert "MPI_Abort" in res.stderr
    assert secs < 30


def test_failed_assert_reports_and_aborts(gpu_built):
    res, secs = run(gpu_built, "assert_rank")
    assert res.returncode != 0
    assert codes(res, "barrier") == {1: ERR_ABORTED, 2: ERR_ABORTED, 3: ERR_ABORTED}
    assert "size < 0" in res.stdout + res.stderr
    assert secs < 30


def test_gpu_usable_after_failures(gpu_built):
    """A failed job leaves the device usable: the next job runs normally."""
    run(gpu_built, "recv_timeout")
    res, _ = run(gpu_built, "ok", ranks=64)
    assert res.returncode == 0, res.stderr
    assert len(codes(res, "barrier")) == 64
