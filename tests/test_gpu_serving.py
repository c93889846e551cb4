"""Serving: PIC jobs of 16, 32 and 64 ranks admitted by HBM footprint into one
persistent launch (worker blocks as rank slots, an admin block, a pinned
admission and completion ring).

Each job's output in the mix must equal its output when it runs alone, and
jobs that run at the same time use disjoint rank slots; in the mix at least
two jobs must actually overlap in time.  With a pool that holds one job at a
time they must run one after another and still give the same results.  Jobs
submitted online (standard input, one line per job) while another job runs
are admitted and run next to it.
"""
import os
import re

import pytest

pytestmark = pytest.mark.gpu

PIC_ARGS = ["12", "128", "64", "40", "4"]
SIZES = [16, 32, 64]


def alone(host, n):
    res = host.run_program("pic", PIC_ARGS, nranks=n, extra=["-t", "128", "--max-seconds", "300"], timeout=400)
    assert res.returncode == 0, res.stderr[-2000:]
    return [ln for ln in res.stdout.splitlines() if ln.startswith("pic ")]


def serve(host, tmp_path, extra):
    jobfile = tmp_path / "jobs.txt"
    jobfile.write_text("".join(f"{n} 0 {' '.join(PIC_ARGS)}\n" for n in SIZES))
    exe = os.path.join(host.BIN, "pic")
    import subprocess
    r = subprocess.run([exe, "---gpumpi", "--serve", str(jobfile), "-t", "128", "--max-seconds", "300", *extra],
                       capture_output=True, text=True, timeout=400)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    per_job = {k: [] for k in range(len(SIZES))}
    times = {}
    for ln in r.stdout.splitlines():
        m = re.match(r"\[job (\d+)\] (pic .*)", ln)
        if m:
            per_job[int(m.group(1))].append(m.group(2))
        m = re.match(r"serve job (\d+) ranks (\d+) exit (\d+) slots (-?\d+) .* start ([0-9.]+) end ([0-9.]+)", ln)
        if m:
            times[int(m.group(1))] = (int(m.group(4)), float(m.group(5)), float(m.group(6)))
    assert "serve summary jobs 3" in r.stdout
    return per_job, times


def strip_time(lines):
    return [ln for ln in lines if not ln.startswith("pic-time")]


def test_mix_equals_alone(gpu_built, tmp_path):
    ref = {k: strip_time(alone(gpu_built, n)) for k, n in enumerate(SIZES)}
    per_job, times = serve(gpu_built, tmp_path, ["-p", "512M"])
    for k in range(len(SIZES)):
        assert strip_time(per_job[k]) == ref[k]
    # disjoint slot ranges for jobs that ran at the same time
    ranges = [(times[k][0], times[k][0] + SIZES[k]) for k in range(len(SIZES))]
    overlaps = 0
    for i in range(3):
        for j in range(i + 1, 3):
            overlap_t = times[i][1] < times[j][2] and times[j][1] < times[i][2]
            overlap_s = ranges[i][0] < ranges[j][1] and ranges[j][0] < ranges[i][1]
            assert not (overlap_t and overlap_s)
            overlaps += overlap_t
    # the three jobs fit the GPU together: they ran side by side
    assert overlaps >= 1


def test_small_pool_runs_jobs_one_at_a_time(gpu_built, tmp_path):
    ref = {k: strip_time(alone(gpu_built, n)) for k, n in enumerate(SIZES)}
    per_job, times = serve(gpu_built, tmp_path, ["-p", "512M", "--pool", "700M"])
    for k in range(len(SIZES)):
        assert strip_time(per_job[k]) == ref[k]
    spans = sorted((times[k][1], times[k][2]) for k in range(3))
    for a, b in zip(spans, spans[1:]):
        assert b[0] >= a[1] - 1e-3


LONG_ARGS = ["150", "256", "128", "60", "50"]


def test_online_submissions_run_beside_a_running_job(gpu_built):
    """Jobs arrive on standard input while a long job runs: they are admitted
    at once, run next to it (their [start, end] lies inside the long job's)
    and give the same output as alone."""
    import subprocess
    import time

    long_ref = strip_time(_alone_args(gpu_built, 16, LONG_ARGS))
    ref = {n: strip_time(alone(gpu_built, n)) for n in (32, 64)}
    exe = os.path.join(gpu_built.BIN, "pic")
    p = subprocess.Popen([exe, "---gpumpi", "--serve", "-", "-t", "128", "-p", "512M", "--max-seconds", "300"],
                         stdin=subprocess.PIPE, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    p.stdin.write(f"16 0 {' '.join(LONG_ARGS)}\n")
    p.stdin.flush()
    time.sleep(1.5)
    p.stdin.write(f"32 0 {' '.join(PIC_ARGS)}\n64 0 {' '.join(PIC_ARGS)}\n")
    p.stdin.flush()
    out, err = p.communicate(timeout=400)   # closes standard input: no more jobs
    assert p.returncode == 0, out[-3000:] + err[-3000:]
    per_job = {k: [] for k in range(3)}
    times = {}
    for ln in out.splitlines():
        m = re.match(r"\[job (\d+)\] (pic .*)", ln)
        if m:
            per_job[int(m.group(1))].append(m.group(2))
        m = re.match(r"serve job (\d+) ranks (\d+) exit (\d+) slots (-?\d+) .* submit ([0-9.]+) start ([0-9.]+) "
                     r"end ([0-9.]+)", ln)
        if m:
            times[int(m.group(1))] = (float(m.group(5)), float(m.group(6)), float(m.group(7)))
    assert sorted(times) == [0, 1, 2]
    assert strip_time(per_job[0]) == long_ref
    assert strip_time(per_job[1]) == ref[32]
    assert strip_time(per_job[2]) == ref[64]
    s0, b0, e0 = times[0]
    for k in (1, 2):
        sk, bk, ek = times[k]
        assert sk > b0 + 1.0          # arrived while job 0 ran
        assert bk < e0 and ek < e0    # admitted and finished while job 0 still ran
    assert "serve summary jobs 3" in out


def _alone_args(host, n, args):
    res = host.run_program("pic", args, nranks=n, extra=["-t", "128", "--max-seconds", "300"], timeout=400)
    assert res.returncode == 0, res.stderr[-2000:]
    return [ln for ln in res.stdout.splitlines() if ln.startswith("pic ")]
