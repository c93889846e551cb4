"""Serving: PIC jobs of 16, 32 and 64 ranks admitted by HBM footprint.

Each job's output in the mix must equal its output when it runs alone; the
jobs run as concurrent kernels in disjoint rank-slot ranges.  With a pool that
holds one job at a time they must run one after another and still give the
same results.
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
    for i in range(3):
        for j in range(i + 1, 3):
            overlap_t = times[i][1] < times[j][2] and times[j][1] < times[i][2]
            overlap_s = ranges[i][0] < ranges[j][1] and ranges[j][0] < ranges[i][1]
            assert not (overlap_t and overlap_s)


def test_small_pool_runs_jobs_one_at_a_time(gpu_built, tmp_path):
    ref = {k: strip_time(alone(gpu_built, n)) for k, n in enumerate(SIZES)}
    per_job, times = serve(gpu_built, tmp_path, ["-p", "512M", "--pool", "700M"])
    for k in range(len(SIZES)):
        assert strip_time(per_job[k]) == ref[k]
    spans = sorted((times[k][1], times[k][2]) for k in range(3))
    for a, b in zip(spans, spans[1:]):
        assert b[0] >= a[1] - 1e-3
