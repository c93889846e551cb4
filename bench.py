#!/usr/bin/env python3
"""Benchmark: batched collectives of the device MPI runtime on one GB300.

Workload (the batched-collectives configuration): 16 communicators of
4, 8, 12, 16, 24, 32, 40, 48, 56, 64, 72, 80, 88, 96, 128 and 256 ranks
(1024 rank blocks), each running Bcast, Allreduce(SUM) and Alltoall on int32
data uniform in [-2^20, 2^20) and FP64 data uniform in [-1, 1), 2^20
elements per rank (Alltoall: 2^20 / P elements to each peer).

One step = all 96 collective calls.  `value` is algorithmic GB/s of the
batched form (one persistent cooperative launch, replayed as a CUDA graph),
with the inputs resident in HBM; algorithmic bytes per call: Bcast P*b,
Allreduce 2*P*n*s, Alltoall 2*P^2*m.  The plain form (one launch per call and
communicator) runs the same schedules on the same buffers for comparison.
`e2e` times the host-buffer entry point (host->device copies of every send
buffer, the batched plan, device->host copies of every result) on a smaller
per-rank count stated in the line.  `cpu_baseline` / `--impl reference` run
the same collectives as an MPI program on the host cores through the hostmpi
oracle (one process per rank).
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "dphpc-project_gb300")
sys.path.insert(0, PKG)

COMM_SIZES = [4, 8, 12, 16, 24, 32, 40, 48, 56, 64, 72, 80, 88, 96, 128, 256]
# the same communicators in 4 groups of 256 rank blocks (end-to-end pipelining;
# 4 groups measured faster than 7)
E2E_GROUPS = [[256], [128, 88, 40], [96, 80, 56, 24], [72, 64, 48, 32, 16, 12, 8, 4]]
WORKLOAD = ("batched collectives: 16 communicators (4..256 ranks, 1024 rank blocks), "
            "Bcast + Allreduce(SUM) + Alltoall, int32 and fp64")


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    def __init__(self, gpu: int, interval_ms: int = 20):
        self.gpu = gpu
        self.interval_ms = interval_ms
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                 "-lms", str(self.interval_ms)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.time()
            while not self.lines and time.time() - t0 < 5 and self.proc.poll() is None:
                time.sleep(0.01)      # the timed region starts once sampling runs
            self.lines.clear()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx = max(mx, float(f[1]))
            except ValueError:
                continue
            for i, n in enumerate(names):
                if f[4 + i].lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# DRAM bytes (read + write) of one batched launch at 2^16 elements per rank,
# from a one-pass ncu capture of dram__bytes_read.sum + dram__bytes_write.sum
# (profiles/gpumpi_plan_kernel_batched_collectives.md); other per-rank counts
# scale it by their elements per rank.
NCU_TRAFFIC_BYTES_2_16 = 1834974208 + 2673922048


ALL_KINDS = ("bcast", "allreduce", "alltoall")


def a2a_per(n: int, p: int) -> int:
    """Elements each rank sends to each peer in the Alltoall of a rank with n
    elements: n / P (at least 1, so that small counts still move data)."""
    return max(1, n // p)


def alg_bytes(sizes, n, kinds=ALL_KINDS):
    total = 0
    for p in sizes:
        for s in (4, 8):
            if "bcast" in kinds:
                total += p * n * s              # Bcast
            if "allreduce" in kinds:
                total += 2 * p * n * s          # Allreduce
            per = a2a_per(n, p)
            if "alltoall" in kinds:
                total += 2 * p * p * per * s    # Alltoall
    return total


def max_over_ranks(dist, torch, secs: float) -> float:
    """Replicas: the job's time is the slowest rank's (gloo all-reduce MAX)."""
    if dist is None:
        return secs
    t = torch.tensor([secs], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Item:
    """One collective call of the workload: its communicator size, type and
    device buffers (send: the input of rank 0..P-1 back to back, recv: the
    outputs; Bcast works in place on `recv`)."""

    def __init__(self, kind, p, dt, count, send, recv):
        self.kind, self.p, self.dt, self.count, self.send, self.recv = kind, p, dt, count, send, recv


def fill_random(torch, t, dt, g):
    if dt == "int32":
        t.random_(-(1 << 20), 1 << 20, generator=g)
    else:
        t.uniform_(-1.0, 1.0, generator=g)


def build_plan(coll, lib, torch, sizes, n, batched, threads, seed=1, kinds=ALL_KINDS):
    """Device buffers and descriptors of the collectives named in kinds, one
    Item per descriptor (same order)."""
    g = torch.Generator(device="cuda").manual_seed(seed)
    dev = torch.device("cuda")
    comms, keep, descs, items = [], [], [], []
    for p in sizes:
        c = coll.Comm(lib, p)
        comms.append(c)
        per = a2a_per(n, p)
        for dt, tdt in (("int32", torch.int32), ("float64", torch.float64)):
            es = 4 if dt == "int32" else 8

            def rnd(count):
                t = torch.empty(count, dtype=tdt, device=dev)
                fill_random(torch, t, dt, g)
                return t

            ptr = lambda t, stride: [t.data_ptr() + r * stride * es for r in range(p)]
            if "bcast" in kinds:
                bc = rnd(p * n)
                items.append(Item("bcast", p, dt, n, None, bc))
                descs.append(coll.make_desc(c, coll.COLL_BCAST, dt, n, None, ptr(bc, n), 0, 0, keep))
            if "allreduce" in kinds:
                ar_in, ar_out = rnd(p * n), torch.empty(p * n, dtype=tdt, device=dev)
                items.append(Item("allreduce", p, dt, n, ar_in, ar_out))
                descs.append(coll.make_desc(c, coll.COLL_ALLREDUCE, dt, n, ptr(ar_in, n), ptr(ar_out, n),
                                            coll.OP_SUM, 0, keep))
            if "alltoall" in kinds:
                a2_in, a2_out = rnd(p * per * p), torch.empty(p * per * p, dtype=tdt, device=dev)
                items.append(Item("alltoall", p, dt, per, a2_in, a2_out))
                descs.append(coll.make_desc(c, coll.COLL_ALLTOALL, dt, per, ptr(a2_in, per * p),
                                            ptr(a2_out, per * p), 0, 0, keep))
    plan = coll.Plan(lib, descs, threads=threads, batched=batched)
    return plan, comms, keep, items, descs


def _bits(torch, t):
    return t.view(torch.int64) if t.dtype == torch.float64 else t


def verify_items(torch, items, sample: int | None = None, seed: int = 5) -> list[str]:
    """Check every call's result against its inputs, bit for bit.

    Bcast: every rank's buffer equals the root's (rank 0).  Alltoall: block q
    of rank r's output equals block r of rank q's input.  Allreduce(SUM): the
    output of every rank equals the rank-order fold acc = x_0; acc = x_q + acc
    (q = 1..P-1) computed with NumPy on the host, the order of the reference's
    MPI_Reduce (gpu_libs/gpu_mpi/mpi.cu:209-225); with `sample`, at that many
    random element positions plus the first and last element of every rank's
    segment, else at every element.  Returns the mismatches found."""
    import numpy as np

    bad = []
    rng = np.random.default_rng(seed)
    for k, it in enumerate(items):
        p, n = it.p, it.count
        if it.kind == "bcast":
            m = _bits(torch, it.recv).view(p, n)
            if not bool((m == m[0:1]).all()):
                bad.append(f"item {k}: bcast P={p} {it.dt}")
        elif it.kind == "alltoall":
            per = n
            src = _bits(torch, it.send).view(p, p, per)
            dst = _bits(torch, it.recv).view(p, p, per)
            if not torch.equal(dst, src.transpose(0, 1)):
                bad.append(f"item {k}: alltoall P={p} {it.dt}")
        elif it.kind == "allreduce":
            x = it.send.view(p, n)
            y = it.recv.view(p, n)
            if sample is not None and sample < n:
                seg = -(-n // p)
                edges = [i for r in range(p) for i in (r * seg, min(n, (r + 1) * seg) - 1) if 0 <= i < n]
                idx = np.unique(np.concatenate([rng.integers(0, n, sample), np.array(edges, dtype=np.int64)]))
                ti = torch.from_numpy(idx).to(x.device)
                xs = x.index_select(1, ti).cpu().numpy()
                ys = y.index_select(1, ti).cpu().numpy()
            else:
                xs = x.cpu().numpy()
                ys = y.cpu().numpy()
            acc = xs[0].copy()
            for q in range(1, p):
                acc = xs[q] + acc
            u = np.uint64 if acc.dtype.itemsize == 8 else np.uint32
            if not bool((ys.view(u) == acc.view(u)[None, :]).all()):
                bad.append(f"item {k}: allreduce P={p} {it.dt}")
    return bad


def time_plan(torch, plan, steps, warmup, stream):
    for _ in range(warmup):
        plan.launch(stream.cuda_stream)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        plan.launch(stream.cuda_stream)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1000.0


def sweep_point(coll, lib, torch, lg: int, stream, peak: float, tune_reps: int, target_s: float = 0.05,
                sync_mode: int = 0):
    """The workload at 2^lg elements per rank: tuned batched plan (CUDA graph)
    against the tuned plain form, results checked after timing."""
    n = 1 << lg
    plan, comms, keep, items, descs = build_plan(coll, lib, torch, COMM_SIZES, n, True, 128, seed=40 + lg)
    plan.close()
    threads, pth, palg = coll.autotune(lib, descs, reps=tune_reps)
    plan = coll.Plan(lib, descs, threads=threads, batched=True)
    g = torch.Generator(device="cuda").manual_seed(60 + lg)
    for it in items:
        fill_random(torch, it.send if it.send is not None else it.recv, it.dt, g)
    if sync_mode:
        plan.set_sync(sync_mode)
    plan.capture(stream.cuda_stream)
    t1 = time_plan(torch, plan, 3, 3, stream) / 3
    steps = int(min(2000, max(10, target_s / max(t1, 1e-7))))
    secs = time_plan(torch, plan, steps, 0, stream)
    bad = verify_items(torch, items, sample=1024)
    if bad or coll.status(lib):
        raise SystemExit(f"sweep 2^{lg}: result mismatch or device error: {bad[:4]}")
    ordered = plan.launch_ordered
    plan.close()
    pdescs = [type(d).from_buffer_copy(d) for d in descs]
    for d, a in zip(pdescs, palg):
        d.algo = a
        d.sync = 0
    plain = coll.Plan(lib, pdescs, threads=threads, batched=False, plain_threads=pth)
    if sync_mode:
        plain.set_sync(sync_mode)
    p1 = time_plan(torch, plain, 1, 1, stream)
    psteps = int(min(200, max(3, target_s / max(p1, 1e-7))))
    psecs = time_plan(torch, plain, psteps, 0, stream)
    plain.close()
    for c in comms:
        c.close()
    nbytes = alg_bytes(COMM_SIZES, n)
    per_step = secs / steps
    gbs = nbytes / per_step / 1e9
    pgbs = nbytes * psteps / psecs / 1e9
    del items
    torch.cuda.empty_cache()
    return {"elements_per_rank": n, "value": round(gbs, 2), "unit": "GB/s", "frac": round(gbs / peak, 4),
            "us_per_step": round(per_step * 1e6, 2), "steps": steps, "threads_per_rank": threads,
            "launch_ordered": bool(ordered), "flag_rounds_calls": sum(1 for d in descs if d.sync),
            "tuned_plain_value": round(pgbs, 2),
            "batched_over_tuned_plain": round(gbs / pgbs, 2), "verified": True,
            "l2_resident": nbytes < 120e6}


# Application runs (extra key `apps`): the programs of the other benchmark
# configurations, on the GPU and on the host cores through hostmpi in the same
# run.  (name, program, arguments, ranks, GPU launcher options, time pattern)
APPS = [
    ("pi_1e7_8ranks", "pi", ["10000000"], 8, [], r"wall clock time = ([0-9.]+)"),
    ("pi_1e7_8ranks_parallel_runs_4_blocks_per_rank", "pi", ["10000000", "4096"], 8, ["--blocks-per-rank", "4"],
     r"wall clock time = ([0-9.]+)"),
    ("p2p_pair_8B_blocking", "p2p_sweep", ["pairs", "block", "3", "3", "2000"], 2, [],
     r"p2p-time bytes \d+ seconds ([0-9.]+)"),
    ("p2p_pair_8B_blocking_one_cluster", "p2p_sweep", ["pairs", "block", "3", "3", "2000"], 2, ["--one-cluster"],
     r"p2p-time bytes \d+ seconds ([0-9.]+)"),
    ("p2p_pair_1MiB_nonblocking", "p2p_sweep", ["pairs", "nb", "20", "20", "200"], 2, [],
     r"p2p-time bytes \d+ seconds ([0-9.]+)"),
    ("p2p_pair_64MiB_nonblocking", "p2p_sweep", ["pairs", "nb", "26", "26", "10"], 2, ["-p", "2G"],
     r"p2p-time bytes \d+ seconds ([0-9.]+)"),
    ("p2p_ring_1024ranks_1MiB", "p2p_sweep", ["ring", "nb", "20", "20", "10"], 1024, ["-p", "8G"],
     r"p2p-time bytes \d+ seconds ([0-9.]+)"),
    ("is_like_sort_2e23_64ranks", "is_sort", ["23", "10"], 64, ["-p", "2G"], r"is-time seconds ([0-9.]+)"),
    ("pic_64ranks_50cycles", "pic", ["50"], 64, ["-p", "4G"], r"pic-time seconds ([0-9.]+)"),
    ("pic_64ranks_50cycles_2_blocks_per_rank", "pic", ["50"], 64, ["-p", "4G", "--blocks-per-rank", "2"],
     r"pic-time seconds ([0-9.]+)"),
    ("pic_64ranks_50cycles_4_blocks_per_rank", "pic", ["50"], 64, ["-p", "4G", "--blocks-per-rank", "4"],
     r"pic-time seconds ([0-9.]+)"),
    ("is_like_sort_2e23_64ranks_2_blocks_per_rank", "is_sort", ["23", "10"], 64, ["-p", "2G", "--blocks-per-rank", "2"],
     r"is-time seconds ([0-9.]+)"),
]
TIME_LINE = re.compile(r"^(wall clock time|p2p-time|is-time|pic-time)")


def _pic_rel(a: list[str], b: list[str]) -> float:
    """Largest relative difference of the energies printed by two PIC runs."""
    worst = 0.0
    for x, y in zip(a, b):
        fx, fy = x.split(), y.split()
        for u, v in zip(fx, fy):
            try:
                fu, fv = float(u), float(v)
            except ValueError:
                continue
            if "e" in u or "." in u:
                worst = max(worst, abs(fu - fv) / max(abs(fv), 1e-300))
    return worst


def app_runs(host, timeout: float = 600.0) -> dict:
    """Each program once on the GPU and once on hostmpi; wall times of the
    programs' own timed regions (MPI_Wtime brackets, slowest rank) and whether
    the results agree (every printed result line, timing lines aside)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("hostmpi_run", os.path.join(ROOT, "oracle", "hostmpi_run.py"))
    oracle = importlib.util.module_from_spec(spec)
    sys.modules[spec.name] = oracle
    spec.loader.exec_module(oracle)
    out = {}
    for name, prog, pargs, ranks, extra, pat in APPS:
        rec = {"ranks": ranks, "args": " ".join(pargs)}
        try:
            g = host.run_program(prog, pargs, nranks=ranks, extra=["--timeout-ms", "60000", *extra], timeout=timeout)
            c = oracle.run_oracle(prog, pargs, nranks=ranks, timeout=timeout)
            mg, mc = re.search(pat, g.stdout), re.search(pat, c.stdout)
            if g.returncode or not mg:
                raise RuntimeError(f"GPU run failed: {g.stderr[-300:]}")
            if c.returncode or not mc:
                raise RuntimeError(f"hostmpi run failed: {c.stderr[-300:]}")
            rg = [ln for ln in g.stdout.splitlines() if ln.strip() and not TIME_LINE.match(ln)]
            rc = [ln for ln in c.stdout.splitlines() if ln.strip() and not TIME_LINE.match(ln)]
            gs, cs = float(mg.group(1)), float(mc.group(1))
            rec.update({"gpu_s": gs, "hostmpi_s": cs, "hostmpi_cores": os.cpu_count(),
                        "hostmpi_over_gpu": round(cs / gs, 2) if gs > 0 else None})
            if prog == "p2p_sweep":
                iters = int(pargs[4])
                rec["gpu_us_per_iter"] = round(1e6 * gs / iters, 3)
                rec["hostmpi_us_per_iter"] = round(1e6 * cs / iters, 3)
                mb = re.search(r"GBps ([0-9.]+)", g.stdout)
                rec["gpu_GBps"] = float(mb.group(1)) if mb else None
            if rg == rc:
                rec["parity"] = "result lines identical"
            elif prog == "pic" and len(rg) == len(rc):
                rel = _pic_rel(rg, rc)
                rec["parity"] = f"energies within {rel:.2e} relative"
                if rel > 1e-10:
                    raise RuntimeError(f"PIC energies differ by {rel:.3e} relative")
            else:
                raise RuntimeError("results differ from hostmpi: " + str([x for x in rg if x not in rc][:3]))
        except Exception as e:  # reported in the line, and the run fails below
            rec["error"] = str(e)[:400]
        out[name] = rec
    return out


def serving_run(host, timeout: float = 600.0) -> dict:
    """The PIC configuration served: 9 jobs of 16, 32 and 64 ranks (full
    grid, 50 cycles) arriving every 200 ms on one server; makespan and the
    50th/99th percentile of job latency (arrival to end) from the server's
    own report, and each job's exit status."""
    import tempfile
    lines = [f"{n} {200 * k} 50 256 128 125 10\n" for k, n in enumerate([16, 32, 64] * 3)]
    with tempfile.NamedTemporaryFile("w", suffix=".jobs", delete=False) as f:
        f.writelines(lines)
        path = f.name
    try:
        exe = os.path.join(host.BIN, "pic")
        r = subprocess.run([exe, "---gpumpi", "--serve", path, "-t", "128", "-p", "2G", "--max-seconds", "300"],
                           capture_output=True, text=True, timeout=timeout)
    finally:
        os.unlink(path)
    m = re.search(r"serve summary jobs (\d+) makespan ([0-9.]+) latency_p50 ([0-9.]+) latency_p99 ([0-9.]+)",
                  r.stdout)
    exits = [int(x) for x in re.findall(r"serve job \d+ ranks \d+ exit (\d+)", r.stdout)]
    if r.returncode or not m:
        return {"error": (r.stdout[-300:] + r.stderr[-300:])}
    return {"jobs": int(m.group(1)), "ranks": "16/32/64 x 3", "arrival_ms": 200, "makespan_s": float(m.group(2)),
            "latency_p50_s": float(m.group(3)), "latency_p99_s": float(m.group(4)),
            "all_exit_0": all(e == 0 for e in exits) and len(exits) == 9}


def allocator_runs(host, lib) -> dict:
    """Device malloc: the churn of the point-to-point configuration (every
    thread, log-uniform 16 B - 4 KiB, up to 8 live objects) and the reference
    allocator benchmark's shape (12 x 1024 threads, one 400-byte object each:
    100 floats), on the runtime's slab allocator and on CUDA's device heap
    (the reference's allocator)."""
    out = {}
    st = host.malloc_churn(lib, 1216, 256, 64, live=8, seed=3, heap_bytes=8 << 30)
    out["churn_1216x256_threads"] = {k: st[k] for k in ("allocs", "failed", "corrupt", "ops_per_s",
                                                         "malloc_cycles_p50", "malloc_cycles_p99",
                                                         "malloc_cycles_mean", "free_cycles_mean")}
    for name, cuda in (("reference_shape_12x1024_400B_slab", False), ("reference_shape_12x1024_400B_cuda_heap", True)):
        st = host.malloc_bench(lib, 12, 1024, 400, heap_bytes=1 << 30, cuda_heap=cuda)
        out[name] = {k: st[k] for k in ("allocs", "failed", "corrupt", "malloc_cycles_mean", "malloc_cycles_p50",
                                        "malloc_cycles_p99", "free_cycles_mean", "free_cycles_p99", "seconds")}
    return out


def host_link(torch, nbytes: int = 1 << 30, reps: int = 3) -> dict:
    """Pinned host <-> device copy bandwidth of this machine right now (GB/s):
    the ceiling of the end-to-end leg, whose copies dominate its time."""
    h = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    out = {}
    for name, dst, src in (("h2d", d, h), ("d2h", h, d)):
        dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            dst.copy_(src, non_blocking=True)
        e1.record()
        torch.cuda.synchronize()
        out[name] = round(nbytes * reps / (e0.elapsed_time(e1) / 1000.0) / 1e9, 1)
    del h, d
    return out


def run_oracle_bench(lg: int, iters: int, ranks: int = 1024, timeout: float = 900):
    exe = os.path.join(ROOT, "oracle", "build", "bin", "coll_bench")
    if not os.path.exists(exe):
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), f"-j{os.cpu_count()}"], check=True,
                       capture_output=True)
    r = subprocess.run([exe, str(lg), str(iters), "---gpumpi", "-n", str(ranks)], capture_output=True,
                       text=True, timeout=timeout)
    m = re.search(r"coll_bench time ([0-9.]+) s bytes ([0-9.]+) GBps ([0-9.]+)", r.stdout)
    if r.returncode != 0 or not m:
        raise RuntimeError(f"oracle benchmark failed: {r.stdout[-500:]} {r.stderr[-500:]}")
    return float(m.group(3)), float(m.group(1)), float(m.group(2))


def reference_arm(args):
    """The same collectives through the hostmpi oracle on the host cores.

    One warm-up invocation of W iterations, then one invocation that runs and
    times K iterations (the program's own MPI_Wtime around its loop), so that
    the 1024 processes start twice, not once per step."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    lg = args.cpu_lg
    run_oracle_bench(lg, args.warmup)
    gbps, secs, nbytes = run_oracle_bench(lg, args.steps)
    cores = os.cpu_count()
    sample = (f"1024 host processes (hostmpi), the same 16 communicators and six collectives, "
              f"2^{lg} elements per rank, {args.steps} timed iterations")
    line = {
        "impl": "reference", "metric": "collective GB/s (batched collectives, algorithmic bytes)",
        "value": round(gbps, 3), "unit": "GB/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1000 * secs / max(1, args.steps), 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32+f64",
        "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "elements_per_rank": 1 << lg, "comm_sizes": COMM_SIZES,
                   "l2": "host memory (not applicable)"},
        "cpu_baseline": {"value": round(gbps, 3), "unit": "GB/s", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(gbps, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--lg", type=int, default=20, help="log2 elements per rank")
    ap.add_argument("--threads", type=int, default=128)
    ap.add_argument("--plain-steps", type=int, default=3)
    ap.add_argument("--e2e-lg", type=int, default=16)
    ap.add_argument("--cpu-lg", type=int, default=16)
    ap.add_argument("--cpu-iters", type=int, default=2)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-apps", action="store_true", help="skip the application runs (extra key apps)")
    ap.add_argument("--sustain-s", type=float, default=3.0,
                    help="seconds of extra replays after the timed region (extra key sustained; 0 = none)")
    ap.add_argument("--no-tune", action="store_true", help="built-in schedules, --threads for every launch")
    ap.add_argument("--tune-reps", type=int, default=3)
    ap.add_argument("--sync-mode", type=int, default=0,
                    help="0: launch-ordered forms when the calls are independent; 1: flag rounds (diagnostic)")
    ap.add_argument("--sweep", default="0,4,8,12,15,17",
                    help="log2 elements per rank of the size sweep (extra key; empty = none)")
    ap.add_argument("--verify-sample", type=int, default=4096,
                    help="element positions per Allreduce checked after the timed region")
    ap.add_argument("--kinds", default=",".join(ALL_KINDS),
                    help="collectives of the timed plan (a subset is a diagnostic run, not the workload)")
    ap.add_argument("--profile-launch", action="store_true",
                    help="bracket one batched launch after the warm-up with cudaProfilerStart/Stop "
                         "(for ncu --profile-from-start off)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    if args.impl == "reference":
        reference_arm(args)
        return

    import torch
    import gpumpi_coll as coll
    import gpumpi_host as host

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")   # replicas only: used for the barrier and max-over-ranks

    lib = coll.bind(host.load_library())
    n = 1 << args.lg
    stream = torch.cuda.Stream()
    peak, peak_kind = load_peaks()

    # batched form, graph-captured; schedules and thread counts from the autotuner
    # (it times candidates on these buffers before the timed region)
    kinds = tuple(k for k in ALL_KINDS if k in args.kinds.split(","))
    plan, comms, keep, items, descs = build_plan(coll, lib, torch, COMM_SIZES, n, True, args.threads, kinds=kinds)
    tuning = None
    plain_threads = plain_algos = None
    threads = args.threads
    if not args.no_tune:
        plan.close()
        t0 = time.perf_counter()
        threads, plain_threads, plain_algos = coll.autotune(lib, descs, reps=args.tune_reps)
        tune_s = time.perf_counter() - t0
        names = {coll.COLL_BCAST: "bcast", coll.COLL_ALLREDUCE: "allreduce", coll.COLL_ALLTOALL: "alltoall"}
        algos = {}
        for d in descs:
            algos.setdefault(names[d.op], {}).setdefault(str(d.algo), 0)
            algos[names[d.op]][str(d.algo)] += 1
        tuning = {"batched_threads": threads, "algo_counts": algos, "seconds": round(tune_s, 2),
                  "flag_rounds_calls": sum(1 for d in descs if d.sync),
                  "plain_threads_counts": {str(t): plain_threads.count(t) for t in sorted(set(plain_threads))}}
        plan = coll.Plan(lib, descs, threads=threads, batched=True)
        # the tuner ran the calls on these buffers: give every input (and the
        # broadcast buffers of the non-root ranks) fresh data, so that the
        # results checked after the timed region come from the timed launches
        g = torch.Generator(device="cuda").manual_seed(11)
        for it in items:
            fill_random(torch, it.send if it.send is not None else it.recv, it.dt, g)
    if args.sync_mode:
        plan.set_sync(args.sync_mode)
    plan.capture(stream.cuda_stream)
    launches0 = lib.gpumpi_kernel_launches()
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            plan.launch(stream.cuda_stream)
    torch.cuda.synchronize()
    if args.profile_launch:
        torch.cuda.profiler.start()
        with torch.cuda.stream(stream):
            plan.launch(stream.cuda_stream)
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        secs = time_plan(torch, plan, args.steps, 0, stream)
    launches = lib.gpumpi_kernel_launches() - launches0 - args.warmup - int(args.profile_launch)
    ordered = plan.launch_ordered
    err = coll.status(lib)
    if err:
        raise SystemExit(f"device error during benchmark: {err}")
    secs = max_over_ranks(dist, torch, secs)
    # the same launch replayed for a few seconds more, clocks sampled: the
    # rate holds beyond the short timed region
    sustained = None
    if args.sustain_s > 0:
        ssteps = max(args.steps, int(args.sustain_s * args.steps / max(secs, 1e-9)))
        with ClockSampler(local, interval_ms=100) as sclocks:
            ssecs = time_plan(torch, plan, ssteps, 0, stream)
        sustained = {"value": round(alg_bytes(COMM_SIZES, n, kinds) * ssteps / ssecs / 1e9, 2), "unit": "GB/s",
                     "steps": ssteps, "seconds": round(ssecs, 3), "clocks": sclocks.summary()}
    # outside the timed region: every call's result against its inputs, bit
    # for bit (reductions at sampled element positions of every rank)
    t0 = time.perf_counter()
    bad = verify_items(torch, items, sample=args.verify_sample)
    verify_s = time.perf_counter() - t0
    if bad:
        raise SystemExit("result mismatch after the timed region: " + "; ".join(bad[:8]))
    nbytes = alg_bytes(COMM_SIZES, n, kinds)
    per_step = secs / args.steps
    value = nbytes * args.steps * world / secs / 1e9
    kernel_gbs = nbytes / per_step / 1e9

    # plain form on the same buffers: one launch per call and communicator, first
    # with the batched launch's schedules and threads per rank (the launch
    # structure is the only difference), then with each launch's own tuned
    # schedule and thread count (a small communicator may use 1024 threads per rank)
    plain = coll.Plan(lib, descs, threads=threads, batched=False)
    if args.sync_mode:
        plain.set_sync(args.sync_mode)
    psecs = time_plan(torch, plain, args.plain_steps, 1, stream)
    plain_gbs = nbytes * args.plain_steps / psecs / 1e9
    plain.close()
    plain_tuned_gbs = None
    if plain_threads:
        pdescs = [type(d).from_buffer_copy(d) for d in descs]
        for d, a in zip(pdescs, plain_algos):
            d.algo = a
            d.sync = 0
        plain = coll.Plan(lib, pdescs, threads=threads, batched=False, plain_threads=plain_threads)
        if args.sync_mode:
            plain.set_sync(args.sync_mode)
        psecs = time_plan(torch, plain, args.plain_steps, 1, stream)
        plain_tuned_gbs = nbytes * args.plain_steps / psecs / 1e9
        plain.close()
    plan.close()
    del items
    torch.cuda.empty_cache()

    # end to end through the host-buffer entry point (smaller per-rank count).
    # The 16 communicators are split into 4 plans (E2E_GROUPS), and each
    # plan's copies in, launch and copies out go on a stream of its own:
    # one plan's device-to-host copies then overlap the next plan's host-to-
    # device copies (the host link carries both directions at once).
    ne = 1 << args.e2e_lg
    link = host_link(torch)
    ecomms, eplans, eparts = [], [], []
    for gi, group in enumerate(E2E_GROUPS):
        eplan, gcomms, gkeep, gitems, gdescs = build_plan(coll, lib, torch, group, ne, True, threads, seed=2 + gi)
        ecomms += gcomms
        sizes_by_comm = {c.h.value: c.n for c in gcomms}
        layout = []
        for d in gdescs:
            p = sizes_by_comm[d.comm]
            es = 4 if d.dtype == coll.DT["int32"] else 8
            nin = {coll.COLL_BCAST: d.count, coll.COLL_ALLREDUCE: d.count, coll.COLL_ALLTOALL: d.count * p}[d.op]
            layout += [nin * es] * p
        total = sum(layout)
        hsend = torch.empty(total, dtype=torch.uint8).pin_memory()
        hrecv = torch.empty(total, dtype=torch.uint8).pin_memory()
        hsend.random_(0, 255)
        hs, hr, off = [], [], 0
        for nb in layout:
            hs.append(hsend.data_ptr() + off)
            hr.append(hrecv.data_ptr() + off)
            off += nb
        eplans.append(eplan)
        eparts.append((eplan, hs, hr, torch.cuda.Stream(), (gkeep, gitems, hsend, hrecv)))
    ebytes = alg_bytes(COMM_SIZES, ne)
    # the copy bandwidth of the end-to-end leg's own pinned buffers (host
    # memory placement varies between boxes and runs)
    probe = eparts[0][4][2]
    pd = torch.empty(probe.numel(), dtype=torch.uint8, device="cuda")
    pd.copy_(probe, non_blocking=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    pd.copy_(probe, non_blocking=True)
    torch.cuda.synchronize()
    buf_h2d = probe.numel() / (time.perf_counter() - t0) / 1e9
    del pd

    def e2e_step():
        h2d = d2h = 0
        for eplan, hs, hr, st, _ in eparts:
            bi, bo = eplan.run_host(hs, hr, st.cuda_stream)
            h2d += bi
            d2h += bo
        for _, _, _, st, _ in eparts:
            st.synchronize()
        return h2d, d2h

    for _ in range(2):
        e2e_step()
    torch.cuda.synchronize()
    e_steps = 3
    t0 = time.perf_counter()
    h2d = d2h = 0
    for _ in range(e_steps):
        h2d, d2h = e2e_step()
    esecs = time.perf_counter() - t0
    e2e_gbs = ebytes * e_steps / esecs / 1e9
    # the same plans without the copies: the device share of an end-to-end step
    t0 = time.perf_counter()
    for _ in range(e_steps):
        for eplan, _, _, st, _ in eparts:
            eplan.launch(st.cuda_stream)
        for _, _, _, st, _ in eparts:
            st.synchronize()
    ekern = (time.perf_counter() - t0) / e_steps
    for ep in eplans:
        ep.close()
    del eparts

    # the same workload over the configuration's range of elements per rank
    sweep = []
    for tok in [t for t in args.sweep.split(",") if t.strip()]:
        lg = int(tok)
        if lg == args.lg:
            continue
        sweep.append(sweep_point(coll, lib, torch, lg, stream, peak, tune_reps=1, sync_mode=args.sync_mode))
    if kinds == ALL_KINDS:
        sweep.append({"elements_per_rank": n, "value": round(kernel_gbs, 2), "unit": "GB/s",
                      "frac": round(kernel_gbs / peak, 4), "us_per_step": round(per_step * 1e6, 2),
                      "steps": args.steps, "threads_per_rank": threads, "launch_ordered": bool(ordered),
                      "tuned_plain_value": round(plain_tuned_gbs, 2) if plain_tuned_gbs else None,
                      "batched_over_tuned_plain": round(kernel_gbs / plain_tuned_gbs, 2) if plain_tuned_gbs else None,
                      "verified": True, "l2_resident": False})
    sweep.sort(key=lambda d: d["elements_per_rank"])

    cpu = None
    if rank == 0 and not args.no_cpu:
        try:
            cgbps, csecs, cbytes = run_oracle_bench(args.cpu_lg, args.cpu_iters)
            cpu = {"value": round(cgbps, 3), "unit": "GB/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": (f"hostmpi, 1024 processes, same communicators and collectives, 2^{args.cpu_lg} "
                              f"elements per rank, {args.cpu_iters} iterations ({csecs:.2f} s timed)")}
        except Exception as e:  # reported, not fatal
            cpu = {"value": None, "unit": "GB/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"failed: {e}"}

    apps = None
    allocator = None
    if rank == 0 and not args.no_apps:
        apps = app_runs(host)
        apps["serving_pic_9_jobs"] = serving_run(host)
        allocator = allocator_runs(host, lib)

    if rank == 0:
        line = {
            "metric": "collective GB/s (batched collectives, algorithmic bytes)",
            "value": round(value, 2),
            "unit": "GB/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": round(per_step * 1000, 4),
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "int32+f64",
            "data": "synthetic (seeded uniform int32 [-2^20,2^20), fp64 [-1,1))",
            "config": {"workload": WORKLOAD if kinds == ALL_KINDS else
                       "diagnostic subset of the batched collectives: " + "+".join(kinds),
                       "elements_per_rank": n, "comm_sizes": COMM_SIZES,
                       "threads_per_rank": threads,
                       "form": "batched, CUDA graph replay, " + ("launch-ordered (independent calls, no flag rounds)"
                                                                  if ordered else "flag rounds"),
                       "tuning": tuning,
                       "l2": "inputs larger than L2 (each step touches ~%.0f GB)" % (nbytes / 1e9),
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "plain": {"value": round(plain_gbs, 2), "unit": "GB/s", "launches_per_step": len(descs),
                      "batched_over_plain": round(value / world / plain_gbs, 2),
                      "threads_per_rank": threads,
                      "tuned_value": round(plain_tuned_gbs, 2) if plain_tuned_gbs else None,
                      "batched_over_tuned_plain": round(value / world / plain_tuned_gbs, 2) if plain_tuned_gbs else None},
            "roofline": {"bound": "hbm", "achieved": round(kernel_gbs, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(kernel_gbs / peak, 4), "peak_kind": peak_kind,
                         "traffic": int(NCU_TRAFFIC_BYTES_2_16 * n / (1 << 16)) if kinds == ALL_KINDS else None,
                         "traffic_note": ("bytes per launch: ncu DRAM read+write of the same launch at 2^16 "
                                          "elements per rank (4.51 GB, 1.12x its algorithmic bytes), scaled by "
                                          "elements per rank"),
                         "algorithmic_bytes": int(nbytes)},
            "e2e": {"value": round(e2e_gbs, 3), "unit": "GB/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "elements_per_rank": ne,
                    "seconds_per_step": round(esecs / e_steps, 5), "plans_only_seconds_per_step": round(ekern, 5),
                    "host_link_GBps": link, "e2e_buffer_h2d_GBps": round(buf_h2d, 1),
                    "form": "gpumpi_plan_run_host, the 16 communicators as 4 batched plans on 4 streams"},
            "sustained": sustained,
            "sweep": sweep,
            "apps": apps,
            "allocator": allocator,
            "verified": True,
            "verification": {"what": "every call of the timed plan after the timed region: Bcast and Alltoall "
                                     "outputs compared with their sources in full, Allreduce outputs of every "
                                     "rank with a NumPy rank-order fold at %d sampled positions plus every "
                                     "segment edge; bitwise" % args.verify_sample,
                             "seconds": round(verify_s, 2)},
            "cpu_baseline": cpu,
            "clocks": clocks.summary(),
            "gpu_launches": int(launches),
        }
        print(json.dumps(line), flush=True)
        bad_apps = [k for k, v in (apps or {}).items() if "error" in v]
        if bad_apps:
            raise SystemExit("application runs failed: " + ", ".join(bad_apps))
    for c in comms + ecomms:
        c.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
