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

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
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


# DRAM bytes (read + write) of one batched launch, from ncu captures
# (dram__bytes_read.sum + dram__bytes_write.sum, one pass): at the full 2^20
# elements per rank, and at 2^15, which other per-rank counts scale from.
NCU_TRAFFIC_BYTES_2_20 = 27657256704 + 39027092480
NCU_TRAFFIC_BYTES_2_15 = 0.979630336e9 + 1.461430e9


ALL_KINDS = ("bcast", "allreduce", "alltoall")


def alg_bytes(sizes, n, kinds=ALL_KINDS):
    total = 0
    for p in sizes:
        for s in (4, 8):
            if "bcast" in kinds:
                total += p * n * s              # Bcast
            if "allreduce" in kinds:
                total += 2 * p * n * s          # Allreduce
            per = n // p
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
        per = n // p
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
    ap.add_argument("--no-tune", action="store_true", help="built-in schedules, --threads for every launch")
    ap.add_argument("--tune-reps", type=int, default=3)
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
                  "plain_threads_counts": {str(t): plain_threads.count(t) for t in sorted(set(plain_threads))}}
        plan = coll.Plan(lib, descs, threads=threads, batched=True)
        # the tuner ran the calls on these buffers: give every input (and the
        # broadcast buffers of the non-root ranks) fresh data, so that the
        # results checked after the timed region come from the timed launches
        g = torch.Generator(device="cuda").manual_seed(11)
        for it in items:
            fill_random(torch, it.send if it.send is not None else it.recv, it.dt, g)
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
    err = coll.status(lib)
    if err:
        raise SystemExit(f"device error during benchmark: {err}")
    secs = max_over_ranks(dist, torch, secs)
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
    psecs = time_plan(torch, plain, args.plain_steps, 1, stream)
    plain_gbs = nbytes * args.plain_steps / psecs / 1e9
    plain.close()
    plain_tuned_gbs = None
    if plain_threads:
        pdescs = [type(d).from_buffer_copy(d) for d in descs]
        for d, a in zip(pdescs, plain_algos):
            d.algo = a
        plain = coll.Plan(lib, pdescs, threads=threads, batched=False, plain_threads=plain_threads)
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
    for ep in eplans:
        ep.close()
    del eparts

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
                       "threads_per_rank": threads, "form": "batched, CUDA graph replay",
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
                         "traffic": (NCU_TRAFFIC_BYTES_2_20 if n == 1 << 20 else
                                     int(NCU_TRAFFIC_BYTES_2_15 * n / (1 << 15))) if kinds == ALL_KINDS else None,
                         "traffic_note": ("bytes per launch, ncu DRAM read+write of this launch at 2^20 elements "
                                          "per rank" if n == 1 << 20 else
                                          "bytes per launch, ncu DRAM read+write at 2^15 elements per rank "
                                          "scaled by elements per rank"),
                         "algorithmic_bytes": int(nbytes)},
            "e2e": {"value": round(e2e_gbs, 3), "unit": "GB/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "elements_per_rank": ne,
                    "form": "gpumpi_plan_run_host, the 16 communicators as 4 batched plans on 4 streams"},
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
    for c in comms + ecomms:
        c.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
