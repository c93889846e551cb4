"""Host collective C ABI (libgpumpi.so) against host folds in rank order."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def coll(gpu_built):
    import importlib.util
    import os
    import sys

    path = os.path.join(gpu_built.PKG, "gpumpi_coll.py")
    spec = importlib.util.spec_from_file_location("gpumpi_coll", path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[spec.name] = mod
    spec.loader.exec_module(mod)
    lib = gpu_built.load_library()
    mod.bind(lib)
    return mod, lib


def _rank_fold(xs, op):
    acc = xs[0].copy()
    for x in xs[1:]:
        if op == "sum":
            acc = x + acc
        elif op == "max":
            acc = np.where(x > acc, x, acc)
        elif op == "min":
            acc = np.where(x > acc, acc, x)
        elif op == "prod":
            acc = x * acc
    return acc


@pytest.mark.parametrize("algo", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("form", ["plain", "batched", "graph", "plain-flags", "graph-flags", "graph-mixed"])
@pytest.mark.parametrize("nranks,count", [(1, 5), (4, 1000), (7, 4097), (64, 1 << 12), (32, 1 << 16)])
def test_capi_collectives(coll, form, nranks, count, algo):
    """Every schedule (algo 1-4 and the size-based choice 0) folds in rank
    order, so each gives the host fold's bits, in the launch-ordered forms
    (the calls are independent), with flag rounds (-flags) and with both in
    one launch (-mixed)."""
    import torch

    mod, lib = coll
    g = torch.Generator().manual_seed(nranks * 1000 + count)
    comm = mod.Comm(lib, nranks)
    keep = []
    descs = []
    cases = []
    # allreduce sum fp64 and max int32, bcast, alltoall, allgather, reduce
    xf = [torch.rand(count, dtype=torch.float64, generator=g) * 2 - 1 for _ in range(nranks)]
    xi = [torch.randint(-(1 << 20), 1 << 20, (count,), dtype=torch.int32, generator=g) for _ in range(nranks)]
    df = [t.cuda() for t in xf]
    di = [t.cuda() for t in xi]
    of = [torch.empty_like(t) for t in df]
    oi = [torch.empty_like(t) for t in di]
    descs.append(mod.make_desc(comm, mod.COLL_ALLREDUCE, "float64", count, [t.data_ptr() for t in df],
                               [t.data_ptr() for t in of], mod.OP_SUM, 0, keep))
    descs.append(mod.make_desc(comm, mod.COLL_ALLREDUCE, "int32", count, [t.data_ptr() for t in di],
                               [t.data_ptr() for t in oi], mod.OP_MAX, 0, keep))
    root = nranks - 1
    bb = [t.clone() for t in df]
    descs.append(mod.make_desc(comm, mod.COLL_BCAST, "float64", count, None, [t.data_ptr() for t in bb],
                               mod.OP_SUM, root, keep))
    per = max(1, count // nranks)
    sa = [torch.randint(0, 1 << 30, (per * nranks,), dtype=torch.int32, generator=g).cuda() for _ in range(nranks)]
    ra = [torch.empty_like(t) for t in sa]
    descs.append(mod.make_desc(comm, mod.COLL_ALLTOALL, "int32", per, [t.data_ptr() for t in sa],
                               [t.data_ptr() for t in ra], 0, 0, keep))
    ag = [torch.empty(count * nranks, dtype=torch.float64, device="cuda") for _ in range(nranks)]
    descs.append(mod.make_desc(comm, mod.COLL_ALLGATHER, "float64", count, [t.data_ptr() for t in df],
                               [t.data_ptr() for t in ag], 0, 0, keep))
    rd = [torch.zeros(count, dtype=torch.float64, device="cuda") for _ in range(nranks)]
    descs.append(mod.make_desc(comm, mod.COLL_REDUCE, "float64", count, [t.data_ptr() for t in df],
                               [t.data_ptr() for t in rd], mod.OP_PROD, 0, keep))
    for d in descs:
        # Reduce has schedules 1 and 2; Allreduce 1-3 (3: every rank pushes its
        # segment); Alltoall/Allgather 1-3 (3: bulk engine)
        d.algo = 2 if (d.op == mod.COLL_REDUCE and algo == 3) else algo
    if form.endswith("-mixed"):
        # every other call keeps its flag rounds inside the launch-ordered plan
        for i, d in enumerate(descs):
            d.sync = i % 2
    plan = mod.Plan(lib, descs, threads=128, batched=not form.startswith("plain"))
    assert plan.launch_ordered
    if form.endswith("-flags"):
        plan.set_sync(1)
        assert not plan.launch_ordered
    if form.startswith("graph"):
        plan.capture()
    for _ in range(2):
        plan.launch()
    torch.cuda.synchronize()
    assert mod.status(lib) is None
    exp_f = _rank_fold([x.numpy() for x in xf], "sum")
    exp_i = _rank_fold([x.numpy() for x in xi], "max")
    exp_p = _rank_fold([x.numpy() for x in xf], "prod")
    for r in range(nranks):
        assert np.array_equal(of[r].cpu().numpy().view(np.uint64), exp_f.view(np.uint64))
        assert np.array_equal(oi[r].cpu().numpy(), exp_i)
        assert np.array_equal(bb[r].cpu().numpy(), xf[root].numpy())
        got = ra[r].cpu().numpy()
        for q in range(nranks):
            assert np.array_equal(got[q * per:(q + 1) * per], sa[q].cpu().numpy()[r * per:(r + 1) * per])
        assert np.array_equal(ag[r].cpu().numpy(), np.concatenate([x.numpy() for x in xf]))
    assert np.array_equal(rd[0].cpu().numpy().view(np.uint64), exp_p.view(np.uint64))
    plan.close()
    comm.close()


@pytest.mark.parametrize("algo", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("per", [3, 17, 250, 333, 4097, 70001])
def test_capi_misaligned_byte_copies(coll, per, algo):
    """Alltoall, Allgather and Bcast of bytes whose buffers start at 16-byte
    phases that differ by rank, so that the pieces of one call reach every
    pairing of source and destination alignment (the copy engine then moves
    the widest units both alignments share, down to single bytes).  Every
    output byte equals the host's, and the bytes just outside each output stay
    untouched."""
    import torch

    mod, lib = coll
    nranks = 6
    g = torch.Generator().manual_seed(per * 10 + algo)
    comm = mod.Comm(lib, nranks)
    keep, descs = [], []
    pad = 32

    def alloc(nbytes, off):
        t = torch.full((nbytes + 2 * pad,), 0xA5, dtype=torch.uint8, device="cuda")
        return t, t.data_ptr() + pad + off

    sends = [torch.randint(0, 256, (per * nranks,), dtype=torch.uint8, generator=g) for _ in range(nranks)]
    s_buf = [alloc(per * nranks, (5 * r + 3) % 16) for r in range(nranks)]
    for (t, ptr), x in zip(s_buf, sends):
        t[ptr - t.data_ptr():ptr - t.data_ptr() + x.numel()] = x.cuda()
    a2a = [alloc(per * nranks, (7 * r + 1) % 16) for r in range(nranks)]
    descs.append(mod.make_desc(comm, mod.COLL_ALLTOALL, "uint8", per, [p for _, p in s_buf],
                               [p for _, p in a2a], 0, 0, keep))
    ag = [alloc(per * nranks, (3 * r + 9) % 16) for r in range(nranks)]
    descs.append(mod.make_desc(comm, mod.COLL_ALLGATHER, "uint8", per, [p for _, p in s_buf],
                               [p for _, p in ag], 0, 0, keep))
    root = 2
    bc = [alloc(per * nranks, (11 * r + 6) % 16) for r in range(nranks)]
    t, ptr = bc[root]
    t[ptr - t.data_ptr():ptr - t.data_ptr() + per * nranks] = sends[root].cuda()
    descs.append(mod.make_desc(comm, mod.COLL_BCAST, "uint8", per * nranks, None, [p for _, p in bc], 0, root,
                               keep))
    for d in descs:
        d.algo = algo
    plan = mod.Plan(lib, descs, threads=128, batched=False)
    plan.launch()
    torch.cuda.synchronize()
    assert mod.status(lib) is None
    host = [x.numpy() for x in sends]

    def body(tp, nbytes):
        t, ptr = tp
        a = t.cpu().numpy()
        o = ptr - t.data_ptr()
        assert (a[:o] == 0xA5).all() and (a[o + nbytes:] == 0xA5).all(), "bytes outside the output changed"
        return a[o:o + nbytes]

    for r in range(nranks):
        exp_a2a = np.concatenate([host[q][r * per:(r + 1) * per] for q in range(nranks)])
        assert np.array_equal(body(a2a[r], per * nranks), exp_a2a)
        exp_ag = np.concatenate([host[q][:per] for q in range(nranks)])
        assert np.array_equal(body(ag[r], per * nranks), exp_ag)
        assert np.array_equal(body(bc[r], per * nranks), host[root])
    plan.close()
    comm.close()


def test_capi_batched_many_comms(coll):
    """Sixteen communicators of uneven sizes in one persistent launch."""
    import torch

    mod, lib = coll
    sizes = [4, 8, 12, 16, 24, 32, 40, 48, 56, 64, 72, 80, 88, 96, 128, 256]
    count = 4096
    comms = [mod.Comm(lib, p) for p in sizes]
    keep, descs, checks = [], [], []
    g = torch.Generator().manual_seed(7)
    for c, p in zip(comms, sizes):
        xs = [torch.randint(-(1 << 20), 1 << 20, (count,), dtype=torch.int32, generator=g) for _ in range(p)]
        ds = [x.cuda() for x in xs]
        outs = [torch.empty_like(d) for d in ds]
        descs.append(mod.make_desc(c, mod.COLL_ALLREDUCE, "int32", count, [d.data_ptr() for d in ds],
                                   [o.data_ptr() for o in outs], mod.OP_SUM, 0, keep))
        checks.append((xs, outs, ds))
    plan = mod.Plan(lib, descs, threads=128, batched=True)
    plan.capture()
    plan.launch()
    plan.launch()
    torch.cuda.synchronize()
    assert mod.status(lib) is None
    for xs, outs, _ in checks:
        exp = _rank_fold([x.numpy().astype(np.int32) for x in xs], "sum").astype(np.int32)
        for o in outs:
            assert np.array_equal(o.cpu().numpy(), exp)
    plan.close()
    for c in comms:
        c.close()


def test_autotune_picks_valid_schedules_and_keeps_results(coll, tmp_path):
    """The autotuner times the candidates, caches the plain results, and the
    tuned plans (plain at per-descriptor schedules and thread counts, batched
    at its own) give the same bits."""

    import torch

    mod, lib = coll
    sizes = [4, 24, 128]
    counts = [1 << 10, 1 << 15, 1 << 18]
    comms = [mod.Comm(lib, p) for p in sizes]
    keep, descs, checks = [], [], []
    g = torch.Generator().manual_seed(11)
    for c, p, n in zip(comms, sizes, counts):
        xs = [torch.rand(n, dtype=torch.float64, generator=g) for _ in range(p)]
        ds = [x.cuda() for x in xs]
        outs = [torch.empty_like(d) for d in ds]
        descs.append(mod.make_desc(c, mod.COLL_ALLREDUCE, "float64", n, [d.data_ptr() for d in ds],
                                   [o.data_ptr() for o in outs], mod.OP_SUM, 0, keep))
        per = n // p
        sa = [torch.randint(0, 1 << 30, (per * p,), dtype=torch.int32, generator=g).cuda() for _ in range(p)]
        ra = [torch.empty_like(t) for t in sa]
        descs.append(mod.make_desc(c, mod.COLL_ALLTOALL, "int32", per, [t.data_ptr() for t in sa],
                                   [t.data_ptr() for t in ra], 0, 0, keep))
        checks.append((xs, ds, outs, sa, ra, per, p))
    cache = str(tmp_path / "tune.txt")
    bt, plain, palgos = mod.autotune(lib, descs, reps=3, cache_path=cache)
    assert bt in (64, 128, 256, 512, 1024)
    assert all(t in (64, 128, 256, 512, 1024) for t in plain)
    assert all(d.algo in (1, 2, 3, 4) for d in descs) and all(a in (1, 2, 3, 4) for a in palgos)
    lines = open(cache).read().splitlines()
    assert len(descs) <= len(lines) <= 5 * len(descs)
    # a second run reads the plain results from the cache and returns the same plain choices
    bt2, plain2, palgos2 = mod.autotune(lib, descs, reps=3, cache_path=cache)
    assert plain2 == plain and palgos2 == palgos
    assert len(open(cache).read().splitlines()) == len(lines)
    pdescs = [type(d).from_buffer_copy(d) for d in descs]
    for d, a in zip(pdescs, palgos):
        d.algo = a
    for batched in (False, True):
        plan = mod.Plan(lib, descs if batched else pdescs, threads=bt, batched=batched, plain_threads=plain)
        plan.launch()
        torch.cuda.synchronize()
        assert mod.status(lib) is None
        for xs, ds, outs, sa, ra, per, p in checks:
            exp = _rank_fold([x.numpy() for x in xs], "sum")
            for o in outs:
                assert np.array_equal(o.cpu().numpy().view(np.uint64), exp.view(np.uint64))
            for r in range(p):
                got = ra[r].cpu().numpy()
                for q in range(p):
                    assert np.array_equal(got[q * per:(q + 1) * per], sa[q].cpu().numpy()[r * per:(r + 1) * per])
        plan.close()
    for c in comms:
        c.close()


def test_plain_plan_launches_with_different_staging_sizes(coll):
    """Plain launches of one plan get different staging areas (a 4-rank launch
    the largest, a 256-rank launch a smaller one); every launch must still be
    allowed its own size after the later picks, and give the rank-order fold."""
    import torch

    mod, lib = coll
    keep, descs, checks, comms = [], [], [], []
    g = torch.Generator().manual_seed(5)
    for p, n in ((4, 1 << 16), (4, 1 << 14), (256, 1 << 12)):
        c = mod.Comm(lib, p)
        comms.append(c)
        xs = [torch.rand(n, dtype=torch.float64, generator=g) for _ in range(p)]
        ds = [x.cuda() for x in xs]
        outs = [torch.empty_like(d) for d in ds]
        descs.append(mod.make_desc(c, mod.COLL_ALLREDUCE, "float64", n, [d.data_ptr() for d in ds],
                                   [o.data_ptr() for o in outs], mod.OP_SUM, 0, keep))
        checks.append((xs, ds, outs))
    plan = mod.Plan(lib, descs, threads=128, batched=False)
    for _ in range(2):
        plan.launch()
        torch.cuda.synchronize()
        assert mod.status(lib) is None
    for xs, ds, outs in checks:
        exp = _rank_fold([x.numpy() for x in xs], "sum")
        for o in outs:
            assert np.array_equal(o.cpu().numpy().view(np.uint64), exp.view(np.uint64))
    plan.close()
    for c in comms:
        c.close()


def test_plan_run_host_with_packed_host_buffers(coll):
    """Host-buffer entry point: per-rank host and device buffers laid out back
    to back (copies merge within one allocation) give the same results as the
    host fold, and the reported byte counts are exact."""
    import torch

    mod, lib = coll
    sizes, n = [4, 12, 48], 3000
    comms = [mod.Comm(lib, p) for p in sizes]
    keep, descs, layout = [], [], []
    g = torch.Generator().manual_seed(21)
    for c, p in zip(comms, sizes):
        din = torch.empty(p * n, dtype=torch.float64, device="cuda")
        dout = torch.empty(p * n, dtype=torch.float64, device="cuda")
        keep.extend([din, dout])
        descs.append(mod.make_desc(c, mod.COLL_ALLREDUCE, "float64", n, [din.data_ptr() + r * n * 8 for r in range(p)],
                                   [dout.data_ptr() + r * n * 8 for r in range(p)], mod.OP_SUM, 0, keep))
        layout.append((p, n * 8))
    total = sum(p * b for p, b in layout)
    hs = torch.rand(total // 8, dtype=torch.float64, generator=g).pin_memory()
    hr = torch.zeros(total // 8, dtype=torch.float64).pin_memory()
    sp, rp, off = [], [], 0
    for p, b in layout:
        for r in range(p):
            sp.append(hs.data_ptr() + off)
            rp.append(hr.data_ptr() + off)
            off += b
    plan = mod.Plan(lib, descs, threads=128, batched=True)
    bi, bo = plan.run_host(sp, rp)
    torch.cuda.synchronize()
    assert mod.status(lib) is None
    assert bi == total and bo == total
    off = 0
    for p, b in layout:
        xs = [hs[(off + r * b) // 8:(off + (r + 1) * b) // 8].numpy() for r in range(p)]
        exp = _rank_fold(xs, "sum")
        for r in range(p):
            got = hr[(off + r * b) // 8:(off + (r + 1) * b) // 8].numpy()
            assert np.array_equal(got.view(np.uint64), exp.view(np.uint64))
        off += p * b
    plan.close()
    for c in comms:
        c.close()


@pytest.mark.parametrize("threads", [64, 256])
def test_dependent_calls_keep_their_flag_rounds(coll, threads):
    """A plan whose second Allreduce reads the first one's output (and whose
    Alltoall writes a buffer the first Allreduce reads) is not launch-ordered:
    its calls synchronise with flags, in order, and give the rank-order
    folds of the chained calls."""
    import torch

    mod, lib = coll
    p, n = 24, 5000
    comm = mod.Comm(lib, p)
    g = torch.Generator().manual_seed(99)
    xs = [torch.rand(n, dtype=torch.float64, generator=g) * 2 - 1 for _ in range(p)]
    d_in = [x.cuda() for x in xs]
    d_mid = [torch.empty_like(d) for d in d_in]
    d_out = [torch.empty_like(d) for d in d_in]
    per = n // p
    a2_in = [torch.rand(per * p, dtype=torch.float64, generator=g).cuda() for _ in range(p)]
    keep = []
    descs = [mod.make_desc(comm, mod.COLL_ALLREDUCE, "float64", n, [t.data_ptr() for t in d_in],
                           [t.data_ptr() for t in d_mid], mod.OP_SUM, 0, keep),
             mod.make_desc(comm, mod.COLL_ALLREDUCE, "float64", n, [t.data_ptr() for t in d_mid],
                           [t.data_ptr() for t in d_out], mod.OP_SUM, 0, keep),
             # writes the first call's input buffers (a write-after-read hazard)
             mod.make_desc(comm, mod.COLL_ALLTOALL, "float64", per, [t.data_ptr() for t in a2_in],
                           [t.data_ptr() for t in d_in], 0, 0, keep)]
    plan = mod.Plan(lib, descs, threads=threads, batched=True)
    assert not plan.launch_ordered
    plan.launch()
    torch.cuda.synchronize()
    assert mod.status(lib) is None
    mid = _rank_fold([x.numpy() for x in xs], "sum")
    out = _rank_fold([mid] * p, "sum")
    for r in range(p):
        assert np.array_equal(d_mid[r].cpu().numpy().view(np.uint64), mid.view(np.uint64))
        assert np.array_equal(d_out[r].cpu().numpy().view(np.uint64), out.view(np.uint64))
        got = d_in[r].cpu().numpy()
        for q in range(p):
            assert np.array_equal(got[q * per:(q + 1) * per], a2_in[q].cpu().numpy()[r * per:(r + 1) * per])
    plan.close()
    comm.close()
