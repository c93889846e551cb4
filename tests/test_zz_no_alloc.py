"""Allocation-free allreduce (gpumpi_allreduce_noalloc) against the plain C ABI.

Callers that may not allocate device memory on their call path (a server
that reserved HBM at start-up, code under a fixed allocator budget, a thread
that must not let cudaMalloc synchronise the device) use this entry point;
its result must equal the allocating collective API's, bit for bit, on
consecutive calls that share its fixed device scratch array.  This file is
collected last so that a failure here stops a `-x` run only after every
other test has run.
"""
import ctypes
import importlib.util
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _coll(host):
    path = os.path.join(host.PKG, "gpumpi_coll.py")
    spec = importlib.util.spec_from_file_location("gpumpi_coll", path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[spec.name] = mod
    spec.loader.exec_module(mod)
    return mod


@pytest.mark.parametrize("calls", [[(4, 1000, "float64", 2), (7, 4097, "int32", 0)],
                                   [(256, 1 << 14, "float64", 2), (3, 5, "float64", 3)]])
def test_noalloc_allreduce_matches_capi(gpu_built, calls):
    import torch

    coll = _coll(gpu_built)
    lib = coll.bind(gpu_built.load_library())
    lib.gpumpi_allreduce_noalloc.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p),
                                             ctypes.c_int, ctypes.c_uint64, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_int, ctypes.c_void_p]
    tdt = {"float64": torch.float64, "int32": torch.int32}
    for nranks, count, dt, redop in calls:  # two calls in a row share the scratch array
        g = torch.Generator().manual_seed(nranks * 7 + count)
        if dt == "int32":
            xs = [torch.randint(-(1 << 20), 1 << 20, (count,), dtype=torch.int32, generator=g) for _ in range(nranks)]
        else:
            xs = [torch.rand(count, dtype=torch.float64, generator=g) * 2 - 1 for _ in range(nranks)]
        dev = [x.cuda() for x in xs]
        out_na = [torch.full_like(d, -7) for d in dev]
        out_ref = [torch.full_like(d, -9) for d in dev]
        send = (ctypes.c_void_p * nranks)(*[d.data_ptr() for d in dev])
        recv = (ctypes.c_void_p * nranks)(*[o.data_ptr() for o in out_na])
        rc = lib.gpumpi_allreduce_noalloc(send, recv, nranks, count, coll.DT[dt], redop, 128, None)
        assert rc == 0, lib.gpumpi_last_error().decode()
        comm = coll.Comm(lib, nranks)
        keep = []
        d = coll.make_desc(comm, coll.COLL_ALLREDUCE, dt, count, [x.data_ptr() for x in dev],
                           [o.data_ptr() for o in out_ref], redop, 0, keep)
        arr = (coll.Desc * 1)(d)
        coll.check(lib, lib.gpumpi_coll_plain(arr, 1, 128, None), "gpumpi_coll_plain")
        torch.cuda.synchronize()
        for a, b in zip(out_na, out_ref):
            assert np.array_equal(a.cpu().numpy().view(np.uint8), b.cpu().numpy().view(np.uint8))
        comm.close()


def test_noalloc_rejects_oversize(gpu_built):
    coll = _coll(gpu_built)
    lib = coll.bind(gpu_built.load_library())
    lib.gpumpi_allreduce_noalloc.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p),
                                             ctypes.c_int, ctypes.c_uint64, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_int, ctypes.c_void_p]
    n = 257
    ptrs = (ctypes.c_void_p * n)(*([1] * n))
    rc = lib.gpumpi_allreduce_noalloc(ptrs, ptrs, n, 16, coll.DT["float64"], 2, 128, None)
    assert rc != 0
    assert b"at most 256" in lib.gpumpi_last_error()
