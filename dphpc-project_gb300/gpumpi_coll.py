"""ctypes binding of the host collective C ABI (include/gpumpi.h, section 2).

Device buffers come from PyTorch (plumbing only); every collective runs in the
CUDA kernels of libgpumpi.so.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_char_p, c_int, c_uint64, c_void_p

COLL_BARRIER, COLL_BCAST, COLL_REDUCE, COLL_ALLREDUCE, COLL_ALLTOALL, COLL_ALLGATHER = range(6)
OP_MAX, OP_MIN, OP_SUM, OP_PROD = range(4)
DT = {"int32": 2, "int64": 20, "float32": 12, "float64": 13, "uint8": 29}


class Desc(ctypes.Structure):
    _fields_ = [
        ("comm", c_void_p),
        ("op", c_int),
        ("dtype", c_int),
        ("redop", c_int),
        ("root", c_int),
        ("count", c_uint64),
        ("sendbufs", POINTER(c_void_p)),
        ("recvbufs", POINTER(c_void_p)),
        ("algo", c_int),
        ("sync", c_int),
    ]


def bind(lib: ctypes.CDLL) -> ctypes.CDLL:
    lib.gpumpi_comm_create.argtypes = [c_int, POINTER(c_void_p)]
    lib.gpumpi_comm_destroy.argtypes = [c_void_p]
    lib.gpumpi_plan_create.argtypes = [POINTER(Desc), c_int, c_int, c_int, POINTER(c_void_p)]
    lib.gpumpi_plan_create_ex.argtypes = [POINTER(Desc), c_int, c_int, c_int, POINTER(c_int), POINTER(c_void_p)]
    lib.gpumpi_autotune.argtypes = [POINTER(Desc), c_int, c_void_p, POINTER(c_int), POINTER(c_int), POINTER(c_int)]
    lib.gpumpi_plan_launch.argtypes = [c_void_p, c_void_p]
    lib.gpumpi_plan_capture.argtypes = [c_void_p, c_void_p]
    lib.gpumpi_plan_set_sync.argtypes = [c_void_p, c_int]
    lib.gpumpi_plan_launch_ordered.argtypes = [c_void_p]
    lib.gpumpi_plan_run_host.argtypes = [c_void_p, POINTER(c_void_p), POINTER(c_void_p), c_void_p,
                                         POINTER(c_uint64), POINTER(c_uint64)]
    lib.gpumpi_plan_destroy.argtypes = [c_void_p]
    lib.gpumpi_coll_plain.argtypes = [POINTER(Desc), c_int, c_int, c_void_p]
    lib.gpumpi_coll_batched.argtypes = [POINTER(Desc), c_int, c_int, c_void_p]
    lib.gpumpi_api_status.argtypes = [c_char_p, c_int]
    lib.gpumpi_last_error.restype = c_char_p
    lib.gpumpi_kernel_launches.restype = c_uint64
    return lib


def check(lib, rc: int, what: str) -> None:
    if rc != 0:
        raise RuntimeError(f"{what} failed ({rc}): {lib.gpumpi_last_error().decode()}")


class Comm:
    def __init__(self, lib, nranks: int):
        self.lib = lib
        self.n = nranks
        h = c_void_p()
        check(lib, lib.gpumpi_comm_create(nranks, ctypes.byref(h)), "gpumpi_comm_create")
        self.h = h

    def close(self):
        if self.h:
            self.lib.gpumpi_comm_destroy(self.h)
            self.h = None


def ptr_array(ptrs):
    arr = (c_void_p * len(ptrs))(*ptrs)
    return arr


def make_desc(comm: Comm, op: int, dtype: str, count: int, send_ptrs=None, recv_ptrs=None,
              redop: int = OP_SUM, root: int = 0, keep: list | None = None, algo: int = 0) -> Desc:
    s = ptr_array(send_ptrs) if send_ptrs is not None else None
    r = ptr_array(recv_ptrs) if recv_ptrs is not None else None
    if keep is not None:
        keep.extend([s, r])
    return Desc(comm.h, op, DT[dtype], redop, root, count,
                ctypes.cast(s, POINTER(c_void_p)) if s is not None else None,
                ctypes.cast(r, POINTER(c_void_p)) if r is not None else None, algo, 0)


class TuneOpts(ctypes.Structure):
    _fields_ = [("reps", c_int), ("cache_path", ctypes.c_char_p), ("verbose", c_int)]


def autotune(lib, descs: list, reps: int = 5, cache_path: str | None = None, verbose: bool = False):
    """gpumpi_autotune: sets every descriptor's algo and sync (the batched
    choice) in place; returns (threads per rank of the batched launch,
    per-descriptor plain-form threads, per-descriptor plain-form algos)."""
    arr = (Desc * len(descs))(*descs)
    plain = (c_int * len(descs))()
    palgo = (c_int * len(descs))()
    bt = c_int(0)
    opts = TuneOpts(reps, cache_path.encode() if cache_path else None, 1 if verbose else 0)
    check(lib, lib.gpumpi_autotune(arr, len(descs), ctypes.byref(opts), ctypes.byref(bt), plain, palgo),
          "gpumpi_autotune")
    for i, d in enumerate(descs):
        d.algo = arr[i].algo
        d.sync = arr[i].sync
    return bt.value, list(plain), list(palgo)


class Plan:
    def __init__(self, lib, descs: list[Desc], threads: int = 128, batched: bool = True,
                 plain_threads: list | None = None):
        self.lib = lib
        arr = (Desc * len(descs))(*descs)
        self._arr = arr
        pt = (c_int * len(descs))(*plain_threads) if plain_threads else None
        h = c_void_p()
        check(lib, lib.gpumpi_plan_create_ex(arr, len(descs), threads, 1 if batched else 0, pt, ctypes.byref(h)),
              "gpumpi_plan_create_ex")
        self.h = h

    def launch(self, stream: int = 0):
        check(self.lib, self.lib.gpumpi_plan_launch(self.h, c_void_p(stream)), "gpumpi_plan_launch")

    def set_sync(self, mode: int):
        """0: launch-ordered forms when the calls are independent; 1: flag rounds."""
        check(self.lib, self.lib.gpumpi_plan_set_sync(self.h, mode), "gpumpi_plan_set_sync")

    @property
    def launch_ordered(self) -> bool:
        return bool(self.lib.gpumpi_plan_launch_ordered(self.h))

    def capture(self, stream: int = 0):
        check(self.lib, self.lib.gpumpi_plan_capture(self.h, c_void_p(stream)), "gpumpi_plan_capture")

    def run_host(self, host_send: list, host_recv: list, stream: int = 0):
        s = ptr_array(host_send)
        r = ptr_array(host_recv)
        bi, bo = c_uint64(), c_uint64()
        check(self.lib, self.lib.gpumpi_plan_run_host(self.h, s, r, c_void_p(stream), ctypes.byref(bi),
                                                       ctypes.byref(bo)), "gpumpi_plan_run_host")
        return bi.value, bo.value

    def close(self):
        if self.h:
            self.lib.gpumpi_plan_destroy(self.h)
            self.h = None


def status(lib) -> str | None:
    buf = ctypes.create_string_buffer(256)
    rc = lib.gpumpi_api_status(buf, 256)
    return None if rc == 0 else buf.value.decode()


def allreduce_check(lib, nranks: int = 4, count: int = 1000) -> bool:
    """One batched FP64 allreduce through the C ABI, compared bit for bit with
    a host fold in rank order (acc = x_0; acc = x_q + acc)."""
    import numpy as np
    import torch

    bind(lib)
    g = torch.Generator(device="cpu").manual_seed(1234)
    xs = [torch.rand(count, dtype=torch.float64, generator=g) * 2 - 1 for _ in range(nranks)]
    dev_in = [x.cuda() for x in xs]
    dev_out = [torch.empty_like(x) for x in dev_in]
    comm = Comm(lib, nranks)
    keep: list = []
    d = make_desc(comm, COLL_ALLREDUCE, "float64", count, [t.data_ptr() for t in dev_in],
                  [t.data_ptr() for t in dev_out], OP_SUM, 0, keep)
    arr = (Desc * 1)(d)
    check(lib, lib.gpumpi_coll_batched(arr, 1, 128, None), "gpumpi_coll_batched")
    torch.cuda.synchronize()
    acc = xs[0].numpy().copy()
    for q in range(1, nranks):
        acc = xs[q].numpy() + acc
    ok = all(np.array_equal(o.cpu().numpy().view(np.uint64), acc.view(np.uint64)) for o in dev_out)
    comm.close()
    return ok
