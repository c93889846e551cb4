"""Host-side helpers for the GB300 device MPI runtime.

Builds the CUDA runtime and the program binaries, runs programs through the
C-ABI launcher (each program executable is a thin `main` around
`gpumpi_main`), and binds the host collective C ABI of libgpumpi.so with
ctypes.  The product path is the CUDA runtime: nothing here
falls back to the CPU; loading libgpumpi.so fails loudly if it is missing.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys
from dataclasses import dataclass

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
BUILD = os.path.join(PKG, "build")
BIN = os.path.join(BUILD, "bin")
LIB = os.path.join(BUILD, "libgpumpi.so")


def _jobs() -> int:
    return max(1, min(32, os.cpu_count() or 1))


def build(verbose: bool = False) -> None:
    """Compile the CUDA runtime and programs (sm_103a)."""
    out = None if verbose else subprocess.PIPE
    r = subprocess.run(["make", "-C", PKG, f"-j{_jobs()}"], stdout=out, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout or "")
        raise RuntimeError(f"build failed in {PKG}")


@dataclass
class RunResult:
    returncode: int
    stdout: str
    stderr: str

    def lines(self, prefix: str = "") -> list[str]:
        return [ln for ln in self.stdout.splitlines() if ln.startswith(prefix)]


def _run(exe: str, args: list[str], nranks: int, extra: list[str], timeout: float) -> RunResult:
    if not os.path.exists(exe):
        raise FileNotFoundError(f"{exe} is not built; run build() first")
    cmd = [exe, *args, "---gpumpi", "-n", str(nranks), *extra]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=timeout)
    return RunResult(r.returncode, r.stdout, r.stderr)


def run_program(name: str, args: list[str] | None = None, nranks: int = 2,
                extra: list[str] | None = None, timeout: float = 300.0) -> RunResult:
    """Run a converted program on the GPU (one rank per thread block)."""
    return _run(os.path.join(BIN, name), args or [], nranks, extra or [], timeout)


def load_library() -> ctypes.CDLL:
    """Load libgpumpi.so (the host collective C ABI)."""
    if not os.path.exists(LIB):
        raise FileNotFoundError(f"{LIB} missing: the CUDA runtime is not built")
    return ctypes.CDLL(LIB, mode=ctypes.RTLD_GLOBAL)


class ChurnStats(ctypes.Structure):
    """gpumpi_churn_stats of include/gpumpi.h."""
    _fields_ = [("allocs", ctypes.c_uint64), ("frees", ctypes.c_uint64), ("failed", ctypes.c_uint64),
                ("corrupt", ctypes.c_uint64), ("misaligned", ctypes.c_uint64), ("seconds", ctypes.c_double),
                ("ops_per_s", ctypes.c_double), ("malloc_cycles_p50", ctypes.c_uint64),
                ("malloc_cycles_p99", ctypes.c_uint64), ("fresh_pages", ctypes.c_uint64),
                ("partial_pops", ctypes.c_uint64), ("partial_full", ctypes.c_uint64),
                ("malloc_cycles_mean", ctypes.c_uint64), ("free_cycles_p50", ctypes.c_uint64),
                ("free_cycles_p99", ctypes.c_uint64), ("free_cycles_mean", ctypes.c_uint64)]


def malloc_churn(lib: ctypes.CDLL, blocks: int, threads: int, iters: int, live: int = 8, seed: int = 1,
                 heap_bytes: int = 0, cuda_heap: bool = False) -> dict:
    """Run gpumpi_malloc_churn (every thread loops malloc/fill/verify/free) and return its stats."""
    f = lib.gpumpi_malloc_churn
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_uint64, ctypes.c_size_t,
                  ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ChurnStats)]
    f.restype = ctypes.c_int
    lib.gpumpi_last_error.restype = ctypes.c_char_p
    st = ChurnStats()
    rc = f(blocks, threads, iters, live, seed, heap_bytes, int(cuda_heap), None, ctypes.byref(st))
    if rc != 0:
        raise RuntimeError(f"gpumpi_malloc_churn failed ({rc}): {lib.gpumpi_last_error().decode()}")
    return {k: getattr(st, k) for k, _ in ChurnStats._fields_}


def malloc_bench(lib: ctypes.CDLL, blocks: int = 12, threads: int = 1024, nbytes: int = 400,
                 heap_bytes: int = 0, cuda_heap: bool = False) -> dict:
    """gpumpi_malloc_bench: one malloc / write / check / free per thread (the
    reference allocator benchmark's shape); returns its stats."""
    f = lib.gpumpi_malloc_bench
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p,
                  ctypes.POINTER(ChurnStats)]
    f.restype = ctypes.c_int
    lib.gpumpi_last_error.restype = ctypes.c_char_p
    st = ChurnStats()
    rc = f(blocks, threads, nbytes, heap_bytes, int(cuda_heap), None, ctypes.byref(st))
    if rc != 0:
        raise RuntimeError(f"gpumpi_malloc_bench failed ({rc}): {lib.gpumpi_last_error().decode()}")
    return {k: getattr(st, k) for k, _ in ChurnStats._fields_}
