"""CPU checks of host-side pieces: the printf formatter and the C ABI library.

The formatter (csrc/fmt.h) is shared by device code and the host; it is
compiled here for the host and compared with the C library's snprintf on
seeded random values and specifications.  The C ABI test loads
libgpumpi.so (no GPU needed to load it) and checks that every function
declared in include/gpumpi.h is exported.
"""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions(path):
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^[A-Za-z_][\w \*]*?\b(gpumpi_\w+)\s*\(", text, flags=re.M)))


@pytest.mark.parametrize("seed", [7, 1234567])
def test_formatter_matches_libc(tmp_path, seed):
    exe = tmp_path / "fmt_check"
    r = subprocess.run(["g++", "-O1", "-std=c++17", "-Wno-format", "-Wno-format-security",
                        "-I", os.path.join(ROOT, "dphpc-project_gb300", "csrc"),
                        os.path.join(ROOT, "tests", "native", "fmt_check.cpp"), "-o", str(exe), "-lm"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe), "100000", str(seed)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-3000:]
    assert "mismatches 0" in r.stdout


def test_header_lists_expected_entry_points():
    names = header_functions(os.path.join(ROOT, "include", "gpumpi.h"))
    for must in ("gpumpi_main", "gpumpi_run_program", "gpumpi_comm_create", "gpumpi_plan_create",
                 "gpumpi_plan_run_host", "gpumpi_allreduce_noalloc", "gpumpi_kernel_launches"):
        assert must in names


def test_capi_library_exports_every_declared_symbol(gpu_built):
    lib_path = os.path.join(gpu_built.PKG, "build", "libgpumpi.so")
    lib = ctypes.CDLL(lib_path)      # loading needs no GPU; nothing is called
    # gpumpi_main is the launcher entry each program executable exports (checked below)
    names = [n for n in header_functions(os.path.join(ROOT, "include", "gpumpi.h")) if n != "gpumpi_main"]
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    nm = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True)
    exported = {ln.split()[-1] for ln in nm.stdout.splitlines() if ln.strip()}
    assert not [n for n in names if n not in exported]


def test_program_binaries_link_the_runtime(gpu_built):
    """Each converted program is an executable exporting the launcher entry."""
    bindir = os.path.join(gpu_built.PKG, "build", "bin")
    progs = sorted(os.listdir(bindir))
    assert {"pi", "kat_p2p", "kat_coll", "coll_bench"} <= set(progs)
    for p in progs:
        nm = subprocess.run(["nm", os.path.join(bindir, p)], capture_output=True, text=True)
        assert "gpumpi_main" in nm.stdout, p


def test_bench_algorithmic_bytes_by_collective():
    """The bench's byte counts: Bcast P*n*s, Allreduce 2*P*n*s, Alltoall 2*P^2*m
    per communicator and type; a subset of collectives counts only its part."""
    import sys
    sys.path.insert(0, ROOT)
    import bench
    n = 1 << 10
    sizes = bench.COMM_SIZES
    per_type = sum(p * n for p in sizes) * (4 + 8)
    assert bench.alg_bytes(sizes, n, ("bcast",)) == per_type
    assert bench.alg_bytes(sizes, n, ("allreduce",)) == 2 * per_type
    assert bench.alg_bytes(sizes, n, ("alltoall",)) == sum(2 * p * p * (n // p) for p in sizes) * (4 + 8)
    assert bench.alg_bytes(sizes, n) == sum(bench.alg_bytes(sizes, n, (k,)) for k in bench.ALL_KINDS)
    assert sum(sizes) == 1024 and len(sizes) == 16
