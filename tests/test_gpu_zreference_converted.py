"""The reference's own MPI programs, converted, on the GPU.

The converted forms of the reference's cpi.c, global_var.c, NPB IS (classes
S, W, A) and NPB DT (class S) live in oracle/_ref/conv (made from the
reference tree by `make -C oracle -f ref.mk conv`, which the build step runs
wherever the tree is present; the directory is generated, never committed,
and travels with the working tree).  cpi.c must print the golden lines,
global_var.c must report no error, and NPB IS and DT must pass their own
verification and print what the oracle build of the same source prints.
When the directory is missing and no reference tree is at hand to make it,
the tests fail with that message rather than skip.
"""
import os
import subprocess

import pytest

from conftest import reference_tree
from test_gpu_converted import GPU_OPTS, HOSTINC, HOSTLIB, NPBDEFS, ORACLE, ROOT, _check, _gpumpicc, _run

pytestmark = pytest.mark.gpu

CONV = os.path.join(ORACLE, "_ref", "conv")


@pytest.fixture(scope="module")
def conv(gpu_built):
    if not os.path.isdir(os.path.join(CONV, "dt_S")):
        ref = reference_tree()
        if ref is None:
            pytest.fail("oracle/_ref/conv (the converted reference programs) is missing and no reference tree "
                        "is present to make it: run `make -C oracle -f ref.mk conv` where the tree is")
        r = subprocess.run(["make", "-C", ORACLE, "-f", "ref.mk", f"REF={ref}", "conv"], capture_output=True,
                           text=True)
        assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    return CONV


def test_gpu_converted_reference_cpi_prints_the_golden_lines(conv, tmp_path):
    exe = str(tmp_path / "cpi")
    _gpumpicc([os.path.join(CONV, "cpi", "cpi.cu"), "-o", exe], cwd=str(tmp_path))
    for line in open(os.path.join(ROOT, "tests", "golden", "cpi_pi.txt")):
        if line.startswith("#") or not line.strip():
            continue
        key, expect = line.rstrip("\n").split(" | ")
        n, ranks = key.split()
        assert expect in _run([exe, n, "---gpumpi", "-n", ranks, *GPU_OPTS])


def test_gpu_converted_reference_global_var_passes(conv, tmp_path):
    exe = str(tmp_path / "global_var")
    _gpumpicc([os.path.join(CONV, "global_var", "global_var.cu"), "-o", exe], cwd=str(tmp_path))
    for ranks in (1, 4, 64):
        out = _run([exe, "---gpumpi", "-n", str(ranks), *GPU_OPTS])
        assert "error" not in out


@pytest.fixture(scope="module")
def npb_is(conv, tmp_path_factory):
    d = tmp_path_factory.mktemp("npb_is")
    npb = os.path.join(CONV, "npb")
    srcs = [os.path.join(npb, "IS", "is.cu"), os.path.join(npb, "common", "c_print_results.cu"),
            os.path.join(npb, "common", "c_timers.cu")]
    exes = {}
    for cls in ("S", "W", "A"):
        inc = "-I" + os.path.join(CONV, "is_" + cls)
        gpu = str(d / ("is_gpu." + cls))
        _gpumpicc([*srcs, inc, *NPBDEFS, "-o", gpu], cwd=str(d))
        host = str(d / ("is_host." + cls))
        _check(subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-w", "-x", "c++", "-I" + HOSTINC,
                               inc, *NPBDEFS, *srcs, "-x", "none", HOSTLIB, "-lpthread", "-o", host],
                              capture_output=True, text=True))
        exes[cls] = (gpu, host)
    return exes


def _stable(text):
    return [x for x in text.splitlines() if "Time in seconds" not in x and "Mop/s" not in x]


@pytest.mark.parametrize("cls,ranks", [("S", 1), ("S", 2), ("S", 4), ("W", 8), ("A", 16)])
def test_gpu_converted_npb_is_verifies_and_matches_hostmpi(npb_is, cls, ranks):
    gpu, host = npb_is[cls]
    got = _run([gpu, "---gpumpi", "-n", str(ranks), "-p", "4G", *GPU_OPTS], timeout=400)
    want = _run([host, "---gpumpi", "-n", str(ranks)], timeout=400)
    assert "Verification    =               SUCCESSFUL" in got
    assert _stable(got) == _stable(want)


@pytest.fixture(scope="module")
def npb_dt(conv, tmp_path_factory):
    d = tmp_path_factory.mktemp("npb_dt")
    npb = os.path.join(CONV, "npb")
    srcs = [os.path.join(npb, "DT", "dt.cu"), os.path.join(npb, "DT", "DGraph.cu"),
            os.path.join(npb, "common", "randdp.cu"), os.path.join(npb, "common", "c_print_results.cu"),
            os.path.join(npb, "common", "c_timers.cu")]
    inc = "-I" + os.path.join(CONV, "dt_S")
    gpu = str(d / "dt_gpu.S")
    _gpumpicc([*srcs, inc, *NPBDEFS, "-o", gpu], cwd=str(d))
    host = str(d / "dt_host.S")
    _check(subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-w", "-x", "c++", "-I" + HOSTINC, inc,
                           *NPBDEFS, *srcs, "-x", "none", HOSTLIB, "-lpthread", "-o", host],
                          capture_output=True, text=True))
    return gpu, host


@pytest.mark.parametrize("graph,ranks", [("BH", 5), ("WH", 8), ("SH", 12), ("SH", 21)])
def test_gpu_converted_npb_dt_verifies_and_matches_hostmpi(npb_dt, graph, ranks):
    gpu, host = npb_dt
    got = _run([gpu, graph, "---gpumpi", "-n", str(ranks), *GPU_OPTS], timeout=400)
    want = _run([host, graph, "---gpumpi", "-n", str(ranks)], timeout=400)
    assert "Verification    =               SUCCESSFUL" in got
    assert _stable(got) == _stable(want)
