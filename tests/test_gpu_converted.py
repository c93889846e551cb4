"""C programs through the source converter and gpumpicc.py onto the GPU.

The converter's test programs (tests/convert_cases/*.c) are converted and
compiled on this machine, run by the device runtime, and must print what the
unmodified C program prints on the hostmpi oracle (fileio.c writes, reads,
seeks and removes files through the launcher's host calls).  When the converted forms
of the reference's own programs are present (oracle/_ref/conv, made from the
reference tree by `make -C oracle -f ref.mk conv`), those run too: cpi.c must
print the golden lines, global_var.c must report no error, and NPB IS and DT
must pass their own verification and print what the oracle build of the same
source prints.
"""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASES = os.path.join(ROOT, "tests", "convert_cases")
ORACLE = os.path.join(ROOT, "oracle")
GPUMPICC = os.path.join(ROOT, "dphpc-project_gb300", "gpumpicc.py")
CONV = os.path.join(ORACLE, "_ref", "conv")
CASE_OPTS = {"globals": 0, "ring": 0, "coalesce": 3, "fileio": 0}
GPU_OPTS = ["--timeout-ms", "20000", "--max-seconds", "200"]
NPBDEFS = ['-DNPBVERSION="3.4.1"', '-DCOMPILETIME="n/a"', '-DMPICC="gcc"', '-DCFLAGS="-O2"', '-DCLINK="gcc"',
           '-DCLINKFLAGS=""', '-DCMPI_LIB="hostmpi"', '-DCMPI_INC=""']
HOSTINC = os.path.join(ORACLE, "hostmpi", "include")
HOSTLIB = os.path.join(ORACLE, "build", "libhostmpi.a")


def _check(r):
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-3000:])


def _gpumpicc(args, cwd):
    r = subprocess.run(["python3", GPUMPICC, *args], capture_output=True, text=True, cwd=cwd)
    _check(r)


def _run(cmd, timeout=300, cwd=None):
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=timeout, cwd=cwd)
    _check(r)
    return r.stdout


@pytest.fixture(scope="module")
def cases(gpu_built, tmp_path_factory):
    d = tmp_path_factory.mktemp("gpu_cases")
    out = {}
    for name, mv in CASE_OPTS.items():
        src = os.path.join(CASES, name + ".c")
        orig = str(d / (name + "_orig"))
        _check(subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-Dmain=hostmpi_user_main", "-I" + HOSTINC, src,
                               HOSTLIB, "-lstdc++", "-lpthread", "-lm", "-o", orig], capture_output=True, text=True))
        gpu = str(d / (name + "_gpu"))
        _gpumpicc(["--max-ranks", "64", "--malloc-version", str(mv), "--outdir", str(d), "--project", CASES, src,
                   "-O3", "-lm", "-o", gpu], cwd=str(d))
        out[name] = (orig, gpu)
    return out


@pytest.mark.parametrize("name", sorted(CASE_OPTS))
@pytest.mark.parametrize("ranks", [1, 3, 8, 64])
def test_gpu_converted_case_matches_the_original_on_hostmpi(cases, name, ranks, tmp_path):
    orig, gpu = cases[name]
    (tmp_path / "host").mkdir()
    (tmp_path / "gpu").mkdir()
    # fileio.c creates, reads and removes files in its working directory (on
    # the GPU through the launcher's host calls)
    want = _run([orig, "---gpumpi", "-n", str(ranks)], cwd=str(tmp_path / "host"))
    got = _run([gpu, "---gpumpi", "-n", str(ranks), *GPU_OPTS], cwd=str(tmp_path / "gpu"))
    assert want.strip() and got == want
    assert not list((tmp_path / "gpu").iterdir())


# ---------------------------------------------------------------- the reference's programs

needs_conv = pytest.mark.skipif(not os.path.isdir(CONV), reason="converted reference programs absent")


@needs_conv
def test_gpu_converted_reference_cpi_prints_the_golden_lines(gpu_built, tmp_path):
    exe = str(tmp_path / "cpi")
    _gpumpicc([os.path.join(CONV, "cpi", "cpi.cu"), "-o", exe], cwd=str(tmp_path))
    for line in open(os.path.join(ROOT, "tests", "golden", "cpi_pi.txt")):
        if line.startswith("#") or not line.strip():
            continue
        key, expect = line.rstrip("\n").split(" | ")
        n, ranks = key.split()
        assert expect in _run([exe, n, "---gpumpi", "-n", ranks, *GPU_OPTS])


@needs_conv
def test_gpu_converted_reference_global_var_passes(gpu_built, tmp_path):
    exe = str(tmp_path / "global_var")
    _gpumpicc([os.path.join(CONV, "global_var", "global_var.cu"), "-o", exe], cwd=str(tmp_path))
    for ranks in (1, 4, 64):
        out = _run([exe, "---gpumpi", "-n", str(ranks), *GPU_OPTS])
        assert "error" not in out


@pytest.fixture(scope="module")
def npb_is(gpu_built, tmp_path_factory):
    if not os.path.isdir(CONV):
        pytest.skip("converted reference programs absent")
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
def npb_dt(gpu_built, tmp_path_factory):
    if not os.path.isdir(os.path.join(CONV, "dt_S")):
        pytest.skip("converted reference programs absent")
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
