"""C programs through the source converter and gpumpicc.py onto the GPU.

The converter's test programs (tests/convert_cases/*.c) are converted and
compiled on this machine, run by the device runtime, and must print what the
unmodified C program prints on the hostmpi oracle (fileio.c writes, reads,
seeks and removes files through the launcher's host calls).  The
reference's own programs through the same path are in
test_gpu_zreference_converted.py.
"""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASES = os.path.join(ROOT, "tests", "convert_cases")
ORACLE = os.path.join(ROOT, "oracle")
GPUMPICC = os.path.join(ROOT, "dphpc-project_gb300", "gpumpicc.py")
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
