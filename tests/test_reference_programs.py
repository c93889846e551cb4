"""The oracle runs the reference's own MPI programs, unmodified.

oracle/ref.mk compiles, by path, the reference's pi example
(toolchain_tests/pi/cpi.c) and the vendored NPB IS kernel
(toolchain_tests/npb/NPB3.4.1/NPB3.4-MPI/IS/is.c, classes S, W and A, whose
built-in full verification checks the ranks against the class's known
answers, is.c:261-296 and 561-629) and NPB DT class S (DT/dt.c, verified
against its known L2 norms, dt.c:78-170, on the BH, WH and SH graphs)
against hostmpi.  Skipped when the
reference tree is not present.
"""
import os
import subprocess

import pytest

from conftest import reference_tree

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = reference_tree()
pytestmark = pytest.mark.skipif(REF is None,
                                reason="reference tree absent")


@pytest.fixture(scope="module")
def ref_built(oracle_built):
    r = subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "-f", "ref.mk", f"REF={REF}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    return os.path.join(ROOT, "oracle", "_ref")


@pytest.mark.parametrize("cls,ranks", [("S", 1), ("S", 2), ("S", 4), ("W", 4), ("W", 8), ("A", 4)])
def test_npb_is_verifies_on_the_oracle(ref_built, cls, ranks):
    r = subprocess.run([os.path.join(ref_built, f"is.{cls}"), "---gpumpi", "-n", str(ranks)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "Verification    =               SUCCESSFUL" in r.stdout


@pytest.mark.parametrize("graph,ranks", [("BH", 5), ("WH", 8), ("SH", 12)])
def test_npb_dt_verifies_on_the_oracle(ref_built, graph, ranks):
    r = subprocess.run([os.path.join(ref_built, "dt.S"), graph, "---gpumpi", "-n", str(ranks)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "Verification    =               SUCCESSFUL" in r.stdout


def test_reference_cpi_runs_on_the_oracle(ref_built):
    r = subprocess.run([os.path.join(ref_built, "cpi"), "100000", "---gpumpi", "-n", "8"],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0
    assert "pi is approximately 3.1415926535981349, Error is 0.0000000000083418" in r.stdout
