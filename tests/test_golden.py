"""Golden vectors from the reference's own pi program (tests/golden/cpi_pi.txt).

The fixture holds the result lines of the reference's toolchain_tests/pi/cpi.c
(MPICH's example) compiled unmodified against the hostmpi oracle; it is
regenerated by tests/golden/make_golden.py.  The oracle's build of our
converted pi program must print the same lines; when the reference tree is
present, the fixture itself is rebuilt and compared.
"""
import os
import tempfile

import pytest

from conftest import reference_tree

HERE = os.path.dirname(os.path.abspath(__file__))
REF = reference_tree()


def golden():
    rows = []
    for ln in open(os.path.join(HERE, "golden", "cpi_pi.txt")):
        if ln.startswith("#") or not ln.strip():
            continue
        key, line = ln.rstrip("\n").split(" | ")
        n, ranks = map(int, key.split())
        rows.append((n, ranks, line))
    return rows


@pytest.mark.parametrize("n,ranks,line", golden())
def test_oracle_pi_matches_reference_program(oracle_built, n, ranks, line):
    res = oracle_built.run_oracle("pi", [str(n)], nranks=ranks, timeout=300)
    assert res.returncode == 0, res.stderr
    assert res.lines("pi is approximately") == [line]


@pytest.mark.skipif(REF is None, reason="reference tree absent")
def test_fixture_reproduces_from_reference_source():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "golden", "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    with tempfile.TemporaryDirectory() as d:
        lines = mod.run_cases(mod.build_cpi(REF, d))
    assert lines == [f"{n} {r} | {line}" for n, r, line in golden()]
