"""The CPU oracle (hostmpi) is pinned against the reference's known answers."""
import pytest

from kat_cases import KAT_CASES, check_all_ok


@pytest.mark.parametrize("prog,scenario,nranks", KAT_CASES)
def test_oracle_known_answers(oracle_built, prog, scenario, nranks):
    args = [scenario] if scenario else []
    res = oracle_built.run_oracle(prog, args, nranks=nranks, timeout=120)
    check_all_ok(res, scenario, nranks)


def test_oracle_pi_rank_order(oracle_built):
    """pi with a rank-order reduction is deterministic and accurate."""
    a = oracle_built.run_oracle("pi", ["1000000"], nranks=8)
    b = oracle_built.run_oracle("pi", ["1000000"], nranks=8)
    assert a.returncode == 0
    assert a.lines("pi bits") == b.lines("pi bits")
    val = float(a.lines("pi is approximately")[0].split()[3].rstrip(","))
    assert abs(val - 3.141592653589793) < 1e-10
