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


@pytest.mark.parametrize("pattern,mode,ranks", [("pairs", "block", 4), ("ring", "block", 5), ("ring", "nb", 3)])
def test_oracle_p2p_sweep_self_checks(oracle_built, pattern, mode, ranks):
    """The sweep verifies every payload itself; blocking and non-blocking forms
    deliver the same bytes, so their checksums agree."""
    res = oracle_built.run_oracle("p2p_sweep", [pattern, mode, "3", "15", "4"], nranks=ranks, timeout=120)
    assert res.returncode == 0, res.stderr
    lines = res.lines("p2p ")
    assert len(lines) == 13 and all(" errors 0 " in ln for ln in lines)
    other = "nb" if mode == "block" else "block"
    res2 = oracle_built.run_oracle("p2p_sweep", [pattern, other, "3", "15", "4"], nranks=ranks, timeout=120)
    assert [ln.split(" checksum ")[1] for ln in res2.lines("p2p ")] == [ln.split(" checksum ")[1] for ln in lines]


@pytest.mark.parametrize("args,ranks", [(["16", "4"], 8), (["11", "3"], 5), (["9", "2"], 64)])
def test_oracle_is_sort_verifies(oracle_built, args, ranks):
    """The bucket sort's own full verification passes on the oracle (sorted
    within and across ranks, every key accounted for), also with ragged and
    nearly empty ranks."""
    res = oracle_built.run_oracle("is_sort", args, nranks=ranks, timeout=120)
    assert res.returncode == 0, res.stderr
    assert res.lines("is verify")[0].endswith("PASSED")
    assert len(res.lines("is iteration")) == int(args[1])


@pytest.mark.parametrize("ranks", [1, 2, 4, 8])
def test_oracle_pic_conserves(oracle_built, ranks):
    """PIC on the oracle: migration keeps every particle (count constant), the
    total energy drifts by less than 1 % over the run, the run is deterministic."""
    args = ["20", "32", "16", "20", "5"]
    a = oracle_built.run_oracle("pic", args, nranks=ranks, timeout=120)
    b = oracle_built.run_oracle("pic", args, nranks=ranks, timeout=120)
    assert a.returncode == 0, a.stderr
    lines = a.lines("pic cycle")
    assert len(lines) == 4
    counts = {int(ln.split()[4]) for ln in lines}
    assert counts == {32 * 16 * 20 * 2}
    totals = [sum(float(x) for x in ln.split()[6::2]) for ln in lines]
    assert max(totals) - min(totals) < 0.01 * totals[0]
    assert a.lines("pic ") == b.lines("pic ")


def test_oracle_allocator_known_answers(oracle_built):
    res = oracle_built.run_oracle("kat_malloc", [], nranks=3, timeout=120)
    assert res.returncode == 0, res.stderr
    assert sorted(res.lines("kat_malloc")) == [f"kat_malloc rank {r} ok" for r in range(3)]
