"""Known-answer scenarios restated from the reference's own tests.

(program, scenario, ranks): tests/cuda_mpi_test.cu, tests/communicator_test.cu,
tests/collectives_test.cu and toolchain_tests/global_var/global_var.c, with the
rank counts those tests use, plus scenarios for calls the reference stubs.
"""

KAT_CASES = [
    ("kat_p2p", "single_int", 2),
    ("kat_p2p", "array16", 2),
    ("kat_p2p", "sendrecv", 2),
    ("kat_p2p", "repeat_sizes", 2),
    ("kat_p2p", "flood", 3),
    ("kat_p2p", "all_to_all", 10),
    ("kat_p2p", "a2a_ids", 10),
    ("kat_p2p", "wildcard", 5),
    ("kat_p2p", "probe_order", 2),
    ("kat_p2p", "large", 4),
    ("kat_p2p", "completion", 4),
    ("kat_p2p", "self_comm", 4),
    ("kat_p2p", "split_p2p", 6),
    ("kat_p2p", "split_p2p", 9),
    ("kat_p2p", "posted_order", 2),
    ("kat_p2p", "posted_order", 3),
    ("kat_p2p", "tiny_stream", 2),
    ("kat_p2p", "tiny_stream", 5),
    ("kat_coll", "reduce_prod", 5),
    ("kat_coll", "allreduce_sum", 7),
    ("kat_coll", "allgather", 7),
    ("kat_coll", "scatter", 5),
    ("kat_coll", "scatterv", 5),
    ("kat_coll", "comm_rank", 5),
    ("kat_coll", "comm_dup_traffic", 2),
    ("kat_coll", "comm_split", 10),
    ("kat_coll", "extras", 7),
    ("kat_coll", "extras", 1),
    ("kat_coll", "extras", 16),
    ("kat_coll", "groups_cart", 6),
    ("kat_coll", "groups_cart", 12),
    ("kat_coll", "user_op", 1),
    ("kat_coll", "user_op", 6),
    ("kat_coll", "user_op", 33),
    ("kat_coll", "parfor", 4),
    ("kat_global", None, 4),
]


def check_all_ok(res, scenario_name, nranks):
    assert res.returncode == 0, (res.returncode, res.stdout[-2000:], res.stderr[-2000:])
    lines = [ln for ln in res.stdout.splitlines() if " rank " in ln and " ok " in ln]
    assert len(lines) == nranks, res.stdout
    bad = [ln for ln in lines if not ln.endswith("ok 1")]
    assert not bad, bad
