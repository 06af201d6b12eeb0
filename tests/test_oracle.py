"""The CPU oracle against the reference's own outputs (golden fixtures).

bound_pools.npz and explore.json were produced by the reference's compiled
bound_flowshop and CPU search (tests/golden/make_golden.py), so these tests
pin the oracle before anything else is checked against it.
"""
import math

import numpy as np
import pytest


def _cases(golden_pools):
    return sorted({k.rsplit("_", 1)[0] for k in golden_pools.files})


def test_oracle_bound_matches_reference(oracle, golden_pools):
    for key in _cases(golden_pools):
        p = golden_pools[key + "_p"].astype(np.int32)
        perms = golden_pools[key + "_perms"].astype(np.int32)
        l1 = golden_pools[key + "_l1"].astype(np.int32)
        l2 = golden_pools[key + "_l2"].astype(np.int32)
        want_lb = golden_pools[key + "_lb"]
        want_arg = golden_pools[key + "_argmax"]
        lb, arg = oracle.Bound(p).eval_batch(perms, l1, l2, want_argmax=True)
        np.testing.assert_array_equal(lb, want_lb, err_msg=key)
        leaf = (l2 - l1) == 1
        arg[leaf] = -1
        np.testing.assert_array_equal(arg, want_arg, err_msg=key + " binding pair")


def test_generator_matches_fixture_instances(oracle, golden_pools):
    for key in _cases(golden_pools):
        n, m, s = (int(t[1:]) for t in key.split("_"))
        np.testing.assert_array_equal(oracle.gen_instance(s, n, m),
                                      golden_pools[key + "_p"].astype(np.int32))


def test_oracle_search_matches_reference(oracle, golden_explore):
    for run in golden_explore:
        p = oracle.gen_instance(run["seed"], run["n"], run["m"])
        neh, _ = oracle.neh(p)
        assert neh == run["neh"]
        rc, st, perm = oracle.Bound(p).explore(ub0=run["ub0"], best=run["best"])
        assert rc == 0
        tag = f"n{run['n']} m{run['m']} s{run['seed']} ub0={run['ub0']} best={run['best']}"
        for k in ("branched", "pruned", "leaves", "improved", "bounded"):
            assert st[k] == run[k], f"{tag}: {k}"
        assert st["best_cost"] == run["optimum"], tag
        assert str(st["coverage"]) == run["coverage"], tag
        if run["perm"] is not None:
            assert list(perm) == run["perm"], tag


def test_oracle_search_matches_reference_above_n20(oracle):
    """The reference's own search rebuilt for n <= 64 (explore_big.json):
    n = 30 to 50, up to 530k child bounds per run — every counter, the
    optimum, its permutation and coverage = n!."""
    import json
    import os
    with open(os.path.join(os.path.dirname(__file__), "golden", "explore_big.json")) as f:
        runs = json.load(f)["runs"]
    assert max(r["n"] for r in runs) == 50 and len(runs) >= 20
    for run in runs:
        p = oracle.gen_instance(run["seed"], run["n"], run["m"])
        assert oracle.neh(p)[0] == run["neh"]
        rc, st, perm = oracle.Bound(p).explore(ub0=run["ub0"], best=run["best"])
        tag = f"n{run['n']} m{run['m']} s{run['seed']} best={run['best']}"
        assert rc == 0, tag
        for k in ("branched", "pruned", "leaves", "improved", "bounded"):
            assert st[k] == run[k], f"{tag}: {k}"
        assert st["best_cost"] == run["optimum"], tag
        assert str(st["coverage"]) == run["coverage"] == str(math.factorial(run["n"])), tag
        if run["perm"] is not None:
            assert list(perm) == run["perm"], tag


def test_coverage_is_n_factorial(oracle, golden_explore):
    import math
    for run in golden_explore:
        assert int(run["coverage"]) == math.factorial(run["n"])


def test_lb_is_a_lower_bound_on_completions(oracle):
    """Every leaf under a node costs at least the node's LB2 (small instance,
    all completions enumerated)."""
    import itertools
    n, m = 7, 4
    p = oracle.gen_instance(11, n, m)
    b = oracle.Bound(p)
    rng = np.random.default_rng(0)
    for _ in range(20):
        perm = rng.permutation(n).astype(np.int32)
        f = int(rng.integers(0, n - 2))
        bk = int(rng.integers(0, n - 2 - f))
        l1, l2 = f - 1, n - bk
        lb, _ = b.eval(perm, l1, l2)
        free = list(perm[l1 + 1:l2])
        best = min(b.makespan(np.concatenate([perm[:l1 + 1], list(q), perm[l2:]]).astype(np.int32))
                   for q in itertools.permutations(free))
        assert lb <= best


def test_early_exit_pair_subset_keeps_tree(oracle):
    """A per-child pair subset settled against best = UB0 leaves the search
    tree unchanged (same counters as the plain search with the same best)."""
    p = oracle.gen_instance(0, 20, 5)
    ub, _ = oracle.neh(p)
    b = oracle.Bound(p)
    rc, plain, perm_plain = b.explore(ub0=ub, best=ub)

    def sel(perm, l1, l2, out, user):
        out[0] = 0
        out[1] = 3
        out[2] = 9
        return 3

    rc2, fast, perm_fast = b.explore(ub0=ub, best=ub, pair_sel=sel)
    for k in ("branched", "pruned", "leaves", "improved", "bounded", "best_cost"):
        assert plain[k] == fast[k], k
    assert fast["early_exits"] > 0
    assert list(perm_plain) == list(perm_fast)


@pytest.mark.skipif("not __import__('oracle.oracle', fromlist=['x']).have_reference()")
def test_reference_harness_live(oracle):
    """Where the reference is built (this container), re-run it live."""
    p = oracle.gen_instance(3, 9, 4)
    ub, _ = oracle.neh(p)
    r = oracle.ref_explore(p, ub0=ub, best=99999)
    rc, st, _ = oracle.Bound(p).explore(ub0=ub)
    assert (st["branched"], st["pruned"], st["leaves"], st["best_cost"]) == (
        r["branched"], r["pruned"], r["leaves"], r["optimum"])
    perms, l1, l2 = oracle.random_pool(5, 9, 500, 0.1)
    np.testing.assert_array_equal(oracle.Bound(p).eval_batch(perms, l1, l2),
                                  oracle.RefBound(p).eval_batch(perms, l1, l2))


@pytest.mark.skipif("not __import__('oracle.oracle', fromlist=['x']).have_reference()")
def test_oracle_matches_the_reference_on_a_sweep(oracle):
    """Where the reference is built: searches over sizes n = 8..16, m = 2..8,
    with no incumbent, the NEH incumbent, and best = the NEH cost — every
    counter, the optimum, its permutation and the coverage equal the
    reference's own run; and bounds of random pools up to n = 40."""
    for s, n, m in [(1, 8, 3), (2, 10, 4), (3, 12, 5), (4, 14, 3), (5, 11, 6), (6, 16, 4),
                    (7, 9, 8), (8, 13, 2)]:
        p = oracle.gen_instance(s, n, m)
        ub, _ = oracle.neh(p)
        for ub0, best in ((None, 99999), (ub, 99999), (ub, ub)):
            r = oracle.ref_explore(p, ub0=ub0, best=best)
            rc, st, perm = oracle.Bound(p).explore(ub0=ub0, best=best)
            assert rc == 0
            tag = (s, n, m, ub0, best)
            for k in ("branched", "pruned", "leaves", "improved", "bounded"):
                assert st[k] == r[k], (tag, k)
            assert st["best_cost"] == r["optimum"], tag
            assert st["coverage"] == int(r["coverage"]) == math.factorial(n), tag
            if st["improved"]:
                assert list(perm) == list(r["perm"]), tag
    for s, n, m in [(11, 25, 5), (12, 33, 7), (13, 40, 12)]:
        p = oracle.gen_instance(s, n, m)
        perms, l1, l2 = oracle.random_pool(s, n, 400, 0.1)
        np.testing.assert_array_equal(oracle.Bound(p).eval_batch(perms, l1, l2),
                                      oracle.RefBound(p).eval_batch(perms, l1, l2))


@pytest.mark.skipif("not __import__('oracle.oracle', fromlist=['x']).have_reference_big()")
def test_oracle_matches_the_reference_above_n20_live(oracle):
    """Where the reference is built: its search compiled for n <= 64, run
    live at n = 25 to 50 next to the oracle."""
    for s, n, m in [(5, 45, 7), (8, 50, 5), (9, 50, 10), (2, 26, 4)]:
        p = oracle.gen_instance(s, n, m)
        ub, _ = oracle.neh(p)
        for best in (99999, ub):
            r = oracle.ref_explore(p, ub0=ub, best=best)
            rc, st, perm = oracle.Bound(p).explore(ub0=ub, best=best, node_cap=2_000_000)
            assert rc == 0
            for k in ("branched", "pruned", "leaves", "improved", "bounded"):
                assert st[k] == r[k], (s, n, m, best, k)
            assert st["best_cost"] == r["optimum"]
            assert st["coverage"] == int(r["coverage"]) == math.factorial(n)
            if st["improved"]:
                assert list(perm) == list(r["perm"])
