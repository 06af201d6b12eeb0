"""GPU search parity at n = 50 against the oracle's sequential search.

* The headline tree (n=50, m=20, seed 0, NEH incumbent): GPU searches
  stopped by a node budget report the exact sequential prefix they stand
  at (`takes`, with the children pruned at birth whose take is still ahead
  removed); the oracle, run for exactly that many takes, must give the
  same branched / pruned / leaves / improved / bounded counters, incumbent
  and coverage — with best = NEH and the reference default best = 99999,
  and at the bench's window as well as smaller ones.
* Complete proofs at n = 50 with m = 5 and m = 10 on instances whose trees
  the oracle finishes in seconds: every counter, the optimum, the optimal
  permutation and coverage = 50!; and the same against the reference's own
  search rebuilt for n <= 64 (tests/golden/explore_big.json).
* Complete proofs of deep subtrees of the headline instance, seeded into
  the GPU search and into the oracle alike.
* Prefixes of small searches (n = 13 to 18) stopped at many points and
  windows (cheap, broad).
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEYS = ("branched", "pruned", "leaves", "improved", "bounded", "best_cost")


@pytest.fixture(scope="module")
def W():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import wsbb_gb300
    from wsbb_gb300 import explorer
    wsbb_gb300.lib()
    return wsbb_gb300, explorer


def check_prefix(E, got, ob, n, ub0, best, tag):
    """The GPU stats `got` of a stopped search against the oracle run for
    exactly got["takes"] takes."""
    pre = E.sequential_prefix(got, n)
    assert pre["takes"] > 0, tag
    rc, want, _ = ob.explore(ub0=ub0, best=best, node_cap=pre["takes"])
    assert rc == 1, f"{tag}: the oracle finished before {pre['takes']} takes"
    for k in KEYS:
        assert pre[k] == want[k], f"{tag}: {k} {pre[k]} != oracle {want[k]}"
    assert pre["coverage"] == want["coverage"], f"{tag}: coverage"
    return pre


@pytest.mark.parametrize("best_mode,window,budget", [("neh", 2048, 600_000),
                                                     ("neh", 16384, 300_000),
                                                     ("default", 4096, 600_000)])
def test_headline_tree_prefix_matches_oracle(W, oracle, best_mode, window, budget):
    Wm, E = W
    n, m, seed = 50, 20, 0
    p = Wm.gen_instance(seed, n, m)
    neh, _ = Wm.neh(p)
    best = neh if best_mode == "neh" else 99999
    ctx = Wm.Context(p)
    got = E.explore(ctx, ub0=neh, best=best, window=window, graph_iters=1,
                    max_bounded=budget)
    assert got["status"] == 1
    pre = check_prefix(E, got, oracle.Bound(p), n, neh, best,
                       f"n50 m20 s0 best={best} w={window}")
    assert pre["bounded"] >= budget


@pytest.mark.parametrize("m,seed", [(5, 8), (5, 24), (5, 32), (5, 39),
                                    (10, 1), (10, 6), (10, 7), (10, 9)])
def test_n50_proof_matches_oracle(W, oracle, m, seed):
    Wm, E = W
    n = 50
    p = Wm.gen_instance(seed, n, m)
    neh, _ = Wm.neh(p)
    ob = oracle.Bound(p)
    ctx = Wm.Context(p)
    for best in (99999, neh):
        rc, want, perm = ob.explore(ub0=neh, best=best)
        assert rc == 0
        for window in (64, 4096):
            got = E.explore(ctx, ub0=neh, best=best, window=window)
            tag = f"n50 m{m} s{seed} best={best} w={window}"
            assert got["status"] == 0, tag
            for k in KEYS:
                assert got[k] == want[k], f"{tag}: {k} {got[k]} != {want[k]}"
            assert got["coverage"] == want["coverage"] == math.factorial(n), tag
            assert got["takes"] == want["branched"] + want["pruned"] + want["leaves"], tag
            assert got["pending"] == 0, tag
            if want["improved"]:
                np.testing.assert_array_equal(got["best_perm"], perm, err_msg=tag)


def test_search_matches_reference_above_n20(W):
    """The reference's own search rebuilt for n <= 64 (golden runs at n = 30
    to 50, tests/golden/explore_big.json) against the GPU search."""
    import json
    import os
    Wm, E = W
    with open(os.path.join(os.path.dirname(__file__), "golden", "explore_big.json")) as f:
        runs = json.load(f)["runs"]
    for run in runs:
        n = run["n"]
        p = Wm.gen_instance(run["seed"], n, run["m"])
        ctx = Wm.Context(p)
        for window in (128, 8192):
            got = E.explore(ctx, ub0=run["ub0"], best=run["best"], window=window)
            tag = f"n{n} m{run['m']} s{run['seed']} best={run['best']} w={window}"
            assert got["status"] == 0, tag
            for k in ("branched", "pruned", "leaves", "improved", "bounded"):
                assert got[k] == run[k], f"{tag}: {k} {got[k]} != {run[k]}"
            assert got["best_cost"] == run["optimum"], tag
            assert str(got["coverage"]) == run["coverage"], tag
            if run["perm"] is not None:
                assert list(got["best_perm"]) == run["perm"], tag


def _subtree_root(p, n, front, back):
    """A begin-end node fixing the NEH order's first `front` jobs at the
    front and its last `back` jobs at the back."""
    import wsbb_gb300 as Wm
    _, order = Wm.neh(p)
    perm = np.asarray(order, dtype=np.int32)
    rec = np.zeros(Wm.node_stride(n) // 2, dtype=np.int16)
    rec[:n] = perm
    rec[n] = front - 1
    rec[n + 1] = n - back
    rec[n + 2] = front + back
    return rec


@pytest.mark.parametrize("front,back,delta", [(17, 15, 20), (20, 10, 20), (19, 13, 60),
                                              (15, 15, -40)])
def test_headline_subtree_proofs_match_oracle(W, oracle, front, back, delta):
    """Deep subtrees of the headline instance (u = n - front - back free
    jobs), explored to the end from the same seeded node and incumbent
    (the NEH cost + delta: above it, leaves improve the incumbent; below
    it, the search proves that nothing in the subtree is that cheap)."""
    Wm, E = W
    n, m = 50, 20
    p = Wm.gen_instance(0, n, m)
    neh, _ = Wm.neh(p)
    ub0 = neh + delta
    ob = oracle.Bound(p)
    rec = _subtree_root(p, n, front, back)
    perm = rec[:n].astype(np.int32)
    lb, _ = ob.eval(perm, int(rec[n]), int(rec[n + 1]))
    assert lb < ub0
    ctx = Wm.Context(p)
    for best in (ub0, 99999):
        rc, want, wperm = ob.explore_seeded(perm[None, :], [rec[n]], [rec[n + 1]], [lb],
                                            ub0=ub0, best=best, node_cap=3_000_000)
        assert rc == 0, "oracle subtree too large for the test"
        for window in (256, 8192):
            E.explore_seed(ctx, rec[None, :], [lb], ub0=ub0, best=best, window=window)
            got = E.explore(ctx, ub0=ub0, best=best, window=window, resume=True)
            tag = f"subtree f{front} b{back} ub0={ub0} best={best} w={window}"
            assert got["status"] == 0, tag
            for k in KEYS:
                assert got[k] == want[k], f"{tag}: {k} {got[k]} != {want[k]}"
            assert got["coverage"] == want["coverage"] == math.factorial(n - front - back), tag
            if want["improved"]:
                np.testing.assert_array_equal(got["best_perm"], wperm, err_msg=tag)


@pytest.mark.parametrize("n,m,seed", [(16, 10, 2), (18, 8, 5), (13, 20, 2)])
def test_stopped_prefixes_match_oracle(W, oracle, n, m, seed):
    """Searches stopped at many node budgets and windows (one father per
    iteration up to wide windows) stand at exact sequential prefixes."""
    Wm, E = W
    p = Wm.gen_instance(seed, n, m)
    neh, _ = Wm.neh(p)
    ob = oracle.Bound(p)
    ctx = Wm.Context(p)
    for ub0, best in ((None, 99999), (neh, neh)):
        full = E.explore(ctx, ub0=ub0, best=best, window=256)
        assert full["pending"] == 0 and full["status"] == 0
        for frac in (0.05, 0.3, 0.7):
            budget = max(1, int(full["bounded"] * frac))
            for window in (1, 64, 1024):
                got = E.explore(ctx, ub0=ub0, best=best, window=window, graph_iters=1,
                                max_bounded=budget)
                if got["status"] == 0:
                    continue  # the budget fell inside the last iteration
                check_prefix(E, got, ob, n, ub0, best,
                             f"n{n} m{m} s{seed} ub0={ub0} best={best} w={window} f={frac}")
