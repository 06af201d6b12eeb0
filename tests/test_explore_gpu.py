"""GPU search parity: the exact DFS on the device against the reference's
recorded search (tests/golden/explore.json) and against the oracle's
sequential search, with windows from 1 (one node per iteration) up, so
that speculative branching, invalidation after incumbent improvements and
the graph / non-graph paths are all exercised."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEYS = ("branched", "pruned", "leaves", "improved", "bounded")


@pytest.fixture(scope="module")
def W():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import wsbb_gb300
    from wsbb_gb300 import explorer
    wsbb_gb300.lib()
    return wsbb_gb300, explorer


def check_equal(got, want, tag):
    for k in KEYS:
        assert got[k] == want[k], f"{tag}: {k} {got[k]} != {want[k]}"
    assert got["best_cost"] == want["best_cost"], tag
    assert got["coverage"] == want["coverage"], tag
    assert got["status"] == 0, tag


def test_search_matches_reference_golden(W, golden_explore):
    Wm, E = W
    for run in golden_explore:
        p = Wm.gen_instance(run["seed"], run["n"], run["m"])
        ctx = Wm.Context(p)
        for window in (1, 64, 4096):
            got = E.explore(ctx, ub0=run["ub0"], best=run["best"], window=window)
            want = dict(run, best_cost=run["optimum"], coverage=int(run["coverage"]))
            tag = f"n{run['n']} m{run['m']} s{run['seed']} ub0={run['ub0']} best={run['best']} w={window}"
            check_equal(got, want, tag)
            if run["perm"] is not None:
                assert list(got["best_perm"]) == run["perm"], tag
            assert got["coverage"] == math.factorial(run["n"])


@pytest.mark.parametrize("n,m,seed", [(12, 5, 3), (14, 10, 4), (11, 20, 5), (16, 5, 6),
                                      (20, 5, 7), (20, 10, 8), (13, 3, 9)])
def test_search_matches_oracle(W, oracle, n, m, seed):
    Wm, E = W
    p = Wm.gen_instance(seed, n, m)
    neh, _ = Wm.neh(p)
    ctx = Wm.Context(p)
    ob = oracle.Bound(p)
    for ub0, best in ((None, 99999), (neh, 99999), (neh, neh)):
        rc, want, perm = ob.explore(ub0=ub0, best=best)
        want = dict(want)
        for window, graph in ((3, False), (17, True), (1024, True)):
            got = E.explore(ctx, ub0=ub0, best=best, window=window, graph=graph,
                            graph_iters=5)
            tag = f"n{n} m{m} s{seed} ub0={ub0} best={best} w={window}"
            check_equal(got, want, tag)
            if want["improved"]:
                np.testing.assert_array_equal(got["best_perm"], perm, err_msg=tag)
            assert got["evaluated"] >= got["bounded"]


def test_iteration_cap_reports_status(W):
    Wm, E = W
    p = Wm.gen_instance(1, 16, 5)
    ctx = Wm.Context(p)
    got = E.explore(ctx, window=2, max_iters=4, graph_iters=2)
    assert got["status"] == 1
    assert got["iterations"] <= 4


def test_capacity_error_is_reported(W):
    """No incumbent: a 4096-wide expansion outgrows a stack sized to the
    minimum (one rewrite region) within a few iterations; the search stops
    with the capacity error instead of writing past the stack."""
    Wm, E = W
    p = Wm.gen_instance(2, 20, 5)
    ctx = Wm.Context(p)
    with pytest.raises(Wm.WsbbError) as ei:
        E.explore(ctx, window=4096, capacity=16 * 4096 + 8192)
    assert ei.value.code == -6
    # the context stays usable
    got = E.explore(ctx, window=64)
    assert got["status"] == 0


def test_autotuned_shapes_keep_the_tree():
    """Every window / tile candidate of the autotuner explores the same tree."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import wsbb_gb300 as W
    from wsbb_gb300 import autotune as A
    from wsbb_gb300.explorer import explore
    p = W.gen_instance(2, 20, 10)
    ub, _ = W.neh(p)
    ctx = W.Context(p)
    choice, results = A.tune(ctx, ub, ub, iters=24, windows=(256, 2048), smem_kbs=(24, 56, 100))
    assert choice in results and len(results) == 6
    assert len({r["bounded"] for r in results if r["window"] == 2048}) == 1
    full = [explore(ctx, ub0=ub, best=ub, window=r["window"], family_smem_kb=r["family_smem_kb"])
            for r in results]
    keys = ("branched", "pruned", "leaves", "improved", "bounded", "best_cost", "coverage")
    assert all(all(f[k] == full[0][k] for k in keys) for f in full)


def test_concurrent_searches_on_many_contexts():
    """Searches on several contexts from several host threads at once (their
    graph captures overlap), and the same instances in one resident launch:
    every arm ends with the same trees."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from wsbb_gb300 import multi_bench
    out = multi_bench.run(instances=9, threads=3, cmp_budget=2 * 10**6, window=512,
                          arms=("resident", "family", "per_child"), full=False)
    for arm in ("resident", "family", "per_child"):
        a = out["arms"][arm]
        assert a["instances"] == 9 and a["same_tree"] and a["finished"], arm
    assert (out["arms"]["resident"]["bounded"] == out["arms"]["family"]["bounded"] ==
            out["arms"]["per_child"]["bounded"] > 0)


def test_node_budget_stops_the_search():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import wsbb_gb300 as W
    from wsbb_gb300.explorer import explore
    p = W.gen_instance(1, 20, 20)
    ub, _ = W.neh(p)
    ctx = W.Context(p)
    full = explore(ctx, ub0=ub)
    budget = full["bounded"] // 10
    for window in (1024, 8192):
        r = explore(ctx, ub0=ub, window=window, max_bounded=budget)
        assert r["status"] == 1 and budget <= r["bounded"] < full["bounded"]
