"""The resident search (wsbb_explore_resident): one cooperative launch of
resident CTAs, a group per instance, fathers stolen between CTAs and from
the instances still running. Its trees must be the graph-launched search's
exactly, alone and with many instances in one launch, and a wait between
CTAs that runs out must end the launch with WSBB_ERR_WATCHDOG."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEYS = ("branched", "pruned", "leaves", "improved", "bounded", "best_cost", "coverage",
        "takes", "pending")


@pytest.fixture(scope="module")
def W():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import wsbb_gb300
    from wsbb_gb300 import explorer
    wsbb_gb300.lib()
    return wsbb_gb300, explorer


def same(got, want, tag):
    for k in KEYS:
        assert got[k] == want[k], f"{tag}: {k} {got[k]} != {want[k]}"
    np.testing.assert_array_equal(got["best_perm"], want["best_perm"], err_msg=tag)


@pytest.mark.parametrize("n,m,seed,best_ub", [(16, 10, 2, False), (18, 8, 5, True),
                                              (50, 5, 32, False), (50, 10, 9, True),
                                              (50, 10, 1, False)])
def test_resident_single_instance_proof(W, oracle, n, m, seed, best_ub):
    Wm, E = W
    p = Wm.gen_instance(seed, n, m)
    neh, _ = Wm.neh(p)
    best = neh if best_ub else 99999
    ctx = Wm.Context(p)
    want = E.explore(ctx, ub0=neh, best=best, window=1024)
    for window in (64, 1024):
        got = E.explore(ctx, ub0=neh, best=best, window=window, resident=True)
        assert got["status"] == 0
        same(got, want, f"n{n} m{m} s{seed} w={window}")
    assert want["coverage"] == math.factorial(n)


def test_resident_headline_prefix_equals_graph_search(W):
    """The headline instance stopped after the same number of iterations:
    the same exact prefix as the graph-launched search."""
    Wm, E = W
    p = Wm.gen_instance(0, 50, 20)
    neh, _ = Wm.neh(p)
    ctx = Wm.Context(p)
    for iters in (40, 200):
        want = E.explore(ctx, ub0=neh, best=neh, window=4096, graph_iters=1, max_iters=iters)
        got = E.explore(ctx, ub0=neh, best=neh, window=4096, max_iters=iters, resident=True)
        assert got["status"] == want["status"] == 1
        assert got["iterations"] == want["iterations"] == iters
        same(got, want, f"headline {iters} iterations")


def test_resident_many_instances_one_launch(W):
    """Twelve mixed instances (n 16 to 100, m 5 to 20) in one launch: those
    that finish equal their own graph-launched searches, the others stop at
    the same iteration count with the same prefix."""
    Wm, E = W
    shapes = [(16, 10, 2), (18, 8, 5), (20, 5, 7), (50, 5, 32), (50, 10, 9), (50, 10, 7),
              (50, 20, 0), (100, 20, 1), (100, 10, 2), (20, 20, 3), (100, 5, 4), (30, 8, 1)]
    ctxs, ubs, wants = [], [], []
    for n, m, s in shapes:
        p = Wm.gen_instance(s, n, m)
        neh, _ = Wm.neh(p)
        ctx = Wm.Context(p)
        ctxs.append(ctx)
        ubs.append(neh)
        wants.append(E.explore(ctx, ub0=neh, best=neh, window=512, graph_iters=1,
                               max_iters=300))
    rc, got = E.explore_resident(ctxs, ub0s=ubs, bests=ubs, window=512, max_iters=300)
    assert rc == 0
    finished = 0
    for (n, m, s), g, w in zip(shapes, got, wants):
        assert g["status"] == w["status"], (n, m, s)
        same(g, w, f"n{n} m{m} s{s}")
        finished += g["status"] == 0
    assert 0 < finished < len(shapes)


def test_resident_small_groups_and_free_thieves(W):
    """Groups capped below an equal share (group_ctas): the CTAs outside
    every group only take fathers from the bound phases, and the trees stay
    the graph-launched search's."""
    Wm, E = W
    p = Wm.gen_instance(9, 50, 10)
    neh, _ = Wm.neh(p)
    ctx = Wm.Context(p)
    want = E.explore(ctx, ub0=neh, best=neh, window=1024)
    rc, got = E.explore_resident([ctx], ub0s=[neh], bests=[neh], window=1024, group_ctas=4)
    assert rc == 0 and got[0]["status"] == 0
    same(got[0], want, "one instance, groups of 4")
    shapes = [(16, 10, 2), (20, 5, 7), (50, 5, 32), (50, 20, 0), (100, 10, 2)]
    ctxs, ubs, wants = [], [], []
    for n, m, sd in shapes:
        q = Wm.gen_instance(sd, n, m)
        ub, _ = Wm.neh(q)
        c = Wm.Context(q)
        ctxs.append(c)
        ubs.append(ub)
        wants.append(E.explore(c, ub0=ub, best=ub, window=512, graph_iters=1, max_iters=200))
    rc, got = E.explore_resident(ctxs, ub0s=ubs, bests=ubs, window=512, max_iters=200,
                                 group_ctas=2)
    assert rc == 0
    for (n, m, sd), g, w in zip(shapes, got, wants):
        assert g["status"] == w["status"], (n, m, sd)
        same(g, w, f"n{n} m{m} s{sd}, groups of 2")


def test_resident_watchdog_ends_the_launch(W):
    """A wait that nothing ends (the self-test flag) runs out after its
    limit: the launch ends with WSBB_ERR_WATCHDOG, and the contexts run a
    normal search afterwards."""
    Wm, E = W
    ctxs = [Wm.Context(Wm.gen_instance(s, 16, 5)) for s in (1, 2, 3)]
    rc, st = E.explore_resident(ctxs, window=64, wait_ms=50, self_test=True, check=False)
    assert rc == -5
    assert all(x["status"] == -5 for x in st)
    rc, st = E.explore_resident(ctxs, window=64)
    assert rc == 0 and all(x["status"] == 0 for x in st)
    for c, x in zip(ctxs, st):
        want = E.explore(c, window=64)
        same(x, want, "after the watchdog")
