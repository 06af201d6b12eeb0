"""The library's hand-off entry points on the GPU: a stopped search resumes
to exactly the uninterrupted search's tree; open nodes exported from one
search and seeded into another cover the tree once between them; and
GpuEngine peers (threads, one context each) share a search to the optimum."""
import math
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def W():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import wsbb_gb300
    return wsbb_gb300


KEYS = ("branched", "pruned", "leaves", "improved", "bounded", "best_cost", "coverage")


def test_resumed_search_equals_uninterrupted(W):
    from wsbb_gb300.explorer import explore
    n, m = 14, 6
    p = W.gen_instance(2, n, m)
    ub, _ = W.neh(p)
    ctx = W.Context(p)
    whole = explore(ctx, ub0=ub, window=256)
    # the budget is checked between graph launches: one iteration each
    kw = dict(ub0=ub, window=256, graph_iters=1)
    st = explore(ctx, **kw, max_bounded=3000)
    stops = 0
    while st["status"] == 1:
        stops += 1
        st = explore(ctx, **kw, resume=True, max_bounded=st["bounded"] + 3000)
    assert stops > 2
    assert {k: st[k] for k in KEYS} == {k: whole[k] for k in KEYS}
    assert st["best_perm"].tolist() == whole["best_perm"].tolist()
    assert st["coverage"] == math.factorial(n)


def test_exported_nodes_seed_another_search(W):
    from wsbb_gb300.explorer import explore, explore_export, explore_seed
    n, m = 14, 6
    p = W.gen_instance(2, n, m)
    opt = explore(W.Context(p))["best_cost"]
    a, b = W.Context(p), W.Context(p)
    st = explore(a, ub0=opt, window=64, graph_iters=1, max_iters=6)
    assert st["status"] == 1
    rec, lbs = explore_export(a, 64)
    assert 0 < len(rec) <= 64 and (lbs < opt).all()
    # exported records are open nodes of the instance, shallowest first
    depth = rec[:, n + 2].astype(int)
    assert (np.diff(depth) >= 0).sum() >= len(depth) // 2
    for r in rec:
        assert sorted(r[:n].tolist()) == list(range(n))
    explore_seed(b, rec, lbs, ub0=opt, window=64)
    sb = explore(b, ub0=opt, window=64, resume=True)
    sa = explore(a, ub0=opt, window=64, resume=True)
    assert sa["status"] == 0 and sb["status"] == 0
    assert sa["coverage"] + sb["coverage"] == math.factorial(n)
    # a resumed search with nothing left to do stops at once
    again = explore(a, ub0=opt, window=64, resume=True)
    assert again["branched"] == sa["branched"] and again["status"] == 0


def test_seed_rejects_records_that_are_not_open_nodes(W):
    from wsbb_gb300 import WsbbError
    from wsbb_gb300.explorer import explore_seed
    n = 10
    ctx = W.Context(W.gen_instance(1, n, 4))
    rec = W.pack_records(np.arange(n)[None, :], [-1], [n])
    bad = rec.copy()
    bad[0, 3] = bad[0, 4]                      # a repeated job
    with pytest.raises(WsbbError):
        explore_seed(ctx, bad, [0], ub0=1000, window=256)
    leaf = W.pack_records(np.arange(n)[None, :], [n - 2], [n])  # one free job
    with pytest.raises(WsbbError):
        explore_seed(ctx, leaf, [0], ub0=1000, window=256)
    explore_seed(ctx, rec, [0], ub0=1000, window=256)   # the root is fine


def test_gpu_peers_share_a_search(W):
    from wsbb_gb300 import peers
    from wsbb_gb300.explorer import explore
    n, m = 16, 6
    p = W.gen_instance(2, n, m)
    ref = explore(W.Context(p), window=256)
    for ub0 in (None, ref["best_cost"]):
        hub = peers.LocalHub(2)
        out = [None, None]
        err = []

        def run(r):
            try:
                eng = peers.GpuEngine(W.Context(p), window=64, graph_iters=1)
                out[r] = peers.peer_search(eng, peers.LocalTransport(hub, r), n, ub0=ub0,
                                           budget=4, share=16)
            except Exception as e:  # reported below
                err.append(e)
                hub.barrier.abort()

        th = [threading.Thread(target=run, args=(r,)) for r in range(2)]
        for t in th:
            t.start()
        for t in th:
            t.join(timeout=600)
        assert not err, err
        assert out[0].best_cost == out[1].best_cost == ref["best_cost"]
        assert out[0].sent + out[1].sent > 0
        assert out[0].counters["branched"] > 0 and out[1].counters["branched"] > 0
        if ub0 is None:
            assert out[0].best_perm.tolist() == out[1].best_perm.tolist()
            from oracle import oracle
            assert oracle.Bound(p).makespan(out[0].best_perm) == ref["best_cost"]
        else:
            # no incumbent moves: no branched node is pruned later, so the
            # peers' subtrees partition the tree
            assert out[0].total_coverage == math.factorial(n)
