"""GPU tests of the learned pair selector: gradients against the numpy
oracle, inference against the oracle forward, training data (logged
children, features, binding-pair labels against the CPU oracle), training,
and the search with the learned K-pair test giving the plain search's tree."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import wsbb_gb300 as W
    from wsbb_gb300 import explorer as E
    from wsbb_gb300 import learned as Lr
    return torch, W, E, Lr


def random_batch(torch, D, P, B, seed):
    rng = np.random.default_rng(seed)
    X = rng.uniform(0, 1.2, (B, D)).astype(np.float32)
    X[:, 40:] = rng.integers(0, 2, (B, D - 40))
    y = rng.integers(0, P, B).astype(np.int32)
    y[::17] = -1
    return X, y


def test_gradients_match_oracle(env):
    torch, W, E, Lr = env
    from oracle import mlp_oracle as M
    model = Lr.Model(50, 20, seed=3)
    X, y = random_batch(torch, model.D, model.P, 256, 0)
    X = M.bf16(X).astype(np.float32)
    dX, dy = torch.from_numpy(X).cuda(), torch.from_numpy(y).cuda()
    g, loss = model.grads(dX.data_ptr(), dy.data_ptr(), len(X))
    wl, gw = M.loss_and_grads(model.get_weights().astype(np.float64), model.D, model.O, model.P,
                              X, y)
    assert abs(loss - wl) <= 1e-3 * abs(wl)
    # fp32 accumulation vs float64: element error bounded relative to the
    # gradient's scale (a bf16 rounding of an activation may flip)
    err = np.abs(g - gw)
    assert np.linalg.norm(g - gw) <= 2e-3 * np.linalg.norm(gw)
    assert err.max() <= 2e-2 * np.abs(gw).max()


def test_inference_matches_oracle_forward(env):
    torch, W, E, Lr = env
    from oracle import mlp_oracle as M
    model = Lr.Model(50, 20, seed=4)
    X, _ = random_batch(torch, model.D, model.P, 333, 1)
    X = M.bf16(X).astype(np.float32)
    dX = torch.from_numpy(X).cuda()
    K = 8
    topk = torch.empty((len(X), K), dtype=torch.int16, device="cuda")
    logits = torch.empty((len(X), model.O), dtype=torch.float32, device="cuda")
    model.topk(dX.data_ptr(), len(X), K, topk.data_ptr(), logits.data_ptr())
    torch.cuda.synchronize()
    _, _, _, Z = M.forward(M.unpack(model.get_weights(), model.D, model.O), X)
    got = logits.cpu().numpy()
    assert np.abs(got - Z).max() <= 2e-2 * np.abs(Z).max()
    tk = topk.cpu().numpy()
    assert (tk >= 0).all() and (tk < model.P).all()
    # the first choice is the oracle's argmax except on near ties
    arg = Z[:, :model.P].argmax(1)
    assert np.mean(tk[:, 0] == arg) > 0.97
    for row in tk:
        assert len(set(row.tolist())) == K


def test_logged_nodes_and_labels_match_oracle(env, oracle):
    torch, W, E, Lr = env
    n, m = 20, 10
    p = W.gen_instance(5, n, m)
    ctx = W.Context(p)
    ub, _ = W.neh(p)
    cap = 20000
    recs = torch.empty((cap, ctx.stride), dtype=torch.uint8, device="cuda")
    got, st = Lr.log_nodes(ctx, recs.data_ptr(), cap, stride=3, ub0=ub, max_iters=64)
    assert 0 < got <= cap
    D = (3 * m + n + 15) // 16 * 16
    X = torch.empty((got, D), dtype=torch.float32, device="cuda")
    y = torch.empty(got, dtype=torch.int32, device="cuda")
    Lr.features(ctx, recs.data_ptr(), got, D, X.data_ptr(), y.data_ptr())
    torch.cuda.synchronize()
    r = recs[:got].cpu().numpy().view(np.int16).reshape(got, -1)
    perms, l1, l2 = W.unpack_records(r, n)
    lb, arg = oracle.Bound(p).eval_batch(perms, l1, l2, want_argmax=True)
    yy = y.cpu().numpy()
    leaf = (l2 - l1) == 1
    np.testing.assert_array_equal(yy[~leaf], arg[~leaf])
    assert (yy[leaf] == -1).all()
    Xn = X.cpu().numpy()
    # mask features: 1 exactly on the free jobs
    for i in range(0, got, max(1, got // 50)):
        free = set(perms[i][l1[i] + 1:l2[i]].tolist())
        assert set(np.nonzero(Xn[i, 3 * m:3 * m + n])[0].tolist()) == free


def trained_model(torch, W, Lr, n, m, seeds, per_seed=20000, epochs=4):
    """Log children of plain searches on `seeds`, train a model on them."""
    D = (3 * m + n + 15) // 16 * 16
    Xs, ys = [], []
    for s in seeds:
        p = W.gen_instance(s, n, m)
        ctx = W.Context(p)
        ub, _ = W.neh(p)
        recs = torch.empty((per_seed, ctx.stride), dtype=torch.uint8, device="cuda")
        got, _ = Lr.log_nodes(ctx, recs.data_ptr(), per_seed, stride=5, ub0=ub, max_iters=200)
        X = torch.empty((got, D), dtype=torch.float32, device="cuda")
        y = torch.empty(got, dtype=torch.int32, device="cuda")
        Lr.features(ctx, recs.data_ptr(), got, D, X.data_ptr(), y.data_ptr())
        Xs.append(X)
        ys.append(y)
    X = torch.cat(Xs)
    y = torch.cat(ys)
    torch.cuda.synchronize()
    model = Lr.Model(n, m, seed=11)
    losses = model.train(X.data_ptr(), y.data_ptr(), len(y), epochs=epochs, batch=1024,
                         lr=2e-3)
    return model, losses, X, y


def test_training_lowers_the_loss(env):
    torch, W, E, Lr = env
    model, losses, X, y = trained_model(torch, W, Lr, 20, 10, seeds=range(100, 104))
    assert losses[-1] < losses[0]
    # top-8 of the trained model holds the binding pair for most nodes
    K = 8
    tk = torch.empty((len(y), K), dtype=torch.int16, device="cuda")
    model.topk(X.data_ptr(), len(y), K, tk.data_ptr())
    torch.cuda.synchronize()
    yy = y.cpu().numpy()
    hit = (tk.cpu().numpy() == yy[:, None]).any(1)[yy >= 0].mean()
    assert hit > 0.5


def test_learned_search_keeps_the_tree(env):
    """Same counters and optimum as the plain search with the same `best`,
    with a share of children settled by the K ranked pairs."""
    torch, W, E, Lr = env
    model, _, _, _ = trained_model(torch, W, Lr, 20, 10, seeds=range(100, 103), epochs=3)
    for seed in (0, 1, 2):
        p = W.gen_instance(seed, 20, 10)
        ctx = W.Context(p)
        ub, _ = W.neh(p)
        plain = E.explore(ctx, ub0=ub, best=ub, window=2048)
        for K in (4, 8):
            for per_child in (False, True):
                got = Lr.explore_learned(ctx, model, K, ub0=ub, best=ub, window=2048,
                                         child_lb2=per_child)
                for k in ("branched", "pruned", "leaves", "improved", "bounded", "best_cost",
                          "coverage", "status"):
                    assert got[k] == plain[k], (seed, K, per_child, k)
                assert got["early"] > 0
    # and against the oracle's sequential search with the same best
    from oracle import oracle as O
    p = W.gen_instance(1, 20, 10)
    ub, _ = W.neh(p)
    rc, want, _ = O.Bound(p).explore(ub0=ub, best=ub)
    got = Lr.explore_learned(W.Context(p), model, 8, ub0=ub, best=ub, window=512)
    for k in ("branched", "pruned", "leaves", "improved", "bounded"):
        assert got[k] == want[k], k


def test_training_gains_early_settles(env):
    """What training gains over the method without it: the same network at
    its seeded initial weights ranks pairs too, and settles fewer children
    with its K pairs than after training; both leave the tree unchanged."""
    torch, W, E, Lr = env
    trained, _, _, _ = trained_model(torch, W, Lr, 20, 10, seeds=range(100, 103), epochs=3)
    start = Lr.Model(20, 10, seed=11)          # trained_model's initial weights
    p = W.gen_instance(0, 20, 10)
    ctx = W.Context(p)
    ub, _ = W.neh(p)
    for K in (4, 8):
        a = Lr.explore_learned(ctx, trained, K, ub0=ub, best=ub, window=2048, child_lb2=True)
        b = Lr.explore_learned(ctx, start, K, ub0=ub, best=ub, window=2048, child_lb2=True)
        for k in ("branched", "pruned", "bounded", "best_cost"):
            assert a[k] == b[k], (K, k)
        assert a["early"] > b["early"], (K, a["early"], b["early"])


def test_model_rejects_mismatched_instance(env):
    torch, W, E, Lr = env
    model = Lr.Model(20, 10)
    ctx = W.Context(W.gen_instance(0, 20, 5))
    with pytest.raises(W.WsbbError):
        Lr.explore_learned(ctx, model, 4, ub0=2000)
