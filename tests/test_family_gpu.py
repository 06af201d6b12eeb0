"""Family bounds (wsbb_decompose_lb2): every child's LB2 from its father,
bit-exact to the oracle's bound of the child record, and the search with
family bounds exploring the same tree as with per-child bounds."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import wsbb_gb300 as W
    return torch, W


def random_fathers(rng, n, count):
    """Father records with every cursor shape: the root, empty fronts or
    backs, two free jobs (leaf children) up to n free."""
    perms = np.array([rng.permutation(n) for _ in range(count)], dtype=np.int32)
    l1 = np.empty(count, np.int32)
    l2 = np.empty(count, np.int32)
    for i in range(count):
        kind = i % 6
        if kind == 0:                      # root
            a, u = -1, n
        elif kind == 1:                    # nothing at the back
            u = int(rng.integers(2, n + 1))
            a = n - 1 - u
        elif kind == 2:                    # nothing at the front
            a, u = -1, int(rng.integers(2, n + 1))
        elif kind == 3:                    # two free jobs: leaves
            a = int(rng.integers(-1, n - 2))
            u = 2
        else:
            a = int(rng.integers(-1, n - 2))
            u = int(rng.integers(2, n - a))
        l1[i], l2[i] = a, a + 1 + u
    return perms, l1, l2


@pytest.mark.parametrize("n,m,count", [(3, 2, 12), (8, 5, 60), (20, 20, 90), (50, 20, 60),
                                       (50, 10, 60), (100, 20, 24), (128, 16, 12),
                                       (33, 7, 40)])
def test_family_bounds_match_oracle(env, oracle, n, m, count):
    torch, W = env
    rng = np.random.default_rng(n * 100 + m)
    p = W.gen_instance(n + m, n, m)
    ctx = W.Context(p)
    perms, l1, l2 = random_fathers(rng, n, count)
    fathers = W.pack_records(perms, l1, l2)
    kids, off = W.expand_children(fathers, n)
    d_f = torch.from_numpy(fathers).cuda()
    d_off = torch.from_numpy(off).cuda()
    lb = torch.full((len(kids),), -7, dtype=torch.int32, device="cuda")
    job = torch.full((len(kids),), -7, dtype=torch.int16, device="cuda")
    ctx.decompose_lb2(d_f.data_ptr(), count, d_off.data_ptr(), lb.data_ptr(), job.data_ptr())
    torch.cuda.synchronize()
    kp, k1, k2 = W.unpack_records(kids, n)
    want = oracle.Bound(p).eval_batch(kp, k1, k2)
    np.testing.assert_array_equal(lb.cpu().numpy(), want)
    # the moved job: the one a child fixes that its father left free
    moved = []
    for f in range(count):
        for c in range(off[f], off[f + 1]):
            a, b = int(k1[c]), int(k2[c])
            fa = int(l1[f])
            moved.append(int(kp[c][fa + 1]) if a > fa else int(kp[c][b]))
    np.testing.assert_array_equal(job.cpu().numpy(), np.array(moved, dtype=np.int16))


@pytest.mark.parametrize("kind", ["int32", "uint16_limit", "uint16_full"])
def test_family_bounds_time_ranges(env, oracle, kind):
    """Both slot forms of the family kernel: processing times too large for
    16-bit bounds ((n + m - 1) * max p > 65535: int32 slots), and instances
    at the 16-bit limit, where the longest staircase path is 65525."""
    torch, W = env
    n, m, count = 20, 6, 120
    rng = np.random.default_rng({"int32": 1, "uint16_limit": 2, "uint16_full": 3}[kind])
    if kind == "int32":
        p = rng.integers(1, 5001, (m, n)).astype(np.int32)
    elif kind == "uint16_limit":
        p = rng.integers(1, 2622, (m, n)).astype(np.int32)
        p[:, ::3] = 2621
    else:
        p = np.full((m, n), 2621, dtype=np.int32)    # every makespan is 25 * 2621
    ctx = W.Context(p)
    perms, l1, l2 = random_fathers(rng, n, count)
    fathers = W.pack_records(perms, l1, l2)
    kids, off = W.expand_children(fathers, n)
    d_f = torch.from_numpy(fathers).cuda()
    d_off = torch.from_numpy(off).cuda()
    lb = torch.full((len(kids),), -7, dtype=torch.int32, device="cuda")
    job = torch.full((len(kids),), -7, dtype=torch.int16, device="cuda")
    ctx.decompose_lb2(d_f.data_ptr(), count, d_off.data_ptr(), lb.data_ptr(), job.data_ptr())
    torch.cuda.synchronize()
    kp, k1, k2 = W.unpack_records(kids, n)
    want = oracle.Bound(p).eval_batch(kp, k1, k2)
    if kind == "uint16_full":
        assert want.max() == 25 * 2621
    np.testing.assert_array_equal(lb.cpu().numpy(), want)


def test_family_bounds_equal_per_child_kernel(env):
    """Same bounds as the pool kernel on the expanded children, at a pool
    size where every CTA takes many fathers."""
    torch, W = env
    n, m, count = 50, 20, 3000
    rng = np.random.default_rng(7)
    p = W.gen_instance(3, n, m)
    ctx = W.Context(p)
    perms, l1, l2 = random_fathers(rng, n, count)
    fathers = W.pack_records(perms, l1, l2)
    kids, off = W.expand_children(fathers, n)
    d_f = torch.from_numpy(fathers).cuda()
    d_k = torch.from_numpy(kids).cuda()
    d_off = torch.from_numpy(off).cuda()
    lb = torch.empty(len(kids), dtype=torch.int32, device="cuda")
    job = torch.empty(len(kids), dtype=torch.int16, device="cuda")
    ref = torch.empty(len(kids), dtype=torch.int32, device="cuda")
    ctx.decompose_lb2(d_f.data_ptr(), count, d_off.data_ptr(), lb.data_ptr(), job.data_ptr())
    ctx.lb2_eval(d_k.data_ptr(), len(kids), ref.data_ptr())
    torch.cuda.synchronize()
    assert torch.equal(lb, ref)


@pytest.mark.parametrize("n,m", [(50, 20), (50, 5), (100, 20)])
def test_family_skips_malformed_fathers(env, oracle, n, m):
    """Fathers the kernel must pass over, between valid ones in one batch
    (so that a group meets them amid its other fathers): a repeated free
    job, a child range of the wrong size, cursors out of range. The valid
    fathers' bounds equal the oracle's; the others' children stay as they
    were."""
    torch, W = env
    rng = np.random.default_rng(n + m)
    p = W.gen_instance(5, n, m)
    ctx = W.Context(p)
    count = 2400 if n <= 50 else 600
    perms, l1, l2 = random_fathers(rng, n, count)
    fathers = W.pack_records(perms, l1, l2)
    kinds = np.zeros(count, dtype=np.int32)            # 0 valid
    kinds[5::7] = 1                                    # a repeated free job
    kinds[3::11] = 2                                   # a child range of the wrong size
    kinds[8::13] = 3                                   # l1 below -1
    sizes = []
    for i in range(count):
        u = int(l2[i] - l1[i] - 1)
        k = 2 if u == 2 else 2 * u
        if kinds[i] == 1:
            if u < 3:
                kinds[i] = 0
            else:
                fathers[i, l1[i] + 2] = fathers[i, l1[i] + 1]
        elif kinds[i] == 2:
            k += 2
        elif kinds[i] == 3:
            fathers[i, n] = -3
        sizes.append(k)
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    d_f = torch.from_numpy(fathers).cuda()
    d_off = torch.from_numpy(off).cuda()
    lb = torch.full((int(off[-1]),), -7, dtype=torch.int32, device="cuda")
    job = torch.full((int(off[-1]),), -7, dtype=torch.int16, device="cuda")
    ctx.decompose_lb2(d_f.data_ptr(), count, d_off.data_ptr(), lb.data_ptr(), job.data_ptr())
    torch.cuda.synchronize()
    lb, job = lb.cpu().numpy(), job.cpu().numpy()
    valid = np.flatnonzero(kinds == 0)
    assert len(valid) > count // 2 and (kinds == 1).sum() > count // 20
    kids, koff = W.expand_children(fathers[valid], n)
    kp, k1, k2 = W.unpack_records(kids, n)
    want = oracle.Bound(p).eval_batch(kp, k1, k2)
    got = np.concatenate([lb[off[f]:off[f + 1]] for f in valid])
    np.testing.assert_array_equal(got, want)
    for f in np.flatnonzero(kinds != 0):
        assert (lb[off[f]:off[f + 1]] == -7).all() and (job[off[f]:off[f + 1]] == -7).all(), f


@pytest.mark.parametrize("n,m,seed,best", [(20, 20, 1, "ub0"), (50, 10, 0, "default"),
                                           (12, 5, 3, "default")])
def test_search_same_tree_family_and_per_child(env, n, m, seed, best):
    torch, W = env
    from wsbb_gb300.explorer import explore
    p = W.gen_instance(seed, n, m)
    ub, _ = W.neh(p)
    b = ub if best == "ub0" else 99999
    ctx = W.Context(p)
    fam = explore(ctx, ub0=ub, best=b, max_iters=120)
    per = explore(ctx, ub0=ub, best=b, max_iters=120, child_lb2=True)
    for k in ("branched", "pruned", "leaves", "improved", "bounded", "evaluated", "discarded",
              "iterations", "best_cost", "status", "coverage", "scanned", "committed"):
        assert fam[k] == per[k], k
