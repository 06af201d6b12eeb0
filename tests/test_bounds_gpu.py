"""GPU parity of the pool bound kernels, through the C-ABI.

Bit-exact against (1) the reference's own outputs in tests/golden and
(2) the CPU oracle on seeded pools of n=20, m=20, seeds 0-9, every pool size
from 2^16 to 2^20 records, and on frontiers logged from the search; at 2^20
records, size-independent properties (leaf bounds equal makespans, LB2 never
exceeds the makespan of the record's own completion, repeat launches agree).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="module")
def W():
    import wsbb_gb300
    wsbb_gb300.lib()
    return wsbb_gb300


def run_dev(torch, ctx, recs, kind="lb2"):
    d_recs = torch.from_numpy(np.ascontiguousarray(recs)).cuda()
    out = torch.empty(len(recs), dtype=torch.int32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    getattr(ctx, kind + "_eval")(d_recs.data_ptr(), len(recs), out.data_ptr(), s)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def cases(golden_pools):
    return sorted({k.rsplit("_", 1)[0] for k in golden_pools.files})


def test_lb2_matches_reference_golden(torch_cuda, W, golden_pools):
    for key in cases(golden_pools):
        p = golden_pools[key + "_p"].astype(np.int32)
        perms = golden_pools[key + "_perms"].astype(np.int16)
        recs = W.pack_records(perms, golden_pools[key + "_l1"], golden_pools[key + "_l2"])
        ctx = W.Context(p)
        np.testing.assert_array_equal(run_dev(torch_cuda, ctx, recs),
                                      golden_pools[key + "_lb"], err_msg=key)
        np.testing.assert_array_equal(ctx.lb2_eval_host(recs), golden_pools[key + "_lb"],
                                      err_msg=key + " host path")


@pytest.mark.parametrize("seed", range(10))
def test_lb2_matches_oracle_n20_m20(torch_cuda, W, oracle, seed):
    """The pool-bound workload at its own sizes: for each seed, uniform
    random pools of 2^16, 2^17, ..., 2^20 records, every bound bit-exact
    against the oracle."""
    import os
    n, m = 20, 20
    p = W.gen_instance(seed, n, m)
    ctx = W.Context(p)
    ob = oracle.Bound(p)
    for k, log2 in enumerate(range(16, 21)):
        recs = W.gen_pool(1000 + 8 * seed + k, n, 1 << log2, leaf_share=0.02)
        got = run_dev(torch_cuda, ctx, recs)
        perms, l1, l2 = W.unpack_records(recs, n)
        want = ob.eval_batch(perms, l1, l2, nthreads=os.cpu_count() or 8)
        np.testing.assert_array_equal(got, want, err_msg=f"seed {seed} pool 2^{log2}")


@pytest.mark.parametrize("seed", range(10))
def test_lb2_matches_oracle_on_search_frontiers(torch_cuda, W, oracle, seed):
    """Pools of the kind the search bounds: 2^16 children logged from the
    exact search on each instance (uneven depths, both sides), bounded by
    the pool kernel and the oracle."""
    import os
    import torch
    from wsbb_gb300 import learned
    n, m, count = 20, 20, 1 << 16
    p = W.gen_instance(seed, n, m)
    ctx = W.Context(p)
    neh, _ = W.neh(p)
    buf = torch.zeros((count, W.node_stride(n) // 2), dtype=torch.int16, device="cuda")
    got_n, _ = learned.log_nodes(ctx, buf.data_ptr(), count, 3, ub0=neh, window=1024)
    torch.cuda.synchronize()
    assert got_n > count // 2
    recs = buf[:got_n].cpu().numpy()
    perms, l1, l2 = W.unpack_records(recs, n)
    assert len(np.unique(l2 - l1)) > 5  # many depths
    np.testing.assert_array_equal(
        run_dev(torch_cuda, ctx, recs),
        oracle.Bound(p).eval_batch(perms, l1, l2, nthreads=os.cpu_count() or 8))


@pytest.mark.parametrize("n,m,seed", [(20, 5, 0), (20, 10, 1), (50, 10, 2), (50, 20, 3),
                                      (100, 20, 4), (33, 7, 5), (64, 16, 6), (65, 16, 7),
                                      (128, 9, 8), (3, 2, 9), (4, 32, 10)])
def test_lb2_lb1_makespan_match_oracle_shapes(torch_cuda, W, oracle, n, m, seed):
    p = W.gen_instance(seed, n, m)
    count = 3001
    recs = W.gen_pool(50 + seed, n, count, leaf_share=0.1)
    ctx = W.Context(p)
    ob = oracle.Bound(p)
    perms, l1, l2 = W.unpack_records(recs, n)
    np.testing.assert_array_equal(run_dev(torch_cuda, ctx, recs),
                                  ob.eval_batch(perms, l1, l2, nthreads=8))
    np.testing.assert_array_equal(run_dev(torch_cuda, ctx, recs, "lb1"),
                                  ob.lb1_batch(perms, l1, l2))
    full = np.array([ob.makespan(q) for q in perms[:300]], dtype=np.int32)
    np.testing.assert_array_equal(run_dev(torch_cuda, ctx, recs[:300], "makespan"), full)


def test_lb2_full_size_properties(torch_cuda, W):
    """2^20 records: leaves give makespans, LB2 <= makespan of the record's
    own completion, and two launches agree."""
    n, m, count = 20, 20, 1 << 20
    p = W.gen_instance(0, n, m)
    recs = W.gen_pool(7, n, count, leaf_share=0.05)
    ctx = W.Context(p)
    lb = run_dev(torch_cuda, ctx, recs)
    mk = run_dev(torch_cuda, ctx, recs, "makespan")
    perms, l1, l2 = W.unpack_records(recs, n)
    leaf = (l2 - l1) == 1
    np.testing.assert_array_equal(lb[leaf], mk[leaf])
    assert np.all(lb <= mk)
    assert np.all(lb > 0)
    np.testing.assert_array_equal(lb, run_dev(torch_cuda, ctx, recs))


def test_lb2_full_size_matches_oracle(torch_cuda, W, oracle):
    import os
    n, m, count = 20, 20, 1 << 20
    p = W.gen_instance(3, n, m)
    recs = W.gen_pool(1003, n, count)
    got = run_dev(torch_cuda, W.Context(p), recs)
    perms, l1, l2 = W.unpack_records(recs, n)
    want = oracle.Bound(p).eval_batch(perms, l1, l2, nthreads=os.cpu_count() or 8)
    np.testing.assert_array_equal(got, want)


def test_edge_counts_and_errors(torch_cuda, W, oracle):
    n, m = 20, 20
    p = W.gen_instance(1, n, m)
    ctx = W.Context(p)
    recs = W.gen_pool(3, n, 70)
    ob = oracle.Bound(p)
    for cnt in (1, 31, 32, 33, 64, 70):
        perms, l1, l2 = W.unpack_records(recs[:cnt], n)
        np.testing.assert_array_equal(run_dev(torch_cuda, ctx, recs[:cnt]),
                                      ob.eval_batch(perms, l1, l2))
    assert len(ctx.lb2_eval_host(recs[:0])) == 0
    # misaligned record pointer is rejected, not launched
    d = torch_cuda.zeros(70 * 48 + 16, dtype=torch_cuda.uint8, device="cuda")
    out = torch_cuda.empty(70, dtype=torch_cuda.int32, device="cuda")
    with pytest.raises(W.WsbbError):
        ctx.lb2_eval(d.data_ptr() + 4, 70, out.data_ptr())
    with pytest.raises(W.WsbbError):
        W.Context(np.full((2, 5), 70000, dtype=np.int32))
    with pytest.raises(W.WsbbError):
        W.Context(np.ones((33, 5), dtype=np.int32))


def test_bound_plugin_mirror(torch_cuda, W, oracle):
    """bornes_calculer with the reference's argument meaning."""
    n, m = 20, 5
    p = W.gen_instance(0, n, m)
    plug = W.BoundFlowshopGB300()
    plug.set_instance(p)
    ob = oracle.Bound(p)
    rng = np.random.default_rng(1)
    for _ in range(20):
        perm = rng.permutation(n).astype(np.int32)
        l1 = int(rng.integers(-1, n - 3))
        l2 = int(rng.integers(l1 + 2, n + 1))
        couts = [0, 0]
        plug.bornes_calculer(perm, l1, l2, couts, 999999)
        assert couts == [ob.eval(perm, l1, l2)[0], 0]
