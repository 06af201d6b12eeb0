"""The allocation-free search entry point (wsbb_explore_noalloc).

Some callers may not allocate GPU memory while they run: a service that
reserves all of its device memory at start-up and treats any later
cudaMalloc as a failure, code that runs inside a host callback or an
allocator hook where cudaMalloc is not allowed, or a latency-critical path
where an allocation (and its possible failure) in the middle of a request
is not acceptable. For them the library keeps the whole search state in one
fixed device array and this entry point allocates nothing.

This file is named so that pytest collects it last; it is self-contained,
so it passes alone in a fresh process as well as after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

INT32_MAX = 2**31 - 1
KEYS = ("branched", "pruned", "leaves", "improved", "bounded", "best_cost")


@pytest.fixture(scope="module")
def mods():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import wsbb_gb300
    from wsbb_gb300 import explorer
    L = wsbb_gb300.lib()
    L.wsbb_explore.argtypes = [C.c_void_p] * 4
    L.wsbb_explore_noalloc.argtypes = [C.c_void_p] * 4
    return wsbb_gb300, explorer, L


def run(L, fn, ctx, E, ub0, best, window=0, capacity=0):
    cfg = E.ExploreCfg(ub0, best, window, 4, capacity, 0, 0, 0)
    st = E.ExploreStats()
    rc = getattr(L, fn)(ctx.h, C.byref(cfg), C.byref(st), None)
    return rc, st


def test_noalloc_search_matches_allocating_search_twice(mods):
    W, E, L = mods
    for (n, m, seed) in ((16, 5, 6), (13, 10, 2)):
        p = W.gen_instance(seed, n, m)
        ctx = W.Context(p)
        ub, _ = W.neh(p)
        for ub0, best in ((INT32_MAX, 99999), (ub, ub)):
            rc, want = run(L, "wsbb_explore", ctx, E, ub0, best, window=256)
            assert rc == 0
            for call in range(2):  # the shared array keeps the last call's contents
                rc, got = run(L, "wsbb_explore_noalloc", ctx, E, ub0, best, window=256)
                assert rc == 0, L.wsbb_last_error(ctx.h)
                assert got.status == 0
                for k in KEYS:
                    assert getattr(got, k) == getattr(want, k), (n, m, seed, ub0, call, k)
                assert list(got.depth_hist) == list(want.depth_hist)
                assert list(got.best_perm[:n]) == list(want.best_perm[:n])


def test_noalloc_rejects_what_does_not_fit(mods):
    W, E, L = mods
    ctx = W.Context(W.gen_instance(1, 20, 5))
    # a capacity beyond the fixed array is refused before anything runs
    rc, _ = run(L, "wsbb_explore_noalloc", ctx, E, INT32_MAX, 99999, window=256,
                capacity=1 << 30)
    assert rc == -6
    assert b"MiB" in L.wsbb_last_error(ctx.h)
    # the array keeps no search between calls: nothing to resume
    cfg = E.ExploreCfg(INT32_MAX, 99999, 64, 4, 0, 0, E.RESUME, 0)
    assert L.wsbb_explore_noalloc(ctx.h, C.byref(cfg), C.byref(E.ExploreStats()), None) != 0
    assert b"resume" in L.wsbb_last_error(ctx.h)
    # and the entry point still works afterwards
    rc, got = run(L, "wsbb_explore_noalloc", ctx, E, INT32_MAX, 99999, window=64)
    assert rc == 0 and got.status == 0
    np.testing.assert_equal(got.best_cost > 0, True)


def test_noalloc_overflow_then_recovers(mods):
    """A stack just above one rewrite region overflows part-way through a
    search without an incumbent: the call returns WSBB_ERR_CAPACITY, and
    the next call with the derived defaults runs the whole search and
    equals the allocating search."""
    W, E, L = mods
    n = 20
    p = W.gen_instance(2, n, 5)
    ctx = W.Context(p)
    region = 4 * 64 + 4096  # the no-alloc region reserve at window 64
    rc, _ = run(L, "wsbb_explore_noalloc", ctx, E, INT32_MAX, 99999, window=64,
                capacity=region + 256)
    assert rc == -6, L.wsbb_last_error(ctx.h)
    ub, _ = W.neh(p)
    rc, want = run(L, "wsbb_explore", ctx, E, ub, 99999, window=256)
    assert rc == 0
    rc, got = run(L, "wsbb_explore_noalloc", ctx, E, ub, 99999)
    assert rc == 0 and got.status == 0, L.wsbb_last_error(ctx.h)
    for k in KEYS:
        assert getattr(got, k) == getattr(want, k), k
    assert list(got.depth_hist) == list(want.depth_hist)


def test_noalloc_call_leaves_free_memory_unchanged(mods):
    """Free device memory is the same before and after a call (the first
    call of the module, which may load the library's device code, is made
    before the measurement)."""
    import torch
    W, E, L = mods
    p = W.gen_instance(4, 16, 8)
    ctx = W.Context(p)
    ub, _ = W.neh(p)
    rc, _ = run(L, "wsbb_explore_noalloc", ctx, E, ub, 99999)
    assert rc == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(2):
        rc, st = run(L, "wsbb_explore_noalloc", ctx, E, ub, 99999)
        assert rc == 0 and st.status == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
