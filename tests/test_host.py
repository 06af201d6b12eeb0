"""Host-side product code (no GPU): the library loads and exports every
declared symbol; its generator, pool maker, NEH and bound precompute equal
the oracle's."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def W():
    import wsbb_gb300
    wsbb_gb300.lib()
    return wsbb_gb300


def declared_functions():
    names = []
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if not fn.endswith(".h"):
            continue
        txt = open(os.path.join(ROOT, "include", fn)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[\w]+\s*\*?\s*(wsbb_\w+)\s*\(", txt, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(W):
    names = declared_functions()
    assert len(names) >= 10
    missing = [n for n in names if not hasattr(W.lib(), n)]
    assert not missing, missing


def test_instances_equal_oracle(W, oracle):
    for (s, n, m) in [(0, 20, 20), (3, 50, 10), (7, 100, 20), (1, 5, 2)]:
        np.testing.assert_array_equal(W.gen_instance(s, n, m), oracle.gen_instance(s, n, m))


def test_taillard_generator_matches_reference_streams(W, oracle):
    """Taillard's generator: the oracle restatement and the library both
    reproduce the streams the reference's own instance_flowshop::unif drew
    (tests/golden/taillard_streams.json), and agree with each other and,
    where it is built, with the reference on more seeds."""
    import json
    with open(os.path.join(ROOT, "tests", "golden", "taillard_streams.json")) as f:
        cases = json.load(f)
    for c in cases:
        want = np.array(c["p"], dtype=np.int32).reshape(c["m"], c["n"])
        np.testing.assert_array_equal(oracle.taillard_instance(c["seed"], c["n"], c["m"]), want)
        np.testing.assert_array_equal(W.taillard_instance(c["seed"], c["n"], c["m"]), want)
    rng = np.random.default_rng(5)
    for seed in [int(x) for x in rng.integers(1, 2**31 - 1, 40)]:
        a = W.taillard_instance(seed, 30, 7)
        np.testing.assert_array_equal(a, oracle.taillard_instance(seed, 30, 7))
        if oracle.have_reference():
            np.testing.assert_array_equal(a, oracle.ref_taillard_instance(seed, 30, 7))
    with pytest.raises(ValueError):
        W.taillard_instance(1, 0, 5)


def test_pools_equal_oracle(W, oracle):
    for (s, n, leaf) in [(1, 20, 0.05), (2, 50, 0.0), (9, 100, 0.2)]:
        rec = W.gen_pool(s, n, 777, leaf)
        perms, l1, l2 = W.unpack_records(rec, n)
        o_perms, o_l1, o_l2 = oracle.random_pool(s, n, 777, leaf)
        np.testing.assert_array_equal(perms, o_perms)
        np.testing.assert_array_equal(l1, o_l1)
        np.testing.assert_array_equal(l2, o_l2)


def test_neh_equals_oracle(W, oracle):
    for (s, n, m) in [(0, 20, 5), (1, 20, 20), (2, 50, 10), (4, 12, 3)]:
        p = W.gen_instance(s, n, m)
        c, perm = W.neh(p)
        oc, operm = oracle.neh(p)
        assert c == oc
        np.testing.assert_array_equal(perm, operm)


def test_precompute_equals_oracle(W, oracle, golden_pools):
    keys = sorted({k.rsplit("_", 1)[0] for k in golden_pools.files})
    for key in keys:
        p = golden_pools[key + "_p"].astype(np.int32)
        m, n = p.shape
        P = m * (m - 1) // 2
        got = {k: np.empty(s, dtype=np.int32) for k, s in
               [("mach0", P), ("mach1", P), ("lag", P * n), ("johnson", P * n),
                ("heads", m), ("tails", m)]}
        rc = W.lib().wsbb_precompute(p.ctypes.data, n, m,
                                     *(got[k].ctypes.data for k in
                                       ("mach0", "mach1", "lag", "johnson", "heads", "tails")))
        assert rc == 0
        want = oracle.Bound(p).tables()
        np.testing.assert_array_equal(got["mach0"], want["mach0"])
        np.testing.assert_array_equal(got["mach1"], want["mach1"])
        np.testing.assert_array_equal(got["lag"], want["lag"].ravel())
        np.testing.assert_array_equal(got["johnson"], want["johnson"].ravel(), err_msg=key)
        np.testing.assert_array_equal(got["heads"], want["min_arr"])
        np.testing.assert_array_equal(got["tails"], want["min_dep"])


def test_precompute_rejects_bad_sizes(W):
    p = np.ones((40, 5), dtype=np.int32)
    z = np.empty(4096, dtype=np.int32)
    assert W.lib().wsbb_precompute(p.ctypes.data, 5, 40, *(z.ctypes.data,) * 6) != 0
    p = np.ones((3, 200), dtype=np.int32)
    assert W.lib().wsbb_precompute(p.ctypes.data, 200, 3, *(z.ctypes.data,) * 6) != 0
    # p1 + lag + p2 of a pair must fit 16 bits: 3 x 20000 fits, 3 x 30000 not
    p = np.full((3, 4), 20000, dtype=np.int32)
    assert W.lib().wsbb_precompute(p.ctypes.data, 4, 3, *(z.ctypes.data,) * 6) == 0
    p = np.full((3, 4), 30000, dtype=np.int32)
    assert W.lib().wsbb_precompute(p.ctypes.data, 4, 3, *(z.ctypes.data,) * 6) != 0


def test_record_layout(W):
    assert W.node_stride(20) == 48
    assert W.node_stride(50) == 112
    assert W.node_stride(100) == 208
    rec = W.pack_records(np.arange(20)[None, :], [3], [17])
    perms, l1, l2 = W.unpack_records(rec, 20)
    assert (l1[0], l2[0]) == (3, 17)
    assert rec.nbytes == 48


def test_child_order_partitions_the_permutations(W):
    """Expanding from the root, keeping one side of every father at random
    (the choice the search makes), reaches every permutation exactly once
    as a leaf; each child fixes one job its father left free."""
    n = 6
    rng = np.random.default_rng(0)
    root = W.pack_records(np.arange(n)[None, :], [-1], [n])
    leaves, stack = [], [root[0]]
    while stack:
        r = stack.pop()
        kids, off = W.expand_children(r[None, :], n)
        u = int(r[n + 1]) - int(r[n]) - 1
        assert len(kids) == (2 if u == 2 else 2 * u)
        if u == 2:
            leaves += [tuple(k[:n]) for k in kids]
            assert all(k[n + 1] - k[n] == 1 and k[n + 2] == n for k in kids)
            continue
        free = set(r[int(r[n]) + 1:int(r[n + 1])].tolist())
        side = int(rng.integers(0, 2))
        for k in kids[side * u:(side + 1) * u]:
            assert sorted(k[:n].tolist()) == list(range(n))
            assert set(k[int(k[n]) + 1:int(k[n + 1])].tolist()) < free
            assert int(k[n + 2]) == int(r[n + 2]) + 1
            stack.append(k)
    assert len(leaves) == 720 and len(set(leaves)) == 720


def test_autotune_cache_and_pick(tmp_path, monkeypatch):
    from wsbb_gb300 import autotune as A
    monkeypatch.setenv("WSBB_GB300_CACHE", str(tmp_path))
    rs = [{"window": 4096, "family_smem_kb": 56, "bounded_per_s": 10.0},
          {"window": 8192, "family_smem_kb": 100, "bounded_per_s": 12.05},
          {"window": 2048, "family_smem_kb": 56, "bounded_per_s": 12.0}]
    assert A.pick(rs) == rs[2]  # within 1 %: the smaller tile and window
    assert A.pick(rs, tolerance=0.0) == rs[1]
    key = A.cache_key("GB300", 50, 20, True)
    assert A.load_cache() == {}
    A.store(key, rs[1])
    A.store(A.cache_key("GB300", 20, 20, False), rs[0])
    data = A.load_cache()
    assert data[key] == rs[1] and len(data) == 2
    assert A.cache_path().startswith(str(tmp_path))


def test_multi_instance_shapes_and_capacity():
    from wsbb_gb300 import multi_bench as M
    shapes = [M.shape_of(i) for i in range(64)]
    assert shapes[:4] == [(20, 5), (50, 5), (100, 5), (20, 10)]
    assert len(set(shapes)) == 9
    assert sum(1 for n, m in shapes if m == 20) == 21
    # 64 stacks share the GPU: 2^23 nodes at n = 20, 2^24 from n = 50 on
    assert M.capacity_of(20) == 1 << 23
    assert M.capacity_of(50) == M.capacity_of(100) == 1 << 24
    total = sum(M.capacity_of(n) * (2 * n + 8 + 15) // 16 * 16 for n, m in shapes)
    assert total < 200 * 2**30
