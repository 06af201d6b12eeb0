"""The reference's incumbent file and work hand-off packet (no GPU): the
reader against a bab.solutions the reference itself wrote, the writer read
back by the reference's own reader (where it was built here), and packet
layout and round trips."""
import json
import os
import tempfile

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def fixture():
    with open(os.path.join(GOLDEN, "bab_solutions_n12m5.json")) as f:
        meta = json.load(f)
    return meta, os.path.join(GOLDEN, "bab_solutions_n12m5.txt")


def test_reader_on_the_reference_file(fixture, oracle):
    from wsbb_gb300 import formats as F
    meta, path = fixture
    n = meta["n"]
    with open(path) as f:
        blocks = F.parse_solutions(f.read(), n)
    res = meta["result"]
    # one block per improvement, each saved before the improvement it
    # records was added: the first is empty, the optimum is never written
    assert len(blocks) == res["improved"] and blocks[0] == []
    costs = [b[0]["cost"] for b in blocks[1:]]
    assert all(len(b) == 1 for b in blocks[1:]) and costs == sorted(costs, reverse=True)
    assert costs[-1] > res["optimum"]
    bound = oracle.Bound(np.array(meta["p"], dtype=np.int32))
    for b in blocks[1:]:
        r = b[0]
        assert sorted(r["perm"].tolist()) == list(range(n))
        assert r["limite2"] - r["limite1"] == 1 and r["depth"] == n
        assert r["couts_somme"] == r["cost"] == bound.makespan(r["perm"])
    assert F.read_solutions(path, n) == []  # what the reference itself would load
    cost, perm = F.best_incumbent(path, n)
    assert cost == costs[-1] and bound.makespan(perm) == cost


def test_writer_round_trip():
    from wsbb_gb300 import formats as F
    n = 7
    sols = [(123, [3, 1, 0, 6, 5, 4, 2]), (120, list(range(n)))]
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "bab.solutions")
        F.write_solutions(path, sols[:1], n)
        F.write_solutions(path, sols[1:], n, append=True)
        blocks = F.parse_solutions(open(path).read(), n)
        assert [[(r["cost"], r["perm"].tolist()) for r in b] for b in blocks] == \
            [[(123, sols[0][1])], [(120, sols[1][1])]]
        assert F.best_incumbent(path, n)[0] == 120
    with pytest.raises(ValueError):
        F.format_solutions([(1, [0, 0, 1])], 3)
    with pytest.raises(ValueError):
        F.format_solutions([(1, list(range(21)))], 21)


def test_reference_reads_the_written_file(fixture, oracle):
    """The reference's own reader seeds its search from our file exactly as
    from the record its harness writes for the same incumbent."""
    if not os.path.exists(oracle._REF_EXPLORE):
        pytest.skip("reference build absent (it only builds where its sources are)")
    from wsbb_gb300 import formats as F
    meta, _ = fixture
    n = meta["n"]
    p = np.array(meta["p"], dtype=np.int32)
    opt, perm = meta["result"]["optimum"], meta["result"]["perm"]
    with tempfile.TemporaryDirectory() as d:
        F.write_solutions(os.path.join(d, "bab.solutions"), [(opt, perm)], n)
        ours = oracle.ref_explore(p, ub0=None, workdir=d)
    theirs = oracle.ref_explore(p, ub0=opt)
    assert ours["preloaded"] == 1
    for k in ("branched", "pruned", "leaves", "improved", "bounded", "optimum", "coverage"):
        assert ours[k] == theirs[k], k


def test_work_packet_layout_and_round_trip():
    import wsbb_gb300 as W
    from wsbb_gb300 import formats as F
    n, count = 12, 9
    rng = np.random.default_rng(3)
    perms = np.array([rng.permutation(n) for _ in range(count)], dtype=np.int32)
    l1 = rng.integers(-1, n - 3, count).astype(np.int32)
    l2 = (l1 + 3 + rng.integers(0, 3, count)).clip(max=n).astype(np.int32)
    rec = W.pack_records(perms, l1, l2)
    lbs = rng.integers(500, 900, count).astype(np.int32)
    be = rng.integers(0, 2, count)
    ranks = rng.integers(0, n, (count, F.MAX_NBJOBS + 1))
    data = F.pack_work(rec, n, lbs, be, ranks)
    assert len(data) == count * 184  # 46 ints per node at MAX_NBJOBS = 20
    a = np.frombuffer(data, dtype="<i4").reshape(count, 46)
    assert (a[:, :n] == perms).all() and (a[:, n:20] == 0).all()
    assert (a[:, 20] == l1).all() and (a[:, 21] == l2).all() and (a[:, 22] == lbs).all()
    assert (a[:, 23] == rec[:, n + 2]).all() and (a[:, 24] == be).all()
    assert (a[:, 25:] == ranks).all()
    r2, lb2, be2, rk2 = F.unpack_work(data, n)
    assert np.array_equal(r2, rec) and np.array_equal(lb2, lbs)
    assert np.array_equal(be2, be) and np.array_equal(rk2, ranks)
    with pytest.raises(ValueError):
        F.unpack_work(data[:-4], n)


def test_empty_packet():
    """A peer with nothing to hand off sends an empty payload."""
    import wsbb_gb300 as W
    from wsbb_gb300 import formats
    n = 7
    empty = np.zeros((0, W.node_stride(n) // 2), np.int16)
    assert formats.pack_work(empty, n, np.zeros(0, np.int32), max_nbjobs=n) == b""
    rec, lbs, be, ranks = formats.unpack_work(b"", n, max_nbjobs=n)
    assert rec.shape == (0, W.node_stride(n) // 2) and len(lbs) == 0
