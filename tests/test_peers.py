"""Peers sharing one search (wsbb_gb300.peers): work hand-off as
BB_PROBLEM_PACKET payloads and termination detection, with world size 2 on
gloo (CPU processes) and 3 in-process peers. The engine here is a CPU test
double with GpuEngine's methods: a plain DFS over the library's records
(BEGIN children only, so every node's children partition its permutations)
bounded by the oracle. The GPU engine is covered in test_peers_gpu.py."""
import math
import os
import socket
import threading

import numpy as np
import pytest

INT32_MAX = 2**31 - 1


class CpuEngine:
    default_budget = 40  # bounded nodes per round

    def __init__(self, p):
        from oracle import oracle
        self.b = oracle.Bound(np.asarray(p, dtype=np.int32))
        self.n = p.shape[1]
        self.stack = []
        self._reset(INT32_MAX)

    def _reset(self, ub):
        self.ub = ub
        self.c = {k: 0 for k in ("branched", "pruned", "leaves", "improved", "bounded",
                                 "evaluated", "discarded")}
        self.cov = 0
        self.best_cost, self.best_perm = INT32_MAX, np.full(self.n, -1, dtype=np.int32)

    def _stats(self):
        return dict(self.c, status=1 if self.stack else 0, best_cost=min(self.ub, self.best_cost),
                    best_perm=self.best_perm.copy(), perm_cost=self.best_cost,
                    coverage=self.cov)

    def start_root(self, ub, budget):
        self._reset(ub)
        perm = list(range(self.n))
        self.stack = [(tuple(perm), -1, self.n, self.b.eval(perm, -1, self.n)[0])]
        return self.run(ub, budget)

    def run(self, ub, budget):
        self.ub = min(self.ub, ub)
        done = 0
        while self.stack and done < budget:
            perm, l1, l2, lb = self.stack.pop()
            u = l2 - l1 - 1
            if lb >= self.ub:
                self.c["pruned"] += 1
                self.cov += math.factorial(u)
                continue
            if u == 0:
                self.c["leaves"] += 1
                self.cov += 1
                self.c["improved"] += 1
                self.ub = self.best_cost = lb
                self.best_perm = np.array(perm, dtype=np.int32)
                continue
            self.c["branched"] += 1
            kids = []
            for i in range(l1 + 1, l2):
                q = list(perm)
                q[l1 + 1], q[i] = q[i], q[l1 + 1]
                kids.append((tuple(q), l1 + 1, l2, self.b.eval(q, l1 + 1, l2)[0]))
            self.c["bounded"] += len(kids)
            self.c["evaluated"] += len(kids)
            done += len(kids)
            kids.sort(key=lambda k: (-k[3], -k[0][l1 + 1]))  # the best on top
            self.stack.extend(kids)
        return self._stats()

    def export(self, k):
        import wsbb_gb300 as W
        take = [e for e in self.stack if e[3] < self.ub][:k]
        ids = {id(e) for e in take}
        self.stack = [e for e in self.stack if id(e) not in ids]
        if not take:
            return np.zeros((0, W.node_stride(self.n) // 2), np.int16), np.zeros(0, np.int32)
        rec = W.pack_records(np.array([e[0] for e in take]), [e[1] for e in take],
                             [e[2] for e in take])
        return rec, np.array([e[3] for e in take], dtype=np.int32)

    def seed(self, rec, lbs, ub):
        self._reset(ub)
        n = self.n
        self.stack = [(tuple(int(x) for x in r[:n]), int(r[n]), int(r[n + 1]), int(lb))
                      for r, lb in zip(rec, lbs)]


def sequential(p, ub0):
    e = CpuEngine(p)
    st = e.start_root(INT32_MAX if ub0 is None else ub0, 10**12)
    return st


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, p, ub0, out):
    import torch.distributed as dist

    from wsbb_gb300 import peers
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        res = peers.peer_search(CpuEngine(p), peers.TorchTransport(), p.shape[1], ub0=ub0,
                                budget=40, share=3)
        out.put((rank, res.best_cost, None if res.best_perm is None else res.best_perm.tolist(),
                 res.total, res.total_coverage, res.sent, res.received, res.rounds,
                 res.counters))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("at_optimum", [False, True])
def test_two_gloo_peers_find_the_optimum_and_cover_the_tree(at_optimum):
    import torch.multiprocessing as mp
    import wsbb_gb300 as W
    n, m = 9, 3
    p = W.gen_instance(5, n, m)
    seq = sequential(p, None)
    ub0 = seq["best_cost"] if at_optimum else None
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, p, ub0, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    (_, c0, p0, t0, cov0, s0, r0, n0, k0), (_, c1, p1, t1, cov1, s1, r1, n1, k1) = res
    assert c0 == c1 == seq["best_cost"]
    assert t0 == t1 and cov0 == cov1 == math.factorial(n)     # every subtree exactly once
    from wsbb_gb300.peers import makespan
    if p0 is not None:
        assert makespan(p, np.array(p0)) == c0
    assert n0 == n1 and s0 + s1 > 0 and s0 + s1 == r0 + r1   # work moved, none lost
    assert t0["branched"] == k0["branched"] + k1["branched"]
    if at_optimum:
        assert p0 is None and p1 is None                    # nothing below the optimum
    else:
        assert p0 == p1


def test_final_permutation_is_the_winners():
    """A peer whose incumbent another peer lowered still holds its own older,
    costlier permutation; the permutation returned is the one of the final
    cost (scripted engines: peer 0 keeps a permutation of cost 120 and runs
    once more after peer 1 found one of cost 100)."""
    import wsbb_gb300 as W
    from wsbb_gb300 import peers

    def st(ub, status, own_cost, perm):
        return dict({k: 0 for k in peers.COUNTERS}, status=status, coverage=0,
                    best_cost=min(ub, own_cost), best_perm=np.array(perm, dtype=np.int32),
                    perm_cost=own_cost)

    class First:   # busy for three rounds, permutation [2, 1, 0] of cost 120
        default_budget = 1
        calls = 0

        def start_root(self, ub, budget):
            return st(ub, 1, 120, [2, 1, 0])

        def run(self, ub, budget):
            self.calls += 1
            return st(ub, 1 if self.calls < 3 else 0, 120, [2, 1, 0])

        def export(self, k):
            if self.calls == 1:
                return W.pack_records(np.array([[0, 1, 2]]), [-1], [3]), np.array([50], np.int32)
            return np.zeros((0, W.node_stride(3) // 2), np.int16), np.zeros(0, np.int32)

    class Second:  # finds [0, 1, 2] of cost 100 in the work it is handed
        default_budget = 1

        def seed(self, recs, lbs, ub):
            assert recs[:, :3].tolist() == [[0, 1, 2]] and lbs.tolist() == [50]

        def run(self, ub, budget):
            return st(ub, 0, 100, [0, 1, 2])

    hub = peers.LocalHub(2)
    out = [None, None]

    def run(r, eng):
        out[r] = peers.peer_search(eng, peers.LocalTransport(hub, r), 3)

    th = [threading.Thread(target=run, args=(0, First())),
          threading.Thread(target=run, args=(1, Second()))]
    for t in th:
        t.start()
    for t in th:
        t.join(timeout=60)
    assert out[0].complete and out[1].complete
    assert out[0].best_cost == out[1].best_cost == 100
    assert out[0].best_perm.tolist() == out[1].best_perm.tolist() == [0, 1, 2]
    assert out[0].sent == out[1].received == 1


def test_makespan_equals_oracle():
    import wsbb_gb300 as W
    from oracle import oracle
    from wsbb_gb300.peers import makespan
    rng = np.random.default_rng(9)
    for n, m in [(9, 3), (20, 20), (50, 10)]:
        p = W.gen_instance(n + m, n, m)
        b = oracle.Bound(p)
        for _ in range(5):
            perm = rng.permutation(n)
            assert makespan(p, perm) == b.makespan(perm)


def test_three_local_peers_and_termination():
    import wsbb_gb300 as W
    from wsbb_gb300 import peers
    n, m = 9, 3
    p = W.gen_instance(5, n, m)
    seq = sequential(p, None)
    hub = peers.LocalHub(3)
    out = [None] * 3

    def run(r):
        out[r] = peers.peer_search(CpuEngine(p), peers.LocalTransport(hub, r), n,
                                   budget=40, share=2)

    th = [threading.Thread(target=run, args=(r,)) for r in range(3)]
    for t in th:
        t.start()
    for t in th:
        t.join(timeout=300)
    assert all(o is not None for o in out)
    assert {o.best_cost for o in out} == {seq["best_cost"]}
    assert {o.total_coverage for o in out} == {math.factorial(n)}
    assert sum(o.received for o in out) == sum(o.sent for o in out) > 0
    assert len({o.rounds for o in out}) == 1            # all stopped at the same round
    assert all(o.complete for o in out)
    assert all(o.counters["branched"] > 0 for o in out)  # every peer worked
    assert out[0].best_perm.tolist() == out[2].best_perm.tolist()


def test_packet_round_trip_keeps_open_nodes():
    """What a donor sends is what the receiver seeds: records and bounds."""
    import wsbb_gb300 as W
    from wsbb_gb300 import formats
    n = 12
    rng = np.random.default_rng(3)
    perms = np.array([rng.permutation(n) for _ in range(10)])
    l1 = rng.integers(-1, 5, 10)
    l2 = l1 + 1 + rng.integers(2, n - 5, 10)
    rec = W.pack_records(perms, l1, l2)
    lbs = rng.integers(100, 900, 10).astype(np.int32)
    back, blb, _, _ = formats.unpack_work(formats.pack_work(rec, n, lbs, max_nbjobs=n), n,
                                          max_nbjobs=n)
    np.testing.assert_array_equal(back, rec)
    np.testing.assert_array_equal(blb, lbs)
