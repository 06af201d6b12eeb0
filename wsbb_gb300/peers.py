"""Peers that share one search: work hand-off and termination detection.

The reference runs one exploration per peer and balances them by work
stealing: an idle peer asks for work and gets a node list in a
BB_PROBLEM_PACKET (src/work_stealing/node.cpp:524-560, 1240-1283), with
termination detected when no peer holds work (node.cpp:837-906,
protocol.cpp:451-552).

Here each peer runs the GPU search on its own context; peers meet at
synchronous rounds:

1. every busy peer searches for a node budget (`wsbb_explore`, resumed);
2. the incumbent cost is min-reduced, so every peer prunes against the best
   one found anywhere;
3. every peer reports whether it is idle (its search complete); when all
   are, the search is over — the check happens at the round barrier, with
   no hand-off in flight, so it cannot fire early;
4. idle peers receive work: each is paired with a busy peer, which takes
   open nodes from the bottom of its stack (the shallowest, largest
   subtrees; `wsbb_explore_export`) and sends them as a BB_PROBLEM_PACKET
   payload (`formats.pack_work`); the receiver seeds its search with them
   (`wsbb_explore_seed`).

The transport is pluggable: torch.distributed (gloo or nccl process groups,
one process per GPU) or in-process threads (several contexts in one
process). So is the engine: `GpuEngine` drives the library; any object with
the same methods can stand in for it.
"""
from __future__ import annotations

import math
import queue
import threading
from dataclasses import dataclass, field

import numpy as np

from . import formats

INT32_MAX = 2**31 - 1

COUNTERS = ("branched", "pruned", "leaves", "improved", "bounded", "evaluated", "discarded")


# ------------------------------------------------------------------ transports

class TorchTransport:
    """Collectives and point-to-point over the default torch.distributed group
    (CPU tensors: use a gloo group, or a gloo subgroup next to nccl)."""

    def __init__(self, group=None):
        import torch.distributed as dist
        self.dist = dist
        self.group = group
        self.rank = dist.get_rank(group)
        self.world = dist.get_world_size(group)

    def allgather(self, values: list[int]) -> list[list[int]]:
        import torch
        t = torch.tensor(values, dtype=torch.int64)
        out = [torch.empty_like(t) for _ in range(self.world)]
        self.dist.all_gather(out, t, group=self.group)
        return [o.tolist() for o in out]

    def _peer(self, r: int) -> int:
        return r if self.group is None else self.dist.get_global_rank(self.group, r)

    def send(self, dst: int, data: bytes) -> None:
        import torch
        self.dist.send(torch.tensor([len(data)], dtype=torch.int64), self._peer(dst),
                       group=self.group)
        if data:
            buf = torch.frombuffer(bytearray(data), dtype=torch.uint8)
            self.dist.send(buf, self._peer(dst), group=self.group)

    def recv(self, src: int) -> bytes:
        import torch
        n = torch.empty(1, dtype=torch.int64)
        self.dist.recv(n, self._peer(src), group=self.group)
        if int(n) == 0:
            return b""
        buf = torch.empty(int(n), dtype=torch.uint8)
        self.dist.recv(buf, self._peer(src), group=self.group)
        return buf.numpy().tobytes()


class LocalHub:
    """Shared state of in-process peers (one thread each). A peer that stops
    without reaching a meeting point breaks the others' waits after
    `timeout` seconds instead of leaving them blocked."""

    def __init__(self, world: int, timeout: float = 600.0):
        self.world = world
        self.timeout = timeout
        self.barrier = threading.Barrier(world, timeout=timeout)
        self.slots: list = [None] * world
        self.boxes = {(s, d): queue.Queue() for s in range(world) for d in range(world)}


class LocalTransport:
    def __init__(self, hub: LocalHub, rank: int):
        self.hub, self.rank, self.world = hub, rank, hub.world

    def allgather(self, values: list[int]) -> list[list[int]]:
        self.hub.barrier.wait()
        self.hub.slots[self.rank] = list(values)
        self.hub.barrier.wait()
        out = [list(v) for v in self.hub.slots]
        self.hub.barrier.wait()
        return out

    def send(self, dst: int, data: bytes) -> None:
        self.hub.boxes[(self.rank, dst)].put(bytes(data))

    def recv(self, src: int) -> bytes:
        return self.hub.boxes[(src, self.rank)].get(timeout=self.hub.timeout)


# --------------------------------------------------------------------- engine
#
# An engine searches on one peer. Its results are dicts with the counters of
# COUNTERS, "coverage", "status" (0: its search is complete), "best_cost"
# (its incumbent, which another peer may have lowered) and "best_perm" /
# "perm_cost": the best permutation it found itself and that permutation's
# makespan (perm[0] < 0 and INT32_MAX when it found none).


def makespan(p: np.ndarray, perm) -> int:
    """Makespan of a full permutation (machine-major times p)."""
    t = np.zeros(p.shape[0], dtype=np.int64)
    for j in perm:
        t[0] += p[0, j]
        for k in range(1, p.shape[0]):
            t[k] = max(t[k], t[k - 1]) + p[k, j]
    return int(t[-1])

class GpuEngine:
    """The library's search on one context, as a peer's engine. Its unit of
    work per round is a number of search iterations (a node count would lag:
    a branched node's children are counted when its subtree is done)."""

    default_budget = 64

    def __init__(self, ctx, best: int = 99999, window: int = 0, capacity: int = 0,
                 family_smem_kb: int = 0, graph_iters: int = 0):
        self.ctx, self.n = ctx, ctx.n
        self.kw = dict(best=best, window=window, capacity=capacity)
        # the iteration budget is checked between graph launches of
        # graph_iters iterations
        self.run_kw = dict(family_smem_kb=family_smem_kb, graph_iters=graph_iters)
        self._perm_key, self._perm_cost = None, INT32_MAX

    def _own(self, st: dict) -> dict:
        perm = st["best_perm"]
        if perm[0] < 0:
            st["perm_cost"] = INT32_MAX
        else:
            key = perm.tobytes()
            if key != self._perm_key:
                self._perm_key, self._perm_cost = key, makespan(self.ctx.p, perm)
            st["perm_cost"] = self._perm_cost
        return st

    def start_root(self, ub: int, budget: int) -> dict:
        from .explorer import explore
        return self._own(explore(self.ctx, ub0=ub, max_iters=budget, **self.run_kw,
                                 **self.kw))

    def seed(self, records: np.ndarray, lbs: np.ndarray, ub: int) -> None:
        from .explorer import explore_seed
        explore_seed(self.ctx, records, lbs, ub0=ub, **self.kw)

    def run(self, ub: int, budget: int) -> dict:
        from .explorer import explore
        return self._own(explore(self.ctx, ub0=ub, resume=True, max_iters=budget,
                                 **self.run_kw, **self.kw))

    def export(self, max_count: int):
        from .explorer import explore_export
        return explore_export(self.ctx, max_count)


# ------------------------------------------------------------------- the peer

@dataclass
class PeerResult:
    best_cost: int
    best_perm: np.ndarray | None
    counters: dict = field(default_factory=dict)  # this peer's, summed over its segments
    coverage: int = 0          # this peer's sum of (n - depth)! over pruned nodes and leaves
    rounds: int = 0
    sent: int = 0              # nodes handed to other peers
    received: int = 0          # nodes taken from other peers
    total: dict = field(default_factory=dict)  # all peers' counters summed
    total_coverage: int = 0
    complete: bool = False     # every peer idle (False: max_rounds ran out)


def peer_search(engine, transport, n: int, ub0: int | None = None, budget: int | None = None,
                share: int = 4096, max_rounds: int = 1_000_000) -> PeerResult:
    """Run one peer of a shared search to its end (every peer calls this).

    Rank 0 starts at the root; the others start idle and get work by
    hand-off. `budget`: the engine's work per round (GpuEngine: search
    iterations; default engine.default_budget); `share`: at most this many
    nodes per hand-off. Returns this peer's result; best_cost, the
    permutation and the totals are the same on every peer.
    """
    rank, world = transport.rank, transport.world
    if budget is None:
        budget = engine.default_budget
    ub = INT32_MAX if ub0 is None else int(ub0)
    res = PeerResult(best_cost=ub, best_perm=None,
                     counters={k: 0 for k in COUNTERS})
    busy = False

    def close_segment(st):
        # a seed restarts the engine's counters: bank the finished segment's
        if st is None:
            return
        for k in COUNTERS:
            res.counters[k] += int(st[k])
        res.coverage += int(st["coverage"])

    own_cost, own_perm = INT32_MAX, None
    st = None
    if rank == 0:
        st = engine.start_root(ub, budget)
        busy = st["status"] != 0
    for rnd in range(max_rounds):
        res.rounds = rnd + 1
        if busy:
            st = engine.run(ub, budget)
            busy = st["status"] != 0
        if st is not None and st["perm_cost"] < own_cost:
            own_cost, own_perm = int(st["perm_cost"]), st["best_perm"].copy()
        mine = min(ub, int(st["best_cost"]) if st is not None else INT32_MAX)
        views = transport.allgather([mine, 0 if busy else 1])
        ub = min(v[0] for v in views)
        idle = [r for r in range(world) if views[r][1]]
        if len(idle) == world:
            res.complete = True
            break
        donors = [r for r in range(world) if not views[r][1]]
        # receiver i (in rank order) is served by donor i mod len(donors)
        pairs = [(donors[i % len(donors)], r) for i, r in enumerate(idle)]
        for d, r in pairs:
            if rank == d:
                recs, lbs = engine.export(share)
                res.sent += len(recs)
                transport.send(r, formats.pack_work(recs, n, lbs, max_nbjobs=n))
            elif rank == r:
                data = transport.recv(d)
                recs, lbs, _, _ = formats.unpack_work(data, n, max_nbjobs=n)
                if len(recs):
                    close_segment(st)
                    st = None
                    engine.seed(recs, lbs, ub)
                    res.received += len(recs)
                    busy = True
    close_segment(st)
    res.best_cost = ub
    # the permutation comes from the peer that found the final cost
    owners = transport.allgather([own_cost, rank])
    holder = min((c, r) for c, r in owners)[1] if min(c for c, _ in owners) == ub else -1
    if holder >= 0:
        if rank == holder:
            for r in range(world):
                if r != rank:
                    transport.send(r, np.asarray(own_perm, dtype="<i4").tobytes())
            res.best_perm = np.asarray(own_perm, dtype=np.int32)
        else:
            res.best_perm = np.frombuffer(transport.recv(holder), dtype="<i4").astype(np.int32)
    # totals over all peers (coverage reaches n!: sent as 32-bit limbs)
    nlimbs = math.factorial(n).bit_length() // 32 + 2
    limbs = [(res.coverage >> (32 * i)) & 0xFFFFFFFF for i in range(nlimbs)]
    gathered = transport.allgather([res.counters[k] for k in COUNTERS] + limbs)
    res.total = {k: sum(g[i] for g in gathered) for i, k in enumerate(COUNTERS)}
    res.total_coverage = sum(sum(l << (32 * i) for i, l in enumerate(g[len(COUNTERS):]))
                             for g in gathered)
    return res
