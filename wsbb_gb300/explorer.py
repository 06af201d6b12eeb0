"""Python front end of the GPU search (wsbb_explore).

`explore()` mirrors the reference CPU search (src/explorer.cu:92-148) with
the same node semantics; the returned dict uses the reference's counter
names where one exists (branched = cpu_explored_nodes, pruned =
boundedNodesDontExplore).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from ._lib import WsbbError, lib
from .bound import Context, node_stride

INT32_MAX = 2**31 - 1
MAX_JOBS = 128


class ExploreCfg(C.Structure):
    _fields_ = [("ub0", C.c_int32), ("best", C.c_int32), ("window", C.c_int32),
                ("graph_iters", C.c_int32), ("capacity", C.c_int64), ("max_iters", C.c_int64),
                ("flags", C.c_int32), ("family_smem_kb", C.c_int32),
                ("max_bounded", C.c_int64)]


class ExploreStats(C.Structure):
    _fields_ = [("branched", C.c_int64), ("pruned", C.c_int64), ("leaves", C.c_int64),
                ("improved", C.c_int64), ("bounded", C.c_int64), ("evaluated", C.c_int64),
                ("discarded", C.c_int64), ("iterations", C.c_int64), ("best_cost", C.c_int32),
                ("status", C.c_int32), ("depth_hist", C.c_uint64 * (MAX_JOBS + 1)),
                ("best_perm", C.c_int32 * MAX_JOBS), ("seconds", C.c_double),
                ("scanned", C.c_int64), ("committed", C.c_int64), ("early", C.c_int64),
                ("settled_fathers", C.c_int64), ("d2h_bytes", C.c_int64),
                ("takes", C.c_int64), ("pending", C.c_int64),
                ("pending_hist", C.c_uint32 * (MAX_JOBS + 1))]


NO_GRAPH = 1
CHILD_LB2 = 2  # bound every child record on its own instead of per father (same bounds)
RESUME = 4     # continue the context's stopped or seeded search
RESIDENT = 8   # run as the resident search (one cooperative launch)


class ResidentOpts(C.Structure):
    _fields_ = [("wait_ms", C.c_int32), ("self_test", C.c_int32), ("group_ctas", C.c_int32)]


def coverage(hist, n: int) -> int:
    """Sum over pruned nodes and leaves of (n - depth)! (weights.cpp)."""
    return sum(int(hist[d]) * math.factorial(n - d) for d in range(n + 1))


def _cfg(ub0, best, window, graph_iters, capacity, max_iters, flags, family_smem_kb,
         max_bounded) -> ExploreCfg:
    return ExploreCfg(INT32_MAX if ub0 is None else int(ub0), int(best), int(window),
                      int(graph_iters), int(capacity), int(max_iters), flags,
                      int(family_smem_kb), int(max_bounded))


def explore(ctx: Context, ub0: int | None = None, best: int = 99999, window: int = 0,
            graph_iters: int = 0, capacity: int = 0, max_iters: int = 0, graph: bool = True,
            stream: int = 0, child_lb2: bool = False, family_smem_kb: int = 0,
            max_bounded: int = 0, resume: bool = False, resident: bool = False) -> dict:
    """The exact GPU search. `child_lb2` bounds each child record on its own
    with the per-node LB2 kernel (the reference GPU kernel's form) instead of
    each father's children together; bounds and tree are the same.
    `resume` continues the context's stopped or seeded search (same window
    and capacity; `ub0` may lower its incumbent); its counters are
    cumulative since the start or the seed."""
    L = lib()
    L.wsbb_explore.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    flags = (0 if graph else NO_GRAPH) | (CHILD_LB2 if child_lb2 else 0) | \
        (RESUME if resume else 0) | (RESIDENT if resident else 0)
    cfg = _cfg(ub0, best, window, graph_iters, capacity, max_iters, flags, family_smem_kb,
               max_bounded)
    st = ExploreStats()
    rc = L.wsbb_explore(ctx.h, C.byref(cfg), C.byref(st), stream or None)
    if rc != 0:
        raise WsbbError(rc, L.wsbb_last_error(ctx.h).decode())
    return stats_dict(st, ctx.n)


def explore_resident(ctxs, ub0s=None, bests=None, window: int = 0, capacity: int = 0,
                     max_iters: int = 0, max_bounded=0, wait_ms: int = 0,
                     self_test: bool = False, stream: int = 0, check: bool = True,
                     group_ctas: int = 0):
    """Search every context's instance in one launch of resident CTAs
    (wsbb_explore_resident): a group of at most `group_ctas` CTAs per
    instance (0: the library's default), fathers stolen between CTAs and
    from instances still running. `ub0s`, `bests`,
    `capacity`, `max_iters` and `max_bounded` may be one value for all or
    one per context. Returns
    (return code, [stats dict per instance]); with `check`, a failure
    raises."""
    L = lib()
    L.wsbb_explore_resident.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p]
    k = len(ctxs)

    def per(v, default):
        if v is None:
            return [default] * k
        return list(v) if isinstance(v, (list, tuple)) else [v] * k
    u, b, mb = per(ub0s, None), per(bests, 99999), per(max_bounded, 0)
    cap, mi = per(capacity, 0), per(max_iters, 0)
    cfgs = (ExploreCfg * k)(*[_cfg(u[i], b[i], window, 0, cap[i], mi[i], 0, 0, mb[i])
                              for i in range(k)])
    hs = (C.c_void_p * k)(*[c.h for c in ctxs])
    st = (ExploreStats * k)()
    opts = ResidentOpts(int(wait_ms), 1 if self_test else 0, int(group_ctas))
    rc = L.wsbb_explore_resident(hs, k, cfgs, C.byref(opts), st, stream or None)
    if rc != 0 and check:
        raise WsbbError(rc, L.wsbb_last_error(ctxs[0].h).decode())
    return rc, [stats_dict(st[i], ctxs[i].n) for i in range(k)]


def explore_seed(ctx: Context, records: np.ndarray, lbs, ub0: int | None = None,
                 best: int = 99999, window: int = 0, capacity: int = 0,
                 stream: int = 0) -> None:
    """Replace the context's search state by one whose stack holds the
    given open nodes (records[0] at the bottom, the last taken first) with
    their bounds; `explore(..., resume=True)` runs it."""
    L = lib()
    L.wsbb_explore_seed.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_int64, C.c_void_p]
    rec = np.ascontiguousarray(records, dtype=np.int16)
    lb = np.ascontiguousarray(lbs, dtype=np.int32)
    if rec.ndim != 2 or rec.shape[1] * 2 != node_stride(ctx.n) or len(lb) != len(rec):
        raise ValueError("records must be (count, wsbb_node_stride(n) / 2) int16 with one bound each")
    cfg = _cfg(ub0, best, window, 0, capacity, 0, 0, 0, 0)
    rc = L.wsbb_explore_seed(ctx.h, C.byref(cfg), rec.ctypes.data, lb.ctypes.data, len(rec),
                             stream or None)
    if rc != 0:
        raise WsbbError(rc, L.wsbb_last_error(ctx.h).decode())


def explore_export(ctx: Context, max_count: int, stream: int = 0):
    """Take up to `max_count` open nodes from the bottom of the context's
    stopped search: (records, bounds) in stack order, bottom first."""
    L = lib()
    L.wsbb_explore_export.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_void_p]
    rec = np.zeros((max(max_count, 0), node_stride(ctx.n) // 2), dtype=np.int16)
    lb = np.zeros(max(max_count, 0), dtype=np.int32)
    got = C.c_int64(0)
    rc = L.wsbb_explore_export(ctx.h, int(max_count), rec.ctypes.data, lb.ctypes.data,
                               C.byref(got), stream or None)
    if rc != 0:
        raise WsbbError(rc, L.wsbb_last_error(ctx.h).decode())
    return rec[:got.value].copy(), lb[:got.value].copy()


def stats_dict(st: ExploreStats, n: int) -> dict:
    return {"branched": st.branched, "pruned": st.pruned, "leaves": st.leaves,
            "improved": st.improved, "bounded": st.bounded, "evaluated": st.evaluated,
            "discarded": st.discarded, "iterations": st.iterations,
            "best_cost": st.best_cost, "status": st.status,
            "coverage": coverage(st.depth_hist, n),
            "best_perm": np.array(st.best_perm[:n], dtype=np.int32),
            "seconds": st.seconds, "scanned": st.scanned, "committed": st.committed,
            "d2h_bytes": st.d2h_bytes, "takes": st.takes, "pending": st.pending,
            "depth_hist": [int(v) for v in st.depth_hist[:n + 1]],
            "pending_hist": [int(v) for v in st.pending_hist[:n + 1]]}


def sequential_prefix(stats: dict, n: int) -> dict:
    """The sequential search's counters after exactly stats["takes"] takes
    (the point where a stopped GPU search stands): children pruned at birth
    whose take is still ahead are removed from pruned and the coverage."""
    hist = [h - p for h, p in zip(stats["depth_hist"], stats["pending_hist"])]
    return {"takes": stats["takes"], "branched": stats["branched"],
            "pruned": stats["pruned"] - stats["pending"], "leaves": stats["leaves"],
            "improved": stats["improved"], "bounded": stats["bounded"],
            "best_cost": stats["best_cost"], "coverage": coverage(hist, n)}
