"""Python mirror of the reference's bound plugin over the GB300 library.

`BoundFlowshopGB300` follows bound_abstract / bound_flowshop
(headers/bound_abstract.h:9-19, src/bound_flowshop.cpp:929-956):
set_instance() runs the precompute, bornes_calculer() bounds one node with
the reference's argument meaning (limite1 = last front position,
limite2 = first back position, couts[0] <- LB, couts[1] <- 0) and
bornes_calculer_pool() bounds a whole pool in one launch — the form the
reference's GPU path (Evaluate_ON_GPU, src/bound_flowshop_gpu.cu:619-674)
uses.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import WsbbError, check, lib


def node_stride(n: int) -> int:
    """Bytes per node record (int16 job[n], limite1, limite2, depth, pad)."""
    return int(lib().wsbb_node_stride(n))


def pack_records(perms, limite1, limite2, depth=None) -> np.ndarray:
    """Pack a pool into the record format; returns a (count, stride/2) int16 array."""
    perms = np.asarray(perms)
    count, n = perms.shape
    w = node_stride(n) // 2
    rec = np.zeros((count, w), dtype=np.int16)
    rec[:, :n] = perms
    l1 = np.asarray(limite1)
    l2 = np.asarray(limite2)
    rec[:, n] = l1
    rec[:, n + 1] = l2
    rec[:, n + 2] = (l1 + 1) + (n - l2) if depth is None else np.asarray(depth)
    return rec


def unpack_records(rec: np.ndarray, n: int):
    rec = np.asarray(rec).reshape(len(rec), -1)
    return (rec[:, :n].astype(np.int32), rec[:, n].astype(np.int32),
            rec[:, n + 1].astype(np.int32))


def expand_children(rec: np.ndarray, n: int):
    """Children of father records in the library's order (host restatement
    of the begin-end branching, src/decompose_beginend.cpp:26-89 with
    bb_problem_calculator::create_raw_problem3 / limites_set,
    src/bb_problem_calculator.cpp:25-48): per father, the u BEGIN children
    (free position l1+1+k moved to l1+1) then the u END children (moved to
    l2-1); a father with two free jobs has the two orders of them as leaves.
    Returns (child records, child_off) with child_off[f] the first child of
    father f."""
    rec = np.asarray(rec)
    out, off = [], [0]
    for r in rec:
        l1, l2, depth = int(r[n]), int(r[n + 1]), int(r[n + 2])
        u = l2 - l1 - 1
        kids = []
        if u == 2:
            for k in range(2):
                c = r.copy()
                c[l1 + 1], c[l1 + 1 + k] = r[l1 + 1 + k], r[l1 + 1]
                c[n], c[n + 1], c[n + 2] = l1 + 2, l2, n
                kids.append(c)
        else:
            for side in (0, 1):
                for k in range(u):
                    c = r.copy()
                    ind = l1 + 1 + k
                    slot = l2 - 1 if side else l1 + 1
                    c[ind], c[slot] = r[slot], r[ind]
                    c[n], c[n + 1] = (l1, l2 - 1) if side else (l1 + 1, l2)
                    c[n + 2] = depth + 1
                    kids.append(c)
        out.extend(kids)
        off.append(off[-1] + len(kids))
    return np.array(out, dtype=np.int16).reshape(-1, rec.shape[1]), np.array(off, np.int64)


def gen_instance(seed: int, n: int, m: int) -> np.ndarray:
    """Seeded instance: p[k, j] uniform in [1, 99] (SplitMix64, machine-major)."""
    p = np.empty(m * n, dtype=np.int32)
    lib().wsbb_gen_instance(seed, n, m, p.ctypes.data)
    return p.reshape(m, n)


def taillard_instance(seed: int, n: int, m: int) -> np.ndarray:
    """Instance from Taillard's generator with time seed `seed`, as the
    reference's instance_flowshop draws it (machine-major m x n)."""
    p = np.empty(m * n, dtype=np.int32)
    rc = lib().wsbb_taillard_instance(int(seed), n, m, p.ctypes.data)
    if rc != 0:
        raise ValueError(f"wsbb_taillard_instance: error {rc}")
    return p.reshape(m, n)


def gen_pool(seed: int, n: int, count: int, leaf_share: float = 0.0) -> np.ndarray:
    """Seeded random pool in the record format."""
    rec = np.empty((count, node_stride(n) // 2), dtype=np.int16)
    rc = lib().wsbb_gen_pool(seed, n, count, leaf_share, rec.ctypes.data)
    if rc != 0:
        raise WsbbError(rc, "gen_pool")
    return rec


def neh(p: np.ndarray):
    """NEH upper bound: (makespan, sequence)."""
    p = np.ascontiguousarray(p, dtype=np.int32)
    m, n = p.shape
    perm = np.empty(n, dtype=np.int32)
    c = lib().wsbb_neh(p.ctypes.data, n, m, perm.ctypes.data)
    return int(c), perm


class Context:
    """An instance resident on one GPU (wsbb_ctx)."""

    def __init__(self, p: np.ndarray, device: int = 0):
        self.p = np.ascontiguousarray(p, dtype=np.int32)
        self.m, self.n = self.p.shape
        self.P = self.m * (self.m - 1) // 2
        self.stride = node_stride(self.n)
        h = C.c_void_p()
        rc = lib().wsbb_ctx_create(self.p.ctypes.data, self.n, self.m, device, C.byref(h))
        if rc != 0:
            raise WsbbError(rc, "wsbb_ctx_create")
        self.h = h

    def close(self) -> None:
        if getattr(self, "h", None):
            lib().wsbb_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def tables(self) -> dict:
        P, n, m = self.P, self.n, self.m
        out = {k: np.empty(s, dtype=np.int32) for k, s in
               [("mach0", P), ("mach1", P), ("lag", P * n), ("johnson", P * n),
                ("heads", m), ("tails", m)]}
        check(self.h, lib().wsbb_ctx_tables(self.h, *(out[k].ctypes.data for k in
                                                      ("mach0", "mach1", "lag", "johnson",
                                                       "heads", "tails"))))
        out["lag"] = out["lag"].reshape(P, n)
        out["johnson"] = out["johnson"].reshape(P, n)
        return out

    # device-pointer entry points (stream-ordered, asynchronous)
    def lb2_eval(self, recs_ptr: int, count: int, out_ptr: int, stream: int = 0) -> None:
        check(self.h, lib().wsbb_lb2_eval(self.h, recs_ptr, count, out_ptr, stream or None))

    def lb1_eval(self, recs_ptr: int, count: int, out_ptr: int, stream: int = 0) -> None:
        check(self.h, lib().wsbb_lb1_eval(self.h, recs_ptr, count, out_ptr, stream or None))

    def makespan_eval(self, recs_ptr: int, count: int, out_ptr: int, stream: int = 0) -> None:
        check(self.h, lib().wsbb_makespan_eval(self.h, recs_ptr, count, out_ptr,
                                               stream or None))

    def decompose_lb2(self, fathers_ptr: int, count: int, child_off_ptr: int, lb_ptr: int,
                      job_ptr: int, stream: int = 0) -> None:
        """Bounds of every child of `count` father records (device), in the
        order of expand_children; child_off (int64, count + 1) on the device."""
        check(self.h, lib().wsbb_decompose_lb2(self.h, fathers_ptr, count, child_off_ptr, lb_ptr,
                                               job_ptr, stream or None))

    # host-buffer entry point (synchronous)
    def lb2_eval_host(self, recs: np.ndarray, out: np.ndarray | None = None) -> np.ndarray:
        recs = np.ascontiguousarray(recs, dtype=np.int16)
        count = recs.shape[0]
        if out is None:
            out = np.empty(count, dtype=np.int32)
        check(self.h, lib().wsbb_lb2_eval_host(self.h, recs.ctypes.data, count,
                                               out.ctypes.data))
        return out


class BoundFlowshopGB300:
    """bound_abstract-shaped plugin: set_instance + bornes_calculer."""

    def __init__(self, device: int = 0):
        self.device = device
        self.ctx: Context | None = None

    def set_instance(self, p: np.ndarray) -> None:
        self.ctx = Context(p, self.device)

    def bornes_calculer(self, permutation, limite1: int, limite2: int, couts, best: int = 999999):
        """Bound one node into couts[0] (couts[1] = 0), like the reference.

        `best` is accepted for interface parity; the reference's own callers
        pass 999999, which never triggers its early exit.
        """
        rec = pack_records(np.asarray(permutation, dtype=np.int16)[None, :self.ctx.n],
                           [limite1], [limite2])
        couts[0] = int(self.ctx.lb2_eval_host(rec)[0])
        couts[1] = 0

    def bornes_calculer_pool(self, recs: np.ndarray) -> np.ndarray:
        return self.ctx.lb2_eval_host(recs)
