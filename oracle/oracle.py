"""TEST INFRASTRUCTURE — ctypes front end of the CPU oracle.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
import this module, and only as the checker (or the timed CPU port). It
loads oracle/_build/liboracle.so (the C restatement, flowshop_oracle.c) and,
where it was built, oracle/_ref/libref_bound.so + oracle/_ref/ref_explore
(the reference's own compiled code; present only in the build container).
"""
from __future__ import annotations

import ctypes as C
import json
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(HERE, "_build", "liboracle.so")
_REF_LIB = os.path.join(HERE, "_ref", "libref_bound.so")
_REF_EXPLORE = os.path.join(HERE, "_ref", "ref_explore")
# the reference's search built with MAX_NBJOBS = 64 (oracle/build.sh)
_REF_EXPLORE_BIG = os.path.join(HERE, "_ref", "ref_explore_big")

INT32_MAX = 2**31 - 1

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def build() -> None:
    subprocess.run(["sh", os.path.join(HERE, "build.sh")], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB):
            build()
        L = C.CDLL(_LIB)
        L.fs_gen_instance.argtypes = [C.c_uint64, C.c_int, C.c_int, _i32p]
        L.fs_taillard_instance.argtypes = [C.c_int64, C.c_int, C.c_int, _i32p]
        L.fs_bound_create.restype = C.c_void_p
        L.fs_bound_create.argtypes = [_i32p, C.c_int, C.c_int]
        L.fs_bound_destroy.argtypes = [C.c_void_p]
        L.fs_bound_pairs.argtypes = [C.c_void_p]
        L.fs_bound_tables.argtypes = [C.c_void_p] + [_i32p] * 6
        L.fs_bound_eval.restype = C.c_int32
        L.fs_bound_eval.argtypes = [C.c_void_p, _i32p, C.c_int, C.c_int, C.c_int32,
                                    C.POINTER(C.c_int32)]
        L.fs_bound_eval_pairs.restype = C.c_int32
        L.fs_bound_eval_pairs.argtypes = [C.c_void_p, _i32p, C.c_int, C.c_int, _i32p, C.c_int]
        L.fs_lb1_eval.restype = C.c_int32
        L.fs_makespan.restype = C.c_int32
        L.fs_makespan.argtypes = [C.c_void_p, _i32p]
        L.fs_bound_eval_batch.argtypes = [C.c_void_p, _i32p, _i32p, _i32p, C.c_int64,
                                          _i32p, C.c_void_p, C.c_int]
        L.fs_explore_seeded.argtypes = [C.c_void_p, _i32p, _i32p, _i32p, _i32p, C.c_int64,
                                        C.c_int32, C.c_int32, C.c_int64, C.c_void_p,
                                        C.c_void_p]
        L.fs_lb1_eval_batch.argtypes = [C.c_void_p, _i32p, _i32p, _i32p, C.c_int64, _i32p]
        L.fs_random_pool.argtypes = [C.c_uint64, C.c_int, C.c_int64, C.c_double,
                                     _i32p, _i32p, _i32p]
        L.fs_neh.restype = C.c_int32
        L.fs_neh.argtypes = [_i32p, C.c_int, C.c_int, _i32p]
        L.fs_explore.restype = C.c_int
        L.fs_explore.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int64,
                                 C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib = L
    return _lib


class FsStats(C.Structure):
    _fields_ = [("branched", C.c_int64), ("pruned", C.c_int64), ("leaves", C.c_int64),
                ("improved", C.c_int64), ("bounded", C.c_int64),
                ("early_exits", C.c_int64), ("best_cost", C.c_int32), ("pad", C.c_int32),
                ("depth_hist", C.c_uint64 * 129)]

    def as_dict(self, n: int) -> dict:
        """Counters; coverage = sum over pruned nodes and leaves of
        (n - depth)! (src/weights.cpp:11-22), in exact integers."""
        import math
        return {"branched": self.branched, "pruned": self.pruned, "leaves": self.leaves,
                "improved": self.improved, "bounded": self.bounded,
                "early_exits": self.early_exits, "best_cost": self.best_cost,
                "coverage": sum(int(self.depth_hist[d]) * math.factorial(n - d)
                                for d in range(n + 1))}


LOG_CB = C.CFUNCTYPE(None, C.POINTER(C.c_int32), C.c_int, C.c_int, C.c_int32, C.c_int32,
                     C.c_void_p)
SEL_CB = C.CFUNCTYPE(C.c_int, C.POINTER(C.c_int32), C.c_int, C.c_int, C.POINTER(C.c_int32),
                     C.c_void_p)


def gen_instance(seed: int, n: int, m: int) -> np.ndarray:
    p = np.empty(m * n, dtype=np.int32)
    lib().fs_gen_instance(seed, n, m, p)
    return p.reshape(m, n)


def taillard_instance(seed: int, n: int, m: int) -> np.ndarray:
    p = np.empty(m * n, dtype=np.int32)
    lib().fs_taillard_instance(seed, n, m, p)
    return p.reshape(m, n)


def random_pool(seed: int, n: int, count: int, leaf_share: float = 0.0):
    perms = np.empty((count, n), dtype=np.int32)
    l1 = np.empty(count, dtype=np.int32)
    l2 = np.empty(count, dtype=np.int32)
    lib().fs_random_pool(seed, n, count, leaf_share, perms, l1, l2)
    return perms, l1, l2


def neh(p: np.ndarray):
    m, n = p.shape
    perm = np.empty(n, dtype=np.int32)
    c = lib().fs_neh(np.ascontiguousarray(p, dtype=np.int32).ravel(), n, m, perm)
    return int(c), perm


class Bound:
    """The oracle bound for one instance (bound_flowshop restated)."""

    def __init__(self, p: np.ndarray):
        self.p = np.ascontiguousarray(p, dtype=np.int32)
        self.m, self.n = self.p.shape
        self.h = lib().fs_bound_create(self.p.ravel(), self.n, self.m)
        if not self.h:
            raise ValueError("oracle: unsupported instance size")
        self.P = lib().fs_bound_pairs(self.h)

    def __del__(self):
        h = getattr(self, "h", None)
        if h and _lib is not None:
            _lib.fs_bound_destroy(h)
            self.h = None

    def tables(self) -> dict:
        P, n, m = self.P, self.n, self.m
        out = {k: np.empty(s, dtype=np.int32) for k, s in
               [("mach0", P), ("mach1", P), ("lag", P * n), ("johnson", P * n),
                ("min_arr", m), ("min_dep", m)]}
        lib().fs_bound_tables(self.h, out["mach0"], out["mach1"], out["lag"],
                              out["johnson"], out["min_arr"], out["min_dep"])
        out["lag"] = out["lag"].reshape(P, n)
        out["johnson"] = out["johnson"].reshape(P, n)
        return out

    def eval(self, perm, l1: int, l2: int, best: int = -1):
        a = C.c_int32(-1)
        v = lib().fs_bound_eval(self.h, np.ascontiguousarray(perm, dtype=np.int32), l1, l2,
                                best, C.byref(a))
        return int(v), int(a.value)

    def eval_pairs(self, perm, l1: int, l2: int, pairs) -> int:
        pr = np.ascontiguousarray(pairs, dtype=np.int32)
        return int(lib().fs_bound_eval_pairs(self.h, np.ascontiguousarray(perm, dtype=np.int32),
                                             l1, l2, pr, len(pr)))

    def eval_batch(self, perms, l1, l2, nthreads: int = 1, want_argmax: bool = False):
        perms = np.ascontiguousarray(perms, dtype=np.int32)
        l1 = np.ascontiguousarray(l1, dtype=np.int32)
        l2 = np.ascontiguousarray(l2, dtype=np.int32)
        cnt = len(l1)
        out = np.empty(cnt, dtype=np.int32)
        arg = np.empty(cnt, dtype=np.int32) if want_argmax else None
        lib().fs_bound_eval_batch(self.h, perms, l1, l2, cnt, out,
                                  arg.ctypes.data if want_argmax else None, nthreads)
        return (out, arg) if want_argmax else out

    def lb1_batch(self, perms, l1, l2):
        perms = np.ascontiguousarray(perms, dtype=np.int32)
        l1 = np.ascontiguousarray(l1, dtype=np.int32)
        l2 = np.ascontiguousarray(l2, dtype=np.int32)
        out = np.empty(len(l1), dtype=np.int32)
        lib().fs_lb1_eval_batch(self.h, perms, l1, l2, len(l1), out)
        return out

    def makespan(self, perm) -> int:
        return int(lib().fs_makespan(self.h, np.ascontiguousarray(perm, dtype=np.int32)))

    def explore(self, ub0: int | None = None, best: int = 99999, node_cap: int = 0,
                log=None, pair_sel=None):
        """Sequential DFS with the reference's semantics; returns (rc, stats, perm)."""
        st = FsStats()
        perm = np.full(self.n, -1, dtype=np.int32)
        lcb = LOG_CB(log) if log is not None else None
        scb = SEL_CB(pair_sel) if pair_sel is not None else None
        rc = lib().fs_explore(self.h, INT32_MAX if ub0 is None else int(ub0), int(best),
                              int(node_cap), C.byref(st), perm.ctypes.data,
                              C.cast(lcb, C.c_void_p) if lcb else None,
                              C.cast(scb, C.c_void_p) if scb else None, None)
        return rc, st.as_dict(self.n), perm

    def explore_seeded(self, perms, l1, l2, lbs, ub0: int | None = None, best: int = 99999,
                       node_cap: int = 0):
        """The sequential DFS over the subtrees of given open nodes (row 0 at
        the stack bottom, the last row taken first); returns (rc, stats, perm)."""
        perms = np.ascontiguousarray(perms, dtype=np.int32).reshape(-1, self.n)
        l1 = np.ascontiguousarray(l1, dtype=np.int32)
        l2 = np.ascontiguousarray(l2, dtype=np.int32)
        lbs = np.ascontiguousarray(lbs, dtype=np.int32)
        st = FsStats()
        perm = np.full(self.n, -1, dtype=np.int32)
        rc = lib().fs_explore_seeded(self.h, perms, l1, l2, lbs, len(l1),
                                     INT32_MAX if ub0 is None else int(ub0), int(best),
                                     int(node_cap), C.byref(st), perm.ctypes.data)
        return rc, st.as_dict(self.n), perm


# ---------------------------------------------------------------- reference

def have_reference() -> bool:
    return os.path.exists(_REF_LIB) and os.path.exists(_REF_EXPLORE)


def have_reference_big() -> bool:
    return have_reference() and os.path.exists(_REF_EXPLORE_BIG)


_ref = None


def ref_lib():
    global _ref
    if _ref is None:
        R = C.CDLL(_REF_LIB)
        R.ref_bound_create.restype = C.c_void_p
        R.ref_bound_create.argtypes = [_i32p, C.c_int, C.c_int]
        R.ref_bound_eval.argtypes = [C.c_void_p, _i32p, _i32p, _i32p, C.c_int64, _i32p,
                                     C.c_void_p]
        R.ref_bound_eval_mt.argtypes = [_i32p, C.c_int, C.c_int, _i32p, _i32p, _i32p,
                                        C.c_int64, _i32p, C.c_int]
        _ref = R
    return _ref


class RefBound:
    """The reference's own bound_flowshop (compiled in place, oracle/_ref)."""

    def __init__(self, p: np.ndarray):
        self.p = np.ascontiguousarray(p, dtype=np.int32)
        self.m, self.n = self.p.shape
        self.h = ref_lib().ref_bound_create(self.p.ravel(), self.n, self.m)

    def eval_batch(self, perms, l1, l2, want_argmax: bool = False):
        perms = np.ascontiguousarray(perms, dtype=np.int32)
        l1 = np.ascontiguousarray(l1, dtype=np.int32)
        l2 = np.ascontiguousarray(l2, dtype=np.int32)
        out = np.empty(len(l1), dtype=np.int32)
        arg = np.empty(len(l1), dtype=np.int32)
        ref_lib().ref_bound_eval(self.h, perms, l1, l2, len(l1), out, arg.ctypes.data)
        return (out, arg) if want_argmax else out

    def eval_batch_mt(self, perms, l1, l2, nthreads: int):
        perms = np.ascontiguousarray(perms, dtype=np.int32)
        out = np.empty(len(l1), dtype=np.int32)
        ref_lib().ref_bound_eval_mt(self.p.ravel(), self.n, self.m, perms,
                                    np.ascontiguousarray(l1, dtype=np.int32),
                                    np.ascontiguousarray(l2, dtype=np.int32), len(l1), out,
                                    nthreads)
        return out


def ref_taillard_instance(seed: int, n: int, m: int) -> np.ndarray:
    """The reference's own instance_flowshop::unif stream for `seed`."""
    R = ref_lib()
    R.ref_taillard.argtypes = [C.c_long, C.c_int, C.c_int, _i32p]
    p = np.empty(m * n, dtype=np.int32)
    R.ref_taillard(seed, n, m, p)
    return p.reshape(m, n)


def ref_explore(p: np.ndarray, ub0: int | None = None, best: int = 99999,
                timeout: float = 600.0, workdir: str | None = None) -> dict:
    """Run the reference's CPU search (oracle/_ref/ref_explore) on `p`.
    `workdir`: the working directory, where the reference reads its initial
    incumbents from bab.solutions (with ub0 None, a file already there is
    kept) and appends every improvement to it; a temporary one if None.
    Instances with n > 20 run on the reference's sources rebuilt with
    MAX_NBJOBS = 64 (oracle/_ref/ref_explore_big)."""
    m, n = p.shape
    exe = _REF_EXPLORE if n <= 20 else _REF_EXPLORE_BIG
    if n > 64:
        raise ValueError("the reference's search is built for n <= 64")
    with tempfile.TemporaryDirectory() as tmp:
        d = workdir or tmp
        r = subprocess.run([exe, str(n), str(m), str(-1 if ub0 is None else ub0),
                            str(best), d.rstrip("/") + "/"],
                           input=" ".join(str(int(x)) for x in p.ravel()),
                           capture_output=True, text=True, timeout=timeout, check=True)
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("RESULT ")][-1]
    return json.loads(line[len("RESULT "):])
