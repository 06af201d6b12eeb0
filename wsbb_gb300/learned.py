"""Python front end of the learned pair selector (include/wsbb_gb300.h).

Device buffers are passed as raw pointers (torch tensors' data_ptr() in the
tests and the bench); the model's weights live on the device.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import WsbbError, lib
from .bound import Context
from .explorer import CHILD_LB2, INT32_MAX, ExploreCfg, ExploreStats, coverage

_declared = False


def _L():
    global _declared
    L = lib()
    if not _declared:
        vp, i64 = C.c_void_p, C.c_int64
        L.wsbb_model_create.argtypes = [C.c_int, C.c_int, C.c_uint64, C.POINTER(vp)]
        L.wsbb_model_destroy.argtypes = [vp]
        L.wsbb_model_last_error.restype = C.c_char_p
        L.wsbb_model_last_error.argtypes = [vp]
        L.wsbb_model_dims.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                      C.POINTER(C.c_int64)]
        L.wsbb_model_get_weights.argtypes = [vp, vp, i64]
        L.wsbb_model_set_weights.argtypes = [vp, vp, i64]
        L.wsbb_model_pack.argtypes = [vp]
        L.wsbb_feature_scale.restype = C.c_float
        L.wsbb_feature_scale.argtypes = [vp]
        L.wsbb_features.argtypes = [vp, vp, i64, C.c_float, C.c_int, vp, vp, vp]
        L.wsbb_model_grads.argtypes = [vp, vp, vp, C.c_int, vp, vp]
        L.wsbb_model_train.argtypes = [vp, vp, vp, i64, C.c_int, C.c_int, C.c_float, C.c_uint64,
                                       vp]
        L.wsbb_model_topk.argtypes = [vp, vp, i64, C.c_int, vp, vp, vp]
        L.wsbb_explore_learned.argtypes = [vp, vp, vp, C.c_int, vp, vp]
        L.wsbb_explore_log.argtypes = [vp, vp, vp, i64, C.c_int, C.POINTER(C.c_int64), vp, vp]
        L.wsbb_explore.argtypes = [vp, vp, vp, vp]
        _declared = True
    return L


class Model:
    """The pair-selector MLP (D -> 128 -> 128 -> P, ReLU) on the GPU."""

    def __init__(self, n: int, m: int, seed: int = 0):
        h = C.c_void_p()
        rc = _L().wsbb_model_create(n, m, seed, C.byref(h))
        if rc != 0:
            raise WsbbError(rc, "wsbb_model_create")
        self.h = h
        self.n, self.m, self.P = n, m, m * (m - 1) // 2
        D, O, npar = C.c_int(), C.c_int(), C.c_int64()
        _L().wsbb_model_dims(h, C.byref(D), C.byref(O), C.byref(npar))
        self.D, self.O, self.nparams = D.value, O.value, npar.value

    def close(self):
        if getattr(self, "h", None):
            _L().wsbb_model_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            raise WsbbError(rc, _L().wsbb_model_last_error(self.h).decode())

    def get_weights(self) -> np.ndarray:
        w = np.empty(self.nparams, dtype=np.float32)
        self._check(_L().wsbb_model_get_weights(self.h, w.ctypes.data, self.nparams))
        return w

    def set_weights(self, w: np.ndarray) -> None:
        w = np.ascontiguousarray(w, dtype=np.float32)
        self._check(_L().wsbb_model_set_weights(self.h, w.ctypes.data, self.nparams))

    def save(self, path: str) -> None:
        np.savez_compressed(path, w=self.get_weights(), n=self.n, m=self.m)

    def load(self, path: str) -> None:
        z = np.load(path)
        assert int(z["n"]) == self.n and int(z["m"]) == self.m
        self.set_weights(z["w"])

    def grads(self, X_ptr: int, y_ptr: int, B: int):
        g = np.empty(self.nparams, dtype=np.float32)
        loss = C.c_float()
        self._check(_L().wsbb_model_grads(self.h, X_ptr, y_ptr, B, g.ctypes.data, C.byref(loss)))
        return g, float(loss.value)

    def train(self, X_ptr: int, y_ptr: int, count: int, epochs: int = 3, batch: int = 4096,
              lr: float = 1e-3, seed: int = 0) -> list[float]:
        losses = np.zeros(epochs, dtype=np.float32)
        self._check(_L().wsbb_model_train(self.h, X_ptr, y_ptr, count, epochs, batch, lr, seed,
                                          losses.ctypes.data))
        return [float(x) for x in losses]

    def topk(self, X_ptr: int, rows: int, K: int, topk_ptr: int, logits_ptr: int = 0,
             stream: int = 0) -> None:
        self._check(_L().wsbb_model_topk(self.h, X_ptr, rows, K, topk_ptr, logits_ptr or None,
                                         stream or None))


def feature_scale(ctx: Context) -> float:
    return float(_L().wsbb_feature_scale(ctx.h))


def features(ctx: Context, recs_ptr: int, count: int, D: int, X_ptr: int, labels_ptr: int = 0,
             stream: int = 0) -> None:
    rc = _L().wsbb_features(ctx.h, recs_ptr, count, feature_scale(ctx), D, X_ptr,
                            labels_ptr or None, stream or None)
    if rc != 0:
        raise WsbbError(rc, "wsbb_features")


def _stats_dict(st: ExploreStats, n: int) -> dict:
    return {"branched": st.branched, "pruned": st.pruned, "leaves": st.leaves,
            "improved": st.improved, "bounded": st.bounded, "evaluated": st.evaluated,
            "discarded": st.discarded, "iterations": st.iterations,
            "best_cost": st.best_cost, "status": st.status,
            "coverage": coverage(st.depth_hist, n), "seconds": st.seconds,
            "early": st.early, "settled_fathers": st.settled_fathers, "best_perm": np.array(st.best_perm[:n], dtype=np.int32)}


def explore_learned(ctx: Context, model: Model, K: int, ub0: int | None = None,
                    best: int | None = None, window: int = 0, max_iters: int = 0,
                    graph_iters: int = 0, stream: int = 0, child_lb2: bool = False,
                    capacity: int = 0, family_smem_kb: int = 0, max_bounded: int = 0) -> dict:
    """The exact search with the learned K-pair test; `best` defaults to ub0.
    `child_lb2`: the test and the full-LB2 fallback per child record (the
    per-node kernels) instead of per father (family bounds)."""
    ub = INT32_MAX if ub0 is None else int(ub0)
    cfg = ExploreCfg(ub, int(ub if best is None else best), int(window), int(graph_iters),
                     int(capacity), int(max_iters), CHILD_LB2 if child_lb2 else 0,
                     int(family_smem_kb), int(max_bounded))
    st = ExploreStats()
    rc = _L().wsbb_explore_learned(ctx.h, C.byref(cfg), model.h, int(K), C.byref(st),
                                   stream or None)
    if rc != 0:
        raise WsbbError(rc, lib().wsbb_last_error(ctx.h).decode())
    return _stats_dict(st, ctx.n)


def log_nodes(ctx: Context, recs_ptr: int, cap: int, stride: int, ub0: int | None = None,
              best: int = 99999, window: int = 0, max_iters: int = 0, stream: int = 0):
    """Plain search that copies a sample of its bounded children (training data)."""
    cfg = ExploreCfg(INT32_MAX if ub0 is None else int(ub0), int(best), int(window), 0, 0,
                     int(max_iters), 0, 0)
    st = ExploreStats()
    got = C.c_int64()
    rc = _L().wsbb_explore_log(ctx.h, C.byref(cfg), recs_ptr, cap, stride, C.byref(got),
                               C.byref(st), stream or None)
    if rc != 0:
        raise WsbbError(rc, lib().wsbb_last_error(ctx.h).decode())
    return int(got.value), _stats_dict(st, ctx.n)
