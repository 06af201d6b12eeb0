"""Loader for the in-tree sm_103a library (wsbb_gb300/_build/libwsbb_gb300.so).

There is no fallback: if the library is missing the import of the bound
or search APIs raises, so nothing can silently run a CPU path instead.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libwsbb_gb300.so")

WSBB_ERRORS = {
    -1: "bad argument", -2: "CUDA error", -3: "out of memory", -4: "value out of range",
    -5: "device watchdog expired", -6: "pool capacity exceeded",
}


class WsbbError(RuntimeError):
    def __init__(self, code: int, msg: str = ""):
        super().__init__(f"wsbb error {code} ({WSBB_ERRORS.get(code, '?')}): {msg}")
        self.code = code


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is not built; run `python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(LIB_PATH)
        vp, i32p, i64 = C.c_void_p, C.POINTER(C.c_int32), C.c_int64
        L.wsbb_node_stride.restype = C.c_size_t
        L.wsbb_node_stride.argtypes = [C.c_int]
        L.wsbb_ctx_create.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.POINTER(vp)]
        L.wsbb_ctx_destroy.argtypes = [vp]
        L.wsbb_last_error.restype = C.c_char_p
        L.wsbb_last_error.argtypes = [vp]
        L.wsbb_ctx_tables.argtypes = [vp] + [vp] * 6
        for name in ("wsbb_lb2_eval", "wsbb_lb1_eval", "wsbb_makespan_eval"):
            getattr(L, name).argtypes = [vp, vp, i64, vp, vp]
        L.wsbb_precompute.argtypes = [vp, C.c_int, C.c_int] + [vp] * 6
        L.wsbb_lb2_eval_host.argtypes = [vp, vp, i64, vp]
        L.wsbb_gen_instance.argtypes = [C.c_uint64, C.c_int, C.c_int, vp]
        L.wsbb_taillard_instance.argtypes = [C.c_int64, C.c_int, C.c_int, vp]
        L.wsbb_neh.restype = C.c_int32
        L.wsbb_neh.argtypes = [vp, C.c_int, C.c_int, vp]
        L.wsbb_gen_pool.argtypes = [C.c_uint64, C.c_int, i64, C.c_double, vp]
        L.wsbb_probe_maxplus_peak.argtypes = [C.c_int, C.POINTER(C.c_double)]
        _declare_optional(L)
        _lib = L
    return _lib


def _declare_optional(L: C.CDLL) -> None:
    """Signatures of entry points added alongside the pool path."""
    vp = C.c_void_p
    if hasattr(L, "wsbb_explore"):
        L.wsbb_explore.argtypes = [vp, vp, vp, vp]
    if hasattr(L, "wsbb_ctx_device_bytes"):
        L.wsbb_ctx_device_bytes.argtypes = [vp]
        L.wsbb_ctx_device_bytes.restype = C.c_size_t
    if hasattr(L, "wsbb_decompose_lb2"):
        L.wsbb_decompose_lb2.argtypes = [vp, vp, C.c_int64, vp, vp, vp, vp]


def check(ctx, rc: int) -> None:
    if rc != 0:
        msg = lib().wsbb_last_error(ctx).decode() if ctx else ""
        raise WsbbError(rc, msg)
