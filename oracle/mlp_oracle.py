"""TEST INFRASTRUCTURE — numpy oracle of the pair-selector MLP.

Only tests/ may import this module. It restates, in float64, the network
the GPU trains and runs (wsbb_gb300/csrc/learned.cu): features and weights
rounded to bf16 as the GPU forward sees them, fp32-style accumulation
replaced by exact float64 sums, ReLU hidden layers, softmax cross-entropy
over the first P of O logits, and the straight-through gradients of the
roundings. The reference has no counterpart (the selector is new).
"""
from __future__ import annotations

import numpy as np

H = 128


def bf16(x) -> np.ndarray:
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    b = a.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(w: np.ndarray, D: int, O: int) -> dict:
    o = 0
    out = {}
    for name, shape in (("W1", (D, H)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)),
                        ("W3", (H, O)), ("b3", (O,))):
        size = int(np.prod(shape))
        out[name] = np.asarray(w[o:o + size], dtype=np.float64).reshape(shape)
        o += size
    assert o == len(w)
    return out


def pack(g: dict) -> np.ndarray:
    return np.concatenate([g[k].ravel() for k in ("W1", "b1", "W2", "b2", "W3", "b3")])


def forward(w: dict, X: np.ndarray, rounding: bool = True):
    r = bf16 if rounding else (lambda v: np.asarray(v, dtype=np.float64))
    A0 = r(X)
    Z1 = A0 @ r(w["W1"]) + w["b1"]
    A1 = r(np.maximum(Z1, 0))
    Z2 = A1 @ r(w["W2"]) + w["b2"]
    A2 = r(np.maximum(Z2, 0))
    Z3 = A2 @ r(w["W3"]) + w["b3"]
    return A0, A1, A2, Z3


def loss_and_grads(wflat: np.ndarray, D: int, O: int, P: int, X: np.ndarray, y: np.ndarray,
                   rounding: bool = True):
    """Summed loss and gradients of the mean loss (rows with y < 0 ignored)."""
    r = bf16 if rounding else (lambda v: np.asarray(v, dtype=np.float64))
    w = unpack(wflat, D, O)
    A0, A1, A2, Z3 = forward(w, X, rounding)
    B = len(X)
    z = Z3[:, :P]
    mx = z.max(axis=1, keepdims=True)
    e = np.exp(z - mx)
    s = e.sum(axis=1, keepdims=True)
    p = e / s
    valid = y >= 0
    loss = float(np.sum((np.log(s[:, 0]) + mx[:, 0] - z[np.arange(B), np.maximum(y, 0)])[valid]))
    dZ3 = np.zeros_like(Z3)
    dZ3[:, :P] = p
    dZ3[valid, y[valid]] -= 1.0
    dZ3[~valid] = 0.0
    dZ3 /= B
    g = {"W3": A2.T @ dZ3, "b3": dZ3.sum(0)}
    dA2 = (dZ3 @ r(w["W3"]).T) * (A2 > 0)
    g["W2"] = A1.T @ dA2
    g["b2"] = dA2.sum(0)
    dA1 = (dA2 @ r(w["W2"]).T) * (A1 > 0)
    g["W1"] = A0.T @ dA1
    g["b1"] = dA1.sum(0)
    return loss, pack(g)
