"""Train the learned pair selector on nodes logged from plain searches.

    python -m wsbb_gb300.train_selector --n 50 --m 20 --seeds 100 199 \
        --nodes 10000000 --out wsbb_gb300/models/selector_n50_m20.npz

For every training seed the plain GPU search runs from the NEH incumbent
and copies a hashed sample of the children it bounds; the GPU computes
their features and binding-pair labels (the first pair reaching LB2); the
model is trained on the GPU (Adam, softmax cross-entropy). Reports the
top-K hit rate (the binding pair among the K ranked first) on nodes of
held-out seeds.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

from .bound import Context, gen_instance, neh
from .learned import Model, features, log_nodes


def feature_width(n: int, m: int) -> int:
    return (3 * m + n + 15) // 16 * 16


def logged_dataset(n: int, m: int, seeds, per_seed: int, stride: int = 64, max_iters: int = 400,
                   window: int = 0):
    """Features X (rows x D, fp32) and labels y (int32) on the GPU."""
    import torch
    D = feature_width(n, m)
    Xs, ys = [], []
    for s in seeds:
        p = gen_instance(s, n, m)
        ctx = Context(p)
        ub, _ = neh(p)
        recs = torch.empty((per_seed, ctx.stride), dtype=torch.uint8, device="cuda")
        got, _ = log_nodes(ctx, recs.data_ptr(), per_seed, stride=stride, ub0=ub,
                           max_iters=max_iters, window=window)
        if got == 0:
            continue
        X = torch.empty((got, D), dtype=torch.float32, device="cuda")
        y = torch.empty(got, dtype=torch.int32, device="cuda")
        features(ctx, recs.data_ptr(), got, D, X.data_ptr(), y.data_ptr())
        torch.cuda.synchronize()
        keep = y >= 0  # leaves have no binding pair
        Xs.append(X[keep])
        ys.append(y[keep])
        del recs
        ctx.close()
    return torch.cat(Xs), torch.cat(ys)


def topk_hit_rate(model: Model, X, y, Ks=(1, 4, 8, 16)) -> dict:
    import torch
    kmax = max(Ks)
    tk = torch.empty((len(y), kmax), dtype=torch.int16, device="cuda")
    model.topk(X.data_ptr(), len(y), kmax, tk.data_ptr())
    torch.cuda.synchronize()
    hits = tk.to(torch.int32) == y[:, None]
    return {f"top{k}": float(hits[:, :k].any(1).float().mean().item()) for k in Ks}


def train(n: int, m: int, train_seeds, nodes: int, epochs: int = 4, batch: int = 4096,
          lr: float = 1e-3, eval_seeds=(0, 1), seed: int = 7, verbose: bool = True):
    per_seed = max(1, nodes // max(1, len(train_seeds)))
    t0 = time.perf_counter()
    X, y = logged_dataset(n, m, train_seeds, per_seed)
    t_log = time.perf_counter() - t0
    model = Model(n, m, seed=seed)
    t0 = time.perf_counter()
    losses = model.train(X.data_ptr(), y.data_ptr(), len(y), epochs=epochs, batch=batch, lr=lr,
                         seed=seed)
    t_train = time.perf_counter() - t0
    Xe, ye = logged_dataset(n, m, eval_seeds, 100000)
    report = {"n": n, "m": m, "train_nodes": int(len(y)), "log_seconds": t_log,
              "train_seconds": t_train, "epoch_loss": losses,
              "heldout_nodes": int(len(ye)), "heldout": topk_hit_rate(model, Xe, ye),
              "train": topk_hit_rate(model, X[:200000], y[:200000])}
    if verbose:
        print(json.dumps(report), flush=True)
    return model, report


def main(argv=None) -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=50)
    ap.add_argument("--m", type=int, default=20)
    ap.add_argument("--seeds", type=int, nargs=2, default=[100, 199])
    ap.add_argument("--nodes", type=int, default=10_000_000)
    ap.add_argument("--epochs", type=int, default=4)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--out", default="")
    a = ap.parse_args(argv)
    model, _ = train(a.n, a.m, range(a.seeds[0], a.seeds[1] + 1), a.nodes, a.epochs, a.batch,
                     a.lr)
    if a.out:
        os.makedirs(os.path.dirname(os.path.abspath(a.out)), exist_ok=True)
        model.save(a.out)


if __name__ == "__main__":
    main(sys.argv[1:])
