"""Search benchmark: time-to-proof and bounded nodes/s of the GPU search.

    python -m wsbb_gb300.search_bench --n 50 --m 10 --seeds 0 1 2 3 4
    python -m wsbb_gb300.search_bench --n 50 --m 10 --best ub0 \
        --model wsbb_gb300/models/selector_n50_m10.npz --K 4 8

Each run proves the optimum of one seeded instance (values uniform in
[1, 99]) from the NEH incumbent, exploring exactly the tree the reference
CPU search explores with the same `best` (side-choice threshold), and
prints one JSON object per run plus a summary. With --model, every
instance is also searched with the learned K-pair test (same tree, checked)
and the speed-up over the plain search at the same `best` is reported.
"""
from __future__ import annotations

import argparse
import json
import sys

from .bound import Context, gen_instance, neh
from .explorer import explore

TREE_KEYS = ("branched", "pruned", "leaves", "improved", "bounded", "best_cost", "coverage")


def run(n: int, m: int, seeds, window: int = 0, max_iters: int = 0, best_mode: str = "default",
        device: int = 0, verbose: bool = True, model_path: str = "", Ks=(8,),
        per_child: bool = False, capacity: int = 0, tune: bool = False) -> dict:
    """`per_child` also runs the search with every child bounded on its own
    (the per-node LB2 kernel) and reports its time and tree check. `tune`
    takes the window and family tile from the autotuner (tuned on the first
    instance, cached per GPU and shape) instead of `window`."""
    model = None
    if model_path:
        from .learned import Model
        model = Model(n, m)
        model.load(model_path)
    runs = []
    kb = 0
    shape = None
    for s in seeds:
        p = gen_instance(s, n, m)
        ub0, _ = neh(p)
        ctx = Context(p, device=device)
        best = 99999 if best_mode == "default" else ub0
        if tune and shape is None:
            from .autotune import tuned
            shape = tuned(ctx, ub0, best, device=device)
            window, kb = shape["window"], shape["family_smem_kb"]
        r = explore(ctx, ub0=ub0, best=best, window=window, max_iters=max_iters,
                    capacity=capacity, family_smem_kb=kb)
        row = {"n": n, "m": m, "seed": s, "neh": ub0, "best": best,
               "optimum": r["best_cost"], "proved": r["status"] == 0,
               "branched": r["branched"], "pruned": r["pruned"], "leaves": r["leaves"],
               "improved": r["improved"], "bounded": r["bounded"],
               "evaluated": r["evaluated"], "iterations": r["iterations"],
               "scanned": r["scanned"], "committed": r["committed"],
               "seconds": r["seconds"],
               "bounded_per_s": r["bounded"] / max(r["seconds"], 1e-12)}
        if per_child:
            q = explore(ctx, ub0=ub0, best=best, window=window, max_iters=max_iters,
                        child_lb2=True, capacity=capacity)
            row["per_child"] = {"seconds": q["seconds"],
                                "same_tree": all(q[k] == r[k] for k in TREE_KEYS),
                                "bounded_per_s": q["bounded"] / max(q["seconds"], 1e-12),
                                "family_speedup": q["seconds"] / max(r["seconds"], 1e-12)}
        if model is not None:
            from .learned import explore_learned
            row["learned"] = {}
            for K in Ks:
                q = explore_learned(ctx, model, K, ub0=ub0, best=best, window=window,
                                    max_iters=max_iters)
                same = all(q[k] == r[k] for k in TREE_KEYS)
                row["learned"][str(K)] = {
                    "seconds": q["seconds"], "early": q["early"],
                    "early_share": q["early"] / max(1, q["evaluated"]),
                    "settled_fathers_share": q["settled_fathers"] / max(1, q["branched"]),
                    "same_tree": same, "speedup": r["seconds"] / max(q["seconds"], 1e-12),
                    "bounded_per_s": q["bounded"] / max(q["seconds"], 1e-12)}
                if per_child:
                    q2 = explore_learned(ctx, model, K, ub0=ub0, best=best, window=window,
                                         max_iters=max_iters, child_lb2=True)
                    row["learned"][str(K)]["per_child"] = {
                        "seconds": q2["seconds"], "early": q2["early"],
                        "same_tree": all(q2[k] == r[k] for k in TREE_KEYS),
                        "speedup_vs_per_child": row["per_child"]["seconds"] /
                        max(q2["seconds"], 1e-12)}
        runs.append(row)
        ctx.close()
        if verbose:
            print(json.dumps(row), flush=True)
    tot_b = sum(r["bounded"] for r in runs)
    tot_s = sum(r["seconds"] for r in runs)
    out = {"runs": runs, "bounded": tot_b, "seconds": tot_s, "shape": shape,
           "bounded_per_s": tot_b / max(tot_s, 1e-12),
           "evaluated": sum(r["evaluated"] for r in runs),
           "all_proved": all(r["proved"] for r in runs)}
    if per_child:
        ps = sum(r["per_child"]["seconds"] for r in runs)
        out["per_child"] = {"seconds": ps, "bounded_per_s": tot_b / max(ps, 1e-12),
                            "family_speedup": ps / max(tot_s, 1e-12),
                            "same_tree": all(r["per_child"]["same_tree"] for r in runs)}
    if model is not None:
        out["learned"] = {}
        for K in Ks:
            ls = sum(r["learned"][str(K)]["seconds"] for r in runs)
            out["learned"][str(K)] = {
                "seconds": ls, "bounded_per_s": tot_b / max(ls, 1e-12),
                "speedup_vs_plain": tot_s / max(ls, 1e-12),
                "same_tree": all(r["learned"][str(K)]["same_tree"] for r in runs)}
            if per_child:
                lp = sum(r["learned"][str(K)]["per_child"]["seconds"] for r in runs)
                out["learned"][str(K)]["per_child"] = {
                    "seconds": lp, "bounded_per_s": tot_b / max(lp, 1e-12),
                    "speedup_vs_per_child": out["per_child"]["seconds"] / max(lp, 1e-12),
                    "same_tree": all(r["learned"][str(K)]["per_child"]["same_tree"]
                                     for r in runs)}
    return out


def main(argv=None) -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=50)
    ap.add_argument("--m", type=int, default=10)
    ap.add_argument("--seeds", type=int, nargs="+", default=[0, 1, 2, 3, 4])
    ap.add_argument("--window", type=int, default=0)
    ap.add_argument("--max-iters", type=int, default=0)
    ap.add_argument("--best", default="default", choices=["default", "ub0"])
    ap.add_argument("--model", default="")
    ap.add_argument("--K", type=int, nargs="+", default=[8])
    ap.add_argument("--per-child", action="store_true",
                    help="also search with per-child LB2 (the per-node kernel)")
    ap.add_argument("--capacity", type=int, default=0,
                    help="stack capacity in nodes (0: the library's default)")
    ap.add_argument("--tune", action="store_true",
                    help="window and family tile from the autotuner")
    a = ap.parse_args(argv)
    out = run(a.n, a.m, a.seeds, a.window, a.max_iters, a.best, model_path=a.model, Ks=a.K,
              per_child=a.per_child, capacity=a.capacity, tune=a.tune)
    summary = {k: v for k, v in out.items() if k != "runs"}
    print(json.dumps({"summary": summary}), flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
