"""Search benchmark: time-to-proof and bounded nodes/s of the GPU search.

    python -m wsbb_gb300.search_bench --n 50 --m 10 --seeds 0 1 2 3 4

Each run proves the optimum of one seeded instance (values uniform in
[1, 99]) from the NEH incumbent, exactly as the reference CPU search would
explore it (same tree), and prints one JSON object per run plus a summary.
"""
from __future__ import annotations

import argparse
import json
import sys

from .bound import Context, gen_instance, neh
from .explorer import explore


def run(n: int, m: int, seeds, window: int = 0, max_iters: int = 0, best_mode: str = "default",
        device: int = 0, verbose: bool = True) -> dict:
    runs = []
    for s in seeds:
        p = gen_instance(s, n, m)
        ub0, _ = neh(p)
        ctx = Context(p, device=device)
        best = 99999 if best_mode == "default" else ub0
        r = explore(ctx, ub0=ub0, best=best, window=window, max_iters=max_iters)
        row = {"n": n, "m": m, "seed": s, "neh": ub0, "best": best,
               "optimum": r["best_cost"], "proved": r["status"] == 0,
               "branched": r["branched"], "pruned": r["pruned"], "leaves": r["leaves"],
               "improved": r["improved"], "bounded": r["bounded"],
               "evaluated": r["evaluated"], "iterations": r["iterations"],
               "scanned": r["scanned"], "committed": r["committed"],
               "seconds": r["seconds"],
               "bounded_per_s": r["bounded"] / max(r["seconds"], 1e-12)}
        runs.append(row)
        ctx.close()
        if verbose:
            print(json.dumps(row), flush=True)
    tot_b = sum(r["bounded"] for r in runs)
    tot_s = sum(r["seconds"] for r in runs)
    return {"runs": runs, "bounded": tot_b, "seconds": tot_s,
            "bounded_per_s": tot_b / max(tot_s, 1e-12),
            "evaluated": sum(r["evaluated"] for r in runs),
            "all_proved": all(r["proved"] for r in runs)}


def main(argv=None) -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=50)
    ap.add_argument("--m", type=int, default=10)
    ap.add_argument("--seeds", type=int, nargs="+", default=[0, 1, 2, 3, 4])
    ap.add_argument("--window", type=int, default=0)
    ap.add_argument("--max-iters", type=int, default=0)
    ap.add_argument("--best", default="default", choices=["default", "ub0"])
    a = ap.parse_args(argv)
    out = run(a.n, a.m, a.seeds, a.window, a.max_iters, a.best)
    summary = {k: v for k, v in out.items() if k != "runs"}
    print(json.dumps({"summary": summary}), flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
