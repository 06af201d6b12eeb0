"""Proof progress of a search that is too large to finish: how much of the
permutation space a fixed amount of search time covers.

    python -m wsbb_gb300.proof_progress --n 50 --m 20 --seed 0 --seconds 60

The search runs from the NEH incumbent in slices (a stopped search resumes
exactly where it stopped) until `seconds` of device time have passed. The
coverage is the reference's own measure of explored work (src/weights.cpp:
11-22, summed at src/tree.cpp:319): every pruned node and leaf at depth d
stands for (n - d)! complete permutations, and a finished proof covers n!.
It is taken at the exact sequential prefix where the search stands
(children pruned at birth whose take is still ahead are not counted), so
it is the coverage the reference's CPU search would report after the same
takes. The time to proof is extrapolated linearly from the covered share,
which a depth-first search reaches unevenly: it is an order of magnitude,
not a prediction.
"""
from __future__ import annotations

import argparse
import json
import math
import sys
import time

from .bound import Context, gen_instance, neh
from .explorer import explore


def run(n: int = 50, m: int = 20, seed: int = 0, best_mode: str = "ub0", seconds: float = 60.0,
        window: int = 16384, family_smem_kb: int = 0, slice_iters: int = 256,
        device: int = 0) -> dict:
    p = gen_instance(seed, n, m)
    ub0, _ = neh(p)
    best = ub0 if best_mode == "ub0" else 99999
    ctx = Context(p, device=device)
    # an explicit capacity: a resumed search must keep its stack's size
    cap = 2 * window * n * n
    r = explore(ctx, ub0=ub0, best=best, window=window, max_iters=slice_iters,
                capacity=cap, family_smem_kb=family_smem_kb)
    dev_s = r["seconds"]
    t0 = time.perf_counter()
    while r["status"] == 1 and dev_s < seconds:
        r = explore(ctx, ub0=ub0, best=best, window=window, max_iters=slice_iters,
                    capacity=cap, family_smem_kb=family_smem_kb, resume=True)
        dev_s += r["seconds"]
    wall = time.perf_counter() - t0
    hist = [h - q for h, q in zip(r["depth_hist"], r["pending_hist"])]
    covered = sum(int(hist[d]) * math.factorial(n - d) for d in range(n + 1))
    share = covered / math.factorial(n)
    out = {"n": n, "m": m, "seed": seed, "neh": ub0, "best": best, "window": window,
           "seconds": dev_s, "wall_seconds": wall, "proved": r["status"] == 0,
           "incumbent": r["best_cost"], "improved": r["improved"], "takes": r["takes"],
           "branched": r["branched"], "bounded": r["bounded"],
           "bounded_per_s": r["bounded"] / max(dev_s, 1e-12),
           "covered_share_of_n_factorial": share,
           "extrapolated_time_to_proof_s": dev_s / share if share > 0 else None,
           "coverage_by_depth": {str(d): int(hist[d]) for d in range(n + 1) if hist[d]}}
    ctx.close()
    return out


def main(argv=None) -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=50)
    ap.add_argument("--m", type=int, default=20)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--best", default="ub0", choices=["default", "ub0"])
    ap.add_argument("--seconds", type=float, default=60.0)
    ap.add_argument("--window", type=int, default=16384)
    a = ap.parse_args(argv)
    print(json.dumps(run(a.n, a.m, a.seed, a.best, a.seconds, a.window)), flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
