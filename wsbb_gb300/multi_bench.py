"""Batched multi-instance throughput: many independent instances searched
concurrently on one GPU.

    python -m wsbb_gb300.multi_bench --instances 64 --threads 8

Instance i (seed i) has n = (20, 50, 100)[i % 3] jobs and m = (5, 10,
20)[(i // 3) % 3] machines, times uniform in [1, 99] and the NEH incumbent;
the side-choice threshold is best = NEH (the learned configuration: a child
whose bound reaches max(best, incumbent) may be settled early) or, with
--best default, the reference's 99999 (every bound below it is summed by
the side choice, so none can be settled early). Every instance
has its own context (tables, search state, stream); `threads` host threads
drive them, so the searches' kernels interleave on the GPU. Each instance
runs to a proven optimum or to `max_iters` batched iterations (the node
budget of the larger ones). The arms run one after the other over all
instances, each timed from a barrier to a barrier:
  family       the search with family bounds
  per_child    the same tree with every child record bounded on its own
  learnable    per-child LB2 again, on the instances whose shape has a
               trained selector in wsbb_gb300/models/ (and more than K pairs)
  learned      the learned K-pair test ahead of per-child LB2 on those
               instances (compare with `learnable`)
and the tree of every instance is checked to be the same in every arm.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import threading
import time

NS, MS = (20, 50, 100), (5, 10, 20)
TREE_KEYS = ("branched", "pruned", "leaves", "improved", "bounded", "best_cost", "coverage")
MODELS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "models")
ARMS = ("family", "per_child", "learnable", "learned")


def shape_of(i: int) -> tuple[int, int]:
    return NS[i % len(NS)], MS[(i // len(NS)) % len(MS)]


def model_path(n: int, m: int) -> str:
    return os.path.join(MODELS, f"selector_n{n}_m{m}.npz")


def capacity_of(n: int, window: int, max_iters: int) -> int:
    """Stack nodes for one instance: room for about window * n / 2 entries
    pushed per iteration, within [2^22, 2^25]."""
    return int(min(1 << 25, max(1 << 22, window * n * max_iters // 2)))


def run(instances: int = 64, threads: int = 8, max_iters: int = 64, window: int = 4096,
        K: int = 16, device: int = 0, arms=ARMS, best_mode: str = "ub0") -> dict:
    from .bound import Context, gen_instance, neh
    from .explorer import explore
    from .learned import Model, explore_learned

    work = [[] for _ in range(threads)]
    for i in range(instances):
        n, m = shape_of(i)
        p = gen_instance(i, n, m)
        ub0, _ = neh(p)
        work[i % threads].append({"seed": i, "n": n, "m": m, "p": p, "ub0": ub0})
    results: dict[str, dict[int, dict]] = {a: {} for a in arms}
    errors: list[str] = []
    bar = threading.Barrier(threads + 1)

    def worker(items):
        try:
            for it in items:
                it["ctx"] = Context(it["p"], device=device)
                if "learned" in arms and os.path.exists(model_path(it["n"], it["m"])) \
                        and it["m"] * (it["m"] - 1) // 2 > K:
                    md = Model(it["n"], it["m"])
                    md.load(model_path(it["n"], it["m"]))
                    it["model"] = md
        except Exception as e:  # reported after the barriers
            errors.append(repr(e))
        bar.wait()
        for arm in arms:
            bar.wait()
            for it in items:
                if "ctx" not in it:
                    continue
                try:
                    best = it["ub0"] if best_mode == "ub0" else 99999
                    kw = dict(ub0=it["ub0"], best=best, window=window, max_iters=max_iters,
                              capacity=capacity_of(it["n"], window, max_iters))
                    if arm == "family":
                        r = explore(it["ctx"], **kw)
                    elif arm == "per_child" or (arm == "learnable" and "model" in it):
                        r = explore(it["ctx"], child_lb2=True, **kw)
                    elif arm == "learned" and "model" in it:
                        r = explore_learned(it["ctx"], it["model"], K, child_lb2=True, **kw)
                    else:
                        continue
                    results[arm][it["seed"]] = r
                except Exception as e:
                    errors.append(f"{arm} seed {it['seed']}: {e!r}")
            bar.wait()
        for it in items:
            if "ctx" in it:
                it["ctx"].close()

    ts = [threading.Thread(target=worker, args=(w,)) for w in work]
    for t in ts:
        t.start()
    bar.wait()  # contexts ready
    out = {"instances": instances, "threads": threads, "max_iters": max_iters, "window": window,
           "K": K, "best": best_mode, "arms": {}}
    for arm in arms:
        bar.wait()
        t0 = time.perf_counter()
        bar.wait()
        wall = time.perf_counter() - t0
        rs = results[arm]
        out["arms"][arm] = {"instances": len(rs), "seconds": wall,
                            "bounded": sum(r["bounded"] for r in rs.values()),
                            "bounded_per_s": sum(r["bounded"] for r in rs.values()) / wall,
                            "proved": sum(1 for r in rs.values() if r["status"] == 0)}
    for t in ts:
        t.join()
    if errors:
        raise RuntimeError("; ".join(errors[:5]))
    base = results.get("family") or results[arms[0]]
    for arm in arms:
        out["arms"][arm]["same_tree"] = all(
            all(r[k] == base[s][k] for k in TREE_KEYS) for s, r in results[arm].items())
    if "learned" in arms and "learnable" in arms and results["learned"]:
        a, b = out["arms"]["learned"], out["arms"]["learnable"]
        out["learned_speedup_vs_per_child"] = b["seconds"] / max(a["seconds"], 1e-12)
        out["learned_instances"] = sorted(results["learned"])
    out["per_shape"] = {}
    for i in range(instances):
        n, m = shape_of(i)
        d = out["per_shape"].setdefault(f"n{n}_m{m}", {"instances": 0, "bounded": 0,
                                                      "proved": 0})
        r = base.get(i)
        if r:
            d["instances"] += 1
            d["bounded"] += r["bounded"]
            d["proved"] += int(r["status"] == 0)
    return out


def main(argv=None) -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--instances", type=int, default=64)
    ap.add_argument("--threads", type=int, default=8)
    ap.add_argument("--max-iters", type=int, default=64)
    ap.add_argument("--window", type=int, default=4096)
    ap.add_argument("--K", type=int, default=16)
    ap.add_argument("--arms", nargs="+", default=list(ARMS))
    ap.add_argument("--best", default="ub0", choices=["ub0", "default"])
    a = ap.parse_args(argv)
    print(json.dumps(run(a.instances, a.threads, a.max_iters, a.window, a.K,
                         arms=tuple(a.arms), best_mode=a.best)), flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
