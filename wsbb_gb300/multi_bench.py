"""Batched multi-instance throughput: many independent instances searched
concurrently on one GPU.

    python -m wsbb_gb300.multi_bench --instances 64 --threads 8

Every instance runs to a proven optimum or to a node budget (`budget`
bounded nodes: 10^9, the cap the workload sets for its n = 100 instances,
applied to every instance so that the ones that cannot be proved in
minutes end too). `resident` is the whole set in one launch of resident
CTAs (wsbb_explore_resident: a group of CTAs per instance, fathers stolen
between CTAs and from the instances still running). Against it stands the
single-instance rate of each shape: the shape's instance with the most
nodes in the launch, alone, the graph-launched search to its proof or
`single_budget` nodes (a small proof's rate says little of a long search's), at window
16384 (the headline's) or, where its stack would overflow, 4096; the time the
set would take run one instance after another at those rates
(`sequential_estimate_s`: each shape's nodes in the resident launch over
its single-instance rate) over the launch's time is `vs_sequential`. The
arms below are then compared at a smaller budget (`cmp_budget`), each over
the same instances and trees, checked equal.

Instance i (seed i) has n = (20, 50, 100)[i % 3] jobs and m = (5, 10,
20)[(i // 3) % 3] machines, times uniform in [1, 99] and the NEH incumbent;
the side-choice threshold is best = NEH (the learned configuration: a child
whose bound reaches max(best, incumbent) may be settled early) or, with
--best default, the reference's 99999 (every bound below it is summed by
the side choice, so none can be settled early). Every instance
has its own context (tables, search state, stream). In the threaded arms
`threads` host threads drive them, so the searches' kernels interleave on
the GPU; each arm is timed from a barrier to a barrier:
  resident     one resident launch over all instances (as above)
  family       the graph-launched search with family bounds
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
ARMS = ("resident", "family", "learnable", "learned")


def shape_of(i: int) -> tuple[int, int]:
    return NS[i % len(NS)], MS[(i // len(NS)) % len(MS)]


def model_path(n: int, m: int) -> str:
    return os.path.join(MODELS, f"selector_n{n}_m{m}.npz")


def capacity_of(n: int) -> int:
    """Stack nodes for one instance of the set (64 of them share the GPU)."""
    return 1 << 24 if n >= 50 else 1 << 23


def run(instances: int = 64, threads: int = 8, budget: int = 10**9, cmp_budget: int = 2 * 10**7,
        window: int = 2048, K: int = 16, device: int = 0, arms=ARMS, best_mode: str = "ub0",
        full: bool = True, single_budget: int = 2 * 10**8) -> dict:
    from .bound import Context, gen_instance, neh
    from ._lib import WsbbError
    from .explorer import explore, explore_resident
    from .learned import Model, explore_learned

    items = []
    for i in range(instances):
        n, m = shape_of(i)
        p = gen_instance(i, n, m)
        ub0, _ = neh(p)
        it = {"seed": i, "n": n, "m": m, "p": p, "ub0": ub0,
              "best": ub0 if best_mode == "ub0" else 99999,
              "ctx": Context(p, device=device)}
        if "learned" in arms and os.path.exists(model_path(n, m)) and m * (m - 1) // 2 > K:
            md = Model(n, m)
            md.load(model_path(n, m))
            it["model"] = md
        items.append(it)
    out = {"instances": instances, "threads": threads, "window": window, "K": K,
           "best": best_mode, "budget": budget, "cmp_budget": cmp_budget}

    def resident(max_bounded):
        t0 = time.perf_counter()
        rc, st = explore_resident([it["ctx"] for it in items], ub0s=[it["ub0"] for it in items],
                                  bests=[it["best"] for it in items], window=window,
                                  capacity=[capacity_of(it["n"]) for it in items],
                                  max_bounded=max_bounded)
        return time.perf_counter() - t0, {it["seed"]: r for it, r in zip(items, st)}

    def summary(wall, rs):
        b = sum(r["bounded"] for r in rs.values())
        return {"instances": len(rs), "seconds": wall, "bounded": b, "bounded_per_s": b / wall,
                "proved": sum(1 for r in rs.values() if r["status"] == 0),
                "at_budget": sum(1 for r in rs.values() if r["status"] == 1),
                "finished": all(r["status"] in (0, 1) for r in rs.values())}

    if full:
        wall, rs = resident(budget)
        out["resident_full"] = summary(wall, rs)
        out["resident_full"]["launch_seconds"] = max(r["seconds"] for r in rs.values())
        out["per_shape"] = {}
        for it in items:
            d = out["per_shape"].setdefault(f"n{it['n']}_m{it['m']}",
                                            {"instances": 0, "bounded": 0, "proved": 0})
            r = rs[it["seed"]]
            d["instances"] += 1
            d["bounded"] += r["bounded"]
            d["proved"] += int(r["status"] == 0)
        # single-instance rates: each shape's heaviest instance alone
        est = 0.0
        heaviest: dict[str, dict] = {}
        for it in items:
            key = f"n{it['n']}_m{it['m']}"
            if key not in heaviest or rs[it["seed"]]["bounded"] > rs[heaviest[key]["seed"]]["bounded"]:
                heaviest[key] = it
        for key, it in heaviest.items():
            d = out["per_shape"][key]
            for w in (16384, 4096):
                try:
                    kw = dict(ub0=it["ub0"], best=it["best"], window=w,
                              capacity=2 * capacity_of(it["n"]))
                    explore(it["ctx"], max_bounded=min(budget, 10**6), **kw)
                    r = explore(it["ctx"], max_bounded=min(budget, single_budget), **kw)
                    break
                except WsbbError as e:
                    if e.code != -6 or w == 4096:
                        raise
            d["single"] = {"seed": it["seed"], "window": w, "bounded": r["bounded"],
                           "seconds": r["seconds"],
                           "bounded_per_s": r["bounded"] / r["seconds"],
                           "proved": r["status"] == 0}
            est += d["bounded"] / d["single"]["bounded_per_s"]
        out["resident_full"]["sequential_estimate_s"] = est
        out["resident_full"]["vs_sequential"] = est / wall

    # the arms at the comparison budget
    results: dict[str, dict[int, dict]] = {a: {} for a in arms}
    errors: list[str] = []
    walls: dict[str, float] = {}
    if "resident" in arms:
        walls["resident"], results["resident"] = resident(cmp_budget)

    def threaded(arm):
        work = [items[t::threads] for t in range(threads)]
        bar = threading.Barrier(threads + 1)

        def worker(mine):
            bar.wait()
            for it in mine:
                try:
                    kw = dict(ub0=it["ub0"], best=it["best"], window=window, graph_iters=1,
                              capacity=capacity_of(it["n"]), max_bounded=cmp_budget)
                    if arm == "family":
                        r = explore(it["ctx"], **kw)
                    elif arm == "per_child" or (arm == "learnable" and "model" in it):
                        r = explore(it["ctx"], child_lb2=True, **kw)
                    elif arm == "learned" and "model" in it:
                        kw.pop("graph_iters")
                        r = explore_learned(it["ctx"], it["model"], K, child_lb2=True,
                                            graph_iters=1, **kw)
                    else:
                        continue
                    results[arm][it["seed"]] = r
                except Exception as e:
                    errors.append(f"{arm} seed {it['seed']}: {e!r}")
            bar.wait()
        ts = [threading.Thread(target=worker, args=(w,)) for w in work]
        for t in ts:
            t.start()
        bar.wait()
        t0 = time.perf_counter()
        bar.wait()
        walls[arm] = time.perf_counter() - t0
        for t in ts:
            t.join()

    for arm in arms:
        if arm != "resident":
            threaded(arm)
    for it in items:
        it["ctx"].close()
    if errors:
        raise RuntimeError("; ".join(errors[:5]))
    out["arms"] = {a: summary(walls[a], results[a]) for a in arms if a in walls}
    base = results.get("resident") or results.get("family")
    for a in out["arms"]:
        out["arms"][a]["same_tree"] = all(
            all(r[k] == base[s][k] for k in TREE_KEYS) for s, r in results[a].items())
    if "learned" in walls and "learnable" in walls and results["learned"]:
        out["learned_instances"] = sorted(results["learned"])
        fam = {s: results["family"][s] for s in results["learned"]} if "family" in results \
            else {}
        out["learned_speedup_vs_per_child"] = walls["learnable"] / max(walls["learned"], 1e-12)
        if fam:
            out["learned_instances_family_seconds_sum"] = sum(r["seconds"] for r in fam.values())
            out["learned_instances_learned_seconds_sum"] = sum(
                r["seconds"] for r in results["learned"].values())
    return out


def main(argv=None) -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--instances", type=int, default=64)
    ap.add_argument("--threads", type=int, default=8)
    ap.add_argument("--budget", type=int, default=10**9)
    ap.add_argument("--cmp-budget", type=int, default=2 * 10**7)
    ap.add_argument("--window", type=int, default=2048)
    ap.add_argument("--K", type=int, default=16)
    ap.add_argument("--arms", nargs="+", default=list(ARMS))
    ap.add_argument("--best", default="ub0", choices=["ub0", "default"])
    a = ap.parse_args(argv)
    print(json.dumps(run(a.instances, a.threads, a.budget, a.cmp_budget, a.window, a.K,
                         arms=tuple(a.arms), best_mode=a.best)), flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
