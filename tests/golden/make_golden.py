"""Generate the golden fixtures from the reference's own compiled code.

Run in the build container, where the reference tree exists:
    sh oracle/build.sh && python tests/golden/make_golden.py

Outputs (committed, small):
  bound_pools.npz   per instance: processing times, a pool of partial
                    permutations (seeded random records plus edge cases)
                    and the LB / binding pair the reference's
                    bound_flowshop::bornes_calculer returns for each
                    (src/bound_flowshop.cpp:929-951, nbFois at :157/:164).
  explore.json      counters of the reference's CPU search
                    (src/explorer.cu:92-148 over src/tree.cpp,
                    src/decompose_beginend.cpp, src/solutions.cpp) for a set
                    of instances and initial-bound / `best` settings.

Instances come from the seeded SplitMix64 generator (values uniform in
[1, 99], machine-major); no public benchmark instance is used.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

BOUND_CASES = [(20, 20, s) for s in range(10)] + [
    (20, 5, 0), (20, 10, 0), (50, 10, 0), (50, 20, 0), (100, 20, 0), (9, 3, 4), (30, 2, 7)]
RECORDS = 200

EXPLORE_CASES = [
    # (n, m, seed, ub0 mode, best mode)
    (10, 5, 0, "none", "default"), (10, 5, 0, "neh", "default"), (10, 5, 0, "neh", "ub0"),
    (20, 5, 0, "none", "default"), (20, 5, 0, "neh", "default"), (20, 5, 0, "neh", "ub0"),
    (20, 5, 1, "neh", "default"),
    (12, 10, 1, "none", "default"), (12, 10, 1, "neh", "ub0"),
    (13, 20, 2, "neh", "default"), (13, 20, 2, "neh", "ub0"),
    (15, 5, 3, "neh", "default"),
]


def edge_records(n: int, rng: np.random.Generator):
    """Root, front-only, back-only, two and three free jobs, leaves."""
    recs = []
    for l1, l2 in [(-1, n), (-1, n - 1), (-1, n - 5), (0, n), (4, n), (n - 4, n),
                   (-1, 2), (n - 4, n - 1), (n // 2 - 2, n // 2 + 1),  # u = 2
                   (n // 2 - 2, n // 2 + 2),  # u = 3
                   (n - 2, n - 1), (-1, 0), (n // 2 - 1, n // 2)]:  # leaves
        if l1 < -1 or l2 > n or l2 <= l1:
            continue
        recs.append((rng.permutation(n).astype(np.int32), l1, l2))
    return recs


def bound_fixture() -> None:
    arrays = {}
    for (n, m, s) in BOUND_CASES:
        p = O.gen_instance(s, n, m)
        perms, l1, l2 = O.random_pool(1000 + s, n, RECORDS, leaf_share=0.05)
        rng = np.random.default_rng(77 + s)
        edges = edge_records(n, rng)
        perms = np.vstack([perms] + [e[0][None, :] for e in edges])
        l1 = np.concatenate([l1, np.array([e[1] for e in edges], dtype=np.int32)])
        l2 = np.concatenate([l2, np.array([e[2] for e in edges], dtype=np.int32)])
        lb, arg = O.RefBound(p).eval_batch(perms, l1, l2, want_argmax=True)
        arg[(l2 - l1) == 1] = -1
        key = f"n{n}_m{m}_s{s}"
        arrays[key + "_p"] = p.astype(np.int16)
        arrays[key + "_perms"] = perms.astype(np.int16 if n > 127 else np.int8)
        arrays[key + "_l1"] = l1.astype(np.int16)
        arrays[key + "_l2"] = l2.astype(np.int16)
        arrays[key + "_lb"] = lb.astype(np.int32)
        arrays[key + "_argmax"] = arg.astype(np.int16)
        print(key, "records", len(lb))
    np.savez_compressed(os.path.join(OUT, "bound_pools.npz"), **arrays)


def explore_fixture() -> None:
    runs = []
    for (n, m, s, ubm, bm) in EXPLORE_CASES:
        p = O.gen_instance(s, n, m)
        neh_cost, _ = O.neh(p)
        ub0 = None if ubm == "none" else neh_cost
        best = 99999 if bm == "default" else neh_cost
        r = O.ref_explore(p, ub0=ub0, best=best)
        run = {"n": n, "m": m, "seed": s, "ub0": ub0, "best": best, "neh": neh_cost,
               "branched": r["branched"], "pruned": r["pruned"], "leaves": r["leaves"],
               "improved": r["improved"], "bounded": r["bounded"], "optimum": r["optimum"],
               "coverage": r["coverage"], "perm": r["perm"] if r["improved"] else None}
        runs.append(run)
        print(run)
    with open(os.path.join(OUT, "explore.json"), "w") as f:
        json.dump({"source": "reference CPU search (oracle/_ref/ref_explore)", "runs": runs},
                  f, indent=1)


if __name__ == "__main__":
    if not O.have_reference():
        sys.exit("oracle/_ref not built: run sh oracle/build.sh where the reference exists")
    bound_fixture()
    explore_fixture()
