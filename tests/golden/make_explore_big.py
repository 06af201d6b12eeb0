"""Generate explore_big.json: the reference's own CPU search above its
shipped size limit, as golden runs for the oracle.

The reference caps n at MAX_NBJOBS = 20 (headers/tree.h:31,
headers/explorer.h:34); oracle/build.sh also compiles its sources with that
constant raised to 64 (oracle/_ref/ref_explore_big). Run in the build
container, where the reference tree exists:
    sh oracle/build.sh && python tests/golden/make_explore_big.py

Each run: n = 30 to 50, m = 5 to 10, the NEH incumbent, best = 99999 (the
reference default) or the NEH cost; the reference's counters (branched =
cpu_explored_nodes, pruned, leaves, improvements, child bounds), its
optimum and permutation, and coverage = n! (src/weights.cpp:11-22).
Instances come from the seeded SplitMix64 generator (values uniform in
[1, 99], machine-major); no public benchmark instance is used.
"""
from __future__ import annotations

import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "explore_big.json")

CASES = [(30, 8, 1), (35, 5, 4), (40, 6, 2), (45, 7, 5), (50, 5, 8), (50, 5, 24),
         (50, 5, 32), (50, 5, 39), (50, 10, 9), (50, 10, 1), (50, 10, 6)]


def main() -> None:
    if not O.have_reference_big():
        raise SystemExit("oracle/_ref/ref_explore_big is not built (run oracle/build.sh "
                         "where the reference tree exists)")
    runs = []
    for n, m, s in CASES:
        p = O.gen_instance(s, n, m)
        neh, _ = O.neh(p)
        for best in (99999, neh):
            r = O.ref_explore(p, ub0=neh, best=best, timeout=600)
            runs.append({"n": n, "m": m, "seed": s, "neh": neh, "ub0": neh, "best": best,
                         "branched": r["branched"], "pruned": r["pruned"],
                         "leaves": r["leaves"], "improved": r["improved"],
                         "bounded": r["bounded"], "optimum": r["optimum"],
                         "coverage": r["coverage"],
                         "perm": r["perm"] if r["improved"] else None})
            print(n, m, s, best, r["bounded"], r["optimum"], flush=True)
    with open(OUT, "w") as f:
        json.dump({"generator": "tests/golden/make_explore_big.py",
                   "reference_build": "oracle/_ref/ref_explore_big (MAX_NBJOBS = 64)",
                   "runs": runs}, f, indent=1)


if __name__ == "__main__":
    main()
