"""Generate the bab.solutions fixture from the reference's own search.

Run in the build container, where the reference tree exists:
    sh oracle/build.sh && python tests/golden/make_solutions.py

The reference's CPU search (oracle/_ref/ref_explore, the reference's tree,
decompose and solutions objects) appends its incumbent list to
bab.solutions after every improvement (solutions::save,
src/solutions.cpp:98-108, in the record format of
src/bb_problem_calculator.cpp:101-144). Outputs (committed, small):
  bab_solutions_n12m5.txt   that file, as the reference wrote it
  bab_solutions_n12m5.json  the instance and the run's result line
The instance comes from the seeded SplitMix64 generator (seed 5).
"""
from __future__ import annotations

import json
import os
import shutil
import sys
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def main() -> None:
    n, m, seed = 12, 5, 5
    p = O.gen_instance(seed, n, m)
    with tempfile.TemporaryDirectory() as d:
        r = O.ref_explore(p, ub0=None, best=99999, workdir=d)
        shutil.copy(os.path.join(d, "bab.solutions"), os.path.join(OUT, "bab_solutions_n12m5.txt"))
    with open(os.path.join(OUT, "bab_solutions_n12m5.json"), "w") as f:
        json.dump({"source": "reference CPU search (oracle/_ref/ref_explore)", "n": n, "m": m,
                   "seed": seed, "max_nbjobs": 20, "p": p.tolist(), "result": r}, f)
    print(json.dumps(r))


if __name__ == "__main__":
    main()
