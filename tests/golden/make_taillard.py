"""Writes tests/golden/taillard_streams.json: instances drawn by the
reference's own generator (instance_flowshop::unif, compiled in place into
oracle/_ref by oracle/build.sh) for a few arbitrary time seeds. Run where
the reference tree is present:

    sh oracle/build.sh && python tests/golden/make_taillard.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle  # noqa: E402

# arbitrary time seeds (none is a published benchmark's), including the
# largest one the modulus allows
CASES = [(1, 20, 5), (12345, 20, 5), (987654321, 50, 10), (2147483646, 20, 20), (42, 100, 5)]


def main() -> None:
    if not oracle.have_reference():
        raise SystemExit("oracle/_ref is not built (no reference tree)")
    out = []
    for seed, n, m in CASES:
        p = oracle.ref_taillard_instance(seed, n, m)
        out.append({"seed": seed, "n": n, "m": m, "p": p.ravel().tolist()})
    with open(os.path.join(HERE, "taillard_streams.json"), "w") as f:
        json.dump(out, f, separators=(",", ":"))


if __name__ == "__main__":
    main()
