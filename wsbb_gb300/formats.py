"""The reference's host-side node formats, either side of the search.

bab.solutions (the incumbent file, src/solutions.cpp:26-108): blocks of a
count line followed by that many records, each record the text form of the
reference's node (src/bb_problem_calculator.cpp:101-144):
    couts[0] couts[1] couts_somme permutation[MAX_NBJOBS] limite1 limite2
    depth job begin_end
The reference appends one block per improvement holding the incumbents as
they were *before* it (solutions::insert saves before adding), so the file
starts with an empty block and never holds the final optimum; its reader
(solutions::readOptimalSolution) takes only the first block.

Work hand-off packet (BB_PROBLEM_PACKET payload, src/work_stealing/
node.cpp:524-560 and 1240-1283): per node, int32
    permutation[MAX_NBJOBS] limite1 limite2 couts_somme depth begin_end
    ranks[MAX_NBJOBS + 1]
(184 bytes at MAX_NBJOBS = 20); the receiver sets couts = {couts_somme, 0}.

Here a node is the library's record (int16 job[n], limite1, limite2,
depth, padding; wsbb_node_stride(n) bytes) plus its bound; the reference's
MAX_NBJOBS (20 in its shipped headers) is a parameter, n <= MAX_NBJOBS.
"""
from __future__ import annotations

import numpy as np

from .bound import node_stride

MAX_NBJOBS = 20


# ------------------------------------------------------------ bab.solutions

def parse_solutions(text: str, n: int, max_nbjobs: int = MAX_NBJOBS) -> list[list[dict]]:
    """Every block of a bab.solutions text, each a list of nodes
    {cost, couts1, perm (n jobs), limite1, limite2, depth, job, begin_end}."""
    tok = text.split()
    pos, blocks = 0, []
    width = 3 + max_nbjobs + 5
    while pos < len(tok):
        count = int(tok[pos])
        pos += 1
        block = []
        for _ in range(count):
            v = [int(x) for x in tok[pos:pos + width]]
            if len(v) < width:
                raise ValueError("bab.solutions: truncated record")
            pos += width
            perm = v[3:3 + max_nbjobs]
            tail = v[3 + max_nbjobs:]
            block.append({"cost": v[0], "couts1": v[1], "couts_somme": v[2],
                          "perm": np.array(perm[:n], dtype=np.int32),
                          "limite1": tail[0], "limite2": tail[1], "depth": tail[2],
                          "job": tail[3], "begin_end": tail[4]})
        blocks.append(block)
    return blocks


def read_solutions(path: str, n: int, max_nbjobs: int = MAX_NBJOBS) -> list[dict]:
    """The incumbents the reference would load from `path`: its first block."""
    with open(path) as f:
        blocks = parse_solutions(f.read(), n, max_nbjobs)
    return blocks[0] if blocks else []


def best_incumbent(path: str, n: int, max_nbjobs: int = MAX_NBJOBS):
    """(cost, permutation) of the best record anywhere in the file (every
    block the reference appended), or (None, None) when it holds none; the
    cost is the search's ub0."""
    with open(path) as f:
        blocks = parse_solutions(f.read(), n, max_nbjobs)
    recs = [r for b in blocks for r in b]
    if not recs:
        return None, None
    r = min(recs, key=lambda x: x["cost"])
    return r["cost"], r["perm"]


def format_solutions(solutions, n: int, max_nbjobs: int = MAX_NBJOBS) -> str:
    """One block in the reference's text form: `solutions` are (cost,
    permutation) pairs of complete schedules, written as leaves (limite1 =
    n - 1, limite2 = n, depth = n)."""
    if n > max_nbjobs:
        raise ValueError("n exceeds MAX_NBJOBS of the file format")
    lines = [f"{len(solutions)} "]
    for cost, perm in solutions:
        perm = [int(x) for x in perm][:n]
        if sorted(perm) != list(range(n)):
            raise ValueError("not a permutation of the n jobs")
        vals = [int(cost), 0, int(cost)] + perm + [0] * (max_nbjobs - n)
        vals += [n - 1, n, n, perm[-1], 0]
        lines.append(" ".join(str(v) for v in vals) + " ")
    return "\n".join(lines) + "\n"


def write_solutions(path: str, solutions, n: int, max_nbjobs: int = MAX_NBJOBS,
                    append: bool = False) -> None:
    """Write (or append) one block; a fresh file seeds the reference's
    incumbent exactly as its own reader expects."""
    with open(path, "a" if append else "w") as f:
        f.write(format_solutions(solutions, n, max_nbjobs))


# ------------------------------------------------------- work hand-off packets

def packet_ints(max_nbjobs: int = MAX_NBJOBS) -> int:
    return 2 * max_nbjobs + 6


def pack_work(records: np.ndarray, n: int, lbs, begin_end=None, ranks=None,
              max_nbjobs: int = MAX_NBJOBS) -> bytes:
    """BB_PROBLEM_PACKET payload of library records (int16 rows of
    wsbb_node_stride(n)/2) with their bounds; begin_end and ranks (count x
    (MAX_NBJOBS + 1)) default to zeros."""
    if n > max_nbjobs:
        raise ValueError("n exceeds MAX_NBJOBS of the packet format")
    if len(records) == 0:
        return b""  # nothing to hand off
    rec = np.asarray(records).reshape(len(records), -1)
    count = len(rec)
    out = np.zeros((count, packet_ints(max_nbjobs)), dtype="<i4")
    out[:, :n] = rec[:, :n]
    k = max_nbjobs
    out[:, k] = rec[:, n]              # limite1
    out[:, k + 1] = rec[:, n + 1]      # limite2
    out[:, k + 2] = np.asarray(lbs)    # couts_somme
    out[:, k + 3] = rec[:, n + 2]      # depth
    if begin_end is not None:
        out[:, k + 4] = np.asarray(begin_end)
    if ranks is not None:
        out[:, k + 5:] = np.asarray(ranks).reshape(count, max_nbjobs + 1)
    return out.tobytes()


def unpack_work(data: bytes, n: int, max_nbjobs: int = MAX_NBJOBS):
    """(records, bounds, begin_end, ranks) of a BB_PROBLEM_PACKET payload;
    records in the library's layout, ready for its kernels."""
    w = packet_ints(max_nbjobs)
    a = np.frombuffer(data, dtype="<i4")
    if a.size % w:
        raise ValueError("payload is not a whole number of nodes")
    a = a.reshape(-1, w)
    k = max_nbjobs
    rec = np.zeros((len(a), node_stride(n) // 2), dtype=np.int16)
    rec[:, :n] = a[:, :n]
    rec[:, n] = a[:, k]
    rec[:, n + 1] = a[:, k + 1]
    rec[:, n + 2] = a[:, k + 3]
    return rec, a[:, k + 2].copy(), a[:, k + 4].copy(), a[:, k + 5:].copy()
