"""Bounded nodes per second of the exact GB300 flowshop search, with the
per-child, learned and CPU arms on the same tree.

Workload (one step = one search): permutation flowshop n = 50 jobs, m = 20
machines (190 machine pairs), processing times uniform in [1, 99] from seed
0; begin-end branching from the NEH incumbent with side-choice threshold
best = NEH (the learned-selector configuration); a step explores the first
250 M nodes of the tree (a node budget: the search commits in DFS order, so
that is the same tree prefix whatever the window), with the window and
family-bounds tile the autotuner picks for this GPU (wsbb_gb300.autotune,
untimed). Every step's counters are checked against the first step's. The search state grows to
gigabytes over a step, far beyond the 129 MB L2; L2 is also flushed between
steps.

  value  bounded nodes (child LB2 evaluations of the tree) per second of
         the search with family bounds (every child of a father bounded
         from the father's shared max-plus pair passes), the search state
         resident in HBM; CUDA events on the launching stream, max over
         ranks
  arms   the same tree searched with per-child LB2 (the reference GPU
         kernel's form), with the learned K-pair test ahead of per-child
         LB2, and with the learned test ahead of family bounds
  e2e    the same metric through the C-ABI from host memory: every step
         creates the context from the host instance (table upload), runs
         the search (state reads, stats and incumbent to the host) and
         destroys it
  roofline  the dominant kernel (family bounds) on a father pool through
         wsbb_decompose_lb2, against the INT32 add/max issue peak measured
         in this run
  cpu_baseline / --impl reference: the CPU port of the reference explorer
         (oracle/, its semantics and counters) on the host cores
Sections: the LB2 pool kernel (n=20 m=20 pools of 2^20 records), the
time-to-proof of the n=50 m=10 instances (seeds 0-4) and 64 mixed instances
searched concurrently (wsbb_gb300.multi_bench).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("bounded nodes/sec & time-to-proof (learned+batched vs plain GPU LB2 vs CPU), "
          "same tree")
UNIT = "bounded nodes/s"
# one step: the first S_NODES tree nodes of the search (the search commits
# in DFS order, so that is the same tree prefix whatever the window)
S_N, S_M, S_NODES, S_ITER_CAP = 50, 20, 250_000_000, 20_000
MODEL = os.path.join(ROOT, "wsbb_gb300", "models", f"selector_n{S_N}_m{S_M}.npz")
TREE_KEYS = ("branched", "pruned", "leaves", "improved", "bounded", "best_cost", "coverage")
# kernels per search iteration (family bounds): commit, doom, select x3,
# region copy, family bounds, choose, kept scan, emit, finish
KERNELS_PER_ITER = 11

POOL_N, POOL_M, POOL, POOL_SEEDS, LEAF_SHARE = 20, 20, 1 << 20, 10, 0.02
# DRAM bytes (read + write) of one roofline launch of the family kernel, from
# the ncu capture summarised in profiles/family_kernel_n50m20.md
FAMILY_DRAM_BYTES_PER_LAUNCH = 4.05e6
PROOF_N, PROOF_M, PROOF_SEEDS = 50, 10, (0, 1, 2, 3, 4)


def workload_config(seed: int, extra: dict | None = None) -> dict:
    cfg = {"workload": f"exact begin-end DFS, n={S_N} jobs m={S_M} machines (190 pairs), "
                       f"seed {seed}, NEH incumbent, best=NEH, the first {S_NODES // 10**6} M tree "
                       "nodes per step (autotuned window and tile)",
           "n": S_N, "m": S_M, "seed": seed, "tree_nodes_per_step": S_NODES,
           "l2": "search state >> L2 (GBs), L2 flushed between steps"}
    if extra:
        cfg.update(extra)
    return cfg


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.rows: list[list[str]] = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.device),
                                      f"--query-gpu={self.Q}", "--format=csv,noheader,nounits"],
                                     capture_output=True, text=True, timeout=5).stdout
                for line in out.strip().splitlines():
                    self.rows.append([x.strip() for x in line.split(",")])
            except Exception:
                pass
            self._stop.wait(0.1)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self) -> dict:
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows if len(r) >= 9
                          for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


# ------------------------------------------------------------ CPU (oracle port)

def cpu_search_rate(seed: int, threads: int, seconds: float, n: int = S_N, m: int = S_M,
                    best_is_ub: bool = True) -> dict:
    """The oracle's sequential explorer (the reference CPU explorer's
    semantics and counters) on the headline instance, capped by takes so
    that one run lasts about `seconds`. With threads > 1, that many
    independent explorer runs of the same sample in parallel (ctypes drops
    the GIL): the throughput of the host cores, as independent reference
    peers would give it."""
    from concurrent.futures import ThreadPoolExecutor

    from oracle import oracle as O
    p = O.gen_instance(seed, n, m)
    ub, _ = O.neh(p)
    best = ub if best_is_ub else 99999
    cap = 500
    while True:
        t0 = time.perf_counter()
        O.Bound(p).explore(ub0=ub, best=best, node_cap=cap)
        dt = time.perf_counter() - t0
        if dt > seconds / 8:
            break
        cap *= 2
    cap = max(cap, int(cap * seconds / max(dt, 1e-3)))

    def one(_):
        rc, st, _ = O.Bound(p).explore(ub0=ub, best=best, node_cap=cap)
        return st["bounded"]

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        total = sum(ex.map(one, range(threads)))
    dt = time.perf_counter() - t0
    return {"value": total / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"first {cap} takes of the n={n} m={m} seed-{seed} search "
                      f"(best={'NEH' if best_is_ub else 99999}), "
                      f"{threads} independent run(s) in parallel, {dt:.1f} s"}


def run_reference(args) -> None:
    rank, world, _ = dist_env()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_search_rate(0, 1, 0.2)
    rates, t0 = [], time.perf_counter()
    for _ in range(args.steps):
        rates.append(cpu_search_rate(0, cores, 3.0))
    wall = time.perf_counter() - t0
    value = statistics.mean(r["value"] for r in rates)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * wall / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "config": workload_config(0, {"parallelism": "host threads"}),
            "cpu_baseline": {"value": value, "unit": UNIT, "kind": "port", "cores": cores,
                             "sample": rates[-1]["sample"] + "; the reference's compiled "
                             "explorer cannot run on this host (its source tree is absent), "
                             "the port reproduces its node counts exactly"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------- GPU arms

def family_alg_ops(recs: np.ndarray, n: int, m: int) -> int:
    """Algorithmic int32 operations of family bounds over a father pool:
    per (pair, free job) 7 in the forward and 12 in the backward max-plus
    pass; per (child, pair) 9 (two ends of the walk, two back terms, the
    max); 2 per (fixed job, machine) for the father's front and back and 4
    per (free job, machine) for the children's. Two-free-job fathers: their
    two leaves' makespans (3 per machine each)."""
    P = m * (m - 1) // 2
    l1 = recs[:, n].astype(np.int64)
    l2 = recs[:, n + 1].astype(np.int64)
    u = l2 - l1 - 1
    fixed = n - u
    ops = np.where(u == 2, 2 * fixed * m + 6 * m,
                   19 * P * u + 9 * P * 2 * u + 2 * fixed * m + 4 * u * m)
    return int(ops.sum())


def father_pool(seed: int, n: int, count: int) -> np.ndarray:
    """Fathers with u free jobs uniform in [3, n], front / back split uniform."""
    import wsbb_gb300 as W
    rng = np.random.default_rng(seed)
    perms = np.argsort(rng.random((count, n)), axis=1).astype(np.int32)
    u = rng.integers(3, n + 1, count)
    f = (rng.random(count) * (n - u + 1)).astype(np.int64)
    l1 = (f - 1).astype(np.int32)
    l2 = (f + u).astype(np.int32)
    return W.pack_records(perms, l1, l2)


def roofline_family(ctx, dev, stream, sptr, peak) -> dict:
    import torch
    import wsbb_gb300 as W
    count = 1 << 15
    recs = father_pool(11, S_N, count)
    u = recs[:, S_N + 1].astype(np.int64) - recs[:, S_N].astype(np.int64) - 1
    nkids = np.where(u == 2, 2, 2 * u)
    off = np.concatenate([[0], np.cumsum(nkids)]).astype(np.int64)
    d_f = torch.from_numpy(recs).to(dev)
    d_off = torch.from_numpy(off).to(dev)
    lb = torch.empty(int(off[-1]), dtype=torch.int32, device=dev)
    job = torch.empty(int(off[-1]), dtype=torch.int16, device=dev)
    for _ in range(3):
        ctx.decompose_lb2(d_f.data_ptr(), count, d_off.data_ptr(), lb.data_ptr(), job.data_ptr(),
                          sptr)
    launches = 20
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(dev)
    e0.record(stream)
    for _ in range(launches):
        ctx.decompose_lb2(d_f.data_ptr(), count, d_off.data_ptr(), lb.data_ptr(), job.data_ptr(),
                          sptr)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    t = e0.elapsed_time(e1) * 1e-3 / launches
    ops = family_alg_ops(recs, S_N, S_M)
    achieved = ops / t
    bytes_ = recs.nbytes + off.nbytes + int(off[-1]) * 6
    return {"bound": "int32", "achieved": achieved / 1e12,
            "peak": peak / 1e12 if peak else None, "unit": "Tops/s",
            "frac": achieved / peak if peak else None,
            "traffic": FAMILY_DRAM_BYTES_PER_LAUNCH,
            "traffic_source": "dram__bytes_read.sum + dram__bytes_write.sum of this launch, "
                              "one ncu capture (profiles/family_kernel_n50m20.md): the tables "
                              "and records stay in L2, far below the algorithmic bytes",
            "algorithmic_bytes": bytes_,
            "peak_note": "the probe's chains issue one thread instruction per counted "
                         "operation (a subtraction and a fused add+max: two operations, two "
                         "instructions) at ~98 % of the SMs' issue rate; the algorithmic "
                         "count counts an add and a max as two operations too",
            "kernel": "family_staged_kernel (wsbb_decompose_lb2)",
            "workload": f"{count} fathers n={S_N} m={S_M}, u uniform in [3, {S_N}]",
            "launch_ms": t * 1e3, "ops_per_launch": ops,
            "peak_source": "measured in this run: add+max chains on every SM "
                           "(wsbb_probe_maxplus_peak)",
            "hbm_achieved_gbs": bytes_ / t / 1e9}


def lb2_pool_section(dev, stream, sptr, peak, launches: int) -> dict:
    """The per-record LB2 kernel on pools of 2^20 records (n=20 m=20,
    seeds 0-9, rotated so that the 503 MB of pools exceed L2)."""
    import torch
    import wsbb_gb300 as W
    ctxs, pools, ops = [], [], []
    P = POOL_M * (POOL_M - 1) // 2
    for s in range(POOL_SEEDS):
        ctxs.append(W.Context(W.gen_instance(s, POOL_N, POOL_M), device=dev.index))
        recs = W.gen_pool(1000 + s, POOL_N, POOL, LEAF_SHARE)
        l1 = recs[:, POOL_N].astype(np.int64)
        l2 = recs[:, POOL_N + 1].astype(np.int64)
        u = l2 - l1 - 1
        ops.append(int(np.where(u == 0, 2 * POOL_N * POOL_M,
                                4 * P * u + 3 * P + 2 * (POOL_N - u) * POOL_M).sum()))
        pools.append(torch.from_numpy(recs).to(dev))
    out = torch.empty(POOL, dtype=torch.int32, device=dev)
    for k in range(3):
        ctxs[k].lb2_eval(pools[k].data_ptr(), POOL, out.data_ptr(), sptr)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(launches)]
    torch.cuda.synchronize(dev)
    for k in range(launches):
        ev[k][0].record(stream)
        ctxs[k % POOL_SEEDS].lb2_eval(pools[k % POOL_SEEDS].data_ptr(), POOL, out.data_ptr(),
                                      sptr)
        ev[k][1].record(stream)
    torch.cuda.synchronize(dev)
    ms = [a.elapsed_time(b) for a, b in ev]
    t = statistics.mean(ms) * 1e-3
    op = statistics.mean(ops[k % POOL_SEEDS] for k in range(launches))
    return {"workload": "LB2 of pools of 2^20 records, n=20 m=20 (190 pairs), seeds 0-9 "
                        "rotated (pools exceed L2)",
            "records_per_s": launches * POOL / (sum(ms) * 1e-3), "launches": launches,
            "roofline": {"bound": "int32", "achieved": op / t / 1e12,
                         "peak": peak / 1e12 if peak else None, "unit": "Tops/s",
                         "frac": op / t / peak if peak else None,
                         "kernel": "lb2_fast_kernel"},
            "hbm_gbs": POOL * 52 / t / 1e9}


def proof_section() -> dict:
    from wsbb_gb300 import search_bench
    out = search_bench.run(PROOF_N, PROOF_M, PROOF_SEEDS, verbose=False, tune=True)
    import wsbb_gb300 as W
    from wsbb_gb300.explorer import explore
    res_s, res_ok = 0.0, True
    for sd in PROOF_SEEDS:
        p = W.gen_instance(sd, PROOF_N, PROOF_M)
        ctx = W.Context(p)
        r = explore(ctx, ub0=W.neh(p)[0], best=99999, window=out["shape"]["window"],
                    resident=True)
        res_s += r["seconds"]
        res_ok = res_ok and r["status"] == 0
        ctx.close()
    return {"workload": f"exact DFS to a proven optimum, n={PROOF_N} m={PROOF_M}, seeds "
                        f"{list(PROOF_SEEDS)}, NEH incumbent, best=99999 (the reference "
                        "default), autotuned window and tile",
            "resident_time_to_proof_s": res_s, "resident_all_proved": res_ok,
            "shape": out["shape"],
            "all_proved": out["all_proved"], "time_to_proof_s": out["seconds"],
            "bounded_nodes": out["bounded"], "bounded_nodes_per_s": out["bounded_per_s"],
            "per_instance": [{k: r[k] for k in ("seed", "optimum", "branched", "pruned",
                                                "leaves", "bounded", "seconds")}
                             for r in out["runs"]]}


def run_roofline_only() -> None:
    """The roofline measurement alone: family bounds on the father pool."""
    import ctypes as C

    import torch

    import wsbb_gb300 as W
    dev = torch.device("cuda", 0)
    ctx = W.Context(W.gen_instance(0, S_N, S_M))
    stream = torch.cuda.current_stream(dev)
    pk = C.c_double(0)
    peak = pk.value if W.lib().wsbb_probe_maxplus_peak(0, C.byref(pk)) == 0 else None
    print(json.dumps(roofline_family(ctx, dev, stream, stream.cuda_stream, peak)), flush=True)


def run_gpu(args) -> None:
    import ctypes as C

    import torch

    import wsbb_gb300 as W
    from wsbb_gb300.explorer import explore
    from wsbb_gb300.learned import Model, explore_learned

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    from wsbb_gb300.replicas import aggregate, replica_seed

    # replicas: rank r searches its own instance (weak scaling)
    seed = replica_seed(rank)
    p = W.gen_instance(seed, S_N, S_M)
    ub0, _ = W.neh(p)
    ctx = W.Context(p, device=local)
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    # launch shapes (window, family-bounds tile) from the autotuner: a short
    # prefix of this search per candidate, untimed
    from wsbb_gb300 import autotune
    shape = autotune.tuned(ctx, ub0, ub0, device=local, node_budget=S_NODES)
    win, kb = shape["window"], shape["family_smem_kb"]

    def step():
        return explore(ctx, ub0=ub0, best=ub0, max_iters=S_ITER_CAP, max_bounded=S_NODES,
                       stream=sptr, window=win,
                       family_smem_kb=kb)

    ref = None
    for _ in range(args.warmup):
        r = step()
        ref = ref or r
    peak = None
    pk = C.c_double(0)
    if W.lib().wsbb_probe_maxplus_peak(local, C.byref(pk)) == 0:
        peak = pk.value

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    same = True
    bounded = 0
    barrier()
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clk:
        t_wall = time.perf_counter()
        for k in range(args.steps):
            flush.zero_()
            ev[k][0].record(stream)
            r = step()
            ev[k][1].record(stream)
            bounded += r["bounded"]
            same &= all(r[key] == ref[key] for key in TREE_KEYS)
        torch.cuda.synchronize(dev)
        t_wall = time.perf_counter() - t_wall
    barrier()
    _, slow_s, value = aggregate(bounded, sum(a.elapsed_time(b) for a, b in ev) * 1e-3)
    total_ms = slow_s * 1e3
    launches = args.steps * (ref["iterations"] * KERNELS_PER_ITER + 1)

    # end to end through the C-ABI from host memory
    L = W.lib()
    h_p = np.ascontiguousarray(p, dtype=np.int32)
    from wsbb_gb300.explorer import ExploreCfg, ExploreStats
    cfg = ExploreCfg(ub0, ub0, win, 0, 0, S_ITER_CAP, 0, kb, S_NODES)
    e2e_steps = max(2, min(args.steps, 5))
    h2d = d2h = 0
    e2e_bounded = 0
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        h = C.c_void_p()
        rc = L.wsbb_ctx_create(h_p.ctypes.data, S_N, S_M, local, C.byref(h))
        if rc != 0:
            raise RuntimeError(f"wsbb_ctx_create failed: {rc}")
        st = ExploreStats()
        rc = L.wsbb_explore(h, C.byref(cfg), C.byref(st), None)
        if rc != 0:
            raise RuntimeError(f"wsbb_explore failed: {rc}")
        h2d = int(L.wsbb_ctx_device_bytes(h)) + C.sizeof(cfg)
        d2h = int(st.d2h_bytes) + C.sizeof(st)
        e2e_bounded += st.bounded
        L.wsbb_ctx_destroy(h)
    _, _, e2e_value = aggregate(e2e_bounded, time.perf_counter() - t0)

    arms = sections = cpu = roof = None
    if rank == 0:
        def arm(r, base_s):
            return {"seconds": r["seconds"], "bounded_per_s": r["bounded"] / r["seconds"],
                    "same_tree": all(r[k] == ref[k] for k in TREE_KEYS),
                    "speedup_vs_per_child_lb2": base_s / r["seconds"]}
        fam = step()
        per = explore(ctx, ub0=ub0, best=ub0, max_iters=S_ITER_CAP, max_bounded=S_NODES,
                      stream=sptr, child_lb2=True,
                      window=win)
        arms = {"per_child_lb2": arm(per, per["seconds"]), "family_lb2": arm(fam, per["seconds"])}
        # the resident search stopped at the step's iteration count: the same prefix
        res = explore(ctx, ub0=ub0, best=ub0, max_iters=fam["iterations"], stream=sptr,
                      window=win, resident=True)
        arms["resident_family_lb2"] = arm(res, per["seconds"])
        if os.path.exists(MODEL):
            model = Model(S_N, S_M)
            model.load(MODEL)
            for K, pc in ((16, True), (4, False)):
                q = explore_learned(ctx, model, K, ub0=ub0, best=ub0, max_iters=S_ITER_CAP,
                                    max_bounded=S_NODES,
                                    stream=sptr, child_lb2=pc, window=win)
                a = arm(q, per["seconds"])
                a["early_share"] = q["early"] / max(1, q["evaluated"])
                a["settled_fathers_share"] = q["settled_fathers"] / max(1, q["branched"])
                arms[f"learned_k{K}_{'per_child' if pc else 'family'}_lb2"] = a
        roof = roofline_family(ctx, dev, stream, sptr, peak)
        sections = {"lb2_pool": lb2_pool_section(dev, stream, sptr, peak, 40)}
        if not args.no_proof:
            sections["time_to_proof"] = proof_section()
        if args.proof_seconds > 0:
            from wsbb_gb300 import proof_progress
            sections["headline_proof_progress"] = {
                "workload": f"the headline search (n={S_N} m={S_M} seed {seed}, NEH "
                            f"incumbent) run for {args.proof_seconds:g} s of device time: "
                            "the share of the n! permutations its exact prefix covers "
                            "(the reference's coverage weights) and the time to proof "
                            "extrapolated linearly from it",
                "runs": [proof_progress.run(S_N, S_M, seed, mode, args.proof_seconds, window=win,
                                            device=local)
                         for mode in ("ub0", "default")]}
        if not args.no_multi:
            from wsbb_gb300 import multi_bench
            sections["multi_instance"] = multi_bench.run()
            sections["multi_instance"]["workload"] = (
                "64 instances, n in {20,50,100} x m in {5,10,20}, seeds 0-63, NEH incumbent, "
                "best=NEH, each to its proof or 10^9 bounded nodes, all in one resident launch "
                "(resident_full); arms compared at 2*10^7 nodes each: the resident launch, "
                "64 graph-launched searches on 8 host threads, and per-child LB2 with and "
                "without the learned test on the m=20 instances with a trained selector")
        if world == 1:
            cores = os.cpu_count() or 1
            cpu = cpu_search_rate(0, cores, 8.0)
            cpu["single_thread"] = cpu_search_rate(0, 1, 4.0)["value"]
            if sections.get("time_to_proof"):
                tp = sections["time_to_proof"]
                c10 = cpu_search_rate(PROOF_SEEDS[0], 1, 4.0, PROOF_N, PROOF_M, False)
                tp["cpu_baseline_1_core"] = c10
                tp["cpu_est_time_to_proof_s_1_core"] = tp["bounded_nodes"] / c10["value"]
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int32", "data": "synthetic",
            "config": workload_config(seed, {"parallelism": f"replicas{world}",
                                             "bounded_per_step": ref["bounded"],
                                             "same_tree_every_step": same,
                                             "window": win, "family_smem_kb": kb,
                                             "shapes": "autotuned (wsbb_gb300.autotune)"}),
            "roofline": roof, "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "steps": e2e_steps},
            "clocks": clk.summary(), "gpu_launches": launches, "wall_s_timed": t_wall,
            "arms": arms, "sections": sections,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="wsbb", choices=["wsbb", "reference"])
    ap.add_argument("--no-proof", action="store_true",
                    help="skip the time-to-proof section (n=50 m=10, seeds 0-4)")
    ap.add_argument("--no-multi", action="store_true",
                    help="skip the multi-instance section (64 concurrent instances)")
    ap.add_argument("--proof-seconds", type=float, default=20.0,
                    help="device seconds of the headline search per best setting for the "
                         "proof-progress section (0: skip it)")
    ap.add_argument("--only", choices=["roofline"], default=None,
                    help="run one measurement alone (a small case for profilers)")
    args = ap.parse_args()
    if args.only == "roofline":
        run_roofline_only()
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
