"""Bounded nodes per second of the GB300 LB2 pool path (and its CPU arms).

Workload (one step = one LB2 launch over one pool): permutation flowshop,
n = 20 jobs, m = 20 machines (190 machine pairs), processing times uniform
in [1, 99] from seeds 0-9; one pool of 2^20 partial permutations per
instance (int16 job ids + begin/end cursors, 48-byte records; seeded
uniform-random front/back splits with a 2 % share of leaves). Steps rotate
over the 10 instances, so the 10 pools (503 MB) exceed the 129 MB L2
between uses of the same pool.

  value  device-resident pools: records bounded / second (CUDA events on
         the launching stream, max over ranks)
  e2e    the same through the synchronous host-buffer C-ABI call
         (wsbb_lb2_eval_host) from pinned memory: upload, bound, download
  cpu_baseline / --impl reference: the CPU port of the reference bound
         (oracle/, bit-exact to the reference's compiled bound_flowshop)
         on the host cores
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

N_JOBS, N_MACH, POOL, SEEDS, LEAF_SHARE = 20, 20, 1 << 20, 10, 0.02
METRIC = "bounded nodes/sec (LB2 pool, n=20 m=20)"
UNIT = "nodes/s"


def workload_config(extra: dict | None = None) -> dict:
    cfg = {"workload": "LB2 pool bounds: n=20 jobs, m=20 machines (190 pairs), seeds 0-9, "
                       "one 2^20-record pool per instance, rotated",
           "n": N_JOBS, "m": N_MACH, "pool_records": POOL, "instances": SEEDS,
           "record_bytes": 48, "leaf_share": LEAF_SHARE,
           "l2": "inputs larger than L2 (10 pools x 50.3 MB rotate)"}
    if extra:
        cfg.update(extra)
    return cfg


def alg_ops(recs: np.ndarray, n: int, m: int) -> int:
    """Algorithmic int32 operations of LB2 over a pool: 4 per (pair,
    unscheduled job) step, 3 per pair epilogue, 2 per (fixed job, machine)
    of the front / back times; a leaf is 2 * n * m (its makespan)."""
    P = m * (m - 1) // 2
    l1 = recs[:, n].astype(np.int64)
    l2 = recs[:, n + 1].astype(np.int64)
    leaf = (l2 - l1) == 1
    u = l2 - l1 - 1
    fixed = n - u
    ops = np.where(leaf, 2 * n * m, 4 * P * u + 3 * P + 2 * fixed * m)
    return int(ops.sum())


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
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def cpu_port_rate(nthreads: int, count: int, seed: int = 0) -> tuple[float, dict]:
    """The CPU port of the reference bound (oracle/) on `count` records."""
    from oracle import oracle as O
    p = O.gen_instance(seed, N_JOBS, N_MACH)
    perms, l1, l2 = O.random_pool(1000 + seed, N_JOBS, count, LEAF_SHARE)
    b = O.Bound(p)
    b.eval_batch(perms[:256], l1[:256], l2[:256], nthreads=nthreads)
    t0 = time.perf_counter()
    b.eval_batch(perms, l1, l2, nthreads=nthreads)
    dt = time.perf_counter() - t0
    return count / dt, {"kind": "port", "cores": nthreads,
                        "sample": f"{count} records of the n=20 m=20 seed-{seed} pool, "
                                  f"{nthreads} host threads, {dt:.2f} s"}


SEARCH_N, SEARCH_M, SEARCH_SEEDS = 50, 10, (0, 1, 2, 3, 4)


def cpu_search_rate(seconds: float = 10.0) -> dict:
    """The oracle's sequential search (the reference CPU explorer's
    semantics, single-threaded like one reference peer) on the first search
    instance, capped by node count: bounded nodes per second."""
    from oracle import oracle as O
    p = O.gen_instance(SEARCH_SEEDS[0], SEARCH_N, SEARCH_M)
    ub, _ = O.neh(p)
    b = O.Bound(p)
    cap = 2000
    while True:
        t0 = time.perf_counter()
        rc, st, _ = b.explore(ub0=ub, node_cap=cap)
        dt = time.perf_counter() - t0
        if dt > seconds / 4 or rc == 0:
            break
        cap *= 4
    return {"value": st["bounded"] / dt, "unit": "bounded nodes/s", "cores": 1, "kind": "port",
            "sample": f"first {cap} takes of the n={SEARCH_N} m={SEARCH_M} seed-"
                      f"{SEARCH_SEEDS[0]} search, {dt:.1f} s"}


def search_section(cpu: bool) -> dict:
    """Time-to-proof of the exact GPU search on the persistent-explorer
    instances (n=50, m=10, seeds 0-4, NEH incumbent)."""
    from wsbb_gb300 import search_bench
    out = search_bench.run(SEARCH_N, SEARCH_M, SEARCH_SEEDS, verbose=False)
    sec = {"workload": f"exact DFS time-to-proof, n={SEARCH_N} m={SEARCH_M}, seeds "
                       f"{list(SEARCH_SEEDS)}, NEH initial incumbent, best=99999; tree "
                       "identical to the reference CPU search",
           "all_proved": out["all_proved"], "time_to_proof_s": out["seconds"],
           "bounded_nodes": out["bounded"], "bounded_nodes_per_s": out["bounded_per_s"],
           "evaluated_bounds": out["evaluated"],
           "per_instance": [{k: r[k] for k in ("seed", "optimum", "branched", "pruned",
                                               "leaves", "bounded", "seconds")}
                            for r in out["runs"]]}
    if cpu:
        c = cpu_search_rate()
        sec["cpu_baseline"] = c
        sec["cpu_est_time_to_proof_s"] = out["bounded"] / c["value"]
    return sec


def run_reference(args) -> None:
    rank, world, _ = dist_env()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    count = 1 << 17
    for _ in range(args.warmup):
        cpu_port_rate(cores, 1 << 12)
    rates = []
    t0 = time.perf_counter()
    for k in range(args.steps):
        r, info = cpu_port_rate(cores, count, seed=k % SEEDS)
        rates.append(r)
    wall = time.perf_counter() - t0
    value = args.steps * count / sum(count / r for r in rates)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * wall / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "config": workload_config({"sample_records_per_step": count}),
            "cpu_baseline": {"value": value, "unit": UNIT, "kind": "port", "cores": cores,
                             "sample": f"{count} records per step of the n=20 m=20 pools "
                                       f"(seeds rotate), {cores} host threads; the reference's "
                                       "compiled bound cannot run on this host (its tree is "
                                       "absent), the port is bit-exact to it"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gpu(args) -> None:
    import torch
    import wsbb_gb300 as W

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    ctxs, d_pools, ops = [], [], []
    for s in range(SEEDS):
        p = W.gen_instance(s, N_JOBS, N_MACH)
        ctxs.append(W.Context(p, device=local))
        recs = W.gen_pool(1000 + s + 100 * rank, N_JOBS, POOL, LEAF_SHARE)
        ops.append(alg_ops(recs, N_JOBS, N_MACH))
        d_pools.append(torch.from_numpy(recs).to(dev))
    out = torch.empty(POOL, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream

    def step(k):
        ctxs[k % SEEDS].lb2_eval(d_pools[k % SEEDS].data_ptr(), POOL, out.data_ptr(), sptr)

    for k in range(args.warmup):
        step(k)
    torch.cuda.synchronize(dev)

    peak = None
    import ctypes as C
    pk = C.c_double(0)
    if W.lib().wsbb_probe_maxplus_peak(local, C.byref(pk)) == 0:
        peak = pk.value

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    barrier()
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clk:
        t_wall = time.perf_counter()
        for k in range(args.steps):
            ev[k][0].record(stream)
            step(k)
            ev[k][1].record(stream)
        torch.cuda.synchronize(dev)
        t_wall = time.perf_counter() - t_wall
    barrier()
    per_launch_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = sum(per_launch_ms)
    if world > 1:
        t = torch.tensor([total_ms], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * args.steps * POOL / (total_ms * 1e-3)
    mean_launch_s = statistics.mean(per_launch_ms) * 1e-3
    ops_per_launch = statistics.mean(ops[k % SEEDS] for k in range(args.steps))
    bytes_per_launch = POOL * (48 + 4)

    # end to end through the host-buffer C-ABI call, pinned host memory
    h_pools = [torch.from_numpy(W.gen_pool(1000 + s + 100 * rank, N_JOBS, POOL, LEAF_SHARE))
               .pin_memory() for s in range(2)]
    h_out = torch.empty(POOL, dtype=torch.int32).pin_memory()
    lib = W.lib()
    for k in range(2):
        lib.wsbb_lb2_eval_host(ctxs[k].h, h_pools[k].data_ptr(), POOL, h_out.data_ptr())
    e2e_steps = max(3, min(args.steps, 30))
    barrier()
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        rc = lib.wsbb_lb2_eval_host(ctxs[k % 2].h, h_pools[k % 2].data_ptr(), POOL,
                                    h_out.data_ptr())
        if rc != 0:
            raise RuntimeError(f"wsbb_lb2_eval_host failed: {rc}")
    e2e_s = time.perf_counter() - t0
    if world > 1:
        t = torch.tensor([e2e_s], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_value = world * e2e_steps * POOL / e2e_s

    search = None
    if not args.no_search:
        search = search_section(cpu=(rank == 0 and world == 1))
    if rank == 0:
        cpu = None
        if world == 1:
            cores = os.cpu_count() or 1
            rate, info = cpu_port_rate(cores, 1 << 19)
            cpu = {"value": rate, "unit": UNIT, **info}
        achieved_ops = ops_per_launch / mean_launch_s
        hbm_peak, hbm_src = 6800.0, "fallback (no MEASURED_PEAKS.json)"
        try:
            with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
                hbm_peak = float(json.load(f)["hbm_gbs"])
                hbm_src = "MEASURED_PEAKS.json hbm_gbs (measured)"
        except Exception:
            pass
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "config": workload_config({"parallelism": f"replicas{world}"}),
            "roofline": {"bound": "int32", "achieved": achieved_ops / 1e12,
                         "peak": (peak / 1e12) if peak else None, "unit": "Tops/s",
                         "frac": (achieved_ops / peak) if peak else None, "traffic": None,
                         "kernel": "lb2_pool_kernel",
                         "peak_source": "measured in this run: add+max chains on every SM "
                                        "(wsbb_probe_maxplus_peak)",
                         "ops_per_launch": ops_per_launch},
            "roofline_hbm": {"bound": "hbm", "achieved": bytes_per_launch / mean_launch_s / 1e9,
                             "peak": hbm_peak, "unit": "GB/s",
                             "frac": bytes_per_launch / mean_launch_s / 1e9 / hbm_peak,
                             "peak_source": hbm_src,
                             "bytes_per_launch": bytes_per_launch},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": UNIT,
                    "h2d_bytes_per_step": POOL * 48, "d2h_bytes_per_step": POOL * 4,
                    "steps": e2e_steps},
            "clocks": clk.summary(),
            "gpu_launches": args.steps,
            "wall_s_timed": t_wall,
            "search": search,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="wsbb", choices=["wsbb", "reference"])
    ap.add_argument("--no-search", action="store_true",
                    help="skip the time-to-proof section (search workload)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
