#!/usr/bin/env python3
"""Throughput of the GCMC trial-move energy path on GB300.

Workload: the batched isotherm (64 independent chains in one persistent
launch per cycle): 16 pressures log-spaced 0.002-1.0 bar at 293 K x 4 seeded
synthetic frameworks (edges 25.6 / 38.4 / 51.2 / 64.0 A; 1536 / 5184 /
12288 / 24000 atoms; kmax 7 / 10 / 12 / 18; alpha 0.24; cutoff 12.5 A),
rigid CO2, uneven initial loadings 0-800 created on the device, equal
insert / delete / displace / rotate mix, FP32 terms with double-float
(~48-bit) accumulation and structure factor.

A step is one cycle of --moves main-loop iterations on every chain.  The
metric counts trial-move energy evaluations the way the reference spends
them: an insertion or deletion is one evaluation, a displacement, rotation
or translation two (old and new position).  A trial position that fails the
1.5 A overlap test still counts (the reference's energy routine is called
and exits early); the evaluations that ran to completion are reported
beside it as full_evals_per_s.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

prints one JSON line.  --impl reference times the CPU oracle (the FP64
restatement of the reference Fortran; the Fortran itself has no compiler on
either machine) on the host cores for the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "trial-move ΔE evals/sec on 1 GB300, batched vs plain at ≤1e-6 rel ΔE err"
UNIT = "evals/s"
RHO = 192.0 / 12.8 ** 3       # framework atoms per A^3
GUEST_REACH = 1.16            # C-O distance of the CO2 guest


def algorithmic_bytes_per_eval(cutoff: float, nk: int) -> float:
    """16 B per unique environment atom within rc + r_mol (x, y, z, q as
    float4) plus 32 B per k-vector (S(k) read and per-k constants)."""
    import math
    nc = RHO * 4.0 / 3.0 * math.pi * (cutoff + GUEST_REACH) ** 3
    return 16.0 * nc + 32.0 * nk


def trial_evals(st) -> int:
    """Energy evaluations of the trial moves in a chain's counters."""
    a = st.attempts
    return int(a[0] + a[1] + 2 * (a[2] + a[3] + a[4] + a[5]))


def workload(tmp: str):
    from fastmc_gb300 import synthetic as syn
    chains = syn.config3_chains()
    dirs = []
    for f in range(4):
        spec = [c for c in chains if c.fw_seed == f + 1][0]
        d = os.path.join(tmp, f"fw{f + 1}")
        syn.write_inputs(d, spec)
        dirs.append(d)
    specs = [{"system": c.fw_seed - 1, "pressure_pa": c.pressure_bar * 1e5, "seed": 1000 + i,
              "create_molecules": c.create_molecules} for i, c in enumerate(chains)]
    return chains, dirs, specs


# ------------------------------------------------------------ CPU oracle arm
def _cpu_chain(args):
    """Run one oracle chain for `seconds` of main-loop work after its
    pre-loading; returns (evals, moves, overlap_exits, seconds)."""
    d, seed, create, seconds = args
    sys.path.insert(0, ROOT)
    from oracle.binding import Oracle
    o = Oracle(d)
    o.seed(seed)
    if create:
        o.create_molecules(1, create)
    evals = moves = full = 0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        for lg in o.run(50):
            moves += 1
            w = 1 if lg.move in (1, 2) else 2
            evals += w
            if not lg.overlap:
                full += w
    return evals, moves, full, time.perf_counter() - t0


def cpu_sample(dirs, specs, seconds: float, cores: int):
    """A bounded sample of the workload: `cores` chains (spread over the four
    frameworks, the lowest initial loadings so the oracle's pre-loading stays
    short), all run concurrently on separate cores for `seconds` each."""
    import multiprocessing as mp
    byfw = {}
    for s in specs:
        byfw.setdefault(s["system"], []).append(s)
    picks = []
    i = 0
    while len(picks) < cores:
        fw = i % 4
        lst = sorted(byfw[fw], key=lambda s: s["create_molecules"])
        picks.append(lst[(i // 4) % len(lst)])
        i += 1
    jobs = [(dirs[p["system"]], p["seed"], min(p["create_molecules"], 20), seconds) for p in picks]
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        res = pool.map(_cpu_chain, jobs)
    evals = sum(r[0] for r in res)
    moves = sum(r[1] for r in res)
    secs = max(r[3] for r in res)
    sample = (f"{cores} oracle chains (4 frameworks, initial loading <= 20 CO2) run "
              f"concurrently for {seconds:.0f} s each after pre-loading; {moves} moves")
    return evals / secs, moves / secs, sample


def oracle_built():
    from oracle import binding
    binding.build()


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = tempfile.mktemp(suffix=".csv")

    def start(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self, t0=None, t1=None):
        """Median SM clock and the throttle reasons seen between host times
        t0 and t1 (seconds since the epoch; all samples when not given)."""
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        import datetime
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 10:
                continue
            try:
                ts = datetime.datetime.strptime(p[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                clk, cmax = float(p[2]), float(p[3])
            except ValueError:
                continue
            if t0 is not None and not (t0 - 0.025 <= ts <= t1 + 0.025):
                continue
            sm.append(clk)
            smax.append(cmax)
            for n, v in zip(names, p[6:10]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "interval_ms": 20, "reasons": sorted(reasons)}


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic():
    """DRAM bytes (read + write) of one step's chain-kernel launches, from
    the committed ncu summary of this workload, if present."""
    p = os.path.join(ROOT, "profiles", "chain_kernel_config3.json")
    try:
        with open(p) as f:
            return json.load(f).get("dram_bytes_per_step")
    except Exception:
        return None


def reduce_over_ranks(dist, device, max_vals, sum_vals):
    """Replicas: the job's time is the slowest rank's, its work the sum of
    every rank's.  Returns (max_vals, sum_vals) over all ranks."""
    if dist is None:
        return list(max_vals), list(sum_vals)
    import torch
    t = torch.tensor(list(max_vals), device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    e = torch.tensor(list(sum_vals), device=device, dtype=torch.float64)
    dist.all_reduce(e)
    return [float(x) for x in t.tolist()], [float(x) for x in e.tolist()]


def plain_single_chain(F, seconds: float = 2.0):
    """The single-chain GPU paths the batched kernel is compared with, on
    config 1 (25.6 A, 1536 atoms, kmax 7, P 0.1 bar, one CTA):
    - "device": one chain run by the persistent kernel (FP32);
    - "per_move_abi": the drop-in path, one C-ABI call per trial insertion /
      deletion and one per commit, driven from the host (FP64, random
      positions from numpy), the way a Fortran host would call it.
    Both in trial-move ΔE evaluations per second."""
    import numpy as np
    from fastmc_gb300 import synthetic as syn
    d = tempfile.mkdtemp()
    syn.write_inputs(d, syn.config1())
    sysm = F.System.load(d)
    out = {}
    b = F.Batch([sysm], [{"seed": 1}], precision=F.FMC_PREC_FP32, guest_capacity=1024)
    b.run(256)
    s0 = b.stats()[0]
    t0 = time.perf_counter()
    dev_ms = 0.0
    while time.perf_counter() - t0 < seconds:
        b.run(1024)
        dev_ms += b.last_timing()[0]
    s1 = b.stats()[0]
    out["device"] = {"value": (trial_evals(s1) - trial_evals(s0)) / (dev_ms / 1000.0), "unit": UNIT,
                     "workload": "config1 one chain, FP32, device-resident"}
    p = F.PlainEngine(sysm, F.FMC_PREC_FP64, 1024)
    rng = np.random.default_rng(1)
    n = evals = 0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        if n == 0 or rng.random() < 0.5:
            ax = rng.normal(size=3)
            ax /= np.linalg.norm(ax)
            xyz = np.outer([0.0, 1.16, -1.16], ax) + rng.uniform(0, 25.6, 3)
            p.insertion(1, xyz)
        else:
            p.deletion(1, int(rng.integers(1, n + 1)))
        evals += 1
        p.commit(float(rng.random()))
        n = p.nummols(1)
    out["per_move_abi"] = {"value": evals / (time.perf_counter() - t0), "unit": UNIT,
                           "workload": "config1 one chain, FP64, host-driven per-move C ABI "
                                       "(insert/delete, wall time)"}
    return out


# ------------------------------------------------------------------ arms
WORKLOAD = ("config3 batched isotherm: 64 chains = 16 pressures 0.002-1 bar x 4 frameworks "
            "25.6/38.4/51.2/64.0 A, CO2, FP32 terms with double-float sums and S(k)")


def run_reference(args, rank, world):
    if rank != 0:
        return
    oracle_built()
    with tempfile.TemporaryDirectory() as tmp:
        chains, dirs, specs = workload(tmp)
        cores = os.cpu_count() or 1
        per = max(2.0, min(20.0, 120.0 / max(1, args.steps + args.warmup)))
        vals = []
        for i in range(args.warmup + args.steps):
            v, mv, sample = cpu_sample(dirs, specs, per, cores)
            if i >= args.warmup:
                vals.append(v)
        value = statistics.mean(vals)
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": per * 1000.0, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "chains": 64,
                   "sample": "CPU oracle chains of the same 4 frameworks, all host cores"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def run_ours(args, rank, world, local_rank):
    import numpy as np
    import torch

    cpu = None
    if rank == 0 and not args.no_cpu:
        # the CPU baseline runs first, in spawned processes, before CUDA starts
        oracle_built()
        with tempfile.TemporaryDirectory() as tmp:
            _, dirs, specs = workload(tmp)
            cores = os.cpu_count() or 1
            v, mv, sample = cpu_sample(dirs, specs, args.cpu_seconds, cores)
            cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample}

    torch.cuda.set_device(local_rank)
    import fastmc_gb300 as F
    from fastmc_gb300 import build
    build.build()
    F.load()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    tmp = tempfile.mkdtemp()
    chains, dirs, specs = workload(tmp)
    for s in specs:  # replicas: every rank runs its own seeded copy of the batch
        s["seed"] += 100000 * rank
    systems = [F.System.load(d) for d in dirs]
    infos = [s.info() for s in systems]
    batch = F.Batch(systems, specs, precision=F.FMC_PREC_FP32, guest_capacity=1024)
    # CTAs per chain, from timed trial cycles (the chains' state is restored
    # afterwards); set-up, outside the timing
    if args.chain_clusters:
        batch.set_chain_cluster([int(v) for v in args.chain_clusters.split(",")])
    elif args.clusters:
        batch.set_cluster([int(v) for v in args.clusters.split(",")])
    elif not args.no_autotune:
        batch.autotune(args.moves)
    per_chain = batch.chain_cluster()
    clusters = [max(v for v, s in zip(per_chain, specs) if s["system"] == i) for i in range(len(systems))]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # > 129 MB L2

    # per step: the host uploads the chains' fugacities (pinned-free host
    # array) and reads every chain's statistics back through the C ABI;
    # the kernel time comes from CUDA events around the cycle's graph
    fug = np.array([s["pressure_pa"] for s in specs], dtype=np.float64)

    def step(timed_ms, wall):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = batch.run(args.moves, fugacity=fug)
        wall.append(time.perf_counter() - t0)
        ms, ev, mv = batch.last_timing()
        timed_ms.append(ms)
        return st

    clocks = ClockSampler(local_rank)
    clocks.start()  # running before the timed region; samples inside it are kept
    time.sleep(0.5)  # nvidia-smi's start-up
    for _ in range(args.warmup):
        step([], [])
    before = batch.stats()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t_start = time.time()
    ms_list, wall = [], []
    for _ in range(args.steps):
        step(ms_list, wall)
    torch.cuda.synchronize()
    t_end = time.time()
    clk = clocks.stop(t_start, t_end)
    after = batch.stats()
    evals = sum(trial_evals(after[c]) - trial_evals(before[c]) for c in range(len(specs)))
    full = sum(after[c].evals - before[c].evals for c in range(len(specs)))
    moves = sum(after[c].moves - before[c].moves for c in range(len(specs)))
    dev_ms = sum(ms_list)
    e2e_s = sum(wall)
    (dev_ms, e2e_s), (evals, moves, full) = reduce_over_ranks(
        dist, "cuda", [dev_ms, e2e_s], [evals, moves, full])
    value = evals / (dev_ms / 1000.0)

    # roofline of the chain kernel: algorithmic bytes of the completed
    # evaluations per launch over the mean launch time
    alg = 0.0
    for c in range(len(specs)):
        inf = infos[specs[c]["system"]]
        alg += (after[c].evals - before[c].evals) * algorithmic_bytes_per_eval(inf.rcut, inf.newld)
    per_launch_bytes = alg / args.steps
    mean_launch_s = (sum(ms_list) / len(ms_list)) / 1000.0
    achieved = per_launch_bytes / mean_launch_s / 1e9
    peak, peak_kind = measured_peak_hbm()

    h2d, d2h = batch.cycle_bytes()  # fugacities up, chain state records down

    if rank == 0:
        ovl = sum(after[c].overlap_exits - before[c].overlap_exits for c in range(len(specs)))
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded frameworks and guests, no dataset)",
            "config": {"workload": WORKLOAD,
                       "chains": len(specs), "moves_per_step_per_chain": args.moves,
                       "parallelism": f"replicas x{world}",
                       "ctas_per_chain_by_framework": clusters,  # the largest per framework
                       "ctas_per_chain": per_chain,
                       "l2": "flushed (256 MB write) before every timed step"},
            "trial_moves_per_s": moves / (dev_ms / 1000.0),
            "full_evals_per_s": full / (dev_ms / 1000.0),
            "overlap_exits_per_step": ovl / args.steps,
            # one chain-kernel launch per cluster-size group per step
            "gpu_launches": args.steps * len(set(per_chain)),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": profiled_traffic(),
                         "peak_source": peak_kind,
                         "algorithmic_bytes_per_launch": per_launch_bytes},
            "clocks": clk,
            "e2e": {"value": evals / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "cpu_baseline": cpu,
        }
        if not args.no_plain:
            out["plain_single_chain"] = plain_single_chain(F)
        print(json.dumps(out), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--moves", type=int, default=256)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="one CTA per chain")
    ap.add_argument("--no-plain", action="store_true", help="skip the single-chain comparison")
    ap.add_argument("--chain-clusters", default="", help="CTAs per chain, one value per chain")
    ap.add_argument("--clusters", default="", help="CTAs per chain per framework, e.g. 1,2,2,4 "
                    "(default: autotuned)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
