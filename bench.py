#!/usr/bin/env python3
"""Throughput of the GCMC trial-move energy path on GB300.

Workload: the batched isotherm (64 independent chains in one persistent
launch per cycle): 16 pressures log-spaced 0.002-1.0 bar at 293 K x 4 seeded
synthetic frameworks (edges 25.6 / 38.4 / 51.2 / 64.0 A; 1536 / 5184 /
12288 / 24000 atoms; kmax 7 / 10 / 12 / 18; alpha 0.24; cutoff 12.5 A),
rigid CO2, uneven initial loadings 0-800 ("create molecules", run on the
device), equal insert / delete / displace / rotate mix, FP32 terms with
double-float (~48-bit) accumulation and structure factor.

A step is one cycle of --moves main-loop iterations on every chain, always
from the same state: the chains' state right after pre-loading is kept on
the device (fmc_batch_snapshot) and put back before every step
(fmc_batch_restore, outside the timed region), so every step does the same
work and the number does not depend on --steps.  The metric counts trial-move
energy evaluations the way the reference spends them: an insertion or
deletion is one evaluation, a displacement, rotation or translation two (old
and new position).  A trial position that fails the 1.5 A overlap test still
counts (the reference's energy routine is called and exits early); the
evaluations that ran to completion are reported beside it
(full_evals_per_s).

The CPU side runs the same 64 chains: the oracle (the FP64 restatement of
the reference Fortran; the Fortran itself has no compiler on either
machine) pre-loads each chain from the same seed, which gives the same
molecules, keeps that state and replays the same cycle from it every step,
one process per host core.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import math
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
NSITE = 3                     # CO2 sites
WORKLOAD = ("batched isotherm: 64 chains = 16 pressures 0.002-1 bar x 4 frameworks "
            "25.6/38.4/51.2/64.0 A, CO2, FP32 terms with double-float sums and S(k); every step "
            "replays the same cycle from the pre-loaded state")


def n_env(cutoff: float) -> float:
    """Unique framework atoms within rc + r_mol of a molecule."""
    return RHO * 4.0 / 3.0 * math.pi * (cutoff + GUEST_REACH) ** 3


def algorithmic_bytes_per_eval(cutoff: float, nk: int) -> float:
    """16 B per unique environment atom within rc + r_mol (x, y, z, q as
    float4) plus 32 B per k-vector (S(k) read and per-k constants)."""
    return 16.0 * n_env(cutoff) + 32.0 * nk


def algorithmic_flops_per_eval(cutoff: float, nk: int) -> float:
    """20 flop per site and environment atom (minimum image, r^2, test), 40
    per site and neighbour within rc (sqrt, two table interpolations, charge
    products), 12 per site and k-vector (recurrence, charge products) and 8
    per k-vector (S-dot, a_k)."""
    nnb = RHO * 4.0 / 3.0 * math.pi * cutoff ** 3
    return 20.0 * NSITE * n_env(cutoff) + 40.0 * NSITE * nnb + 12.0 * NSITE * nk + 8.0 * nk


def trial_evals(st) -> int:
    """Energy evaluations of the trial moves in a chain's counters (a swap
    is a deletion and an insertion, an acting switch two of each)."""
    a = st.attempts
    return int(a[0] + a[1] + 2 * (a[2] + a[3] + a[4] + a[5] + a[6]) + 4 * a[7])


def workload(tmp: str):
    from fastmc_gb300 import synthetic as syn
    chains = syn.isotherm_chains()
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
def _cpu_worker(conn, jobs, moves, core):
    """One host process: pre-load its chains with the oracle (same seed and
    count as the device chains), keep each state, then per command replay
    `moves` moves of every chain from its kept state and report the work."""
    sys.path.insert(0, ROOT)
    if core is not None:
        try:
            os.sched_setaffinity(0, {core})
        except (AttributeError, OSError):
            pass
    from oracle.binding import Oracle
    sims = []
    for d, seed, create in jobs:
        o = Oracle(d)
        o.seed(seed)
        if create:
            o.create_molecules(1, create)
        o.save_state()
        sims.append(o)
    conn.send(("ready", sum(o.nummols(o.locguest(1)) for o in sims)))
    while True:
        cmd = conn.recv()
        if cmd != "step":
            break
        evals = full = nmov = 0
        t0 = time.perf_counter()
        for o in sims:
            o.restore_state()
            for lg in o.run(moves):
                nmov += 1
                w = 0 if lg.move == 0 else (1 if lg.move in (1, 2) else 2)
                evals += w
                if not lg.overlap:
                    full += w
        conn.send((evals, full, nmov, time.perf_counter() - t0))
    conn.close()


class CpuChains:
    """The workload's chains on `procs` host processes (chains spread by an
    estimate of their cost, largest first), each chain pre-loaded once."""

    def __init__(self, dirs, specs, chain_ids, procs, moves, pin=False):
        import multiprocessing as mp
        ctx = mp.get_context("spawn")
        cost = {}
        for c in chain_ids:
            s = specs[c]
            nk = (7, 10, 12, 18)[s["system"]] ** 3
            cost[c] = nk * (1.0 + s["create_molecules"] / 100.0)
        bins = [[] for _ in range(procs)]
        load = [0.0] * procs
        for c in sorted(chain_ids, key=lambda c: -cost[c]):
            i = min(range(procs), key=lambda k: load[k])
            bins[i].append(c)
            load[i] += cost[c]
        self.conns, self.procs = [], []
        for i, b in enumerate(bins):
            if not b:
                continue
            jobs = [(dirs[specs[c]["system"]], specs[c]["seed"], specs[c]["create_molecules"]) for c in b]
            a, bconn = ctx.Pipe()
            p = ctx.Process(target=_cpu_worker, args=(bconn, jobs, moves, i if pin else None))
            p.start()
            self.conns.append(a)
            self.procs.append(p)
        self.loaded = sum(c.recv()[1] for c in self.conns)
        self.nchains = len(chain_ids)

    def step(self):
        """One replay of every chain; (evals, full evals, moves, wall s)."""
        t0 = time.perf_counter()
        for c in self.conns:
            c.send("step")
        res = [c.recv() for c in self.conns]
        wall = time.perf_counter() - t0
        return (sum(r[0] for r in res), sum(r[1] for r in res), sum(r[2] for r in res), wall)

    def close(self):
        for c in self.conns:
            c.send("stop")
        for p in self.procs:
            p.join()


def cpu_arm(dirs, specs, steps, warmup, moves, cores):
    """The CPU oracle on all `cores` host cores, the same 64 chains and
    pre-loaded states as the device batch; evals/s over the timed steps."""
    cc = CpuChains(dirs, specs, list(range(len(specs))), cores, moves)
    try:
        for _ in range(warmup):
            cc.step()
        ev = fu = mv = 0
        wall = 0.0
        for _ in range(steps):
            e, f, m, w = cc.step()
            ev, fu, mv, wall = ev + e, fu + f, mv + m, wall + w
    finally:
        cc.close()
    return {"value": ev / wall, "full_evals_per_s": fu / wall, "moves": mv, "seconds": wall,
            "loaded_molecules": cc.loaded}


def cpu_one_core(dirs, specs, moves):
    """The oracle on one pinned core: two chains of each framework (the
    chains 4 f + 1 and 4 f + 9 of framework f's 16 pressures), one replay."""
    ids = []
    for f in range(4):
        fc = [c for c, s in enumerate(specs) if s["system"] == f]
        ids += [fc[1], fc[9]]
    cc = CpuChains(dirs, specs, ids, 1, moves, pin=True)
    try:
        cc.step()  # warm-up
        e, f, m, w = cc.step()
    finally:
        cc.close()
    return {"value": e / w, "unit": UNIT, "cores": 1, "full_evals_per_s": f / w,
            "sample": f"oracle pinned to one core: chains {ids} (2 per framework), {m} moves "
                      f"replayed from their pre-loaded states"}


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
    """DRAM bytes (read + write) of one step's chain-kernel launches (the
    unit `achieved` is quoted in) of this workload, from the committed ncu
    summary, if present."""
    p = os.path.join(ROOT, "profiles", "chain_kernel_isotherm64.json")
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


def plain_paths(F, batch, systems, dirs, specs, snap_stats, moves, clusters):
    """The single-chain GPU paths on the same workload and states:
    - "device": every chain run alone (the others paused), from its
      pre-loaded state, on the cluster size that is fastest for a lone chain
      of its framework (4 or 8 CTAs, tried on one chain per framework);
    - "per_move_abi": the drop-in, one C-ABI call per trial move and one per
      commit driven from the host (FP64; insert / delete / displace / rotate
      in equal shares with numpy draws), on one chain per framework loaded
      with that chain's molecules, ~1 s each.
    Both in trial-move evaluations per second."""
    import numpy as np
    out = {}
    n = len(specs)
    best = {}
    for f in range(len(systems)):
        c = [i for i, s in enumerate(specs) if s["system"] == f][8]
        tbest = None
        for cs in (4, 8):
            sizes = [0] * n
            sizes[c] = cs
            batch.set_chain_cluster(sizes)
            batch.restore()
            batch.run(moves)
            ms = batch.last_timing()[0]
            if tbest is None or ms < tbest:
                tbest, best[f] = ms, cs
    ev = 0
    ms_tot = 0.0
    for c in range(n):
        sizes = [0] * n
        sizes[c] = best[specs[c]["system"]]
        batch.set_chain_cluster(sizes)
        batch.restore()
        st = batch.run(moves)
        ev += trial_evals(st[c]) - trial_evals(snap_stats[c])
        ms_tot += batch.last_timing()[0]
    batch.set_chain_cluster(clusters)
    batch.restore()
    out["device"] = {"value": ev / (ms_tot / 1000.0), "unit": UNIT,
                     "workload": "the same 64 chains and states, one chain at a time (FP32, "
                                 "device-resident), cluster per framework " +
                                 str([best[f] for f in range(len(systems))])}
    out["per_move_abi"] = per_move_abi(F, batch, systems, dirs, specs)
    return out


def per_move_abi(F, batch, systems, dirs, specs, seconds=1.0):
    """The drop-in path: one C-ABI call per trial move and one per commit,
    driven from the host through ctypes the way a Fortran host calls it
    (FP64; insert / delete / displace / rotate in equal shares, the draws
    made ahead with numpy), on chain 8 of each framework loaded with that
    chain's pre-loaded molecules, for about `seconds` each.  Beside it the
    CPU oracle on one core runs the same moves with the same decisions
    (energy routine, then the commit), the serial host path the drop-in
    replaces.  Both in trial-move evaluations per second."""
    import ctypes as C
    import numpy as np
    from fastmc_gb300 import _lib as L
    from oracle.binding import Oracle
    lib = L.load()
    res = L.MoveResult()
    acc = C.c_int()
    dp = C.POINTER(C.c_double)
    tot = {"gpu_ev": 0, "gpu_s": 0.0, "cpu_ev": 0, "cpu_s": 0.0}
    for f in range(len(systems)):
        c = [i for i, s in enumerate(specs) if s["system"] == f][8]
        x, m = batch.coords(c)
        mols = x[:9 * m].reshape(m, 3, 3)
        L_box = systems[f].info().cell[0]
        p = F.PlainEngine(systems[f], F.FMC_PREC_FP64, 1024)
        for mol in mols:
            p.insertion(1, mol)
            p.commit(0.0)
        nm = p.nummols(1)
        rng = np.random.default_rng(1 + f)
        nplan = 20000
        kinds = rng.integers(0, 4, nplan)
        u = rng.random(nplan)
        rande = rng.random(nplan)
        ax = rng.normal(size=(nplan, 3))
        ax /= np.linalg.norm(ax, axis=1)[:, None]
        ins = np.ascontiguousarray(np.einsum("i,nj->nij", np.array([0.0, 1.16, -1.16]), ax) +
                                   rng.uniform(0, L_box, (nplan, 1, 3)))
        th = rng.uniform(0, math.pi / 3, nplan)
        abcq = np.zeros((nplan, 7))
        abcq[:, :3] = rng.uniform(-0.25, 0.25, (nplan, 3))
        abcq[kinds == 3, :3] = 0.0  # rotation: no shift
        abcq[:, 3] = np.cos(th / 2)
        abcq[:, 4:] = np.sin(th / 2)[:, None] * ax
        done = []  # (kind, choice, accepted) to replay on the CPU
        evals = 0
        t0 = time.perf_counter()
        k = 0
        while time.perf_counter() - t0 < seconds and k < nplan:
            kd = int(kinds[k]) if nm else 0
            ch = 1 + int(u[k] * nm) if nm else 0
            if kd == 0:
                lib.fmc_insertion(p._h, 1, ins[k].ctypes.data_as(dp), C.byref(res))
                evals += 1
            elif kd == 1:
                lib.fmc_deletion(p._h, 1, ch, C.byref(res))
                evals += 1
            else:
                lib.fmc_displace(p._h, 1, ch, abcq[k].ctypes.data_as(dp), C.byref(res))
                evals += 2
            lib.fmc_metropolis_commit(p._h, float(rande[k]), C.byref(acc))
            done.append((kd, ch, acc.value))
            nm += acc.value if kd == 0 else (-acc.value if kd == 1 else 0)
            k += 1
        tot["gpu_s"] += time.perf_counter() - t0
        tot["gpu_ev"] += evals
        p.close()
        # the same moves and decisions on the oracle, one core
        o = Oracle(dirs[f])
        for mol in mols:
            o.apply_move(1, 1, 0, mol, True)
        t0 = time.perf_counter()
        cev = 0
        for k, (kd, ch, a) in enumerate(done[:2000]):
            if kd == 0:
                o.insertion_energy(1, ins[k])
                o.apply_move(1, 1, 0, ins[k], bool(a))
                cev += 1
            elif kd == 1:
                o.deletion_energy(1, ch)
                o.apply_move(2, 1, ch, None, bool(a))
                cev += 1
            else:
                o.displace_energy(1, ch, abcq[k])
                o.apply_move(3, 1, ch, abcq[k], bool(a))
                cev += 2
        tot["cpu_s"] += time.perf_counter() - t0
        tot["cpu_ev"] += cev
        o.close()
    gpu = tot["gpu_ev"] / tot["gpu_s"]
    cpu = tot["cpu_ev"] / tot["cpu_s"]
    return {"value": gpu, "unit": UNIT, "oracle_1core_same_moves": cpu, "ratio_to_1core": gpu / cpu,
            "workload": "chain 8 of each framework with its pre-loaded molecules, FP64, one C-ABI "
                        "call per move and one per commit from the host (ctypes), wall time; the "
                        "oracle replays the first 2000 of those moves with the same decisions"}


def widom_102A(F, tmp, gcmc_moves=4096):
    """Test insertions into the large framework: 1e7 Widom trials (a 100^3 grid x 10
    orientations, one launch) against the 102.4 A framework (98304 atoms,
    cutoff 14 A, kmax 20) with 2000 CO2 loaded, FP32 terms; then GCMC moves
    of that chain (its cluster autotuned, speculative rounds on): a sample
    of gcmc_moves moves timed, rate per second."""
    from fastmc_gb300 import synthetic as syn
    d = os.path.join(tmp, "widom102")
    syn.write_inputs(d, syn.widom_102A())
    sysm = F.System.load(d)
    b = F.Batch([sysm], [{"seed": 5}], precision=F.FMC_PREC_FP32, guest_capacity=2048)
    b.widom_grid(0, (10, 10, 10), 1, seed=1)  # warm-up
    t0 = time.perf_counter()
    h, nok, ntot = b.widom_grid(0, (100, 100, 100), 10, seed=2)
    s = time.perf_counter() - t0
    b.set_speculation(8)
    b.autotune(256)
    b.run(256)  # warm-up
    st0 = b.stats()[0]
    t0 = time.perf_counter()
    b.run(gcmc_moves)
    sm = time.perf_counter() - t0
    st1 = b.stats()[0]
    return {"value": ntot / s, "unit": "trial insertions/s", "trials": ntot,
            "non_overlapping": nok, "henry": h, "seconds": s,
            "gcmc": {"moves": gcmc_moves, "seconds": sm, "moves_per_s": gcmc_moves / sm,
                     "evals_per_s": (trial_evals(st1) - trial_evals(st0)) / sm,
                     "ctas": b.cluster()[0], "molecules": int(st1.nummols)},
            "workload": "102.4 A, 98304 atoms, 2000 CO2, cutoff 14 A, kmax 20, FP32"}


def sampled_energy_adjoint(F, tmp, nsnap=4096):
    """The sampled energy and its adjoint over a batch of frozen snapshots of
    the 51.2 A framework (12288 atoms, cutoff 12.5 A, alpha 0.24, kmax 12):
    8 FP32 chains pre-loaded with 400 CO2 and run 100 moves each give the
    states (at 0.1 bar a longer run empties them); snapshot q keeps N_q
    (uniform 50-400, at most the state's count) molecules of a random order
    of state q mod 8.  One call (fmc_adjoint_eval_batch, FP32
    pair terms and phases, FP64 sums) returns every snapshot's energy,
    dE/d(guest coordinates) (3N x FP32) and dE/d(eps, sigma, lambda) of the 4
    framework types; the FP64 call on the same batch gives the reference
    gradient.  Host wall time around the call, inputs on the device."""
    import numpy as np
    import torch
    from fastmc_gb300 import synthetic as syn
    from fastmc_gb300.adjoint import Adjoint
    d = os.path.join(tmp, "snapshots51")
    syn.write_inputs(d, syn.single_chain_51A())
    sysm = F.System.load(d)
    b = F.Batch([sysm], [{"seed": 40 + c} for c in range(8)], precision=F.FMC_PREC_FP32,
                guest_capacity=512)
    b.run(100)
    states = []
    for c in range(8):
        x, n = b.coords(c)
        states.append(x[:9 * n].reshape(n, 3, 3))
    rng = np.random.default_rng(11)
    nm = rng.integers(50, 401, size=nsnap)
    parts = []
    for q in range(nsnap):
        st = states[q % 8]
        parts.append(st[rng.permutation(len(st))[:nm[q]]])
    nm = [len(p_) for p_ in parts]
    x = torch.tensor(np.concatenate(parts), dtype=torch.float64, device="cuda")
    adj = Adjoint(sysm)
    p0 = adj.base_params()
    adj.evaluate_batch(x, nm, p0, "fp32")  # warm-up
    times = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e32, g32, p32 = adj.evaluate_batch(x, nm, p0, "fp32")
        times.append(time.perf_counter() - t0)
    t0 = time.perf_counter()
    e64, g64, p64 = adj.evaluate_batch(x, nm, p0, "fp64")
    t64 = time.perf_counter() - t0
    g64n, g32n = g64.cpu().numpy(), g32.cpu().numpy()
    s = min(times)
    return {"value": nsnap / s, "unit": "snapshots/s", "snapshots": nsnap,
            "guest_molecules": int(sum(nm)), "seconds_fp32": s, "seconds_fp64": t64,
            "max_rel_energy_err_fp32": float(np.max(np.abs(e32 - e64) / np.abs(e64))),
            "max_site_grad_err_fp32_rel_to_max": float(np.abs(g32n - g64n).max() / np.abs(g64n).max()),
            "max_param_grad_rel_err_fp32": float(np.max(np.abs(p32 - p64)) / np.abs(p64).max()),
            "workload": f"{nsnap} snapshots, 51.2 A, 12288 framework atoms, 50-400 CO2, "
                        "cutoff 12.5 A, kmax 12, FP32 terms"}


# ------------------------------------------------------------------ arms
def run_reference(args, rank, world):
    if rank != 0:
        return
    oracle_built()
    cores = os.cpu_count() or 1
    with tempfile.TemporaryDirectory() as tmp:
        _, dirs, specs = workload(tmp)
        r = cpu_arm(dirs, specs, args.steps, args.warmup, args.moves, cores)
    value = r["value"]
    sample = (f"the oracle on {cores} processes: the same 64 chains, each pre-loaded from its seed "
              f"({r['loaded_molecules']} molecules), {args.moves} moves replayed from that state per "
              f"step; {r['moves']} timed moves")
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * r["seconds"] / max(1, args.steps), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "chains": len(specs), "moves_per_step_per_chain": args.moves,
                   "same_config": True},
        "full_evals_per_s": r["full_evals_per_s"],
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def run_ours(args, rank, world, local_rank):
    import numpy as np
    import torch

    cpu = cpu1 = None
    tmp = tempfile.mkdtemp()
    chains, dirs, specs = workload(tmp)
    if rank == 0 and not args.no_cpu:
        # the CPU baselines run first, in spawned processes, before CUDA starts
        oracle_built()
        cores = os.cpu_count() or 1
        r = cpu_arm(dirs, specs, args.cpu_steps, 1, args.moves, cores)
        cpu = {"value": r["value"], "unit": UNIT, "cores": cores, "kind": "port",
               "full_evals_per_s": r["full_evals_per_s"],
               "sample": f"the oracle on {cores} processes, the same 64 chains and pre-loaded states "
                         f"({r['loaded_molecules']} molecules), {args.cpu_steps} replays of the "
                         f"{args.moves}-move cycle ({r['moves']} moves, {r['seconds']:.1f} s)"}
        cpu1 = cpu_one_core(dirs, specs, args.moves)

    torch.cuda.set_device(local_rank)
    import fastmc_gb300 as F
    from fastmc_gb300 import build
    build.build()
    F.load()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    for s in specs:  # replicas: every rank runs its own seeded copy of the batch
        s["seed"] += 100000 * rank
    systems = [F.System.load(d) for d in dirs]
    infos = [s.info() for s in systems]
    batch = F.Batch(systems, specs, precision=F.FMC_PREC_FP32, guest_capacity=1024)
    batch.snapshot()  # the pre-loaded state every step starts from
    if args.speculate:
        batch.set_speculation(args.speculate)
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
    batch.restore()
    snap = batch.stats()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # > 129 MB L2
    fug = np.array([s["pressure_pa"] for s in specs], dtype=np.float64)

    def step(ms_list, wall):
        batch.restore()   # the same starting state for every step
        flush.zero_()     # and a cold L2
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = batch.run(args.moves, fugacity=fug)  # public call: fugacities up, records down
        wall.append(time.perf_counter() - t0)
        ms_list.append(batch.last_timing()[0])   # CUDA events around the cycle's graph
        return st

    clocks = ClockSampler(local_rank)
    clocks.start()  # running before the timed region; samples inside it are kept
    time.sleep(0.5)  # nvidia-smi's start-up
    for _ in range(args.warmup):
        step([], [])
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t_start = time.time()
    ms_list, wall = [], []
    for _ in range(args.steps):
        after = step(ms_list, wall)
    torch.cuda.synchronize()
    t_end = time.time()
    clk = clocks.stop(t_start, t_end)
    # per step (every step does the same work from the same state)
    n = len(specs)
    ev1 = sum(trial_evals(after[c]) - trial_evals(snap[c]) for c in range(n))
    full1 = sum(after[c].evals - snap[c].evals for c in range(n))
    mv1 = sum(after[c].moves - snap[c].moves for c in range(n))
    ovl1 = sum(after[c].overlap_exits - snap[c].overlap_exits for c in range(n))
    dev_ms = sum(ms_list)
    e2e_s = sum(wall)
    (dev_ms, e2e_s), (evals, moves, full) = reduce_over_ranks(
        dist, "cuda", [dev_ms, e2e_s], [ev1 * args.steps, mv1 * args.steps, full1 * args.steps])
    value = evals / (dev_ms / 1000.0)

    # rooflines of the chain kernel (the only kernel in the timed step):
    # algorithmic bytes and flops of the completed evaluations per step over
    # the mean step time
    alg_b = alg_f = 0.0
    for c in range(n):
        inf = infos[specs[c]["system"]]
        fe = after[c].evals - snap[c].evals
        alg_b += fe * algorithmic_bytes_per_eval(inf.rcut, inf.newld)
        alg_f += fe * algorithmic_flops_per_eval(inf.rcut, inf.newld)
    mean_s = (sum(ms_list) / len(ms_list)) / 1000.0
    achieved = alg_b / mean_s / 1e9
    peak, peak_kind = measured_peak_hbm()
    import ctypes as C
    from fastmc_gb300 import _lib as L
    fp32 = C.c_double()
    L.check(L.load().fmc_measure_fp32_peak(C.byref(fp32)))

    h2d, d2h = batch.cycle_bytes()  # fugacities up, chain state records down
    loads = [snap[c].nummols for c in range(n)]
    # each chain's own device time in the last step (its CTAs' kernel time)
    chain_ms = {}
    for f in range(len(systems)):
        t = sorted((after[c].device_ns - snap[c].device_ns) / 1e6 for c in range(n)
                   if specs[c]["system"] == f)
        chain_ms[f"fw{f + 1}"] = {"max": t[-1], "median": t[len(t) // 2]}

    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded frameworks and guests, no dataset)",
            "config": {"workload": WORKLOAD,
                       "chains": n, "moves_per_step_per_chain": args.moves,
                       "parallelism": f"replicas x{world}",
                       "ctas_per_chain_by_framework": clusters,  # the largest per framework
                       "ctas_per_chain": per_chain,
                       "molecules_at_step_start": {"total": sum(loads), "max": max(loads),
                                                   "mean": sum(loads) / n},
                       "same_config": True,
                       "speculative_proposals": args.speculate,
                       "l2": "flushed (256 MB write) before every timed step"},
            "trial_moves_per_s": moves / (dev_ms / 1000.0),
            "full_evals_per_s": full / (dev_ms / 1000.0),
            "overlap_exits_per_step": ovl1,
            "chain_ms_per_step": chain_ms,
            # one chain-kernel launch per cluster-size group per step
            "gpu_launches": args.steps * len(set(per_chain)),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": profiled_traffic(),
                         "peak_source": peak_kind,
                         "algorithmic_bytes_per_launch": alg_b},
            "roofline_flops": {"achieved": alg_f / mean_s / 1e12, "peak": fp32.value,
                               "unit": "TFLOP/s", "frac": alg_f / mean_s / 1e12 / fp32.value,
                               "peak_source": "FP32 FMA loop measured in this run "
                                              "(fmc_measure_fp32_peak)",
                               "algorithmic_flops_per_launch": alg_f},
            "clocks": clk,
            "e2e": {"value": evals / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "cpu_baseline": cpu,
            "cpu_baseline_1core": cpu1,
        }
        if not args.no_plain:
            out["plain_single_chain"] = plain_paths(F, batch, systems, dirs, specs, snap, args.moves,
                                                    per_chain)
        if not args.no_widom:
            out["widom_102A"] = widom_102A(F, tmp)
        if not args.no_adjoint:
            out["sampled_energy_adjoint"] = sampled_energy_adjoint(F, tmp, args.snapshots)
        print(json.dumps(out), flush=True)
    if dist:
        dist.destroy_process_group()


def profile_case(args):
    """A small fixed workload for ncu captures of the chain kernel: the
    first `--chains` chains (from `--first`) of one framework with their
    initial loadings, `--launches` cycles of `--moves` moves, printing the
    device time of each.  Launches in order: the pre-loading launch (when
    the chains pre-load guests), then one chain-kernel launch per cycle, so
    `ncu -k regex:chain_kernel -s 2 -c 1` captures the second cycle."""
    import fastmc_gb300 as F
    from fastmc_gb300 import build
    from fastmc_gb300 import synthetic as syn
    build.build()
    chains = syn.isotherm_chains()
    sel = [(i, c) for i, c in enumerate(chains) if c.fw_seed == args.framework]
    sel = sel[args.first:args.first + args.chains]
    d = os.path.join(tempfile.mkdtemp(), "fw")
    syn.write_inputs(d, sel[0][1])
    sysm = F.System.load(d)
    specs = [{"system": 0, "pressure_pa": c.pressure_bar * 1e5, "seed": 1000 + i,
              "create_molecules": c.create_molecules} for i, c in sel]
    prec = F.FMC_PREC_FP64 if args.fp64 else F.FMC_PREC_FP32
    b = F.Batch([sysm], specs, precision=prec, guest_capacity=1024)
    b.set_cluster([args.cluster])
    if args.speculate and not args.fp64:
        b.set_speculation(args.speculate)
    for it in range(args.launches):
        st = b.run(args.moves)
        ms, ev, mv = b.last_timing()
        print(f"launch {it}: {ms:.3f} ms, {mv} moves, {ev} full evaluations, "
              f"N = {[s.nummols for s in st]}", flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--moves", type=int, default=256)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=3, help="timed replays of the CPU baseline")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="one CTA per chain")
    ap.add_argument("--no-plain", action="store_true", help="skip the single-chain comparison")
    ap.add_argument("--no-widom", action="store_true",
                    help="skip timing 1e7 Widom trials against the 102.4 A framework")
    ap.add_argument("--no-adjoint", action="store_true",
                    help="skip timing the sampled-energy adjoint of 4096 snapshots (51.2 A box)")
    ap.add_argument("--adjoint-only", action="store_true",
                    help="time only the sampled-energy adjoint and print its JSON line")
    ap.add_argument("--snapshots", type=int, default=4096, help="snapshots of the adjoint batch")
    ap.add_argument("--speculate", type=int, default=8,
                    help="speculative proposals per round at most (2..8; 0: off); the chains' "
                         "moves are the same either way")
    ap.add_argument("--chain-clusters", default="", help="CTAs per chain, one value per chain")
    ap.add_argument("--clusters", default="", help="CTAs per chain per framework, e.g. 1,2,2,4 "
                    "(default: autotuned)")
    ap.add_argument("--profile-case", action="store_true",
                    help="run the small profiling workload below instead of the benchmark")
    ap.add_argument("--framework", type=int, default=4, choices=[1, 2, 3, 4])
    ap.add_argument("--chains", type=int, default=1)
    ap.add_argument("--first", type=int, default=0, help="first chain of the framework")
    ap.add_argument("--launches", type=int, default=3)
    ap.add_argument("--fp64", action="store_true")
    ap.add_argument("--cluster", type=int, default=1, help="CTAs per chain (1..8)")
    args = ap.parse_args()
    if args.profile_case:
        profile_case(args)
        return
    if args.adjoint_only:
        import fastmc_gb300 as F
        with tempfile.TemporaryDirectory() as tmp:
            print(json.dumps(sampled_energy_adjoint(F, tmp, args.snapshots)), flush=True)
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
