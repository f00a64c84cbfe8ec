"""Small, fixed workloads for profiling the chain kernel.

    python -m fastmc_gb300.profile_case --framework 4 --chains 1 --moves 64 --launches 3 [--cluster 4]

builds one of the four batched-isotherm frameworks (1: 25.6 A ... 4: 64.0 A),
creates the first `--chains` chains of that framework with their initial
loadings, and runs `--launches` cycles of `--moves` moves, printing the
device time of each.  Kernel launches in order: the "create molecules"
launch (when a chain pre-loads guests), then one chain-kernel launch per
cycle, so `ncu -k regex:chain_kernel -s 2 -c 1` captures the second cycle.
"""
from __future__ import annotations

import argparse
import os
import tempfile


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--framework", type=int, default=4, choices=[1, 2, 3, 4])
    ap.add_argument("--chains", type=int, default=1)
    ap.add_argument("--first", type=int, default=0, help="index of the first chain of the framework")
    ap.add_argument("--moves", type=int, default=64)
    ap.add_argument("--launches", type=int, default=3)
    ap.add_argument("--fp64", action="store_true")
    ap.add_argument("--cluster", type=int, default=1, help="CTAs per chain (1..8)")
    args = ap.parse_args()

    from . import build, synthetic as syn
    build.build()
    from . import _lib as L
    from . import api as F
    chains = syn.config3_chains()
    sel = [(i, c) for i, c in enumerate(chains) if c.fw_seed == args.framework]
    sel = sel[args.first:args.first + args.chains]
    d = os.path.join(tempfile.mkdtemp(), "fw")
    syn.write_inputs(d, sel[0][1])
    sysm = F.System.load(d)
    specs = [{"system": 0, "pressure_pa": c.pressure_bar * 1e5, "seed": 1000 + i,
              "create_molecules": c.create_molecules} for i, c in sel]
    prec = L.FMC_PREC_FP64 if args.fp64 else L.FMC_PREC_FP32
    b = F.Batch([sysm], specs, precision=prec, guest_capacity=1024)
    b.set_cluster([args.cluster])
    for it in range(args.launches):
        st = b.run(args.moves)
        ms, ev, mv = b.last_timing()
        print(f"launch {it}: {ms:.3f} ms, {mv} moves, {ev} full evaluations, "
              f"N = {[s.nummols for s in st]}", flush=True)


if __name__ == "__main__":
    main()
