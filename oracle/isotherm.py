"""The oracle against the reference's own isotherm statistics.

TEST INFRASTRUCTURE ONLY.  run_test.py of the reference validates a build
by running the ten CALF-20 CO2/N2 inputs of its test directory (copied to
tests/golden/calf20/isotherm/ by tests/golden/make_golden.py) for their own
750000 equilibration and 500000 production moves, with every move of the
CONTROL files (insert, delete, displace, swap, switch, jump), and accepts a
point when the published average uptakes (reference_dict, kept in
tests/golden/golden.json) lie within [0.8 (avg - se), 1.2 (avg + se)] of the
run's averages, se being the "standard error" the reference prints (the
weighted standard deviation of the window averages).  This script runs the
oracle on the same inputs the same way (one process per point, spawn pool)
and applies that band; it also reports the band with se = 0:

    python oracle/isotherm.py [--seed S] [--workers W] [--out results.json]

With --device the ten points run instead as ten device-resident chains of
the CUDA library in one batch, from the same CONTROL files with all six
moves (FP64: the CALF-20 cell is a parallelepiped, which the FP32 path
refuses), and their CO2 and N2 averages and standard errors (from the
chains' window statistics) are checked the same way.

    python oracle/isotherm.py --device [--seed S] [--moves N] [--out results.json]
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import shutil
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLD = os.path.join(ROOT, "tests", "golden")


def control_numbers(ctl: str):
    """(total pressure in bar as run_test.py sums it, steps, equilibration)."""
    p, steps, eq = 0.0, 0, 0
    with open(ctl) as f:
        for line in f:
            w = line.split()
            if "pressure" in line:
                p += float(w[2])
            elif w and w[0] == "steps":
                steps = int(w[1])
            elif w and w[0] == "equilibration":
                eq = int(w[1])
    return p, steps, eq


def run_point(job):
    name, seed = job
    sys.path.insert(0, ROOT)
    from oracle.binding import Oracle
    ctl = os.path.join(GOLD, "calf20", "isotherm", name, "CONTROL")
    p, steps, eq = control_numbers(ctl)
    with tempfile.TemporaryDirectory() as d:
        for f in ("CONFIG", "FIELD"):
            shutil.copy(os.path.join(GOLD, "calf20", f), d)
        shutil.copy(ctl, d)
        o = Oracle(d)
        o.seed(seed)
        t0 = time.time()
        o.run(eq + steps)
        s1, s2 = o.stats(1), o.stats(2)
        return {"point": name, "pressure_bar": p, "moves": eq + steps,
                "avg_co2": s1[0], "avg_n2": s2[0], "se_co2": s1[29], "se_n2": s2[29],
                "production_moves": int(s1[8]),
                "windows": int(s1[9]), "seconds": time.time() - t0}


def run_device(seed: int, moves: int):
    sys.path.insert(0, ROOT)
    import fastmc_gb300 as F
    names = sorted(os.listdir(os.path.join(GOLD, "calf20", "isotherm")))
    rows, systems, tmp = [], [], tempfile.mkdtemp()
    for i, name in enumerate(names):
        ctl = os.path.join(GOLD, "calf20", "isotherm", name, "CONTROL")
        p, steps, eq = control_numbers(ctl)
        d = os.path.join(tmp, name)
        os.makedirs(d)
        for f in ("CONFIG", "FIELD"):
            shutil.copy(os.path.join(GOLD, "calf20", f), d)
        shutil.copy(ctl, os.path.join(d, "CONTROL"))
        systems.append(F.System.load(d))
        rows.append({"point": name, "pressure_bar": p, "moves": moves or eq + steps})
    b = F.Batch(systems, [{"system": i, "seed": seed + i} for i in range(len(names))],
                precision=F.FMC_PREC_FP64, guest_capacity=256)
    total = rows[0]["moves"]
    t0 = time.time()
    done = 0
    while done < total:
        n = min(50000, total - done)
        b.run(n)
        done += n
    st = b.stats()
    for i, r in enumerate(rows):
        r.update({"avg_co2": st[i].guest_avg_n[0], "avg_n2": st[i].guest_avg_n[1],
                  "se_co2": st[i].guest_se_n[0], "se_n2": st[i].guest_se_n[1],
                  "production_moves": int(st[i].prodcount), "windows": int(st[i].windows),
                  "status": int(st[i].status), "seconds": time.time() - t0})
    shutil.rmtree(tmp, ignore_errors=True)
    return rows


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--device", action="store_true")
    ap.add_argument("--moves", type=int, default=0)
    ap.add_argument("--seed", type=int, default=12345)
    ap.add_argument("--workers", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--out", default=None)
    a = ap.parse_args()
    with open(os.path.join(GOLD, "golden.json")) as f:
        ref = {float(k): v for k, v in json.load(f)["isotherm_avg_guests"].items()}
    if a.device:
        rows = run_device(a.seed, a.moves)
    else:
        names = sorted(os.listdir(os.path.join(GOLD, "calf20", "isotherm")))
        with mp.get_context("spawn").Pool(min(a.workers, len(names))) as pool:
            rows = pool.map(run_point, [(n, a.seed) for n in names])
    ok_all = True
    for r in rows:
        key = min(ref, key=lambda k: abs(k - r["pressure_bar"]))
        co2, n2 = ref[key]
        r["reference_co2"], r["reference_n2"] = co2, n2
        def band(avg, se, v):
            return 0.8 * (avg - se) <= v <= 1.2 * (avg + se)
        r["pass"] = bool(band(r["avg_co2"], r["se_co2"], co2) and band(r["avg_n2"], r["se_n2"], n2))
        r["pass_se0"] = bool(band(r["avg_co2"], 0.0, co2) and band(r["avg_n2"], 0.0, n2))
        if a.device:
            r["pass"] = r["pass"] and r["status"] == 0
        ok_all &= r["pass"]
        print("P %.6f bar  CO2 %7.3f +- %6.3f (ref %6.2f)  N2 %6.3f +- %5.3f (ref %5.3f)  %s%s"
              % (r["pressure_bar"], r["avg_co2"], r["se_co2"], co2, r["avg_n2"], r["se_n2"], n2,
                 "PASS" if r["pass"] else "FAIL", "" if r["pass_se0"] else " (outside with se = 0)"))
    if a.out:
        with open(a.out, "w") as f:
            json.dump({"seed": a.seed, "device": a.device, "rows": rows, "all_pass": ok_all}, f, indent=1)
    sys.exit(0 if ok_all else 1)


if __name__ == "__main__":
    main()
