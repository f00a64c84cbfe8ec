"""Regenerate the golden fixtures from the reference tree.

Run in a checkout where the reference is available:

    python tests/golden/make_golden.py /path/to/FastMC

It copies the reference's own CALF-20 test inputs (test/CONFIG and
test/FIELD) into tests/golden/calf20/, writes a CONTROL with the test's
cutoff and Ewald precision (test/T293.0P0.002P0.008/CONTROL without its
jump, swap and switch move lines, so that device-resident chains, which
refuse swap moves, can run it), keeps the test's CONTROL with all six
moves as CONTROL_all_moves, copies the ten isotherm CONTROL files
(test/T293.0P*/CONTROL) under calf20/isotherm/, and records in golden.json
the known answers of run_test.py: the initial "Electrostatic energy"
(reference_energy) and the average CO2 and N2 uptakes per total pressure
(reference_dict) with the test's acceptance band.
"""
from __future__ import annotations

import json
import os
import re
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref: str) -> None:
    out = os.path.join(HERE, "calf20")
    os.makedirs(out, exist_ok=True)
    for f in ("CONFIG", "FIELD"):
        shutil.copyfile(os.path.join(ref, "test", f), os.path.join(out, f))
    ctl_src = os.path.join(ref, "test", "T293.0P0.002P0.008", "CONTROL")
    keep = []
    with open(ctl_src) as f:
        for line in f:
            low = line.strip().lower()
            if low.startswith("move") and any(k in low for k in ("swap", "switch", "jump")):
                continue
            keep.append(line)
    with open(os.path.join(out, "CONTROL"), "w") as f:
        f.writelines(keep)
    shutil.copyfile(ctl_src, os.path.join(out, "CONTROL_all_moves"))
    with open(os.path.join(ref, "run_test.py")) as f:
        src = f.read()
    m = re.search(r"reference_energy\s*=\s*([-0-9.eE+]+)", src)
    if not m:
        raise SystemExit("reference_energy not found in run_test.py")
    iso = {}
    body = re.search(r"reference_dict\s*=\s*\{(.*?)\}", src, re.S)
    if not body:
        raise SystemExit("reference_dict not found in run_test.py")
    for key, co2, n2 in re.findall(r"([0-9.]+)\s*:\s*\[\s*([0-9.]+)\s*,\s*([0-9.]+)\s*\]", body.group(1)):
        iso[key] = [float(co2), float(n2)]
    iso_dir = os.path.join(out, "isotherm")
    for d in sorted(os.listdir(os.path.join(ref, "test"))):
        src_ctl = os.path.join(ref, "test", d, "CONTROL")
        if d.startswith("T") and os.path.isfile(src_ctl):
            os.makedirs(os.path.join(iso_dir, d), exist_ok=True)
            shutil.copyfile(src_ctl, os.path.join(iso_dir, d, "CONTROL"))
    golden = {
        "calf20_electrostatic_energy_kcal": float(m.group(1)),
        "source": "run_test.py reference_energy; gcmc.f prints ecoul/engunit with f22.6",
        "tolerance_abs": 5e-7,
        "isotherm_avg_guests": iso,
        "isotherm_source": ("run_test.py reference_dict: total pressure (bar, the sum of the "
                            "CONTROL pressures) -> average CO2 and N2 guests; a run passes when "
                            "each lies in [0.8 (avg - se), 1.2 (avg + se)]"),
    }
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(golden, f, indent=1)
    print("wrote", out, golden)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path to the reference checkout>")
    main(sys.argv[1])
