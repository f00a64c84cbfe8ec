"""Regenerate the golden fixtures from the reference tree.

Run in a checkout where the reference is available:

    python tests/golden/make_golden.py /path/to/FastMC

It copies the reference's own CALF-20 test inputs (test/CONFIG and
test/FIELD) into tests/golden/calf20/, writes a CONTROL with the test's
cutoff and Ewald precision (test/T293.0P0.002P0.008/CONTROL without its
jump, swap and switch move lines, so that device-resident chains, which
refuse swap moves, can run it), keeps the test's CONTROL with all six
moves as CONTROL_all_moves, and records the known answer printed by the
reference, the initial "Electrostatic energy" of run_test.py
(reference_energy), in golden.json.
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
    golden = {
        "calf20_electrostatic_energy_kcal": float(m.group(1)),
        "source": "run_test.py reference_energy; gcmc.f prints ecoul/engunit with f22.6",
        "tolerance_abs": 5e-7,
    }
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(golden, f, indent=1)
    print("wrote", out, golden)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
