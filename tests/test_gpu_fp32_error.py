"""FP32 path against the FP64 oracle, move by move on identical states.

The per-move ABI of an FP32 engine evaluates trial insertions, deletions
and displacements of a state copied from the oracle; the error of estep
against the oracle's FP64 value is the FP32 path's ΔE error.  Tolerances:
insertion and deletion ≤ 1e-6 of |ΔE|; a displacement's ΔE is the
difference of two energies of the same molecule, so its error is bounded by
1e-6 of the larger of |ΔE| and the molecule's energy before the move.
"""
import math

import numpy as np
import pytest

from fastmc_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

REL = 1e-6


def _state(oracle_lib, fmc_lib, d, ncreate, seed):
    o = oracle_lib.Oracle(d)
    o.seed(seed)
    if ncreate:
        o.create_molecules(1, ncreate)
    xyz = o.coords(o.locguest(1)).reshape(-1, 3, 3)
    sysm = fmc_lib.System.load(d)
    engines = {}
    for name, prec in (("fp32", fmc_lib.FMC_PREC_FP32), ("fp64", fmc_lib.FMC_PREC_FP64)):
        p = fmc_lib.PlainEngine(sysm, prec, 1024)
        for m in xyz:
            assert not p.insertion(1, m)["overlap"]
            assert p.commit(0.0)
        engines[name] = p
    return o, engines, len(xyz)


def _errors(o, eng, n, box, ntrial, seed):
    rng = np.random.default_rng(seed)
    out = {"insert": [], "delete": [], "displace": []}
    mism = 0
    for _ in range(100000):
        if len(out["insert"]) >= ntrial:
            break
        ax = rng.normal(size=3)
        ax /= np.linalg.norm(ax)
        xyz = np.outer([0.0, 1.16, -1.16], ax) + rng.uniform(0, box, 3)
        ref = o.insertion_energy(1, xyz)
        got = eng["fp32"].insertion(1, xyz)
        if got["overlap"] != ref["overlap"]:
            mism += 1
            continue
        if not ref["overlap"]:
            out["insert"].append((got["estep"], ref["estep"], abs(ref["estep"])))
    for c in rng.integers(1, n + 1, size=min(ntrial, n)):
        ref = o.deletion_energy(1, int(c))
        got = eng["fp32"].deletion(1, int(c))
        out["delete"].append((got["estep"], ref["estep"], abs(ref["estep"])))
    tries = 0
    while len(out["displace"]) < ntrial and tries < 20 * ntrial:
        tries += 1
        c = int(rng.integers(1, n + 1))
        a, b, cc = rng.uniform(-0.25, 0.25, 3)
        th = rng.uniform(0.0, 0.5)
        ax = rng.normal(size=3)
        ax /= np.linalg.norm(ax)
        abcq = [a, b, cc, math.cos(th / 2), *(math.sin(th / 2) * ax)]
        ref = o.displace_energy(1, c, abcq)
        got = eng["fp32"].displace(1, c, abcq)
        if got["overlap"] != ref["overlap"]:
            mism += 1
            continue
        if ref["overlap"]:
            continue
        e_old = eng["fp64"].guest_energy(1, c)["estep"]
        out["displace"].append((got["estep"], ref["estep"], max(abs(ref["estep"]), abs(e_old))))
    return out, mism


@pytest.mark.parametrize("case", ["25A", "51A_100"])
def test_fp32_delta_e_error(fmc_lib, oracle_lib, inputs_dir, case):
    if case == "25A":
        spec, ncreate, box = syn.single_chain_25A(), 20, 25.6
    else:
        spec, ncreate, box = syn.single_chain_51A(), 100, 51.2
    d = inputs_dir(spec, "fp32err_" + case)
    o, eng, n = _state(oracle_lib, fmc_lib, d, ncreate, seed=5)
    assert n == ncreate
    res, mism = _errors(o, eng, n, box, ntrial=60, seed=1)
    assert mism == 0
    for kind, rows in res.items():
        assert len(rows) >= 20, (kind, len(rows))
        v = np.array(rows)
        err = np.abs(v[:, 0] - v[:, 1])
        rel_de = err / np.abs(v[:, 1])
        rel = err / v[:, 2]
        print(f"{case} {kind}: n={len(v)} max|err|={err.max():.3g} kcal/mol "
              f"max rel |dE|={rel_de.max():.3g} max rel scale={rel.max():.3g}")
        assert rel.max() <= REL, (kind, rel.max())
