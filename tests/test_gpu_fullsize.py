"""Parity at the full sizes of the larger configurations, on states loaded
on the device and replayed into the oracle:

- the 51.2 A framework (12288 atoms, kmax 12) with 400 CO2: insertion,
  deletion and displacement energies through the per-move ABI, FP64 to
  1e-9 and FP32 to 1e-6 of the oracle;
- the 102.4 A framework (98304 atoms, cutoff 14 A, kmax 20) with 2000 CO2:
  Widom test insertions (widom_grid's energy, gcmc.f:2454-2548) at random
  positions, FP32 to 1e-6 of the oracle.
"""
import math

import numpy as np
import pytest

from fastmc_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

TMPL = np.array([0.0, 1.16, -1.16])


def _loaded(fmc_lib, d, n, seed=5):
    """A device batch whose chain created n molecules; their coordinates."""
    b = fmc_lib.Batch([fmc_lib.System.load(d)], [{"seed": seed, "create_molecules": n}],
                      precision=fmc_lib.FMC_PREC_FP32, guest_capacity=max(64, n + 16))
    x, m = b.coords(0)
    assert m == n
    return b, x[:9 * n].reshape(n, 3, 3)


def _random_molecule(rng, box):
    ax = rng.normal(size=3)
    ax /= np.linalg.norm(ax)
    return np.outer(TMPL, ax) + rng.uniform(0, box, 3)


def test_51A_full_size_per_move(fmc_lib, oracle_lib, inputs_dir):
    d = inputs_dir(syn.single_chain_51A(), "full_51A")
    _, xyz = _loaded(fmc_lib, d, 400)
    o = oracle_lib.Oracle(d)
    sysm = fmc_lib.System.load(d)
    eng = {p: fmc_lib.PlainEngine(sysm, p, 512) for p in (fmc_lib.FMC_PREC_FP64, fmc_lib.FMC_PREC_FP32)}
    for m in xyz:
        o.apply_move(1, 1, 0, m, True)
        for p in eng.values():
            assert not p.insertion(1, m)["overlap"]
            assert p.commit(0.0)
    tol = {fmc_lib.FMC_PREC_FP64: 1e-9, fmc_lib.FMC_PREC_FP32: 1e-6}
    rng = np.random.default_rng(11)
    nins = 0
    for _ in range(3000):
        if nins >= 10:
            break
        m = _random_molecule(rng, 51.2)
        ref = o.insertion_energy(1, m)
        for prec, p in eng.items():
            got = p.insertion(1, m)
            assert got["overlap"] == ref["overlap"]
            if not ref["overlap"]:
                assert abs(got["estep"] - ref["estep"]) <= tol[prec] * max(abs(ref["estep"]), 1.0)
        nins += not ref["overlap"]
    assert nins >= 5
    for c in rng.integers(1, 401, size=10):
        ref = o.deletion_energy(1, int(c))
        for prec, p in eng.items():
            got = p.deletion(1, int(c))
            assert abs(got["estep"] - ref["estep"]) <= tol[prec] * max(abs(ref["estep"]), 1.0)
    ndis = 0
    for _ in range(200):
        if ndis >= 10:
            break
        c = int(rng.integers(1, 401))
        th = rng.uniform(0.0, 0.5)
        ax = rng.normal(size=3)
        ax /= np.linalg.norm(ax)
        abcq = [*rng.uniform(-0.25, 0.25, 3), math.cos(th / 2), *(math.sin(th / 2) * ax)]
        ref = o.displace_energy(1, c, abcq)
        if ref["overlap"]:
            continue
        e_old = abs(o.deletion_energy(1, c)["estep"])
        for prec, p in eng.items():
            got = p.displace(1, c, abcq)
            assert not got["overlap"]
            assert abs(got["estep"] - ref["estep"]) <= tol[prec] * max(abs(ref["estep"]), e_old, 1.0)
        ndis += 1
    assert ndis >= 5


def test_102A_full_size_widom(fmc_lib, oracle_lib, inputs_dir):
    d = inputs_dir(syn.widom_102A(), "full_102A")
    b, xyz = _loaded(fmc_lib, d, 2000)
    o = oracle_lib.Oracle(d)
    for m in xyz:
        o.apply_move(1, 1, 0, m, True)
    rng = np.random.default_rng(13)
    pos = np.array([_random_molecule(rng, 102.4) for _ in range(20000)])
    est, ovl = b.widom_positions(0, pos)
    free = np.flatnonzero(ovl == 0)[:12]
    hit = np.flatnonzero(ovl != 0)[:20]
    assert len(free) >= 3
    for i in np.concatenate([free, hit]):
        ref = o.insertion_energy(1, pos[i])
        assert bool(ovl[i]) == bool(ref["overlap"]), i
        if not ref["overlap"]:
            assert abs(est[i] - ref["estep"]) <= 1e-6 * max(abs(ref["estep"]), 1.0), (i, est[i], ref["estep"])
