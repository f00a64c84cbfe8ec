"""Widom test insertions (widom_grid, gcmc.f:2454-2548) on the GPU against
the oracle's insertion energies on the same state."""
import math

import numpy as np
import pytest

from fastmc_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

KBOLTZ = 1.9872041e-3  # kcal/mol/K


@pytest.fixture(scope="module")
def small(inputs_dir):
    return inputs_dir(syn.small_test_spec(seed=4, kmax=6, pressure_bar=5.0, create=10), "wd_small")


def _oracle_with_state(oracle_lib, d, xyz):
    """An oracle holding the given guest coordinates (molecule order)."""
    o = oracle_lib.Oracle(d)
    for m in xyz:
        o.apply_move(1, 1, 0, m, True)
    return o


@pytest.mark.parametrize("precision,rel", [("fp64", 1e-9), ("fp32", 1e-6)])
def test_widom_positions_match_oracle(fmc_lib, oracle_lib, small, precision, rel):
    prec = fmc_lib.FMC_PREC_FP64 if precision == "fp64" else fmc_lib.FMC_PREC_FP32
    sysm = fmc_lib.System.load(small)
    b = fmc_lib.Batch([sysm], [{"seed": 77}], precision=prec, guest_capacity=64)
    b.run(50)
    before = b.stats()[0]
    x, n = b.coords(0)
    state = x[:9 * n].reshape(n, 3, 3)
    o = _oracle_with_state(oracle_lib, small, state)
    rng = np.random.default_rng(9)
    pos = []
    for _ in range(4000):
        ax = rng.normal(size=3)
        ax /= np.linalg.norm(ax)
        pos.append(np.outer([0.0, 1.16, -1.16], ax) + rng.uniform(0, 25.6, 3))
    pos = np.array(pos)
    est, ovl = b.widom_positions(0, pos)
    nfree = 0
    for i, p in enumerate(pos):
        ref = o.insertion_energy(1, p)
        assert bool(ovl[i]) == bool(ref["overlap"]), i
        if ref["overlap"]:
            continue
        nfree += 1
        assert abs(est[i] - ref["estep"]) <= rel * max(abs(ref["estep"]), 1.0), (i, est[i], ref["estep"])
    assert nfree >= 5
    after = b.stats()[0]
    assert (after.nummols, after.energy, after.moves) == (before.nummols, before.energy, before.moves)


def test_widom_grid_henry(fmc_lib, oracle_lib, small):
    """A 4x4x4 grid x 3 orientations: the positions the GPU used, fed to the
    oracle, give the same energies and the same Henry average."""
    sysm = fmc_lib.System.load(small)
    b = fmc_lib.Batch([sysm], [{"seed": 5}], precision=fmc_lib.FMC_PREC_FP32, guest_capacity=64)
    b.run(20)
    x, n = b.coords(0)
    o = _oracle_with_state(oracle_lib, small, x[:9 * n].reshape(n, 3, 3))
    (henry, nok, ntot), est, ovl, xyz = b.widom_grid(0, (4, 4, 4), 3, seed=123, details=True)
    assert ntot == 4 * 4 * 4 * 3
    temp = sysm.info().temperature
    hsum = 0.0
    for t in range(ntot):
        ref = o.insertion_energy(1, xyz[t])
        assert bool(ovl[t]) == bool(ref["overlap"]), t
        if not ref["overlap"]:
            assert abs(est[t] - ref["estep"]) <= 1e-6 * max(abs(ref["estep"]), 1.0)
            hsum += math.exp(-ref["estep"] / KBOLTZ / temp)
    assert nok == int(np.sum(ovl == 0))
    assert abs(henry - hsum / ntot) <= 1e-5 * max(abs(hsum / ntot), 1e-300)
    # grid points: molecule centres at the grid fractions (1-based)
    L = 25.6
    cen = xyz.mean(axis=1)
    frac = np.round(cen / L * 4) / 4
    assert np.allclose(cen, frac * L, atol=0.2)
    # same seed, same result
    again = b.widom_grid(0, (4, 4, 4), 3, seed=123)
    assert again == (henry, nok, ntot)
