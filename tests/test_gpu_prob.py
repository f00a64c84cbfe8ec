"""Probability grids (storeprob, utility_pack.f:621-687) accumulated on the
device after every production move, against the oracle's grids for the
same chain."""
import os

import numpy as np
import pytest

from fastmc_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def _prob_dir(inputs_dir):
    spec = syn.small_test_spec(seed=4, kmax=6, pressure_bar=5.0, create=20,
                               move_mix=(("insert", 0.1), ("displace", 0.3), ("jump", 0.6)))
    spec.overlap = 1.0
    spec.probability = [[0], [1, 2, 3]]
    spec.grid_spacing = 0.8
    spec.grid_factor = (2, 2, 2)
    return inputs_dir(spec, "gpu_prob")


def _oracle_grids(oracle_lib, d, n):
    o = oracle_lib.Oracle(d)
    o.seed(9)
    o.create_molecules(1, 20)
    logs = o.run(n)
    return logs, np.stack([o.prob_grid(k + 1) for k in range(o.prob_info()[3])])


@pytest.mark.parametrize("csize", [1, 2])
def test_prob_grid_fp64_matches_oracle(fmc_lib, oracle_lib, inputs_dir, csize):
    d = _prob_dir(inputs_dir)
    n = 300
    _, ref = _oracle_grids(oracle_lib, d, n)
    b = fmc_lib.Batch([fmc_lib.System.load(d)], [{"seed": 9}], precision=fmc_lib.FMC_PREC_FP64,
                      guest_capacity=64)
    b.set_cluster([csize])
    b.run(n)
    assert b.prob_info(0) == ((16, 16, 16), 2)
    got = b.prob_grid(0)
    assert got.shape == ref.shape
    # atomics add in another order: equal to rounding
    assert np.allclose(got, ref, rtol=1e-10, atol=1e-10)
    assert np.isclose(got[0].sum(), ref[0].sum(), rtol=1e-12)


def test_prob_grid_fp32_matches_oracle(fmc_lib, oracle_lib, inputs_dir):
    """An FP32 chain whose decisions match the oracle's over the run bins
    the same points (positions agree to ~1e-13 A after the double-float
    geometry)."""
    d = _prob_dir(inputs_dir)
    n = 120
    logs, ref = _oracle_grids(oracle_lib, d, n)
    b = fmc_lib.Batch([fmc_lib.System.load(d)], [{"seed": 9}], precision=fmc_lib.FMC_PREC_FP32,
                      guest_capacity=64)
    b.set_log(n)
    b.run(n)
    got_logs = b.log(0, n)
    assert [(g.move, g.choice, g.accepted) for g in got_logs] == \
           [(r.move, r.choice, r.accepted) for r in logs]
    got = b.prob_grid(0)
    assert np.allclose(got, ref, rtol=1e-7, atol=1e-7)


def test_prob_grid_untouched_by_autotune_and_checkpoint(fmc_lib, inputs_dir, tmp_path):
    """The autotuner's trial cycles leave the grids as they were, and a
    checkpoint carries them."""
    d = _prob_dir(inputs_dir)
    sysm = fmc_lib.System.load(d)
    a = fmc_lib.Batch([sysm], [{"seed": 9}, {"seed": 10}], precision=fmc_lib.FMC_PREC_FP32,
                      guest_capacity=64)
    a.run(50)
    before = [a.prob_grid(c) for c in range(2)]
    a.autotune(32)
    for c in range(2):
        assert np.array_equal(a.prob_grid(c), before[c])
    path = str(tmp_path / "p.ckpt")
    a.save(path)
    b = fmc_lib.Batch([sysm], [{"seed": 9}, {"seed": 10}], precision=fmc_lib.FMC_PREC_FP32,
                      guest_capacity=64)
    b.load(path)
    for c in range(2):
        assert np.array_equal(b.prob_grid(c), before[c])


def _energy_dir(tmp_path):
    """One guest type with a centre-of-mass grid and the energy grids (an
    'e' line, storeenprob) on an open framework (48 atoms per cell)."""
    spec = syn.small_test_spec(seed=4, kmax=5, pressure_bar=5.0, create=10,
                               move_mix=(("insert", 0.2), ("delete", 0.2), ("displace", 0.6)))
    spec.overlap = 1.5
    spec.probability = [[0], "energy"]
    spec.grid_spacing = 0.8
    d = str(tmp_path / "egrid")
    syn.write_inputs(d, spec, uc=syn.make_unit_cell(4, natoms=48))
    # the guest's sites moved off its centre (the reference's set-up leaves
    # half of that offset in the template): test insertions at grid points
    # then have their centres off the cell's faces, where the binning wraps
    # and the last bit of the centre picks the bins
    path = os.path.join(d, "FIELD")
    lines = open(path).read().split("\n")
    i0 = next(i for i, l in enumerate(lines) if l.startswith("&guest CO2"))
    for i in range(i0 + 3, i0 + 6):
        w = lines[i].split()
        x, y, z = float(w[3]) + 0.4, float(w[4]) + 0.3, float(w[5]) + 0.2
        lines[i] = f"{w[0]:<8s}{float(w[1]):14.6f}{float(w[2]):14.6f}{x:14.6f}{y:14.6f}{z:14.6f}"
    open(path, "w").write("\n".join(lines))
    return d


@pytest.mark.parametrize("prec,csize,n", [("fp64", 1, 400), ("fp64", 2, 400), ("fp32", 1, 200)])
def test_energy_grids_follow_oracle(fmc_lib, oracle_lib, tmp_path, prec, csize, n):
    """The energy grids as the main loop fills them (storeenprob with the
    main program's guest_toten, 0, and molecule 0: a count at the centre of
    the accepted move's last positions, nothing in the energy grid) next to
    the centre-of-mass grid, against the oracle's three grids; FP32 over a
    run whose decisions are the oracle's."""
    d = _energy_dir(tmp_path)
    o = oracle_lib.Oracle(d)
    o.seed(3)
    o.create_molecules(1, 10)
    logs = o.run(n)
    ref = np.stack([o.prob_grid(k + 1) for k in range(3)])
    p = fmc_lib.FMC_PREC_FP64 if prec == "fp64" else fmc_lib.FMC_PREC_FP32
    b = fmc_lib.Batch([fmc_lib.System.load(d)], [{"seed": 3}], precision=p, guest_capacity=64)
    b.set_cluster([csize])
    b.set_log(n)
    b.run(n)
    got_logs = b.log(0, n)
    assert [(g.move, g.choice, g.accepted) for g in got_logs] == \
           [(r.move, r.choice, r.accepted) for r in logs]
    assert b.prob_info(0)[1] == 3
    got = b.prob_grid(0)
    assert sum(r.accepted for r in logs) >= n // 10
    assert np.all(got[1] == 0.0) and got[2].sum() > 0
    tol = 1e-10 if prec == "fp64" else 1e-7
    assert np.allclose(got, ref, rtol=tol, atol=tol)


def test_widom_energy_grid(fmc_lib, oracle_lib, tmp_path):
    """widom_grid's test insertions fill the energy grids with their energies
    and counts (gcmc.f:2529-2532): the device grids gain what the oracle's
    storeenprob bins for the same trials (positions and energies the device
    reports); the centre-of-mass grid is left alone.  No centre sits exactly on
    a bin edge (the guest's centre is off its rotation origin, and the grid
    has 7 points a side against 16 bins a cell): there the reference's
    equitable binning moves by a whole bin with the last bit of the centre,
    which the device's fused multiply-adds and the host's rounding set
    differently."""
    d = _energy_dir(tmp_path)
    b = fmc_lib.Batch([fmc_lib.System.load(d)], [{"seed": 3}], precision=fmc_lib.FMC_PREC_FP64,
                      guest_capacity=64)
    before = b.prob_grid(0)
    (henry, nok, ntot), est, ovl, xyz = b.widom_grid(0, (7, 7, 7), 2, seed=7, details=True)
    after = b.prob_grid(0)
    assert nok >= 50
    o = oracle_lib.Oracle(d)
    for t in np.flatnonzero(ovl == 0):
        o.store_energy(1, xyz[t], est[t])
    ref = np.stack([o.prob_grid(k + 1) for k in range(3)])
    diff = after - before
    assert np.all(diff[0] == 0.0)
    assert np.allclose(diff[1:], ref[1:], rtol=1e-10, atol=1e-10 * np.abs(ref[1]).max())
    assert np.isclose(diff[2].sum(), nok, rtol=1e-12)
