"""Probability grids (storeprob, utility_pack.f:621-687) accumulated on the
device after every production move, against the oracle's grids for the
same chain."""
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
