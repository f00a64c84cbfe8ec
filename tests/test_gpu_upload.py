"""fmc_upload_system (the host's start-up arrays) against fmc_system_load
(the input files): the same device state and the same results, bit for
bit, on the per-move path and in device-resident chains, for an
orthorhombic synthetic framework and the reference's CALF-20 test system
(parallelepiped cell)."""
import numpy as np
import pytest

from conftest import CALF20
from fastmc_gb300 import synthetic as syn
from test_host_setup import host_arrays

pytestmark = pytest.mark.gpu


def _pair(fmc_lib, oracle_lib, d):
    return fmc_lib.System.load(d), fmc_lib.System.upload(host_arrays(oracle_lib, d))


def test_upload_per_move_bitwise(fmc_lib, oracle_lib, inputs_dir):
    d = inputs_dir(syn.small_test_spec(seed=4, kmax=6, pressure_bar=5.0), "upload_pm")
    a, b = _pair(fmc_lib, oracle_lib, d)
    pa, pb = (fmc_lib.PlainEngine(s, fmc_lib.FMC_PREC_FP64, 64) for s in (a, b))
    rng = np.random.default_rng(4)
    n = 0
    for _ in range(4000):
        ax = rng.normal(size=3)
        ax /= np.linalg.norm(ax)
        xyz = np.outer([0.0, 1.16, -1.16], ax) + rng.uniform(0, 25.6, 3)
        ra, rb = pa.insertion(1, xyz), pb.insertion(1, xyz)
        assert ra["overlap"] == rb["overlap"]
        assert ra["estep"] == rb["estep"] and np.array_equal(ra["delE"], rb["delE"])
        assert pa.commit(0.0) == pb.commit(0.0)
        n = pa.nummols(1)
        if n == 8:
            break
    assert n == 8 and pb.nummols(1) == 8
    for c in range(1, 9):
        assert pa.deletion(1, c)["estep"] == pb.deletion(1, c)["estep"]
    assert np.array_equal(pa.sk(), pb.sk())
    assert np.array_equal(pa.full_ewald(), pb.full_ewald())


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_upload_chains_bitwise(fmc_lib, oracle_lib, inputs_dir, prec):
    d = inputs_dir(syn.small_test_spec(seed=5, kmax=8, ntile=3, pressure_bar=5.0, create=30), "upload_ch")
    a, b = _pair(fmc_lib, oracle_lib, d)
    p = fmc_lib.FMC_PREC_FP32 if prec == "fp32" else fmc_lib.FMC_PREC_FP64
    logs = []
    for s in (a, b):
        bt = fmc_lib.Batch([s], [{"seed": 3}, {"seed": 4}], precision=p, guest_capacity=128)
        bt.set_log(300)
        bt.run(300)
        logs.append([[(r.move, r.choice, r.overlap, r.accepted, r.estep) for r in bt.log(c, 300)]
                     for c in range(2)])
    assert logs[0] == logs[1]


def test_upload_calf20_known_answer(fmc_lib, oracle_lib):
    """The reference's own test system through the uploaded arrays: the
    electrostatic energy it prints, and the same per-move energies as the
    file-loaded system on its parallelepiped cell."""
    import json
    import os
    from conftest import GOLDEN
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        g = json.load(f)
    a, b = _pair(fmc_lib, oracle_lib, CALF20)
    pa, pb = (fmc_lib.PlainEngine(s, fmc_lib.FMC_PREC_FP64, 16) for s in (a, b))
    ea, eb = pa.full_ewald(), pb.full_ewald()
    assert abs(eb[0] - g["calf20_electrostatic_energy_kcal"]) < g["tolerance_abs"]
    assert np.array_equal(ea, eb)
    cell = np.array(a.info().cell).reshape(3, 3)
    rng = np.random.default_rng(6)
    tmpl = np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 1.16], [0.0, 0.0, -1.16]])
    for _ in range(200):
        xyz = tmpl + rng.uniform(0, 1, 3) @ cell
        ra, rb = pa.insertion(1, xyz), pb.insertion(1, xyz)
        assert ra["overlap"] == rb["overlap"] and ra["estep"] == rb["estep"]
