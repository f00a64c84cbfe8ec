"""Device state handling of batches: snapshots that replay a state exactly,
paused chains, checkpoints that are checked before they are loaded, and
the running structure factor of long FP32 chains against a fresh FP64
recomputation (drift).
"""
import json
import os
import struct

import numpy as np
import pytest

from fastmc_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small(inputs_dir):
    return inputs_dir(syn.small_test_spec(seed=5, kmax=8, ntile=3, pressure_bar=5.0, create=40), "st_small")


def _logs(b, n):
    return [[(r.move, r.choice, r.overlap, r.accepted, r.estep) for r in b.log(c, n)]
            for c in range(b.nchains)]


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_snapshot_replays_exactly(fmc_lib, small, prec):
    p = fmc_lib.FMC_PREC_FP32 if prec == "fp32" else fmc_lib.FMC_PREC_FP64
    b = fmc_lib.Batch([fmc_lib.System.load(small)], [{"seed": 3}, {"seed": 4}], precision=p,
                      guest_capacity=256)
    b.set_cluster([2])
    b.run(50)
    b.snapshot()
    s0 = b.stats()
    b.set_log(200)
    b.run(200)
    a = _logs(b, 200)
    sa = b.stats()
    for _ in range(2):
        b.restore()
        assert [s.moves for s in b.stats()] == [s.moves for s in s0]
        b.set_log(200)
        b.run(200)
        assert _logs(b, 200) == a
        sb = b.stats()
        assert [(s.nummols, s.energy, s.moves) for s in sb] == [(s.nummols, s.energy, s.moves) for s in sa]


def test_paused_chain_keeps_its_state(fmc_lib, small):
    sysm = fmc_lib.System.load(small)
    b = fmc_lib.Batch([sysm], [{"seed": 7}, {"seed": 8}, {"seed": 9}], guest_capacity=256)
    b.run(20)
    s0 = b.stats()
    x0 = b.coords(1)
    b.set_chain_cluster([1, 0, 2])
    b.run(100)
    s1 = b.stats()
    assert s1[1].moves == s0[1].moves and s1[1].energy == s0[1].energy
    assert np.array_equal(b.coords(1)[0], x0[0])
    assert s1[0].moves == s0[0].moves + 100 and s1[2].moves == s0[2].moves + 100
    # a paused chain that runs again continues as if never paused
    ref = fmc_lib.Batch([sysm], [{"seed": 8}], guest_capacity=256)
    ref.run(20)
    b.set_chain_cluster([1, 1, 1])
    b.run(60)
    ref.run(60)
    assert b.stats()[1].energy == ref.stats()[0].energy
    with pytest.raises(fmc_lib.FmcError):
        b.set_chain_cluster([0, 0, 0])


def _hdr_offsets():
    """Byte offsets in a checkpoint file: magic (8) and six ints, then the
    state records array (a u64 count, then the records)."""
    return 8 + 6 * 4 + 8


def test_checkpoint_load_rejects_corrupt_file(fmc_lib, small, tmp_path):
    """A checkpoint whose counts or order entries are out of range is
    refused (FMC_ERR_INPUT) before anything is uploaded: the batch keeps
    its state."""
    from fastmc_gb300 import _lib as L
    sysm = fmc_lib.System.load(small)
    b = fmc_lib.Batch([sysm], [{"seed": 7}, {"seed": 8}], guest_capacity=256)
    b.run(30)
    path = str(tmp_path / "c.ckpt")
    b.save(path)
    b.run(30)  # move on, so that a successful load would be visible
    before = [(s.moves, s.nummols, s.energy) for s in b.stats()]
    raw = open(path, "rb").read()
    rec = _hdr_offsets()
    # ChainHdr: u[97] c cd cm (100 floats), ir jr, then nummols[4]
    off_nummols = rec + 100 * 4 + 2 * 4
    bad = bytearray(raw)
    bad[off_nummols:off_nummols + 4] = struct.pack("<i", 100000)
    p2 = str(tmp_path / "bad.ckpt")
    open(p2, "wb").write(bytes(bad))
    rc = L.load().fmc_batch_load(b._h, p2.encode())
    assert rc == L.FMC_ERR_INPUT
    assert [(s.moves, s.nummols, s.energy) for s in b.stats()] == before
    # a truncated file is refused the same way
    open(p2, "wb").write(raw[: len(raw) // 2])
    assert L.load().fmc_batch_load(b._h, p2.encode()) == L.FMC_ERR_INPUT
    assert [(s.moves, s.nummols, s.energy) for s in b.stats()] == before
    # the intact file still loads
    b.load(path)
    assert [s.moves for s in b.stats()] != [m for m, _, _ in before]


def _oracle_of(oracle_lib, d, xyz_mols):
    """A fresh oracle holding the given molecules (inserted and committed):
    its S(k) and energy are FP64 functions of the configuration alone."""
    o = oracle_lib.Oracle(d)
    for m in xyz_mols:
        o.apply_move(1, 1, 0, m, True)
    return o


def test_fp32_structure_factor_does_not_drift(fmc_lib, oracle_lib, tmp_path):
    """FP32 chains keep their guests' S(k) as double-float sums of the
    per-molecule terms each move adds and removes.  A molecule's term is
    computed by the same arithmetic whenever its position is evaluated, so
    the running sum stays the sum of the current molecules' terms: after
    about 1e6 accepted moves per chain it differs from a fresh FP64
    recomputation from the coordinates by the FP32 rounding of the terms,
    as it does after 1e4, not by an error that grows with the moves.  The
    running energy (FP64 sums of FP32 move energies) is compared with the
    oracle's energy of the final configuration."""
    # an open framework (24 atoms per 12.8 A cell) so that about half of the
    # displacements and rotations are accepted
    spec = syn.small_test_spec(seed=4, kmax=7, pressure_bar=5.0, create=60,
                               move_mix=(("displace", 0.5), ("rotate", 0.5)))
    d = str(tmp_path / "drift")
    syn.write_inputs(d, spec, uc=syn.make_unit_cell(4, natoms=24))
    sysm = fmc_lib.System.load(d)
    info = sysm.info()
    nch = 8
    b = fmc_lib.Batch([sysm], [{"seed": 100 + c} for c in range(nch)],
                      precision=fmc_lib.FMC_PREC_FP32, guest_capacity=128)
    mol = info.guest_mol[0]
    report = []
    accepted = np.zeros(nch)
    e_err = []
    for nmoves in (20000, 180000, 2000000):
        b.run(nmoves)
        st = b.stats()
        accepted = np.array([sum(s.accepts) for s in st], dtype=float)
        worst = 0.0
        for c in range(nch):
            x, n = b.coords(c)
            mols = x[:9 * n].reshape(n, 3, 3)
            o = _oracle_of(oracle_lib, d, mols)
            ref = o.sk()[:, mol - 1, :]
            got = b.sk(c, info.newld, info.maxmls)[:, mol - 1, :]
            worst = max(worst, np.abs(got - ref).max() / max(1.0, np.abs(ref).max()))
            if c == 0:
                e_err.append(abs(st[0].energy - o.energy(o.locguest(1))))
            o.close()
        report.append({"accepted_per_chain": float(accepted.mean()), "sk_rel_err": worst,
                       "energy_abs_err_chain0": e_err[-1]})
    out = os.environ.get("FMC_DRIFT_REPORT")
    if out:
        with open(out, "w") as f:
            json.dump(report, f, indent=1)
    print("drift", json.dumps(report))
    assert accepted.mean() >= 1e6
    errs = [r["sk_rel_err"] for r in report]
    assert max(errs) < 1e-5
    assert errs[2] < 4.0 * max(errs[0], 1e-9)  # no growth with the number of moves


def test_speculation_changes_nothing(fmc_lib, tmp_path):
    """Speculative rounds (fmc_batch_set_speculation) draw proposals ahead,
    test their overlaps together and undo the draws after the first one
    that passes: the chains' moves, decisions and energies are bit for bit
    those of the sequential loop, on one CTA and on a cluster, with every
    round size."""
    spec = syn.small_test_spec(seed=5, kmax=8, ntile=3, pressure_bar=5.0, create=60)
    d = str(tmp_path / "spec")
    syn.write_inputs(d, spec)
    sysm = fmc_lib.System.load(d)
    b = fmc_lib.Batch([sysm], [{"seed": 3}, {"seed": 4}, {"seed": 5}],
                      precision=fmc_lib.FMC_PREC_FP32, guest_capacity=256)
    b.set_chain_cluster([1, 2, 1])
    b.snapshot()
    runs = []
    for k in (0, 2, 5, 8):
        b.restore()
        b.set_speculation(k)
        b.set_log(400)
        b.run(400)
        runs.append((_logs(b, 400), [(s.nummols, s.energy, s.moves, s.overlap_exits, tuple(s.accepts))
                                     for s in b.stats()]))
    assert sum(r[2] for r in runs[0][0][0]) >= 100  # overlap exits to batch
    for r in runs[1:]:
        assert r == runs[0]
