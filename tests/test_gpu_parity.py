"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

FP64 mode must match the oracle to 1e-9 relative per move (and bit-exact
decisions); the reference's own known answer (CALF-20 electrostatic
energy) must come out of the GPU structure-factor kernel.
"""
import json
import math
import os

import numpy as np
import pytest

from conftest import CALF20, GOLDEN
from fastmc_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

REL = 1e-9   # FP64 parity tolerance per energy term


def close(a, b, rel=REL, scale=1.0):
    return abs(a - b) <= rel * max(abs(a), abs(b), scale)


def golden():
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        return json.load(f)


def test_gpu_calf20_kat(fmc_lib, oracle_lib):
    """K4 structure factor on the GPU reproduces the reference's printed
    electrostatic energy of its own test system."""
    sysm = fmc_lib.System.load(CALF20)
    plain = fmc_lib.PlainEngine(sysm, fmc_lib.FMC_PREC_FP64, 16)
    out = plain.full_ewald()
    g = golden()
    assert abs(out[0] - g["calf20_electrostatic_energy_kcal"]) < g["tolerance_abs"], out
    # framework S(k) against the oracle's ckcsum/ckssum
    o = oracle_lib.Oracle(CALF20)
    so, sg = o.sk(), plain.sk()
    tot = sysm.info().maxmls
    assert np.allclose(sg[:, tot, :], so[:, tot, :], rtol=1e-10, atol=1e-10 * np.abs(so).max())


@pytest.fixture(scope="module")
def small(inputs_dir):
    return inputs_dir(syn.small_test_spec(seed=4, kmax=6, pressure_bar=5.0, create=10), "gpu_small")


def _free_positions(o, n, seed, box=25.6):
    rng = np.random.default_rng(seed)
    tmpl = np.array([[0, 0, 0], [0, 0, 1.16], [0, 0, -1.16]])
    out = []
    for _ in range(200000):
        ax = rng.normal(size=3)
        ax /= np.linalg.norm(ax)
        xyz = np.outer([0, 1.16, -1.16], ax) + rng.uniform(0, box, 3)
        if not o.insertion_energy(1, xyz)["overlap"]:
            out.append(xyz)
            if len(out) == n:
                break
    return out


def _cmp(res, ref, maxmls, keys=("estep", "ewld1", "ewld2", "vdw", "delrc")):
    assert res["overlap"] == ref["overlap"]
    if ref["overlap"]:
        return
    for k in keys:
        assert close(res[k], ref[k], scale=1e-6), (k, res[k], ref[k])
    for m in range(maxmls):
        assert close(res["delE"][m], ref["delE"][m], scale=1e-6), ("delE", m, res["delE"], ref["delE"])


def test_gpu_per_move_abi_fp64(fmc_lib, oracle_lib, small):
    """insertion / deletion / displace_guest / commit through the C ABI, FP64,
    against the oracle on the same state."""
    o = oracle_lib.Oracle(small)
    sysm = fmc_lib.System.load(small)
    plain = fmc_lib.PlainEngine(sysm, fmc_lib.FMC_PREC_FP64, 64)
    maxmls = sysm.info().maxmls
    pos = _free_positions(o, 14, seed=1)
    assert len(pos) >= 10
    # build the same guest population on both sides
    inserted = 0
    for xyz in pos[:10]:
        ref = o.insertion_energy(1, xyz)
        res = plain.insertion(1, xyz)
        _cmp(res, ref, maxmls)
        # rande 0 accepts any non-overlapping insertion; an overlapping one
        # (with a guest inserted earlier in this loop) is rejected on both sides
        assert plain.commit(0.0) == (not ref["overlap"])
        o.apply_move(1, 1, 0, xyz, not ref["overlap"])
        inserted += not ref["overlap"]
        if inserted == 8:
            break
    assert plain.nummols(1) == o.nummols(o.locguest(1)) == inserted >= 6
    assert np.allclose(plain.coords(1), o.coords(o.locguest(1)), rtol=0, atol=1e-12)
    # trial insertions, including overlapping ones
    rng = np.random.default_rng(3)
    for xyz in pos[8:] + [pos[0] + 0.3]:
        _cmp(plain.insertion(1, xyz), o.insertion_energy(1, xyz), maxmls)
    # deletions of every molecule
    for c in range(1, inserted + 1):
        _cmp(plain.deletion(1, c), o.deletion_energy(1, c), maxmls)
    # displacements with random shift and rotation
    for _ in range(12):
        c = int(rng.integers(1, inserted + 1))
        a, b, cc = rng.uniform(-0.6, 0.6, 3)
        th = rng.uniform(0, 1.0)
        ax = rng.normal(size=3)
        ax /= np.linalg.norm(ax)
        q = [math.cos(th / 2), *(math.sin(th / 2) * ax)]
        abcq = [a, b, cc, *q]
        # displace_guest reports estep and delE only (gcmc.f:2886-2898)
        _cmp(plain.displace(1, c, abcq), o.displace_energy(1, c, abcq), maxmls, keys=("estep",))
    # commit a displacement and a deletion on both, then compare S(k)
    abcq = [0.2, -0.1, 0.05, 1.0, 0.0, 0.0, 0.0]
    r = plain.displace(1, 3, abcq)
    if not r["overlap"]:
        assert plain.commit(0.0) or r["estep"] > 0
        o.apply_move(3, 1, 3, abcq, True)
    plain.deletion(1, 5)
    plain.commit(0.0)
    o.apply_move(2, 1, 5, None, True)
    assert plain.nummols(1) == o.nummols(o.locguest(1))
    sg, so = plain.sk(), o.sk()
    assert np.allclose(sg, so, rtol=1e-10, atol=1e-10 * np.abs(so).max())
    eg = plain.energy()
    mol = o.locguest(1)
    assert close(eg[mol - 1], o.energy(mol), rel=1e-9, scale=1e-6)


def _oracle_chain(oracle_lib, d, seed, ncreate, nmoves):
    o = oracle_lib.Oracle(d)
    o.seed(seed)
    if ncreate:
        o.create_molecules(1, ncreate)
    return o, o.run(nmoves)


def test_gpu_chain_fp64_matches_oracle(fmc_lib, oracle_lib, small):
    """A whole chain on the device (RNG, proposals, Metropolis, commit) in
    FP64 follows the oracle move by move: identical decisions, estep to
    1e-9 relative."""
    n = 600
    o, ref = _oracle_chain(oracle_lib, small, 77, 10, n)
    sysm = fmc_lib.System.load(small)
    b = fmc_lib.Batch([sysm], [{"seed": 77}], precision=fmc_lib.FMC_PREC_FP64, guest_capacity=64)
    b.set_log(n)
    b.run(n)
    got = b.log(0, n)
    assert len(got) == n
    for i, (g, r) in enumerate(zip(got, ref)):
        assert (g.move, g.choice, g.overlap, g.accepted) == (r.move, r.choice, r.overlap, r.accepted), i
        assert g.rande == r.rande, i
        if not r.overlap:
            assert close(g.estep, r.estep, scale=1e-6), (i, g.estep, r.estep)
        assert g.nmols_after == r.nmols_after
    st = b.stats()[0]
    mol = o.locguest(1)
    assert st.nummols == o.nummols(mol)
    # energy(mol) is a running sum of delE: compare on the scale of the moves
    scale = max(abs(r.estep) for r in ref)
    assert close(st.energy, o.energy(mol), rel=1e-9, scale=scale)
    ostats = o.stats(1)
    assert st.attempts[0] == ostats[10] and st.accepts[0] == ostats[11]


def test_gpu_batch_chains_independent(fmc_lib, small):
    """Chains in one launch do not interact: a 3-chain batch reproduces
    three single-chain runs bit for bit."""
    sysm = fmc_lib.System.load(small)
    seeds = [5, 6, 7]
    b = fmc_lib.Batch([sysm], [{"seed": s} for s in seeds], precision=fmc_lib.FMC_PREC_FP64,
                      guest_capacity=64)
    b.run(200)
    multi = b.stats()
    for i, s in enumerate(seeds):
        one = fmc_lib.Batch([sysm], [{"seed": s}], precision=fmc_lib.FMC_PREC_FP64, guest_capacity=64)
        one.run(200)
        st = one.stats()[0]
        assert st.nummols == multi[i].nummols
        assert st.energy == multi[i].energy
        assert list(st.accepts) == list(multi[i].accepts)


def _jump_dir(inputs_dir):
    """Jump-heavy moves (gcmc.f:1937-2039) with no deletions and a 1.0 A
    overlap distance, so that some jumps land free and are accepted."""
    spec = syn.small_test_spec(seed=4, kmax=6, pressure_bar=5.0, create=20,
                               move_mix=(("insert", 0.1), ("displace", 0.3), ("jump", 0.6)))
    spec.overlap = 1.0
    return inputs_dir(spec, "gpu_jump")


def test_gpu_chain_fp64_jump_matches_oracle(fmc_lib, oracle_lib, inputs_dir):
    """Jump moves in an FP64 device chain follow the oracle move by move."""
    d = _jump_dir(inputs_dir)
    n = 600
    o, ref = _oracle_chain(oracle_lib, d, 9, 20, n)
    sysm = fmc_lib.System.load(d)
    b = fmc_lib.Batch([sysm], [{"seed": 9}], precision=fmc_lib.FMC_PREC_FP64, guest_capacity=64)
    b.set_log(n)
    b.run(n)
    got = b.log(0, n)
    for i, (g, r) in enumerate(zip(got, ref)):
        assert (g.move, g.choice, g.overlap, g.accepted) == (r.move, r.choice, r.overlap, r.accepted), i
        assert g.rande == r.rande, i
        if not r.overlap:
            assert close(g.estep, r.estep, scale=1e-6), (i, g.estep, r.estep)
    jumps = [r for r in ref if r.move == 6]
    assert len(jumps) > 100 and sum(r.accepted for r in jumps) >= 5
    st = b.stats()[0]
    ostats = o.stats(1)
    assert st.attempts[5] == ostats[23] and st.accepts[5] == ostats[24]
    mol = o.locguest(1)
    assert close(st.energy, o.energy(mol), rel=1e-9, scale=max(abs(r.estep) for r in ref))
    x, nm = b.coords(0)
    assert np.allclose(x[:9 * nm].reshape(-1, 3), o.coords(mol), rtol=0, atol=1e-9)


def test_gpu_chain_fp32_jump(fmc_lib, oracle_lib, inputs_dir):
    """Jump moves built in FP32 hi/lo geometry on the device: same moves as
    the oracle until the first decision at the Metropolis threshold, with
    estep within 1e-6 of the larger of |estep| and the jumping molecule's
    energy before the move (the oracle's deletion energy of that molecule)."""
    d = _jump_dir(inputs_dir)
    n = 600
    _, ref = _oracle_chain(oracle_lib, d, 9, 20, n)
    o = oracle_lib.Oracle(d)
    o.seed(9)
    o.create_molecules(1, 20)
    e_old = []
    for r in ref:
        e_old.append(o.deletion_energy(1, r.choice)["estep"] if r.move in (3, 6) else 0.0)
        step = o.run(1)[0]
        assert (step.move, step.choice, step.accepted) == (r.move, r.choice, r.accepted)
    sysm = fmc_lib.System.load(d)
    b = fmc_lib.Batch([sysm], [{"seed": 9}], precision=fmc_lib.FMC_PREC_FP32, guest_capacity=64)
    b.set_log(n)
    b.run(n)
    got = b.log(0, n)
    njump = 0
    for i, (g, r) in enumerate(zip(got, ref)):
        assert (g.move, g.choice) == (r.move, r.choice), i
        if g.overlap != r.overlap or g.accepted != r.accepted:
            break  # a threshold decision; the chains part here
        if r.overlap:
            continue
        assert abs(g.estep - r.estep) <= 1e-6 * max(abs(r.estep), abs(e_old[i]), 1.0), \
            (i, g.estep, r.estep, e_old[i])
        njump += r.move == 6
    assert njump >= 20


def _two_guest_dir(inputs_dir):
    """CO2 and a two-site dipolar guest in one framework (each type has its
    own pressure, loading and guest-guest terms with the other), moves that
    keep both populations: insert, displace, rotate, jump."""
    spec = syn.small_test_spec(seed=4, kmax=6, pressure_bar=5.0, create=10,
                               move_mix=(("insert", 0.1), ("displace", 0.3), ("jump", 0.3),
                                         ("rotate", 0.3)))
    spec.overlap = 1.0
    spec.second_guest = True
    spec.create2 = 8
    return inputs_dir(spec, "gpu_two_guests")


def _two_guest_oracle(oracle_lib, d, n):
    o = oracle_lib.Oracle(d)
    o.seed(7)
    o.create_molecules(1, 10)
    o.create_molecules(2, 8)
    return o, o.run(n)


def test_gpu_two_guest_types_fp64(fmc_lib, oracle_lib, inputs_dir):
    """Two guest types (the multi-type kernel: per-type accumulators, S(k),
    delE of the other types): an FP64 chain follows the oracle move by move."""
    d = _two_guest_dir(inputs_dir)
    n = 400
    o, ref = _two_guest_oracle(oracle_lib, d, n)
    b = fmc_lib.Batch([fmc_lib.System.load(d)], [{"seed": 7}], precision=fmc_lib.FMC_PREC_FP64,
                      guest_capacity=64)
    b.set_log(n)
    b.run(n)
    got = b.log(0, n)
    for i, (g, r) in enumerate(zip(got, ref)):
        assert (g.move, g.iguest, g.choice, g.overlap, g.accepted) == \
               (r.move, r.iguest, r.choice, r.overlap, r.accepted), i
        if not r.overlap:
            assert close(g.estep, r.estep, scale=1e-6), (i, g.estep, r.estep)
    assert {r.iguest for r in ref if r.accepted} == {1, 2}
    x, m = b.coords(0)  # guest type 1
    assert m == o.nummols(o.locguest(1))
    assert np.allclose(x[:9 * m].reshape(-1, 3), o.coords(o.locguest(1)), rtol=0, atol=1e-9)


def test_gpu_two_guest_types_fp32(fmc_lib, oracle_lib, inputs_dir):
    """The same on the FP32 multi-type kernel, until the first decision at
    the Metropolis threshold; estep within 1e-6 of max(|estep|, 1)."""
    d = _two_guest_dir(inputs_dir)
    n = 400
    _, ref = _two_guest_oracle(oracle_lib, d, n)
    b = fmc_lib.Batch([fmc_lib.System.load(d)], [{"seed": 7}], precision=fmc_lib.FMC_PREC_FP32,
                      guest_capacity=64)
    b.set_log(n)
    b.run(n)
    got = b.log(0, n)
    nfull = 0
    for i, (g, r) in enumerate(zip(got, ref)):
        assert (g.move, g.iguest, g.choice) == (r.move, r.iguest, r.choice), i
        if g.overlap != r.overlap or g.accepted != r.accepted:
            break
        if not r.overlap:
            assert abs(g.estep - r.estep) <= 2e-6 * max(abs(r.estep), 1.0), (i, g.estep, r.estep)
            nfull += 1
    assert nfull >= 10


def _switch_dir(inputs_dir):
    """Two guest types with switch moves (mc_switch, gcmc.f:2041-2267, which
    returns without acting unless two other guest types hold molecules) and
    "sampling accepted", so the production block reads the `accepted` a
    switch leaves behind."""
    spec = syn.small_test_spec(seed=4, kmax=6, pressure_bar=5.0, create=6,
                               move_mix=(("insert", 0.2), ("displace", 0.3), ("switch", 0.5)))
    spec.overlap = 1.0
    spec.second_guest = True
    spec.create2 = 4
    spec.accepted_sampling = True
    return inputs_dir(spec, "gpu_switch")


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_gpu_switch_no_op(fmc_lib, oracle_lib, inputs_dir, prec):
    """Switch moves on the device: the same move sequence as the oracle, a
    switch keeps the previous `accepted`, and (FP64, move by move) the same
    decisions and production count."""
    d = _switch_dir(inputs_dir)
    n = 400
    o = oracle_lib.Oracle(d)
    o.seed(7)
    o.create_molecules(1, 6)
    o.create_molecules(2, 4)
    ref = o.run(n)
    p = fmc_lib.FMC_PREC_FP64 if prec == "fp64" else fmc_lib.FMC_PREC_FP32
    b = fmc_lib.Batch([fmc_lib.System.load(d)], [{"seed": 7}], precision=p, guest_capacity=64)
    b.set_log(n)
    b.run(n)
    got = b.log(0, n)
    assert sum(r.move == 0 for r in ref) >= 100
    same = True
    for i, (g, r) in enumerate(zip(got, ref)):
        assert (g.move, g.iguest, g.choice) == (r.move, r.iguest, r.choice), i
        if g.move == 0:
            assert g.accepted == (got[i - 1].accepted if i else 0), i
        if g.overlap != r.overlap or g.accepted != r.accepted:
            assert prec == "fp32", i
            same = False
            break
        if not r.overlap and r.move != 0:
            assert abs(g.estep - r.estep) <= (1e-9 if prec == "fp64" else 2e-6) * max(abs(r.estep), 1.0), i
    if prec == "fp64":
        assert same and b.stats()[0].prodcount == o.prodcount() == sum(r.accepted for r in ref)


def _swap_dir(inputs_dir):
    """CO2 and the two-site dipolar guest, 8 and 6 molecules, with swap moves."""
    spec = syn.small_test_spec(seed=4, kmax=6, pressure_bar=5.0, create=8,
                               move_mix=(("insert", 0.2), ("displace", 0.3), ("swap", 0.5)))
    spec.overlap = 1.0
    spec.second_guest = True
    spec.create2 = 6
    return inputs_dir(spec, "gpu_swap")


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_gpu_swap_per_move(fmc_lib, oracle_lib, inputs_dir, prec):
    """fmc_swap against the oracle's mc_swap (gcmc.f:2269-2452) on the same
    loaded state, with the same draws: swaps the reference's test rejects,
    swaps forced through (rande -1) and overlapping ones, the engine taking
    its numbers only when the reference draws them.  estepi, estepj
    and every decision agree (FP64 to 1e-9, FP32 to 2e-6 of max(|e|, 1));
    after the sequence both guest types' coordinates, S(k) and energies
    agree, so rejections restored the state and acceptances committed both
    halves."""
    d = _swap_dir(inputs_dir)
    o = oracle_lib.Oracle(d)
    o.seed(5)
    o.create_molecules(1, 8)
    o.create_molecules(2, 6)
    p = fmc_lib.PlainEngine(fmc_lib.System.load(d),
                            fmc_lib.FMC_PREC_FP64 if prec == "fp64" else fmc_lib.FMC_PREC_FP32, 64)
    moved = 0.0  # sum of |energy change| committed: the scale of the running energies' error
    for g, ns in ((1, 3), (2, 2)):
        for m in o.coords(o.locguest(g)).reshape(-1, ns, 3):
            r = p.insertion(g, m)
            assert not r["overlap"]
            assert p.commit(0.0)
            moved += abs(r["estep"])
    tol = 1e-9 if prec == "fp64" else 2e-6
    rng = np.random.default_rng(3)
    nacc = nrej = nov = 0
    for t in range(24):
        ig = 1 + t % 2
        jg = 3 - ig
        choice = int(rng.integers(1, p.nummols(ig) + 1))
        th = rng.uniform(0, 2 * math.pi)
        ax = rng.normal(size=3)
        ax /= np.linalg.norm(ax)
        q = [math.cos(th / 2), *(math.sin(th / 2) * ax)]
        rande = [-1.0, -1.0] if t % 3 == 0 else list(rng.uniform(size=2))
        ei, ej, ov, acc = o.swap(ig, choice, jg, q, rande)
        draws = iter(rande)
        got = p.swap(ig, choice, jg, q, lambda: next(draws))
        assert (got["overlap"], got["accepted"]) == (ov, acc), t
        assert abs(got["estepi"] - ei) <= tol * max(abs(ei), 1.0), (t, got["estepi"], ei)
        if not ov:
            assert abs(got["estepj"] - ej) <= tol * max(abs(ej), 1.0), (t, got["estepj"], ej)
        nacc += acc
        nov += ov
        moved += abs(ei) + abs(ej) if acc else 0.0
        nrej += not acc and not ov
    assert nacc >= 2 and nrej >= 4 and nov >= 1
    for g in (1, 2):
        m = o.locguest(g)
        assert p.nummols(g) == o.nummols(m)
        assert np.allclose(p.coords(g), o.coords(m), rtol=0, atol=1e-9)
    so = o.sk()
    assert np.allclose(p.sk(), so, rtol=0, atol=(1e-10 if prec == "fp64" else 1e-5) * np.abs(so).max())
    eg = p.energy()
    for g in (1, 2):
        m = o.locguest(g)
        assert abs(eg[m - 1] - o.energy(m)) <= tol * moved, (g, eg[m - 1], o.energy(m), moved)


def test_gpu_swap_pending_refuses_other_moves(fmc_lib, inputs_dir):
    """Between fmc_swap and fmc_swap_finish the engine refuses other moves,
    and a finished rejection leaves coordinates and S(k) as they were."""
    import ctypes as C
    from fastmc_gb300 import _lib as L
    d = _swap_dir(inputs_dir)
    p = fmc_lib.PlainEngine(fmc_lib.System.load(d), fmc_lib.FMC_PREC_FP64, 64)
    rng = np.random.default_rng(2)
    for g, n in ((1, 4), (2, 3)):
        while p.nummols(g) < n:
            x = rng.uniform(0, 25.6, 3)
            m = np.array([[0.0, 0.0, 0.0], [1.16, 0.0, 0.0], [-1.16, 0.0, 0.0]])[:3 if g == 1 else 2] + x
            if not p.insertion(g, m)["overlap"]:
                p.commit(0.0)
    x0, s0 = [p.coords(g).copy() for g in (1, 2)], p.sk().copy()
    q = (C.c_double * 4)(1.0, 0.0, 0.0, 0.0)
    r = L.SwapResult()
    L.check(L.load().fmc_swap(p._h, 1, 2, 2, q, C.byref(r)))
    with pytest.raises(fmc_lib.FmcError):
        p.deletion(1, 1)
    assert p.nummols(1) == 3 and p.nummols(2) == 3 + (not r.overlap)
    L.check(L.load().fmc_swap_finish(p._h, 0))
    assert [p.nummols(g) for g in (1, 2)] == [4, 3]
    assert all(np.array_equal(p.coords(g), x) for g, x in zip((1, 2), x0))
    assert np.array_equal(p.sk(), s0)
    with pytest.raises(fmc_lib.FmcError):
        L.check(L.load().fmc_swap_finish(p._h, 0))


def _calf20_positions(o, n, seed, iguest=1):
    """Trial positions of a guest inside CALF-20's parallelepiped cell (random
    fractional centre and orientation) that the oracle finds free of overlap."""
    cell = np.array(o.array("cell")).reshape(3, 3)
    tm = np.array(o.array("guest_tmpl"))[:9].reshape(3, 3) if iguest == 1 else None
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(20000):
        th = rng.uniform(0, 2 * math.pi)
        ax = rng.normal(size=3)
        ax /= np.linalg.norm(ax)
        c, s = math.cos(th), math.sin(th)
        K = np.array([[0, -ax[2], ax[1]], [ax[2], 0, -ax[0]], [-ax[1], ax[0], 0]])
        R = np.eye(3) + s * K + (1 - c) * K @ K
        xyz = tm @ R.T + rng.uniform(0, 1, 3) @ cell
        if not o.insertion_energy(iguest, xyz)["overlap"]:
            out.append(xyz)
            if len(out) == n:
                break
    return out


def test_gpu_calf20_per_move_fp64(fmc_lib, oracle_lib):
    """The per-move C ABI on the reference's own test system (CALF-20,
    parallelepiped cell, imcon 3, two guest types) against the oracle:
    insertions, deletions, displacements and the committed S(k), FP64."""
    o = oracle_lib.Oracle(CALF20)
    sysm = fmc_lib.System.load(CALF20)
    assert sysm.info().imcon == 3
    plain = fmc_lib.PlainEngine(sysm, fmc_lib.FMC_PREC_FP64, 64)
    maxmls = sysm.info().maxmls
    pos = _calf20_positions(o, 16, seed=3)
    assert len(pos) >= 12
    inserted = 0
    for xyz in pos:
        ref = o.insertion_energy(1, xyz)
        _cmp(plain.insertion(1, xyz), ref, maxmls)
        ok = not ref["overlap"]
        assert plain.commit(0.0) == ok
        o.apply_move(1, 1, 0, xyz, ok)
        inserted += ok
        if inserted == 10:
            break
    assert inserted >= 8
    assert np.allclose(plain.coords(1), o.coords(o.locguest(1)), rtol=0, atol=1e-12)
    for c in range(1, inserted + 1):
        _cmp(plain.deletion(1, c), o.deletion_energy(1, c), maxmls)
    rng = np.random.default_rng(8)
    nd = 0
    for _ in range(40):
        c = int(rng.integers(1, inserted + 1))
        th = rng.uniform(0, 0.8)
        ax = rng.normal(size=3)
        ax /= np.linalg.norm(ax)
        abcq = [*rng.uniform(-0.4, 0.4, 3), math.cos(th / 2), *(math.sin(th / 2) * ax)]
        ref = o.displace_energy(1, c, abcq)
        _cmp(plain.displace(1, c, abcq), ref, maxmls, keys=("estep",))
        nd += not ref["overlap"]
    assert nd >= 10
    plain.deletion(1, 2)
    plain.commit(0.0)
    o.apply_move(2, 1, 2, None, True)
    sg, so = plain.sk(), o.sk()
    assert np.allclose(sg, so, rtol=1e-10, atol=1e-10 * np.abs(so).max())


@pytest.mark.parametrize("csize", [1, 2])
def test_gpu_calf20_chain_fp64(fmc_lib, oracle_lib, csize):
    """A device-resident FP64 chain on CALF-20 with the test's CONTROL (CO2
    and N2, insert / delete / displace, probability grids) follows the
    oracle move by move on the parallelepiped cell, on one CTA and on a
    2-CTA cluster (each CTA scans its share of the framework atoms)."""
    n = 3000
    o = oracle_lib.Oracle(CALF20)
    o.seed(12345)
    ref = o.run(n)
    b = fmc_lib.Batch([fmc_lib.System.load(CALF20)], [{"seed": 12345}],
                      precision=fmc_lib.FMC_PREC_FP64, guest_capacity=64)
    b.set_cluster([csize])
    b.set_log(n)
    b.run(n)
    got = b.log(0, n)
    nacc = nfull = 0
    for i, (g, r) in enumerate(zip(got, ref)):
        assert (g.move, g.iguest, g.choice, g.overlap, g.accepted) == \
               (r.move, r.iguest, r.choice, r.overlap, r.accepted), i
        assert g.rande == r.rande, i
        if not r.overlap:
            assert close(g.estep, r.estep, scale=1e-6), (i, g.estep, r.estep)
            nfull += 1
        nacc += r.accepted
    assert nacc >= 50 and nfull >= 200
    st = b.stats()[0]
    assert st.nummols == o.nummols(o.locguest(1))


def test_gpu_calf20_per_move_fp32(fmc_lib, oracle_lib):
    """The FP32 path on CALF-20's parallelepiped cell (minimum images through
    whole cell translations taken off in hi/lo pairs, fractional coordinates
    in double-float): insertion, deletion and displacement estep against the
    oracle to 1e-6 of max(|estep|, the molecule's energy, 1 kcal/mol), the
    same overlap outcomes, and S(k) after the commits."""
    o = oracle_lib.Oracle(CALF20)
    sysm = fmc_lib.System.load(CALF20)
    plain = fmc_lib.PlainEngine(sysm, fmc_lib.FMC_PREC_FP32, 64)
    pos = _calf20_positions(o, 16, seed=3)
    inserted = 0
    for xyz in pos:
        ref = o.insertion_energy(1, xyz)
        got = plain.insertion(1, xyz)
        assert got["overlap"] == ref["overlap"]
        if not ref["overlap"]:
            assert abs(got["estep"] - ref["estep"]) <= 1e-6 * max(abs(ref["estep"]), 1.0)
        ok = not ref["overlap"]
        assert plain.commit(0.0) == ok
        o.apply_move(1, 1, 0, xyz, ok)
        inserted += ok
        if inserted == 10:
            break
    assert inserted >= 8
    eown = {}
    for c in range(1, inserted + 1):
        ref = o.deletion_energy(1, c)
        eown[c] = abs(ref["estep"])
        got = plain.deletion(1, c)
        assert abs(got["estep"] - ref["estep"]) <= 1e-6 * max(abs(ref["estep"]), 1.0)
    rng = np.random.default_rng(8)
    nd = 0
    for _ in range(40):
        c = int(rng.integers(1, inserted + 1))
        th = rng.uniform(0, 0.8)
        ax = rng.normal(size=3)
        ax /= np.linalg.norm(ax)
        abcq = [*rng.uniform(-0.4, 0.4, 3), math.cos(th / 2), *(math.sin(th / 2) * ax)]
        ref = o.displace_energy(1, c, abcq)
        got = plain.displace(1, c, abcq)
        assert got["overlap"] == ref["overlap"]
        if not ref["overlap"]:
            tol = 1e-6 * max(abs(ref["estep"]), eown[c], 1.0)
            assert abs(got["estep"] - ref["estep"]) <= tol, (c, got["estep"], ref["estep"])
            nd += 1
    assert nd >= 10
    plain.deletion(1, 2)
    plain.commit(0.0)
    o.apply_move(2, 1, 2, None, True)
    sg, so = plain.sk(), o.sk()
    assert np.allclose(sg, so, rtol=0, atol=2e-6 * np.abs(so).max())


@pytest.mark.parametrize("csize", [1, 2])
def test_gpu_calf20_all_moves_fp32(fmc_lib, oracle_lib, csize):
    """The reference's own test input unchanged (CALF-20, parallelepiped
    cell; CO2 and N2; insert / delete / displace / swap / switch / jump) in
    a batched FP32 chain, on one CTA and on a 2-CTA cluster: the chain
    follows the oracle move by move until its first decision at a
    threshold (estep to 2e-6 of max(|estep|, 30 kcal/mol), swaps to 1e-5
    of max(|estep|, 100)), over at least 500 moves."""
    import shutil
    import tempfile
    n = 3000
    with tempfile.TemporaryDirectory() as d:
        for f in ("CONFIG", "FIELD"):
            shutil.copy(os.path.join(CALF20, f), d)
        shutil.copy(os.path.join(CALF20, "CONTROL_all_moves"), os.path.join(d, "CONTROL"))
        o = oracle_lib.Oracle(d)
        o.seed(31)
        ref = o.run(n)
        b = fmc_lib.Batch([fmc_lib.System.load(d)], [{"seed": 31}],
                          precision=fmc_lib.FMC_PREC_FP32, guest_capacity=64)
        b.set_cluster([csize])
        b.set_log(n)
        b.run(n)
        got = b.log(0, n)
    assert all(s.status == 0 for s in b.stats())
    _, ncmp = _follow(got, ref, "fp32", (7,), 1e-5)
    kinds = {r.move for r in ref[:ncmp]}
    assert ncmp >= 500 and {1, 2, 3, 6, 7} <= kinds, (ncmp, kinds)


def test_gpu_window_statistics_two_guests_fp64(fmc_lib, oracle_lib, inputs_dir):
    """Per guest type <N> and the reference's "standard error" (the weighted
    standard deviation of the window averages, gcmc.f:1218-1241) from the
    device chain's windows equal the oracle's."""
    spec = syn.small_test_spec(seed=4, kmax=6, pressure_bar=5.0, create=10,
                               move_mix=(("insert", 0.1), ("displace", 0.3), ("jump", 0.3),
                                         ("rotate", 0.3)))
    spec.overlap = 1.0
    spec.second_guest = True
    spec.create2 = 8
    spec.steps = 100  # 100-move windows
    d = inputs_dir(spec, "gpu_two_guests_windows")
    n = 400
    o, _ = _two_guest_oracle(oracle_lib, d, n)
    b = fmc_lib.Batch([fmc_lib.System.load(d)], [{"seed": 7}], precision=fmc_lib.FMC_PREC_FP64,
                      guest_capacity=64)
    b.run(n)
    st = b.stats()[0]
    assert st.windows == 4
    for g in (1, 2):
        ref = o.stats(g)
        assert close(st.guest_avg_n[g - 1], ref[0], rel=1e-12, scale=1e-12), (g, st.guest_avg_n[g - 1], ref[0])
        assert close(st.guest_se_n[g - 1], ref[29], rel=1e-9, scale=1e-9), (g, st.guest_se_n[g - 1], ref[29])


def _open_dir(tmp_path, name, mix, ntypes):
    """An open framework (48 atoms per 12.8 A cell), 1.5 A overlap distance,
    CO2 plus the two-site dipolar guest (and the three-site linear one):
    8 / 6 (/ 6) molecules pre-loaded, none of them on the LJ wall."""
    spec = syn.small_test_spec(seed=4, kmax=6, pressure_bar=5.0, create=8, move_mix=mix)
    spec.overlap = 1.5
    spec.second_guest = True
    spec.create2 = 6
    if ntypes == 3:
        spec.third_guest = True
        spec.create3 = 6
    d = str(tmp_path / name)
    syn.write_inputs(d, spec, uc=syn.make_unit_cell(4, natoms=48))
    return d


def _follow(got, ref, prec, kinds, tol_kind):
    """Move-by-move comparison of a device chain's log with the oracle's:
    move, guest type and molecule always; FP64 every decision, rande and
    count, estep to 1e-9; FP32 until the first decision that differs (a
    decision at the threshold), estep to 2e-6 of max(|estep|, 30 kcal/mol)
    (the FP32 error follows the moving molecule's energies, not their
    difference; measured at most 5.4e-5 kcal/mol on identical states), moves
    of the given kinds to tol_kind of max(|estep|, 100) (they add energies
    of several molecules).  The given kinds' estep is compared also when
    they overlapped.  Returns the number of the given kinds compared and
    the number of moves compared."""
    nk = 0
    ncmp = 0
    for i, (g, r) in enumerate(zip(got, ref)):
        assert (g.move, g.iguest, g.choice) == (r.move, r.iguest, r.choice), i
        if prec == "fp32" and (g.overlap != r.overlap or g.accepted != r.accepted):
            break
        ncmp += 1
        assert (g.overlap, g.accepted) == (r.overlap, r.accepted), i
        if prec == "fp64":
            assert g.rande == r.rande, i
            assert g.nmols_after == r.nmols_after, i
        if r.move in kinds:
            tol = 1e-9 * max(abs(r.estep), 1.0) if prec == "fp64" else tol_kind * max(abs(r.estep), 100.0)
            assert abs(g.estep - r.estep) <= tol, (i, g.estep, r.estep)
            nk += 1
        elif not r.overlap:
            tol = 1e-9 * max(abs(r.estep), 1.0) if prec == "fp64" else 2e-6 * max(abs(r.estep), 30.0)
            assert abs(g.estep - r.estep) <= tol, (i, g.estep, r.estep)
    return nk, ncmp


def _final_state(b, o, types):
    """FP64 chain 0 against the oracle at the end: every guest type's count
    and coordinates in molecule order, and S(k)."""
    for gg in types:
        m = o.locguest(gg)
        x, cnt = _batch_coords(b, gg)
        assert cnt == o.nummols(m)
        assert np.allclose(x, o.coords(m), rtol=0, atol=1e-9)
    info = b.systems[0].info()
    so = o.sk()
    assert np.allclose(b.sk(0, info.newld, info.maxmls), so, rtol=0, atol=1e-9 * np.abs(so).max())


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_gpu_chain_swaps_follow_oracle(fmc_lib, oracle_lib, tmp_path, prec):
    """Swap moves inside device-resident chains (mc_swap, gcmc.f:2269-2452):
    the chain follows the oracle move by move -- the swapped molecule, the
    partner type and orientation drawn, both tests with the second number
    drawn only when the first passes, acceptances (3 here; with the
    reference's tests, whose volume is in cubic angstroms, a swap is
    accepted only when the deletion releases more than about 69 kT) and
    about 300 rejections that put the state back.  FP64: every decision,
    estep (deletion plus insertion) to 1e-9, and at the end both guest
    types' coordinates and S(k).  FP32: until the first decision at a
    threshold, swaps' estep to 1e-5 of max(|estep|, 100 kcal/mol)."""
    d = _open_dir(tmp_path, "swap", (("insert", 0.2), ("displace", 0.3), ("swap", 0.5)), 2)
    n = 600
    o = oracle_lib.Oracle(d)
    o.seed(5)
    o.create_molecules(1, 8)
    o.create_molecules(2, 6)
    ref = o.run(n)
    p = fmc_lib.FMC_PREC_FP64 if prec == "fp64" else fmc_lib.FMC_PREC_FP32
    b = fmc_lib.Batch([fmc_lib.System.load(d)], [{"seed": 5}], precision=p, guest_capacity=64)
    b.set_log(n)
    b.run(n)
    got = b.log(0, n)
    swaps = [r for r in ref if r.move == 7]
    assert len(swaps) >= 250 and sum(r.accepted for r in swaps) >= 2
    nsw, _ = _follow(got, ref, prec, (7,), 1e-5)
    assert nsw >= 50
    if prec == "fp64":
        st = b.stats()[0]
        assert st.attempts[6] == len(swaps) and st.accepts[6] == sum(r.accepted for r in swaps)
        _final_state(b, o, (1, 2))


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_gpu_chain_switch_follows_oracle(fmc_lib, oracle_lib, tmp_path, prec):
    """The acting mc_switch (gcmc.f:2041-2267) inside device-resident chains
    with three guest types: a molecule and one of another type that holds
    molecules exchange centres of mass, both deletions and both insertions
    committed before the decision (also an insertion that overlaps, whose
    commit adds the structure factor the partner's deletion left, as the
    reference's accept_move does; the second insertion is evaluated against
    that state, so estep and whether a number is drawn follow it), decided
    as a displacement on estepi + estepj, rejections putting everything
    back.  About 490 switches: 18 accepted, 71 with an overlap, 440 with a
    number drawn.  FP64: every decision, rande and count, estep to 1e-9
    (overlapping switches included), and at the end all three types'
    coordinates and S(k).  FP32: until the first decision at a threshold,
    switches' estep to 1e-5 of max(|estep|, 100 kcal/mol)."""
    d = _open_dir(tmp_path, "switch", (("displace", 0.4), ("switch", 0.6)), 3)
    n = 800
    o = oracle_lib.Oracle(d)
    o.seed(5)
    for gg, k in ((1, 8), (2, 6), (3, 6)):
        o.create_molecules(gg, k)
    ref = o.run(n)
    p = fmc_lib.FMC_PREC_FP64 if prec == "fp64" else fmc_lib.FMC_PREC_FP32
    b = fmc_lib.Batch([fmc_lib.System.load(d)], [{"seed": 5}], precision=p, guest_capacity=64)
    b.set_log(n)
    b.run(n)
    got = b.log(0, n)
    sw = [r for r in ref if r.move == 8]
    assert len(sw) >= 400 and sum(r.accepted for r in sw) >= 10 and sum(r.overlap for r in sw) >= 30
    nsw, _ = _follow(got, ref, prec, (8,), 1e-5)
    assert nsw >= 50
    if prec == "fp64":
        st = b.stats()[0]
        assert st.attempts[7] == len(sw) and st.accepts[7] == sum(r.accepted for r in sw)
        _final_state(b, o, (1, 2, 3))


def _batch_coords(b, iguest):
    """Site coordinates of one guest type of chain 0 (molecule order)."""
    import ctypes as C
    from fastmc_gb300 import _lib as L
    out = np.zeros(1 << 14)
    n = C.c_int()
    L.check(L.load().fmc_batch_get_coords_type(b._h, 0, iguest, out.ctypes.data_as(L.dp), out.size,
                                               C.byref(n)))
    ns = b.systems[0].info().guest_nsites[iguest - 1]
    return out[:3 * ns * n.value].reshape(-1, 3), n.value


def test_gpu_reference_all_moves_control_fp64(fmc_lib, oracle_lib):
    """The reference's own test input with all six moves (CALF-20, CO2 and
    N2, insert / delete / displace / swap / switch / jump in equal shares)
    in a device-resident FP64 chain, move by move against the oracle."""
    import os
    import shutil
    import tempfile
    n = 3000
    with tempfile.TemporaryDirectory() as d:
        for f in ("CONFIG", "FIELD"):
            shutil.copy(os.path.join(CALF20, f), d)
        shutil.copy(os.path.join(CALF20, "CONTROL_all_moves"), os.path.join(d, "CONTROL"))
        o = oracle_lib.Oracle(d)
        o.seed(31)
        ref = o.run(n)
        b = fmc_lib.Batch([fmc_lib.System.load(d)], [{"seed": 31}],
                          precision=fmc_lib.FMC_PREC_FP64, guest_capacity=64)
        b.set_log(n)
        b.run(n)
        got = b.log(0, n)
    kinds = set()
    for i, (g, r) in enumerate(zip(got, ref)):
        assert (g.move, g.iguest, g.choice, g.overlap, g.accepted) == \
               (r.move, r.iguest, r.choice, r.overlap, r.accepted), i
        if r.move != 0:  # a switch that does nothing draws nothing (logged -1 / 0)
            assert g.rande == r.rande, i
        if not r.overlap and r.move != 0:
            assert close(g.estep, r.estep, scale=1e-6), (i, g.estep, r.estep)
        kinds.add(r.move)
    assert {1, 2, 3, 6, 7}.issubset(kinds)


def test_gpu_commit_with_host_decision(fmc_lib, oracle_lib, small):
    """fmc_commit: the host decides (here at random) and the device commits
    accordingly; the oracle given the same decisions ends in the same state
    (coordinates, S(k), energy)."""
    o = oracle_lib.Oracle(small)
    plain = fmc_lib.PlainEngine(fmc_lib.System.load(small), fmc_lib.FMC_PREC_FP64, 64)
    rng = np.random.default_rng(12)
    pos = _free_positions(o, 12, seed=9)
    n = 0
    for xyz in pos:
        acc = bool(rng.random() < 0.7)
        r = plain.insertion(1, xyz)
        ov = o.insertion_energy(1, xyz)["overlap"]
        assert r["overlap"] == ov
        plain.commit_decided(acc)
        o.apply_move(1, 1, 0, xyz, acc and not ov)
        n += acc and not ov
    for _ in range(6):
        c = int(rng.integers(1, n + 1))
        acc = bool(rng.random() < 0.5)
        plain.deletion(1, c)
        plain.commit_decided(acc)
        o.apply_move(2, 1, c, None, acc)
        n -= acc
    assert plain.nummols(1) == o.nummols(o.locguest(1)) == n
    assert np.allclose(plain.coords(1), o.coords(o.locguest(1)), rtol=0, atol=1e-12)
    so = o.sk()
    assert np.allclose(plain.sk(), so, rtol=0, atol=1e-10 * np.abs(so).max())
