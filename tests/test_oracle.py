"""The CPU oracle against the reference's own known answer and its own
internal identities.  These run on the CPU only."""
import json
import math
import os

import numpy as np
import pytest

from conftest import CALF20, GOLDEN
from fastmc_gb300 import synthetic as syn


def golden():
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        return json.load(f)


def test_calf20_electrostatic_kat(oracle_lib):
    """Initial electrostatic energy of the reference test system equals the
    value the reference prints (run_test.py:39, gcmc.f:585-586)."""
    o = oracle_lib.Oracle(CALF20)
    e = o.setup_energies()
    g = golden()
    assert abs(e["ecoul"] - g["calf20_electrostatic_energy_kcal"]) < g["tolerance_abs"]
    # the k-machinery the KAT pins (utility_pack.f:412-423, ewald.f:91-94)
    assert (e["kmax1"], e["kmax2"], e["kmax3"]) == (9, 8, 8)
    assert e["newld"] == 870
    assert abs(e["alpha"] - 0.2539648) < 1e-6


def test_duni_reproducible_and_uniform(oracle_lib):
    a = oracle_lib.duni_sequence(12345, 20000)
    b = oracle_lib.duni_sequence(12345, 20000)
    c = oracle_lib.duni_sequence(54321, 20000)
    assert np.array_equal(a, b)
    assert not np.array_equal(a, c)
    assert a.min() >= 0.0 and a.max() < 1.0
    assert abs(a.mean() - 0.5) < 0.01
    # REAL*4 values: every draw is a float32 number
    assert np.array_equal(a.astype(np.float32).astype(np.float64), a)


@pytest.fixture(scope="module")
def small_dir(inputs_dir):
    return inputs_dir(syn.small_test_spec(seed=3, kmax=5, pressure_bar=1.0, create=12), "orc_small")


def test_insert_delete_reciprocity(oracle_lib, small_dir):
    """Deleting a just-inserted molecule costs exactly its insertion energy:
    deletion's estep is the molecule's own energy (energy_eval receives
    -estep, gcmc.f:1795) and its delE is the negative (mc_moves.f:477).
    This checks the structure-factor and tail bookkeeping of accept_move."""
    o = oracle_lib.Oracle(small_dir)
    o.seed(11)
    o.create_molecules(1, 12)
    rng = np.random.default_rng(5)
    tmpl = np.array([[0, 0, 0], [0, 0, 1.16], [0, 0, -1.16]])
    done = 0
    for _ in range(20000):
        c = rng.uniform(0, 25.6, 3)
        xyz = tmpl + c
        ins = o.insertion_energy(1, xyz)
        if ins["overlap"]:
            continue
        o.apply_move(1, 1, 0, xyz, True)
        n = o.nummols(o.locguest(1))
        dele = o.deletion_energy(1, n)
        assert math.isclose(ins["estep"], dele["estep"], rel_tol=1e-9, abs_tol=1e-9)
        mol = o.locguest(1)
        assert math.isclose(ins["delE"][mol - 1], -dele["delE"][mol - 1], rel_tol=1e-9, abs_tol=1e-9)
        o.apply_move(2, 1, n, None, True)
        done += 1
        if done == 5:
            break
    assert done >= 3


def test_chain_deterministic(oracle_lib, small_dir):
    runs = []
    for _ in range(2):
        o = oracle_lib.Oracle(small_dir)
        o.seed(77)
        o.create_molecules(1, 12)
        logs = o.run(300)
        runs.append([(l.move, l.choice, l.overlap, l.accepted, l.estep) for l in logs])
    assert runs[0] == runs[1]
    kinds = {r[0] for r in runs[0]}
    assert {1, 2, 3, 5} <= kinds


def test_move_mix_and_counts(oracle_lib, small_dir):
    o = oracle_lib.Oracle(small_dir)
    o.seed(5)
    o.create_molecules(1, 12)
    logs = o.run(400)
    st = o.stats(1)
    ins = sum(1 for l in logs if l.move == 1)
    dele = sum(1 for l in logs if l.move == 2)
    assert st[10] == ins and st[12] == dele
    assert st[11] == sum(1 for l in logs if l.move == 1 and l.accepted)
    # an overlapped insertion never draws the Metropolis number (gcmc.f:1730-1736)
    assert all(l.rande == -1.0 for l in logs if l.move == 1 and l.overlap)


JUMP_MIX = (("insert", 0.1), ("displace", 0.3), ("jump", 0.6))


def jump_spec():
    """Jump-heavy moves on the small framework, no deletions (the molecules
    stay) and a 1.0 A overlap distance, so that some jumps land free."""
    spec = syn.small_test_spec(seed=4, kmax=6, pressure_bar=5.0, create=20, move_mix=JUMP_MIX)
    spec.overlap = 1.0
    return spec


def test_jump_moves(oracle_lib, inputs_dir):
    """mc_jump (gcmc.f:1937-2039): counted in jump_count / accept_jump, a
    negative estep is accepted without a Metropolis draw, and after a run of
    jumps the running energy equals the energy of the final configuration
    rebuilt by inserting its molecules one by one into an empty framework."""
    d = inputs_dir(jump_spec(), "orc_jump")
    o = oracle_lib.Oracle(d)
    o.seed(9)
    o.create_molecules(1, 20)
    mol = o.locguest(1)
    logs = o.run(600)
    st = o.stats(1)
    jumps = [l for l in logs if l.move == 6]
    assert len(jumps) == st[23] and sum(l.accepted for l in jumps) == st[24]
    assert st[24] >= 5 and sum(l.overlap for l in jumps) >= 5
    for l in jumps:
        if l.overlap:
            assert not l.accepted and l.rande == -1.0
        elif l.estep < 0:
            assert l.accepted and l.rande == -1.0
        else:
            assert l.rande >= 0.0
    xyz = o.coords(mol).reshape(-1, 3, 3)
    assert len(xyz) == 20
    f = oracle_lib.Oracle(d)
    for m in xyz:
        f.apply_move(1, 1, 0, m, True)
    assert math.isclose(o.energy(mol), f.energy(mol), rel_tol=1e-12)


def prob_spec():
    """Jump-heavy moves with two probability grids (centre of mass; the
    three sites) on 0.8 A voxels of the 12.8 A unit cell (grid factor 2)."""
    spec = jump_spec()
    spec.probability = [[0], [1, 2, 3]]
    spec.grid_spacing = 0.8
    spec.grid_factor = (2, 2, 2)
    return spec


def test_probability_grid_oracle(oracle_lib, inputs_dir):
    """storeprob (utility_pack.f:621-687) after every production move: each
    binned point spreads weight 1 over eight voxels, so a grid's total is
    the number of binned points summed over the moves; the grid covers the
    unit cell (cell / grid factor)."""
    d = inputs_dir(prob_spec(), "orc_prob")
    o = oracle_lib.Oracle(d)
    o.seed(9)
    o.create_molecules(1, 20)
    logs = o.run(300)
    na, nb, nc, nsub = o.prob_info()
    assert (na, nb, nc, nsub) == (16, 16, 16, 2)
    assert o.prodcount() == 300
    pts = sum(l.nmols_after for l in logs)
    g1, g2 = o.prob_grid(1), o.prob_grid(2)
    assert math.isclose(g1.sum(), pts, rel_tol=1e-12)
    assert math.isclose(g2.sum(), 3 * pts, rel_tol=1e-12)
    assert g1.min() >= 0.0 and g2.min() >= 0.0


def test_cube_writer_layout(tmp_path):
    from fastmc_gb300.cube import fortran_e15_6, write_prob_cube
    assert fortran_e15_6(0.0) == "   0.000000E+00"
    assert fortran_e15_6(1.2345678) == "   0.123457E+01"
    assert fortran_e15_6(3.0e-5) == "   0.300000E-04"
    g = np.arange(2 * 3 * 7, dtype=float).reshape(2, 3, 7)
    p = tmp_path / "prob.cube"
    write_prob_cube(str(p), g, 10, [6.4, 0, 0, 0, 6.4, 0, 0, 0, 6.4], atoms=[(6, 1.0, 2.0, 3.0)])
    lines = p.read_text().splitlines()
    assert lines[0] == "probability cube file"
    assert lines[2].split()[0] == "1"
    assert int(lines[3].split()[0]) == 2 and int(lines[5].split()[0]) == 7
    vals = [float(v) for ln in lines[7:] for v in ln.split()]
    vol = (6.4 * 1.889725989) ** 3 / 42
    assert np.allclose(vals, g.reshape(-1) / vol / 10, rtol=1e-5)
    # six values per line, and a break at the end of every c row of 7
    assert [len(ln.split()) for ln in lines[7:9]] == [6, 1]


def _duni_state(seed):
    """duni's initial state for a seed (utility_pack.f:2796-2852, the seed
    hook ms = seed % 1000, sec = (seed // 1000) % 60), in float32."""
    f = np.float32
    ms, sec = seed % 1000, (seed // 1000) % 60
    i, j, k, l = (ms * 3) % 177 + 1, (sec * 23) % 177 + 1, (ms * 5) % 177 + 1, (sec * 3) % 168
    u = []
    for _ in range(97):
        s, t = f(0), f(0.5)
        for _ in range(24):
            m = (((i * j) % 179) * k) % 179
            i, j, k = j, k, m
            l = (53 * l + 1) % 169
            if (l * m) % 64 >= 32:
                s = f(s + t)
            t = f(0.5 * t)
        u.append(s)
    return dict(u=u, ir=97, jr=33, c=f(362436 / 16777216), cd=f(7654321 / 16777216),
                cm=f(16777213 / 16777216))


def _refill32(h):
    """The device's warp-parallel refill (refill_draws): 32 steps at once,
    lane k reading u[ir-k], u[jr-k] and c after k+1 steps in closed form."""
    f = np.float32
    ir0, jr0 = h["ir"], h["jr"]
    c0, cd, cm = (int(h[x] * f(16777216)) for x in ("c", "cd", "cm"))
    out, writes = [], []
    for lane in range(32):
        ir, jr = (ir0 - 1 - lane) % 97, (jr0 - 1 - lane) % 97
        uni = f(h["u"][ir] - h["u"][jr])
        if uni < 0:
            uni = f(uni + f(1))
        ci = int(np.fmod(c0 - (lane + 1) * cd, cm))
        if ci < 0:
            ci += cm
        c = f(f(ci) * f(1 / 16777216))
        o = f(uni - c)
        if o < 0:
            o = f(o + f(1))
        writes.append((ir, uni))
        out.append(o)
    for ir, uni in writes:
        h["u"][ir] = uni
    h["c"] = c
    h["ir"] = ir0 - 32 if ir0 - 32 > 0 else ir0 - 32 + 97
    h["jr"] = jr0 - 32 if jr0 - 32 > 0 else jr0 - 32 + 97
    return out


def test_parallel_generator_refill_matches_duni(oracle_lib):
    """The lane-parallel refill reproduces duni's sequence bit for bit."""
    for seed in (77, 12345, 59999):
        h = _duni_state(seed)
        got = []
        for _ in range(40):
            got += _refill32(h)
        ref = oracle_lib.duni_sequence(seed, 32 * 40)
        assert np.array_equal(np.array(got, dtype=np.float64), ref), seed


SWITCH_MIX = (("insert", 0.2), ("displace", 0.3), ("switch", 0.5))


def switch_spec():
    """Two guest types with switch moves and production statistics after
    accepted moves only, so that the `accepted` a switch leaves matters."""
    spec = syn.small_test_spec(seed=4, kmax=6, pressure_bar=5.0, create=6, move_mix=SWITCH_MIX)
    spec.overlap = 1.0
    spec.second_guest = True
    spec.create2 = 4
    spec.accepted_sampling = True
    return spec


def test_switch_returns_without_partners(oracle_lib, inputs_dir):
    """mc_switch (gcmc.f:2041-2267) returns before any draw unless two guest
    types other than the chosen one hold molecules.  With two guest types
    every switch leaves the configuration alone, and the production block
    (gcmc.f:1050-1083, with "sampling accepted") sees the previous move's
    `accepted`, which the main loop does not reset."""
    d = inputs_dir(switch_spec(), "orc_switch")
    o = oracle_lib.Oracle(d)
    o.seed(3)
    o.create_molecules(1, 6)
    o.create_molecules(2, 4)
    logs = o.run(500)
    counts = {1: 6, 2: 4}
    prev = 0
    nsw = 0
    for l in logs:
        if l.move == 0:
            nsw += 1
            assert l.accepted == prev and l.nmols_after == counts[l.iguest]
            assert l.estep == 0.0 and not l.overlap
        counts[l.iguest] = l.nmols_after
        prev = l.accepted
    assert nsw >= 150
    assert sum(1 for l in logs if l.move == 0 and l.accepted) >= 10
    assert o.prodcount() == sum(l.accepted for l in logs)


SWAP_MIX = (("insert", 0.2), ("displace", 0.3), ("swap", 0.5))


def swap_spec():
    """Two guest types (CO2 and a two-site dipolar molecule) with swap moves."""
    spec = syn.small_test_spec(seed=4, kmax=6, pressure_bar=5.0, create=8, move_mix=SWAP_MIX)
    spec.overlap = 1.0
    spec.second_guest = True
    spec.create2 = 6
    return spec


def _state(o):
    mols = [o.locguest(1), o.locguest(2)]
    return ([o.coords(m).copy() for m in mols], [o.energy(m) for m in mols], o.sk().copy())


def _same(a, b):
    return (all(np.array_equal(x, y) for x, y in zip(a[0], b[0])) and a[1] == b[1]
            and np.array_equal(a[2], b[2]))


def test_swap_reject_restores_and_accept_equals_delete_insert(oracle_lib, inputs_dir):
    """mc_swap (gcmc.f:2269-2452): a rejected swap leaves coordinates,
    energies and S(k) bit for bit as they were; an accepted one leaves the
    same state as deleting the molecule and inserting the partner type at
    its centre of mass (rotated by q) through accept_move."""
    d = inputs_dir(swap_spec(), "orc_swap")

    def fresh():
        o = oracle_lib.Oracle(d)
        o.seed(5)
        o.create_molecules(1, 8)
        o.create_molecules(2, 6)
        return o

    o = fresh()
    before = _state(o)
    th = 0.7
    q = [math.cos(th / 2), math.sin(th / 2) * 0.6, 0.0, math.sin(th / 2) * 0.8]
    nrej = nacc = 0
    for choice in range(1, 9):
        ei, ej, ov, acc = o.swap(1, choice, 2, q, [math.inf, math.inf])
        assert not acc and _same(_state(o), before)
        nrej += 1
    for choice in (3, 5, 7, 2):
        o = fresh()
        ref = fresh()
        ei, ej, ov, acc = o.swap(1, choice, 2, q, [-1.0, -1.0])
        assert acc == (not ov)
        if ov:
            assert _same(_state(o), before)
            continue
        nacc += 1
        assert math.isclose(ei, ref.deletion_energy(1, choice)["estep"] * -1.0, rel_tol=1e-12)
        ref.apply_move(2, 1, choice, None, True)
        xyz2 = np.asarray(o.coords(o.locguest(2))).reshape(-1, 2, 3)[-1]
        e2 = ref.insertion_energy(2, xyz2)
        assert not e2["overlap"] and math.isclose(ej, e2["estep"], rel_tol=1e-12, abs_tol=1e-12)
        ref.apply_move(1, 2, 0, xyz2, True)
        assert _same(_state(o), _state(ref))
    assert nrej == 8 and nacc >= 2


def test_swap_moves_in_a_chain(oracle_lib, inputs_dir):
    """Swaps in the main loop: counted in swap_count / accept_swap, and after
    a run the running energy of each guest type and S(k) equal those of the
    final configuration rebuilt molecule by molecule in an empty framework."""
    d = inputs_dir(swap_spec(), "orc_swap")
    o = oracle_lib.Oracle(d)
    o.seed(5)
    o.create_molecules(1, 8)
    o.create_molecules(2, 6)
    logs = o.run(600)
    sw = {g: [l for l in logs if l.move == 7 and l.iguest == g] for g in (1, 2)}
    for g in (1, 2):
        st = o.stats(g)
        assert len(sw[g]) == st[25] and sum(l.accepted for l in sw[g]) == st[26]
    assert len(sw[1]) + len(sw[2]) >= 100
    f = oracle_lib.Oracle(d)
    for g, ns in ((1, 3), (2, 2)):
        for m in o.coords(o.locguest(g)).reshape(-1, ns, 3):
            f.apply_move(1, g, 0, m, True)
    for g in (1, 2):
        assert math.isclose(o.energy(o.locguest(g)), f.energy(f.locguest(g)), rel_tol=1e-10, abs_tol=1e-9)
    assert np.allclose(o.sk(), f.sk(), rtol=0, atol=1e-9)


def test_reference_test_control_all_moves(oracle_lib, tmp_path):
    """The reference's own test input (CALF-20 with CO2 and three-site N2,
    insert / delete / displace / swap / switch / jump in equal shares,
    probability grids) runs in the oracle with every move kind, and the
    running energies and S(k) equal those of the final configuration rebuilt
    molecule by molecule."""
    import shutil
    src = os.path.join(os.path.dirname(__file__), "golden", "calf20")
    for f in ("CONFIG", "FIELD"):
        shutil.copy(os.path.join(src, f), tmp_path / f)
    shutil.copy(os.path.join(src, "CONTROL_all_moves"), tmp_path / "CONTROL")
    o = oracle_lib.Oracle(str(tmp_path))
    o.seed(11)
    o.create_molecules(1, 20)
    o.create_molecules(2, 20)
    kinds = set()
    for _ in range(5):  # the loading drains at these pressures: check along the way
        logs = o.run(100)
        kinds |= {l.move for l in logs}
        f = oracle_lib.Oracle(str(tmp_path))
        for g in (1, 2):
            for m in o.coords(o.locguest(g)).reshape(-1, 3, 3):
                f.apply_move(1, g, 0, m, True)
        for g in (1, 2):
            assert math.isclose(o.energy(o.locguest(g)), f.energy(f.locguest(g)),
                                rel_tol=1e-9, abs_tol=1e-8)
        assert np.allclose(o.sk(), f.sk(), rtol=0, atol=1e-9)
    assert {0, 1, 2, 3, 6, 7} <= kinds, kinds


def test_switch_with_three_guest_types(oracle_lib, inputs_dir):
    """mc_switch (gcmc.f:2041-2267) acting: with three loaded guest types a
    molecule and one of another type exchange centres of mass.  Counted in
    switch_count / accept_switch; along the run the running energies and
    S(k) equal those of the configuration rebuilt molecule by molecule, so
    accepted switches committed all four halves and rejected ones restored
    the state; an accepted switch keeps every type's count."""
    spec = syn.small_test_spec(seed=4, kmax=6, pressure_bar=5.0, create=8,
                               move_mix=(("displace", 0.4), ("switch", 0.6)))
    spec.overlap = 1.0
    spec.second_guest = True
    spec.create2 = 6
    spec.third_guest = True
    spec.create3 = 6
    d = inputs_dir(spec, "orc_switch3")
    o = oracle_lib.Oracle(d)
    o.seed(5)
    for g, n in ((1, 8), (2, 6), (3, 6)):
        o.create_molecules(g, n)
    nsite = {1: 3, 2: 2, 3: 3}
    logs = []
    for _ in range(4):
        part = o.run(150)
        logs += part
        f = oracle_lib.Oracle(d)
        for g in (1, 2, 3):
            for m in o.coords(o.locguest(g)).reshape(-1, nsite[g], 3):
                f.apply_move(1, g, 0, m, True)
        for g in (1, 2, 3):
            assert math.isclose(o.energy(o.locguest(g)), f.energy(f.locguest(g)),
                                rel_tol=1e-9, abs_tol=1e-8), g
        assert np.allclose(o.sk(), f.sk(), rtol=0, atol=1e-9)
    sw = [l for l in logs if l.move == 8]
    for g in (1, 2, 3):
        st = o.stats(g)
        mine = [l for l in sw if l.iguest == g]
        assert len(mine) == st[27] and sum(l.accepted for l in mine) == st[28]
    assert len(sw) >= 150 and sum(l.accepted for l in sw) >= 3
    assert [o.nummols(o.locguest(g)) for g in (1, 2, 3)] == [8, 6, 6]


def test_isotherm_fixtures_match_reference_keys():
    """Each of the ten isotherm inputs maps to one published uptake of
    run_test.py by its summed pressure, with the run length the reference
    test uses (750000 + 500000 moves)."""
    from oracle.isotherm import GOLD, control_numbers
    g = golden()
    keys = [float(k) for k in g["isotherm_avg_guests"]]
    names = sorted(os.listdir(os.path.join(GOLD, "calf20", "isotherm")))
    assert len(names) == len(keys) == 10
    seen = set()
    for n in names:
        p, steps, eq = control_numbers(os.path.join(GOLD, "calf20", "isotherm", n, "CONTROL"))
        k = min(keys, key=lambda v: abs(v - p))
        assert abs(k - p) < 1e-9 and (steps, eq) == (500000, 750000), n
        seen.add(k)
    assert len(seen) == 10


@pytest.mark.parametrize("name", ["isotherm_oracle.json", "isotherm_device.json"])
def test_recorded_isotherm_passes_reference_band(name):
    """The recorded isotherm runs (the oracle on CPU; FP64 device-resident
    chains on a GB300 with the ten CONTROL files unchanged, swap and switch
    included) re-checked against run_test.py's criterion from the published
    uptakes: both guests' averages within [0.8 (avg - se), 1.2 (avg + se)]
    at all ten pressures, with the reference's run length."""
    with open(os.path.join(GOLDEN, name)) as f:
        rec = json.load(f)
    ref = {float(k): v for k, v in golden()["isotherm_avg_guests"].items()}
    assert len(rec["rows"]) == 10
    for r in rec["rows"]:
        k = min(ref, key=lambda v: abs(v - r["pressure_bar"]))
        assert abs(k - r["pressure_bar"]) < 1e-5
        co2, n2 = ref[k]
        assert r.get("status", 0) == 0 and r["moves"] == 1250000
        for avg, se, v in ((r["avg_co2"], r["se_co2"], co2), (r["avg_n2"], r["se_n2"], n2)):
            assert 0.8 * (avg - se) <= v <= 1.2 * (avg + se), (r["point"], avg, se, v)


def test_energy_grids_as_the_main_loop_fills_them(oracle_lib, tmp_path):
    """storeenprob from the main loop (gcmc.f:1131-1134) gets the main
    program's guest_toten, which stays 0, and molecule 0: every accepted
    production move adds a count at the centre of mass of the move's last
    positions (weight 1 spread over 8 voxels) and nothing to the energy
    grid.  The grids follow the site grid in the guest type's block."""
    spec = syn.small_test_spec(seed=4, kmax=5, pressure_bar=5.0, create=10,
                               move_mix=(("insert", 0.2), ("delete", 0.2), ("displace", 0.6)))
    spec.overlap = 1.5
    spec.probability = [[0], "energy"]
    spec.grid_spacing = 0.8
    d = str(tmp_path / "energy_grid")
    syn.write_inputs(d, spec, uc=syn.make_unit_cell(4, natoms=48))  # an open framework
    o = oracle_lib.Oracle(d)
    o.seed(3)
    o.create_molecules(1, 10)
    logs = o.run(400)
    assert o.prob_info()[3] == 3
    site, energy, count = (o.prob_grid(k) for k in (1, 2, 3))
    nacc = sum(1 for r in logs if r.accepted)
    assert nacc >= 50
    assert np.all(energy == 0.0)
    assert count.sum() == pytest.approx(nacc, rel=1e-12)
    assert site.sum() == pytest.approx(sum(r.nmols_after for r in logs), rel=1e-12)


def test_preload_prefilter_changes_nothing(oracle_lib, inputs_dir):
    """insert_guests' framework pre-test skips only trial positions that
    insertion() rejects anyway: with it on and off the same molecules are
    created after the same number of trials, and the chains continue
    identically."""
    d = inputs_dir(syn.small_test_spec(seed=5, kmax=6, ntile=3, pressure_bar=5.0), "prefilter")
    runs = []
    for on in (True, False):
        o = oracle_lib.Oracle(d)
        o.set_prefilter(on)
        o.seed(31)
        it = o.create_molecules(1, 25)
        mol = o.locguest(1)
        x = o.coords(mol)
        lg = [(r.move, r.choice, r.overlap, r.accepted, r.estep) for r in o.run(300)]
        runs.append((it, x, o.sk(), lg))
    (i1, x1, s1, l1), (i2, x2, s2, l2) = runs
    assert i1 == i2 and i1 > 25
    assert np.array_equal(x1, x2)
    assert np.array_equal(s1, s2)
    assert l1 == l2


def test_oracle_state_save_restore_replays(oracle_lib, inputs_dir):
    """orc_save_state / orc_restore_state: every replay from the saved
    state makes the same moves with the same energies."""
    d = inputs_dir(syn.small_test_spec(seed=5, kmax=6, ntile=3, pressure_bar=5.0, create=20), "replay")
    o = oracle_lib.Oracle(d)
    o.seed(9)
    o.create_molecules(1, 20)
    o.save_state()
    a = [(r.move, r.choice, r.accepted, r.estep) for r in o.run(200)]
    for _ in range(2):
        o.restore_state()
        assert [(r.move, r.choice, r.accepted, r.estep) for r in o.run(200)] == a
