"""The reference's restart files (revive, utility_pack.f:2299-2344; revread,
gcmc.f:447-474) for device-resident chains: REVIVE as Fortran unformatted
sequential records and REVCON in CONFIG's layout, written from a chain and
read back into one.  The records are parsed here the way a Fortran
unformatted read sees them (a 4-byte count before and after each record)."""
import os
import struct

import numpy as np
import pytest

from fastmc_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def read_records(path):
    out = []
    with open(path, "rb") as f:
        raw = f.read()
    i = 0
    while i < len(raw):
        (n,) = struct.unpack_from("<i", raw, i)
        data = raw[i + 4:i + 4 + n]
        (m,) = struct.unpack_from("<i", raw, i + 4 + n)
        assert m == n
        out.append(data)
        i += 8 + n
    return out


def write_records(path, recs):
    with open(path, "wb") as f:
        for r in recs:
            f.write(struct.pack("<i", len(r)) + r + struct.pack("<i", len(r)))


def parse_revive(path, maxmls, natoms, ntpguest):
    """revread's reads (gcmc.f:461-471) for a system with maxmls molecule
    types of natoms[m] sites."""
    r = read_records(path)
    prod = struct.unpack("<i", r[0])[0]
    nm = list(struct.unpack(f"<{maxmls}i", r[1]))
    cs = np.frombuffer(r[2], dtype="<f8")
    assert cs.size == 16 * ntpguest + 1
    natms = struct.unpack("<i", r[3])[0]
    xyz = {}
    for m in range(1, maxmls + 1):
        x, y, z = (np.frombuffer(r[4 + 3 * (m - 1) + d], dtype="<f8") for d in range(3))
        assert x.size == nm[m - 1] * natoms[m]
        xyz[m] = np.stack([x, y, z], axis=1).reshape(-1)
    en = np.frombuffer(r[4 + 3 * maxmls], dtype="<f8")
    assert len(r) == 5 + 3 * maxmls and en.size == ntpguest
    return prod, nm, cs, natms, xyz, en


@pytest.fixture(scope="module")
def sysdir(inputs_dir):
    return inputs_dir(syn.small_test_spec(seed=4, kmax=6, pressure_bar=5.0, create=10), "revive_small")


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_revive_round_trip(fmc_lib, oracle_lib, sysdir, tmp_path, prec):
    """A chain's REVIVE holds its state as revive writes it (production flag,
    every molecule type's count, the open window's sums with the production
    count, the atom count, coordinates in molecule order -- the framework's
    from CONFIG --, energy(1..ntpguest)); REVCON lists guests then framework
    with the reference's formats; read into another chain, the molecules
    are where they were and the chain's S(k) and energies, rebuilt from
    them, equal the running ones."""
    p = fmc_lib.FMC_PREC_FP64 if prec == "fp64" else fmc_lib.FMC_PREC_FP32
    sysm = fmc_lib.System.load(sysdir)
    info = sysm.info()
    b = fmc_lib.Batch([sysm], [{"seed": 11}, {"seed": 12}], precision=p, guest_capacity=64)
    b.run(400)
    d = str(tmp_path / "branch01")
    os.makedirs(d)
    b.write_revive(0, d)
    o = oracle_lib.Oracle(sysdir)
    mol = o.locguest(1)
    fw = [m for m in range(1, info.maxmls + 1) if m != mol][0]
    nfw = o.nummols(fw)  # the framework: nfw molecules (tiles of the unit cell)
    natoms = {mol: 3, fw: o.coords(fw).shape[0] // nfw}
    st = b.stats()[0]
    prod, nm, cs, natms, xyz, en = parse_revive(os.path.join(d, "REVIVE"), info.maxmls, natoms, 1)
    x, n = b.coords(0)
    assert nm[mol - 1] == n == st.nummols and nm[fw - 1] == nfw
    assert natms == 3 * n + nfw * natoms[fw]
    assert np.array_equal(xyz[mol], x[:9 * n])
    assert np.array_equal(xyz[fw], o.coords(fw).reshape(-1))
    assert prod in (0, 1)
    assert cs[0] >= 0 and np.all(np.isfinite(cs))
    # REVCON: title, levcfg / imcon / energy, cell, then every atom
    lines = open(os.path.join(d, "REVCON")).read().split("\n")
    title = open(os.path.join(sysdir, "CONFIG")).readline().rstrip("\n")
    assert lines[0].rstrip() == title[:80].rstrip() and len(lines[0]) == 80
    assert int(lines[1][:10]) == 0 and int(lines[1][10:20]) == info.imcon and len(lines[1]) == 40
    cell = np.array([[float(l[20 * j:20 * j + 20]) for j in range(3)] for l in lines[2:5]])
    assert np.allclose(cell.reshape(-1), info.cell, rtol=1e-12)
    at = lines[5:5 + 2 * natms]
    assert int(at[0][8:18]) == 1 and int(at[2 * natms - 2][8:18]) == natms
    got = np.array([[float(l[20 * j:20 * j + 20]) for j in range(3)] for l in at[1::2]]).reshape(-1)
    want = np.concatenate([xyz[mol], xyz[fw]])
    assert np.allclose(got, want, rtol=1e-9, atol=1e-9)
    assert all(len(l) == 60 for l in at[1::2])
    # read back into chain 1
    b.read_revive(1, d)
    s0, s1 = b.stats()[0], b.stats()[1]
    x1, n1 = b.coords(1)
    assert n1 == n
    if prec == "fp64":
        assert np.array_equal(x1[:9 * n], x[:9 * n])
    else:
        assert np.allclose(x1[:9 * n], x[:9 * n], rtol=0, atol=1e-11)
    sk0, sk1 = b.sk(0, info.newld, info.maxmls), b.sk(1, info.newld, info.maxmls)
    tol = 1e-9 if prec == "fp64" else 2e-6
    assert np.allclose(sk1, sk0, rtol=0, atol=tol * np.abs(sk0).max())
    assert abs(s1.energy - s0.energy) <= tol * max(1.0, abs(s0.energy)) * 10
    # and the restarted chain runs on
    b.run(100)
    assert all(s.status == 0 for s in b.stats())


def test_revive_from_the_oracle(fmc_lib, oracle_lib, sysdir, tmp_path):
    """A REVIVE written the way revive writes it from the oracle's state
    after 300 moves (its coordinates in molecule order), read into a device
    chain: the chain holds exactly those molecules, and its S(k) and
    energy equal the oracle's running ones (FP64, 1e-9)."""
    o = oracle_lib.Oracle(sysdir)
    o.seed(21)
    o.create_molecules(1, 10)
    o.run(300)
    sysm = fmc_lib.System.load(sysdir)
    info = sysm.info()
    mol = o.locguest(1)
    fw = [m for m in range(1, info.maxmls + 1) if m != mol][0]
    n = o.nummols(mol)
    recs = [struct.pack("<i", 0),
            struct.pack(f"<{info.maxmls}i", *[o.nummols(m) for m in range(1, info.maxmls + 1)]),
            np.zeros(17).tobytes(), struct.pack("<i", 3 * n + o.coords(fw).shape[0])]
    for m in range(1, info.maxmls + 1):
        c = o.coords(m).reshape(-1, 3)
        recs += [np.ascontiguousarray(c[:, d]).tobytes() for d in range(3)]
    recs.append(np.zeros(1).tobytes())
    d = str(tmp_path / "orc")
    os.makedirs(d)
    write_records(os.path.join(d, "REVIVE"), recs)
    b = fmc_lib.Batch([sysm], [{"seed": 5}], precision=fmc_lib.FMC_PREC_FP64, guest_capacity=64)
    b.read_revive(0, d)
    x, nn = b.coords(0)
    assert nn == n
    assert np.array_equal(x[:9 * n], o.coords(mol).reshape(-1))
    so = o.sk()
    assert np.allclose(b.sk(0, info.newld, info.maxmls), so, rtol=0, atol=1e-9 * np.abs(so).max())
    e = o.energy(mol)
    assert abs(b.stats()[0].energy - e) <= 1e-9 * max(1.0, abs(e)) * 10


def test_revive_rejects_damaged_file(fmc_lib, sysdir, tmp_path):
    """A REVIVE whose records do not fit the system (a wrong length, a count
    above the capacity, another framework) is refused with FMC_ERR_INPUT or
    FMC_ERR_CAPACITY and the chain keeps its state."""
    from fastmc_gb300 import _lib as L
    sysm = fmc_lib.System.load(sysdir)
    b = fmc_lib.Batch([sysm], [{"seed": 3}], precision=fmc_lib.FMC_PREC_FP64, guest_capacity=64)
    b.run(200)
    d = str(tmp_path / "good")
    os.makedirs(d)
    b.write_revive(0, d)
    before = (b.stats()[0].nummols, b.stats()[0].energy)
    recs = read_records(os.path.join(d, "REVIVE"))
    cases = []
    bad = list(recs)
    bad[2] = bad[2][:-8]  # chainstats one value short
    cases.append((bad, L.FMC_ERR_INPUT))
    info = sysm.info()
    mol = info.guest_mol[0]
    fw = [m for m in range(1, info.maxmls + 1) if m != mol][0]
    nm = list(struct.unpack(f"<{info.maxmls}i", recs[1]))
    big = list(nm)
    big[mol - 1] = 1000  # guest count above the capacity
    bad = list(recs)
    bad[1] = struct.pack(f"<{info.maxmls}i", *big)
    cases.append((bad, None))
    bad = list(recs)
    fwi = 4 + 3 * (fw - 1)
    arr = np.frombuffer(recs[fwi], dtype="<f8").copy()
    arr[0] += 0.5
    bad[fwi] = arr.tobytes()
    cases.append((bad, L.FMC_ERR_INPUT))
    for k, (rr, code) in enumerate(cases):
        dd = str(tmp_path / f"bad{k}")
        os.makedirs(dd)
        write_records(os.path.join(dd, "REVIVE"), rr)
        rc = L.load().fmc_batch_read_revive(b._h, 0, dd.encode())
        assert rc != 0 and (code is None or rc == code), (k, rc)
        assert (b.stats()[0].nummols, b.stats()[0].energy) == before
