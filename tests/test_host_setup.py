"""The library's host set-up (readers, tables, k-vectors) against the
oracle, and the C-ABI surface.  CPU only: no kernel is launched."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import CALF20, ROOT
from fastmc_gb300 import synthetic as syn


def header_functions():
    with open(os.path.join(ROOT, "include", "fastmc_gb300.h")) as f:
        txt = f.read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(fmc_[a-z_0-9]+)\s*\(", txt)))


def test_library_exports_every_header_symbol(fmc_lib):
    import fastmc_gb300._lib as L
    lib = L.load()
    names = header_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n
        assert n in L.SIGNATURES, n
    assert lib.fmc_version().startswith(b"fastmc_gb300")


@pytest.mark.parametrize("which", ["calf20", "single25", "small"])
def test_setup_matches_oracle(fmc_lib, oracle_lib, inputs_dir, which):
    if which == "calf20":
        d = CALF20
    elif which == "single25":
        d = inputs_dir(syn.single_chain_25A(), "cfg1")
    else:
        d = inputs_dir(syn.small_test_spec(seed=9, kmax=6, create=5), "small9")
    s = fmc_lib.System.load(d)
    inf = s.info()
    o = oracle_lib.Oracle(d).setup_energies()
    assert inf.alpha == o["alpha"]
    assert tuple(inf.kmax) == (o["kmax1"], o["kmax2"], o["kmax3"])
    assert inf.newld == o["newld"]
    assert inf.sumchg == o["sumchg"]
    assert inf.volm == o["volm"]
    assert inf.engunit == o["engunit"]
    assert inf.overlap == o["overlap"] == 1.5


def test_tables_match_oracle(fmc_lib, oracle_lib, inputs_dir):
    d = inputs_dir(syn.single_chain_25A(), "cfg1")
    orc = oracle_lib.Oracle(d)
    out = np.zeros(2000)
    n = orc.lib.orc_get_erc(orc._h, out.ctypes.data_as(C.POINTER(C.c_double)), 2000)
    assert n == 1254  # mxegrd = int(12.5/0.01+0.5)+4 (utility_pack.f:996)
    s = fmc_lib.System.load(d)
    assert s.info().mxegrd == n
    assert abs(s.info().drewd - 0.01) < 1e-15


def test_config_errors_are_reported(fmc_lib, tmp_path):
    import fastmc_gb300._lib as L
    with pytest.raises(L.FmcError) as e:
        fmc_lib.System.load(str(tmp_path / "missing"))
    assert e.value.code == 4
    d = tmp_path / "swap"
    spec = syn.small_test_spec()
    spec.move_mix = (("insert", 0.5), ("swap", 0.5))
    syn.write_inputs(str(d), spec)
    with pytest.raises(L.FmcError) as e:
        fmc_lib.System.load(str(d))
    assert "swap" in str(e.value)


def test_synthetic_framework_properties():
    uc = syn.make_unit_cell(1)
    d = uc.xyz[:, None, :] - uc.xyz[None, :, :]
    d -= syn.UNIT_CELL * np.round(d / syn.UNIT_CELL)
    r2 = np.einsum("ijk,ijk->ij", d, d) + np.eye(len(uc.xyz)) * 1e9
    assert np.sqrt(r2.min()) >= syn.MIN_SEP
    assert abs(uc.charges.sum()) < 1e-9
    assert np.bincount(uc.types).tolist() == [48, 48, 48, 48]
    assert np.all((uc.eps >= 0.02) & (uc.eps <= 0.10))
    assert np.all((uc.sigma >= 2.5) & (uc.sigma <= 3.8))
    chains = syn.isotherm_chains()
    assert len(chains) == 64
    assert sorted({round(c.box, 6) for c in chains}) == [25.6, 38.4, 51.2, 64.0]


def test_probability_inputs(fmc_lib, tmp_path):
    """CONTROL probability blocks and grid keywords load, with and without
    an 'e' line (storeenprob's two energy grids, readinputs.f:652-670)."""
    spec = syn.small_test_spec()
    spec.probability = [[0], [1, 2, 3]]
    spec.grid_spacing = 0.8
    spec.grid_factor = (2, 2, 2)
    d = tmp_path / "prob"
    syn.write_inputs(str(d), spec)
    fmc_lib.System.load(str(d))
    txt = (d / "CONTROL").read_text().replace("  3 1 2 3\n", "  3 1 2 3\n  e\n").replace(
        "probability 2", "probability 3")
    (d / "CONTROL").write_text(txt)
    fmc_lib.System.load(str(d))


def test_swap_and_switch_set_up(fmc_lib, tmp_path):
    """Swap needs a partner type (refused with one guest type); switch loads
    with any number of guest types (it acts from three on)."""
    import fastmc_gb300._lib as L

    def spec(mix, ntypes):
        s = syn.small_test_spec(move_mix=mix)
        s.second_guest = ntypes >= 2
        s.third_guest = ntypes >= 3
        return s
    for mix, ntypes, ok in (((("insert", 0.5), ("switch", 0.5)), 1, True),
                            ((("insert", 0.5), ("switch", 0.5)), 2, True),
                            ((("insert", 0.5), ("switch", 0.5)), 3, True),
                            ((("insert", 0.5), ("displace", 0.5)), 3, True),
                            ((("insert", 0.5), ("swap", 0.5)), 1, False),
                            ((("insert", 0.5), ("swap", 0.5)), 2, True)):
        d = tmp_path / f"s{len(list(tmp_path.iterdir()))}"
        syn.write_inputs(str(d), spec(mix, ntypes))
        if ok:
            assert fmc_lib.System.load(str(d)).info().ntpguest == ntypes
        else:
            with pytest.raises(L.FmcError) as e:
                fmc_lib.System.load(str(d))
            assert "swap" in str(e.value)


def test_peng_robinson_fugacity(fmc_lib, oracle_lib, tmp_path):
    """CONTROL "fugacity" (fugacity / calc_fugacity, utility_pack.f:1206-1500):
    the set-up's Peng-Robinson fugacities equal the oracle's bit for bit, the
    CO2 fugacity coefficient at 293 K falls with pressure as the equation of
    state gives it (0.994 at 1 bar, 0.94 at 10 bar, 0.78 at 40 bar), and for a
    mixture the reference's fugacity is phi * y * p (the mole fraction times
    the partial pressure)."""
    cases = [(0.1, None), (1.0, None), (10.0, None), (40.0, None), (0.15, 0.85)]
    bounds = {1.0: (0.990, 0.997), 10.0: (0.93, 0.955), 40.0: (0.75, 0.81)}
    for k, (p1, p2) in enumerate(cases):
        spec = syn.small_test_spec(pressure_bar=p1)
        spec.fugacity = True
        if p2 is not None:
            spec.second_guest = True
            spec.pressure2_bar = p2
        d = tmp_path / f"f{k}"
        syn.write_inputs(str(d), spec)
        got = list(fmc_lib.System.load(str(d)).info().fugacity)
        o = oracle_lib.Oracle(str(d))
        ng = 1 if p2 is None else 2
        assert got[:ng] == [o.fugacity(g) for g in range(1, ng + 1)]
        if p2 is None:
            phi = got[0] / (p1 * 1e5)
            lo, hi = bounds.get(p1, (0.999, 1.0))
            assert lo < phi < hi, (p1, phi)
        else:
            tot = p1 + p2
            for g, p in ((0, p1), (1, p2)):
                phi = got[g] / ((p / tot) * p * 1e5)
                assert 0.995 < phi < 1.0, (g, phi)
    # without the directive the fugacity is the partial pressure
    spec = syn.small_test_spec(pressure_bar=10.0)
    d = tmp_path / "plain"
    syn.write_inputs(str(d), spec)
    assert fmc_lib.System.load(str(d)).info().fugacity[0] == 10.0e5


def test_reference_isotherm_inputs_load(fmc_lib, tmp_path):
    """The ten reference isotherm inputs load in the set-up as they are (all
    six moves, probability grids, ewald precision, CALF-20's parallelepiped
    cell) with the guests' partial pressures as fugacities."""
    import shutil
    from oracle.isotherm import GOLD, control_numbers
    base = os.path.join(GOLD, "calf20")
    for name in sorted(os.listdir(os.path.join(base, "isotherm"))):
        d = tmp_path / name
        d.mkdir()
        for f in ("CONFIG", "FIELD"):
            shutil.copy(os.path.join(base, f), d / f)
        ctl = os.path.join(base, "isotherm", name, "CONTROL")
        shutil.copy(ctl, d / "CONTROL")
        info = fmc_lib.System.load(str(d)).info()
        assert info.ntpguest == 2 and info.imcon == 3
        p, _, _ = control_numbers(ctl)
        assert abs(sum(info.fugacity[:2]) - p * 1e5) < 1e-6 * p * 1e5


UPLOAD_FIELDS = ("imcon", "cell", "engunit", "temp", "rcut", "alpha", "kmax", "newld", "epsq",
                 "overlap", "surftol", "eqsteps", "nwindsteps", "minchk", "laccsample", "ntpatm",
                 "mxegrd", "drewd", "dlrpot", "erc", "ntpvdw", "vvv", "ltpvdw", "prmvdw", "lstvdw",
                 "steadd", "maxmls", "numatoms", "nummols", "is_guest", "ltype", "charge", "mass",
                 "frozen", "fw_xyz", "ntpguest", "guest_tmpl", "fugacity", "delr", "disp_ratio",
                 "tran_ratio", "rota_ratio", "move_freq", "create")


def host_arrays(oracle_lib, d):
    """The start-up arrays of a host that read the inputs in `d` itself (the
    oracle plays that host), by fmc_system_desc field name."""
    o = oracle_lib.Oracle(d)
    return {k: o.array(k) for k in UPLOAD_FIELDS}


@pytest.mark.parametrize("which", ["synthetic", "calf20"])
def test_upload_system_matches_load(fmc_lib, oracle_lib, inputs_dir, which):
    """fmc_upload_system from a host's arrays gives the system
    fmc_system_load builds from the files (orthorhombic and parallelepiped
    cells)."""
    from conftest import CALF20
    d = CALF20 if which == "calf20" else inputs_dir(
        syn.small_test_spec(seed=4, kmax=6, pressure_bar=5.0, create=10), "upload")
    a = fmc_lib.System.load(d).info()
    b = fmc_lib.System.upload(host_arrays(oracle_lib, d)).info()
    for name, _ in a._fields_:
        va, vb = getattr(a, name), getattr(b, name)
        if hasattr(va, "__len__"):
            va, vb = list(va), list(vb)
        if name in ("mcsteps",):
            continue  # a run length the descriptor does not carry
        assert va == vb, (name, va, vb)


def test_upload_system_refuses_inconsistent_arrays(fmc_lib, oracle_lib, inputs_dir):
    from fastmc_gb300 import _lib as L
    d = inputs_dir(syn.small_test_spec(seed=4, kmax=6, pressure_bar=5.0), "upload_bad")
    arr = host_arrays(oracle_lib, d)
    bad = dict(arr, newld=arr["newld"] + 1)
    with pytest.raises(fmc_lib.FmcError) as e:
        fmc_lib.System.upload(bad)
    assert e.value.code == L.FMC_ERR_INPUT and "newld" in str(e.value)
    bad = dict(arr, lstvdw=np.full_like(arr["lstvdw"], 99))
    with pytest.raises(fmc_lib.FmcError) as e:
        fmc_lib.System.upload(bad)
    assert e.value.code == L.FMC_ERR_ARG
