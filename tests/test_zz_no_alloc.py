"""fmc_full_ewald_noalloc (the allocation-free full Ewald recomputation,
scratch in static device memory) against fmc_full_ewald, through the C ABI.

Both compute the reciprocal sum in FP64; they differ only in the order the
per-k energy terms are added, so results agree to REL relative and the
reset guest S(k) is the same.
"""
import ctypes as C
import json
import os

import numpy as np
import pytest

from conftest import CALF20, GOLDEN
from fastmc_gb300 import _lib as L
from fastmc_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

REL = 1e-10


def noalloc(plain):
    out = (C.c_double * 4)()
    rc = L.load().fmc_full_ewald_noalloc(plain._h, out)
    return rc, np.array(out[:])


def allocs():
    a, f = C.c_int64(), C.c_int64()
    L.check(L.load().fmc_alloc_count(C.byref(a), C.byref(f)))
    return a.value, f.value


def close(a, b):
    scale = np.maximum(np.maximum(np.abs(a), np.abs(b)), 1e-6)
    return np.all(np.abs(a - b) <= REL * scale)


def _populate(plain, n, seed, box):
    """Insert up to n CO2 at random non-overlapping positions."""
    rng = np.random.default_rng(seed)
    done = 0
    for _ in range(20000):
        ax = rng.normal(size=3)
        ax /= np.linalg.norm(ax)
        xyz = np.outer([0.0, 1.16, -1.16], ax) + rng.uniform(0, box, 3)
        r = plain.insertion(1, xyz)
        if plain.commit(0.0):
            done += 1
            if done == n:
                break
        else:
            assert r["overlap"]
    return done


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_noalloc_matches_full_ewald(fmc_lib, inputs_dir, precision):
    d = inputs_dir(syn.small_test_spec(seed=4, kmax=6, pressure_bar=5.0), "noalloc_small")
    sysm = fmc_lib.System.load(d)
    prec = fmc_lib.FMC_PREC_FP64 if precision == "fp64" else fmc_lib.FMC_PREC_FP32
    plain = fmc_lib.PlainEngine(sysm, prec, 64)
    assert _populate(plain, 12, seed=11, box=25.6) >= 8
    ref = plain.full_ewald()
    sk_ref = plain.sk()
    # two calls in a row: each agrees with the allocating entry point and
    # leaves the same guest S(k); neither allocates or frees device memory
    for _ in range(2):
        a0 = allocs()
        rc, out = noalloc(plain)
        assert rc == L.FMC_OK, L.last_error()
        assert allocs() == a0
        assert close(out, ref), (out, ref)
        sk = plain.sk()
        assert np.allclose(sk, sk_ref, rtol=0, atol=1e-12 * np.abs(sk_ref).max())
    # the allocating entry point, for contrast, is seen by the counter
    a0 = allocs()
    plain.full_ewald()
    assert allocs()[0] > a0[0]
    # and the engine keeps working from that state
    assert plain.deletion(1, 1)["overlap"] == 0


def test_noalloc_calf20_known_answer(fmc_lib):
    """The reference's own test system (no guests): the electrostatic
    energy it prints."""
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        g = json.load(f)
    plain = fmc_lib.PlainEngine(fmc_lib.System.load(CALF20), fmc_lib.FMC_PREC_FP64, 16)
    ref = plain.full_ewald()
    for _ in range(2):
        rc, out = noalloc(plain)
        assert rc == L.FMC_OK, L.last_error()
        assert abs(out[0] - g["calf20_electrostatic_energy_kcal"]) < g["tolerance_abs"]
        assert close(out, ref)


def test_noalloc_refuses_too_many_kvectors(fmc_lib, inputs_dir):
    """kmax 34 in a 25.6 A box gives more k-vectors than the static scratch
    covers: refused on the host before any launch."""
    d = inputs_dir(syn.small_test_spec(seed=4, kmax=34), "noalloc_kmax34")
    sysm = fmc_lib.System.load(d)
    assert sysm.info().newld > 65528
    plain = fmc_lib.PlainEngine(sysm, fmc_lib.FMC_PREC_FP64, 16)
    rc, _ = noalloc(plain)
    assert rc == L.FMC_ERR_ARG
    assert "65528" in L.last_error()
