"""Host side of the swap binding (PlainEngine.swap) against a stand-in for
the two C entry points, no GPU: the second Metropolis number is taken only
when the first passes testi (gcmc.f:2404-2410), an overlapping swap takes
none, and fmc_swap_finish always follows with the decision."""
import ctypes as C

import pytest

from fastmc_gb300 import _lib as L
from fastmc_gb300 import api


class _FakeLib:
    def __init__(self, overlap, testi, testj):
        self.res = (overlap, testi, testj)
        self.finished = []

    def fmc_swap(self, h, iguest, choice, jguest, q, res):
        r = res  # byref is the identity here
        r.estepi, r.estepj = -1.5, 2.5
        r.overlap, r.testi, r.testj = self.res
        return L.FMC_OK

    def fmc_swap_finish(self, h, accepted):
        self.finished.append(accepted)
        return L.FMC_OK


def _engine():
    e = api.PlainEngine.__new__(api.PlainEngine)
    e._h = None

    class _Info:
        guest_nsites = (3, 2)
    e._info = _Info()
    return e


@pytest.mark.parametrize("overlap,testi,testj,draws,taken,accepted", [
    (1, 0.0, 0.0, [0.1, 0.1], 0, False),     # overlap: no number drawn
    (0, 0.5, 0.9, [0.7, 0.1], 1, False),     # first test fails: one number
    (0, 0.5, 0.9, [0.2, 0.95], 2, False),    # second test fails: two numbers
    (0, 0.5, 0.9, [0.2, 0.3], 2, True),      # both pass
])
def test_swap_draws_like_the_reference(monkeypatch, overlap, testi, testj, draws, taken, accepted):
    fake = _FakeLib(overlap, testi, testj)
    monkeypatch.setattr(L, "load", lambda *a, **k: fake)
    monkeypatch.setattr(C, "byref", lambda x: x)
    it = iter(draws)
    used = []

    def rande():
        v = next(it)
        used.append(v)
        return v
    r = _engine().swap(1, 1, 2, [1.0, 0.0, 0.0, 0.0], rande)
    assert len(used) == taken and r["accepted"] == accepted
    assert fake.finished == [int(accepted)]
    assert (r["estepi"], r["estepj"]) == (-1.5, 2.5) and r["newxyz"].shape == (2, 3)


def test_swap_finishes_when_the_draw_raises(monkeypatch):
    fake = _FakeLib(0, 0.5, 0.9)
    monkeypatch.setattr(L, "load", lambda *a, **k: fake)
    monkeypatch.setattr(C, "byref", lambda x: x)

    def boom():
        raise RuntimeError("generator failed")
    with pytest.raises(RuntimeError):
        _engine().swap(1, 1, 2, [1.0, 0.0, 0.0, 0.0], boom)
    assert fake.finished == [0]  # rolled back
