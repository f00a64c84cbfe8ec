"""ctypes binding of the CPU oracle (oracle/fmc_oracle.h).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, to check results or as the timed CPU reference.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libfmc_oracle.so")


class MoveLog(C.Structure):
    _fields_ = [("move", C.c_int), ("iguest", C.c_int), ("choice", C.c_int),
                ("overlap", C.c_int), ("accepted", C.c_int), ("nmols_after", C.c_int),
                ("estep", C.c_double), ("rande", C.c_double), ("dele_other", C.c_double),
                ("newxyz", C.c_double * 9)]


def build() -> str:
    """Compile the oracle with its Makefile (g++ only)."""
    res = subprocess.run(["make", "-s", "-C", HERE], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + res.stdout + res.stderr)
    return LIB


_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        lib = C.CDLL(LIB)
        d, i, vp = C.c_double, C.c_int, C.c_void_p
        dp = C.POINTER(C.c_double)
        sig = {
            "orc_last_error": (C.c_char_p, []),
            "orc_create": (vp, [C.c_char_p]),
            "orc_destroy": (None, [vp]),
            "orc_setup_energies": (None, [vp, dp]),
            "orc_seed": (None, [vp, C.c_longlong]),
            "orc_ntpguest": (i, [vp]),
            "orc_maxmls": (i, [vp]),
            "orc_nummols": (i, [vp, i]),
            "orc_numatoms": (i, [vp, i]),
            "orc_locguest": (i, [vp, i]),
            "orc_newld": (i, [vp]),
            "orc_energy": (d, [vp, i]),
            "orc_get_coords": (i, [vp, i, dp, i]),
            "orc_get_sk": (i, [vp, dp, i]),
            "orc_run": (i, [vp, i, C.POINTER(MoveLog), i]),
            "orc_create_molecules": (i, [vp, i, i]),
            "orc_insertion_energy": (i, [vp, i, dp, dp]),
            "orc_deletion_energy": (i, [vp, i, i, dp]),
            "orc_displace_energy": (i, [vp, i, i, dp, dp]),
            "orc_apply_move": (i, [vp, i, i, i, dp, i]),
            "orc_stats": (None, [vp, i, dp]),
            "orc_prob_info": (i, [vp, C.POINTER(C.c_int)]),
            "orc_prob_grid": (i, [vp, i, dp, i]),
            "orc_store_energy": (i, [vp, i, dp, d]),
            "orc_prodcount": (C.c_longlong, [vp]),
            "orc_swap": (i, [vp, i, i, i, dp, dp, dp]),
            "orc_fugacity": (d, [vp, i]),
            "orc_duni_sequence": (None, [C.c_longlong, i, dp]),
            "orc_get_erc": (i, [vp, dp, i]),
            "orc_get_vvv": (i, [vp, i, dp, i]),
            "orc_set_prefilter": (None, [vp, i]),
            "orc_get_array": (i, [vp, C.c_char_p, dp, i]),
            "orc_save_state": (i, [vp]),
            "orc_restore_state": (i, [vp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


class Oracle:
    """One oracle simulation (reference start-up done on construction)."""

    def __init__(self, directory: str):
        lib = load()
        h = lib.orc_create(directory.encode())
        if not h:
            raise RuntimeError("oracle: " + lib.orc_last_error().decode())
        self._h = C.c_void_p(h)
        self.lib = lib

    def close(self):
        if self._h:
            self.lib.orc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc):
        if rc < 0:
            raise RuntimeError("oracle: " + self.lib.orc_last_error().decode())
        return rc

    def setup_energies(self):
        out = (C.c_double * 13)()
        self.lib.orc_setup_energies(self._h, out)
        keys = ["vdw", "ecoul", "dlpoly", "ewald1", "alpha", "kmax1", "kmax2", "kmax3",
                "newld", "volm", "engunit", "sumchg", "overlap"]
        return dict(zip(keys, out[:]))

    def seed(self, s: int):
        self.lib.orc_seed(self._h, s)

    def create_molecules(self, iguest: int, n: int) -> int:
        return self._ck(self.lib.orc_create_molecules(self._h, iguest, n))

    def set_prefilter(self, on: bool):
        self.lib.orc_set_prefilter(self._h, int(on))

    def array(self, name: str):
        """A set-up array of the upload descriptor by field name."""
        import numpy as np
        n = self.lib.orc_get_array(self._h, name.encode(), None, 0)
        if n < 0:
            raise KeyError(name)
        out = np.zeros(max(1, n))
        self._ck(self.lib.orc_get_array(self._h, name.encode(),
                                        out.ctypes.data_as(C.POINTER(C.c_double)), out.size))
        return out[:n]

    def save_state(self):
        self._ck(self.lib.orc_save_state(self._h))

    def restore_state(self):
        self._ck(self.lib.orc_restore_state(self._h))

    def run(self, nsteps: int):
        logs = (MoveLog * max(1, nsteps))()
        self._ck(self.lib.orc_run(self._h, nsteps, logs, nsteps))
        return list(logs[:nsteps])

    def run_nolog(self, nsteps: int) -> int:
        return self._ck(self.lib.orc_run(self._h, nsteps, None, 0))

    def nummols(self, mol: int) -> int:
        return self.lib.orc_nummols(self._h, mol)

    def locguest(self, ig: int) -> int:
        return self.lib.orc_locguest(self._h, ig)

    def energy(self, mol: int) -> float:
        return self.lib.orc_energy(self._h, mol)

    def maxmls(self) -> int:
        return self.lib.orc_maxmls(self._h)

    def newld(self) -> int:
        return self.lib.orc_newld(self._h)

    def coords(self, mol: int):
        import numpy as np
        n = self.lib.orc_nummols(self._h, mol) * self.lib.orc_numatoms(self._h, mol)
        out = np.zeros(max(1, 3 * n))
        self.lib.orc_get_coords(self._h, mol, out.ctypes.data_as(C.POINTER(C.c_double)), n)
        return out[:3 * n].reshape(n, 3)

    def sk(self):
        import numpy as np
        nk, nm = self.newld(), self.maxmls() + 1
        out = np.zeros(2 * nk * nm)
        self._ck(self.lib.orc_get_sk(self._h, out.ctypes.data_as(C.POINTER(C.c_double)), out.size))
        return out.reshape(nk, nm, 2)

    def _energy_out(self):
        return (C.c_double * (7 + self.maxmls()))()

    @staticmethod
    def _unpack(o, maxmls):
        return {"estep": o[0], "ewld1": o[1], "ewld2": o[2], "vdw": o[3], "delrc": o[4],
                "overlap": bool(o[5]), "surface": bool(o[6]), "delE": list(o[7:7 + maxmls])}

    def insertion_energy(self, iguest: int, xyz):
        import numpy as np
        a = np.ascontiguousarray(np.asarray(xyz, dtype=np.float64).reshape(-1))
        o = self._energy_out()
        self._ck(self.lib.orc_insertion_energy(self._h, iguest, a.ctypes.data_as(C.POINTER(C.c_double)), o))
        return self._unpack(o, self.maxmls())

    def deletion_energy(self, iguest: int, choice: int):
        o = self._energy_out()
        self._ck(self.lib.orc_deletion_energy(self._h, iguest, choice, o))
        return self._unpack(o, self.maxmls())

    def displace_energy(self, iguest: int, choice: int, abcq):
        import numpy as np
        a = np.ascontiguousarray(np.asarray(abcq, dtype=np.float64))
        o = self._energy_out()
        self._ck(self.lib.orc_displace_energy(self._h, iguest, choice, a.ctypes.data_as(C.POINTER(C.c_double)), o))
        return self._unpack(o, self.maxmls())

    def apply_move(self, kind: int, iguest: int, choice: int, params, accepted: bool):
        import numpy as np
        a = np.ascontiguousarray(np.asarray(params if params is not None else [0.0] * 9,
                                            dtype=np.float64).reshape(-1))
        self._ck(self.lib.orc_apply_move(self._h, kind, iguest, choice,
                                         a.ctypes.data_as(C.POINTER(C.c_double)), int(accepted)))

    def prob_info(self):
        """(ngrida, ngridb, ngridc, number of probability subgrids)."""
        out = (C.c_int * 4)()
        self.lib.orc_prob_info(self._h, out)
        return tuple(out)

    def prob_grid(self, sub: int):
        """Probability subgrid `sub` (1-based) as an (na, nb, nc) array."""
        import numpy as np
        na, nb, nc, _ = self.prob_info()
        out = np.zeros(na * nb * nc)
        self._ck(self.lib.orc_prob_grid(self._h, sub, out.ctypes.data_as(C.POINTER(C.c_double)), out.size))
        return out.reshape(na, nb, nc)

    def store_energy(self, iguest: int, xyz, energy: float) -> None:
        """storeenprob of given site coordinates and energy (a Widom trial)."""
        import numpy as np
        a = np.ascontiguousarray(np.asarray(xyz, dtype=np.float64).reshape(-1))
        self._ck(self.lib.orc_store_energy(self._h, iguest, a.ctypes.data_as(C.POINTER(C.c_double)),
                                           float(energy)))

    def fugacity(self, iguest: int) -> float:
        """gstfuga(iguest) in Pa."""
        return self.lib.orc_fugacity(self._h, iguest)

    def prodcount(self) -> int:
        return self.lib.orc_prodcount(self._h)

    def swap(self, iguest: int, choice: int, jguest: int, q, rande):
        """One swap with its draws given: (estepi, estepj, overlap, accepted)."""
        qa = (C.c_double * 4)(*[float(v) for v in q])
        ra = (C.c_double * 2)(*[float(v) for v in rande])
        out = (C.c_double * 4)()
        self._ck(self.lib.orc_swap(self._h, iguest, choice, jguest, qa, ra, out))
        return out[0], out[1], bool(out[2]), bool(out[3])

    def stats(self, iguest: int = 1):
        out = (C.c_double * 30)()
        self.lib.orc_stats(self._h, iguest, out)
        return list(out[:])


def duni_sequence(seed: int, n: int):
    import numpy as np
    out = np.zeros(n)
    load().orc_duni_sequence(seed, n, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out
