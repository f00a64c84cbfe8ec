"""Python API over the C ABI (include/fastmc_gb300.h).

    sys = System.load("inputs/")            # FIELD, CONFIG, CONTROL
    plain = PlainEngine(sys)                # per-move drop-in path
    r = plain.insertion(1, xyz)             # insertion (mc_moves.f:150)
    acc = plain.commit(rande)               # energy_eval + accept_move

    batch = Batch([sys], chains)            # device-resident chains
    stats = batch.run(256)                  # 256 main-loop iterations

Every call goes to the CUDA library; a missing library raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Callable, List, Optional, Sequence

import numpy as np

from . import _lib as L


class System:
    """Host-side inputs and tables of one framework (the reference start-up)."""

    def __init__(self, handle: int):
        self._h = C.c_void_p(handle)

    @classmethod
    def load(cls, directory: str) -> "System":
        lib = L.load()
        h = C.c_void_p()
        L.check(lib.fmc_system_load(directory.encode(), C.byref(h)))
        return cls(h.value)

    # fields of fmc_system_desc by kind, for System.upload
    _DESC_INT = ("imcon", "newld", "eqsteps", "nwindsteps", "minchk", "laccsample", "ntpatm",
                 "mxegrd", "ntpvdw", "maxmls", "ntpguest")
    _DESC_DBL = ("engunit", "temp", "rcut", "alpha", "epsq", "overlap", "surftol", "drewd", "dlrpot")
    _DESC_IARR = ("ltpvdw", "lstvdw", "numatoms", "nummols", "is_guest", "ltype", "frozen", "create")
    _DESC_DARR = ("erc", "vvv", "prmvdw", "steadd", "charge", "mass", "fw_xyz", "guest_tmpl",
                  "fugacity", "delr", "disp_ratio", "tran_ratio", "rota_ratio")

    @classmethod
    def upload(cls, arrays: dict) -> "System":
        """fmc_upload_system: the system from a host's start-up arrays,
        given by the field names of fmc_system_desc (scalars, "cell" with 9
        values, "kmax" with 3, arrays as sequences; "create" may be left
        out)."""
        d = L.SystemDesc()
        keep = []
        for k in cls._DESC_INT:
            setattr(d, k, int(np.asarray(arrays[k]).reshape(-1)[0]))
        for k in cls._DESC_DBL:
            setattr(d, k, float(np.asarray(arrays[k]).reshape(-1)[0]))
        d.cell = (C.c_double * 9)(*[float(v) for v in arrays["cell"]])
        d.kmax = (C.c_int * 3)(*[int(v) for v in arrays["kmax"]])
        for k in cls._DESC_IARR:
            if k not in arrays:
                continue
            a = np.ascontiguousarray(np.asarray(arrays[k]).astype(np.int32))
            keep.append(a)
            setattr(d, k, a.ctypes.data_as(L.ip))
        for k in cls._DESC_DARR:
            a = np.ascontiguousarray(np.asarray(arrays[k], dtype=np.float64))
            keep.append(a)
            setattr(d, k, a.ctypes.data_as(L.dp))
        mf = np.ascontiguousarray(np.asarray(arrays["move_freq"], dtype=np.float32))
        keep.append(mf)
        d.move_freq = mf.ctypes.data_as(C.POINTER(C.c_float))
        h = C.c_void_p()
        L.check(L.load().fmc_upload_system(C.byref(d), C.byref(h)))
        return cls(h.value)

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def info(self) -> L.SystemInfo:
        inf = L.SystemInfo()
        L.check(L.load().fmc_system_get_info(self._h, C.byref(inf)))
        return inf

    def set_fugacity(self, iguest: int, pascal: float) -> None:
        L.check(L.load().fmc_system_set_fugacity(self._h, iguest, pascal))

    def close(self) -> None:
        if self._h and self._h.value:
            L.load().fmc_system_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _result_dict(r: L.MoveResult, maxmls: int, ns: int) -> dict:
    return {
        "estep": r.estep, "ewld1": r.ewld1, "ewld2": r.ewld2, "vdw": r.vdw,
        "delrc": r.delrc, "delE": np.array(r.delE[:maxmls]), "overlap": bool(r.overlap),
        "surface": bool(r.surface), "surface_old": bool(r.surface_old), "status": r.status,
        "newxyz": np.array(r.newxyz[:3 * ns]).reshape(ns, 3),
    }


class PlainEngine:
    """Per-move drop-in: device mirror of one chain driven by the host."""

    def __init__(self, system: System, precision: int = L.FMC_PREC_FP64,
                 guest_capacity: int = 1024):
        self.system = system
        self._info = system.info()
        h = C.c_void_p()
        L.check(L.load().fmc_plain_create(system.handle, precision, guest_capacity, C.byref(h)))
        self._h = h

    def _ns(self, iguest: int) -> int:
        return self._info.guest_nsites[iguest - 1]

    def full_ewald(self) -> np.ndarray:
        out = (C.c_double * 4)()
        L.check(L.load().fmc_full_ewald(self._h, out))
        return np.array(out[:])

    def insertion(self, iguest: int, xyz) -> dict:
        a = np.ascontiguousarray(np.asarray(xyz, dtype=np.float64).reshape(-1))
        r = L.MoveResult()
        L.check(L.load().fmc_insertion(self._h, iguest, a.ctypes.data_as(L.dp), C.byref(r)))
        return _result_dict(r, self._info.maxmls, self._ns(iguest))

    def deletion(self, iguest: int, choice: int) -> dict:
        r = L.MoveResult()
        L.check(L.load().fmc_deletion(self._h, iguest, choice, C.byref(r)))
        return _result_dict(r, self._info.maxmls, self._ns(iguest))

    def guest_energy(self, iguest: int, choice: int) -> dict:
        r = L.MoveResult()
        L.check(L.load().fmc_guest_energy(self._h, iguest, choice, C.byref(r)))
        return _result_dict(r, self._info.maxmls, self._ns(iguest))

    def displace(self, iguest: int, choice: int, abcq: Sequence[float]) -> dict:
        a = np.ascontiguousarray(np.asarray(abcq, dtype=np.float64))
        r = L.MoveResult()
        L.check(L.load().fmc_displace(self._h, iguest, choice, a.ctypes.data_as(L.dp), C.byref(r)))
        return _result_dict(r, self._info.maxmls, self._ns(iguest))

    def commit(self, rande: float) -> bool:
        """energy_eval with the host's uniform number, then the commit."""
        acc = C.c_int()
        L.check(L.load().fmc_metropolis_commit(self._h, rande, C.byref(acc)))
        return bool(acc.value)

    def commit_decided(self, accepted: bool) -> None:
        """The commit of the last evaluated move with the caller's decision."""
        L.check(L.load().fmc_commit(self._h, int(accepted)))

    def swap(self, iguest: int, choice: int, jguest: int, q: Sequence[float],
             rande: Callable[[], float]) -> dict:
        """mc_swap: molecule `choice` of iguest replaced by a molecule of
        jguest at its centre of mass rotated by q, decided as the reference
        decides (gcmc.f:2371-2411) with numbers taken from `rande()` only
        when the reference draws them; rolled back unless accepted."""
        qa = np.ascontiguousarray(np.asarray(q, dtype=np.float64))
        if qa.size != 4:
            raise ValueError("q has 4 components")
        r = L.SwapResult()
        L.check(L.load().fmc_swap(self._h, iguest, choice, jguest, qa.ctypes.data_as(L.dp), C.byref(r)))
        accepted = False
        try:
            if not r.overlap and rande() < r.testi:
                accepted = rande() < r.testj
        finally:
            L.check(L.load().fmc_swap_finish(self._h, int(accepted)))
        nj = self._ns(jguest)
        return {"estepi": r.estepi, "estepj": r.estepj, "overlap": bool(r.overlap),
                "accepted": accepted, "testi": r.testi, "testj": r.testj,
                "newxyz": np.array(r.newxyz[:3 * nj]).reshape(nj, 3)}

    def nummols(self, iguest: int = 1) -> int:
        n = C.c_int()
        L.check(L.load().fmc_plain_get_nummols(self._h, iguest, C.byref(n)))
        return n.value

    def coords(self, iguest: int = 1) -> np.ndarray:
        n = self.nummols(iguest)
        ns = self._ns(iguest)
        out = np.zeros(max(1, 3 * ns * n))
        L.check(L.load().fmc_plain_get_coords(self._h, iguest, out.ctypes.data_as(L.dp), out.size))
        return out[:3 * ns * n].reshape(n * ns, 3)

    def sk(self) -> np.ndarray:
        nk, nm = self._info.newld, self._info.maxmls + 1
        out = np.zeros(2 * nk * nm)
        L.check(L.load().fmc_plain_get_sk(self._h, out.ctypes.data_as(L.dp), out.size))
        return out.reshape(nk, nm, 2)

    def energy(self) -> np.ndarray:
        out = np.zeros(self._info.maxmls)
        L.check(L.load().fmc_plain_get_energy(self._h, out.ctypes.data_as(L.dp), out.size))
        return out

    def close(self) -> None:
        if self._h and self._h.value:
            L.load().fmc_plain_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Device-resident GCMC chains over one or more systems."""

    def __init__(self, systems: List[System], chains: Sequence[dict],
                 precision: int = L.FMC_PREC_FP32, guest_capacity: int = 1024):
        self.systems = systems
        arr = (C.c_void_p * len(systems))(*[s.handle.value for s in systems])
        specs = (L.ChainSpec * len(chains))()
        for i, c in enumerate(chains):
            specs[i].system = int(c.get("system", 0))
            specs[i].pressure_pa = float(c.get("pressure_pa", -1.0))
            specs[i].seed = int(c.get("seed", i + 1))
            specs[i].create_molecules = int(c.get("create_molecules", -1))
        h = C.c_void_p()
        L.check(L.load().fmc_batch_create(arr, len(systems), specs, len(chains), precision,
                                          guest_capacity, C.byref(h)))
        self._h = h
        self.nchains = len(chains)
        self._nsys = len(systems)
        self._sys_of = [int(c.get("system", 0)) for c in chains]

    def set_log(self, cap: int) -> None:
        L.check(L.load().fmc_batch_set_log(self._h, cap))

    def run(self, nmoves: int, fugacity: Optional[np.ndarray] = None):
        st = (L.ChainStats * self.nchains)()
        if fugacity is not None:
            f = np.ascontiguousarray(np.asarray(fugacity, dtype=np.float64))
            L.check(L.load().fmc_batch_run_cycle(self._h, nmoves, f.ctypes.data_as(L.dp), st))
        else:
            L.check(L.load().fmc_batch_run(self._h, nmoves, st))
        return st

    def stats(self):
        st = (L.ChainStats * self.nchains)()
        L.check(L.load().fmc_batch_get_stats(self._h, st))
        return st

    def log(self, chain: int, cap: int):
        buf = (L.MoveLog * max(1, cap))()
        n = C.c_int()
        L.check(L.load().fmc_batch_get_log(self._h, chain, buf, cap, C.byref(n)))
        return list(buf[:n.value])

    def coords(self, chain: int, cap: int = 1 << 16) -> np.ndarray:
        out = np.zeros(cap)
        n = C.c_int()
        L.check(L.load().fmc_batch_get_coords(self._h, chain, out.ctypes.data_as(L.dp), cap, C.byref(n)))
        return out, n.value

    def sk(self, chain: int, nk: int, maxmls: int) -> np.ndarray:
        out = np.zeros(2 * nk * (maxmls + 1))
        L.check(L.load().fmc_batch_get_sk(self._h, chain, out.ctypes.data_as(L.dp), out.size))
        return out.reshape(nk, maxmls + 1, 2)

    def write_revive(self, chain: int, directory: str):
        """The reference's REVIVE and REVCON for one chain, into directory."""
        L.check(L.load().fmc_batch_write_revive(self._h, chain, directory.encode()))

    def read_revive(self, chain: int, directory: str):
        """Restart one chain from directory/REVIVE as the reference does."""
        L.check(L.load().fmc_batch_read_revive(self._h, chain, directory.encode()))

    def set_speculation(self, kmax: int):
        """Speculative proposals per round at most (2..8; 0 or 1: off)."""
        L.check(L.load().fmc_batch_set_speculation(self._h, int(kmax)))

    def set_cluster(self, sizes):
        """CTAs per chain for the chains of each system (1..8)."""
        a = (C.c_int * len(sizes))(*[int(v) for v in sizes])
        L.check(L.load().fmc_batch_set_cluster(self._h, a, len(sizes)))

    def cluster(self):
        n = self._nsys
        a = (C.c_int * n)()
        L.check(L.load().fmc_batch_get_cluster(self._h, a, n))
        return list(a)

    def autotune(self, nmoves: int = 256):
        """Pick per-system cluster sizes by timed trial cycles (the chains'
        state is left unchanged); returns the sizes."""
        n = self._nsys
        a = (C.c_int * n)()
        L.check(L.load().fmc_batch_autotune(self._h, nmoves, a, n))
        return list(a)

    def snapshot(self) -> None:
        """Keep a device copy of every chain's state (fmc_batch_snapshot)."""
        L.check(L.load().fmc_batch_snapshot(self._h))

    def restore(self) -> None:
        """Put the last snapshot back (fmc_batch_restore)."""
        L.check(L.load().fmc_batch_restore(self._h))

    def save(self, path: str) -> None:
        """Checkpoint every chain's device state for an exact resume."""
        L.check(L.load().fmc_batch_save(self._h, os.fsencode(path)))

    def load(self, path: str) -> None:
        """Resume from a checkpoint of a batch built the same way."""
        L.check(L.load().fmc_batch_load(self._h, os.fsencode(path)))

    def widom_grid(self, chain: int, ngrid, nstep: int, seed: int = 1, iguest: int = 1,
                   details: bool = False):
        """Widom test insertions on a grid (widom_grid): returns
        (henry, non_overlapping, total) and, with details, per-trial
        estep, overlap flags and site coordinates."""
        g = (C.c_int * 3)(*[int(v) for v in ngrid])
        h = C.c_double()
        cnt = (C.c_int64 * 2)()
        nt = int(ngrid[0]) * int(ngrid[1]) * int(ngrid[2]) * int(nstep)
        ns = self.systems[self._sys_of[chain]].info().guest_nsites[iguest - 1]
        est = np.zeros(nt) if details else None
        ovl = np.zeros(nt, dtype=np.int32) if details else None
        xyz = np.zeros(nt * ns * 3) if details else None
        L.check(L.load().fmc_widom_grid(
            self._h, chain, iguest, g, nstep, seed, C.byref(h), cnt,
            est.ctypes.data_as(L.dp) if details else None,
            ovl.ctypes.data_as(L.ip) if details else None,
            xyz.ctypes.data_as(L.dp) if details else None))
        out = (h.value, cnt[0], cnt[1])
        if details:
            return out, est, ovl, xyz.reshape(nt, ns, 3)
        return out

    def widom_positions(self, chain: int, xyz, iguest: int = 1):
        """Test-insertion energies (kcal/mol) and overlap flags at given site
        coordinates, shape (npos, natms, 3)."""
        a = np.ascontiguousarray(np.asarray(xyz, dtype=np.float64))
        npos = a.shape[0]
        est = np.zeros(npos)
        ovl = np.zeros(npos, dtype=np.int32)
        L.check(L.load().fmc_widom_positions(self._h, chain, iguest, npos, a.ctypes.data_as(L.dp),
                                             est.ctypes.data_as(L.dp), ovl.ctypes.data_as(L.ip)))
        return est, ovl

    def set_chain_cluster(self, sizes) -> None:
        """CTAs per chain (1..8), one entry per chain."""
        a = (C.c_int * len(sizes))(*[int(v) for v in sizes])
        L.check(L.load().fmc_batch_set_chain_cluster(self._h, a, len(sizes)))

    def chain_cluster(self):
        n = self.nchains
        a = (C.c_int * n)()
        L.check(L.load().fmc_batch_get_chain_cluster(self._h, a, n))
        return list(a)

    def prob_info(self, chain: int):
        """((na, nb, nc) voxels of the unit cell, number of probability grids)."""
        ng = (C.c_int * 3)()
        n = C.c_int()
        L.check(L.load().fmc_batch_prob_info(self._h, chain, ng, C.byref(n)))
        return tuple(ng), n.value

    def prob_grid(self, chain: int):
        """The chain's probability grids, shape (grids, na, nb, nc): sums of
        the equitable_bin weights over the production moves so far."""
        (na, nb, nc), n = self.prob_info(chain)
        out = np.zeros((n, na, nb, nc))
        for k in range(n):
            g = out[k]
            L.check(L.load().fmc_batch_prob_grid(self._h, chain, k, g.ctypes.data_as(L.dp), g.size))
        return out

    def cycle_bytes(self):
        """(host->device, device->host) bytes of one run() call with a
        fugacity array."""
        h, d = C.c_int64(), C.c_int64()
        L.check(L.load().fmc_batch_cycle_bytes(self._h, C.byref(h), C.byref(d)))
        return h.value, d.value

    def last_timing(self):
        ms = C.c_double()
        ev = C.c_int64()
        mv = C.c_int64()
        L.check(L.load().fmc_batch_last_timing(self._h, C.byref(ms), C.byref(ev), C.byref(mv)))
        return ms.value, ev.value, mv.value

    def close(self) -> None:
        if self._h and self._h.value:
            L.load().fmc_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
