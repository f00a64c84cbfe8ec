"""ctypes binding of include/fastmc_gb300.h.

The CUDA library is loaded from the package's _build directory; there is no
CPU fallback: if the library is missing, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libfastmc_gb300.so")

FMC_OK = 0
FMC_ERR_ARG = 1
FMC_ERR_CUDA = 2
FMC_ERR_CAPACITY = 3
FMC_ERR_INPUT = 4
FMC_ERR_DEVICE = 5
FMC_ERR_STATE = 6
FMC_ERR_NODEVICE = 7
FMC_PREC_FP64 = 0
FMC_PREC_FP32 = 1
MAX_MOLTYPES = 8
MAX_GUEST_TYPES = 4
MAX_SITES = 8

MOVE_NAMES = {1: "insert", 2: "delete", 3: "displace", 4: "translate", 5: "rotate", 6: "jump",
              7: "swap"}


class SystemInfo(C.Structure):
    _fields_ = [("imcon", C.c_int), ("maxmls", C.c_int), ("ntpguest", C.c_int),
                ("ntpatm", C.c_int), ("n_framework", C.c_int), ("kmax", C.c_int * 3),
                ("newld", C.c_int), ("mxegrd", C.c_int),
                ("guest_mol", C.c_int * MAX_GUEST_TYPES),
                ("guest_nsites", C.c_int * MAX_GUEST_TYPES),
                ("guest_insert", C.c_int * MAX_GUEST_TYPES),
                ("alpha", C.c_double), ("rcut", C.c_double), ("volm", C.c_double),
                ("engunit", C.c_double), ("temperature", C.c_double), ("sumchg", C.c_double),
                ("drewd", C.c_double), ("cell", C.c_double * 9),
                ("fugacity", C.c_double * MAX_GUEST_TYPES),
                ("ewald3en", C.c_double * MAX_GUEST_TYPES),
                ("mcsteps", C.c_int), ("eqsteps", C.c_int), ("nwindsteps", C.c_int),
                ("overlap", C.c_double)]


class SystemDesc(C.Structure):
    """fmc_system_desc: a host's start-up arrays (fmc_upload_system)."""
    _fields_ = [("imcon", C.c_int), ("cell", C.c_double * 9), ("engunit", C.c_double),
                ("temp", C.c_double), ("rcut", C.c_double), ("alpha", C.c_double),
                ("kmax", C.c_int * 3), ("newld", C.c_int), ("epsq", C.c_double),
                ("overlap", C.c_double), ("surftol", C.c_double), ("eqsteps", C.c_int),
                ("nwindsteps", C.c_int), ("minchk", C.c_int), ("laccsample", C.c_int),
                ("ntpatm", C.c_int), ("mxegrd", C.c_int), ("drewd", C.c_double),
                ("dlrpot", C.c_double), ("erc", C.POINTER(C.c_double)), ("ntpvdw", C.c_int),
                ("vvv", C.POINTER(C.c_double)), ("ltpvdw", C.POINTER(C.c_int)),
                ("prmvdw", C.POINTER(C.c_double)), ("lstvdw", C.POINTER(C.c_int)),
                ("steadd", C.POINTER(C.c_double)), ("maxmls", C.c_int),
                ("numatoms", C.POINTER(C.c_int)), ("nummols", C.POINTER(C.c_int)),
                ("is_guest", C.POINTER(C.c_int)), ("ltype", C.POINTER(C.c_int)),
                ("charge", C.POINTER(C.c_double)), ("mass", C.POINTER(C.c_double)),
                ("frozen", C.POINTER(C.c_int)), ("fw_xyz", C.POINTER(C.c_double)),
                ("ntpguest", C.c_int), ("guest_tmpl", C.POINTER(C.c_double)),
                ("fugacity", C.POINTER(C.c_double)), ("delr", C.POINTER(C.c_double)),
                ("disp_ratio", C.POINTER(C.c_double)), ("tran_ratio", C.POINTER(C.c_double)),
                ("rota_ratio", C.POINTER(C.c_double)), ("move_freq", C.POINTER(C.c_float)),
                ("create", C.POINTER(C.c_int))]


class MoveResult(C.Structure):
    _fields_ = [("estep", C.c_double), ("ewld1", C.c_double), ("ewld2", C.c_double),
                ("vdw", C.c_double), ("delrc", C.c_double),
                ("delE", C.c_double * MAX_MOLTYPES), ("overlap", C.c_int),
                ("surface", C.c_int), ("surface_old", C.c_int), ("status", C.c_int),
                ("newxyz", C.c_double * (3 * MAX_SITES))]


class SwapResult(C.Structure):
    _fields_ = [("estepi", C.c_double), ("estepj", C.c_double), ("testi", C.c_double),
                ("testj", C.c_double), ("overlap", C.c_int), ("pad", C.c_int),
                ("newxyz", C.c_double * (3 * MAX_SITES))]


class ChainSpec(C.Structure):
    _fields_ = [("system", C.c_int), ("pressure_pa", C.c_double), ("seed", C.c_int64),
                ("create_molecules", C.c_int)]


class ChainStats(C.Structure):
    _fields_ = [("moves", C.c_int64), ("evals", C.c_int64), ("overlap_exits", C.c_int64),
                ("attempts", C.c_int64 * 8), ("accepts", C.c_int64 * 8),
                ("nummols", C.c_int), ("status", C.c_int), ("energy", C.c_double),
                ("avg_n", C.c_double), ("avg_e", C.c_double), ("avg_en", C.c_double),
                ("avg_n2", C.c_double), ("avg_e2", C.c_double), ("avg_nf", C.c_double),
                ("qst", C.c_double), ("cv", C.c_double), ("prodcount", C.c_int64),
                ("windows", C.c_int64), ("device_ns", C.c_int64),
                ("guest_avg_n", C.c_double * MAX_GUEST_TYPES),
                ("guest_se_n", C.c_double * MAX_GUEST_TYPES),
                ("phase_cycles", C.c_int64 * 16)]


class MoveLog(C.Structure):
    _fields_ = [("move", C.c_int), ("iguest", C.c_int), ("choice", C.c_int),
                ("overlap", C.c_int), ("accepted", C.c_int), ("nmols_after", C.c_int),
                ("estep", C.c_double), ("rande", C.c_double), ("newxyz", C.c_double * 9)]


vp = C.c_void_p
pp = C.POINTER(C.c_void_p)
dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int)
i64p = C.POINTER(C.c_int64)

# name -> (restype, argtypes); the full exported C ABI
SIGNATURES = {
    "fmc_last_error": (C.c_int, [C.c_char_p, C.c_int]),
    "fmc_version": (C.c_char_p, []),
    "fmc_system_load": (C.c_int, [C.c_char_p, pp]),
    "fmc_upload_system": (C.c_int, [C.POINTER(SystemDesc), pp]),
    "fmc_system_free": (C.c_int, [vp]),
    "fmc_system_get_info": (C.c_int, [vp, C.POINTER(SystemInfo)]),
    "fmc_system_set_fugacity": (C.c_int, [vp, C.c_int, C.c_double]),
    "fmc_plain_create": (C.c_int, [vp, C.c_int, C.c_int, pp]),
    "fmc_plain_destroy": (C.c_int, [vp]),
    "fmc_full_ewald": (C.c_int, [vp, dp]),
    "fmc_full_ewald_noalloc": (C.c_int, [vp, dp]),
    "fmc_insertion": (C.c_int, [vp, C.c_int, dp, C.POINTER(MoveResult)]),
    "fmc_deletion": (C.c_int, [vp, C.c_int, C.c_int, C.POINTER(MoveResult)]),
    "fmc_displace": (C.c_int, [vp, C.c_int, C.c_int, dp, C.POINTER(MoveResult)]),
    "fmc_guest_energy": (C.c_int, [vp, C.c_int, C.c_int, C.POINTER(MoveResult)]),
    "fmc_metropolis_commit": (C.c_int, [vp, C.c_double, ip]),
    "fmc_commit": (C.c_int, [vp, C.c_int]),
    "fmc_swap": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, dp, C.POINTER(SwapResult)]),
    "fmc_swap_finish": (C.c_int, [vp, C.c_int]),
    "fmc_plain_get_nummols": (C.c_int, [vp, C.c_int, ip]),
    "fmc_plain_get_coords": (C.c_int, [vp, C.c_int, dp, C.c_int]),
    "fmc_plain_get_sk": (C.c_int, [vp, dp, C.c_int]),
    "fmc_plain_get_energy": (C.c_int, [vp, dp, C.c_int]),
    "fmc_batch_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.POINTER(ChainSpec),
                                   C.c_int, C.c_int, C.c_int, pp]),
    "fmc_batch_destroy": (C.c_int, [vp]),
    "fmc_batch_set_log": (C.c_int, [vp, C.c_int]),
    "fmc_batch_run": (C.c_int, [vp, C.c_int, C.POINTER(ChainStats)]),
    "fmc_batch_run_cycle": (C.c_int, [vp, C.c_int, dp, C.POINTER(ChainStats)]),
    "fmc_batch_get_stats": (C.c_int, [vp, C.POINTER(ChainStats)]),
    "fmc_batch_get_log": (C.c_int, [vp, C.c_int, C.POINTER(MoveLog), C.c_int, ip]),
    "fmc_batch_get_coords": (C.c_int, [vp, C.c_int, dp, C.c_int, ip]),
    "fmc_batch_get_coords_type": (C.c_int, [vp, C.c_int, C.c_int, dp, C.c_int, ip]),
    "fmc_batch_get_sk": (C.c_int, [vp, C.c_int, dp, C.c_int]),
    "fmc_batch_last_timing": (C.c_int, [vp, dp, i64p, i64p]),
    "fmc_batch_cycle_bytes": (C.c_int, [vp, i64p, i64p]),
    "fmc_batch_set_cluster": (C.c_int, [vp, ip, C.c_int]),
    "fmc_batch_set_speculation": (C.c_int, [vp, C.c_int]),
    "fmc_batch_write_revive": (C.c_int, [vp, C.c_int, C.c_char_p]),
    "fmc_batch_read_revive": (C.c_int, [vp, C.c_int, C.c_char_p]),
    "fmc_batch_get_cluster": (C.c_int, [vp, ip, C.c_int]),
    "fmc_batch_autotune": (C.c_int, [vp, C.c_int, ip, C.c_int]),
    "fmc_batch_save": (C.c_int, [vp, C.c_char_p]),
    "fmc_batch_load": (C.c_int, [vp, C.c_char_p]),
    "fmc_widom_grid": (C.c_int, [vp, C.c_int, C.c_int, ip, C.c_int, C.c_int64, dp, i64p, dp, ip,
                                 dp]),
    "fmc_widom_positions": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, dp, dp, ip]),
    "fmc_batch_prob_info": (C.c_int, [vp, C.c_int, ip, ip]),
    "fmc_batch_set_chain_cluster": (C.c_int, [vp, ip, C.c_int]),
    "fmc_adjoint_create": (C.c_int, [vp, C.POINTER(vp)]),
    "fmc_adjoint_info": (C.c_int, [vp, ip, ip, dp]),
    "fmc_adjoint_eval": (C.c_int, [vp, C.c_int, vp, dp, dp, vp, dp]),
    "fmc_adjoint_eval_batch": (C.c_int, [vp, C.c_int, ip, vp, dp, C.c_int, dp, vp, dp]),
    "fmc_adjoint_destroy": (C.c_int, [vp]),
    "fmc_batch_get_chain_cluster": (C.c_int, [vp, ip, C.c_int]),
    "fmc_batch_prob_grid": (C.c_int, [vp, C.c_int, C.c_int, dp, C.c_int64]),
    "fmc_alloc_count": (C.c_int, [i64p, i64p]),
    "fmc_measure_fp32_peak": (C.c_int, [dp]),
    "fmc_batch_snapshot": (C.c_int, [vp]),
    "fmc_batch_restore": (C.c_int, [vp]),
}

_lib = None


class FmcError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"fastmc_gb300 error {code}: {msg}")
        self.code = code


def load(path: str = LIB_PATH) -> C.CDLL:
    """Load the CUDA library and bind every entry point of the header."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FmcError(-1, f"CUDA library not built: {path} (run fastmc_gb300.build)")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error() -> str:
    buf = C.create_string_buffer(1024)
    load().fmc_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(code: int) -> None:
    if code != FMC_OK:
        raise FmcError(code, last_error())
