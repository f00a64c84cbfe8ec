"""Build the CUDA library (sm_103a) in-tree.

    python -m fastmc_gb300.build

produces fastmc_gb300/_build/libfastmc_gb300.so.  Each translation unit is
compiled by its own nvcc process (in parallel), then linked.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libfastmc_gb300.so")

GENCODE = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = [GENCODE, "-std=c++17", "-O3", "-lineinfo", "-diag-suppress", "1444",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-Xcompiler", "-Wno-deprecated-declarations"]
SOURCES = ["chain_f32_g1.cu", "chain_f32_g4.cu", "chain_f64.cu", "engine.cu", "host_setup.cpp",
           "adjoint.cu"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build")
    return path


def _flags():
    """FMC_PHASE_TIMERS=1 in the environment builds the per-phase move-loop
    clocks in (fmc_chain_stats.phase_cycles)."""
    extra = ["-DFMC_PHASE_TIMERS"] if os.environ.get("FMC_PHASE_TIMERS") == "1" else []
    return NVCC_FLAGS + extra


def _compile(src: str) -> str:
    obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
    cmd = [nvcc(), *_flags(), "-c", os.path.join(CSRC, src), "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    return obj


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "fastmc_gb300.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _obj_stale(src: str) -> bool:
    """An object needs compiling when it is missing or older than its
    source or any header (every source includes the headers)."""
    obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [os.path.join(CSRC, src), os.path.join(HERE, "..", "include", "fastmc_gb300.h"),
            os.path.abspath(__file__)]
    deps += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and not _stale():
        return LIB
    todo = [s for s in SOURCES if force or _obj_stale(s)]
    with cf.ThreadPoolExecutor(max_workers=max(1, len(todo))) as ex:
        list(ex.map(_compile, todo))
    objs = [os.path.join(OUT_DIR, os.path.basename(s) + ".o") for s in SOURCES]
    cmd = [nvcc(), GENCODE, "-shared", "-o", LIB, *objs, "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
