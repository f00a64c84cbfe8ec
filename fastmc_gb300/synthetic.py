"""Synthetic GCMC inputs in the reference's FIELD / CONFIG / CONTROL formats.

The benchmark configurations have no public dataset; these seeded inputs
stand in for them.  The unit cell is a 12.8 A cube with 192 framework atoms
(48 of each of 4 types) placed uniformly with a 1.8 A periodic minimum
separation.  Per type, epsilon ~ U(0.02, 0.10) kcal/mol and
sigma ~ U(2.5, 3.8) A, combined with Lorentz-Berthelot mixing and written
as explicit ``lj`` pair lines (vdw_terms.f:1-179 parses them).  Charges are
N(0, 0.4) e per atom, shifted to a net zero cell charge.  The unit cell is
tiled n x n x n into an orthorhombic (imcon=2) frozen framework.  The guest
is rigid 3-site CO2 (C +0.70 e, O -0.35 e, C-O 1.16 A; eps_C 0.054,
eps_O 0.157 kcal/mol; sigma_C 2.80, sigma_O 3.05 A).

File formats follow readinputs.f:11-307 (FIELD), readinputs.f:309-513
(CONFIG, levcfg 0, three 20-column coordinate fields) and
readinputs.f:515-944 (CONTROL).  Random numbers come from numpy's PCG64
with the stated seeds, so every file is reproducible.
"""
from __future__ import annotations

import dataclasses
import math
import os
from typing import List, Optional, Sequence

import numpy as np

UNIT_CELL = 12.8
ATOMS_PER_UNIT = 192
N_FW_TYPES = 4
MIN_SEP = 1.8
FW_NAMES = ["Fw1", "Fw2", "Fw3", "Fw4"]
CO2_SITES = [  # name, mass, charge, z offset along the molecular axis
    ("Cg", 12.0107, 0.70, 0.0),
    ("Og", 15.9994, -0.35, 1.16),
    ("Og", 15.9994, -0.35, -1.16),
]
GUEST_LJ = {"Cg": (0.054, 2.80), "Og": (0.157, 3.05)}
# optional second guest type: a two-site dipolar molecule (N2-like, 1.10 A)
GUEST2_SITES = [  # name, mass, charge, z offset
    ("Na", 14.0067, 0.20, 0.55),
    ("Nb", 14.0067, -0.20, -0.55),
]
GUEST2_LJ = {"Na": (0.072, 3.31), "Nb": (0.072, 3.31)}
# optional third guest type: a neutral three-site linear molecule
GUEST3_SITES = [  # name, mass, charge, z offset
    ("Ma", 15.9994, 0.25, 0.90),
    ("Mb", 12.0107, -0.50, 0.0),
    ("Mc", 15.9994, 0.25, -0.90),
]
GUEST3_LJ = {"Ma": (0.10, 3.00), "Mb": (0.06, 2.90), "Mc": (0.10, 3.00)}


@dataclasses.dataclass
class UnitCell:
    xyz: np.ndarray        # (192, 3) positions in [0, 12.8)
    types: np.ndarray      # (192,) 0..3
    charges: np.ndarray    # (192,)
    eps: np.ndarray        # (4,) kcal/mol
    sigma: np.ndarray      # (4,) A


def make_unit_cell(seed: int, natoms: int = ATOMS_PER_UNIT) -> UnitCell:
    """One 12.8 A unit cell: uniform positions with a 1.8 A periodic minimum
    separation (rejection sampling), natoms / 4 atoms of each of 4 types
    (192 for the benchmark frameworks; fewer gives an open framework for
    tests that need accepted moves)."""
    if natoms % N_FW_TYPES:
        raise ValueError("natoms must be a multiple of the 4 framework types")
    rng = np.random.Generator(np.random.PCG64(seed))
    pos = np.empty((natoms, 3))
    n = 0
    tries = 0
    while n < natoms:
        tries += 1
        if tries > 1_000_000:
            raise RuntimeError("could not place framework atoms")
        p = rng.uniform(0.0, UNIT_CELL, size=3)
        if n:
            d = pos[:n] - p
            d -= UNIT_CELL * np.round(d / UNIT_CELL)
            if np.min(np.einsum("ij,ij->i", d, d)) < MIN_SEP * MIN_SEP:
                continue
        pos[n] = p
        n += 1
    types = np.repeat(np.arange(N_FW_TYPES), natoms // N_FW_TYPES)
    rng.shuffle(types)
    eps = rng.uniform(0.02, 0.10, size=N_FW_TYPES)
    sigma = rng.uniform(2.5, 3.8, size=N_FW_TYPES)
    q = rng.normal(0.0, 0.4, size=natoms)
    q = q - q.mean()
    q = np.round(q, 10)
    q[-1] -= q.sum()  # exact zero in the written precision
    q = np.round(q, 10)
    return UnitCell(pos, types, q, eps, sigma)


@dataclasses.dataclass
class GcmcSpec:
    """One GCMC chain: framework tiling and run settings."""
    ntile: int = 2
    fw_seed: int = 1
    alpha: float = 0.26
    kmax: int = 7
    cutoff: float = 12.5
    delr: float = 0.5
    temperature: float = 293.0
    pressure_bar: float = 0.1
    steps: int = 100000
    equilibration: int = 0
    accepted_sampling: bool = False  # production statistics after accepted moves only
    fugacity: bool = False           # Peng-Robinson fugacities from the pressures
    create_molecules: int = 0
    move_mix: Sequence[tuple] = (("insert", 0.25), ("delete", 0.25),
                                 ("displace", 0.25), ("rotate", 0.25))
    overlap: Optional[float] = None
    title: str = "synthetic framework"
    # probability grids: one entry per grid, the guest sites binned into it
    # (0 = the centre of mass); grid spacing (A) and unit-cell factors
    probability: Optional[Sequence[Sequence[int]]] = None
    grid_spacing: Optional[float] = None
    grid_factor: Optional[Sequence[int]] = None
    # a second guest type (GUEST2_SITES) with its own pressure and count
    second_guest: bool = False
    pressure2_bar: float = 5.0
    create2: int = 0
    # a third guest type (GUEST3_SITES; needs the second)
    third_guest: bool = False
    pressure3_bar: float = 5.0
    create3: int = 0

    @property
    def box(self) -> float:
        return UNIT_CELL * self.ntile


def _lb(eps_i, sig_i, eps_j, sig_j):
    return math.sqrt(eps_i * eps_j), 0.5 * (sig_i + sig_j)


def field_text(spec: GcmcSpec, uc: UnitCell) -> str:
    if spec.third_guest and not spec.second_guest:
        raise ValueError("a third guest type needs the second")
    nmt = 2 + int(spec.second_guest) + int(spec.third_guest)
    lines = [spec.title, "UNITS   kcal", f"molecular types {nmt}"]
    lines.append("&guest CO2 rigid three site")
    lines.append("NUMMOLS 0")
    lines.append(f"ATOMS {len(CO2_SITES)}")
    for name, mass, chg, z in CO2_SITES:
        lines.append(f"{name:<8s}{mass:14.6f}{chg:14.6f}{0.0:14.6f}{0.0:14.6f}{z:14.6f}")
    lines.append("rigid 1")
    lines.append("3 1 2 3")
    lines.append("finish")
    if spec.second_guest:
        lines.append("&guest N2 rigid two site")
        lines.append("NUMMOLS 0")
        lines.append(f"ATOMS {len(GUEST2_SITES)}")
        for name, mass, chg, z in GUEST2_SITES:
            lines.append(f"{name:<8s}{mass:14.6f}{chg:14.6f}{0.0:14.6f}{0.0:14.6f}{z:14.6f}")
        lines.append("rigid 1")
        lines.append("2 1 2")
        lines.append("finish")
    if spec.third_guest:
        lines.append("&guest M3 rigid three site")
        lines.append("NUMMOLS 0")
        lines.append(f"ATOMS {len(GUEST3_SITES)}")
        for name, mass, chg, z in GUEST3_SITES:
            lines.append(f"{name:<8s}{mass:14.6f}{chg:14.6f}{0.0:14.6f}{0.0:14.6f}{z:14.6f}")
        lines.append("rigid 1")
        lines.append("3 1 2 3")
        lines.append("finish")
    lines.append("Framework")
    lines.append(f"NUMMOLS {spec.ntile ** 3}")
    lines.append(f"ATOMS {len(uc.types)}")
    for t, q in zip(uc.types, uc.charges):
        lines.append(f"{FW_NAMES[t]:<8s}{20.0:14.6f}{q:20.12f}      1      1")
    lines.append("finish")
    # van der Waals: every pair of the 6 unique names, Lorentz-Berthelot
    names = (["Cg", "Og"] + (["Na", "Nb"] if spec.second_guest else [])
             + (["Ma", "Mb", "Mc"] if spec.third_guest else []) + FW_NAMES)
    params = {"Cg": GUEST_LJ["Cg"], "Og": GUEST_LJ["Og"], **GUEST2_LJ, **GUEST3_LJ}
    for i, n in enumerate(FW_NAMES):
        params[n] = (float(uc.eps[i]), float(uc.sigma[i]))
    pairs = []
    for a in range(len(names)):
        for b in range(a, len(names)):
            pairs.append((names[a], names[b]))
    lines.append(f"VDW {len(pairs)}")
    for a, b in pairs:
        e, s = _lb(*params[a], *params[b])
        lines.append(f"{a:<8s}{b:<8s}lj {e:.12f} {s:.12f}")
    lines.append("close")
    return "\n".join(lines) + "\n"


def config_text(spec: GcmcSpec, uc: UnitCell) -> str:
    n = spec.ntile
    L = spec.box
    natoms = len(uc.types) * n ** 3
    out = [spec.title, f"{0:10d}{2:10d}{natoms:10d}"]
    out.append(f"{L:20.12f}{0.0:20.12f}{0.0:20.12f}")
    out.append(f"{0.0:20.12f}{L:20.12f}{0.0:20.12f}")
    out.append(f"{0.0:20.12f}{0.0:20.12f}{L:20.12f}")
    k = 0
    for ix in range(n):
        for iy in range(n):
            for iz in range(n):
                off = np.array([ix, iy, iz], dtype=float) * UNIT_CELL
                for a in range(len(uc.types)):
                    k += 1
                    p = uc.xyz[a] + off
                    out.append(f"{FW_NAMES[uc.types[a]]:<8s}{k:10d}")
                    out.append(f"{p[0]:20.12f}{p[1]:20.12f}{p[2]:20.12f}")
    return "\n".join(out) + "\n"


def control_text(spec: GcmcSpec) -> str:
    lines = ["GCMC synthetic run",
             f"temperature  {spec.temperature:.6f}",
             f"steps  {spec.steps}",
             f"equilibration  {spec.equilibration}",
             f"cutoff  {spec.cutoff:.6f} angstrom",
             f"delr  {spec.delr:.6f} angstrom",
             f"ewald sum {spec.alpha:.6f} {spec.kmax} {spec.kmax} {spec.kmax}"]
    if spec.grid_spacing is not None:
        lines.append(f"grid spacing {spec.grid_spacing:.6f}")
    if spec.grid_factor is not None:
        lines.append("grid factor " + " ".join(str(int(v)) for v in spec.grid_factor))
    if spec.overlap is not None:
        lines.append(f"overlap {spec.overlap:.6f}")
    if spec.accepted_sampling:
        lines.append("sampling accepted")
    if spec.fugacity:
        lines.append("fugacity")
    lines.append("&guest 1")
    lines.append(f"  pressure (bar) {spec.pressure_bar:.9f}")
    if spec.create_molecules:
        lines.append(f"  create molecules {spec.create_molecules}")
    if spec.probability:
        lines.append(f"  probability {len(spec.probability)}")
        for sites in spec.probability:
            if isinstance(sites, str):  # "energy": the energy probability grids
                lines.append("  " + sites)
            else:
                lines.append("  " + " ".join(str(int(v)) for v in [len(sites), *sites]))
    lines.append("&end")
    if spec.second_guest:
        lines.append("&guest 2")
        lines.append(f"  pressure (bar) {spec.pressure2_bar:.9f}")
        if spec.create2:
            lines.append(f"  create molecules {spec.create2}")
        lines.append("&end")
    if spec.third_guest:
        lines.append("&guest 3")
        lines.append(f"  pressure (bar) {spec.pressure3_bar:.9f}")
        if spec.create3:
            lines.append(f"  create molecules {spec.create3}")
        lines.append("&end")
    for name, f in spec.move_mix:
        lines.append(f"move {name} {f:.6f}")
    lines.append("finish")
    return "\n".join(lines) + "\n"


def write_inputs(directory: str, spec: GcmcSpec, uc: Optional[UnitCell] = None) -> str:
    """Write FIELD, CONFIG and CONTROL for `spec` into `directory`."""
    os.makedirs(directory, exist_ok=True)
    if uc is None:
        uc = make_unit_cell(spec.fw_seed)
    with open(os.path.join(directory, "FIELD"), "w") as f:
        f.write(field_text(spec, uc))
    with open(os.path.join(directory, "CONFIG"), "w") as f:
        f.write(config_text(spec, uc))
    with open(os.path.join(directory, "CONTROL"), "w") as f:
        f.write(control_text(spec))
    return directory


# ------------------------------------------------- the benchmark workloads
def single_chain_25A() -> GcmcSpec:
    """Plain FP64 single chain: 2x2x2 tiling (25.6 A, 1536 atoms),
    alpha 0.26, kmax 7, T 293 K, P 0.1 bar, equal move mix, seed 1."""
    return GcmcSpec(ntile=2, fw_seed=1, alpha=0.26, kmax=7, pressure_bar=0.1,
                    steps=100000, title="single chain 25.6A 1536 atoms")


def single_chain_51A() -> GcmcSpec:
    """Larger single chain: 4x4x4 tiling (51.2 A, 12288 atoms), 400 CO2
    pre-loaded at random non-overlapping positions, alpha 0.24, kmax 12."""
    return GcmcSpec(ntile=4, fw_seed=2, alpha=0.24, kmax=12, pressure_bar=0.1,
                    steps=1000000, create_molecules=400,
                    title="single chain 51.2A 12288 atoms")


ISOTHERM_TILES = (2, 3, 4, 5)
ISOTHERM_KMAX = (7, 10, 12, 18)
ISOTHERM_ALPHA = 0.24
ISOTHERM_PRESSURES = tuple(float(p) for p in np.logspace(np.log10(0.002), 0.0, 16))


def isotherm_chains() -> List[GcmcSpec]:
    """Batched isotherm: 16 pressures log-spaced 0.002-1.0 bar x 4 frameworks
    (edges 25.6/38.4/51.2/64.0 A, framework seeds 1..4, kmax 7/10/12/18).
    The 64.0 A box holds 24000 atoms at the tiled density (5^3 unit cells).
    Initial guest counts are uneven: chain c of a framework starts with
    floor(f_c * Nmax) guests, Nmax = 800 (L/64)^3 and
    f_c = ((7 c + 3 f) mod 16) / 15."""
    out = []
    for f, (nt, km) in enumerate(zip(ISOTHERM_TILES, ISOTHERM_KMAX)):
        L = UNIT_CELL * nt
        nmax = 800.0 * (L / 64.0) ** 3
        for c, p in enumerate(ISOTHERM_PRESSURES):
            frac = ((7 * c + 3 * f) % 16) / 15.0
            out.append(GcmcSpec(ntile=nt, fw_seed=f + 1, alpha=ISOTHERM_ALPHA,
                                kmax=km, pressure_bar=p, steps=1000000,
                                create_molecules=int(frac * nmax),
                                title=f"isotherm fw{f + 1} {L:.1f}A P={p:.4g}bar"))
    return out


def widom_102A() -> GcmcSpec:
    """Large framework: 8x8x8 tiling (102.4 A, 98304 atoms), 2000 CO2,
    cutoff 14 A, alpha 0.22, kmax 20."""
    return GcmcSpec(ntile=8, fw_seed=5, alpha=0.22, kmax=20, cutoff=14.0,
                    pressure_bar=0.1, steps=10000000, create_molecules=2000,
                    title="widom 102.4A 98304 atoms")


def small_test_spec(seed: int = 7, kmax: int = 5, ntile: int = 2,
                    pressure_bar: float = 10.0, create: int = 0,
                    cutoff: float = 12.5, move_mix: Optional[Sequence[tuple]] = None) -> GcmcSpec:
    """A small case for parity tests (seconds on the oracle)."""
    spec = GcmcSpec(ntile=ntile, fw_seed=seed, alpha=0.26, kmax=kmax,
                    pressure_bar=pressure_bar, steps=10000, create_molecules=create,
                    cutoff=cutoff, title=f"test seed{seed}")
    if move_mix is not None:
        spec.move_mix = tuple(move_mix)
    return spec
