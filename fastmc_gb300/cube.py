"""Cube files of probability grids, in the layout of the reference's
writeprob (utility_pack.f:768-871): two title lines, the atom count and
origin, the three voxel vectors of the unit cell in bohr, the framework
atoms, then grid / voxel volume / production moves, six values per line
and a line break at the end of every c row.

The reference maps framework masses to atomic numbers with its own table;
here the caller passes the atomic numbers with the coordinates.
"""
from __future__ import annotations

from typing import Iterable, Sequence, Tuple

import numpy as np

ANGS2BOHR = 1.889725989  # utility_pack.f:100


def fortran_e15_6(v: float) -> str:
    """A value as Fortran's E15.6 edit descriptor writes it (0.ddddddE+xx)."""
    if v == 0.0:
        return "0.000000E+00".rjust(15)
    s = f"{abs(v):.5e}"  # d.ddddde+xx: six significant digits
    digits = s[0] + s[2:7]
    exp = int(s[8:]) + 1
    sign = "-" if v < 0 else ""
    return f"{sign}0.{digits}E{exp:+03d}".rjust(15)


def voxel_volume(gcell: Sequence[float], na: int, nb: int, nc: int) -> float:
    """writeprob's voxel volume from the unit cell rows (any length unit)."""
    c = gcell
    return ((c[1] * c[5] - c[2] * c[4]) / (na * nb) * c[6] / nc +
            (c[2] * c[3] - c[0] * c[5]) / (na * nb) * c[7] / nc +
            (c[0] * c[4] - c[1] * c[3]) / (na * nb) * c[8] / nc)


def write_prob_cube(path: str, grid: np.ndarray, prodcount: int, ucell: Sequence[float],
                    atoms: Iterable[Tuple[int, float, float, float]] = ()) -> None:
    """Write one probability grid (na, nb, nc) accumulated over `prodcount`
    production moves.  ucell: the unit (folding) cell, rows a, b, c in A;
    atoms: (atomic number, x, y, z in A) of the framework atoms to list."""
    g = np.asarray(grid, dtype=np.float64)
    na, nb, nc = g.shape
    gcell = [v * ANGS2BOHR for v in ucell]
    vol = voxel_volume(gcell, na, nb, nc)
    atoms = list(atoms)
    out = ["probability cube file", "outer loop a, middle loop b, inner loop c",
           f"{len(atoms):6d}{0.0:12.6f}{0.0:12.6f}{0.0:12.6f}"]
    for n, row in zip((na, nb, nc), (gcell[0:3], gcell[3:6], gcell[6:9])):
        out.append(f"{n:6d}" + "".join(f"{v / n:12.6f}" for v in row))
    for z, x, y, w in atoms:
        out.append(f"{int(z):6d}{0.0:12.6f}{x * ANGS2BOHR:12.6f}{y * ANGS2BOHR:12.6f}{w * ANGS2BOHR:12.6f}")
    line, ip = [], 0
    flat = g.reshape(-1) / vol / float(prodcount)
    for j, v in enumerate(flat, start=1):
        ip += 1
        line.append(fortran_e15_6(float(v)))
        if j % nc == 0 or ip == 6:
            out.append("".join(line))
            line, ip = [], 0
    if line:
        out.append("".join(line))
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")


def write_energy_cube(path: str, energy: np.ndarray, count: np.ndarray, cell: Sequence[float],
                      atoms: Iterable[Tuple[int, float, float, float]] = ()) -> None:
    """Write a guest type's energy probability grid in the layout of the
    reference's writeenprob (utility_pack.f:689-778): the energy sums over
    the counts of the guest type's last two grids (0 where nothing was
    counted), the voxel vectors as the cell rows over the grid counts as
    writeenprob writes them (in A, not converted), framework atoms in bohr."""
    e = np.asarray(energy, dtype=np.float64)
    c = np.asarray(count, dtype=np.float64)
    na, nb, nc = e.shape
    atoms = list(atoms)
    out = ["Energy histogram cube file", "outer loop a, middle loop b, inner loop c",
           f"{len(atoms):6d}{0.0:12.6f}{0.0:12.6f}{0.0:12.6f}"]
    for n, row in zip((na, nb, nc), (cell[0:3], cell[3:6], cell[6:9])):
        out.append(f"{n:6d}" + "".join(f"{v / n:12.6f}" for v in row))
    for z, x, y, w in atoms:
        out.append(f"{int(z):6d}{0.0:12.6f}{x * ANGS2BOHR:12.6f}{y * ANGS2BOHR:12.6f}{w * ANGS2BOHR:12.6f}")
    line, ip = [], 0
    flat_e, flat_c = e.reshape(-1), c.reshape(-1)
    for j in range(1, flat_e.size + 1):
        ip += 1
        v = flat_e[j - 1] / flat_c[j - 1] if flat_c[j - 1] > 0.0 else 0.0
        line.append(fortran_e15_6(float(v)))
        if j % nc == 0 or ip == 6:
            out.append("".join(line))
            line, ip = [], 0
    if line:
        out.append("".join(line))
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")
