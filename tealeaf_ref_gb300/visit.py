"""VTK output of a chunk, in the format the reference's visit subroutine writes (visit.f90:26-139).

Each call writes ``tea.<chunk>.<step>.vtk``: a legacy ASCII VTK rectilinear grid with the vertex
coordinates and three cell fields, ``density``, ``energy`` (the reference writes energy0, the
generated state, which its time loop never changes) and ``temperature`` (u). Values are
written one per line in Fortran ``E12.4`` form. The calls also maintain the index file
``tea.visit``: a ``!NBLOCKS`` header on the first call, then one line per chunk file.
"""
from __future__ import annotations

import os
from typing import Sequence

import numpy as np


def fortran_e(x: float, w: int = 12, d: int = 4) -> str:
    """``x`` in Fortran ``Ew.d`` edit form: ``0.dddd`` mantissa times a power of ten,
    right-justified in ``w`` characters (e.g. 100.0 -> ``  0.1000E+03``)."""
    x = float(x)
    if x == 0.0:
        body = "0." + "0" * d + "E+00"
    else:
        sci = "%.*e" % (d - 1, abs(x))  # d significant digits: "d.ddd e+XX"
        mant, exp = sci.split("e")
        digits = mant.replace(".", "")
        e = int(exp) + 1  # 0.dddd form
        ee = "%+03d" % e if abs(e) <= 99 else "%+04d" % e
        body = "0." + digits + ("E" + ee if abs(e) <= 99 else ee)
        if x < 0:
            body = "-" + body
    return body.rjust(w)


def _name(prefix: str, chunk: int, step: int) -> str:
    # chunk and step numbers written as (n + 100000) with the leading digit replaced by '.'
    c = "." + str(chunk + 100000)[1:]
    s = "." + str(step + 100000)[1:]
    return prefix + c + s + ".vtk"


def write_vtk(path: str, xv: Sequence[float], yv: Sequence[float], density: np.ndarray, energy: np.ndarray,
              temperature: np.ndarray) -> None:
    """One chunk file: vertex coordinates xv (x_cells+1), yv (y_cells+1) and three
    (y_cells, x_cells) cell fields, x fastest."""
    nyc, nxc = density.shape
    lines = ["# vtk DataFile Version 3.0", "vtk output", "ASCII", "DATASET RECTILINEAR_GRID",
             "DIMENSIONS%12d%12d 1" % (nxc + 1, nyc + 1), "X_COORDINATES %5d double" % (nxc + 1)]
    lines += [fortran_e(v) for v in xv]
    lines.append("Y_COORDINATES %5d double" % (nyc + 1))
    lines += [fortran_e(v) for v in yv]
    lines += ["Z_COORDINATES 1 double", "0", "CELL_DATA %20d" % (nxc * nyc), "FIELD FieldData 3"]
    for name, field in (("density", density), ("energy", energy), ("temperature", temperature)):
        lines.append("%s 1 %20d double" % (name, nxc * nyc))
        lines += [fortran_e(v) for v in np.asarray(field, dtype=np.float64).ravel()]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


class Visit:
    """The reference's visit() for one chunk: call ``write(step, ...)`` where diffuse.f90 calls
    visit (every visit_frequency steps and at the end of the run)."""

    def __init__(self, directory: str, deck, prefix: str = "tea", nblocks: int = 1):
        self.dir = directory
        self.prefix = prefix
        os.makedirs(directory, exist_ok=True)
        dx = (deck.xmax - deck.xmin) / deck.x_cells
        dy = (deck.ymax - deck.ymin) / deck.y_cells
        # vertexx(j) = xmin + dx * (j - x_min), j = x_min .. x_max+1 (initialise_chunk_kernel.f90)
        self.xv = [deck.xmin + dx * j for j in range(deck.x_cells + 1)]
        self.yv = [deck.ymin + dy * k for k in range(deck.y_cells + 1)]
        self.index = os.path.join(directory, prefix + ".visit")
        with open(self.index, "w") as f:
            f.write("!NBLOCKS %5d\n" % nblocks)

    def write(self, step: int, density: np.ndarray, energy0: np.ndarray, u: np.ndarray) -> str:
        name = _name(self.prefix, 1, step)
        with open(self.index, "a") as f:
            f.write(name + "\n")
        path = os.path.join(self.dir, name)
        write_vtk(path, self.xv, self.yv, density, energy0, u)
        return path


def read_vtk_fields(path: str):
    """The three cell fields of a file written by write_vtk, as (y_cells, x_cells) arrays."""
    with open(path) as f:
        lines = f.read().split("\n")
    dims = lines[4].split()
    nx, ny = int(dims[1]) - 1, int(dims[2]) - 1
    out = {}
    i = 0
    while i < len(lines):
        parts = lines[i].split()
        if len(parts) == 4 and parts[0] in ("density", "energy", "temperature") and parts[3] == "double":
            n = int(parts[2])
            out[parts[0]] = np.array([float(v) for v in lines[i + 1:i + 1 + n]]).reshape(ny, nx)
            i += n
        i += 1
    return out
