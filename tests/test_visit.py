"""VTK output (the reference's visit.f90 format): number formatting and file structure on
CPU; the written fields against the GPU chunk's fields."""
import os

import numpy as np
import pytest

from helpers import small_deck
from tealeaf_ref_gb300 import visit


@pytest.mark.parametrize("x,want", [(100.0, "  0.1000E+03"), (0.0, "  0.0000E+00"), (1.0e-4, "  0.1000E-03"),
                                    (25.0, "  0.2500E+02"), (-2.71828, " -0.2718E+01"), (0.99996, "  0.1000E+01"),
                                    (123456.0, "  0.1235E+06")])
def test_fortran_e12_4(x, want):
    assert visit.fortran_e(x) == want


def test_vtk_file_structure(tmp_path):
    d = small_deck(nx=3, ny=2, steps=1)
    v = visit.Visit(str(tmp_path), d)
    rho = np.array([[1.0, 2.0, 3.0], [4.0, 5.0, 6.0]])
    path = v.write(7, rho, rho * 10, rho * 100)
    assert os.path.basename(path) == "tea.00001.00007.vtk"
    lines = open(path).read().split("\n")
    assert lines[:4] == ["# vtk DataFile Version 3.0", "vtk output", "ASCII", "DATASET RECTILINEAR_GRID"]
    assert lines[4] == "DIMENSIONS" + "%12d%12d" % (4, 3) + " 1"
    assert lines[5] == "X_COORDINATES     4 double"
    assert open(os.path.join(str(tmp_path), "tea.visit")).read().split("\n")[:2] == ["!NBLOCKS     1",
                                                                                  "tea.00001.00007.vtk"]
    f = visit.read_vtk_fields(path)
    np.testing.assert_allclose(f["density"], rho)
    np.testing.assert_allclose(f["temperature"], rho * 100)


@pytest.mark.gpu
def test_run_deck_visit_files(tmp_path):
    from tealeaf_ref_gb300 import native

    d = small_deck(nx=31, ny=23, steps=4, n_rect=3, n_circ=1)
    d.visit_frequency = 2
    native.run_deck(d, visit_dir=str(tmp_path))
    idx = open(os.path.join(str(tmp_path), "tea.visit")).read().split()
    # steps 2 and 4 from the loop, step 4 again at the end of the run
    assert idx == ["!NBLOCKS", "1", "tea.00001.00002.vtk", "tea.00001.00004.vtk", "tea.00001.00004.vtk"]
    with native.Chunk.from_deck(d) as c:
        rho, e0 = c.download("density"), c.download("energy1")
        for _ in range(4):
            c.tea_leaf(d)
        u = c.download("u")
    f = visit.read_vtk_fields(os.path.join(str(tmp_path), "tea.00001.00004.vtk"))
    # E12.4 keeps four significant digits: up to half a unit in the fourth, 5e-4 relative
    np.testing.assert_allclose(f["density"], rho, rtol=5e-4)
    np.testing.assert_allclose(f["energy"], e0, rtol=5e-4)
    np.testing.assert_allclose(f["temperature"], u, rtol=5e-4)
