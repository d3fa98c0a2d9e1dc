"""Pin the CPU oracle against the reference's own known answers (no GPU).

The reference's Benchmarks/tea_bm_{1..4}.out were produced by a single task and thread with
IEEE floating point; the serial oracle follows the same loop and operation order without
FMA contraction, so its step-10 field summary reproduces every printed digit and its
per-step CG iteration counts are identical.  tea.in (PPCG, halo depth 2, test problem 4)
must reproduce the reference's QA temperature within the reference's own 1e-5 bar
(field_summary.f90:104-129).
"""
import numpy as np
import pytest

from oracle import oracle
from tealeaf_ref_gb300 import deck as dk


def _run(golden, name):
    g = golden["benchmarks"][name]
    return g, oracle.run_deck(dk.parse_deck(g["deck"]))


def _check_exact(g, res):
    assert [s.reported_iterations for s in res.solves] == g["iterations"]
    for want in g["summaries"]:
        got = dict(res.summaries)[want["step"]]
        # the .out files print 17 significant digits: equal to within one unit there
        for k, v in zip(("volume", "mass", "energy", "temperature"), (got[0], got[1], got[2], got[3])):
            assert abs(v - want[k]) <= 1e-16 * abs(want[k]) * 10, (k, v, want[k])
        assert abs(got[1] / got[0] - want["density"]) <= 1e-15 * want["density"]
    for err, want in zip([s.conduction_error for s in res.solves], g["conduction_errors"]):
        assert abs(err - want) <= 5e-7 * want  # printed with 7 digits


@pytest.mark.parametrize("name", ["tea_bm_1", "tea_bm_2", "tea_bm_3"])
def test_benchmark_exact(golden, name):
    g, res = _run(golden, name)
    _check_exact(g, res)


def test_benchmark_exact_1000(golden):
    g, res = _run(golden, "tea_bm_4")
    _check_exact(g, res)


def test_ppcg_deck_qa(golden):
    d = dk.parse_deck(golden["ppcg_deck"])
    assert d.solver == "ppcg" and d.halo_depth == 2 and d.effective_inner_steps() == 124
    res = oracle.run_deck(d)
    temp = res.summaries[-1][1][3]
    qa = golden["qa_temperature"]["4"]
    assert abs(100.0 * (temp / qa) - 100.0) < 0.001


def test_oracle_eigenvalues_match_numpy():
    rng = np.random.default_rng(3)
    for n in (1, 2, 5, 20, 60):
        d = rng.uniform(0.5, 5.0, n)
        off = rng.uniform(-1.0, 1.0, max(n - 1, 0))
        T = np.diag(d) + np.diag(off, 1) + np.diag(off, -1)
        want = np.linalg.eigvalsh(T)
        got = oracle.tridiag_eigenvalues(d, off)
        np.testing.assert_allclose(got, want, rtol=1e-13, atol=1e-13 * np.max(np.abs(want)))


def test_oracle_reflective_and_jacobi_quirk():
    """With reflective boundaries the Jacobi kernel still reads the never-updated halo of
    its un array (vector_r), i.e. zero: the oracle keeps that behaviour."""
    d = dk.seeded_deck(12, 2, 0, 5, steps=1, max_iters=5, solver="jacobi", eps=1e-30)
    d.reflective_boundary = True
    c = oracle.Chunk.from_deck(d)
    c.tea_leaf(d)
    r = c.array("r")
    h = c.h
    assert np.all(r[:h, :] == 0.0) and np.all(r[:, :h] == 0.0)


def test_exact_summary_helper_matches_serial_summary():
    """The correctly rounded field summary the full-size parity tests use agrees with the
    oracle's serial field_summary to within the serial sums' own rounding bound (4e-16 per
    summed cell, as for the other reductions)."""
    import sys
    import os
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from helpers import exact_summary, small_deck

    d = small_deck(nx=120, ny=77, steps=1)
    o = oracle.Chunk.from_deck(d)
    o.tea_leaf(d)
    np.testing.assert_allclose(exact_summary(o), o.field_summary(), rtol=max(1e-12, 4e-16 * d.x_cells * d.y_cells))
