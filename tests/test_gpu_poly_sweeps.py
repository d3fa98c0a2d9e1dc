"""The FP64 PPCG inner step and the FP64 Chebyshev iteration as one staged sweep each (the
default without a preconditioner and without reflective boundaries) against the two one-step
kernels (TL_PPCG_INNER_SWEEP=0, TL_CHEBY_SWEEP=0): the same bits in u (Chebyshev: also w, r
and p), and the same iteration counts, inner-step counts and error, on meshes with several
strips, a last strip a few columns wide, an odd width, a mesh narrower than one strip, a larger
halo depth, the reciprocal and plain coefficients, and a 4000^2 mesh.  The Chebyshev cases end
after an odd and after an even number of sweeps (u ping-pongs between two fields)."""
import numpy as np
import pytest

from helpers import small_deck

pytestmark = pytest.mark.gpu

DECKS = {
    "ppcg_1030x700": dict(nx=1030, ny=700),
    "ppcg_1031x517_odd": dict(nx=1031, ny=517),
    "ppcg_97x300_narrow": dict(nx=97, ny=300),
    "ppcg_600x433_halo2": dict(nx=600, ny=433, halo_depth=2),
    "ppcg_600x433_coef1": dict(nx=600, ny=433, coefficient=1),
    "ppcg_4000x4000": dict(nx=4000, ny=4000, max_iters=30),
    "ppcg_600x433_inner7": dict(nx=600, ny=433, ppcg_inner_steps=7),
}


@pytest.mark.parametrize("name", list(DECKS))
def test_inner_sweep_gives_the_same_bits(name, monkeypatch):
    from tealeaf_ref_gb300 import native

    kw = dict(solver="ppcg", ppcg_inner_steps=10, ch_cg_presteps=20, ch_cg_epslim=1e30, max_iters=60, steps=1)
    kw.update(DECKS[name])
    d = small_deck(**kw)
    runs = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("TL_PPCG_INNER_SWEEP", mode)
        with native.Chunk.from_deck(d) as c:
            i = c.tea_leaf(d)
            runs[mode] = ((i.reported_iterations, i.error, i.ppcg_inner_iters, i.cg_calc_steps),
                          {f: c.download(f) for f in ("u", "sd", "rtemp", "utemp")})
    info0, f0 = runs["0"]
    info1, f1 = runs["1"]
    assert info0[2] > 0, info0  # inner steps ran
    assert info1 == info0, (info1, info0)
    for k in f0:  # sd too: the last inner step's, with an odd step count as with an even one
        assert np.array_equal(f1[k].view(np.uint64), f0[k].view(np.uint64)), k


CHEBY_DECKS = {
    "cheby_1030x700_its301": dict(nx=1030, ny=700, max_iters=301),
    "cheby_1031x517_its300": dict(nx=1031, ny=517, max_iters=300),
    "cheby_97x300_narrow": dict(nx=97, ny=300, max_iters=251),
    "cheby_600x433_halo2_coef1": dict(nx=600, ny=433, halo_depth=2, coefficient=1, max_iters=240),
    "cheby_converged_257x129": dict(nx=257, ny=129, max_iters=20000, eps=1e-10),
    "cheby_4000x4000": dict(nx=4000, ny=4000, max_iters=61),
}


@pytest.mark.parametrize("name", list(CHEBY_DECKS))
def test_cheby_sweep_gives_the_same_bits(name, monkeypatch):
    from tealeaf_ref_gb300 import native

    kw = dict(solver="chebyshev", ch_cg_presteps=20, ch_cg_epslim=1e30, steps=1)
    kw.update(CHEBY_DECKS[name])
    d = small_deck(**kw)
    runs = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("TL_CHEBY_SWEEP", mode)
        with native.Chunk.from_deck(d) as c:
            i = c.tea_leaf(d)
            runs[mode] = ((i.reported_iterations, i.error, i.cheby_calc_steps, i.cg_calc_steps),
                          {f: c.download(f) for f in ("u", "w", "r", "p")})
    info0, f0 = runs["0"]
    info1, f1 = runs["1"]
    assert info0[2] > 20, info0  # Chebyshev iterations ran
    assert info1 == info0, (info1, info0)
    for k in f0:
        assert np.array_equal(f1[k].view(np.uint64), f0[k].view(np.uint64)), k


def test_cheby_sweep_exit_on_an_unchecked_iteration(monkeypatch):
    """tl_eps times the initial residual set to 1.5: the stale error the reference square-roots
    each Chebyshev iteration (tea_solve.f90:273,402) falls below it a few iterations after the
    switch, on an iteration whose residual is not checked -- one whose w and r the staged sweep
    leaves unwritten.  The solve forms them afterwards; every field matches the two kernels."""
    from tealeaf_ref_gb300 import native

    d = small_deck(nx=600, ny=433, solver="chebyshev", ch_cg_presteps=20, ch_cg_epslim=1e30, max_iters=300,
                   steps=1)
    with native.Chunk.from_deck(d) as c:
        r0 = c.tea_leaf(d).initial_residual
    d.eps = 1.5 / r0
    runs = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("TL_CHEBY_SWEEP", mode)
        with native.Chunk.from_deck(d) as c:
            i = c.tea_leaf(d)
            runs[mode] = ((i.reported_iterations, i.error, i.cheby_calc_steps),
                          {f: c.download(f) for f in ("u", "w", "r", "p")})
    info0, f0 = runs["0"]
    info1, f1 = runs["1"]
    assert 0 < info0[2] and info0[0] < d.max_iters, info0  # it switched and exited early
    assert info1 == info0, (info1, info0)
    for k in f0:
        assert np.array_equal(f1[k].view(np.uint64), f0[k].view(np.uint64)), k
