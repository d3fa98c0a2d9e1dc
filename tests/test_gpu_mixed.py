"""The mixed-precision form (FP32 inner CG inside FP64 iterative refinement) against the
FP64 oracle: the same field-summary (1e-10) and per-cell u (1e-8) bars as the FP64 form."""
import numpy as np
import pytest

from helpers import small_deck
from tealeaf_ref_gb300 import deck as dk

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b) / np.abs(b)))


CASES = [
    dict(),
    dict(coefficient=1),
    dict(reflective=True),
    dict(nx=200, ny=131, n_rect=6, n_circ=3),
    dict(precond="jac_diag"),
    dict(precond="jac_diag", reflective=True, nx=200, ny=131),
    dict(precond="jac_diag", nx=1030, ny=700, steps=2),
]


@pytest.mark.parametrize("case", CASES, ids=["-".join("%s%s" % kv for kv in c.items()) or "default" for c in CASES])
def test_mixed_cg_matches_fp64_oracle(case):
    from oracle import oracle
    from tealeaf_ref_gb300 import native

    kw = dict(nx=67, ny=45, steps=3, n_rect=4, n_circ=2, max_iters=20000)
    kw.update(case)
    d = small_deck(**kw)
    ro = oracle.run_deck(d)
    opts = native.opts_from_deck(d, precision="mixed")
    with native.Chunk.from_deck(d) as c:
        infos, recomputed = [], []
        for _ in range(d.end_step):
            infos.append(c.tea_leaf(opts, d.initial_timestep))
            # the true residual the solve reports, recomputed by the per-kernel entry points
            c.update_halo(["u"])
            c.calc_residual()
            recomputed.append(np.sqrt(abs(c.calc_2norm(1))))
        s = c.field_summary()
        u = c.download("u")
    o = oracle.Chunk.from_deck(d)
    for _ in range(d.end_step):
        o.tea_leaf(d)
    assert _rel(s, ro.summaries[-1][1]) < 1e-10
    assert _rel(u, np.array(o.interior("u"))) < 1e-8
    for i, rr in zip(infos, recomputed):
        assert i.outer_iterations >= 1
        assert i.true_residual <= 1e-9 * i.initial_residual
        assert native.STOP_REASONS[i.stop_reason] in ("eps", "floor", "stall", "reject")
        assert 0.0 < i.residual_floor < i.true_residual * 1e3
        # near the floor the residual is rounding noise, so the two evaluations agree in size only
        assert rr <= 2.0 * i.true_residual + 16.0 * i.residual_floor


def test_mixed_cg_inner_cap():
    """max_inner_iters stops the FP32 CG process; the accepted corrections remain in u."""
    from tealeaf_ref_gb300 import native

    d = small_deck(nx=64, ny=64, steps=1, n_rect=3, n_circ=1, max_iters=20000)
    opts = native.opts_from_deck(d, precision="mixed", max_inner_iters=12)
    with native.Chunk.from_deck(d) as c:
        i = c.tea_leaf(opts, d.initial_timestep)
    assert native.STOP_REASONS[i.stop_reason] == "cap"
    assert i.reported_iterations == 12
    assert i.true_residual < i.initial_residual


def test_mixed_cg_reference_deck(golden):
    """tea_bm_2 (250^2, default coefficient) in the mixed form against the reference's output."""
    from tealeaf_ref_gb300 import native

    g = golden["benchmarks"]["tea_bm_2"]
    d = dk.parse_deck(g["deck"])
    res = native.run_deck(d, precision="mixed")
    s = res.summaries[-1][1]
    want = g["summaries"][-1]
    ref = [want["volume"], want["mass"], want["energy"], want["temperature"]]
    assert _rel(s, ref) < 1e-10


POLY_CASES = [
    dict(solver="ppcg", ppcg_inner_steps=10, ch_cg_presteps=20),
    dict(solver="ppcg", ppcg_inner_steps=10, ch_cg_presteps=20, coefficient=1),
    dict(solver="ppcg", ppcg_inner_steps=8, ch_cg_presteps=20, reflective=True),
    dict(solver="ppcg", ppcg_inner_steps=5, ch_cg_presteps=20, nx=131, ny=77),
    dict(solver="chebyshev", ch_cg_presteps=20),
    dict(solver="chebyshev", ch_cg_presteps=20, coefficient=1),
    dict(solver="chebyshev", ch_cg_presteps=20, reflective=True),
    dict(solver="chebyshev", ch_cg_presteps=30, nx=131, ny=77),
    dict(solver="ppcg", ppcg_inner_steps=10, ch_cg_presteps=20, precond="jac_diag"),
    dict(solver="ppcg", ppcg_inner_steps=8, ch_cg_presteps=20, precond="jac_diag", reflective=True),
    dict(solver="chebyshev", ch_cg_presteps=20, precond="jac_diag"),
    dict(solver="chebyshev", ch_cg_presteps=20, precond="jac_diag", reflective=True),
]


@pytest.mark.parametrize("case", POLY_CASES, ids=["-".join("%s%s" % kv for kv in c.items()) for c in POLY_CASES])
def test_mixed_chebyshev_ppcg_match_fp64_oracle(case):
    """FP32 inner sweeps (PPCG's preconditioner steps; Chebyshev iterations on a correction in FP64
    refinement) against the FP64 oracle at the FP64 form's bars."""
    from oracle import oracle
    from tealeaf_ref_gb300 import native

    kw = dict(nx=67, ny=45, steps=3, n_rect=4, n_circ=2, max_iters=20000)
    kw.update(case)
    d = small_deck(**kw)
    ro = oracle.run_deck(d)
    opts = native.opts_from_deck(d, precision="mixed")
    with native.Chunk.from_deck(d) as c:
        infos = [c.tea_leaf(opts, d.initial_timestep) for _ in range(d.end_step)]
        s = c.field_summary()
        u = c.download("u")
    o = oracle.Chunk.from_deck(d)
    for _ in range(d.end_step):
        o.tea_leaf(d)
    assert _rel(s, ro.summaries[-1][1]) < 1e-10
    assert _rel(u, np.array(o.interior("u"))) < 1e-8
    for i in infos:
        assert i.reported_iterations < d.max_iters
        if d.solver == "chebyshev":
            assert native.STOP_REASONS[i.stop_reason] in ("eps", "floor", "stall", "reject")
            assert i.true_residual <= 1e-9 * i.initial_residual


def test_mixed_ppcg_reference_deck(golden):
    """The reference's tea.in (PPCG, 1000^2, halo depth 2, test problem 4) in the mixed form:
    the reference's QA temperature (its own 1e-5 bar) and the FP64 form's summary (1e-10)."""
    from tealeaf_ref_gb300 import native

    d = dk.parse_deck(golden["ppcg_deck"])
    r64 = native.run_deck(d)
    rmx = native.run_deck(d, precision="mixed")
    assert _rel(rmx.summaries[-1][1], r64.summaries[-1][1]) < 1e-10
    qa = float(golden["qa_temperature"]["4"])
    assert abs(rmx.summaries[-1][1][3] - qa) <= 1e-5 * abs(qa)


def test_mixed_rejected_for_jacobi_and_preconditioners():
    from tealeaf_ref_gb300 import native

    for kw in (dict(solver="jacobi"), dict(solver="cg", precond="jac_block"),
               dict(solver="ppcg", ppcg_inner_steps=4, precond="jac_block")):
        d = small_deck(nx=16, ny=16, **kw)
        with native.Chunk.from_deck(d) as c:
            with pytest.raises(native.TeaLeafError) as e:
                c.tea_leaf(native.opts_from_deck(d, precision="mixed"), d.initial_timestep)
            assert e.value.code == -1


@pytest.mark.parametrize("solver", ["ppcg", "chebyshev"])
@pytest.mark.parametrize("reflective", [False, True])
@pytest.mark.parametrize("precond", ["none", "jac_diag"])
def test_blocked_poly_sweeps_bitwise(solver, reflective, precond, monkeypatch):
    """The temporally blocked FP32 sweeps (several polynomial steps per pass over the mesh)
    give the bits of the one-step sweeps: same solution and iteration counts for 3 and 4
    steps per sweep, 2 or 4 columns per lane, TMA or cp.async staging, on a mesh whose width
    and height cut the warp strips and row ranges raggedly."""
    from tealeaf_ref_gb300 import native

    d = small_deck(nx=301, ny=133, steps=2, n_rect=4, n_circ=2, solver=solver, ppcg_inner_steps=10,
                   ch_cg_presteps=20, reflective=reflective, max_iters=20000, precond=precond)
    opts = native.opts_from_deck(d, precision="mixed")
    runs = []
    # steps per sweep x columns per lane of the warp strips (2 or 4) x staging (TMA or cp.async)
    for per_sweep, cols, tma in (("1", "2", "1"), ("4", "2", "1"), ("3", "2", "1"), ("4", "4", "1"),
                                 ("3", "4", "1"), ("4", "2", "0"), ("4", "4", "0")):
        monkeypatch.setenv("TL_POLY_STEPS_PER_SWEEP", per_sweep)
        monkeypatch.setenv("TL_POLY_COLS", cols)
        monkeypatch.setenv("TL_POLY_TMA", tma)
        with native.Chunk.from_deck(d) as c:
            its = [c.tea_leaf(opts, d.initial_timestep).reported_iterations for _ in range(d.end_step)]
            runs.append((c.download("u"), its))
    for u, its in runs[1:]:
        assert its == runs[0][1]
        np.testing.assert_array_equal(u, runs[0][0])


@pytest.mark.parametrize("solver", ["ppcg", "chebyshev"])
def test_blocked_sweep_wait_is_bounded(solver, monkeypatch):
    """The blocked FP32 polynomial sweep's waits for staged rows end by themselves: with one
    row's mbarrier armed and its tensor copies never issued (TL_POLY_TEST_HOLD=1), the waiting
    warp gives up after a bounded number of polls, waits (bounded) for its other copies in
    flight and returns; the later sweeps of the solve return at once, the solve reports
    TL_ERR_TIMEOUT, and the same context then solves normally."""
    import time

    from tealeaf_ref_gb300 import native

    d = small_deck(nx=300, ny=160, steps=1, n_rect=4, n_circ=2, max_iters=20000, solver=solver,
                   ch_cg_presteps=20, ppcg_inner_steps=10)
    opts = native.opts_from_deck(d, precision="mixed")
    monkeypatch.delenv("TL_POLY_TMA", raising=False)
    monkeypatch.delenv("TL_POLY_STEPS_PER_SWEEP", raising=False)
    with native.Chunk.from_deck(d) as c:
        monkeypatch.setenv("TL_POLY_TEST_HOLD", "1")
        t0 = time.perf_counter()
        with pytest.raises(native.TeaLeafError) as e:
            c.tea_leaf(opts, d.initial_timestep)
        assert e.value.code == -5  # TL_ERR_TIMEOUT
        assert time.perf_counter() - t0 < 60
        monkeypatch.delenv("TL_POLY_TEST_HOLD")
        c.generate(d)
        c.reset_eigen()
        info = c.tea_leaf(opts, d.initial_timestep)
        assert info.reported_iterations > 0
