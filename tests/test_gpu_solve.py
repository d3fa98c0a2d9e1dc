"""Whole-solve parity on the GPU.

* The reference's own benchmark decks (Benchmarks/tea_bm_{1..6}.in, CG, tl_eps 1e-15):
  the step-10 field summary must match the reference's printed values to 1e-10 relative
  and every per-step iteration count to within one iteration (reduction order differs).
* Synthetic decks of every solver, coefficient and preconditioner: field summaries within
  1e-10 and per-cell u within 1e-8 of the oracle run on the same deck (the accuracy bar of
  the FP64 form), iteration counts within a few percent.
"""
import numpy as np
import pytest

from helpers import small_deck
from tealeaf_ref_gb300 import deck as dk

pytestmark = pytest.mark.gpu


def _summary_close(a, b, rtol):
    a, b = np.asarray(a), np.asarray(b)
    return np.all(np.abs(a - b) <= rtol * np.abs(b)), np.max(np.abs(a - b) / np.abs(b))


@pytest.mark.parametrize("bm", [1, 2, 3, 4, 5, 6])
def test_reference_benchmark_decks(golden, bm):
    from tealeaf_ref_gb300 import native

    g = golden["benchmarks"]["tea_bm_%d" % bm]
    d = dk.parse_deck(g["deck"])
    res = native.run_deck(d)
    want = g["summaries"][-1]
    step, s = res.summaries[-1]
    assert step == want["step"]
    got = [s[0], s[1], s[2], s[3]]
    ref = [want["volume"], want["mass"], want["energy"], want["temperature"]]
    ok, worst = _summary_close(got, ref, 1e-10)
    assert ok, "field summary rel diff %.3e" % worst
    its = [x["reported_iterations"] for x in res.solves]
    assert len(its) == len(g["iterations"])
    # At tl_eps 1e-15 the step at which sqrt(rrn) crosses eps * initial residual depends on the
    # rounding of the dot products of the last iterations (block-partitioned sums here, the
    # Fortran's OpenMP reduction there), so the counts agree to a fraction of a percent, not
    # exactly; the field summary above is the accuracy bar.
    for a, b in zip(its, g["iterations"]):
        assert abs(a - b) <= max(2, int(0.005 * b)), (its, g["iterations"])


SOLVE_CASES = [
    dict(solver="cg"),
    dict(solver="cg", coefficient=1),
    dict(solver="cg", precond="jac_diag"),
    dict(solver="cg", precond="jac_block"),
    dict(solver="cg", reflective=True),
    dict(solver="chebyshev", ch_cg_presteps=20),
    dict(solver="chebyshev", ch_cg_presteps=20, precond="jac_diag"),
    dict(solver="ppcg", ppcg_inner_steps=10, ch_cg_presteps=20),
    dict(solver="ppcg", ppcg_inner_steps=10, ch_cg_presteps=20, halo_depth=2),
    dict(solver="ppcg", ppcg_inner_steps=6, ch_cg_presteps=15, precond="jac_block"),
    dict(solver="ppcg", ppcg_inner_steps=8, ch_cg_presteps=20, reflective=True),
    dict(solver="jacobi", max_iters=300, eps=1e-10),
    dict(solver="jacobi", max_iters=301, eps=1e-10, reflective=True),
    dict(solver="jacobi", max_iters=20000, eps=1e-5, nx=24, ny=17, n_rect=2, n_circ=0),
]


@pytest.mark.parametrize("case", SOLVE_CASES, ids=["-".join("%s%s" % kv for kv in c.items()) for c in SOLVE_CASES])
def test_solvers_against_oracle(case):
    from oracle import oracle
    from tealeaf_ref_gb300 import native

    kw = dict(nx=67, ny=45, steps=3, n_rect=4, n_circ=2)
    kw.update(case)
    d = small_deck(**kw)
    ro = oracle.run_deck(d)
    with native.Chunk.from_deck(d) as c:
        sums = [c.field_summary()]
        infos = []
        for _ in range(d.end_step):
            infos.append(c.tea_leaf(d))
        sums.append(c.field_summary())
        u_gpu = c.download("u")
    o = oracle.Chunk.from_deck(d)
    for _ in range(d.end_step):
        o.tea_leaf(d)
    u_ref = np.array(o.interior("u"))
    ok, worst = _summary_close(sums[-1], ro.summaries[-1][1], 1e-10)
    assert ok, "summary rel diff %.3e" % worst
    rel = np.max(np.abs(u_gpu - u_ref) / np.abs(u_ref))
    assert rel < 1e-8, "per-cell u rel diff %.3e" % rel
    for gi, oi in zip(infos, ro.solves):
        n_o = oi.reported_iterations
        # Chebyshev tests its residual only every 10th iteration (tea_solve.f90:273)
        slack = 10 if d.solver == "chebyshev" else max(2, int(0.03 * n_o))
        assert abs(gi.reported_iterations - n_o) <= slack, (gi.reported_iterations, n_o)


def test_config1_256_against_oracle():
    """Synthetic config 1 (256^2, 3 rectangles, reciprocal-density keyword, CG, 10 steps)."""
    from oracle import oracle
    from tealeaf_ref_gb300 import native

    d = dk.config_deck(1)
    ro = oracle.run_deck(d)
    rg = native.run_deck(d)
    ok, worst = _summary_close(rg.summaries[-1][1], ro.summaries[-1][1], 1e-10)
    assert ok, worst
    for gi, oi in zip(rg.solves, ro.solves):
        assert abs(gi["reported_iterations"] - oi.reported_iterations) <= 2


def test_repeatable_bitwise():
    """Fixed-order reductions: two identical runs give identical bits."""
    from tealeaf_ref_gb300 import native

    d = small_deck(nx=129, ny=77, steps=2)
    a = native.run_deck(d).summaries[-1][1]
    b = native.run_deck(d).summaries[-1][1]
    np.testing.assert_array_equal(a, b)


def test_breakdown_reported():
    """Zero energy everywhere gives u0 = 0 and r = 0 exactly, so pw = 0 and alpha = 0/0:
    reported as TL_ERR_BREAKDOWN instead of iterating on NaNs as the reference would."""
    from tealeaf_ref_gb300 import native

    d = small_deck(nx=16, ny=16, n_rect=0, n_circ=0)
    d.states[0].energy = 0.0
    with native.Chunk.from_deck(d) as c:
        with pytest.raises(native.TeaLeafError) as e:
            c.tea_leaf(d)
        assert e.value.code == -4


@pytest.mark.parametrize("case", [dict(), dict(precond="jac_diag"), dict(reflective=True),
                                  dict(solver="ppcg", ppcg_inner_steps=8, ch_cg_presteps=20)],
                         ids=["cg", "jac_diag", "reflective", "ppcg-presteps"])
def test_persistent_cg_matches_batched(case, monkeypatch):
    """The persistent cooperative CG kernel (one launch for many iterations, grid barriers)
    against the batched fused kernels on the same deck: field summary 1e-10, u 1e-8, iteration
    counts within a few (different reduction trees)."""
    from tealeaf_ref_gb300 import native

    kw = dict(nx=203, ny=151, steps=3, n_rect=4, n_circ=2, max_iters=20000)
    kw.update(case)
    d = small_deck(**kw)
    runs = []
    for forced in ("0", "1"):
        monkeypatch.setenv("TL_CG_PERSISTENT", forced)
        with native.Chunk.from_deck(d) as c:
            its = [c.tea_leaf(d).reported_iterations for _ in range(d.end_step)]
            runs.append((c.field_summary(), c.download("u"), its))
    (s0, u0, i0), (s1, u1, i1) = runs
    ok, worst = _summary_close(s1, s0, 1e-10)
    assert ok, worst
    assert np.max(np.abs(u1 - u0) / np.abs(u0)) < 1e-8
    for a, b in zip(i1, i0):
        assert abs(a - b) <= max(2, int(0.01 * b)), (i1, i0)


def test_persistent_cg_barrier_wait_is_bounded(monkeypatch):
    """The persistent kernel's grid-barrier waits end by themselves: made to wait for an
    arrival that never comes, every CTA gives up after about a second, the solve returns
    TL_ERR_TIMEOUT, and the context solves normally afterwards."""
    import time

    from tealeaf_ref_gb300 import native

    d = small_deck(nx=64, ny=64, steps=1, n_rect=2, n_circ=1)
    monkeypatch.setenv("TL_CG_PERSISTENT", "1")
    with native.Chunk.from_deck(d) as c:
        monkeypatch.setenv("TL_CG_BARRIER_EXTRA", "1")
        t0 = time.perf_counter()
        with pytest.raises(native.TeaLeafError) as e:
            c.tea_leaf(d)
        assert e.value.code == -5  # TL_ERR_TIMEOUT
        assert time.perf_counter() - t0 < 60
        monkeypatch.delenv("TL_CG_BARRIER_EXTRA")
        c.generate(d)
        info = c.tea_leaf(d)
        assert info.reported_iterations > 0


@pytest.mark.parametrize("reflective", [False, True])
def test_jacobi_bitwise(reflective):
    """The device-resident Jacobi loop computes each update with the reference's bits, so
    after the same number of iterations (tl_eps too small to stop either run) u is
    bit-for-bit the oracle's, and a solve that reaches an exact fixed point stops at the
    oracle's iteration."""
    from oracle import oracle
    from tealeaf_ref_gb300 import native

    d = small_deck(nx=75, ny=41, steps=2, solver="jacobi", max_iters=400, eps=1e-300, reflective=reflective)
    o = oracle.Chunk.from_deck(d)
    want = [o.tea_leaf(d).reported_iterations for _ in range(d.end_step)]
    with native.Chunk.from_deck(d) as c:
        got = [c.tea_leaf(d).reported_iterations for _ in range(d.end_step)]
        np.testing.assert_array_equal(c.download("u"), np.array(o.interior("u")))
    assert got == want


@pytest.mark.parametrize("case", [dict(), dict(precond="jac_diag"), dict(reflective=True), dict(halo_depth=2),
                                  dict(precision="mixed"), dict(precision="mixed", reflective=True)],
                         ids=["none", "jac_diag", "reflective", "halo2", "mixed", "mixed-reflective"])
def test_fused_ppcg_matches_per_kernel_path(case, monkeypatch):
    """The PPCG outer iterations with device scalars (fused sweeps, one status read per
    iteration) against the per-kernel path with host scalars on the same deck: field summary
    1e-10, u 1e-8, iteration counts within a few (different reduction trees)."""
    from tealeaf_ref_gb300 import native

    case = dict(case)
    precision = case.pop("precision", "fp64")
    kw = dict(nx=203, ny=151, steps=3, n_rect=4, n_circ=2, max_iters=20000, solver="ppcg", ppcg_inner_steps=10,
              ch_cg_presteps=20)
    kw.update(case)
    d = small_deck(**kw)
    opts = native.opts_from_deck(d, precision=precision)
    runs = []
    for fused in ("0", "1"):
        monkeypatch.setenv("TL_PPCG_FUSED", fused)
        with native.Chunk.from_deck(d) as c:
            infos = [c.tea_leaf(opts, d.initial_timestep) for _ in range(d.end_step)]
            runs.append((c.field_summary(), c.download("u"), infos))
    (s0, u0, i0), (s1, u1, i1) = runs
    ok, worst = _summary_close(s1, s0, 1e-10)
    assert ok, worst
    assert np.max(np.abs(u1 - u0) / np.abs(u0)) < 1e-8
    for a, b in zip(i1, i0):
        assert a.ppcg_inner_iters > 0
        assert abs(a.reported_iterations - b.reported_iterations) <= max(2, int(0.01 * b.reported_iterations))
        assert abs(a.ppcg_inner_iters - b.ppcg_inner_iters) <= 10 * max(2, int(0.01 * b.reported_iterations))


def test_two_contexts_interleaved_bitwise():
    """Two contexts of different shapes alive at once, their solves interleaved (FP64 CG and
    mixed PPCG): each ends with the bits of the same deck solved alone.  Covers the per-context
    graphs and state and the process-wide caches (tensor maps, launch shapes)."""
    from tealeaf_ref_gb300 import native

    da = small_deck(nx=203, ny=151, steps=3, n_rect=4, n_circ=2, max_iters=20000)
    db = small_deck(nx=301, ny=133, steps=3, n_rect=3, n_circ=1, max_iters=20000, solver="ppcg",
                    ppcg_inner_steps=10, ch_cg_presteps=20, seed=11)
    oa = native.opts_from_deck(da)
    ob = native.opts_from_deck(db, precision="mixed")

    def alone(d, o):
        with native.Chunk.from_deck(d) as c:
            for _ in range(d.end_step):
                c.tea_leaf(o, d.initial_timestep)
            return c.download("u")

    ua, ub = alone(da, oa), alone(db, ob)
    with native.Chunk.from_deck(da) as ca, native.Chunk.from_deck(db) as cb:
        for _ in range(3):
            ca.tea_leaf(oa, da.initial_timestep)
            cb.tea_leaf(ob, db.initial_timestep)
        np.testing.assert_array_equal(ca.download("u"), ua)
        np.testing.assert_array_equal(cb.download("u"), ub)


@pytest.mark.parametrize("case", [dict(), dict(precond="jac_diag"), dict(precond="jac_block"), dict(reflective=True),
                                  dict(solver="jacobi", max_iters=300, eps=1e-10)],
                         ids=["cg", "jac_diag", "jac_block", "reflective", "jacobi"])
def test_setup_cache_bitwise(case, monkeypatch):
    """Kx, Ky, Di and the preconditioner set-up are rebuilt only when density or dt changed
    since the last solve: the cached run gives the bits of a run that rebuilds them every time
    step (TL_SETUP_CACHE=0), as the reference's tea_leaf_common_init does."""
    from tealeaf_ref_gb300 import native

    kw = dict(nx=203, ny=151, steps=3, n_rect=4, n_circ=2, max_iters=20000)
    kw.update(case)
    d = small_deck(**kw)
    runs = []
    for cache in ("1", "0"):
        monkeypatch.setenv("TL_SETUP_CACHE", cache)
        with native.Chunk.from_deck(d) as c:
            its = [c.tea_leaf(d).reported_iterations for _ in range(d.end_step)]
            runs.append((c.field_summary(), c.download("u"), c.download("kx"), its))
    for a, b in zip(runs[0], runs[1]):
        np.testing.assert_array_equal(a, b)


def test_setup_cache_follows_density_and_dt():
    """A solve after a new density (upload, staged take, field upload) or a new dt rebuilds the
    set-up: each result equals a fresh context's on the same state, bit for bit."""
    from tealeaf_ref_gb300 import native

    d = small_deck(nx=130, ny=97, steps=1, n_rect=3, n_circ=1, max_iters=20000)
    with native.Chunk.from_deck(d) as c:
        dens, ener = c.download("density"), c.download("energy1")
    dens2 = dens * (1.0 + 0.25 * np.sin(np.arange(dens.size)).reshape(dens.shape))
    dt, dt2 = d.initial_timestep, 0.5 * d.initial_timestep

    def fresh(density, energy, step_dt):
        with native.Chunk.from_deck(d) as c:
            c.upload_state(density, energy)
            c.tea_leaf(d, step_dt)
            return c.download("u")

    with native.Chunk.from_deck(d) as c:
        c.tea_leaf(d, dt)
        c.upload_state(dens2, ener)
        c.tea_leaf(d, dt)
        np.testing.assert_array_equal(c.download("u"), fresh(dens2, ener, dt))
        c.upload_state(dens2, ener)
        c.tea_leaf(d, dt2)
        np.testing.assert_array_equal(c.download("u"), fresh(dens2, ener, dt2))
        c.upload("density", dens)
        c.upload("energy1", ener)
        c.tea_leaf(d, dt2)
        np.testing.assert_array_equal(c.download("u"), fresh(dens, ener, dt2))
        c.stage_state(dens2, ener)
        c.take_staged()
        c.tea_leaf(d, dt2)
        np.testing.assert_array_equal(c.download("u"), fresh(dens2, ener, dt2))
        c.wait_transfers()


@pytest.mark.parametrize("case", [dict(), dict(nx=1030, ny=700), dict(reflective=True, nx=1030, ny=700),
                                  dict(solver="ppcg", ppcg_inner_steps=10, ch_cg_presteps=20),
                                  dict(solver="jacobi", max_iters=200, eps=1e-10),
                                  dict(precision="mixed", nx=1030, ny=700)],
                         ids=["cg-persistent", "cg-batched", "cg-reflective", "ppcg", "jacobi", "mixed-cg"])
def test_tea_leaf_summary_bitwise(case):
    """tl_tea_leaf_summary (finalise fused with field_summary, and with the CG loop's last
    deferred u update on the batched path) gives the bits of tl_tea_leaf followed by
    tl_field_summary: the summary, energy1, u and the iteration counts."""
    from tealeaf_ref_gb300 import native

    case = dict(case)
    precision = case.pop("precision", "fp64")
    kw = dict(nx=203, ny=151, steps=2, n_rect=4, n_circ=2, max_iters=20000)
    kw.update(case)
    d = small_deck(**kw)
    opts = native.opts_from_deck(d, precision=precision)
    runs = []
    for fused in (False, True):
        with native.Chunk.from_deck(d) as c:
            out = []
            for _ in range(d.end_step):
                if fused:
                    info, s = c.tea_leaf_summary(opts, d.initial_timestep)
                else:
                    info = c.tea_leaf(opts, d.initial_timestep)
                    s = c.field_summary()
                out.append((info.reported_iterations, s))
            runs.append((out, c.download("energy1"), c.download("u")))
    (o0, e0, u0), (o1, e1, u1) = runs
    for (i0, s0), (i1, s1) in zip(o0, o1):
        assert i0 == i1
        np.testing.assert_array_equal(s0, s1)
    np.testing.assert_array_equal(e0, e1)
    np.testing.assert_array_equal(u0, u1)


def test_finalise_field_summary_entry_point():
    """tl_finalise_field_summary: the drop-in for tea_leaf_kernel_finalise followed by
    field_summary_kernel gives the bits of the two calls, and the oracle's summary to 1e-12."""
    from oracle import oracle
    from tealeaf_ref_gb300 import native

    d = small_deck(nx=97, ny=61, steps=1)
    o = oracle.Chunk.from_deck(d)
    o.common_init(d.initial_timestep)
    o.finalise()
    want = o.field_summary()
    res = []
    for fused in (False, True):
        with native.Chunk.from_deck(d) as c:
            c.common_init(d.initial_timestep)
            if fused:
                s = c.finalise_field_summary()
            else:
                c.finalise()
                s = c.field_summary()
            res.append((s, c.download("energy1")))
    np.testing.assert_array_equal(res[0][0], res[1][0])
    np.testing.assert_array_equal(res[0][1], res[1][1])
    assert np.max(np.abs(res[1][0] - want) / np.abs(want)) < 1e-12
