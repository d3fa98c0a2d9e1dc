"""Per-kernel parity: each C-ABI entry point against the oracle's restatement of the same
reference subroutine, on odd-sized grids (every strip / block edge path), for both
coefficient keywords, all three preconditioners and reflective boundaries.

Tolerances: set-up arithmetic (generation, Kx/Ky, Di) is bit-exact; one application of
the pre-scaled 5-point operator differs from the reference's unscaled, unfused form by a
few ulp of the largest term, so fields are compared norm-wise at 1e-12.  Reductions are
compared at max(1e-12, 4e-16 * n) relative for n summed terms: the oracle sums
sequentially, as the reference does, and that order carries up to ~n*eps of rounding error
(the GPU's two-level tree sum is closer to the exact value)."""
import numpy as np
import pytest

from helpers import oracle_field, pair, rel_inf, small_deck

pytestmark = pytest.mark.gpu

TOL = 1e-12


def red_tol(d):
    return max(TOL, 4e-16 * d.x_cells * d.y_cells)


CASES = [
    dict(nx=37, ny=23),
    dict(nx=64, ny=64, coefficient=1),
    dict(nx=300, ny=9, precond="jac_diag"),
    dict(nx=19, ny=41, precond="jac_block"),
    dict(nx=33, ny=17, reflective=True),
    dict(nx=513, ny=130, n_rect=6, n_circ=3),
]


def _ids(c):
    return "-".join("%s%s" % (k, v) for k, v in c.items())


@pytest.mark.parametrize("case", CASES, ids=[_ids(c) for c in CASES])
def test_generate_and_common_init(case):
    d = small_deck(**case)
    o, g = pair(d)
    for f in ("density", "energy1", "u"):
        np.testing.assert_array_equal(g.download(f), oracle_field(o, f), err_msg=f)
    o.common_init(d.initial_timestep)
    g.common_init(d.initial_timestep)
    for f in ("kx", "ky", "di", "u", "u0"):
        np.testing.assert_array_equal(g.download(f), oracle_field(o, f), err_msg=f)
    if d.preconditioner == "jac_diag":
        np.testing.assert_array_equal(g.download("mi"), oracle_field(o, "mi"))
    for f in ("w", "r"):
        assert rel_inf(g.download(f), oracle_field(o, f)) < TOL, f


@pytest.mark.parametrize("case", CASES, ids=[_ids(c) for c in CASES])
def test_cg_kernels(case):
    d = small_deck(**case)
    o, g = pair(d)
    dt = d.initial_timestep
    o.common_init(dt)
    g.common_init(dt)
    halo = ["u"]
    o.update_halo(halo, 1)
    g.update_halo(halo, 1)
    o.calc_residual()
    g.calc_residual()
    assert rel_inf(g.download("r"), oracle_field(o, "r")) < TOL
    for which in (0, 1):
        a, b = g.calc_2norm(which), o.calc_2norm(which)
        assert abs(a - b) <= red_tol(d) * abs(b)
    rro_g, rro_o = g.cg_init(), o.cg_init()
    assert abs(rro_g - rro_o) <= red_tol(d) * abs(rro_o)
    o.update_halo(["u", "p"], 1)
    g.update_halo(["u", "p"], 1)
    rro = rro_o
    for it in range(3):
        pw_g, pw_o = g.cg_calc_w(), o.cg_calc_w()
        assert abs(pw_g - pw_o) <= red_tol(d) * abs(pw_o), it
        assert rel_inf(g.download("w"), oracle_field(o, "w")) < TOL
        alpha = rro / pw_o
        rrn_g, rrn_o = g.cg_calc_ur(alpha), o.cg_calc_ur(alpha)
        assert abs(rrn_g - rrn_o) <= max(1e-11, red_tol(d)) * abs(rrn_o), it
        for f in ("u", "r"):
            assert rel_inf(g.download(f), oracle_field(o, f)) < 1e-11, f
        beta = rrn_o / rro
        g.cg_calc_p(beta)
        o.cg_calc_p(beta, 0)
        assert rel_inf(g.download("p"), oracle_field(o, "p")) < 1e-11
        o.update_halo(["p"], 1)
        g.update_halo(["p"], 1)
        rro = rrn_o
        # re-sync the GPU state to the oracle so later iterations compare kernels, not drift
        for f in ("u", "r", "p", "z"):
            g.upload(f, oracle_field(o, f))
        g.update_halo(["p"], 1)


@pytest.mark.parametrize("case", CASES[:5], ids=[_ids(c) for c in CASES[:5]])
def test_cheby_ppcg_jacobi_kernels(case):
    d = small_deck(**case)
    o, g = pair(d)
    dt = d.initial_timestep
    o.common_init(dt)
    g.common_init(dt)
    o.calc_residual()
    g.calc_residual()
    theta, a, b = 3.7, 0.61, 0.23
    o.cheby_init(theta)
    g.cheby_init(theta)
    for f in ("w", "r", "p", "u"):
        assert rel_inf(g.download(f), oracle_field(o, f)) < TOL, f
    o.update_halo(["u"], 1)
    g.update_halo(["u"], 1)
    o.cheby_iterate(a, b)
    g.cheby_iterate(a, b)
    for f in ("w", "r", "p", "u"):
        assert rel_inf(g.download(f), oracle_field(o, f)) < 1e-11, f
    # PPCG pieces
    for f in ("u", "r", "p", "w"):
        g.upload(f, oracle_field(o, f))
    for step in (1, 2, 3):
        ro, rg = o.ppcg_init(step, 1), g.ppcg_init(step, True)
        assert abs(rg - ro) <= TOL * max(abs(ro), 1e-300), step
        assert rel_inf(g.download("p"), oracle_field(o, "p")) < TOL
    o.ppcg_init_sd(theta)
    g.ppcg_init_sd(theta)
    for f in ("sd", "rtemp", "utemp"):
        assert rel_inf(g.download(f), oracle_field(o, f)) < TOL, f
    for _ in range(2):
        o.update_halo(["sd", "r"], 1)
        g.update_halo(["sd", "r"], 1)
        o.ppcg_inner(a, b)
        g.ppcg_inner(a, b)
        for f in ("sd", "rtemp", "utemp"):
            assert rel_inf(g.download(f), oracle_field(o, f)) < 1e-11, f
        for f in ("sd", "rtemp", "utemp", "z"):
            g.upload(f, oracle_field(o, f))
    o.ppcg_update_z()
    g.ppcg_update_z()
    np.testing.assert_array_equal(g.download("z"), oracle_field(o, "z"))
    o.ppcg_store_r()
    g.ppcg_store_r()
    np.testing.assert_array_equal(g.download("r_store"), oracle_field(o, "r_store"))
    zr_g, zr_o = g.ppcg_calc_zrnorm(True), o.ppcg_calc_zrnorm(1)
    assert abs(zr_g - zr_o) <= red_tol(d) * abs(zr_o)
    # perturb r so that (r - r_store).z is not zero
    r = oracle_field(o, "r") * 1.001
    o.interior("r")[...] = r
    g.upload("r", r)
    rr_g, rr_o = g.ppcg_calc_rrn(), o.ppcg_calc_rrn()
    assert abs(rr_g - rr_o) <= max(1e-10, red_tol(d)) * abs(rr_o)
    # Jacobi
    for f in ("u",):
        g.upload(f, oracle_field(o, f))
    e_g, e_o = g.jacobi_solve(), o.jacobi_solve()
    assert abs(e_g - e_o) <= max(1e-11, red_tol(d)) * abs(e_o)
    # the reference's operation order and a correctly rounded quotient: the same bits
    np.testing.assert_array_equal(g.download("u"), oracle_field(o, "u"))


@pytest.mark.parametrize("case", CASES, ids=[_ids(c) for c in CASES])
def test_finalise_and_field_summary(case):
    d = small_deck(**case)
    o, g = pair(d)
    so, sg = o.field_summary(), g.field_summary()
    np.testing.assert_allclose(sg, so, rtol=max(1e-13, red_tol(d)))
    o.common_init(d.initial_timestep)
    g.common_init(d.initial_timestep)
    o.finalise()
    g.finalise()
    np.testing.assert_array_equal(g.download("energy1"), oracle_field(o, "energy1"))


def test_reflective_halo_update():
    d = small_deck(nx=21, ny=13, reflective=True)
    o, g = pair(d)
    o.common_init(d.initial_timestep)
    g.common_init(d.initial_timestep)
    # the reflective copy only changes halo cells; check its effect through the operator
    o.update_halo(["u"], 1)
    g.update_halo(["u"], 1)
    o.calc_residual()
    g.calc_residual()
    assert rel_inf(g.download("r"), oracle_field(o, "r")) < TOL


def test_errors_are_reported():
    from tealeaf_ref_gb300 import native
    with pytest.raises(native.TeaLeafError) as e:
        native.Chunk(0, 10)
    assert e.value.code == -1
    with pytest.raises(native.TeaLeafError):
        native.Chunk(10, 10, coefficient=3)
    with pytest.raises(native.TeaLeafError):
        native.Chunk(10, 10, halo_depth=2, precond=3)
    c = native.Chunk(8, 8, dx=1.0, dy=1.0)
    with pytest.raises(native.TeaLeafError):
        c.calc_2norm(2)
    with pytest.raises(native.TeaLeafError):
        c.ppcg_init(4, False)
