"""The GPU reverse sweep (tl_adjoint_*) through the C ABI: against the FP64 CPU adjoint
(oracle/adjoint.py), against central finite differences of the GPU forward solves, and
through the torch.autograd binding."""
import numpy as np
import pytest

from helpers import rel_inf, small_deck

pytestmark = pytest.mark.gpu


def _geom(d):
    return (d.xmax - d.xmin) / d.x_cells, (d.ymax - d.ymin) / d.y_cells, d.initial_timestep


def _problem(d):
    """GPU chunk, its generated density/energy, and the target u: the CPU forward from the
    density perturbed by 1% N(0,1) (seed 4)."""
    from oracle import adjoint
    from tealeaf_ref_gb300 import native
    from tealeaf_ref_gb300.adjoint import perturbed_density

    c = native.Chunk.from_deck(d)
    rho, e0 = c.download("density"), c.download("energy1")
    dx, dy, dt = _geom(d)
    _, us = adjoint.forward(perturbed_density(rho, 4), e0, d.coefficient, dx, dy, dt, d.end_step)
    return c, rho, e0, us[-1]


CASES = [
    dict(),
    dict(coefficient=1),
    dict(recompute=True),
    dict(reflective=True),
    dict(nx=96, ny=41, n_rect=5, n_circ=2),
]


@pytest.mark.parametrize("case", CASES, ids=["-".join("%s%s" % kv for kv in c.items()) or "default" for c in CASES])
def test_adjoint_matches_cpu_adjoint(case):
    from oracle import adjoint
    from tealeaf_ref_gb300 import native
    from tealeaf_ref_gb300.adjoint import squared_error_gradient

    case = dict(case)
    recompute = case.pop("recompute", False)
    kw = dict(nx=57, ny=43, steps=3, n_rect=4, n_circ=1, max_iters=20000)
    kw.update(case)
    d = small_deck(**kw)
    c, rho, e0, target = _problem(d)
    with c:
        loss, g_rho, g_e, info = squared_error_gradient(c, rho, e0, target, native.opts_from_deck(d),
                                                        d.initial_timestep, d.end_step, recompute=recompute)
    dx, dy, dt = _geom(d)
    loss_c, gc_rho, gc_e = adjoint.squared_error_loss(rho, e0, target, d.coefficient, dx, dy, dt, d.end_step)
    assert abs(loss - loss_c) <= 1e-9 * loss_c
    assert rel_inf(g_rho, gc_rho) <= 1e-9
    assert rel_inf(g_e, gc_e) <= 1e-9
    assert info.reported_iterations > 0


def test_adjoint_energy_seed():
    """A loss on the final energy1 (e_bar seed, no u_bar) against the CPU adjoint."""
    from oracle import adjoint
    from tealeaf_ref_gb300 import native

    d = small_deck(nx=40, ny=33, steps=2, n_rect=3, n_circ=1, max_iters=20000)
    c, rho, e0, _ = _problem(d)
    with c:
        c.adjoint_begin(d.end_step)
        for _ in range(d.end_step):
            c.record_step(native.opts_from_deck(d), d.initial_timestep)
        e_final = c.download("energy1")
        g_rho, g_e, _ = c.adjoint_backward(None, 2.0 * e_final)
    dx, dy, dt = _geom(d)
    es, us = adjoint.forward(rho, e0, d.coefficient, dx, dy, dt, d.end_step)
    gc_rho, gc_e = adjoint.backward(rho, es, us, d.coefficient, dx, dy, dt, e_bar=2.0 * us[-1] / rho)
    assert rel_inf(g_rho, gc_rho) <= 1e-9
    assert rel_inf(g_e, gc_e) <= 1e-9


def test_adjoint_matches_finite_differences():
    """dL/d density at 16 seeded cells against central differences of the GPU forward solves
    (h = 1e-4 relative: at smaller steps the solves' rounding, ~1e-12 of L, dominates the
    ~1e-10 change of L that one cell makes)."""
    from tealeaf_ref_gb300 import native
    from tealeaf_ref_gb300.adjoint import forward_loss, squared_error_gradient

    d = small_deck(nx=64, ny=64, steps=3, n_rect=4, n_circ=1, max_iters=20000)
    c, rho, e0, target = _problem(d)
    opts = native.opts_from_deck(d)
    with c:
        _, g_rho, _, _ = squared_error_gradient(c, rho, e0, target, opts, d.initial_timestep, d.end_step,
                                                rho_only=True)
        rng = np.random.Generator(np.random.PCG64(4))
        cells = [tuple(x) for x in np.stack([rng.integers(0, d.y_cells, 16), rng.integers(0, d.x_cells, 16)], 1)]
        gmax = float(np.max(np.abs(g_rho)))
        for idx in cells:
            h = 1e-4 * rho[idx]
            p, m = rho.copy(), rho.copy()
            p[idx] += h
            m[idx] -= h
            fd = (forward_loss(c, p, e0, target, opts, d.initial_timestep, d.end_step) -
                  forward_loss(c, m, e0, target, opts, d.initial_timestep, d.end_step)) / (2 * h)
            assert abs(fd - g_rho[idx]) <= 1e-6 * abs(g_rho[idx]) + 1e-9 * gmax, (idx, fd, g_rho[idx])


def test_torch_autograd_function():
    torch = pytest.importorskip("torch")
    from tealeaf_ref_gb300 import native
    from tealeaf_ref_gb300.adjoint import squared_error_gradient, tea_leaf_steps

    d = small_deck(nx=48, ny=36, steps=2, n_rect=3, n_circ=1, max_iters=20000)
    c, rho, e0, target = _problem(d)
    opts = native.opts_from_deck(d)
    with c:
        density = torch.tensor(rho, requires_grad=True)
        energy = torch.tensor(e0, requires_grad=True)
        u = tea_leaf_steps(density, energy, c, opts, d.initial_timestep, d.end_step)
        loss = ((u - torch.from_numpy(target)) ** 2).sum()
        loss.backward()
        loss_ref, g_rho, g_e, _ = squared_error_gradient(c, rho, e0, target, opts, d.initial_timestep, d.end_step)
    assert abs(float(loss) - loss_ref) <= 1e-14 * loss_ref
    assert rel_inf(density.grad.numpy(), g_rho) <= 1e-14
    assert rel_inf(energy.grad.numpy(), g_e) <= 1e-14


def test_adjoint_zero_seed_and_state_errors():
    from tealeaf_ref_gb300 import native

    d = small_deck(nx=20, ny=16, steps=2, n_rect=2, n_circ=0, max_iters=5000)
    opts = native.opts_from_deck(d)
    with native.Chunk.from_deck(d) as c:
        with pytest.raises(native.TeaLeafError) as e:
            c.adjoint_backward(np.zeros((16, 20)))
        assert e.value.code == -7  # TL_ERR_STATE: nothing recorded
        c.adjoint_begin(1)
        c.record_step(opts, d.initial_timestep)
        with pytest.raises(native.TeaLeafError) as e:
            c.record_step(opts, d.initial_timestep)
        assert e.value.code == -7  # tape full
        g_rho, g_e, info = c.adjoint_backward(np.zeros((16, 20)))
        assert not np.any(g_rho) and not np.any(g_e)
        c.adjoint_end()
        with pytest.raises(native.TeaLeafError):
            c.adjoint_begin(0)
