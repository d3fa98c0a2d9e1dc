"""The CPU adjoint (oracle/adjoint.py) that checks the GPU reverse sweep: its forward model
against the C oracle's tea_leaf() solves, its gradients against central finite differences."""
import numpy as np
import pytest

from helpers import small_deck


def _state(d):
    from oracle import oracle

    o = oracle.Chunk.from_deck(d)
    return np.array(o.interior("density")), np.array(o.interior("energy1"))


@pytest.mark.parametrize("coefficient", [1, 2])
def test_forward_model_matches_oracle_solves(coefficient):
    """u after three steps: exact sparse solves vs the oracle's CG at tl_eps 1e-15."""
    from oracle import adjoint, oracle

    d = small_deck(nx=23, ny=17, steps=3, n_rect=3, n_circ=1, coefficient=coefficient, max_iters=5000)
    rho, e0 = _state(d)
    dx, dy = (d.xmax - d.xmin) / d.x_cells, (d.ymax - d.ymin) / d.y_cells
    _, us = adjoint.forward(rho, e0, coefficient, dx, dy, d.initial_timestep, 3)
    o = oracle.Chunk.from_deck(d)
    for _ in range(3):
        o.tea_leaf(d)
    u = np.array(o.interior("u"))
    assert np.max(np.abs(u - us[-1])) <= 1e-11 * np.max(np.abs(u))


@pytest.mark.parametrize("coefficient", [1, 2])
def test_cpu_adjoint_matches_finite_differences(coefficient):
    """Every cell's dL/d density and dL/d energy0 against central differences, h = 1e-4
    relative.  One cell moves L by ~1e-10 of its value per unit relative step, so at h = 1e-6
    the rounding of the solves and of L (~1e-12 of L) leaves ~1e-5 relative noise in the
    difference quotient; at 1e-4 the noise and the O(h^2) truncation are both ~1e-8."""
    from oracle import adjoint

    d = small_deck(nx=11, ny=8, steps=3, n_rect=2, n_circ=1, coefficient=coefficient)
    rho, e0 = _state(d)
    dx, dy, dt = (d.xmax - d.xmin) / d.x_cells, (d.ymax - d.ymin) / d.y_cells, d.initial_timestep
    rng = np.random.Generator(np.random.PCG64(3))
    _, us = adjoint.forward(rho, e0, coefficient, dx, dy, dt, 3)
    target = us[-1] * (1.0 + 0.05 * rng.standard_normal(rho.shape))

    def loss(r, e):
        return adjoint.squared_error_loss(r, e, target, coefficient, dx, dy, dt, 3)[0]

    _, g_rho, g_e = adjoint.squared_error_loss(rho, e0, target, coefficient, dx, dy, dt, 3)
    for grad, base, which in ((g_rho, rho, 0), (g_e, e0, 1)):
        fd = np.zeros_like(base)
        for idx in np.ndindex(base.shape):
            # L is quadratic in energy (u is linear in it): central differences are exact
            # there for any step, so the energy step is sized by the field, not the cell
            h = 1e-4 * (abs(base[idx]) if which == 0 else float(np.max(np.abs(base))))
            p, m = base.copy(), base.copy()
            p[idx] += h
            m[idx] -= h
            lp = loss(p, e0) if which == 0 else loss(rho, p)
            lm = loss(m, e0) if which == 0 else loss(rho, m)
            fd[idx] = (lp - lm) / (2 * h)
        err = np.abs(fd - grad)
        assert np.all(err <= 1e-6 * np.abs(grad) + 1e-9 * np.max(np.abs(grad))), float(np.max(err / np.abs(grad)))
