"""The host math of the CG -> Chebyshev / PPCG switch in the product library (no GPU): the
Lanczos eigenvalue estimate against numpy and the Chebyshev coefficients against the recurrence
of tea_leaf_cheby.f90:178-205 evaluated in Python."""
import numpy as np
import pytest

from tealeaf_ref_gb300 import native


def _tridiag(alphas, betas):
    n = alphas.size
    d = 1.0 / alphas
    d[1:] += betas[:-1] / alphas[:-1]
    off = np.sqrt(betas[:-1]) / alphas[:-1]
    return np.diag(d) + np.diag(off, 1) + np.diag(off, -1)


@pytest.mark.parametrize("n,seed", [(1, 0), (2, 1), (7, 2), (40, 3), (400, 4)])
def test_cg_eigenvalues_match_numpy(n, seed):
    rng = np.random.default_rng(seed)
    alphas = rng.uniform(0.05, 2.0, n)
    betas = rng.uniform(0.01, 0.9, n)
    lo, hi = native.cg_eigenvalues(alphas, betas)
    ev = np.linalg.eigvalsh(_tridiag(alphas, betas))
    assert abs(lo - ev[0]) <= 1e-12 * max(1.0, abs(ev[-1]))
    assert abs(hi - ev[-1]) <= 1e-12 * abs(ev[-1])


def test_cg_eigenvalues_of_a_real_cg_run():
    """Coefficients of CG on a 1-D Laplacian-like SPD matrix give eigenvalue bounds inside its
    spectrum (Ritz values) close to the extremes."""
    n = 60
    A = np.diag(np.full(n, 2.5)) + np.diag(np.full(n - 1, -1.0), 1) + np.diag(np.full(n - 1, -1.0), -1)
    b = np.random.default_rng(9).random(n)
    x = np.zeros(n)
    r = b.copy()
    p = r.copy()
    rr = r @ r
    al, be = [], []
    for _ in range(n):
        w = A @ p
        alpha = rr / (p @ w)
        x += alpha * p
        r -= alpha * w
        rrn = r @ r
        beta = rrn / rr
        al.append(alpha)
        be.append(beta)
        p = r + beta * p
        rr = rrn
        if rrn < 1e-28:
            break
    lo, hi = native.cg_eigenvalues(np.array(al), np.array(be))
    ev = np.linalg.eigvalsh(A)
    assert ev[0] - 1e-9 <= lo <= ev[0] * 1.01
    assert ev[-1] * 0.99 <= hi <= ev[-1] + 1e-9


def test_cg_eigenvalues_failure_is_reported():
    with pytest.raises(native.TeaLeafError) as e:
        native.cg_eigenvalues(np.array([-1.0, -2.0]), np.array([0.5, 0.5]))
    assert e.value.code == -6  # TL_ERR_EIGEN


def test_cheby_coefficients_recurrence():
    eigmin, eigmax, n = 0.013, 7.9, 25
    theta, a, b = native.cheby_coefficients(eigmin, eigmax, n)
    t = (eigmax + eigmin) / 2
    delta = (eigmax - eigmin) / 2
    sigma = t / delta
    rho_old = 1.0 / sigma
    assert theta == t
    for i in range(n):
        rho_new = 1.0 / (2.0 * sigma - rho_old)
        assert a[i] == rho_new * rho_old
        assert b[i] == 2.0 * rho_new / delta
        rho_old = rho_new
