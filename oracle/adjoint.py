"""FP64 CPU forward model and adjoint of a run of tea_leaf() time steps.

TEST INFRASTRUCTURE ONLY: imported by tests/ and bench.py's adjoint check as the checker
of the GPU adjoint (tl_adjoint_*).  The product (tealeaf_ref_gb300) never imports it.

The reference has no adjoint; this module restates the forward step of the reference and
differentiates it by hand.  One time step on one chunk (every face external):

  b = energy1 * density                         (tea_leaf_common_kernel.f90:67-72)
  Kx(j) = (w(j-1) + w(j)) / (2 w(j-1) w(j))     (:94-101), w = density (coefficient 1) or
                                                1/density (coefficient 2, :75-92); external
                                                faces zero (:104-141)
  A u = u + sum over interior faces f=(L,R) of c_f (u_L - u_R) on both cells, c_f = rx Kx_f
        or ry Ky_f, rx = dt/dx^2, ry = dt/dy^2 (the operator of :208-244 with Di of :144-152)
  energy1' = u / density                        (tea_leaf_kernel_finalise, :179-206)

The linear systems are solved exactly (sparse LU), so this is the gradient of the exact-solve
map, the same quantity the GPU reverse sweep computes.
"""
from __future__ import annotations

from typing import List, Optional, Tuple

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def _w(density: np.ndarray, coefficient: int) -> np.ndarray:
    return density if coefficient == 1 else 1.0 / density


def face_coefficients(density: np.ndarray, coefficient: int) -> Tuple[np.ndarray, np.ndarray]:
    """Interior-face Kx (ny, nx-1) between columns j, j+1 and Ky (ny-1, nx) between rows."""
    w = _w(density, coefficient)
    kx = (w[:, :-1] + w[:, 1:]) / (2.0 * w[:, :-1] * w[:, 1:])
    ky = (w[:-1, :] + w[1:, :]) / (2.0 * w[:-1, :] * w[1:, :])
    return kx, ky


def operator(density: np.ndarray, coefficient: int, rx: float, ry: float) -> sp.csc_matrix:
    """A as a sparse matrix over the interior cells (row-major, x fastest)."""
    ny, nx = density.shape
    kx, ky = face_coefficients(density, coefficient)
    cx, cy = rx * kx, ry * ky
    idx = np.arange(nx * ny).reshape(ny, nx)
    diag = np.ones((ny, nx))
    diag[:, :-1] += cx
    diag[:, 1:] += cx
    diag[:-1, :] += cy
    diag[1:, :] += cy
    le, ri = idx[:, :-1].ravel(), idx[:, 1:].ravel()
    bo, to = idx[:-1, :].ravel(), idx[1:, :].ravel()
    rows = np.concatenate([idx.ravel(), le, ri, bo, to])
    cols = np.concatenate([idx.ravel(), ri, le, to, bo])
    vals = np.concatenate([diag.ravel(), -cx.ravel(), -cx.ravel(), -cy.ravel(), -cy.ravel()])
    return sp.csc_matrix((vals, (rows, cols)), shape=(nx * ny, nx * ny))


def forward(density: np.ndarray, energy0: np.ndarray, coefficient: int, dx: float, dy: float, dt: float,
            nsteps: int) -> Tuple[List[np.ndarray], List[np.ndarray]]:
    """Input energies e_t and solutions u_t of nsteps time steps."""
    lu = spla.splu(operator(density, coefficient, dt / (dx * dx), dt / (dy * dy)))
    es, us = [], []
    e = energy0
    for _ in range(nsteps):
        es.append(e)
        u = lu.solve((e * density).ravel()).reshape(e.shape)
        us.append(u)
        e = u / density
    return es, us


def backward(density: np.ndarray, es: List[np.ndarray], us: List[np.ndarray], coefficient: int, dx: float,
             dy: float, dt: float, u_bar: Optional[np.ndarray] = None,
             e_bar: Optional[np.ndarray] = None) -> Tuple[np.ndarray, np.ndarray]:
    """(dL/d density, dL/d energy0) for dL/du_final = u_bar and dL/d energy_final = e_bar."""
    rx, ry = dt / (dx * dx), dt / (dy * dy)
    lu = spla.splu(operator(density, coefficient, rx, ry))
    w = _w(density, coefficient)
    dw = np.ones_like(density) if coefficient == 1 else -1.0 / (density * density)
    rho_bar = np.zeros_like(density)
    eb = np.zeros_like(density) if e_bar is None else np.array(e_bar, dtype=np.float64)
    T = len(es)
    for t in range(T - 1, -1, -1):
        u = us[t]
        ub = eb / density
        if t == T - 1 and u_bar is not None:
            ub = ub + u_bar
        rho_bar -= eb * u / (density * density)
        lam = lu.solve(ub.ravel(), trans="T").reshape(u.shape)
        kxb = -rx * (lam[:, :-1] - lam[:, 1:]) * (u[:, :-1] - u[:, 1:])
        kyb = -ry * (lam[:-1, :] - lam[1:, :]) * (u[:-1, :] - u[1:, :])
        wb = np.zeros_like(density)
        wb[:, :-1] += kxb * (-0.5 / (w[:, :-1] ** 2))
        wb[:, 1:] += kxb * (-0.5 / (w[:, 1:] ** 2))
        wb[:-1, :] += kyb * (-0.5 / (w[:-1, :] ** 2))
        wb[1:, :] += kyb * (-0.5 / (w[1:, :] ** 2))
        rho_bar += lam * es[t] + wb * dw
        eb = lam * density
    return rho_bar, eb


def squared_error_loss(density, energy0, u_target, coefficient, dx, dy, dt, nsteps):
    """L = sum (u_final - u_target)^2, and its gradients (L, dL/d density, dL/d energy0)."""
    es, us = forward(density, energy0, coefficient, dx, dy, dt, nsteps)
    diff = us[-1] - u_target
    rho_bar, e0_bar = backward(density, es, us, coefficient, dx, dy, dt, u_bar=2.0 * diff)
    return float(np.sum(diff * diff)), rho_bar, e0_bar
