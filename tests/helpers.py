"""Shared helpers for the parity tests: the same deck on the CPU oracle and on the GPU."""
from __future__ import annotations

import numpy as np

from tealeaf_ref_gb300 import deck as dk


def small_deck(nx=37, ny=23, solver="cg", coefficient=dk.RECIP_CONDUCTIVITY, precond="none", reflective=False,
               halo_depth=1, seed=7, n_rect=3, n_circ=2, max_iters=2000, steps=2, eps=1e-15, **kw) -> dk.Deck:
    d = dk.seeded_deck(nx, n_rect, n_circ, seed, steps=steps, max_iters=max_iters, solver=solver, eps=eps,
                       coefficient=coefficient)
    d.y_cells = ny
    d.preconditioner = precond
    d.reflective_boundary = reflective
    d.halo_depth = halo_depth
    for k, v in kw.items():
        setattr(d, k, v)
    return d


def rel_inf(a: np.ndarray, b: np.ndarray) -> float:
    """max |a-b| / max |b| (norm-wise relative difference)."""
    scale = float(np.max(np.abs(b))) or 1.0
    return float(np.max(np.abs(a - b))) / scale


def pair(deck):
    """(oracle chunk, gpu chunk) generated from the same deck."""
    from oracle import oracle
    from tealeaf_ref_gb300 import native

    o = oracle.Chunk.from_deck(deck)
    g = native.Chunk.from_deck(deck)
    return o, g


GPU_FIELDS = ["density", "energy1", "u", "u0", "r", "w", "p", "z", "kx", "ky", "di", "mi", "sd", "utemp", "rtemp",
              "r_store"]


def oracle_field(o, name):
    return np.array(o.interior(name))


def exact_summary(o) -> np.ndarray:
    """The oracle's field summary (vol, mass, ie, temp; field_summary_kernel.f90:44-62) with
    every product rounded as the oracle rounds it and each sum correctly rounded (math.fsum).
    The oracle's own serial sums over millions of cells carry a rounding error that grows with
    the cell count (2e-10 relative for the mass at 8192^2), which the GPU's tree sums do not
    share; comparing with the correctly rounded sums keeps the 1e-10 bar about the fields."""
    import math

    dx, dy = o.geometry()[:2]
    vol = dx * dy
    rho = np.array(o.interior("density"))
    mass = vol * rho
    ie = mass * np.array(o.interior("energy1"))
    temp = mass * np.array(o.interior("u"))
    return np.array([math.fsum(np.full(rho.size, vol)), math.fsum(mass.ravel()), math.fsum(ie.ravel()),
                     math.fsum(temp.ravel())])
