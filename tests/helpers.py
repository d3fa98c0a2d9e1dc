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
