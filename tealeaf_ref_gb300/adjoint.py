"""Differentiable time stepping: a torch.autograd.Function over the C ABI's adjoint entry
points (tl_adjoint_begin / tl_adjoint_record_step / tl_adjoint_backward).

forward: (density, energy0) -> u after `nsteps` tea_leaf() time steps on a Chunk, each
step recorded on the tape (its input energy1, and its solution u unless recompute=True, in
which case the reverse sweep re-solves each step from its input energy1).
backward: dL/du -> (dL/d density, dL/d energy0) by the reverse sweep on the GPU.

Tensors cross as host float64 arrays (the C ABI takes plain pointers); results come back on
the input's device.
"""
from __future__ import annotations

from typing import Optional

import numpy as np

from . import native


def _host(t) -> np.ndarray:
    return np.ascontiguousarray(t.detach().to("cpu", dtype=_torch().float64).numpy())


def _torch():
    import torch

    return torch


def perturbed_density(density: np.ndarray, seed: int = 4, scale: float = 0.01) -> np.ndarray:
    """density * (1 + scale * N(0,1)) per cell, from numpy's PCG64 stream with ``seed``: the
    density of the forward run that makes the target field of the adjoint problem."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return density * (1.0 + scale * rng.standard_normal(density.shape))


def _make_function():
    torch = _torch()

    class TeaLeafSteps(torch.autograd.Function):
        @staticmethod
        def forward(ctx, density, energy0, chunk, opts, dt, nsteps, recompute):
            chunk.upload_state(_host(density), _host(energy0))
            chunk.adjoint_begin(nsteps, store_solutions=not recompute)
            infos = [chunk.record_step(opts, dt) for _ in range(nsteps)]
            u = chunk.download("u")
            ctx.chunk = chunk
            ctx.infos = infos
            return torch.from_numpy(u).to(density.device)

        @staticmethod
        def backward(ctx, u_bar):
            rho_bar, e0_bar, info = ctx.chunk.adjoint_backward(_host(u_bar))
            ctx.chunk.reverse_info = info
            dev = u_bar.device
            return (torch.from_numpy(rho_bar).to(dev), torch.from_numpy(e0_bar).to(dev), None, None, None, None,
                    None)

    return TeaLeafSteps


_FN = None


def tea_leaf_steps(density, energy0, chunk: "native.Chunk", opts: "native.SolveOpts", dt: float, nsteps: int,
                   recompute: bool = False):
    """u after ``nsteps`` time steps from (density, energy0), differentiable in both (float64
    tensors of shape (y_cells, x_cells)).  The chunk's fields are overwritten."""
    global _FN
    if _FN is None:
        _FN = _make_function()
    return _FN.apply(density, energy0, chunk, opts, dt, nsteps, recompute)


def squared_error_gradient(chunk: "native.Chunk", density: np.ndarray, energy0: np.ndarray, u_target: np.ndarray,
                           opts: "native.SolveOpts", dt: float, nsteps: int, recompute: bool = False,
                           rho_only: bool = False):
    """L = sum (u_final - u_target)^2 and (dL/d density, dL/d energy0, reverse SolveInfo),
    through the C ABI without torch."""
    chunk.upload_state(density, energy0)
    chunk.adjoint_begin(nsteps, store_solutions=not recompute)
    for _ in range(nsteps):
        chunk.record_step(opts, dt)
    diff = chunk.download("u") - u_target
    rho_bar, e0_bar, info = chunk.adjoint_backward(2.0 * diff, want_energy0=not rho_only)
    return float(np.sum(diff * diff)), rho_bar, e0_bar, info


def forward_loss(chunk: "native.Chunk", density: np.ndarray, energy0: np.ndarray, u_target: np.ndarray,
                 opts: "native.SolveOpts", dt: float, nsteps: int, out: Optional[np.ndarray] = None) -> float:
    """L = sum (u_final - u_target)^2 of a plain forward run (no tape)."""
    chunk.upload_state(density, energy0)
    for _ in range(nsteps):
        chunk.tea_leaf(opts, dt)
    diff = chunk.download("u", out=out) - u_target
    return float(np.sum(diff * diff))
