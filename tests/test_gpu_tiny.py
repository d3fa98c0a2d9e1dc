"""Degenerate mesh shapes on the GPU against the oracle: one-cell-wide and one-cell-high
chunks, 2x2 and a few cells, where a thread block, a warp strip, a row range or a 16-byte
vector covers more than the whole mesh.  Every solver, preconditioner, boundary mode and
precision form; field summary within 1e-10 and per-cell u within 1e-8 of the oracle."""
import numpy as np
import pytest

from helpers import small_deck
from tealeaf_ref_gb300 import deck as dk

pytestmark = pytest.mark.gpu

SIZES = [(2, 1), (1, 2), (1, 9), (9, 1), (2, 2), (3, 5), (31, 1), (1, 33), (6, 5)]

CASES = [
    dict(solver="cg"),
    dict(solver="cg", persistent="0"),
    dict(solver="cg", precond="jac_diag"),
    dict(solver="cg", precond="jac_block"),
    dict(solver="cg", reflective=True),
    dict(solver="cg", coefficient=dk.CONDUCTIVITY, halo_depth=2),
    dict(solver="chebyshev", ch_cg_presteps=20),
    dict(solver="ppcg", ppcg_inner_steps=4, ch_cg_presteps=20),
    dict(solver="jacobi", max_iters=5000, eps=1e-10),
    dict(solver="jacobi", max_iters=5000, eps=1e-10, reflective=True),
    dict(solver="cg", precision="mixed"),
    dict(solver="ppcg", ppcg_inner_steps=4, ch_cg_presteps=20, precision="mixed"),
    dict(solver="chebyshev", ch_cg_presteps=20, precision="mixed"),
]


def tiny_deck(nx, ny, **kw):
    """Ambient state, a rectangle over the lower left and a circle at the upper right: any
    mesh of two or more cells gets at least two different states."""
    d = small_deck(nx=nx, ny=ny, n_rect=0, n_circ=0, steps=2, **kw)
    d.states.append(dk.State(density=0.5, energy=10.0, geometry=1, xmin=0.0, xmax=4.0, ymin=0.0, ymax=6.5))
    d.states.append(dk.State(density=0.1, energy=25.0, geometry=2, xmin=7.5, ymin=7.0, radius=3.0))
    return d


@pytest.mark.parametrize("size", SIZES, ids=["%dx%d" % s for s in SIZES])
@pytest.mark.parametrize("case", CASES, ids=["-".join("%s%s" % kv for kv in c.items()) for c in CASES])
def test_tiny_mesh_against_oracle(size, case, monkeypatch):
    from oracle import oracle
    from tealeaf_ref_gb300 import native

    case = dict(case)
    precision = case.pop("precision", "fp64")
    if "persistent" in case:
        monkeypatch.setenv("TL_CG_PERSISTENT", case.pop("persistent"))
    d = tiny_deck(*size, **case)
    o = oracle.Chunk.from_deck(d)
    o_infos = [o.tea_leaf(d) for _ in range(d.end_step)]
    opts = native.opts_from_deck(d, precision=precision)
    with native.Chunk.from_deck(d) as c:
        g_infos = [c.tea_leaf(opts, d.initial_timestep) for _ in range(d.end_step)]
        summary = c.field_summary()
        u = c.download("u")
    u_ref = np.array(o.interior("u"))
    want = o.field_summary()
    assert np.all(np.abs(summary - want) <= 1e-10 * np.abs(want)), (summary, want)
    assert np.max(np.abs(u - u_ref) / np.abs(u_ref)) < 1e-8
    if precision == "fp64":
        for gi, oi in zip(g_infos, o_infos):
            slack = 10 if d.solver == "chebyshev" else 2
            assert abs(gi.reported_iterations - oi.reported_iterations) <= slack, (gi, oi)
