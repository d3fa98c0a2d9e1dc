"""The FP64 CG matvec sweep with its input rows staged one row ahead in shared memory and its
products Di p on the integer pipes (the default), and the staged sweep with FP64 products
(TL_CG_EMU=0), against the sweep with direct loads (TL_CG_STAGE=0): the same bits in u, r,
p and w, the same iteration counts and error.  Meshes are chosen for
the staging's edges: several strips, a last strip a few columns wide, an odd width (a thread
with one column), a mesh narrower than one strip, reflective boundaries, jac_diag and the
PPCG variant of the sweep; and a 4000^2 mesh, where a warp's row step is long enough for a
neighbouring warp to run a row step ahead (what would expose a ring entry written by one
thread and read by another)."""
import numpy as np
import pytest

from helpers import small_deck

pytestmark = pytest.mark.gpu

DECKS = {
    "cg_1030x700": dict(nx=1030, ny=700, max_iters=300, steps=1),
    "cg_4000x4000": dict(nx=4000, ny=4000, max_iters=200, steps=1),
    "cg_1031x517_odd": dict(nx=1031, ny=517, max_iters=200, steps=1),
    "cg_jac_diag_600x433": dict(nx=600, ny=433, precond="jac_diag", max_iters=200, steps=1),
    "cg_reflective_300x211": dict(nx=300, ny=211, reflective=True, max_iters=200, steps=1),
    "cg_narrow_97x300": dict(nx=97, ny=300, max_iters=150, steps=1),
    "ppcg_1030x700": dict(nx=1030, ny=700, solver="ppcg", ppcg_inner_steps=10, ch_cg_presteps=20,
                          ch_cg_epslim=1e30, max_iters=40, steps=1),
}


@pytest.mark.parametrize("name", list(DECKS))
def test_staged_sweep_gives_the_same_bits(name, monkeypatch):
    from tealeaf_ref_gb300 import native

    d = small_deck(**DECKS[name])
    monkeypatch.setenv("TL_CG_PERSISTENT", "0")  # the fused sweeps at every mesh size
    runs = {}
    for mode in ("0", "1e0", "1e1"):
        monkeypatch.setenv("TL_CG_STAGE", mode[0])
        monkeypatch.setenv("TL_CG_EMU", mode[2:] or "0")
        with native.Chunk.from_deck(d) as c:
            i = c.tea_leaf(d)
            runs[mode] = (i.reported_iterations, i.error, {f: c.download(f) for f in ("u", "r", "p", "w")})
    its0, err0, f0 = runs["0"]
    assert its0 > 10
    for mode in ("1e0", "1e1"):
        its, err, f = runs[mode]
        assert its == its0 and err == err0, (mode, its, its0, err, err0)
        for k in f0:
            assert np.array_equal(f[k].view(np.uint64), f0[k].view(np.uint64)), (mode, k)
