"""The integer-pipe FP64 multiply on the GPU (csrc/tl_fp64emu.cuh).

* dmul_int against mul.rn.f64 on the same seeded operands of every class, through the
  diagnostic entry tl_fp64_emu_check: the same bits (any NaN for a NaN).
* The FP64 Jacobi sweep with some or all of its seven products on the integer pipes
  (TL_JACOBI_INT) against the sweep with FP64 multiplies only: the same bits in u and the
  same iteration counts and error, on meshes with several CTAs per row and reflective
  boundaries.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import small_deck

pytestmark = pytest.mark.gpu

SIGN = np.uint64(1 << 63)
FRAC = np.uint64((1 << 52) - 1)


def _operands(n, seed):
    g = np.random.Generator(np.random.PCG64(seed))

    def with_exp(e):
        m = g.integers(0, 2**64, n, dtype=np.uint64) & (FRAC | SIGN)
        return (m | (np.asarray(e, dtype=np.uint64) << np.uint64(52))).view(np.float64)

    classes = [
        lambda: g.integers(0, 2**64, n, dtype=np.uint64).view(np.float64),  # any class
        lambda: with_exp(g.integers(983, 1063, n)),                          # normal, narrow range
        lambda: with_exp(g.integers(0, 2047, n)),                            # any exponent
        lambda: with_exp(np.where(g.integers(0, 2, n) == 1, g.integers(1, 41, n), g.integers(2006, 2047, n))),
    ]
    a = np.empty(n)
    b = np.empty(n)
    k = g.integers(0, len(classes), n)
    for i, draw in enumerate(classes):
        sel = k == i
        a[sel], b[sel] = draw()[sel], draw()[sel]
    # few significand bits: exact products and ties
    few = g.integers(0, 5, n) == 0
    for x in (a, b):
        u = x.view(np.uint64)
        drop = g.integers(0, 53, n).astype(np.uint64)
        mask = ~((np.uint64(1) << drop) - np.uint64(1))
        u[few] = (u[few] & ~FRAC) | (u[few] & FRAC & mask[few])
    a[g.integers(0, 17, n) == 0] = -0.0
    return a, b


def _same(x, y):
    return (x.view(np.uint64) == y.view(np.uint64)) | (np.isnan(x) & np.isnan(y))


def test_integer_multiply_matches_fp64_instruction():
    from tealeaf_ref_gb300 import native

    lib = native.load()
    n = 1 << 22
    ptr = lambda x: x.ctypes.data_as(C.POINTER(C.c_double))
    for seed in (11, 12):
        a, b = _operands(n, seed)
        emu, hw = np.empty(n), np.empty(n)
        assert lib.tl_fp64_emu_check(ptr(a), ptr(b), n, ptr(emu), ptr(hw)) == 0
        ok = _same(emu, hw)
        bad = np.flatnonzero(~ok)[:5]
        assert ok.all(), [(a[i].hex(), b[i].hex(), hw[i].hex(), emu[i].hex()) for i in bad]
        with np.errstate(all="ignore"):
            assert _same(hw, a * b).all()  # and mul.rn.f64 is numpy's IEEE product


DECKS = {
    "jacobi_600x433": dict(nx=600, ny=433, solver="jacobi", max_iters=300, steps=2),
    "jacobi_reflective_300x211": dict(nx=300, ny=211, solver="jacobi", reflective=True, max_iters=300, steps=1),
    "jacobi_coef1_257x129": dict(nx=257, ny=129, solver="jacobi", coefficient=1, max_iters=200, steps=1),
}


@pytest.mark.parametrize("name", list(DECKS))
def test_jacobi_integer_products_give_the_same_bits(name, monkeypatch):
    from tealeaf_ref_gb300 import native

    d = small_deck(**DECKS[name])
    runs = {}
    for mask in ("0", "0x40", "0x1b", "0x3f", "0x7f"):
        monkeypatch.setenv("TL_JACOBI_INT", mask)
        with native.Chunk.from_deck(d) as c:
            infos = [c.tea_leaf(d) for _ in range(d.end_step)]
            runs[mask] = ([(i.reported_iterations, i.error) for i in infos], c.download("u"))
    its0, u0 = runs["0"]
    assert its0[0][0] > 10
    for mask, (its, u) in runs.items():
        assert its == its0, (mask, its, its0)
        assert np.array_equal(u.view(np.uint64), u0.view(np.uint64)), mask

