"""tl_cg_calc_w_noalloc: the allocation-free variant of the CG matvec entry point.

It serves callers that own all device memory themselves and cannot let the library
allocate (no tl_ctx): a Fortran driver whose fields already sit on the GPU under OpenACC or
CUDA Fortran, or a time loop that must never call cudaMalloc.  The tests build the
reference-layout device arrays themselves (the caller's role) and call the entry point twice
in a row with different p vectors:

* against the oracle's tea_leaf_cg_calc_w on the oracle's own arrays (the reference's
  layout, halo depth 1 and 2, with and without reflective boundaries, the mirrored halos of
  p written by the caller), at the tolerance of the other kernel tests;
* against the context-based tl_cg_calc_w on the same data.

This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from helpers import rel_inf, small_deck

pytestmark = pytest.mark.gpu


def _reference_layout(interior: np.ndarray, h: int) -> np.ndarray:
    ny, nx = interior.shape
    a = np.zeros((ny + 2 * h, nx + 2 * h), dtype=np.float64)
    a[h:h + ny, h:h + nx] = interior
    return a


def _noalloc(L, torch, nx, ny, h, p, kx, ky, di, rx, ry):
    """One call on device copies of full (halo-including) arrays; returns (w, pw)."""
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (p, kx, ky, di)]
    w = torch.full_like(dev[0], float("nan"))
    torch.cuda.synchronize()
    pw = C.c_double()
    rc = L.tl_cg_calc_w_noalloc(nx, ny, h, dev[0].data_ptr(), w.data_ptr(), dev[1].data_ptr(), dev[2].data_ptr(),
                                dev[3].data_ptr(), rx, ry, C.byref(pw))
    assert rc == 0, L.tl_last_error()
    return w.cpu().numpy(), pw.value


@pytest.mark.parametrize("h", [1, 2])
@pytest.mark.parametrize("reflective", [False, True])
def test_cg_calc_w_noalloc_matches_oracle(h, reflective):
    torch = pytest.importorskip("torch")
    from oracle import oracle
    from tealeaf_ref_gb300 import native

    L = native.load()
    d = small_deck(nx=97, ny=61, n_rect=4, n_circ=2, halo_depth=h, reflective=reflective)
    dt = d.initial_timestep
    rx, ry = dt / (d.dx * d.dx), dt / (d.dy * d.dy)
    red_tol = max(1e-12, 4e-16 * d.x_cells * d.y_cells)
    o = oracle.Chunk.from_deck(d)
    o.common_init(dt)
    o.calc_residual()
    o.cg_init()
    kx, ky, di = (np.array(o.array(n)) for n in ("kx", "ky", "di"))
    p0 = np.array(o.interior("p"))
    rng = np.random.Generator(np.random.PCG64(17))
    for call, p_int in enumerate((p0, 0.5 * p0 + 1e-3 * rng.standard_normal(p0.shape))):
        o.interior("p")[...] = p_int
        o.update_halo(["p"], h)  # the mirrored halo of p, as the caller's update_halo writes it
        p_full = np.array(o.array("p"))
        pw_ref = o.cg_calc_w()
        w_ref = np.array(o.interior("w"))
        w, pw = _noalloc(L, torch, d.x_cells, d.y_cells, h, p_full, kx, ky, di, rx, ry)
        w_int = w[h:h + d.y_cells, h:h + d.x_cells]
        assert np.all(np.isfinite(w_int)), call
        assert rel_inf(w_int, w_ref) < 1e-12, call
        assert abs(pw - pw_ref) <= red_tol * abs(pw_ref), (call, pw, pw_ref)


def test_cg_calc_w_noalloc_matches_context_entry_point():
    torch = pytest.importorskip("torch")
    from tealeaf_ref_gb300 import native

    L = native.load()
    h = 1
    d = small_deck(nx=97, ny=61, n_rect=4, n_circ=2)
    dt = d.initial_timestep
    rx, ry = dt / (d.dx * d.dx), dt / (d.dy * d.dy)
    red_tol = max(1e-12, 4e-16 * d.x_cells * d.y_cells)
    with native.Chunk.from_deck(d) as c:
        c.common_init(dt)
        c.calc_residual()
        c.cg_init()
        # Without reflective boundaries the boundary faces (Kx at j = 1 and x_cells+1, Ky at
        # k = 1 and y_cells+1) are zero and the halo of p is zero: zero-filled halos match.
        kx = _reference_layout(c.download("kx"), h)
        ky = _reference_layout(c.download("ky"), h)
        di = _reference_layout(c.download("di"), h)
        p0 = c.download("p")
        for call, p_host in enumerate((p0, 0.5 * p0 + 1e-3 * np.sin(np.arange(p0.size)).reshape(p0.shape))):
            c.upload("p", p_host)
            pw_ref = c.cg_calc_w()
            w_ref = c.download("w")
            w, pw = _noalloc(L, torch, d.x_cells, d.y_cells, h, _reference_layout(p_host, h), kx, ky, di, rx, ry)
            w_int = w[h:h + d.y_cells, h:h + d.x_cells]
            assert np.all(np.isfinite(w_int)), call
            assert rel_inf(w_int, w_ref) < 1e-12, call
            assert abs(pw - pw_ref) <= red_tol * abs(pw_ref), (call, pw, pw_ref)


def test_cg_calc_w_noalloc_rejects_bad_sizes():
    from tealeaf_ref_gb300 import native

    L = native.load()
    pw = C.c_double()
    dummy = C.c_void_p(1)
    assert L.tl_cg_calc_w_noalloc(8, 16385, 1, dummy, dummy, dummy, dummy, dummy, 1.0, 1.0, C.byref(pw)) == -1
    assert b"16384" in L.tl_last_error()
    assert L.tl_cg_calc_w_noalloc(0, 8, 1, dummy, dummy, dummy, dummy, dummy, 1.0, 1.0, C.byref(pw)) == -1
    assert L.tl_cg_calc_w_noalloc(8, 8, 1, None, dummy, dummy, dummy, dummy, 1.0, 1.0, C.byref(pw)) == -1
    # the guard widens before adding the halo: no int overflow for extreme arguments
    big = 2 ** 31 - 1
    assert L.tl_cg_calc_w_noalloc(big, 8, big, dummy, dummy, dummy, dummy, dummy, 1.0, 1.0, C.byref(pw)) == -1
    assert b"too large" in L.tl_last_error()
