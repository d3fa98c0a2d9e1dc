"""tl_cg_calc_w_noalloc: the allocation-free variant of the CG matvec entry point.

It serves callers that own all device memory themselves and cannot let the library
allocate (no tl_ctx).  The test builds the reference-layout device arrays itself (the
caller's role), calls the entry point twice in a row with different p vectors, and checks
each result against the context-based tl_cg_calc_w on the same data, at the tolerance the
other kernel tests use.  This file is collected last on purpose."""
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
        kx = torch.from_numpy(_reference_layout(c.download("kx"), h)).cuda()
        ky = torch.from_numpy(_reference_layout(c.download("ky"), h)).cuda()
        di = torch.from_numpy(_reference_layout(c.download("di"), h)).cuda()
        p0 = c.download("p")
        for call, p_host in enumerate((p0, 0.5 * p0 + 1e-3 * np.sin(np.arange(p0.size)).reshape(p0.shape))):
            c.upload("p", p_host)
            pw_ref = c.cg_calc_w()
            w_ref = c.download("w")
            p = torch.from_numpy(_reference_layout(p_host, h)).cuda()
            w = torch.full_like(p, float("nan"))
            torch.cuda.synchronize()
            pw = C.c_double()
            rc = L.tl_cg_calc_w_noalloc(d.x_cells, d.y_cells, h, p.data_ptr(), w.data_ptr(), kx.data_ptr(),
                                        ky.data_ptr(), di.data_ptr(), rx, ry, C.byref(pw))
            assert rc == 0, L.tl_last_error()
            w_int = w.cpu().numpy()[h:h + d.y_cells, h:h + d.x_cells]
            assert np.all(np.isfinite(w_int)), call
            assert rel_inf(w_int, w_ref) < 1e-12, call
            assert abs(pw.value - pw_ref) <= red_tol * abs(pw_ref), (call, pw.value, pw_ref)


def test_cg_calc_w_noalloc_rejects_bad_sizes():
    from tealeaf_ref_gb300 import native

    L = native.load()
    pw = C.c_double()
    dummy = C.c_void_p(1)
    assert L.tl_cg_calc_w_noalloc(8, 16385, 1, dummy, dummy, dummy, dummy, dummy, 1.0, 1.0, C.byref(pw)) == -1
    assert b"16384" in L.tl_last_error()
    assert L.tl_cg_calc_w_noalloc(0, 8, 1, dummy, dummy, dummy, dummy, dummy, 1.0, 1.0, C.byref(pw)) == -1
    assert L.tl_cg_calc_w_noalloc(8, 8, 1, None, dummy, dummy, dummy, dummy, 1.0, 1.0, C.byref(pw)) == -1
