"""Pipelined host transfers (tl_stage_state, tl_take_staged, tl_fetch_field, tl_wait_transfers)
against the synchronous upload / solve / download sequence: bitwise-equal energies step by step,
and the staging-state errors."""
import numpy as np
import pytest

from helpers import small_deck

pytestmark = pytest.mark.gpu


def _states(d, n, seed):
    """n (density, energy) pairs: the generated state with seeded perturbations."""
    from tealeaf_ref_gb300 import native

    with native.Chunk.from_deck(d) as c:
        rho, e = c.download("density"), c.download("energy1")
    rng = np.random.default_rng(seed)
    return [(rho * (1 + 0.1 * rng.random(rho.shape)), e * (1 + 0.1 * rng.random(e.shape))) for _ in range(n)]


@pytest.mark.parametrize("case", [dict(), dict(reflective=True), dict(solver="ppcg", ppcg_inner_steps=8,
                                                                      ch_cg_presteps=20)],
                         ids=["cg", "reflective", "ppcg"])
def test_pipelined_matches_synchronous(case):
    from tealeaf_ref_gb300 import native

    kw = dict(nx=97, ny=61, steps=1, n_rect=3, n_circ=1)
    kw.update(case)
    d = small_deck(**kw)
    states = _states(d, 5, 7)
    with native.Chunk.from_deck(d) as c:
        want = []
        for rho, e in states:
            c.upload_state(rho, e)
            c.tea_leaf(d)
            want.append(c.download("energy1"))
    pins = [native.PinnedArray(states[0][0].shape) for _ in range(2 * len(states) + len(states))]
    try:
        for i, (rho, e) in enumerate(states):
            pins[2 * i].array[:] = rho
            pins[2 * i + 1].array[:] = e
        outs = [p.array for p in pins[2 * len(states):]]
        with native.Chunk.from_deck(d) as c:
            c.stage_state(pins[0].array, pins[1].array)
            c.stage_state(pins[2].array, pins[3].array)
            for s in range(len(states)):
                c.take_staged()
                c.tea_leaf(d)
                c.fetch("energy1", outs[s])
                if s + 2 < len(states):
                    c.stage_state(pins[2 * (s + 2)].array, pins[2 * (s + 2) + 1].array)
            c.wait_transfers()
        for s in range(len(states)):
            np.testing.assert_array_equal(outs[s], want[s])
    finally:
        for p in pins:
            p.close()


def test_staging_state_errors():
    from tealeaf_ref_gb300 import native

    d = small_deck(nx=32, ny=24, steps=1, n_rect=1, n_circ=0)
    rho, e = _states(d, 1, 3)[0]
    with native.Chunk.from_deck(d) as c:
        with pytest.raises(native.TeaLeafError) as ex:
            c.take_staged()
        assert ex.value.code == -7  # TL_ERR_STATE: nothing staged
        c.stage_state(rho, e)
        c.stage_state(rho, e)
        with pytest.raises(native.TeaLeafError) as ex:
            c.stage_state(rho, e)
        assert ex.value.code == -7  # TL_ERR_STATE: both slots hold a staged pair
        c.take_staged()
        c.take_staged()
        c.wait_transfers()
        np.testing.assert_array_equal(c.download("density"), rho)
        np.testing.assert_array_equal(c.download("energy1"), e)


def test_fetch_snapshot_is_taken_in_stream_order():
    """A fetch queued between two solves returns the field as it was after the first one,
    although the second solve is under way when the copy to the host runs."""
    from tealeaf_ref_gb300 import native

    d = small_deck(nx=128, ny=96, steps=1, n_rect=2, n_circ=1)
    with native.Chunk.from_deck(d) as c:
        c.tea_leaf(d)
        first = c.download("u")
        out = np.zeros_like(first)
        c.fetch("u", out)
        c.tea_leaf(d)
        c.wait_transfers()
        np.testing.assert_array_equal(out, first)
        assert not np.array_equal(c.download("u"), first)


@pytest.mark.parametrize("pad", [4, 70], ids=["contiguous", "row-by-row"])
def test_host_row_stride(pad):
    """Host arrays with a row stride ld > x_cells (a Fortran array with halo columns): the
    interior moves in both directions and the host's extra columns are left untouched.  ld =
    x_cells + 4 moves as one contiguous copy; x_cells + 70 exceeds the context's stride and goes
    row by row."""
    import ctypes as C

    from tealeaf_ref_gb300 import native

    d = small_deck(nx=37, ny=23, steps=1, n_rect=2, n_circ=1)
    nx, ny, ld = d.x_cells, d.y_cells, d.x_cells + pad
    rng = np.random.default_rng(5)
    rho = rng.random((ny, nx)) + 0.5
    e = rng.random((ny, nx)) + 1.0
    big_rho = np.full((ny, ld), -7.0)
    big_e = np.full((ny, ld), -7.0)
    big_rho[:, :nx] = rho
    big_e[:, :nx] = e
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    with native.Chunk.from_deck(d) as c:
        L = c.L
        assert L.tl_upload_state(c.ptr, dp(big_rho), dp(big_e), ld) == 0
        np.testing.assert_array_equal(c.download("density"), rho)
        np.testing.assert_array_equal(c.download("energy1"), e)
        out = np.full((ny, ld), 3.5)
        assert L.tl_download_field(c.ptr, native.FIELD["density"], dp(out), ld) == 0
        np.testing.assert_array_equal(out[:, :nx], rho)
        assert np.all(out[:, nx:] == 3.5)
        assert L.tl_upload_field(c.ptr, native.FIELD["u"], dp(big_e), ld) == 0
        np.testing.assert_array_equal(c.download("u"), e)
        # pipelined forms
        assert L.tl_stage_state(c.ptr, dp(big_e), dp(big_rho), ld) == 0
        assert L.tl_take_staged(c.ptr) == 0
        out2 = np.full((ny, ld), 4.5)
        assert L.tl_fetch_field(c.ptr, native.FIELD["density"], dp(out2), ld) == 0
        assert L.tl_wait_transfers(c.ptr) == 0
        np.testing.assert_array_equal(out2[:, :nx], e)
        assert np.all(out2[:, nx:] == 4.5)
        np.testing.assert_array_equal(c.download("energy1"), rho)


def test_device_bytes_counts_buffers_made_on_first_use():
    """tl_device_bytes grows when the precision form's FP32 fields and the transfer staging
    fields are first made."""
    from tealeaf_ref_gb300 import native

    d = small_deck(nx=64, ny=48, steps=1, n_rect=2, n_circ=1)
    with native.Chunk.from_deck(d) as c:
        b0 = c.device_bytes()
        assert b0 > 25 * 8 * (48 + 2) * 64  # the field slab at least
        c.tea_leaf(native.opts_from_deck(d, precision="mixed"), d.initial_timestep)
        b1 = c.device_bytes()
        assert b1 > b0
        c.download("u")  # the staging fields of the host transfers
        assert c.device_bytes() > b1
