"""The C-ABI library builds for sm_103a, loads, and exports every entry point that
include/tealeaf_gb300.h declares (no GPU needed: nothing is called that touches a device)."""
import ctypes
import os
import re

from tealeaf_ref_gb300 import build, native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "tealeaf_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(tl_[a-z0-9_]+)\s*\(", txt)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("tl_create", "tl_cg_calc_w", "tl_cg_calc_ur", "tl_cg_calc_p", "tl_tea_leaf", "tl_jacobi_solve",
              "tl_ppcg_inner", "tl_cheby_iterate", "tl_field_summary"):
        assert s in syms


def test_library_exports_every_declared_symbol():
    path = build.build()
    lib = ctypes.CDLL(path)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_covers_header():
    assert set(declared_symbols()) <= set(native.SIGNATURES)


def test_null_arguments_rejected_without_gpu():
    lib = native.load()
    assert lib.tl_destroy(None) == -1
    assert lib.tl_field_summary(None, None, None, None, None) == -1
    out = ctypes.c_void_p()
    assert lib.tl_create(0, 4, 1, 1, 1, 0, 1.0, 1.0, ctypes.byref(out)) == -1
    assert b"x_cells" in lib.tl_last_error()


def test_create_validates_arguments_without_gpu():
    """tl_create rejects what the reference's read_input rejects before touching a device."""
    lib = native.load()
    out = ctypes.c_void_p()
    cases = [
        ((4, 0, 1, 1, 1, 0, 1.0, 1.0), b"x_cells and y_cells"),
        ((65537, 4, 1, 1, 1, 0, 1.0, 1.0), b"x_cells and y_cells"),
        ((4, 4, 0, 1, 1, 0, 1.0, 1.0), b"halo exchange depth"),
        ((4, 4, 1, 3, 1, 0, 1.0, 1.0), b"coefficient"),
        ((4, 4, 1, 1, 4, 0, 1.0, 1.0), b"preconditioner"),
        ((4, 4, 2, 1, 3, 0, 1.0, 1.0), b"block jacobi"),
        ((4, 4, 1, 1, 1, 0, 0.0, 1.0), b"dx and dy"),
    ]
    for args, msg in cases:
        assert lib.tl_create(*args, ctypes.byref(out)) == -1, args
        assert msg in lib.tl_last_error(), (args, lib.tl_last_error())
        assert not out.value


def test_transfer_calls_reject_null_context_without_gpu():
    lib = native.load()
    buf = (ctypes.c_double * 4)()
    assert lib.tl_stage_state(None, buf, buf, 2) == -1
    assert lib.tl_take_staged(None) == -1
    assert lib.tl_fetch_field(None, 3, buf, 2) == -1
    assert lib.tl_wait_transfers(None) == -1
