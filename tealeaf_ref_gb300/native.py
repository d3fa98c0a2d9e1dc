"""ctypes binding of libtealeaf_gb300.so (include/tealeaf_gb300.h).

This mirrors the reference's interface for the solve path: a ``Chunk`` owns one
single-tile chunk resident on the GPU and exposes each per-tile kernel of
kernels/tea_leaf_*_kernel.f90 under the reference's name, ``tea_leaf()`` for a whole
implicit solve (tea_solve.f90), ``field_summary()`` and the reference's main loop
(``run_deck``: start.f90 + diffuse.f90).  Every call goes through the C ABI; there is
no CPU fallback -- a missing library or GPU raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading
from dataclasses import dataclass
from typing import List, Optional

import numpy as np

from . import build as _build
from .deck import Deck

TL_OK = 0
ERRORS = {-1: "TL_ERR_ARG", -2: "TL_ERR_CUDA", -3: "TL_ERR_ALLOC", -4: "TL_ERR_BREAKDOWN", -5: "TL_ERR_TIMEOUT",
          -6: "TL_ERR_EIGEN", -7: "TL_ERR_STATE"}

FIELD = {"density": 1, "energy0": 2, "energy1": 3, "u": 4, "p": 5, "sd": 6, "r": 7, "z": 8, "kx": 9, "ky": 10,
         "di": 11, "u0": 12, "w": 13, "mi": 14, "utemp": 15, "rtemp": 16, "r_store": 17}


class TeaLeafError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "TL_ERR"), code, msg))
        self.code = code


PRECISION = {"fp64": 0, "mixed": 1}
# tl_solve_info.stop_reason of the mixed form (TL_STOP_*)
STOP_REASONS = {0: "none", 1: "eps", 2: "floor", 3: "stall", 4: "reject", 5: "cap"}


class SolveOpts(C.Structure):
    _fields_ = [("solver", C.c_int), ("max_iters", C.c_int), ("eps", C.c_double), ("ch_cg_presteps", C.c_int),
                ("ch_cg_epslim", C.c_double), ("ppcg_inner_steps", C.c_int), ("check_result", C.c_int),
                ("precision", C.c_int), ("inner_tol", C.c_double), ("max_inner_iters", C.c_int)]


class SolveInfo(C.Structure):
    _fields_ = [("n_exit", C.c_int), ("reported_iterations", C.c_int), ("ppcg_inner_iters", C.c_int),
                ("cg_calc_steps", C.c_int), ("cheby_calc_steps", C.c_int), ("est_itc", C.c_int),
                ("initial_residual", C.c_double), ("error", C.c_double), ("exact_error", C.c_double),
                ("eigmin", C.c_double), ("eigmax", C.c_double), ("solve_seconds", C.c_double),
                ("kernel_launches", C.c_longlong), ("outer_iterations", C.c_int), ("stop_reason", C.c_int),
                ("true_residual", C.c_double), ("residual_floor", C.c_double)]

    def as_dict(self):
        return {f[0]: getattr(self, f[0]) for f in self._fields_}

    @property
    def conduction_error(self) -> float:
        return self.error / self.initial_residual if self.initial_residual else float("nan")


_lock = threading.Lock()
_lib = None

_D, _I, _P = C.c_double, C.c_int, C.c_void_p
_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int)
SIGNATURES = {
    "tl_last_error": (C.c_char_p, []),
    "tl_set_device": (_I, [_I]),
    "tl_host_register": (_I, [_P, C.c_ulonglong]),
    "tl_host_alloc": (_I, [C.c_ulonglong, C.POINTER(C.c_void_p)]),
    "tl_host_free": (_I, [_P]),
    "tl_host_unregister": (_I, [_P]),
    "tl_create": (_I, [_I, _I, _I, _I, _I, _I, _D, _D, C.POINTER(_P)]),
    "tl_destroy": (_I, [_P]),
    "tl_device_bytes": (_I, [_P, C.POINTER(C.c_ulonglong)]),
    "tl_upload_field": (_I, [_P, _I, _DP, _I]),
    "tl_download_field": (_I, [_P, _I, _DP, _I]),
    "tl_upload_state": (_I, [_P, _DP, _DP, _I]),
    "tl_generate_chunk": (_I, [_P, _I, _DP, _DP, _DP, _DP, _DP, _DP, _DP, _IP, _D, _D]),
    "tl_field_summary": (_I, [_P, _DP, _DP, _DP, _DP]),
    "tl_common_init": (_I, [_P, _D]),
    "tl_calc_residual": (_I, [_P]),
    "tl_calc_2norm": (_I, [_P, _I, _DP]),
    "tl_finalise": (_I, [_P]),
    "tl_finalise_field_summary": (_I, [_P, _DP, _DP, _DP, _DP]),
    "tl_cg_init": (_I, [_P, _DP]),
    "tl_cg_calc_w": (_I, [_P, _DP]),
    "tl_cg_calc_ur": (_I, [_P, _D, _DP]),
    "tl_cg_calc_p": (_I, [_P, _D, _I]),
    "tl_cheby_init": (_I, [_P, _D]),
    "tl_cheby_iterate": (_I, [_P, _D, _D]),
    "tl_ppcg_init_sd": (_I, [_P, _D]),
    "tl_ppcg_init": (_I, [_P, _I, _I, _DP]),
    "tl_ppcg_inner": (_I, [_P, _D, _D]),
    "tl_ppcg_calc_zrnorm": (_I, [_P, _I, _DP]),
    "tl_ppcg_update_z": (_I, [_P]),
    "tl_ppcg_store_r": (_I, [_P]),
    "tl_ppcg_calc_rrn": (_I, [_P, _DP]),
    "tl_jacobi_solve": (_I, [_P, _DP]),
    "tl_update_halo": (_I, [_P, _I, _I]),
    "tl_tea_leaf": (_I, [_P, C.POINTER(SolveOpts), _D, C.POINTER(SolveInfo)]),
    "tl_tea_leaf_summary": (_I, [_P, C.POINTER(SolveOpts), _D, C.POINTER(SolveInfo), _DP]),
    "tl_reset_eigen": (_I, [_P]),
    "tl_cg_eigenvalues": (_I, [_DP, _DP, _I, _DP, _DP]),
    "tl_cheby_coefficients": (_I, [_D, _D, _I, _DP, _DP, _DP]),
    "tl_stage_state": (_I, [_P, _DP, _DP, _I]),
    "tl_take_staged": (_I, [_P]),
    "tl_fetch_field": (_I, [_P, _I, _DP, _I]),
    "tl_wait_transfers": (_I, [_P]),
    "tl_adjoint_begin": (_I, [_P, _I, _I]),
    "tl_adjoint_record_step": (_I, [_P, C.POINTER(SolveOpts), _D, C.POINTER(SolveInfo)]),
    "tl_adjoint_backward": (_I, [_P, _DP, _DP, _I, _DP, _DP, C.POINTER(SolveInfo)]),
    "tl_adjoint_end": (_I, [_P]),
    # diagnostic, not in the public header: the integer-pipe FP64 multiply against mul.rn.f64
    "tl_fp64_emu_check": (_I, [_DP, _DP, C.c_longlong, _DP, _DP]),
    "tl_cg_calc_w_noalloc": (_I, [_I, _I, _I, _P, _P, _P, _P, _P, _D, _D, _DP]),
    "tl_profile": (_I, [_P, _I]),
    "tl_profile_read": (_I, [_P, _I, _DP, C.POINTER(C.c_longlong)]),
}

KERNEL_TIMERS = {"cg_matvec": 0, "cg_update": 1, "cheby_iterate": 2, "ppcg_inner": 3, "jacobi": 4,
                 "mix_matvec": 5, "mix_update": 6, "poly_step": 7}


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load the solver library (building it with nvcc when absent or stale)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if build_if_missing:
            _build.build()
        if not os.path.exists(_build.LIB):
            raise TeaLeafError(-2, "libtealeaf_gb300.so is missing; run tealeaf_ref_gb300.build")
        L = C.CDLL(_build.LIB)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
        return L


class _HostAllocation:
    """Owner of one tl_host_alloc block: freed when the last numpy view of it is gone."""

    def __init__(self, nbytes: int):
        p = C.c_void_p()
        _check(load().tl_host_alloc(nbytes, C.byref(p)))
        self.ptr = p.value

    def __del__(self):
        try:
            if self.ptr:
                load().tl_host_free(self.ptr)
                self.ptr = None
        except Exception:
            pass


class PinnedArray:
    """A numpy array in page-locked host memory allocated by the CUDA driver (tl_host_alloc),
    zero-filled; the memory lives as long as any view of ``array``.  ``register=True``
    instead registers an ordinary numpy array (tl_host_register), the form a driver that owns
    its arrays uses."""

    def __init__(self, shape, dtype=np.float64, register: bool = False):
        self._registered = register
        if register:
            self.array = np.zeros(shape, dtype=dtype)
            _check(load().tl_host_register(self.array.ctypes.data, self.array.nbytes))
            return
        nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        owner = _HostAllocation(nbytes)
        buf = (C.c_char * nbytes).from_address(owner.ptr)
        buf._owner = owner  # the buffer (the base of every view) keeps the allocation alive
        self.array = np.frombuffer(buf, dtype=dtype).reshape(shape)
        self.array[...] = 0

    def close(self):
        if self.array is None:
            return
        if self._registered:
            load().tl_host_unregister(self.array.ctypes.data)
        self.array = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def set_device(device: int) -> None:
    """Select the CUDA device that later Chunk()s are created on (one process per GPU)."""
    _check(load().tl_set_device(device))


def _check(rc: int):
    if rc != TL_OK:
        raise TeaLeafError(rc, (_lib.tl_last_error() or b"").decode())


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_DP)


def opts_from_deck(deck: Deck, precision: str = "fp64", inner_tol: float = 0.0,
                   max_inner_iters: int = 0) -> SolveOpts:
    """Solve options from a deck; ``precision`` "mixed" selects the precision form (FP32 sweeps
    inside FP64 refinement; CG, Chebyshev and PPCG without preconditioner)."""
    return SolveOpts(solver=deck.solver_id, max_iters=deck.max_iters, eps=deck.eps, ch_cg_presteps=deck.ch_cg_presteps,
                     ch_cg_epslim=deck.ch_cg_epslim, ppcg_inner_steps=deck.effective_inner_steps(),
                     check_result=int(deck.check_result), precision=PRECISION[precision], inner_tol=inner_tol,
                     max_inner_iters=max_inner_iters)


def cg_eigenvalues(alphas: np.ndarray, betas: np.ndarray) -> tuple:
    """Extreme eigenvalues of the Lanczos tridiagonal of CG coefficients alphas(1..n), betas(1..n)
    (tl_cg_eigenvalues; host math, no GPU), unscaled."""
    a = np.ascontiguousarray(alphas, dtype=np.float64)
    b = np.ascontiguousarray(betas, dtype=np.float64)
    if a.shape != b.shape or a.ndim != 1:
        raise ValueError("alphas and betas must be 1-D arrays of the same length")
    lo, hi = C.c_double(), C.c_double()
    _check(load().tl_cg_eigenvalues(_dp(a), _dp(b), a.size, C.byref(lo), C.byref(hi)))
    return lo.value, hi.value


def cheby_coefficients(eigmin: float, eigmax: float, n: int) -> tuple:
    """(theta, ch_alphas(1..n), ch_betas(1..n)) of the Chebyshev iteration (tl_cheby_coefficients)."""
    a, b, th = np.zeros(n), np.zeros(n), C.c_double()
    _check(load().tl_cheby_coefficients(eigmin, eigmax, n, _dp(a), _dp(b), C.byref(th)))
    return th.value, a, b


class Chunk:
    """One chunk of x_cells x y_cells cells on the current CUDA device."""

    def __init__(self, x_cells: int, y_cells: int, halo_depth: int = 1, coefficient: int = 1, precond: int = 1,
                 reflective: bool = False, dx: float = 1.0, dy: float = 1.0):
        self.L = load()
        self.nx, self.ny = x_cells, y_cells
        self.dx, self.dy = dx, dy
        ptr = _P()
        _check(self.L.tl_create(x_cells, y_cells, halo_depth, coefficient, precond, int(bool(reflective)), dx, dy,
                                C.byref(ptr)))
        self.ptr = ptr
        self._xfer_refs = []  # host arrays of pipelined transfers in flight

    @classmethod
    def from_deck(cls, deck: Deck, generate: bool = True) -> "Chunk":
        c = cls(deck.x_cells, deck.y_cells, deck.halo_depth, deck.coefficient, deck.precond_id,
                deck.reflective_boundary, deck.dx, deck.dy)
        if generate:
            c.generate(deck)
        return c

    def close(self):
        if getattr(self, "ptr", None):
            self.L.tl_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- data movement ----
    def upload(self, field: str, host: np.ndarray) -> None:
        a = np.ascontiguousarray(host, dtype=np.float64)
        if a.shape != (self.ny, self.nx):
            raise ValueError("expected shape (y_cells, x_cells)")
        _check(self.L.tl_upload_field(self.ptr, FIELD[field], _dp(a), self.nx))

    def download(self, field: str, out: Optional[np.ndarray] = None) -> np.ndarray:
        """Interior of a field as (y_cells, x_cells); into ``out`` when given (C-contiguous float64)."""
        if out is None:
            out = np.empty((self.ny, self.nx), dtype=np.float64)
        elif out.shape != (self.ny, self.nx) or out.dtype != np.float64 or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous float64 array of shape (y_cells, x_cells)")
        _check(self.L.tl_download_field(self.ptr, FIELD[field], _dp(out), self.nx))
        return out

    def upload_state(self, density: np.ndarray, energy: np.ndarray) -> None:
        d = np.ascontiguousarray(density, dtype=np.float64)
        e = np.ascontiguousarray(energy, dtype=np.float64)
        _check(self.L.tl_upload_state(self.ptr, _dp(d), _dp(e), self.nx))

    # ---- pipelined transfers (copies overlapping the solves) ----
    def stage_state(self, density: np.ndarray, energy: np.ndarray) -> None:
        """Start copying (density, energy1) into a staging slot; the arrays (page-locked, e.g.
        PinnedArray) are kept referenced until wait_transfers()."""
        for a in (density, energy):
            if a.shape != (self.ny, self.nx) or a.dtype != np.float64 or not a.flags.c_contiguous:
                raise ValueError("expected C-contiguous float64 arrays of shape (y_cells, x_cells)")
        _check(self.L.tl_stage_state(self.ptr, _dp(density), _dp(energy), self.nx))
        self._xfer_refs.append((density, energy))

    def take_staged(self) -> None:
        _check(self.L.tl_take_staged(self.ptr))

    def fetch(self, field: str, out: np.ndarray) -> None:
        """Start copying a snapshot of a field into out (valid after wait_transfers())."""
        if out.shape != (self.ny, self.nx) or out.dtype != np.float64 or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous float64 array of shape (y_cells, x_cells)")
        _check(self.L.tl_fetch_field(self.ptr, FIELD[field], _dp(out), self.nx))
        self._xfer_refs.append((out,))

    def wait_transfers(self) -> None:
        _check(self.L.tl_wait_transfers(self.ptr))
        self._xfer_refs = []

    def device_bytes(self) -> int:
        v = C.c_ulonglong()
        _check(self.L.tl_device_bytes(self.ptr, C.byref(v)))
        return v.value

    # ---- generation / summary ----
    def generate(self, deck: Deck) -> None:
        den, en, xmin, xmax, ymin, ymax, rad, geom = deck.state_arrays()
        _check(self.L.tl_generate_chunk(self.ptr, len(deck.states), _dp(den), _dp(en), _dp(xmin), _dp(xmax),
                                        _dp(ymin), _dp(ymax), _dp(rad), geom.ctypes.data_as(_IP), deck.xmin,
                                        deck.ymin))

    def field_summary(self) -> np.ndarray:
        v = [C.c_double() for _ in range(4)]
        _check(self.L.tl_field_summary(self.ptr, *[C.byref(x) for x in v]))
        return np.array([x.value for x in v])

    # ---- whole solve ----
    def tea_leaf(self, deck_or_opts, dt: Optional[float] = None) -> SolveInfo:
        if isinstance(deck_or_opts, Deck):
            o = opts_from_deck(deck_or_opts)
            dt = deck_or_opts.initial_timestep if dt is None else dt
        else:
            o = deck_or_opts
        info = SolveInfo()
        _check(self.L.tl_tea_leaf(self.ptr, C.byref(o), dt, C.byref(info)))
        return info

    def tea_leaf_summary(self, deck_or_opts, dt: Optional[float] = None):
        """tea_leaf() of a time step followed by field_summary, the summary formed by the solve's
        finalise sweep (tl_tea_leaf_summary): (SolveInfo, [vol, mass, ie, temp])."""
        if isinstance(deck_or_opts, Deck):
            o = opts_from_deck(deck_or_opts)
            dt = deck_or_opts.initial_timestep if dt is None else dt
        else:
            o = deck_or_opts
        info = SolveInfo()
        out = np.zeros(4)
        _check(self.L.tl_tea_leaf_summary(self.ptr, C.byref(o), dt, C.byref(info), _dp(out)))
        return info, out

    # ---- adjoint (tl_adjoint_*) ----
    def adjoint_begin(self, max_steps: int, store_solutions: bool = True) -> None:
        _check(self.L.tl_adjoint_begin(self.ptr, max_steps, int(store_solutions)))

    def record_step(self, deck_or_opts, dt: Optional[float] = None) -> SolveInfo:
        """tea_leaf() for one time step, recorded on the adjoint tape."""
        opts = deck_or_opts if isinstance(deck_or_opts, SolveOpts) else opts_from_deck(deck_or_opts)
        if dt is None:
            dt = deck_or_opts.initial_timestep
        info = SolveInfo()
        _check(self.L.tl_adjoint_record_step(self.ptr, C.byref(opts), dt, C.byref(info)))
        return info

    def adjoint_backward(self, u_bar: Optional[np.ndarray], e_bar: Optional[np.ndarray] = None,
                         want_energy0: bool = True):
        """(dL/d density, dL/d initial energy1 or None, SolveInfo of the reverse solves)."""
        def arg(a):
            if a is None:
                return None, None
            a = np.ascontiguousarray(a, dtype=np.float64)
            if a.shape != (self.ny, self.nx):
                raise ValueError("expected shape (y_cells, x_cells)")
            return a, _dp(a)
        ub, ubp = arg(u_bar)
        eb, ebp = arg(e_bar)
        rho_bar = np.empty((self.ny, self.nx), dtype=np.float64)
        e0_bar = np.empty((self.ny, self.nx), dtype=np.float64) if want_energy0 else None
        info = SolveInfo()
        _check(self.L.tl_adjoint_backward(self.ptr, ubp, ebp, self.nx, _dp(rho_bar),
                                          _dp(e0_bar) if e0_bar is not None else None, C.byref(info)))
        return rho_bar, e0_bar, info

    def adjoint_end(self) -> None:
        _check(self.L.tl_adjoint_end(self.ptr))

    def reset_eigen(self) -> None:
        _check(self.L.tl_reset_eigen(self.ptr))

    def profile(self, enable: bool = True) -> None:
        """Time every launch of the fused loop kernels with CUDA events on the solver stream."""
        _check(self.L.tl_profile(self.ptr, int(enable)))

    def profile_read(self, kernel: str):
        """(total ms, launches) of one timed kernel since profile(True)."""
        ms, n = C.c_double(), C.c_longlong()
        _check(self.L.tl_profile_read(self.ptr, KERNEL_TIMERS[kernel], C.byref(ms), C.byref(n)))
        return ms.value, n.value

    # ---- per-kernel entry points (reference names) ----
    def _scalar(self, fn, *args) -> float:
        out = C.c_double()
        _check(fn(self.ptr, *args, C.byref(out)))
        return out.value

    def common_init(self, dt: float) -> None:
        _check(self.L.tl_common_init(self.ptr, dt))

    def calc_residual(self) -> None:
        _check(self.L.tl_calc_residual(self.ptr))

    def calc_2norm(self, norm_array: int) -> float:
        return self._scalar(self.L.tl_calc_2norm, norm_array)

    def finalise(self) -> None:
        _check(self.L.tl_finalise(self.ptr))

    def finalise_field_summary(self) -> np.ndarray:
        """tea_leaf_kernel_finalise then field_summary_kernel in one sweep."""
        v = [C.c_double() for _ in range(4)]
        _check(self.L.tl_finalise_field_summary(self.ptr, *[C.byref(x) for x in v]))
        return np.array([x.value for x in v])

    def cg_init(self) -> float:
        return self._scalar(self.L.tl_cg_init)

    def cg_calc_w(self) -> float:
        return self._scalar(self.L.tl_cg_calc_w)

    def cg_calc_ur(self, alpha: float) -> float:
        return self._scalar(self.L.tl_cg_calc_ur, alpha)

    def cg_calc_p(self, beta: float, ppcg_active: bool = False) -> None:
        _check(self.L.tl_cg_calc_p(self.ptr, beta, int(ppcg_active)))

    def cheby_init(self, theta: float) -> None:
        _check(self.L.tl_cheby_init(self.ptr, theta))

    def cheby_iterate(self, ch_alpha: float, ch_beta: float) -> None:
        _check(self.L.tl_cheby_iterate(self.ptr, ch_alpha, ch_beta))

    def ppcg_init_sd(self, theta: float) -> None:
        _check(self.L.tl_ppcg_init_sd(self.ptr, theta))

    def ppcg_init(self, step: int, ppcg_active: bool) -> float:
        return self._scalar(self.L.tl_ppcg_init, step, int(ppcg_active))

    def ppcg_inner(self, ch_alpha: float, ch_beta: float) -> None:
        _check(self.L.tl_ppcg_inner(self.ptr, ch_alpha, ch_beta))

    def ppcg_calc_zrnorm(self, ppcg_active: bool) -> float:
        return self._scalar(self.L.tl_ppcg_calc_zrnorm, int(ppcg_active))

    def ppcg_update_z(self) -> None:
        _check(self.L.tl_ppcg_update_z(self.ptr))

    def ppcg_store_r(self) -> None:
        _check(self.L.tl_ppcg_store_r(self.ptr))

    def ppcg_calc_rrn(self) -> float:
        return self._scalar(self.L.tl_ppcg_calc_rrn)

    def jacobi_solve(self) -> float:
        return self._scalar(self.L.tl_jacobi_solve)

    def update_halo(self, fields, depth: int = 1) -> None:
        mask = 0
        for f in fields:
            mask |= 1 << FIELD[f]
        _check(self.L.tl_update_halo(self.ptr, mask, depth))


@dataclass
class RunResult:
    summaries: List[tuple]  # (step, np.array([vol, mass, ie, temp]))
    solves: List[dict]


def run_deck(deck: Deck, max_steps: Optional[int] = None, precision: str = "fp64", inner_tol: float = 0.0,
             visit_dir: Optional[str] = None) -> RunResult:
    """The reference's main program on one GPU chunk: start (generate, set_field, first
    field_summary; start.f90:98-125) then the diffuse loop (diffuse.f90:43-105).  With
    ``visit_dir`` and a non-zero visit_frequency, VTK files are written there where the loop
    calls visit (every visit_frequency steps and at the end; diffuse.f90:58-59,89)."""
    opts = opts_from_deck(deck, precision, inner_tol)
    with Chunk.from_deck(deck) as c:
        summaries = [(0, c.field_summary())]
        solves = []
        vis = None
        if visit_dir and deck.visit_frequency:
            from .visit import Visit

            vis = Visit(visit_dir, deck)
            density = c.download("density")
            energy0 = c.download("energy1")  # set_field copied energy0 into energy1

            def visit(step):
                vis.write(step, density, energy0, c.download("u"))
        step, time = 0, 0.0
        g_small = float(np.float32(1.0e-16))
        while True:
            step += 1
            dt = deck.initial_timestep
            # the summary steps of diffuse.f90:58-61 and the last step: the solve's finalise
            # sweep forms the field summary too (tl_tea_leaf_summary)
            done = (time + dt) + g_small > deck.end_time or step >= deck.end_step or \
                bool(max_steps and step >= max_steps)
            want = done or bool(deck.summary_frequency and step % deck.summary_frequency == 0)
            if want:
                info, summ = c.tea_leaf_summary(opts, dt)
                summaries.append((step, summ))
            else:
                info = c.tea_leaf(opts, dt)
            solves.append(info.as_dict())
            time = time + dt
            if vis and step % deck.visit_frequency == 0:
                visit(step)
            if done:
                if vis:
                    visit(step)
                break
        return RunResult(summaries, solves)
