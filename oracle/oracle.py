"""ctypes binding for the CPU oracle (oracle/tealeaf_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the CPU
baseline legs of bench.py, as the checker.  The product (tealeaf_ref_gb300) never
imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading
from dataclasses import dataclass
from typing import List, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")

# array ids (tealeaf_oracle.h)
ARRAYS = ["density", "energy0", "energy1", "u", "u0", "r", "r_store", "mi", "w", "z", "utemp", "rtemp",
          "di", "kx", "ky", "p", "sd", "cp", "bfp"]
FIELD_IDS = {"density": 1, "energy0": 2, "energy1": 3, "u": 4, "p": 5, "sd": 6, "r": 7, "z": 8, "kx": 9,
             "ky": 10, "di": 11}

_lock = threading.Lock()
_libs = {}


def build(force: bool = False) -> None:
    """Compile the oracle libraries with oracle/Makefile (make rebuilds what is stale: the
    sources or the recipe changed)."""
    subprocess.run(["make", "-s", "-C", HERE] + (["-B"] if force else []), check=True)


class _Opts(C.Structure):
    _fields_ = [("solver", C.c_int), ("max_iters", C.c_int), ("eps", C.c_double), ("ch_cg_presteps", C.c_int),
                ("ch_cg_epslim", C.c_double), ("ppcg_inner_steps", C.c_int), ("check_result", C.c_int)]


class _Persist(C.Structure):
    _fields_ = [("first", C.c_int), ("eigmin", C.c_double), ("eigmax", C.c_double), ("theta", C.c_double),
                ("cn", C.c_double)]


class _Info(C.Structure):
    _fields_ = [("n_exit", C.c_int), ("reported_iterations", C.c_int), ("ppcg_inner_iters", C.c_int),
                ("cg_calc_steps", C.c_int), ("cheby_calc_steps", C.c_int), ("est_itc", C.c_int),
                ("initial_residual", C.c_double), ("error", C.c_double), ("exact_error", C.c_double),
                ("eigmin", C.c_double), ("eigmax", C.c_double), ("status", C.c_int)]


VARIANTS = {False: "liboracle.so", True: "liboracle_omp.so", "omp": "liboracle_omp.so",
            "par": "liboracle_par.so"}


def lib(threaded=False):
    """threaded: False -- the serial checker (pinned bit-exact to the reference's outputs);
    True / "omp" -- the OpenMP timing build (FMA contraction, the CPU baseline);
    "par" -- the OpenMP checker (no contraction; global sums over per-thread partials)."""
    name = VARIANTS[threaded]
    with _lock:
        if name in _libs:
            return _libs[name]
        build()
        L = C.CDLL(os.path.join(BUILD, name))
        D, I, P = C.c_double, C.c_int, C.c_void_p
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int)
        sig = {
            "tlo_create": (P, [I, I, I, D, D, D, D, I, I, I]),
            "tlo_destroy": (None, [P]),
            "tlo_array": (dp, [P, I, ip, ip]),
            "tlo_geometry": (None, [P, dp, dp, dp, dp]),
            "tlo_generate": (None, [P, I, dp, dp, dp, dp, dp, dp, dp, ip]),
            "tlo_start_fields": (None, [P]),
            "tlo_field_summary": (None, [P, dp]),
            "tlo_tea_leaf": (I, [P, C.POINTER(_Opts), C.POINTER(_Persist), D, C.POINTER(_Info)]),
            "tlo_common_init": (None, [P, D]),
            "tlo_calc_residual": (None, [P]),
            "tlo_calc_2norm": (D, [P, I]),
            "tlo_finalise": (None, [P]),
            "tlo_cg_init": (D, [P]),
            "tlo_cg_calc_w": (D, [P]),
            "tlo_cg_calc_ur": (D, [P, D]),
            "tlo_cg_calc_p": (None, [P, D, I]),
            "tlo_cheby_init": (None, [P, D]),
            "tlo_cheby_iterate": (None, [P, D, D]),
            "tlo_ppcg_init_sd": (None, [P, D]),
            "tlo_ppcg_init": (D, [P, I, I]),
            "tlo_ppcg_inner": (None, [P, D, D]),
            "tlo_ppcg_calc_zrnorm": (D, [P, I]),
            "tlo_ppcg_update_z": (None, [P]),
            "tlo_ppcg_store_r": (None, [P]),
            "tlo_ppcg_calc_rrn": (D, [P]),
            "tlo_jacobi_solve": (D, [P]),
            "tlo_update_halo": (None, [P, ip, I]),
            "tlo_calc_eigenvalues": (I, [dp, dp, I, dp, dp]),
            "tlo_calc_ch_coefs": (None, [dp, dp, D, D, dp, I]),
            "tlo_tridiag_eigenvalues": (None, [dp, dp, I, dp]),
        }
        for fn, (res, args) in sig.items():
            f = getattr(L, fn)
            f.restype = res
            f.argtypes = args
        _libs[name] = L
        return L


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


@dataclass
class SolveInfo:
    n_exit: int
    reported_iterations: int
    ppcg_inner_iters: int
    cg_calc_steps: int
    cheby_calc_steps: int
    est_itc: int
    initial_residual: float
    error: float
    exact_error: float
    eigmin: float
    eigmax: float
    status: int

    @property
    def conduction_error(self) -> float:
        return self.error / self.initial_residual if self.initial_residual else float("nan")


class Chunk:
    """One single-tile chunk in the reference's layout (halo depth h on every side)."""

    def __init__(self, x_cells, y_cells, halo_depth=1, xmin=0.0, ymin=0.0, xmax=10.0, ymax=10.0,
                 coefficient=1, precond=1, reflective=False, threaded=False):
        self.L = lib(threaded)
        self.h = halo_depth
        self.nx, self.ny = x_cells, y_cells
        self.ptr = self.L.tlo_create(x_cells, y_cells, halo_depth, xmin, ymin, xmax, ymax, coefficient, precond,
                                     int(bool(reflective)))
        if not self.ptr:
            raise ValueError("invalid chunk dimensions")
        self.persist = _Persist(first=1)

    @classmethod
    def from_deck(cls, deck, threaded=False) -> "Chunk":
        c = cls(deck.x_cells, deck.y_cells, deck.halo_depth, deck.xmin, deck.ymin, deck.xmax, deck.ymax,
                deck.coefficient, deck.precond_id, deck.reflective_boundary, threaded)
        c.generate(deck)
        c.start_fields()
        return c

    def __del__(self):
        try:
            if self.ptr:
                self.L.tlo_destroy(self.ptr)
                self.ptr = None
        except Exception:
            pass

    def array(self, name: str) -> np.ndarray:
        """Numpy view (shape (dim_y, dim_x), x fastest) of a field including its halo."""
        dx, dy = C.c_int(), C.c_int()
        p = self.L.tlo_array(self.ptr, ARRAYS.index(name), C.byref(dx), C.byref(dy))
        return np.ctypeslib.as_array(p, shape=(dy.value, dx.value))

    def interior(self, name: str) -> np.ndarray:
        a = self.array(name)
        if name in ("cp", "bfp"):
            return a
        h = self.h
        return a[h:h + self.ny, h:h + self.nx]

    def geometry(self):
        v = [C.c_double() for _ in range(4)]
        self.L.tlo_geometry(self.ptr, *[C.byref(x) for x in v])
        return tuple(x.value for x in v)

    def generate(self, deck) -> None:
        arrs = deck.state_arrays()
        geom = arrs[-1]
        self._keep = arrs
        self.L.tlo_generate(self.ptr, len(deck.states), *[_dp(a) for a in arrs[:-1]],
                            geom.ctypes.data_as(C.POINTER(C.c_int)))

    def start_fields(self) -> None:
        self.L.tlo_start_fields(self.ptr)

    def field_summary(self) -> np.ndarray:
        out = np.zeros(4)
        self.L.tlo_field_summary(self.ptr, _dp(out))
        return out

    def tea_leaf(self, deck, dt: Optional[float] = None) -> SolveInfo:
        o = _Opts(solver=deck.solver_id, max_iters=deck.max_iters, eps=deck.eps, ch_cg_presteps=deck.ch_cg_presteps,
                  ch_cg_epslim=deck.ch_cg_epslim, ppcg_inner_steps=deck.effective_inner_steps(),
                  check_result=int(deck.check_result))
        info = _Info()
        self.L.tlo_tea_leaf(self.ptr, C.byref(o), C.byref(self.persist),
                            deck.initial_timestep if dt is None else dt, C.byref(info))
        return SolveInfo(*[getattr(info, f[0]) for f in _Info._fields_])

    def update_halo(self, fields, depth: int) -> None:
        mask = np.zeros(12, dtype=np.int32)
        for f in fields:
            mask[FIELD_IDS[f]] = 1
        self.L.tlo_update_halo(self.ptr, mask.ctypes.data_as(C.POINTER(C.c_int)), depth)

    def __getattr__(self, name):
        # single-kernel calls: chunk.cg_calc_w() -> tlo_cg_calc_w(ptr)
        if name.startswith("_") or name in ("L", "ptr"):
            raise AttributeError(name)
        fn = getattr(self.__dict__["L"], "tlo_" + name)
        return lambda *a: fn(self.ptr, *a)


@dataclass
class RunResult:
    summaries: List[tuple]  # (step, [vol, mass, ie, temp])
    solves: List[SolveInfo]


def run_deck(deck, threaded: bool = False, max_steps: Optional[int] = None) -> RunResult:
    """The reference's main program on one chunk: start (tea_leaf.f90, start.f90) then
    diffuse (diffuse.f90:43-105) with field summaries every summary_frequency steps and
    at the end."""
    c = Chunk.from_deck(deck, threaded)
    summaries = [(0, c.field_summary())]
    solves = []
    step, time = 0, 0.0
    g_small = float(np.float32(1.0e-16))
    while True:
        step += 1
        dt = deck.initial_timestep
        solves.append(c.tea_leaf(deck, dt))
        time = time + dt
        done = time + g_small > deck.end_time or step >= deck.end_step or (max_steps and step >= max_steps)
        if deck.summary_frequency and step % deck.summary_frequency == 0 and not done:
            summaries.append((step, c.field_summary()))
        if done:
            summaries.append((step, c.field_summary()))
            break
    return RunResult(summaries, solves)


def tridiag_eigenvalues(d: np.ndarray, off: np.ndarray) -> np.ndarray:
    L = lib()
    d = np.ascontiguousarray(d, dtype=np.float64)
    off = np.ascontiguousarray(off, dtype=np.float64)
    out = np.zeros_like(d)
    L.tlo_tridiag_eigenvalues(_dp(d), _dp(off), len(d), _dp(out))
    return out
