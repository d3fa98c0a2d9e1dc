#!/usr/bin/env python3
"""Benchmark of TeaLeaf's implicit solve (tea_leaf(), tea_solve.f90:37-503) on GB300.

Default line (the headline): FP64 CG cell-iterations/s at 8192^2.  Workload: 8192 x 8192
cells on the 10 x 10 domain, ambient state (density 100, energy 1e-4) + 16 seeded rectangles
(density U[0.1,1], energy U[1,25]) + 4 seeded circles (density 0.1, energy 25),
reciprocal-density coefficient keyword, dt 0.004, tl_eps 1e-15, CG, FP64.  A step is one
tea_leaf() time-step solve through the C ABI capped at --iters CG iterations (tl_max_iters,
default 500): set-up, initial residual, the fused CG iterations, finalise.  At this size a full
time step needs tens of thousands of iterations, so the cap keeps a step under a second;
iterations are the work unit of the metric (cells x iterations / time), as in the reference's
own grind figures.

--solver jacobi | chebyshev | ppcg: the same line for the 4096^2 workloads (8 seeded
rectangles; Jacobi seed 2; Chebyshev / PPCG seed 3 with 20 CG presteps, tl_ch_cg_epslim large
so that the switch of tea_solve.f90:160-174 comes right after them, PPCG 10 inner steps), a
step capped at --iters iterations (default 100 / 100 / 30), cell-iterations/s with the
reference's iteration count (PPCG: outer iterations, each with its inner steps).

value  : device time (CUDA events on the solver stream) of the K timed steps, inputs
         resident in HBM (every field is larger than L2).
e2e    : the same steps through the C ABI with host buffers, host wall clock: every step's
         density/energy copied from pinned host memory and its energy copied back.  Two forms
         exist: synchronous (upload, solve, download) and pipelined (tl_stage_state two steps
         ahead on an upload stream, tl_fetch_field on a download stream, so the copies overlap
         the solves).  The steady-state step time of each, from untimed runs of one and three
         steps, picks the form the timed steps use; the other form is timed too and reported
         beside it.
roofline: the dominant kernel of the line timed per launch with CUDA events recorded on the
         solver stream during the timed steps, against its algorithmic bytes per cell;
         `traffic` from the ncu capture summarised in profiles/roofline_traffic.json.
cpu_baseline: the CPU port of the reference kernels (oracle/, OpenMP over all host cores) on
         a bounded sample of the same workload (steps capped at --cpu-iters iterations; the
         solver lines use the GPU's own window).

--impl reference times that CPU port alone as the reference arm, with the same config dict
(the sample window is reported beside it).  Under torchrun (N>1) every rank runs an
independent replica of the workload on its own GPU (the solve has no multi-GPU decomposition
here), barrier + max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BYTES_PER_CELL_IT = 96      # whole FP64 CG iteration (12 streams)
FP64_OPS_PER_CLOCK_SM = 2   # FP64 pipe peak that ncu reports for GB300: 2 thread-operations per clock per SM
FALLBACK_HBM_GBS = 6800.0

# Dominant kernel of each line: timer id (tl_profile), what it is, algorithmic bytes per cell per
# launch, FP64 operations per cell per launch, and how many of those issue on the FP64 pipe (the
# rest are products computed on the integer pipes with the same bits).
#  cg        fused sweep 1: r, p_old, Kx, Ky, u read; p, w, u written (the u += alpha p of the
#            previous iteration folded in; Di, stored, is not counted because the reference
#            recomputes it); p update 1, A p 5, p.w 1, deferred u 1 FP64 operations (Di p on
#            the integer pipes)
#  jacobi    u0, un, Kx, Ky read; u written; 15 operations (the reference's bits: every product
#            and sum rounded separately, the quotient by a corrected reciprocal; six of the
#            seven products on the integer pipes)
#  chebyshev u, u0, p, Kx, Ky read; p, u written; A u 5, r 1, p 2, u 1 (Di u and b r on the
#            integer pipes; w and r are written too on the iterations whose residual the
#            reference checks, and on the last)
#  ppcg      sd, rtemp, utemp, Kx, Ky read; sd, rtemp, utemp written; A sd 5, rtemp 1, sd 2, utemp 1
#            (Di sd and b rtemp on the integer pipes)
KERNELS = {
    "cg": ("cg_matvec", "k_fused_cg_ws (p = r + beta p, w = A p, p.w, deferred u += alpha p; input rows staged "
                        "one row ahead in shared memory; Di p on the integer pipes)", 64, 8, 7),
    "jacobi": ("jacobi", "k_fused_jacobi (u = (u0 + neighbour fluxes of un) / denominator, sum |u - un|; six "
                         "products on the integer pipes)", 40, 15, 9),
    "chebyshev": ("cheby_iterate", "FP64 Chebyshev iteration (k_cheby_iter_ws: w = A u, r = u0 - w, p = a p + b r, "
                                   "u += p in one staged sweep; Di u and b r on the integer pipes)", 56, 9, 7),
    "ppcg": ("ppcg_inner", "FP64 PPCG inner step (k_ppcg_inner_ws: rtemp -= A sd, sd = a sd + b rtemp, utemp += sd in "
                           "one staged sweep; Di sd and b rtemp on the integer pipes)", 64, 9, 7),
}
# The precision form's dominant kernels (FP32 streams, 4 B each): the FP32 CG sweep 1 (r, p_old,
# Kx, Ky, d read; p, w, d written) and one blocked FP32 polynomial step of Chebyshev (d, r, p, Kx,
# Ky read; p, d written) or PPCG (sd, rtemp, utemp, Kx, Ky read; sd, rtemp, utemp written).
MIXED_KERNELS = {
    "cg": ("mix_matvec", "k_mix_w (FP32 p update + matvec + p.w + deferred d += alpha p)", 32),
    "chebyshev": ("poly_step", "k_poly_tb (temporally blocked FP32 Chebyshev steps), per step", 28),
    "ppcg": ("poly_step", "k_poly_tb (temporally blocked FP32 PPCG inner steps), per step", 32),
}
DEFAULT_ITERS = {"cg": 500, "jacobi": 100, "chebyshev": 100, "ppcg": 30}


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--solver", default="cg", choices=["cg", "jacobi", "chebyshev", "ppcg"],
                    help="cg: the 8192^2 headline; jacobi / chebyshev / ppcg: the 4096^2 workloads")
    ap.add_argument("--cells", type=int, default=None, help="mesh size (default 8192 for cg, 4096 otherwise)")
    ap.add_argument("--iters", type=int, default=None, help="iterations per step (tl_max_iters)")
    ap.add_argument("--cpu-iters", type=int, default=None,
                    help="iterations per CPU sample step (default 50 for cg, the GPU window otherwise)")
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"],
                    help="form timed in the main loop (mixed: FP32 steps inside FP64 refinement)")
    ap.add_argument("--no-mixed-compare", action="store_true",
                    help="skip the full-solve FP64 vs mixed time-to-solution comparison")
    ap.add_argument("--delta", type=float, default=0.0, help="mixed: residual replacement factor (0: library default)")
    ap.add_argument("--adjoint", action="store_true",
                    help="instead of the CG line: the adjoint problem (2048^2, 10 steps; gradient of "
                         "sum (u - u_target)^2 wrt density), forward + reverse time and finite-difference checks")
    ap.add_argument("--fd-cells", type=int, default=16, help="adjoint: cells for the per-cell difference check")
    ap.add_argument("--no-workloads", action="store_true",
                    help="cg line: skip the compact measurements of the other workloads (Jacobi / Chebyshev / "
                         "PPCG at 4096^2 with their CPU baselines, the Chebyshev / PPCG time to solution in both "
                         "forms, the 2048^2 adjoint)")
    ap.add_argument("--compare-fp64", action="store_true",
                    help="chebyshev / ppcg: also solve the first time step from the generated state to tl_eps "
                         "in the FP64 and the mixed form and report time, true residual and their differences")
    a = ap.parse_args(argv)
    if a.cells is None:
        a.cells = 8192 if a.solver == "cg" else 4096
    if a.iters is None:
        a.iters = DEFAULT_ITERS[a.solver]
    if a.cpu_iters is None:
        a.cpu_iters = 50 if a.solver == "cg" else a.iters
    return a


def workload(args):
    """The deck of the line: config 5 (cg), config 2 (jacobi) or config 3 (chebyshev / ppcg)."""
    from tealeaf_ref_gb300 import deck as dk

    if args.solver == "cg":
        d = dk.config_deck(5, cells=args.cells)
    elif args.solver == "jacobi":
        d = dk.config_deck(2, solver="jacobi", cells=args.cells)
    else:
        d = dk.config_deck(3, solver=args.solver, cells=args.cells)
        d.ch_cg_presteps = 20
        d.ch_cg_epslim = 1e30
    d.max_iters = args.iters
    return d


def workload_text(args):
    n = args.cells
    if args.solver == "cg":
        return ("TeaLeaf implicit diffusion, FP64 CG, %dx%d cells, 16 rectangles + 4 circles (seed 5), "
                "reciprocal-density keyword, dt 0.004, tl_eps 1e-15; step = one tea_leaf() solve capped at "
                "%d iterations" % (n, n, args.iters))
    if args.solver == "jacobi":
        return ("TeaLeaf implicit diffusion, FP64 Jacobi, %dx%d cells, 8 rectangles (seed 2), reciprocal-density "
                "keyword, dt 0.004, tl_eps 1e-15; step = one tea_leaf() solve capped at %d iterations"
                % (n, n, args.iters))
    extra = ", 10 inner steps" if args.solver == "ppcg" else ""
    return ("TeaLeaf implicit diffusion, FP64 %s, %dx%d cells, 8 rectangles (seed 3), reciprocal-density keyword, "
            "dt 0.004, tl_eps 1e-15, 20 CG presteps then the switch%s; step = one tea_leaf() solve capped at %d "
            "iterations" % ("Chebyshev" if args.solver == "chebyshev" else "PPCG", n, n, extra, args.iters))


def config_json(args, world=None):
    """The config dict of the line, identical in both arms."""
    if world is None:
        world = int(os.environ.get("WORLD_SIZE", "1"))
    return {
        "workload": workload_text(args),
        "cells": args.cells * args.cells,
        "iterations_per_step": args.iters,
        "solver": args.solver,
        "precision": args.precision,
        "l2": "inputs larger than L2 (each field %.0f MB)" % ((args.cells + 2) * (args.cells + 20) * 8 / 1e6),
        "parallelism": "replicas" if world > 1 else "single",
    }


def metric_name(args):
    names = {"cg": "CG", "jacobi": "Jacobi", "chebyshev": "Chebyshev", "ppcg": "PPCG"}
    form = "FP64" if args.precision == "fp64" else "FP32 steps with FP64 refinement"
    return "%s cell-iterations/s (%s, %d^2)" % (names[args.solver], form, args.cells)


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        try:
            with open(p) as f:
                j = json.load(f)
            v = j.get("hbm_gbs") or j.get("hbm_GBps") or j.get("hbm")
            if isinstance(v, dict):
                v = v.get("burst") or v.get("value")
            if v:
                return float(v), "measured"
        except Exception:
            pass
    return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic(kernel_key):
    """DRAM bytes per cell of a launch of the line's kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "roofline_traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        j = json.load(f)
    k = j.get("kernels", {}).get(kernel_key)
    return k


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, mx, pw, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
                pw.append(float(parts[3]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm), "power_w": statistics.median(pw) if pw else None}


def cpu_port_steps(d, iters, steps, warmup, density=None, energy=None):
    """Time the OpenMP CPU port (oracle) on one-step solves capped at `iters` iterations.
    Returns (seconds, iterations, cores)."""
    from oracle import oracle

    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    dd = d.replace(max_iters=iters)
    c = oracle.Chunk(dd.x_cells, dd.y_cells, dd.halo_depth, dd.xmin, dd.ymin, dd.xmax, dd.ymax, dd.coefficient,
                     dd.precond_id, dd.reflective_boundary, threaded=True)
    if density is not None:
        # state taken from the GPU generator; halo cells get the ambient density, as
        # generate_chunk gives them (boundary faces are zeroed afterwards, but their
        # coefficient is still formed from it)
        dens = c.array("density")
        dens[...] = 100.0
        c.interior("density")[...] = density
        c.interior("energy1")[...] = energy
    else:
        c.generate(dd)
        c.start_fields()
    for _ in range(warmup):
        c.tea_leaf(dd)
    times, its = [], 0
    for _ in range(steps):
        t0 = time.perf_counter()
        info = c.tea_leaf(dd)
        times.append(time.perf_counter() - t0)
        its += min(info.n_exit, iters)
    return sum(times), its, cores


def cpu_sample_text(args, steps, iters):
    return ("%d timed one-step solves capped at %d iterations each (%s), %dx%d cells, OpenMP CPU port of the "
            "reference kernels (oracle/)" % (steps, iters, args.solver, args.cells, args.cells))


def mixed_vs_fp64(chunk, d, args):
    """Time to solution of the first time step of the workload (generated initial state,
    tl_eps 1e-15, no iteration cap) in the FP64 form and in the mixed form.  Both results'
    true residuals ||u0 - A u|| are computed in FP64 after the solve (tl_calc_residual,
    tl_calc_2norm), and the mixed result's field summary and u are compared with the FP64
    form's.  The chunk's state is restored afterwards."""
    import numpy as np

    from tealeaf_ref_gb300 import native

    dens0 = chunk.download("density")
    ener0 = chunk.download("energy1")
    chunk.generate(d)
    dens = chunk.download("density")
    ener = chunk.download("energy1")
    full = d.replace(max_iters=200000)
    out = {}
    runs = {}
    for prec in ("fp64", "mixed"):
        chunk.upload_state(dens, ener)
        info = chunk.tea_leaf(native.opts_from_deck(full, prec, inner_tol=args.delta), full.initial_timestep)
        summary, u = chunk.field_summary(), chunk.download("u")
        chunk.update_halo(["u"])
        chunk.calc_residual()
        true_res = float(np.sqrt(abs(chunk.calc_2norm(1))))
        runs[prec] = (info, summary, u)
        out[prec] = {"seconds": info.solve_seconds, "iterations": info.reported_iterations,
                     "relative_true_residual": true_res / info.initial_residual}
        if prec == "mixed":
            out[prec].update(residual_replacements=info.outer_iterations,
                             stop=native.STOP_REASONS.get(info.stop_reason, "?"),
                             true_residual_over_floor=info.true_residual / info.residual_floor)
    (i64, s64, u64), (imx, smx, umx) = runs["fp64"], runs["mixed"]
    out["time_ratio_mixed_over_fp64"] = imx.solve_seconds / i64.solve_seconds
    out["field_summary_max_rel_diff"] = float(np.max(np.abs(smx - s64) / np.abs(s64)))
    out["u_max_rel_diff"] = float(np.max(np.abs(umx - u64) / np.abs(u64)))
    out["workload"] = "first time step of the %dx%d workload from its generated state, tl_eps %g" % (
        args.cells, args.cells, full.eps)
    out["against_oracle"] = ("the FP64 form is held to the oracle at this size on capped windows "
                             "(tests/test_gpu_configs.py); the mixed form is compared with the FP64 form here")
    chunk.upload_state(dens0, ener0)
    return out


def solve_time_to_solution(d, args):
    """Chebyshev / PPCG: the first time step from the generated state solved to tl_eps 1e-15 in
    the FP64 and the mixed form (the 4096^2 workload's time to solution)."""
    import numpy as np

    from tealeaf_ref_gb300 import native

    full = d.replace(max_iters=50000, ch_cg_epslim=1.0)
    first = {}
    for form in ("fp64", "mixed"):
        o = native.opts_from_deck(full, form)
        o.check_result = 1
        with native.Chunk.from_deck(full) as c:
            i = c.tea_leaf(o, full.initial_timestep)
            first[form] = (i, c.field_summary(), c.download("u"))
    (i64, s64, u64), (imx, smx, umx) = first["fp64"], first["mixed"]
    return {
        "workload": "first time step of the %dx%d workload from its generated state, tl_eps 1e-15, "
                    "tl_ch_cg_epslim 1 (the deck default)" % (args.cells, args.cells),
        "fp64": {"seconds": i64.solve_seconds, "iterations": i64.reported_iterations,
                 "relative_true_residual": i64.exact_error / i64.initial_residual},
        "mixed": {"seconds": imx.solve_seconds, "iterations": imx.reported_iterations, "cg_presteps": imx.cg_calc_steps,
                  "relative_true_residual": imx.exact_error / imx.initial_residual,
                  "stop": native.STOP_REASONS.get(imx.stop_reason, str(imx.stop_reason))},
        "time_ratio_mixed_over_fp64": imx.solve_seconds / i64.solve_seconds,
        "field_summary_max_rel_diff": float(max(abs(a - b) / abs(b) for a, b in zip(smx, s64))),
        "u_max_rel_diff": float((np.abs(umx - u64) / np.abs(u64)).max()),
    }


def run_adjoint(args):
    """The adjoint problem: density and energy from the seeded generator (8 rectangles, seed 4),
    u_target from a forward run on density * (1 + 0.01 N(0,1)) (seed 4), loss
    sum (u_final - u_target)^2 after 10 FP64 CG time steps, gradient wrt the per-cell density by
    the reverse sweep (tl_adjoint_*), with each step's u checkpointed on the device.  Checked
    by central differences of the same forward: along a seeded +-1 direction scaled by density
    (h 1e-5), and per cell (4th-order, h 1e-3 relative) on seeded cells among those whose
    gradient is at least 0.1 of the largest -- cells with smaller gradients change L by less
    than the rounding noise of the forward solves (~1e-11 of L)."""
    import numpy as np

    from tealeaf_ref_gb300 import deck as dk
    from tealeaf_ref_gb300 import native
    from tealeaf_ref_gb300.adjoint import forward_loss, perturbed_density, squared_error_gradient

    cells = args.cells if args.cells != 8192 else 2048
    d = dk.config_deck(4, cells=cells)
    T, dt = d.end_step, d.initial_timestep
    opts = native.opts_from_deck(d)
    with native.Chunk.from_deck(d) as c:
        rho, e0 = c.download("density"), c.download("energy1")
        forward_loss(c, perturbed_density(rho, 4), e0, np.zeros_like(rho), opts, dt, T)
        target = c.download("u")
        t0 = time.perf_counter()
        loss0 = forward_loss(c, rho, e0, target, opts, dt, T)
        t_fwd = time.perf_counter() - t0
        t0 = time.perf_counter()
        loss, g, _, rinfo = squared_error_gradient(c, rho, e0, target, opts, dt, T, rho_only=True)
        t_both = time.perf_counter() - t0
        rng = np.random.Generator(np.random.PCG64(4))
        v = rho * rng.choice([-1.0, 1.0], size=rho.shape)
        h = 1e-5
        fd_dir = (forward_loss(c, rho + h * v, e0, target, opts, dt, T) -
                  forward_loss(c, rho - h * v, e0, target, opts, dt, T)) / (2 * h)
        g_dir = float(np.sum(g * v))
        gmax = float(np.max(np.abs(g)))
        big = np.argwhere(np.abs(g) >= 0.1 * gmax)
        pick = big[rng.choice(len(big), size=min(args.fd_cells, len(big)), replace=False)]
        per_cell = []
        for idx in map(tuple, pick):
            hh = 1e-3 * rho[idx]

            def at(s):
                p = rho.copy()
                p[idx] += s * hh
                return forward_loss(c, p, e0, target, opts, dt, T)

            fd = (8 * (at(1) - at(-1)) - (at(2) - at(-2))) / (12 * hh)
            per_cell.append({"cell": [int(idx[0]), int(idx[1])], "grad": float(g[idx]), "fd": fd,
                             "rel_err": abs(fd - g[idx]) / abs(g[idx])})
    out = {
        "metric": "adjoint: forward + reverse time for d/d(density) of sum (u - u_target)^2 (FP64, %d^2, %d steps)"
                  % (cells, T),
        "value": t_both,
        "unit": "s",
        "higher_is_better": False,
        "forward_s": t_fwd,
        "reverse_s": t_both - t_fwd,
        "reverse_cg_iterations": rinfo.reported_iterations,
        "loss": loss,
        "loss_forward_only": loss0,
        "fd_directional": {"h": h, "direction": "density * (+-1, seeded)", "fd": fd_dir, "adjoint": g_dir,
                           "rel_err": abs(fd_dir - g_dir) / abs(g_dir)},
        "fd_cells": {"h_rel": 1e-3, "stencil": "4th-order central", "selection": "seeded, |g| >= 0.1 max|g|",
                     "max_rel_err": max(x["rel_err"] for x in per_cell), "cells": per_cell},
        "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": "adjoint problem: %dx%d cells, 8 rectangles (seed 4), reciprocal-density keyword, "
                               "dt 0.004, %d FP64 CG steps at tl_eps 1e-15, per-step u checkpoints" % (cells, cells, T)},
    }
    print(json.dumps(out), flush=True)


def run_reference(args):
    """The reference arm: the CPU port of the reference kernels on all host cores, on a bounded
    sample of the same workload (steps capped at --cpu-iters iterations), rank 0 only."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    d = workload(args)
    iters = args.cpu_iters
    total, its, cores = cpu_port_steps(d, iters, args.steps, args.warmup)
    cells = args.cells * args.cells
    value = cells * its / total
    sample = cpu_sample_text(args, args.steps, iters)
    out = {
        "impl": "reference",
        "metric": metric_name(args),
        "value": value,
        "unit": "cell-iterations/s",
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": config_json(args),
        "cpu_sample": {"iterations_per_step": iters, "steps": args.steps, "warmup_steps": args.warmup,
                       "what": "each step is a bounded sample of the workload's step: the same solve capped at "
                               "%d iterations" % iters},
        "cpu_baseline": {"value": value, "unit": "cell-iterations/s", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "cell-iterations/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
    }
    print(json.dumps(out), flush=True)


def compact_line(solver, steps=5, warmup=2, cpu_steps=1):
    """A compact measurement of one 4096^2 solver line (device-timed steps with the line's kernel
    timer, its roofline figure and the CPU port on the same window), for the record of the
    headline run."""
    from tealeaf_ref_gb300 import native

    a = parse(["--solver", solver, "--steps", str(steps), "--warmup", str(warmup)])
    d = workload(a)
    opts = native.opts_from_deck(d)
    dt = d.initial_timestep
    cells = a.cells * a.cells
    timer, kernel_text, kbytes, kops, _ = KERNELS[solver]
    with native.Chunk.from_deck(d) as c:
        for _ in range(warmup):
            c.tea_leaf(opts, dt)
        c.profile(True)
        infos = [c.tea_leaf(opts, dt) for _ in range(steps)]
        k_ms, k_n = c.profile_read(timer)
        c.profile(False)
        dens, ener = c.download("density"), c.download("energy1")
    dev_s = sum(i.solve_seconds for i in infos)
    its = sum(min(i.n_exit, a.iters) for i in infos)
    peak, _ = measured_peaks()
    t_launch = k_ms / k_n * 1e-3 if k_n else None
    out = {"metric": metric_name(a), "value": cells * its / dev_s, "unit": "cell-iterations/s",
           "ms_per_step": 1e3 * dev_s / steps, "steps": steps, "warmup": warmup, "config": config_json(a, 1),
           "roofline": {"kernel": kernel_text, "algorithmic_bytes_per_cell": kbytes,
                        "launch_ms": k_ms / k_n if k_n else None,
                        "achieved_gbs": kbytes * cells / t_launch / 1e9 if t_launch else None,
                        "frac": kbytes * cells / t_launch / 1e9 / peak if t_launch else None}}
    try:
        total, cits, cores = cpu_port_steps(d, a.cpu_iters, cpu_steps, 1, dens, ener)
        out["cpu_baseline"] = {"value": cells * cits / total, "unit": "cell-iterations/s", "cores": cores,
                               "kind": "port", "sample": cpu_sample_text(a, cpu_steps, a.cpu_iters)}
    except Exception as e:  # the baseline is reported, never required
        out["cpu_baseline"] = {"value": None, "sample": "failed: %s" % e}
    return out


def adjoint_timing():
    """The 2048^2 adjoint problem's forward and reverse times and its directional
    finite-difference check (the per-cell checks: --adjoint)."""
    import numpy as np

    from tealeaf_ref_gb300 import deck as dk
    from tealeaf_ref_gb300 import native
    from tealeaf_ref_gb300.adjoint import forward_loss, perturbed_density, squared_error_gradient

    d = dk.config_deck(4)
    T, dt = d.end_step, d.initial_timestep
    opts = native.opts_from_deck(d)
    with native.Chunk.from_deck(d) as c:
        rho, e0 = c.download("density"), c.download("energy1")
        forward_loss(c, perturbed_density(rho, 4), e0, np.zeros_like(rho), opts, dt, T)
        target = c.download("u")
        t0 = time.perf_counter()
        forward_loss(c, rho, e0, target, opts, dt, T)
        t_fwd = time.perf_counter() - t0
        t0 = time.perf_counter()
        loss, g, _, rinfo = squared_error_gradient(c, rho, e0, target, opts, dt, T, rho_only=True)
        t_both = time.perf_counter() - t0
        rng = np.random.Generator(np.random.PCG64(4))
        v = rho * rng.choice([-1.0, 1.0], size=rho.shape)
        h = 1e-5
        fd = (forward_loss(c, rho + h * v, e0, target, opts, dt, T) -
              forward_loss(c, rho - h * v, e0, target, opts, dt, T)) / (2 * h)
        gd = float(np.sum(g * v))
    return {"workload": "adjoint problem: 2048x2048 cells, 8 rectangles (seed 4), 10 FP64 CG steps, loss "
                        "sum (u - u_target)^2, gradient wrt density",
            "forward_s": t_fwd, "forward_and_reverse_s": t_both, "reverse_s": t_both - t_fwd,
            "reverse_cg_iterations": rinfo.reported_iterations,
            "fd_directional": {"h": h, "fd": fd, "adjoint": gd, "rel_err": abs(fd - gd) / abs(gd)}}


def other_workloads():
    """The record of every other workload, measured after the headline (rank 0, one GPU)."""
    out = {}
    for s in ("jacobi", "chebyshev", "ppcg"):
        try:
            out[s] = compact_line(s)
        except Exception as e:
            out[s] = {"failed": str(e)}
    for s in ("ppcg", "chebyshev"):
        try:
            a = parse(["--solver", s])
            out["%s_time_to_solution" % s] = solve_time_to_solution(workload(a), a)
        except Exception as e:
            out["%s_time_to_solution" % s] = {"failed": str(e)}
    try:
        out["adjoint"] = adjoint_timing()
    except Exception as e:
        out["adjoint"] = {"failed": str(e)}
    return out


def e2e_legs(chunk, opts, dt, args, grp, cells):
    """End to end through the C ABI with pinned host buffers.  The steady-state step time of each
    form (synchronous; pipelined), from untimed runs of one and of three steps (the difference
    over two steps leaves out the pipelined form's fill), picks the form of the timed steps; the
    other form is then timed too.  Returns the e2e dict and the host arrays (density, energy) for
    the CPU leg."""
    from tealeaf_ref_gb300 import native, replicas

    world = grp.world
    pins = [native.PinnedArray((args.cells, args.cells)) for _ in range(3)]
    dens, ener, out = (p.array for p in pins)
    chunk.download("density", out=dens)
    chunk.download("energy1", out=ener)
    chunk.upload_state(dens, ener)
    chunk.tea_leaf(opts, dt)

    def sync_steps(n):
        its, parts = 0, [0.0, 0.0, 0.0]
        grp.barrier()
        t0 = time.perf_counter()
        for _ in range(n):
            ta = time.perf_counter()
            chunk.upload_state(dens, ener)
            tb = time.perf_counter()
            info = chunk.tea_leaf(opts, dt)
            tc = time.perf_counter()
            chunk.download("energy1", out=out)
            td = time.perf_counter()
            its += min(info.n_exit, args.iters)
            parts[0] += tb - ta
            parts[1] += info.solve_seconds
            parts[2] += td - tc
        wall = grp.max(time.perf_counter() - t0)
        return wall, its, {k: 1e3 * v / n for k, v in zip(("upload", "solve_device", "download"), parts)}

    def pipelined_steps(n):
        its, parts = 0, [0.0, 0.0, 0.0, 0.0]
        grp.barrier()
        t0 = time.perf_counter()
        for _ in range(min(2, n)):
            chunk.stage_state(dens, ener)
        for s in range(n):
            ta = time.perf_counter()
            chunk.take_staged()
            tb = time.perf_counter()
            info = chunk.tea_leaf(opts, dt)
            tc = time.perf_counter()
            its += min(info.n_exit, args.iters)
            chunk.fetch("energy1", out)
            if s + 2 < n:
                chunk.stage_state(dens, ener)
            td = time.perf_counter()
            parts[0] += tb - ta
            parts[1] += tc - tb
            parts[2] += info.solve_seconds
            parts[3] += td - tc
        chunk.wait_transfers()
        wall = grp.max(time.perf_counter() - t0)
        return wall, its, {k: 1e3 * v / n for k, v in zip(("take", "solve_host", "solve_device", "fetch_stage"), parts)}

    forms = {"synchronous": sync_steps, "pipelined": pipelined_steps}
    # the untimed pick: steady-state step time of each form
    probe = {}
    for name, fn in forms.items():
        one = fn(1)[0]
        probe[name] = max(fn(3)[0] - one, 0.0) / 2
    chosen = min(probe, key=probe.get)
    other = "pipelined" if chosen == "synchronous" else "synchronous"
    with Clocks(grp.local) as clk:
        wall, its, parts = forms[chosen](args.steps)
    o_wall, o_its, o_parts = forms[other](args.steps)
    e2e = {"value": replicas.whole_job_rate(world, cells, its, wall), "unit": "cell-iterations/s",
           "h2d_bytes_per_step": 2 * cells * 8, "d2h_bytes_per_step": cells * 8,
           "ms_per_step": 1e3 * wall / args.steps, "form": chosen,
           "form_choice": "the faster steady-state step of the two forms (untimed runs of 3 and 1 steps, "
                          "difference / 2): %s" % (
               ", ".join("%s %.1f ms" % (k, 1e3 * v) for k, v in probe.items())),
           "ms_per_step_parts": parts,
           "other_form": {"form": other, "value": replicas.whole_job_rate(world, cells, o_its, o_wall),
                          "ms_per_step": 1e3 * o_wall / args.steps, "ms_per_step_parts": o_parts},
           "clocks": clk.summary()}
    return e2e, dens, ener, pins


def main(argv=None):
    args = parse(argv)
    if args.impl == "reference":
        run_reference(args)
        return
    if args.adjoint:
        run_adjoint(args)
        return
    from tealeaf_ref_gb300 import replicas

    grp = replicas.init()
    world, rank, local = grp.world, grp.rank, grp.local

    from tealeaf_ref_gb300 import native

    native.set_device(local)
    d = workload(args)
    opts = native.opts_from_deck(d, args.precision, inner_tol=args.delta)
    dt = d.initial_timestep
    cells = args.cells * args.cells
    if args.precision == "mixed" and args.solver == "jacobi":
        raise SystemExit("the precision form is built for CG, Chebyshev and PPCG")
    timer, kernel_text, kbytes, kops, kpipe = KERNELS[args.solver]
    if args.precision == "mixed":
        timer, kernel_text, kbytes = MIXED_KERNELS[args.solver]

    chunk = native.Chunk.from_deck(d)
    for _ in range(args.warmup):
        chunk.tea_leaf(opts, dt)

    # ---- device-resident timed region (per-launch timers on, CUDA events on the solve stream) ----
    chunk.profile(True)
    grp.barrier()
    infos = []
    with Clocks(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            infos.append(chunk.tea_leaf(opts, dt))
        wall = time.perf_counter() - t0
    grp.barrier()
    dev_s = sum(i.solve_seconds for i in infos)
    its = sum(min(i.n_exit, args.iters) for i in infos)
    launches = sum(i.kernel_launches for i in infos)
    k_ms, k_n = chunk.profile_read(timer)
    up_ms, up_n = chunk.profile_read("cg_update")
    chunk.profile(False)
    t_max = grp.max(dev_s)
    value = replicas.whole_job_rate(world, cells, its, t_max)

    # ---- end to end through the C ABI with host buffers ----
    e2e, dens, ener, pins = (None, None, None, None)
    if not args.no_e2e:
        e2e, dens, ener, pins = e2e_legs(chunk, opts, dt, args, grp, cells)

    peak, peak_kind = measured_peaks()
    t_launch = k_ms / k_n * 1e-3 if k_n else None
    achieved = kbytes * cells / t_launch / 1e9 if t_launch else None
    traffic = ncu_traffic(args.solver if args.precision == "fp64" else None)
    roofline = {
        "bound": "hbm",
        "kernel": kernel_text,
        "achieved": achieved,
        "peak": peak,
        "unit": "GB/s",
        "frac": achieved / peak if achieved else None,
        "peak_source": peak_kind,
        "traffic": traffic["bytes_per_cell"] * cells if traffic else None,
        "traffic_source": traffic.get("source") if traffic else None,
        "algorithmic_bytes_per_cell": kbytes,
        "launch_ms": k_ms / k_n if k_n else None,
        "launches": k_n,
    }
    if args.solver == "cg":
        roofline["update_kernel_launch_ms"] = up_ms / up_n if up_n else None
        roofline["iteration_gbs_at_96B"] = BYTES_PER_CELL_IT * cells * its / dev_s / 1e9 if dev_s else None
        if dev_s:
            roofline["iteration_frac_at_96B"] = roofline["iteration_gbs_at_96B"] / peak
    if t_launch and args.precision == "fp64":
        import torch

        sms = torch.cuda.get_device_properties(local).multi_processor_count
        mhz = clk.summary().get("sm_max_mhz") or 2070.0
        fp64_peak = FP64_OPS_PER_CLOCK_SM * sms * mhz * 1e6
        fp64_achieved = kpipe * cells / t_launch
        roofline["fp64_issue"] = {
            "ops_per_cell": kops, "fp64_pipe_ops_per_cell": kpipe, "achieved_tops": fp64_achieved / 1e12,
            "peak_tops": fp64_peak / 1e12, "frac": fp64_achieved / fp64_peak,
            "peak_source": "%d FP64 thread-ops per clock per SM (ncu's FP64 pipe peak) x %d SMs x %.0f MHz"
                           % (FP64_OPS_PER_CLOCK_SM, sms, mhz)}
        roofline["note"] = "FP64 issue rate (0.63 T ops/s) bounds the sweep before HBM does"

    extra = None
    if rank == 0 and world == 1:
        if args.solver == "cg" and not args.no_mixed_compare:
            extra = ("mixed_vs_fp64", mixed_vs_fp64(chunk, d, args))
        elif args.solver in ("chebyshev", "ppcg") and args.compare_fp64:
            extra = ("time_to_solution", solve_time_to_solution(d, args))

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            total, cits, cores = cpu_port_steps(d, args.cpu_iters, args.cpu_steps, 1, dens, ener)
            cpu = {"value": cells * cits / total, "unit": "cell-iterations/s", "cores": cores, "kind": "port",
                   "sample": cpu_sample_text(args, args.cpu_steps, args.cpu_iters)}
        except Exception as e:  # the baseline is reported, never required
            cpu = {"value": None, "unit": "cell-iterations/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": "failed: %s" % e}

    if rank == 0:
        out = {
            "metric": metric_name(args),
            "value": value,
            "unit": "cell-iterations/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": 1e3 * t_max / args.steps,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64" if args.precision == "fp64" else "f32+f64",
            "data": "synthetic",
            "config": config_json(args, world),
            "iterations_per_step": [i.reported_iterations for i in infos],
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": launches,
            "clocks": clk.summary(),
            "wall_s_timed": wall,
        }
        if args.solver == "ppcg":
            out["ppcg_inner_per_step"] = [i.ppcg_inner_iters for i in infos]
        if extra:
            out[extra[0]] = extra[1]
    if pins:
        for p in pins:
            p.close()
    chunk.close()
    if rank == 0:
        if world == 1 and args.solver == "cg" and args.precision == "fp64" and not args.no_workloads:
            out["other_workloads"] = other_workloads()
        print(json.dumps(out), flush=True)
    grp.close()


if __name__ == "__main__":
    main()
