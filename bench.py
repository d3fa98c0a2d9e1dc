#!/usr/bin/env python3
"""Benchmark: FP64 CG cell-iterations/s of TeaLeaf's implicit solve at 8192^2 on GB300.

Workload (synthetic config 5): 8192 x 8192 cells on the 10 x 10 domain, ambient state
(density 100, energy 1e-4) + 16 seeded rectangles (density U[0.1,1], energy U[1,25]) +
4 seeded circles (density 0.1, energy 25), reciprocal-density coefficient keyword,
dt 0.004, tl_eps 1e-15, CG, FP64.  A step is one tea_leaf() time-step solve through the
C ABI capped at --iters CG iterations (tl_max_iters, default 500): Kx/Ky/Di set-up, initial
residual, --iters fused CG iterations, finalise.  At this size a full time step needs tens
of thousands of iterations, so the cap keeps a step under a second; iterations are the work
unit of the metric (cells x iterations / time), as in the reference's own grind figures.

value  : device time (CUDA events on the solver stream) of the K timed steps, inputs
         resident in HBM (every step reads ~14 fields of 0.54 GB: larger than L2).
e2e    : the same steps through the C ABI with host buffers, host wall clock: every step's
         density/energy copied from pinned host memory and its energy copied back, the copies
         pipelined on their own streams (tl_stage_state two steps ahead, tl_fetch_field) so
         they overlap the solves; e2e.synchronous is the upload/solve/download form.
roofline: the dominant kernel (fused p-update + matvec + p.w sweep) timed per launch with
         CUDA events during the timed steps, against 64 B/cell of compulsory traffic (the
         p update and matvec streams plus the deferred u += alpha p of the previous step).
cpu_baseline: the CPU port (oracle/, OpenMP over all host cores) on a bounded sample of
         the same workload (one time-step solve capped at --cpu-iters iterations).

--impl reference times that CPU port alone as the reference arm.  Under torchrun (N>1)
every rank runs an independent replica of the workload on its own GPU (the solve has no
multi-GPU decomposition here), barrier + max-over-ranks time.
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

# compulsory traffic of the fused sweep: r, p_old, Kx, Ky, u read; p, w, u written (8 B each).
# The u += alpha p of the previous step is folded into it; Di (stored, 8 B more) is not
# counted because the reference recomputes it from Kx, Ky.
BYTES_PER_CELL_MATVEC = 64
BYTES_PER_CELL_IT = 96      # whole FP64 CG iteration (12 streams)
FP64_OPS_MATVEC = 8         # FP64 operations per cell of the matvec sweep: p update 1, A p 5, p.w 1, deferred u 1
FP64_OPS_PER_CLOCK_SM = 2   # FP64 pipe peak that ncu reports for GB300: 2 thread-operations per clock per SM
FALLBACK_HBM_GBS = 6800.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cells", type=int, default=8192)
    ap.add_argument("--iters", type=int, default=500, help="CG iterations per step (tl_max_iters)")
    ap.add_argument("--cpu-iters", type=int, default=5, help="CG iterations per CPU sample step")
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"],
                    help="form timed in the main loop (mixed: FP32 CG steps with FP64 residual replacement)")
    ap.add_argument("--no-mixed-compare", action="store_true",
                    help="skip the full-solve FP64 vs mixed time-to-solution comparison")
    ap.add_argument("--delta", type=float, default=0.0, help="mixed: residual replacement factor (0: library default)")
    ap.add_argument("--adjoint", action="store_true",
                    help="instead of the CG line: the adjoint problem (2048^2, 10 steps; gradient of "
                         "sum (u - u_target)^2 wrt density), forward + reverse time and finite-difference checks")
    ap.add_argument("--fd-cells", type=int, default=8, help="adjoint: cells for the per-cell difference check")
    ap.add_argument("--solver", default="cg", choices=["cg", "jacobi", "chebyshev", "ppcg"],
                    help="jacobi / chebyshev / ppcg: instead of the CG line, time steps of that solver on the "
                         "4096^2 workloads (Jacobi: 8 rectangles, seed 2, capped at --iters; Chebyshev / PPCG: "
                         "seed 3, 20 CG presteps, PPCG 10 inner steps, solved to tl_eps) and report per-kernel "
                         "GB/s from a separately profiled step")
    ap.add_argument("--compare-fp64", action="store_true",
                    help="chebyshev / ppcg with --precision mixed: also solve the first time step from the "
                         "generated state in both forms and report time, true residual and the mixed form's "
                         "field-summary and per-cell u differences")
    ap.add_argument("--ch-cg-epslim", type=float, default=None,
                    help="chebyshev / ppcg: override tl_ch_cg_epslim (the error below which CG hands over "
                         "after its presteps; a large value switches right after them)")
    return ap.parse_args()


def workload(args):
    from tealeaf_ref_gb300 import deck as dk

    d = dk.config_deck(5, cells=args.cells)
    d.max_iters = args.iters
    return d


def config_json(args, d):
    return {
        "workload": "TeaLeaf implicit diffusion, FP64 CG, %dx%d cells, 16 rectangles + 4 circles (seed 5), "
                    "reciprocal-density keyword, dt 0.004, tl_eps 1e-15; step = one tea_leaf() solve capped at "
                    "%d iterations" % (args.cells, args.cells, args.iters),
        "cells": args.cells * args.cells,
        "iterations_per_step": args.iters,
        "solver": "cg",
        "precision": "fp64",
        "l2": "inputs larger than L2 (each field %.0f MB, ~14 fields touched per step)" % (
            (args.cells + 2) * (args.cells + 18) * 8 / 1e6),
    }


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


def ncu_traffic():
    p = os.path.join(ROOT, "profiles", "roofline_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return None


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
    """Time the OpenMP CPU port (oracle) on one-step solves capped at `iters` iterations."""
    from oracle import oracle

    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    dd = d.replace(max_iters=iters)
    c = oracle.Chunk(dd.x_cells, dd.y_cells, dd.halo_depth, dd.xmin, dd.ymin, dd.xmax, dd.ymax, dd.coefficient,
                     dd.precond_id, dd.reflective_boundary, threaded=True)
    if density is not None:
        # state taken from the GPU generator (the CPU generator is slow at this size); halo
        # cells get the ambient density, as generate_chunk gives them (boundary faces are
        # zeroed afterwards, but their coefficient is still formed from it)
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
        its += info.n_exit if info.n_exit <= iters else iters
    return sum(times), its, cores


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
    chunk.upload_state(dens0, ener0)
    return out


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


# Compulsory bytes per cell of one launch (or one step) of each timed kernel: FP64 Chebyshev
# iterate 56 B (u, u0, p, Kx, Ky read; p, u written), PPCG inner step 64 B (sd, rtemp, utemp,
# Kx, Ky read; sd, rtemp, utemp written), Jacobi 40 B (u0, un, Kx, Ky read; u written); the
# FP32 forms at 4 B per stream: PPCG inner step 32 B, Chebyshev step on a correction 28 B
# (d, r, p, Kx, Ky read; p, d written); FP32 CG sweeps 32 B (r, p_old, Kx, Ky, d read; p, w, d
# written) and 12 B (w, r read; r written).
KERNEL_BYTES = {"cheby_iterate": 56, "ppcg_inner": 64, "jacobi": 40, "mix_matvec": 32, "mix_update": 12,
                "cg_matvec": 64, "cg_update": 24}
POLY_BYTES = {"ppcg": 32, "chebyshev": 28}


def run_solver(args):
    """Time steps of the Jacobi, Chebyshev or PPCG solver (FP64 or mixed form) on the 4096^2
    workloads; per-kernel times come from one more step run with the kernel timers on (the
    host-driven loops wait for each timed launch, so that step is not part of the timing)."""
    from tealeaf_ref_gb300 import deck as dk
    from tealeaf_ref_gb300 import native

    cells_n = args.cells if args.cells != 8192 else 4096
    if args.solver == "jacobi":
        d = dk.config_deck(2, solver="jacobi", cells=cells_n)
        d.max_iters = args.iters
    else:
        d = dk.config_deck(3, solver=args.solver, cells=cells_n)
        d.ch_cg_presteps = 20
        if args.ch_cg_epslim is not None:
            d.ch_cg_epslim = args.ch_cg_epslim
    opts = native.opts_from_deck(d, args.precision)
    dt = d.initial_timestep
    cells = cells_n * cells_n
    with native.Chunk.from_deck(d) as c:
        for _ in range(args.warmup):
            c.tea_leaf(opts, dt)
        infos = []
        with Clocks(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
            for _ in range(args.steps):
                infos.append(c.tea_leaf(opts, dt))
        dev_s = sum(i.solve_seconds for i in infos)
        c.profile(True)
        pinfo = c.tea_leaf(opts, dt)
        kernels = {}
        for name, kid in native.KERNEL_TIMERS.items():
            ms, n = c.profile_read(name)
            if not n:
                continue
            basis = (POLY_BYTES[args.solver] if name == "poly_step" else KERNEL_BYTES[name])
            avg = ms / n * 1e-3
            kernels[name] = {"launches": n, "ms_avg": 1e3 * avg, "bytes_per_cell": basis,
                             "gbs": basis * cells / avg / 1e9}
        c.profile(False)
    compare = None
    if args.compare_fp64 and args.precision == "mixed" and args.solver != "jacobi":
        first = {}
        for form in ("fp64", "mixed"):
            o = native.opts_from_deck(d, form)
            o.check_result = 1
            with native.Chunk.from_deck(d) as c:
                i = c.tea_leaf(o, dt)
                first[form] = (i, c.field_summary(), c.download("u"))
        (i64, s64, u64), (imx, smx, umx) = first["fp64"], first["mixed"]
        compare = {
            "workload": "first time step of the %dx%d workload from its generated state, tl_eps 1e-15" % (cells_n,
                                                                                                        cells_n),
            "fp64": {"seconds": i64.solve_seconds, "iterations": i64.reported_iterations,
                     "relative_true_residual": i64.exact_error / i64.initial_residual},
            "mixed": {"seconds": imx.solve_seconds, "iterations": imx.reported_iterations,
                      "cg_presteps": imx.cg_calc_steps,
                      "relative_true_residual": imx.exact_error / imx.initial_residual,
                      "stop": native.STOP_REASONS.get(imx.stop_reason, str(imx.stop_reason))},
            "time_ratio_mixed_over_fp64": imx.solve_seconds / i64.solve_seconds,
            "field_summary_max_rel_diff": float(max(abs(a - b) / abs(b) for a, b in zip(smx, s64))),
            "u_max_rel_diff": float((abs(umx - u64) / abs(u64)).max()),
        }
    peak, peak_kind = measured_peaks()
    for k in kernels.values():
        k["frac_of_peak"] = k["gbs"] / peak
    out = {
        "metric": "%s time per time step (%s, %d^2)" % (args.solver, args.precision, cells_n),
        "value": dev_s / args.steps,
        "unit": "s",
        "higher_is_better": False,
        "n_gpus": 1,
        "steps": args.steps,
        "warmup": args.warmup,
        "iterations_per_step": [i.reported_iterations for i in infos],
        "ppcg_inner_per_step": [i.ppcg_inner_iters for i in infos],
        "cg_presteps_per_step": [i.cg_calc_steps for i in infos],
        "cell_iterations_per_s": cells * sum(i.reported_iterations for i in infos) / dev_s,
        "kernels": kernels,
        "peak_gbs": peak,
        "peak_source": peak_kind,
        "profiled_step_iterations": pinfo.reported_iterations,
        "mixed_vs_fp64": compare,
        "dtype": "f64" if args.precision == "fp64" else "f32+f64",
        "data": "synthetic",
        "clocks": clk.summary(),
        "config": {"workload": "TeaLeaf implicit diffusion, %s (%s), %dx%d cells, 8 rectangles, reciprocal-density "
                               "keyword, dt 0.004, tl_eps 1e-15%s" % (
                                   args.solver, args.precision, cells_n, cells_n,
                                   ", capped at %d iterations" % args.iters if args.solver == "jacobi" else
                                   ", 20 CG presteps" + (", 10 PPCG inner steps" if args.solver == "ppcg" else ""))},
    }
    print(json.dumps(out), flush=True)


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    d = workload(args)
    iters = args.cpu_iters
    total, its, cores = cpu_port_steps(d, iters, args.steps, args.warmup)
    cells = args.cells * args.cells
    value = cells * its / total
    out = {
        "impl": "reference",
        "metric": "CG cell-iterations/s (FP64, %d^2)" % args.cells,
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
        "config": dict(config_json(args, d), cpu_sample_iterations_per_step=iters),
        "cpu_baseline": {"value": value, "unit": "cell-iterations/s", "cores": cores, "kind": "port",
                         "sample": "%d timed one-step solves capped at %d CG iterations each, %dx%d cells, "
                                   "OpenMP CPU port of the reference kernels" % (args.steps, iters, args.cells,
                                                                                 args.cells)},
        "e2e": {"value": value, "unit": "cell-iterations/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
    }
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.adjoint:
        run_adjoint(args)
        return
    if args.solver != "cg":
        run_solver(args)
        return
    from tealeaf_ref_gb300 import replicas

    grp = replicas.init()
    world, rank, local = grp.world, grp.rank, grp.local

    import numpy as np

    from tealeaf_ref_gb300 import native

    native.set_device(local)
    d = workload(args)
    opts = native.opts_from_deck(d, args.precision, inner_tol=args.delta)
    dt = d.initial_timestep
    cells = args.cells * args.cells

    chunk = native.Chunk.from_deck(d)
    for _ in range(args.warmup):
        chunk.tea_leaf(opts, dt)

    barrier = grp.barrier
    max_over_ranks = grp.max

    # ---- device-resident timed region ----
    chunk.profile(True)
    barrier()
    infos = []
    with Clocks(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            infos.append(chunk.tea_leaf(opts, dt))
        wall = time.perf_counter() - t0
    barrier()
    dev_s = sum(i.solve_seconds for i in infos)
    its = sum(min(i.n_exit, args.iters) for i in infos)
    launches = sum(i.kernel_launches for i in infos)
    mv_ms, mv_n = chunk.profile_read("cg_matvec")
    up_ms, up_n = chunk.profile_read("cg_update")
    chunk.profile(False)
    t_max = max_over_ranks(dev_s)
    value = replicas.whole_job_rate(world, cells, its, t_max)

    # ---- end to end through the C ABI with host buffers ----
    e2e = None
    if not args.no_e2e:
        pins = [native.PinnedArray((args.cells, args.cells)) for _ in range(3)]
        dens, ener, out = (p.array for p in pins)
        chunk.download("density", out=dens)
        chunk.download("energy1", out=ener)
        chunk.upload_state(dens, ener)
        chunk.tea_leaf(opts, dt)
        barrier()
        # Synchronous form: upload, solve, download, one after the other.
        s_its = 0
        t0 = time.perf_counter()
        for _ in range(args.steps):
            chunk.upload_state(dens, ener)
            s_its += min(chunk.tea_leaf(opts, dt).n_exit, args.iters)
            chunk.download("energy1", out=out)
        s_wall = max_over_ranks(time.perf_counter() - t0)
        barrier()
        # Pipelined form (the headline): each step's inputs are staged two steps ahead on the
        # upload stream and its energy is fetched on the download stream, so the copies run
        # during the solves.  Every step still moves its own inputs and result across the link.
        e_its = 0
        parts = [0.0, 0.0, 0.0, 0.0]  # take (host), solve (host), solve (device), fetch + stage (host)
        with Clocks(local) as clk_e2e:
            t0 = time.perf_counter()
            for _ in range(min(2, args.steps)):
                chunk.stage_state(dens, ener)
            for s in range(args.steps):
                ta = time.perf_counter()
                chunk.take_staged()
                tb = time.perf_counter()
                info = chunk.tea_leaf(opts, dt)
                tc = time.perf_counter()
                e_its += min(info.n_exit, args.iters)
                chunk.fetch("energy1", out)
                if s + 2 < args.steps:
                    chunk.stage_state(dens, ener)
                td = time.perf_counter()
                parts[0] += tb - ta
                parts[1] += tc - tb
                parts[2] += info.solve_seconds
                parts[3] += td - tc
            chunk.wait_transfers()
            e_wall = time.perf_counter() - t0
        barrier()
        e_wall = max_over_ranks(e_wall)
        e2e = {"value": replicas.whole_job_rate(world, cells, e_its, e_wall), "unit": "cell-iterations/s",
               "h2d_bytes_per_step": 2 * cells * 8, "d2h_bytes_per_step": cells * 8,
               "ms_per_step": 1e3 * e_wall / args.steps, "transfers": "pipelined (tl_stage_state/tl_fetch_field)",
               "ms_per_step_parts": {k: 1e3 * v / args.steps for k, v in
                                     zip(("take", "solve_host", "solve_device", "fetch_stage"), parts)},
               "synchronous": {"value": replicas.whole_job_rate(world, cells, s_its, s_wall),
                               "ms_per_step": 1e3 * s_wall / args.steps},
               "clocks": clk_e2e.summary()}

    peak, peak_kind = measured_peaks()
    t_launch = mv_ms / mv_n * 1e-3 if mv_n else None
    achieved = BYTES_PER_CELL_MATVEC * cells / t_launch / 1e9 if t_launch else None
    traffic = ncu_traffic()
    per_launch_traffic = None
    if traffic and traffic.get("cells"):
        per_launch_traffic = traffic["bytes_per_cell"] * cells
    roofline = {
        "bound": "hbm",
        "kernel": "k_fused_cg_w (p = r + beta p, w = A p, p.w)",
        "achieved": achieved,
        "peak": peak,
        "unit": "GB/s",
        "frac": achieved / peak if achieved else None,
        "peak_source": peak_kind,
        "traffic": per_launch_traffic,
        "algorithmic_bytes_per_cell": BYTES_PER_CELL_MATVEC,
        "launch_ms": mv_ms / mv_n if mv_n else None,
        "launches": mv_n,
        "update_kernel_launch_ms": up_ms / up_n if up_n else None,
        "iteration_gbs_at_96B": BYTES_PER_CELL_IT * cells * its / dev_s / 1e9 if dev_s else None,
        "note": "FP64 issue rate (measured 0.60 T DFMA/s) bounds the sweep before HBM does",
    }
    if t_launch:
        import torch

        sms = torch.cuda.get_device_properties(local).multi_processor_count
        mhz = clk.summary().get("sm_max_mhz") or 2070.0
        fp64_peak = FP64_OPS_PER_CLOCK_SM * sms * mhz * 1e6
        fp64_achieved = FP64_OPS_MATVEC * cells / t_launch
        roofline["fp64_issue"] = {
            "ops_per_cell": FP64_OPS_MATVEC, "achieved_tops": fp64_achieved / 1e12, "peak_tops": fp64_peak / 1e12,
            "frac": fp64_achieved / fp64_peak,
            "peak_source": "%d FP64 thread-ops per clock per SM (ncu's FP64 pipe peak) x %d SMs x %.0f MHz"
                           % (FP64_OPS_PER_CLOCK_SM, sms, mhz)}

    mixed_cmp = None
    if rank == 0 and world == 1 and not args.no_mixed_compare:
        mixed_cmp = mixed_vs_fp64(chunk, d, args)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            total, cits, cores = cpu_port_steps(d, args.cpu_iters, args.cpu_steps, 1, dens if e2e else None,
                                                ener if e2e else None)
            cpu = {"value": cells * cits / total, "unit": "cell-iterations/s", "cores": cores, "kind": "port",
                   "sample": "%d one-step solves capped at %d CG iterations, %dx%d cells, OpenMP CPU port of the "
                             "reference kernels (oracle/)" % (args.cpu_steps, args.cpu_iters, args.cells,
                                                              args.cells)}
        except Exception as e:  # the baseline is reported, never required
            cpu = {"value": None, "unit": "cell-iterations/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": "failed: %s" % e}

    if rank == 0:
        out = {
            "metric": ("CG cell-iterations/s (FP64, %d^2)" % args.cells if args.precision == "fp64" else
                       "CG cell-iterations/s (FP32 steps with FP64 residual replacement, %d^2)" % args.cells),
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
            "config": dict(config_json(args, d), parallelism="replicas" if world > 1 else "single",
                           precision=args.precision),
            "roofline": roofline,
            "cpu_baseline": cpu,
            "mixed_vs_fp64": mixed_cmp,
            "e2e": e2e,
            "gpu_launches": launches,
            "clocks": clk.summary(),
            "wall_s_timed": wall,
        }
        print(json.dumps(out), flush=True)
    chunk.close()
    grp.close()


if __name__ == "__main__":
    main()
