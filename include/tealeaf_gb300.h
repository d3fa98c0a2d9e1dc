/*
 * tealeaf_gb300.h -- C ABI of the GB300 (sm_103a) TeaLeaf implicit-diffusion solver.
 *
 * Drop-in boundary: each entry point below replaces one per-tile kernel subroutine
 * that the reference's solver drivers (tea_leaf_*.f90) call under
 * IF (use_fortran_kernels); the citation on each line names that subroutine.  A
 * Fortran driver binds these with BIND(C), VALUE scalars and TYPE(C_PTR) for the
 * context.
 *
 * Conventions
 *  - One context (tl_ctx) owns one chunk of x_cells * y_cells cells resident in
 *    GPU memory, with the reference's index convention j = 1..x_cells (x fastest),
 *    k = 1..y_cells.  Host arrays are exchanged as dense column-major interiors
 *    with a caller-given leading dimension (>= x_cells).
 *  - Every function returns an int status: TL_OK (0) or a negative TL_ERR_* code;
 *    tl_last_error() returns a message for the last failure on the calling thread.
 *  - Reductions that the reference returns by reference (rro, pw, rrn, norm, error)
 *    are written to the caller's double* after the stream has synchronised.
 *  - A context is not thread-safe; all work runs on the context's CUDA stream.
 *  - Field arithmetic is FP64.  The 5-point operator is applied with face
 *    coefficients pre-scaled once per solve (rx*Kx, ry*Ky) and fused multiply-adds,
 *    so single-kernel results agree with the reference to rounding (a few ulp), not
 *    bit-for-bit; reductions use a fixed-order two-level sum, so results are
 *    reproducible run to run.
 */
#ifndef TEALEAF_GB300_H
#define TEALEAF_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define TL_OK 0
#define TL_ERR_ARG -1        /* invalid argument (null pointer, bad size, bad id) */
#define TL_ERR_CUDA -2       /* a CUDA runtime call failed */
#define TL_ERR_ALLOC -3      /* device allocation failed */
#define TL_ERR_BREAKDOWN -4  /* NaN/Inf in a solver scalar (pw, rro, rrn) */
#define TL_ERR_TIMEOUT -5    /* a bounded device-side wait expired */
#define TL_ERR_EIGEN -6      /* eigenvalue estimate failed (tea_solve.f90:192) */
#define TL_ERR_STATE -7      /* call made in an invalid state (e.g. solve before init) */

/* ---- constants shared with the reference (data.f90:57-66, 40-51) -------- */
#define TL_CONDUCTIVITY 1
#define TL_RECIP_CONDUCTIVITY 2
#define TL_PREC_NONE 1
#define TL_PREC_JAC_DIAG 2
#define TL_PREC_JAC_BLOCK 3

#define TL_SOLVER_JACOBI 1
#define TL_SOLVER_CG 2
#define TL_SOLVER_CHEBY 3
#define TL_SOLVER_PPCG 4

/* field ids (reference FIELD_* numbering where one exists) */
#define TL_FIELD_DENSITY 1
#define TL_FIELD_ENERGY0 2
#define TL_FIELD_ENERGY1 3
#define TL_FIELD_U 4
#define TL_FIELD_P 5
#define TL_FIELD_SD 6
#define TL_FIELD_R 7
#define TL_FIELD_Z 8
#define TL_FIELD_KX 9
#define TL_FIELD_KY 10
#define TL_FIELD_DI 11
#define TL_FIELD_U0 12
#define TL_FIELD_W 13
#define TL_FIELD_MI 14
#define TL_FIELD_UTEMP 15
#define TL_FIELD_RTEMP 16
#define TL_FIELD_R_STORE 17

typedef struct tl_ctx tl_ctx;

/* Options of one implicit solve: the deck keywords read in read_input.f90:194-263. */
typedef struct tl_solve_opts {
  int solver;            /* TL_SOLVER_* */
  int max_iters;         /* tl_max_iters */
  double eps;            /* tl_eps */
  int ch_cg_presteps;    /* tl_ch_cg_presteps */
  double ch_cg_epslim;   /* tl_ch_cg_epslim */
  int ppcg_inner_steps;  /* tl_ppcg_inner_steps (after the PPCG default) */
  int check_result;      /* tl_check_result */
  /* Precision form (no reference counterpart): TL_PRECISION_FP64 runs the reference's
   * algorithm in FP64.  TL_PRECISION_MIXED (CG, Chebyshev and PPCG, without a preconditioner
   * or with jac_diag):
   * CG runs on FP32 vectors and FP32 copies of the operator (and of Mi), with FP64 reductions
   * and step coefficients, the solution accumulated in FP64 and the residual periodically
   * replaced by the FP64 true residual u0 - A u (the search direction is kept across replacements);
   * PPCG runs its inner Chebyshev steps in FP32 inside the FP64 outer iteration; Chebyshev,
   * after its FP64 CG presteps, runs FP32 Chebyshev cycles on the correction inside FP64
   * iterative refinement. */
  int precision;
  double inner_tol;      /* mixed: replace the residual each time it has fallen by this
                            factor since the last replacement (0: 0.5) */
  int max_inner_iters;   /* mixed: cap on FP32 CG steps (0: max_iters) */
} tl_solve_opts;

#define TL_PRECISION_FP64 0
#define TL_PRECISION_MIXED 1

/* Outcome of one solve (the lines tea_solve.f90:435-456 prints, plus counters). */
typedef struct tl_solve_info {
  int n_exit;               /* loop index at exit: iterations performed, or max_iters+1 */
  int reported_iterations;  /* "Iteration count" = n_exit - 1 */
  int ppcg_inner_iters;     /* "PPCG Iteration count" */
  int cg_calc_steps;
  int cheby_calc_steps;
  int est_itc;
  double initial_residual;  /* sqrt(|r.r|) at solve start */
  double error;             /* final error variable (conduction error = error/initial_residual) */
  double exact_error;       /* sqrt(|b-Ax|^2) when check_result */
  double eigmin, eigmax;
  double solve_seconds;     /* device time of the whole call (CUDA events on its stream) */
  long long kernel_launches; /* kernels this call launched */
  int outer_iterations;     /* mixed: accepted residual replacements (0 for the FP64 form) */
  int stop_reason;          /* mixed: TL_STOP_* (0 for the FP64 form) */
  double true_residual;     /* mixed: final sqrt(|u0 - A u|^2) computed in FP64 */
  double residual_floor;    /* mixed: eps_64 * ||(|u0| + |Di u| + sum |c u_nb|)||_2 of the
                               final u, the rounding level of the FP64 residual */
} tl_solve_info;

/* Why the mixed-precision solve stopped (tl_solve_info.stop_reason). */
#define TL_STOP_EPS 1      /* true residual < tl_eps * initial residual (tea_solve.f90:410) */
#define TL_STOP_FLOOR 2    /* true residual within TL_FLOOR_FACTOR of residual_floor */
#define TL_STOP_STALL 3    /* three replacements in a row each lowered it by < 10% */
#define TL_STOP_REJECT 4   /* two corrections in a row did not lower it */
#define TL_STOP_CAP 5      /* max_inner_iters FP32 CG steps */
#define TL_FLOOR_FACTOR 16.0

/* Kernel ids for the per-kernel timers (tl_profile_read). */
#define TL_KERNEL_CG_MATVEC 0     /* fused p update + w = A p + p.w sweep of the CG loop */
#define TL_KERNEL_CG_UPDATE 1     /* fused u, r update + r.r sweep of the CG loop */
#define TL_KERNEL_CHEBY_ITERATE 2 /* Chebyshev iteration (tea_leaf_kernel_cheby_iterate), FP64 form */
#define TL_KERNEL_PPCG_INNER 3    /* one PPCG inner step (tea_leaf_kernel_ppcg_inner), FP64 form */
#define TL_KERNEL_JACOBI 4        /* Jacobi sweep with its L1 error (tea_leaf_jacobi_solve_kernel) */
#define TL_KERNEL_MIX_MATVEC 5    /* mixed CG: FP32 p update + w = A p + p.w sweep */
#define TL_KERNEL_MIX_UPDATE 6    /* mixed CG: FP32 r update + r.r sweep */
#define TL_KERNEL_POLY_STEP 7     /* mixed Chebyshev / PPCG: one FP32 polynomial step (the time of a
                                     block of steps, its set-up included, per step) */
#define TL_NUM_KERNEL_TIMERS 8

/* ---- context ----------------------------------------------------------- */

/* Allocate a chunk on the current CUDA device.  Replaces build_field.f90 allocation for
 * the solver fields; halo_depth is accepted (>= 1) for interface parity -- a single
 * chunk on one GPU needs only a one-cell halo.  dx, dy are the cell widths
 * (celldx(x_min), celldy(y_min)).  reflective: the reference's reflective_boundary. */
int tl_create(int x_cells, int y_cells, int halo_depth, int coefficient, int preconditioner,
              int reflective_boundary, double dx, double dy, tl_ctx** out);
int tl_destroy(tl_ctx* ctx);
const char* tl_last_error(void);
/* Make `device` the calling thread's current CUDA device for later tl_create calls (one
 * process per GPU; the reference's one-MPI-rank-per-chunk layout, tea.f90:43-76). */
int tl_set_device(int device);
/* Total device bytes the context holds: the field slab and scratch, plus the buffers made on
 * first use (FP32 fields of the precision form, adjoint checkpoints, transfer staging). */
int tl_device_bytes(const tl_ctx* ctx, unsigned long long* bytes);

/* Page-lock (register) an existing host array so that uploads/downloads run at full link
 * speed without staging -- e.g. the Fortran driver's density/energy1 arrays.  bytes > 0. */
int tl_host_register(void* host, unsigned long long bytes);
int tl_host_unregister(void* host);
/* Allocate / free page-locked host memory from the CUDA driver (cudaHostAlloc), for host
 * arrays that cross the boundary every time step.  On a Grace host (64 KB base pages), copies
 * from memory registered with tl_host_register stall a solve running at the same time
 * (measured: a 100-iteration 8192^2 CG solve took 317 ms instead of 135 ms under a concurrent
 * 1.6 GB upload), and copies made between solves run at a few GB/s; memory from
 * tl_host_alloc copies at ~200 GB/s and slows a concurrent solve by ~5%.  A Fortran driver
 * maps it with C_F_POINTER. */
int tl_host_alloc(unsigned long long bytes, void** host);
int tl_host_free(void* host);

/* Host <-> device copies of one field's interior (x_cells x y_cells, leading dimension ld).
 * The host array moves as one contiguous copy and is unpacked / packed on the device (the
 * first call allocates the staging fields); a download with ld > x_cells copies row by row so
 * that the host columns beyond x_cells are not written. */
int tl_upload_field(tl_ctx* ctx, int field, const double* host, int ld);
int tl_download_field(tl_ctx* ctx, int field, double* host, int ld);
/* Set density and energy1 from host arrays (the state after start.f90:113-123 for a chunk
 * generated on the host; reflective halos are primed).  Work fields are left as they are:
 * every solve initialises what it reads. */
int tl_upload_state(tl_ctx* ctx, const double* density, const double* energy1, int ld);

/* Pipelined transfers (no counterpart in the reference): host copies that overlap the solves.
 * tl_stage_state starts copying a (density, energy1) pair from page-locked host memory into one
 * of two device staging slots and returns at once; the host arrays must stay unchanged until
 * the pair has been taken and tl_wait_transfers has returned (or the next tl_take_staged of
 * that slot has run).  At most two pairs are staged (TL_ERR_STATE beyond).
 * tl_take_staged queues, ahead of the next solve, the move of the oldest staged pair into the
 * fields (the device waits for its copy; reflective halos are primed); TL_ERR_STATE if none.
 * tl_fetch_field snapshots a field after the work queued so far and copies the snapshot to
 * host memory on a separate stream, returning at once; the host array is valid after
 * tl_wait_transfers.  A typical step: take the staged pair, solve, fetch energy1, stage the
 * pair for the step after next -- the copies then run during the solves. */
int tl_stage_state(tl_ctx* ctx, const double* density, const double* energy1, int ld);
int tl_take_staged(tl_ctx* ctx);
int tl_fetch_field(tl_ctx* ctx, int field, double* host, int ld);
int tl_wait_transfers(tl_ctx* ctx);

/* ---- chunk generation and summary (generate_chunk, field_summary) -------- */

/* generate_chunk_kernel.f90:80-140 + set_field_kernel.f90:41-47 on the device.
 * States are given in deck order (index 0 = state 1, the background); the dx/100 extent
 * nudge of read_input.f90:352-359 is applied inside.  geometry: 1 rectangle, 2 circle,
 * 3 point.  xmin, ymin: domain origin. */
int tl_generate_chunk(tl_ctx* ctx, int nstates, const double* density, const double* energy,
                      const double* xmin, const double* xmax, const double* ymin, const double* ymax,
                      const double* radius, const int* geometry, double domain_xmin, double domain_ymin);
/* field_summary_kernel.f90:26-64: vol, mass, ie, temp (volume = dx*dy). */
int tl_field_summary(tl_ctx* ctx, double* vol, double* mass, double* ie, double* temp);

/* ---- per-kernel entry points (the drop-in boundary) --------------------- */

/* tea_leaf_common_init_kernel (kernels/tea_leaf_common_kernel.f90:26-177), driven as in
 * tea_leaf_common.f90:24-55: rx = dt/dx^2, ry = dt/dy^2, u = u0 = energy1*density, Kx, Ky,
 * zero-flux boundary faces, Di, preconditioner set-up, r = u - A u. */
int tl_common_init(tl_ctx* ctx, double dt);
/* tea_leaf_calc_residual_kernel (common_kernel.f90:208-244): r = u0 - A u. */
int tl_calc_residual(tl_ctx* ctx);
/* tea_leaf_calc_2norm_kernel (common_kernel.f90:246-274): norm_array 0 -> u0.u0, 1 -> r.r. */
int tl_calc_2norm(tl_ctx* ctx, int norm_array, double* norm);
/* tea_leaf_kernel_finalise (common_kernel.f90:179-206): energy1 = u/density. */
int tl_finalise(tl_ctx* ctx);
/* tea_leaf_kernel_finalise followed by field_summary_kernel (field_summary_kernel.f90:26-64),
 * in one sweep: energy1 = u/density, then vol, mass, ie, temp of the new state -- the same
 * values (bit for bit) as tl_finalise + tl_field_summary. */
int tl_finalise_field_summary(tl_ctx* ctx, double* vol, double* mass, double* ie, double* temp);
/* tea_leaf_cg_init_kernel (kernels/tea_leaf_cg_kernel.f90:31-112): p = r (or M^-1 r), rro = r.p. */
int tl_cg_init(tl_ctx* ctx, double* rro);
/* tea_leaf_cg_calc_w_kernel (cg_kernel.f90:114-156): w = A p, pw = p.w. */
int tl_cg_calc_w(tl_ctx* ctx, double* pw);
/* tea_leaf_cg_calc_ur_kernel (cg_kernel.f90:198-304): u += alpha p, r -= alpha w,
 * (z = M^-1 r), rrn = r.r or r.z. */
int tl_cg_calc_ur(tl_ctx* ctx, double alpha, double* rrn);
/* tea_leaf_cg_calc_p_kernel (cg_kernel.f90:306-347): p = r + beta p, or z + beta p when
 * preconditioned or ppcg_active (tl_ppcg_active). */
int tl_cg_calc_p(tl_ctx* ctx, double beta, int ppcg_active);
/* tea_leaf_kernel_cheby_init (kernels/tea_leaf_cheby_kernel.f90:30-109). */
int tl_cheby_init(tl_ctx* ctx, double theta);
/* tea_leaf_kernel_cheby_iterate (cheby_kernel.f90:111-200) with ch_alphas(step), ch_betas(step). */
int tl_cheby_iterate(tl_ctx* ctx, double ch_alpha, double ch_beta);
/* tea_leaf_kernel_ppcg_init_sd (kernels/tea_leaf_ppcg_kernel.f90:31-88). */
int tl_ppcg_init_sd(tl_ctx* ctx, double theta);
/* tea_leaf_ppcg_init_kernel (ppcg_kernel.f90:90-201), step 1, 2 or 3. */
int tl_ppcg_init(tl_ctx* ctx, int step, int ppcg_active, double* rro);
/* tea_leaf_kernel_ppcg_inner (ppcg_kernel.f90:204-310) on the chunk interior. */
int tl_ppcg_inner(tl_ctx* ctx, double ch_alpha, double ch_beta);
/* tea_leaf_ppcg_calc_zrnorm_kernel (ppcg_kernel.f90:411-451). */
int tl_ppcg_calc_zrnorm(tl_ctx* ctx, int ppcg_active, double* rrn);
/* tea_leaf_ppcg_update_z_kernel (ppcg_kernel.f90:453-477): z = utemp. */
int tl_ppcg_update_z(tl_ctx* ctx);
/* tea_leaf_ppcg_store_r_kernel (ppcg_kernel.f90:507-530): r_store = r. */
int tl_ppcg_store_r(tl_ctx* ctx);
/* tea_leaf_ppcg_calc_rrn_kernel (ppcg_kernel.f90:532-561): rrn = (r - r_store).z. */
int tl_ppcg_calc_rrn(tl_ctx* ctx, double* rrn);
/* tea_leaf_jacobi_solve_kernel (kernels/tea_leaf_jacobi_kernel.f90:26-77): error = sum|u-un|. */
int tl_jacobi_solve(tl_ctx* ctx, double* error);
/* update_halo (update_halo.f90:32-91) for one chunk: the reflective copy of the fields in
 * mask (bit f set for field id f, ids 1..11) when reflective_boundary; a no-op otherwise. */
int tl_update_halo(tl_ctx* ctx, int field_mask, int depth);

/* No counterpart in the reference.  tea_leaf_cg_calc_w_kernel (w = A p, pw = p.w) applied
 * to device arrays the caller owns, laid out exactly as the reference's fields
 * (1-h : x_cells+h, 1-h : y_cells+h, x fastest; Kx/Ky/Di as built by tea_leaf_common), for
 * callers that cannot allocate device memory -- they manage every device buffer themselves
 * (e.g. a Fortran driver keeping its fields on the GPU through OpenACC or CUDA Fortran), run
 * under a fixed memory budget, or must not call cudaMalloc/cudaFree inside their time loop.
 * Needs no tl_ctx and allocates nothing: the row sums of p.w use a fixed device array of
 * 16384 + 32 doubles inside the library, so y_cells must be <= 16384 (larger sizes are
 * rejected with TL_ERR_ARG).  Each call looks up the array's device address on the current
 * device; the first call on a device also loads the library's device code there, so make it
 * before any stream capture.  Runs on the legacy default stream and returns after pw is on
 * the host.  That stream does not wait for streams created with cudaStreamNonBlocking (e.g.
 * OpenACC async queues): finish the writes of p, Kx, Ky and Di there first.  Calls that
 * overlap on the GPU share the array and race. */
int tl_cg_calc_w_noalloc(int x_cells, int y_cells, int halo_depth, const double* p, double* w, const double* kx,
                         const double* ky, const double* di, double rx, double ry, double* pw);

/* ---- whole solve -------------------------------------------------------- */

/* tea_leaf() (tea_solve.f90:37-503) for one time step: initialisation, the CG /
 * Chebyshev / PPCG / Jacobi iteration with its switch rules, optional exact residual,
 * finalise.  Scalars stay on the device; the host reads a status word once per batch
 * of iterations.  Eigenvalue estimates persist in the context across calls, as the
 * reference's SAVE variables do. */
int tl_tea_leaf(tl_ctx* ctx, const tl_solve_opts* opts, double dt, tl_solve_info* info);
/* tl_tea_leaf for a time step after which the driver calls field_summary (diffuse.f90:58-61,
 * field_summary.f90:27-101): the solve's finalise sweep also forms the summary; summary[0..3] =
 * vol, mass, ie, temp, bit for bit those of tl_field_summary after tl_tea_leaf. */
int tl_tea_leaf_summary(tl_ctx* ctx, const tl_solve_opts* opts, double dt, tl_solve_info* info, double* summary);
/* Forget the saved eigenvalue estimates (the reference's 'first' flag becomes true). */
int tl_reset_eigen(tl_ctx* ctx);

/* Host math of the CG -> Chebyshev / PPCG switch, as tl_tea_leaf runs it (no device work, no
 * context).  tl_cg_eigenvalues: extreme eigenvalues of the Lanczos tridiagonal built from
 * cg_alphas(1..nsteps), cg_betas(1..nsteps) (tea_leaf_cheby.f90:142-176), by Sturm-sequence
 * bisection; unscaled (the solve then takes 0.95 eigmin, 1.05 eigmax); TL_ERR_EIGEN when the
 * estimate is negative or not finite (tea_solve.f90:192).  tl_cheby_coefficients: theta and
 * the Chebyshev coefficients ch_alphas(1..n), ch_betas(1..n) (tea_leaf_cheby.f90:178-205),
 * written to [0, n). */
int tl_cg_eigenvalues(const double* cg_alphas, const double* cg_betas, int nsteps, double* eigmin, double* eigmax);
int tl_cheby_coefficients(double eigmin, double eigmax, int n, double* ch_alphas, double* ch_betas, double* theta);

/* ---- adjoint (no counterpart in the reference) --------------------------- */

/* Reverse mode of a run of tea_leaf() time steps: gradients of a loss on the final u (and/or
 * energy1) with respect to the density field and the initial energy1.  One step is
 * b = energy1*density, A(density) u = b (A from Kx, Ky of tea_leaf_common_kernel.f90:75-152),
 * energy1' = u/density (finalise).  The reverse step solves A lambda = u_bar with the FP64 CG
 * solve (A is symmetric) and chains dA/dKx, dA/dKy through the face formula to density.
 * The exact-solve gradient: the recorded solves are taken as converged.
 *
 * tl_adjoint_begin allocates a tape for up to max_steps steps: each step's input energy1
 * (and its solution u when store_solutions = 1; otherwise the reverse sweep recomputes u
 * from the input energy1 with the recorded options).  Calling it again clears the tape. */
int tl_adjoint_begin(tl_ctx* ctx, int max_steps, int store_solutions);
/* tl_tea_leaf on the current fields, recording the step on the tape (TL_ERR_STATE if no tape
 * or the tape is full). */
int tl_adjoint_record_step(tl_ctx* ctx, const tl_solve_opts* opts, double dt, tl_solve_info* info);
/* Reverse sweep over the recorded steps.  u_bar: dL/du of the last step's solution, e_bar:
 * dL/d energy1 after the last step (host arrays, x_cells x y_cells, row stride ld; either may be
 * NULL for zero).  density_bar (required) and energy0_bar (NULL to skip) receive dL/d density
 * and dL/d energy1 at the first recorded step's input.  info sums the reverse solves
 * (reported_iterations, solve_seconds, kernel_launches).  The chunk's fields are left
 * overwritten; the tape is kept (call again with another u_bar). */
int tl_adjoint_backward(tl_ctx* ctx, const double* u_bar, const double* e_bar, int ld, double* density_bar,
                        double* energy0_bar, tl_solve_info* info);
/* Free the tape. */
int tl_adjoint_end(tl_ctx* ctx);

/* ---- profiling (the reference's profiler_on timers, definitions.f90:107-121) ---- */

/* Enable (1) or disable (0) CUDA-event timing of every launch of the solver-loop kernels
 * (TL_KERNEL_*) on the context's stream; enabling also clears the accumulated totals.  The
 * host-driven loops (Chebyshev, PPCG, Jacobi) wait for each timed launch, which adds launch
 * gaps to the solve time while timing is on. */
int tl_profile(tl_ctx* ctx, int enable);
/* Accumulated device time (ms) and launch count of one TL_KERNEL_* since tl_profile(ctx,1). */
int tl_profile_read(tl_ctx* ctx, int kernel_id, double* total_ms, long long* launches);

#ifdef __cplusplus
}
#endif
#endif
