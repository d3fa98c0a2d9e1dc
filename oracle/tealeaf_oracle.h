/*
 * tealeaf_oracle.h -- CPU oracle for the TeaLeaf implicit-diffusion solve.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C, serial, FP64 restatement of the
 * reference's solver kernels (kernels/tea_leaf_*_kernel.f90), drivers
 * (tea_leaf_*.f90) and control flow (tea_solve.f90), plus the setup and summary
 * steps needed to run the reference's own benchmark decks (initialise_chunk,
 * generate_chunk, set_field, field_summary).  It is used by the tests, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker; the
 * product path (tealeaf_ref_gb300) never links or calls it.
 *
 * Parity pin: the serial build reproduces the reference's Benchmarks/tea_bm_{1..4}.out
 * step-10 field summaries and per-step CG iteration counts (see tests/test_oracle_golden.py).
 *
 * Layout follows the reference: every 2-D field is (x_min-h : x_max+h, y_min-h : y_max+h),
 * column-major with x fastest, x_min = y_min = 1, h = halo depth.
 */
#ifndef TEALEAF_ORACLE_H
#define TEALEAF_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* data.f90:57-66 */
#define TLO_CONDUCTIVITY 1
#define TLO_RECIP_CONDUCTIVITY 2
#define TLO_PREC_NONE 1
#define TLO_PREC_JAC_DIAG 2
#define TLO_PREC_JAC_BLOCK 3

/* data.f90:40-51 (field ids used by update_halo masks) */
enum {
  TLO_F_DENSITY = 1, TLO_F_ENERGY0 = 2, TLO_F_ENERGY1 = 3, TLO_F_U = 4, TLO_F_P = 5,
  TLO_F_SD = 6, TLO_F_R = 7, TLO_F_Z = 8, TLO_F_KX = 9, TLO_F_KY = 10, TLO_F_DI = 11,
  TLO_NUM_FIELDS = 11
};

/* Extra ids for field access (arrays not addressable through update_halo). */
enum {
  TLO_A_DENSITY = 0, TLO_A_ENERGY0, TLO_A_ENERGY1, TLO_A_U, TLO_A_U0, TLO_A_R, TLO_A_R_STORE,
  TLO_A_MI, TLO_A_W, TLO_A_Z, TLO_A_UTEMP, TLO_A_RTEMP, TLO_A_DI, TLO_A_KX, TLO_A_KY,
  TLO_A_P, TLO_A_SD, TLO_A_CP, TLO_A_BFP, TLO_NUM_ARRAYS
};

/* solvers (read_input.f90:225-244) */
enum { TLO_SOLVER_JACOBI = 1, TLO_SOLVER_CG = 2, TLO_SOLVER_CHEBY = 3, TLO_SOLVER_PPCG = 4 };

typedef struct tlo_chunk tlo_chunk;

typedef struct tlo_opts {
  int solver;            /* TLO_SOLVER_* */
  int max_iters;         /* tl_max_iters */
  double eps;            /* tl_eps */
  int ch_cg_presteps;    /* tl_ch_cg_presteps */
  double ch_cg_epslim;   /* tl_ch_cg_epslim */
  int ppcg_inner_steps;  /* tl_ppcg_inner_steps (already defaulted) */
  int check_result;      /* tl_check_result */
} tlo_opts;

/* Values the reference keeps in SAVE variables across calls of tea_leaf()
 * (tea_solve.f90:55,58). */
typedef struct tlo_persist {
  int first;
  double eigmin, eigmax, theta, cn;
} tlo_persist;

typedef struct tlo_solve_info {
  int n_exit;               /* value of n after the DO loop (iterations performed, or max_iters+1) */
  int reported_iterations;  /* "Iteration count" line: n-1 */
  int ppcg_inner_iters;
  int cg_calc_steps, cheby_calc_steps, est_itc;
  double initial_residual;  /* sqrt(|r.r|) at solve start */
  double error;             /* final error variable */
  double exact_error;       /* sqrt(|b-Ax|^2) when check_result */
  double eigmin, eigmax;
  int status;               /* 0 ok, 1 eigenvalue failure */
} tlo_solve_info;

tlo_chunk* tlo_create(int x_cells, int y_cells, int halo_depth, double xmin, double ymin,
                      double xmax, double ymax, int coefficient, int precond, int reflective);
void tlo_destroy(tlo_chunk* c);
/* Pointer to a field's storage and its dimensions (with halo: (nx+2h) x (ny+2h);
 * cp/bfp: nx x ny). */
double* tlo_array(tlo_chunk* c, int array_id, int* dim_x, int* dim_y);
void tlo_geometry(const tlo_chunk* c, double* dx, double* dy, double* rx, double* ry);

/* States 1..n (index 0 = state 1, the background).  Extents are the deck's values;
 * the dx/100 nudge of read_input.f90:352-359 is applied here. geometry: 1 rect, 2 circle, 3 point. */
void tlo_generate(tlo_chunk* c, int nstates, const double* density, const double* energy,
                  const double* xmin, const double* xmax, const double* ymin, const double* ymax,
                  const double* radius, const int* geometry);
/* start.f90:113-123: prime halos (reflective only) and energy1 = energy0. */
void tlo_start_fields(tlo_chunk* c);
/* field_summary_kernel.f90:26-64 -> out[0..3] = vol, mass, ie, temp */
void tlo_field_summary(tlo_chunk* c, double* out);

/* tea_solve.f90:37-503 */
int tlo_tea_leaf(tlo_chunk* c, const tlo_opts* o, tlo_persist* ps, double dt, tlo_solve_info* info);

/* Single kernels (one call of the reference's per-tile kernel on the single tile). */
void tlo_common_init(tlo_chunk* c, double dt);
void tlo_calc_residual(tlo_chunk* c);
double tlo_calc_2norm(tlo_chunk* c, int norm_array);
void tlo_finalise(tlo_chunk* c);
double tlo_cg_init(tlo_chunk* c);
double tlo_cg_calc_w(tlo_chunk* c);
double tlo_cg_calc_ur(tlo_chunk* c, double alpha);
void tlo_cg_calc_p(tlo_chunk* c, double beta, int ppcg_active);
void tlo_cheby_init(tlo_chunk* c, double theta);
void tlo_cheby_iterate(tlo_chunk* c, double ch_alpha, double ch_beta);
void tlo_ppcg_init_sd(tlo_chunk* c, double theta);
double tlo_ppcg_init(tlo_chunk* c, int step, int ppcg_active);
void tlo_ppcg_inner(tlo_chunk* c, double ch_alpha, double ch_beta);
double tlo_ppcg_calc_zrnorm(tlo_chunk* c, int ppcg_active);
void tlo_ppcg_update_z(tlo_chunk* c);
void tlo_ppcg_store_r(tlo_chunk* c);
double tlo_ppcg_calc_rrn(tlo_chunk* c);
double tlo_jacobi_solve(tlo_chunk* c);
/* fields[1..11] mask as in the reference (index 0 unused) */
void tlo_update_halo(tlo_chunk* c, const int* fields, int depth);

/* Host scalar math (tea_leaf_cheby.f90:142-205).  Returns 0 on success. */
int tlo_calc_eigenvalues(const double* cg_alphas, const double* cg_betas, int nsteps,
                         double* eigmin, double* eigmax);
void tlo_calc_ch_coefs(double* ch_alphas, double* ch_betas, double eigmin, double eigmax,
                       double* theta, int n);
/* All eigenvalues of the symmetric tridiagonal (d[0..n-1], off[0..n-2]) in ascending order. */
void tlo_tridiag_eigenvalues(const double* d, const double* off, int n, double* out);

#ifdef __cplusplus
}
#endif
#endif
