/*
 * tealeaf_oracle.c -- CPU oracle for the TeaLeaf implicit-diffusion solve.
 *
 * TEST INFRASTRUCTURE ONLY (see tealeaf_oracle.h).  Serial FP64 restatement of the
 * reference's solver path.  Loop order (k outer, j inner) and the operation order
 * inside each expression follow the reference, and the file is compiled with
 * -ffp-contract=off, so that the serial build reproduces the reference's IEEE
 * (no-FMA, no-reassociation) benchmark outputs.  The OpenMP pragmas only take effect
 * in the separately-built variants: the timing variant (liboracle_omp.so, compiled as the
 * reference compiles its kernels: -O3 -funroll-loops with FMA contraction), whose results
 * are therefore not bit-identical to the serial build, and the parallel checker
 * (liboracle_par.so, -ffp-contract=off), whose per-cell arithmetic is the serial build's
 * and whose global sums add per-thread partials.
 *
 * Citations are file:line in the reference (UK-MAC/TeaLeaf_ref).
 */
#include "tealeaf_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

struct tlo_chunk {
  int nx, ny, h, ldx;
  int coefficient, precond, reflective;
  double xmin, ymin, dx, dy;
  double rx, ry;
  double* a[TLO_NUM_ARRAYS];
  /* mesh coordinates, initialise_chunk_kernel.f90:44-51, stored from index 1-h-2 so that
   * every halo cell has a coordinate; element i is at [i + voff] */
  int voff;
  double *vertexx, *vertexy, *cellx, *celly;
};

/* (j,k) -> offset in an (x_min-h:x_max+h, y_min-h:y_max+h) array */
#define IX(j, k) ((size_t)((k) + c->h - 1) * (size_t)c->ldx + (size_t)((j) + c->h - 1))
/* (j,k) -> offset in an (x_min:x_max, y_min:y_max) array (tri_cp, tri_bfp) */
#define IXI(j, k) ((size_t)((k)-1) * (size_t)c->nx + (size_t)((j)-1))

#define DENSITY c->a[TLO_A_DENSITY]
#define ENERGY0 c->a[TLO_A_ENERGY0]
#define ENERGY1 c->a[TLO_A_ENERGY1]
#define U c->a[TLO_A_U]
#define U0 c->a[TLO_A_U0]
#define R c->a[TLO_A_R]
#define R_STORE c->a[TLO_A_R_STORE]
#define MI c->a[TLO_A_MI]
#define W c->a[TLO_A_W]
#define Z c->a[TLO_A_Z]
#define UTEMP c->a[TLO_A_UTEMP]
#define RTEMP c->a[TLO_A_RTEMP]
#define DI c->a[TLO_A_DI]
#define KX c->a[TLO_A_KX]
#define KY c->a[TLO_A_KY]
#define P c->a[TLO_A_P]
#define SD c->a[TLO_A_SD]
#define CP c->a[TLO_A_CP]
#define BFP c->a[TLO_A_BFP]

/* ------------------------------------------------------------------------- */
/* chunk set-up: build_field.f90 (allocate + zero), initialise_chunk.f90:34-35, */
/* initialise_chunk_kernel.f90:58-130                                          */
/* ------------------------------------------------------------------------- */

tlo_chunk* tlo_create(int x_cells, int y_cells, int halo_depth, double gxmin, double gymin,
                      double gxmax, double gymax, int coefficient, int precond, int reflective) {
  if (x_cells < 1 || y_cells < 1 || halo_depth < 1) return NULL;
  tlo_chunk* c = (tlo_chunk*)calloc(1, sizeof(tlo_chunk));
  c->nx = x_cells;
  c->ny = y_cells;
  c->h = halo_depth;
  c->ldx = x_cells + 2 * halo_depth;
  c->coefficient = coefficient;
  c->precond = precond;
  c->reflective = reflective;
  c->xmin = gxmin;
  c->ymin = gymin;
  /* initialise_chunk.f90:34-35: REAL() of the cell count is exact for these sizes */
  c->dx = (gxmax - gxmin) / (double)(float)x_cells;
  c->dy = (gymax - gymin) / (double)(float)y_cells;
  size_t n = (size_t)c->ldx * (size_t)(y_cells + 2 * halo_depth);
  for (int i = 0; i < TLO_NUM_ARRAYS; ++i) {
    size_t sz = (i == TLO_A_CP || i == TLO_A_BFP) ? (size_t)x_cells * (size_t)y_cells : n;
    c->a[i] = (double*)calloc(sz, sizeof(double));
  }
  const int h = halo_depth, voff = h + 2;
  c->voff = voff;
  c->vertexx = (double*)calloc((size_t)x_cells + 2 * (size_t)voff + 2, sizeof(double));
  c->vertexy = (double*)calloc((size_t)y_cells + 2 * (size_t)voff + 2, sizeof(double));
  c->cellx = (double*)calloc((size_t)x_cells + 2 * (size_t)voff + 2, sizeof(double));
  c->celly = (double*)calloc((size_t)y_cells + 2 * (size_t)voff + 2, sizeof(double));
  /* vertexx(j) = xmin + dx*float(j-x_min) */
  for (int j = 1 - voff; j <= x_cells + voff + 1; ++j) c->vertexx[j + voff] = gxmin + c->dx * (double)(float)(j - 1);
  for (int k = 1 - voff; k <= y_cells + voff + 1; ++k) c->vertexy[k + voff] = gymin + c->dy * (double)(float)(k - 1);
  /* cellx(j) = 0.5*(vertexx(j)+vertexx(j+1)) */
  for (int j = 1 - voff; j <= x_cells + voff; ++j) c->cellx[j + voff] = 0.5 * (c->vertexx[j + voff] + c->vertexx[j + voff + 1]);
  for (int k = 1 - voff; k <= y_cells + voff; ++k) c->celly[k + voff] = 0.5 * (c->vertexy[k + voff] + c->vertexy[k + voff + 1]);
  return c;
}

void tlo_destroy(tlo_chunk* c) {
  if (!c) return;
  for (int i = 0; i < TLO_NUM_ARRAYS; ++i) free(c->a[i]);
  free(c->vertexx);
  free(c->vertexy);
  free(c->cellx);
  free(c->celly);
  free(c);
}

double* tlo_array(tlo_chunk* c, int id, int* dim_x, int* dim_y) {
  if (id < 0 || id >= TLO_NUM_ARRAYS) return NULL;
  if (id == TLO_A_CP || id == TLO_A_BFP) {
    *dim_x = c->nx;
    *dim_y = c->ny;
  } else {
    *dim_x = c->ldx;
    *dim_y = c->ny + 2 * c->h;
  }
  return c->a[id];
}

void tlo_geometry(const tlo_chunk* c, double* dx, double* dy, double* rx, double* ry) {
  *dx = c->dx;
  *dy = c->dy;
  *rx = c->rx;
  *ry = c->ry;
}

/* generate_chunk_kernel.f90:80-140 with the state nudge of read_input.f90:352-359 */
void tlo_generate(tlo_chunk* c, int nstates, const double* sden, const double* sen,
                  const double* sxmin_in, const double* sxmax_in, const double* symin_in,
                  const double* symax_in, const double* srad, const int* sgeom) {
  const int h = c->h, nx = c->nx, ny = c->ny, vo = c->voff;
  for (int k = 1 - h; k <= ny + h; ++k)
    for (int j = 1 - h; j <= nx + h; ++j) ENERGY0[IX(j, k)] = sen[0];
  for (int k = 1 - h; k <= ny + h; ++k)
    for (int j = 1 - h; j <= nx + h; ++j) DENSITY[IX(j, k)] = sden[0];
  for (int s = 1; s < nstates; ++s) {
    const double sxmin = sxmin_in[s] + c->dx / 100.0, symin = symin_in[s] + c->dy / 100.0;
    const double sxmax = sxmax_in[s] - c->dx / 100.0, symax = symax_in[s] - c->dy / 100.0;
    const double x_cent = sxmin, y_cent = symin;
    for (int k = 1 - h; k <= ny + h; ++k) {
      for (int j = 1 - h; j <= nx + h; ++j) {
        if (sgeom[s] == 1) {
          if (j >= 1 && j <= nx && k >= 1 && k <= ny) {
            if (c->vertexx[j + 1 + vo] >= sxmin && c->vertexx[j + vo] < sxmax) {
              if (c->vertexy[k + 1 + vo] >= symin && c->vertexy[k + vo] < symax) {
                ENERGY0[IX(j, k)] = sen[s];
                DENSITY[IX(j, k)] = sden[s];
              }
            }
          }
        } else if (sgeom[s] == 2) {
          const double ddx = c->cellx[j + vo] - x_cent, ddy = c->celly[k + vo] - y_cent;
          const double radius = sqrt(ddx * ddx + ddy * ddy);
          if (radius <= srad[s]) {
            ENERGY0[IX(j, k)] = sen[s];
            DENSITY[IX(j, k)] = sden[s];
          }
        } else if (sgeom[s] == 3) {
          if (c->vertexx[j + vo] == x_cent && c->vertexy[k + vo] == y_cent) {
            ENERGY0[IX(j, k)] = sen[s];
            DENSITY[IX(j, k)] = sden[s];
          }
        }
      }
    }
  }
  /* generate_chunk.f90 passes field%u as the "u0" argument: u = energy0*density */
  for (int k = 1 - h; k <= ny + h; ++k)
    for (int j = 1 - h; j <= nx + h; ++j) U[IX(j, k)] = ENERGY0[IX(j, k)] * DENSITY[IX(j, k)];
}

void tlo_start_fields(tlo_chunk* c) {
  int fields[TLO_NUM_FIELDS + 1] = {0};
  fields[TLO_F_DENSITY] = 1;
  fields[TLO_F_ENERGY0] = 1;
  fields[TLO_F_ENERGY1] = 1;
  tlo_update_halo(c, fields, c->h); /* start.f90:113-118 */
  for (int k = 1; k <= c->ny; ++k)  /* set_field_kernel.f90:41-47 */
    for (int j = 1; j <= c->nx; ++j) ENERGY1[IX(j, k)] = ENERGY0[IX(j, k)];
}

/* field_summary_kernel.f90:44-62 (volume = dx*dy, initialise_chunk_kernel.f90:107-113) */
void tlo_field_summary(tlo_chunk* c, double* out) {
  double vol = 0.0, mass = 0.0, ie = 0.0, temp = 0.0;
  const double cell_vol = c->dx * c->dy;
  for (int k = 1; k <= c->ny; ++k) {
    for (int j = 1; j <= c->nx; ++j) {
      const double cell_mass = cell_vol * DENSITY[IX(j, k)];
      vol = vol + cell_vol;
      mass = mass + cell_mass;
      ie = ie + cell_mass * ENERGY1[IX(j, k)];
      temp = temp + cell_mass * U[IX(j, k)];
    }
  }
  out[0] = vol;
  out[1] = mass;
  out[2] = ie;
  out[3] = temp;
}

/* ------------------------------------------------------------------------- */
/* reflective boundary: update_halo.f90:49-91, update_halo_kernel.f90:136-195 */
/* ------------------------------------------------------------------------- */

static void halo_cell(tlo_chunk* c, double* m, int depth) {
  const int nx = c->nx, ny = c->ny;
  for (int k = 1 - depth; k <= ny + depth; ++k)
    for (int j = 1; j <= depth; ++j) m[IX(1 - j, k)] = m[IX(0 + j, k)];
  for (int k = 1 - depth; k <= ny + depth; ++k)
    for (int j = 1; j <= depth; ++j) m[IX(nx + j, k)] = m[IX(nx + 1 - j, k)];
  for (int k = 1; k <= depth; ++k)
    for (int j = 1 - depth; j <= nx + depth; ++j) m[IX(j, 1 - k)] = m[IX(j, 0 + k)];
  for (int k = 1; k <= depth; ++k)
    for (int j = 1 - depth; j <= nx + depth; ++j) m[IX(j, ny + k)] = m[IX(j, ny + 1 - k)];
}

void tlo_update_halo(tlo_chunk* c, const int* fields, int depth) {
  /* A single chunk with a single tile has no MPI exchange and no tile-tile copies;
   * only the external reflective update runs, and only if reflective_boundary. */
  if (!c->reflective) return;
  /* field -> array binding of update_halo.f90:64-80 (FIELD_R is vector_rtemp) */
  static const int arr[TLO_NUM_FIELDS + 1] = {-1, TLO_A_DENSITY, TLO_A_ENERGY0, TLO_A_ENERGY1, TLO_A_U,
                                               TLO_A_P, TLO_A_SD, TLO_A_RTEMP, TLO_A_Z, TLO_A_KX,
                                               TLO_A_KY, TLO_A_DI};
  for (int f = 1; f <= TLO_NUM_FIELDS; ++f)
    if (fields[f] == 1) halo_cell(c, c->a[arr[f]], depth);
}

/* ------------------------------------------------------------------------- */
/* preconditioners: tea_leaf_common_kernel.f90:276-468                        */
/* ------------------------------------------------------------------------- */

static void diag_init(tlo_chunk* c) { /* :276-307 */
  const int h = c->h;
  for (int k = 2 - h; k <= c->ny + h - 1; ++k)
    for (int j = 2 - h; j <= c->nx + h - 1; ++j) MI[IX(j, k)] = (DI[IX(j, k)] != 0.0) ? 1.0 / DI[IX(j, k)] : 0.0;
}

static void diag_solve(tlo_chunk* c, const double* r, double* z) { /* :309-335, depth 0 */
  for (int k = 1; k <= c->ny; ++k)
    for (int j = 1; j <= c->nx; ++j) z[IX(j, k)] = MI[IX(j, k)] * r[IX(j, k)];
}

static void block_init(tlo_chunk* c) { /* :337-376, jac_block_size = 4 */
  const double ry = c->ry;
  for (int ko = 1; ko <= c->ny; ko += 4) {
    const int bottom = ko, top = (ko + 3 < c->ny) ? ko + 3 : c->ny;
    for (int j = 1; j <= c->nx; ++j) {
      int k = bottom;
      CP[IXI(j, k)] = (-KY[IX(j, k + 1)] * ry) / DI[IX(j, k)];
      for (k = bottom + 1; k <= top; ++k) {
        BFP[IXI(j, k)] = 1.0 / (DI[IX(j, k)] - (-KY[IX(j, k)] * ry) * CP[IXI(j, k - 1)]);
        CP[IXI(j, k)] = (-KY[IX(j, k + 1)] * ry) * BFP[IXI(j, k)];
      }
    }
  }
}

static void block_solve_rows(tlo_chunk* c, const double* r, double* z, int bottom, int top) {
  const double ry = c->ry;
  double dp_l[4], z_l[4];
  for (int j = 1; j <= c->nx; ++j) {
    int k = bottom;
    dp_l[0] = r[IX(j, k)] / DI[IX(j, k)];
    for (k = bottom + 1; k <= top; ++k)
      dp_l[k - bottom] = (r[IX(j, k)] - (-KY[IX(j, k)] * ry) * dp_l[k - bottom - 1]) * BFP[IXI(j, k)];
    k = top;
    z_l[k - bottom] = dp_l[k - bottom];
    for (k = top - 1; k >= bottom; --k) z_l[k - bottom] = dp_l[k - bottom] - CP[IXI(j, k)] * z_l[k - bottom + 1];
    for (k = bottom; k <= top; ++k) z[IX(j, k)] = z_l[k - bottom];
  }
}

static void block_solve(tlo_chunk* c, const double* r, double* z) { /* :378-468 */
  const int ny = c->ny;
  const int k_extra = ny - ny % 4;
  for (int ko = 1; ko <= k_extra; ko += 4) block_solve_rows(c, r, z, ko, ko + 3);
  for (int ki = k_extra + 1; ki <= ny; ki += 4) {
    const int bottom = ki < ny ? ki : ny, top = (ki + 3 < ny) ? ki + 3 : ny;
    block_solve_rows(c, r, z, bottom, top);
  }
}

static void precond_apply(tlo_chunk* c, const double* r, double* z) {
  if (c->precond == TLO_PREC_JAC_BLOCK)
    block_solve(c, r, z);
  else if (c->precond == TLO_PREC_JAC_DIAG)
    diag_solve(c, r, z);
}

/* ------------------------------------------------------------------------- */
/* tea_leaf_common                                                            */
/* ------------------------------------------------------------------------- */

/* tea_leaf_common.f90:24-55 + tea_leaf_common_kernel.f90:26-177 */
void tlo_common_init(tlo_chunk* c, double dt) {
  const int h = c->h, nx = c->nx, ny = c->ny;
  c->rx = dt / (c->dx * c->dx);
  c->ry = dt / (c->dy * c->dy);
  const double rx = c->rx, ry = c->ry;
#pragma omp parallel for
  for (int k = 1; k <= ny; ++k)
    for (int j = 1; j <= nx; ++j) {
      U[IX(j, k)] = ENERGY1[IX(j, k)] * DENSITY[IX(j, k)];
      U0[IX(j, k)] = ENERGY1[IX(j, k)] * DENSITY[IX(j, k)];
    }
#pragma omp parallel for
  for (int k = 1 - h; k <= ny + h; ++k)
    for (int j = 1 - h; j <= nx + h; ++j)
      W[IX(j, k)] = (c->coefficient == TLO_RECIP_CONDUCTIVITY) ? 1.0 / DENSITY[IX(j, k)] : DENSITY[IX(j, k)];
#pragma omp parallel for
  for (int k = 2 - h; k <= ny + h; ++k)
    for (int j = 2 - h; j <= nx + h; ++j) {
      KX[IX(j, k)] = (W[IX(j - 1, k)] + W[IX(j, k)]) / (2.0 * W[IX(j - 1, k)] * W[IX(j, k)]);
      KY[IX(j, k)] = (W[IX(j, k - 1)] + W[IX(j, k)]) / (2.0 * W[IX(j, k - 1)] * W[IX(j, k)]);
    }
  if (!c->reflective) { /* every face of the single tile is external: zero_boundary all true */
    for (int k = 1 - h; k <= ny + h; ++k)
      for (int j = 1 - h; j <= 1; ++j) KX[IX(j, k)] = 0.0;
    for (int k = 1 - h; k <= ny + h; ++k)
      for (int j = nx + 1; j <= nx + h; ++j) KX[IX(j, k)] = 0.0;
    for (int k = 1 - h; k <= 1; ++k)
      for (int j = 1 - h; j <= nx + h; ++j) KY[IX(j, k)] = 0.0;
    for (int k = ny + 1; k <= ny + h; ++k)
      for (int j = 1 - h; j <= nx + h; ++j) KY[IX(j, k)] = 0.0;
  }
#pragma omp parallel for
  for (int k = 2 - h; k <= ny + h - 1; ++k)
    for (int j = 2 - h; j <= nx + h - 1; ++j)
      DI[IX(j, k)] = (1.0 + ry * (KY[IX(j, k + 1)] + KY[IX(j, k)])) + rx * (KX[IX(j + 1, k)] + KX[IX(j, k)]);
  if (c->precond == TLO_PREC_JAC_BLOCK)
    block_init(c);
  else if (c->precond == TLO_PREC_JAC_DIAG)
    diag_init(c);
#pragma omp parallel for
  for (int k = 1; k <= ny; ++k)
    for (int j = 1; j <= nx; ++j) {
      W[IX(j, k)] = (DI[IX(j, k)] * U[IX(j, k)] - ry * (KY[IX(j, k + 1)] * U[IX(j, k + 1)] + KY[IX(j, k)] * U[IX(j, k - 1)])) -
                    rx * (KX[IX(j + 1, k)] * U[IX(j + 1, k)] + KX[IX(j, k)] * U[IX(j - 1, k)]);
      R[IX(j, k)] = U[IX(j, k)] - W[IX(j, k)];
    }
}

/* 5-point operator, tea_leaf_common_kernel.f90:235-237 and cg_kernel.f90:145-147 */
static inline double smvp(const tlo_chunk* c, const double* v, int j, int k) {
  return (c->a[TLO_A_DI][IX(j, k)] * v[IX(j, k)] -
          c->ry * (c->a[TLO_A_KY][IX(j, k + 1)] * v[IX(j, k + 1)] + c->a[TLO_A_KY][IX(j, k)] * v[IX(j, k - 1)])) -
         c->rx * (c->a[TLO_A_KX][IX(j + 1, k)] * v[IX(j + 1, k)] + c->a[TLO_A_KX][IX(j, k)] * v[IX(j - 1, k)]);
}

void tlo_calc_residual(tlo_chunk* c) { /* common_kernel.f90:208-244 */
#pragma omp parallel for
  for (int k = 1; k <= c->ny; ++k)
    for (int j = 1; j <= c->nx; ++j) R[IX(j, k)] = U0[IX(j, k)] - smvp(c, U, j, k);
}

double tlo_calc_2norm(tlo_chunk* c, int norm_array) { /* common_kernel.f90:246-274 */
  const double* arr = (norm_array == 0) ? U0 : R;
  double norm = 0.0;
#pragma omp parallel for reduction(+ : norm)
  for (int k = 1; k <= c->ny; ++k)
    for (int j = 1; j <= c->nx; ++j) norm = norm + arr[IX(j, k)] * arr[IX(j, k)];
  return norm;
}

void tlo_finalise(tlo_chunk* c) { /* common_kernel.f90:179-206 */
#pragma omp parallel for
  for (int k = 1; k <= c->ny; ++k)
    for (int j = 1; j <= c->nx; ++j) ENERGY1[IX(j, k)] = U[IX(j, k)] / DENSITY[IX(j, k)];
}

/* ------------------------------------------------------------------------- */
/* tea_leaf_cg: kernels/tea_leaf_cg_kernel.f90                                */
/* ------------------------------------------------------------------------- */

double tlo_cg_init(tlo_chunk* c) { /* :31-112 */
  double rro = 0.0;
#pragma omp parallel for
  for (int k = 1; k <= c->ny; ++k)
    for (int j = 1; j <= c->nx; ++j) {
      P[IX(j, k)] = 0.0;
      Z[IX(j, k)] = 0.0;
    }
  if (c->precond != TLO_PREC_NONE) {
    precond_apply(c, R, Z);
    for (int k = 1; k <= c->ny; ++k)
      for (int j = 1; j <= c->nx; ++j) P[IX(j, k)] = Z[IX(j, k)];
  } else {
#pragma omp parallel for
    for (int k = 1; k <= c->ny; ++k)
      for (int j = 1; j <= c->nx; ++j) P[IX(j, k)] = R[IX(j, k)];
  }
#pragma omp parallel for reduction(+ : rro)
  for (int k = 1; k <= c->ny; ++k)
    for (int j = 1; j <= c->nx; ++j) rro = rro + R[IX(j, k)] * P[IX(j, k)];
  return rro;
}

double tlo_cg_calc_w(tlo_chunk* c) { /* :114-156 */
  double pw = 0.0;
#pragma omp parallel for reduction(+ : pw)
  for (int k = 1; k <= c->ny; ++k) {
    for (int j = 1; j <= c->nx; ++j) W[IX(j, k)] = smvp(c, P, j, k);
    for (int j = 1; j <= c->nx; ++j) pw = pw + W[IX(j, k)] * P[IX(j, k)];
  }
  return pw;
}

double tlo_cg_calc_ur(tlo_chunk* c, double alpha) { /* :198-304 */
  double rrn = 0.0;
  const int nx = c->nx, ny = c->ny;
  if (c->precond == TLO_PREC_JAC_DIAG) {
    for (int k = 1; k <= ny; ++k)
      for (int j = 1; j <= nx; ++j) U[IX(j, k)] = U[IX(j, k)] + alpha * P[IX(j, k)];
    for (int k = 1; k <= ny; ++k)
      for (int j = 1; j <= nx; ++j) {
        R[IX(j, k)] = R[IX(j, k)] - alpha * W[IX(j, k)];
        Z[IX(j, k)] = MI[IX(j, k)] * R[IX(j, k)];
        rrn = rrn + R[IX(j, k)] * Z[IX(j, k)];
      }
  } else if (c->precond == TLO_PREC_JAC_BLOCK) {
    for (int k = 1; k <= ny; ++k)
      for (int j = 1; j <= nx; ++j) U[IX(j, k)] = U[IX(j, k)] + alpha * P[IX(j, k)];
    for (int k = 1; k <= ny; ++k)
      for (int j = 1; j <= nx; ++j) R[IX(j, k)] = R[IX(j, k)] - alpha * W[IX(j, k)];
    block_solve(c, R, Z);
    for (int k = 1; k <= ny; ++k)
      for (int j = 1; j <= nx; ++j) rrn = rrn + R[IX(j, k)] * Z[IX(j, k)];
  } else {
#pragma omp parallel for
    for (int k = 1; k <= ny; ++k)
      for (int j = 1; j <= nx; ++j) U[IX(j, k)] = U[IX(j, k)] + alpha * P[IX(j, k)];
#pragma omp parallel for reduction(+ : rrn)
    for (int k = 1; k <= ny; ++k)
      for (int j = 1; j <= nx; ++j) {
        R[IX(j, k)] = R[IX(j, k)] - alpha * W[IX(j, k)];
        rrn = rrn + R[IX(j, k)] * R[IX(j, k)];
      }
  }
  return rrn;
}

void tlo_cg_calc_p(tlo_chunk* c, double beta, int ppcg_active) { /* :306-347 */
  const double* src = (c->precond != TLO_PREC_NONE || ppcg_active) ? Z : R;
#pragma omp parallel for
  for (int k = 1; k <= c->ny; ++k)
    for (int j = 1; j <= c->nx; ++j) P[IX(j, k)] = src[IX(j, k)] + beta * P[IX(j, k)];
}

/* ------------------------------------------------------------------------- */
/* tea_leaf_cheby: kernels/tea_leaf_cheby_kernel.f90                          */
/* ------------------------------------------------------------------------- */

void tlo_cheby_init(tlo_chunk* c, double theta) { /* :30-109 */
  const int nx = c->nx, ny = c->ny;
  for (int k = 1; k <= ny; ++k)
    for (int j = 1; j <= nx; ++j) {
      W[IX(j, k)] = smvp(c, U, j, k);
      R[IX(j, k)] = U0[IX(j, k)] - W[IX(j, k)];
    }
  if (c->precond != TLO_PREC_NONE) {
    precond_apply(c, R, Z);
    for (int k = 1; k <= ny; ++k)
      for (int j = 1; j <= nx; ++j) P[IX(j, k)] = Z[IX(j, k)] / theta;
  } else {
    for (int k = 1; k <= ny; ++k)
      for (int j = 1; j <= nx; ++j) P[IX(j, k)] = R[IX(j, k)] / theta;
  }
  for (int k = 1; k <= ny; ++k)
    for (int j = 1; j <= nx; ++j) U[IX(j, k)] = U[IX(j, k)] + P[IX(j, k)];
}

void tlo_cheby_iterate(tlo_chunk* c, double ch_alpha, double ch_beta) { /* :111-200 */
  const int nx = c->nx, ny = c->ny;
  const double rx = c->rx, ry = c->ry;
#pragma omp parallel for
  for (int k = 1; k <= ny; ++k)
    for (int j = 1; j <= nx; ++j) {
      W[IX(j, k)] = ((1.0 + ry * (KY[IX(j, k + 1)] + KY[IX(j, k)])) + rx * (KX[IX(j + 1, k)] + KX[IX(j, k)])) * U[IX(j, k)] -
                    ry * (KY[IX(j, k + 1)] * U[IX(j, k + 1)] + KY[IX(j, k)] * U[IX(j, k - 1)]) -
                    rx * (KX[IX(j + 1, k)] * U[IX(j + 1, k)] + KX[IX(j, k)] * U[IX(j - 1, k)]);
      R[IX(j, k)] = U0[IX(j, k)] - W[IX(j, k)];
    }
  if (c->precond != TLO_PREC_NONE) {
    precond_apply(c, R, Z);
    for (int k = 1; k <= ny; ++k)
      for (int j = 1; j <= nx; ++j) P[IX(j, k)] = ch_alpha * P[IX(j, k)] + ch_beta * Z[IX(j, k)];
  } else {
#pragma omp parallel for
    for (int k = 1; k <= ny; ++k)
      for (int j = 1; j <= nx; ++j) P[IX(j, k)] = ch_alpha * P[IX(j, k)] + ch_beta * R[IX(j, k)];
  }
#pragma omp parallel for
  for (int k = 1; k <= ny; ++k)
    for (int j = 1; j <= nx; ++j) U[IX(j, k)] = U[IX(j, k)] + P[IX(j, k)];
}

/* ------------------------------------------------------------------------- */
/* tea_leaf_ppcg: kernels/tea_leaf_ppcg_kernel.f90                            */
/* ------------------------------------------------------------------------- */

void tlo_ppcg_init_sd(tlo_chunk* c, double theta) { /* :31-88 */
  const double theta_r = 1.0 / theta;
  const double* src = (c->precond != TLO_PREC_NONE) ? Z : R;
  for (int k = 1; k <= c->ny; ++k)
    for (int j = 1; j <= c->nx; ++j) {
      SD[IX(j, k)] = src[IX(j, k)] * theta_r;
      RTEMP[IX(j, k)] = R[IX(j, k)];
      UTEMP[IX(j, k)] = SD[IX(j, k)];
    }
}

double tlo_ppcg_init(tlo_chunk* c, int step, int ppcg_active) { /* :90-201 */
  const int nx = c->nx, ny = c->ny;
  double rro = 0.0;
  if (step == 1) {
    for (int k = 1; k <= ny; ++k)
      for (int j = 1; j <= nx; ++j) {
        P[IX(j, k)] = 0.0;
        Z[IX(j, k)] = 0.0;
      }
  } else if (step == 3) {
    for (int k = 1; k <= ny; ++k)
      for (int j = 1; j <= nx; ++j) P[IX(j, k)] = 0.0;
  }
  if (c->precond != TLO_PREC_NONE || (ppcg_active && step == 3)) {
    if (step == 1 || step == 2) precond_apply(c, R, Z);
    if (step == 1 || step == 3)
      for (int k = 1; k <= ny; ++k)
        for (int j = 1; j <= nx; ++j) P[IX(j, k)] = Z[IX(j, k)];
  } else {
    if (step == 1)
      for (int k = 1; k <= ny; ++k)
        for (int j = 1; j <= nx; ++j) P[IX(j, k)] = R[IX(j, k)];
  }
  if (step == 1 || step == 3)
    for (int k = 1; k <= ny; ++k)
      for (int j = 1; j <= nx; ++j) rro = rro + R[IX(j, k)] * P[IX(j, k)];
  return rro;
}

/* :204-310 on the interior (the bounds of a single external tile, tea_leaf_ppcg.f90:358-387) */
void tlo_ppcg_inner(tlo_chunk* c, double ch_alpha, double ch_beta) {
  const int nx = c->nx, ny = c->ny;
#pragma omp parallel for
  for (int k = 1; k <= ny; ++k)
    for (int j = 1; j <= nx; ++j) RTEMP[IX(j, k)] = RTEMP[IX(j, k)] - smvp(c, SD, j, k);
  if (c->precond == TLO_PREC_JAC_DIAG) {
    for (int k = 1; k <= ny; ++k)
      for (int j = 1; j <= nx; ++j) {
        SD[IX(j, k)] = ch_alpha * SD[IX(j, k)] + ch_beta * MI[IX(j, k)] * RTEMP[IX(j, k)];
        UTEMP[IX(j, k)] = UTEMP[IX(j, k)] + SD[IX(j, k)];
      }
  } else if (c->precond == TLO_PREC_JAC_BLOCK) {
    block_solve(c, RTEMP, Z);
    for (int k = 1; k <= ny; ++k)
      for (int j = 1; j <= nx; ++j) {
        SD[IX(j, k)] = ch_alpha * SD[IX(j, k)] + ch_beta * Z[IX(j, k)];
        UTEMP[IX(j, k)] = UTEMP[IX(j, k)] + SD[IX(j, k)];
      }
  } else {
#pragma omp parallel for
    for (int k = 1; k <= ny; ++k)
      for (int j = 1; j <= nx; ++j) {
        SD[IX(j, k)] = ch_alpha * SD[IX(j, k)] + ch_beta * RTEMP[IX(j, k)];
        UTEMP[IX(j, k)] = UTEMP[IX(j, k)] + SD[IX(j, k)];
      }
  }
}

double tlo_ppcg_calc_zrnorm(tlo_chunk* c, int ppcg_active) { /* :411-451 */
  double norm = 0.0;
  const double* a = (c->precond != TLO_PREC_NONE || ppcg_active) ? Z : R;
  for (int k = 1; k <= c->ny; ++k)
    for (int j = 1; j <= c->nx; ++j) norm = norm + a[IX(j, k)] * R[IX(j, k)];
  return norm;
}

void tlo_ppcg_update_z(tlo_chunk* c) { /* :453-477 */
  for (int k = 1; k <= c->ny; ++k)
    for (int j = 1; j <= c->nx; ++j) Z[IX(j, k)] = UTEMP[IX(j, k)];
}

void tlo_ppcg_store_r(tlo_chunk* c) { /* :507-530 */
  for (int k = 1; k <= c->ny; ++k)
    for (int j = 1; j <= c->nx; ++j) R_STORE[IX(j, k)] = R[IX(j, k)];
}

double tlo_ppcg_calc_rrn(tlo_chunk* c) { /* :532-561 */
  double rrn = 0.0;
  for (int k = 1; k <= c->ny; ++k)
    for (int j = 1; j <= c->nx; ++j) rrn = rrn + (R[IX(j, k)] - R_STORE[IX(j, k)]) * Z[IX(j, k)];
  return rrn;
}

/* ------------------------------------------------------------------------- */
/* tea_leaf_jacobi: kernels/tea_leaf_jacobi_kernel.f90:26-77; un = vector_r   */
/* (tea_leaf_jacobi.f90:36-38)                                                */
/* ------------------------------------------------------------------------- */

double tlo_jacobi_solve(tlo_chunk* c) {
  const int nx = c->nx, ny = c->ny;
  const double rx = c->rx, ry = c->ry;
  double* un = R;
  double error = 0.0;
  for (int k = 1; k <= ny; ++k)
    for (int j = 1; j <= nx; ++j) un[IX(j, k)] = U[IX(j, k)];
#pragma omp parallel for reduction(+ : error)
  for (int k = 1; k <= ny; ++k)
    for (int j = 1; j <= nx; ++j) {
      U[IX(j, k)] = ((U0[IX(j, k)] + rx * (KX[IX(j + 1, k)] * un[IX(j + 1, k)] + KX[IX(j, k)] * un[IX(j - 1, k)])) +
                     ry * (KY[IX(j, k + 1)] * un[IX(j, k + 1)] + KY[IX(j, k)] * un[IX(j, k - 1)])) /
                    ((1.0 + rx * (KX[IX(j, k)] + KX[IX(j + 1, k)])) + ry * (KY[IX(j, k)] + KY[IX(j, k + 1)]));
      error = error + fabs(U[IX(j, k)] - un[IX(j, k)]);
    }
  return error;
}

/* ------------------------------------------------------------------------- */
/* host scalar math                                                           */
/* ------------------------------------------------------------------------- */

/* Number of eigenvalues of the symmetric tridiagonal T (diagonal d, off-diagonal e)
 * that are strictly less than x: the Sturm sequence count from the LDL^T
 * factorisation of T - xI (Golub & Van Loan, Matrix Computations, sec. 8.4.1). */
static int sturm_count(const double* d, const double* e, int n, double x, double pivmin) {
  int count = 0;
  double q = d[0] - x;
  if (fabs(q) < pivmin) q = -pivmin;
  if (q < 0.0) ++count;
  for (int i = 1; i < n; ++i) {
    q = d[i] - x - (e[i - 1] * e[i - 1]) / q;
    if (fabs(q) < pivmin) q = -pivmin;
    if (q < 0.0) ++count;
  }
  return count;
}

/* k-th smallest eigenvalue (0-based) by bisection on the Sturm count, refined until
 * the bracketing interval cannot be split further in FP64. */
static double kth_eigenvalue(const double* d, const double* e, int n, int kth, double lo, double hi, double pivmin) {
  for (int it = 0; it < 2000; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (!(mid > lo && mid < hi)) break;
    if (sturm_count(d, e, n, mid, pivmin) > kth)
      hi = mid;
    else
      lo = mid;
  }
  return 0.5 * (lo + hi);
}

void tlo_tridiag_eigenvalues(const double* d, const double* off, int n, double* out) {
  if (n <= 0) return;
  /* Gershgorin interval */
  double lo = d[0], hi = d[0], tmax = 0.0;
  for (int i = 0; i < n; ++i) {
    const double rad = (i > 0 ? fabs(off[i - 1]) : 0.0) + (i < n - 1 ? fabs(off[i]) : 0.0);
    if (d[i] - rad < lo) lo = d[i] - rad;
    if (d[i] + rad > hi) hi = d[i] + rad;
    if (fabs(d[i]) > tmax) tmax = fabs(d[i]);
    if (i < n - 1 && fabs(off[i]) > tmax) tmax = fabs(off[i]);
  }
  const double pad = 2.0 * 2.220446049250313e-16 * (fabs(lo) > fabs(hi) ? fabs(lo) : fabs(hi)) + 1e-300;
  lo -= pad;
  hi += pad;
  const double pivmin = 1e-300 + 2.2250738585072014e-308 * (tmax * tmax > 1.0 ? tmax * tmax : 1.0);
  for (int k = 0; k < n; ++k) out[k] = kth_eigenvalue(d, off, n, k, lo, hi, pivmin);
}

/* tea_leaf_cheby.f90:142-176: Lanczos tridiagonal from the CG coefficients, its extreme
 * eigenvalues (the reference uses implicit QL; bisection on Sturm counts is used here). */
int tlo_calc_eigenvalues(const double* cg_alphas, const double* cg_betas, int nsteps, double* eigmin, double* eigmax) {
  if (nsteps <= 0) return 1;
  double* diag = (double*)calloc((size_t)nsteps, sizeof(double));
  double* off = (double*)calloc((size_t)nsteps, sizeof(double));
  double* ev = (double*)calloc((size_t)nsteps, sizeof(double));
  for (int n = 1; n <= nsteps; ++n) {
    diag[n - 1] = 1.0 / cg_alphas[n - 1];
    if (n > 1) diag[n - 1] = diag[n - 1] + cg_betas[n - 2] / cg_alphas[n - 2];
    if (n < nsteps) off[n - 1] = sqrt(cg_betas[n - 1]) / cg_alphas[n - 1]; /* couples n and n+1 */
  }
  tlo_tridiag_eigenvalues(diag, off, nsteps, ev);
  *eigmin = ev[0];
  *eigmax = ev[nsteps - 1];
  free(diag);
  free(off);
  free(ev);
  if (*eigmin < 0.0 || *eigmax < 0.0) return 1;
  return 0;
}

void tlo_calc_ch_coefs(double* ch_alphas, double* ch_betas, double eigmin, double eigmax, double* theta, int n) {
  /* tea_leaf_cheby.f90:178-205 */
  *theta = (eigmax + eigmin) / 2;
  const double delta = (eigmax - eigmin) / 2;
  const double sigma = *theta / delta;
  double rho_old = 1.0 / sigma;
  for (int i = 0; i < n; ++i) {
    const double rho_new = 1.0 / (2.0 * sigma - rho_old);
    ch_alphas[i] = rho_new * rho_old;
    ch_betas[i] = 2.0 * rho_new / delta;
    rho_old = rho_new;
  }
}

/* ------------------------------------------------------------------------- */
/* tea_leaf_ppcg.f90:211-431 (single tile, every face external)               */
/* ------------------------------------------------------------------------- */

static void run_ppcg_inner_steps(tlo_chunk* c, const double* ch_alphas, const double* ch_betas, double theta,
                                 int inner_steps) {
  if (inner_steps < 0) return;
  tlo_ppcg_init_sd(c, theta);
  const int h = c->h;
  int fields[TLO_NUM_FIELDS + 1];
  for (int cur = 1; cur <= inner_steps; cur += h) {
    memset(fields, 0, sizeof(fields));
    fields[TLO_F_SD] = 1;
    fields[TLO_F_R] = 1;
    tlo_update_halo(c, fields, h);
    memset(fields, 0, sizeof(fields));
    fields[TLO_F_SD] = 1;
    for (int bounds_extra = h - 1; bounds_extra >= 0; --bounds_extra) {
      const int step = cur + h - 1 - bounds_extra;
      tlo_ppcg_inner(c, ch_alphas[step - 1], ch_betas[step - 1]);
      if (c->reflective) tlo_update_halo(c, fields, 1); /* :316-339 */
      if (step == inner_steps) break;
    }
  }
  tlo_ppcg_update_z(c);
}

/* ------------------------------------------------------------------------- */
/* tea_leaf(): tea_solve.f90:37-503                                           */
/* ------------------------------------------------------------------------- */

#define SETF(...)                                       \
  do {                                                  \
    memset(fields, 0, sizeof(fields));                  \
    int ids_[] = {__VA_ARGS__};                         \
    for (size_t i_ = 0; i_ < sizeof(ids_) / sizeof(int); ++i_) fields[ids_[i_]] = 1; \
  } while (0)

int tlo_tea_leaf(tlo_chunk* c, const tlo_opts* o, tlo_persist* ps, double dt, tlo_solve_info* info) {
  const int use_cg = o->solver == TLO_SOLVER_CG, use_cheby = o->solver == TLO_SOLVER_CHEBY;
  const int use_ppcg = o->solver == TLO_SOLVER_PPCG, use_jacobi = o->solver == TLO_SOLVER_JACOBI;
  const int max_iters = o->max_iters;
  int fields[TLO_NUM_FIELDS + 1];
  double old_error, error = 0.0, exact_error = 0.0, initial_residual;
  double rro = 0.0, pw = 0.0, rrn = 0.0, alpha, beta;
  const int ncoef = max_iters + 2 > o->ppcg_inner_steps + 1 ? max_iters + 2 : o->ppcg_inner_steps + 1;
  double* cg_alphas = (double*)calloc((size_t)max_iters + 1, sizeof(double));
  double* cg_betas = (double*)calloc((size_t)max_iters + 1, sizeof(double));
  double* ch_alphas = (double*)calloc((size_t)ncoef, sizeof(double));
  double* ch_betas = (double*)calloc((size_t)ncoef, sizeof(double));
  int est_itc = 0, cheby_calc_steps = 0, max_cheby_iters = 0, ppcg_inner_iters = 0, cg_calc_steps = 0;
  int ch_switch_check = 0, ppcg_active = 0, n;
  memset(info, 0, sizeof(*info));

  SETF(TLO_F_ENERGY1, TLO_F_DENSITY);
  tlo_update_halo(c, fields, c->h);
  tlo_common_init(c, dt);
  SETF(TLO_F_U);
  tlo_update_halo(c, fields, 1);
  tlo_calc_residual(c);
  initial_residual = tlo_calc_2norm(c, 1);
  old_error = initial_residual;
  initial_residual = sqrt(fabs(initial_residual));

  if (use_cg || use_cheby || use_ppcg) {
    rro = tlo_cg_init(c);
    SETF(TLO_F_U, TLO_F_P);
    tlo_update_halo(c, fields, 1);
    SETF(TLO_F_P);
  } else if (use_jacobi) {
    SETF(TLO_F_U);
  }

  for (n = 1; n <= max_iters; ++n) {
    if (!ch_switch_check) {
      if (cheby_calc_steps > 0)
        ch_switch_check = 1;
      else if (!ps->first && use_ppcg && n > 1)
        ch_switch_check = 1;
      else if (fabs(old_error) <= o->ch_cg_epslim && n >= o->ch_cg_presteps)
        ch_switch_check = 1;
      else
        ch_switch_check = 0;
    }

    if ((use_cheby || use_ppcg) && ch_switch_check) {
      if (cheby_calc_steps == 0) {
        max_cheby_iters = max_iters - n + 2;
        if (ps->first) {
          const int bad = tlo_calc_eigenvalues(cg_alphas + 1, cg_betas + 1, n - 1, &ps->eigmin, &ps->eigmax);
          ps->first = 0;
          if (bad) {
            info->status = 1;
            break;
          }
          ps->eigmin = ps->eigmin * 0.95;
          ps->eigmax = ps->eigmax * 1.05;
        }
        if (use_cheby) {
          tlo_calc_ch_coefs(ch_alphas + 1, ch_betas + 1, ps->eigmin, ps->eigmax, &ps->theta, max_cheby_iters);
          SETF(TLO_F_U);
        } else if (use_ppcg) {
          tlo_calc_ch_coefs(ch_alphas + 1, ch_betas + 1, ps->eigmin, ps->eigmax, &ps->theta, o->ppcg_inner_steps);
          ppcg_active = 1;
        }
        ps->cn = ps->eigmax / ps->eigmin;

        rro = tlo_ppcg_init(c, 2, ppcg_active);
        run_ppcg_inner_steps(c, ch_alphas + 1, ch_betas + 1, ps->theta, o->ppcg_inner_steps);
        ppcg_inner_iters = ppcg_inner_iters + o->ppcg_inner_steps;
        rro = tlo_ppcg_init(c, 3, ppcg_active);
        SETF(TLO_F_P);
        tlo_update_halo(c, fields, 1);
      }

      if (use_cheby) {
        if (cheby_calc_steps == 0) {
          /* tea_leaf_cheby.f90:208-252 (its 'error' argument is old_error) */
          const double bb = tlo_calc_2norm(c, 0);
          tlo_cheby_init(c, ps->theta);
          tlo_update_halo(c, fields, 1);
          tlo_cheby_iterate(c, ch_alphas[1], ch_betas[1]);
          old_error = tlo_calc_2norm(c, 1);
          const double it_alpha = o->eps / 2.0 * sqrt(bb / old_error);
          const double gamm = (sqrt(ps->cn) - 1.0) / (sqrt(ps->cn) + 1.0);
          est_itc = (int)lround(log(it_alpha) / log(gamm));
          cheby_calc_steps = 1;
        } else {
          tlo_cheby_iterate(c, ch_alphas[cheby_calc_steps], ch_betas[cheby_calc_steps]);
          if (n >= est_itc && n % 10 == 0) error = tlo_calc_2norm(c, 1);
        }
      } else if (use_ppcg) {
        pw = tlo_cg_calc_w(c);
        tlo_ppcg_store_r(c);
        rro = tlo_ppcg_calc_zrnorm(c, ppcg_active);
        alpha = rro / pw;
        rrn = tlo_cg_calc_ur(c, alpha);
        run_ppcg_inner_steps(c, ch_alphas + 1, ch_betas + 1, ps->theta, o->ppcg_inner_steps);
        ppcg_inner_iters = ppcg_inner_iters + o->ppcg_inner_steps;
        rrn = tlo_ppcg_calc_rrn(c);
        beta = rrn / rro;
        tlo_cg_calc_p(c, beta, ppcg_active);
        error = rrn;
        rro = rrn;
      }
      cheby_calc_steps = cheby_calc_steps + 1;
    } else if (use_cg || use_cheby || use_ppcg) {
      fields[TLO_F_P] = 1;
      cg_calc_steps = cg_calc_steps + 1;
      pw = tlo_cg_calc_w(c);
      alpha = rro / pw;
      cg_alphas[n] = alpha;
      rrn = tlo_cg_calc_ur(c, alpha);
      beta = rrn / rro;
      cg_betas[n] = beta;
      tlo_cg_calc_p(c, beta, ppcg_active);
      error = rrn;
      rro = rrn;
    } else if (use_jacobi) {
      error = tlo_jacobi_solve(c);
    }

    tlo_update_halo(c, fields, 1);
    error = sqrt(fabs(error));
    if (fabs(error) < o->eps * initial_residual) break;
    old_error = error;
  }
  (void)pw;

  if (o->check_result) {
    SETF(TLO_F_U);
    tlo_update_halo(c, fields, 1);
    tlo_calc_residual(c);
    exact_error = tlo_calc_2norm(c, 1);
    exact_error = sqrt(exact_error);
  }

  info->n_exit = n;
  info->reported_iterations = n - 1;
  info->ppcg_inner_iters = ppcg_inner_iters;
  info->cg_calc_steps = cg_calc_steps;
  info->cheby_calc_steps = cheby_calc_steps;
  info->est_itc = est_itc;
  info->initial_residual = initial_residual;
  info->error = error;
  info->exact_error = exact_error;
  info->eigmin = ps->eigmin;
  info->eigmax = ps->eigmax;

  if (info->status == 0) {
    tlo_finalise(c);
    SETF(TLO_F_ENERGY1);
    tlo_update_halo(c, fields, 1);
  }
  free(cg_alphas);
  free(cg_betas);
  free(ch_alphas);
  free(ch_betas);
  return info->status;
}
