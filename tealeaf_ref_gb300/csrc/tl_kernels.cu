// tl_kernels.cu -- set-up, summary, halo and per-kernel (drop-in) kernels of the TeaLeaf
// GB300 solver.  Each __global__ cites the reference subroutine whose loop it replaces.
//
// The 5-point operator (tea_leaf_common_kernel.f90:235-237) is applied as
//   A v = Di*v - cy(j,k+1) v(j,k+1) - cy(j,k) v(j,k-1) - cx(j+1,k) v(j+1,k) - cx(j,k) v(j-1,k)
// with cx = rx*Kx, cy = ry*Ky pre-scaled once per solve: one multiply and four FMAs per
// cell instead of the seven double operations of the unscaled form.  FP64 issue rate, not
// HBM bandwidth, bounds these kernels on GB300, so fewer double operations per cell is
// the first-order optimisation.  Di itself is built with the reference's exact operation
// order (no contraction).
#include "tl_kernels.cuh"

#include <cmath>

namespace tl {

namespace {

constexpr int TB = 256;        // threads per block for the row kernels
constexpr int RED_ROWS = 256;  // max gridDim.y of reducing row kernels

__device__ __forceinline__ double apply_A(const double* __restrict__ v, const double* __restrict__ cx,
                                          const double* __restrict__ cy, const double* __restrict__ di,
                                          long long c, int ld) {
  double a = di[c] * v[c];
  a = fma(-cy[c + ld], v[c + ld], a);
  a = fma(-cy[c], v[c - ld], a);
  a = fma(-cx[c + 1], v[c + 1], a);
  a = fma(-cx[c], v[c - 1], a);
  return a;
}

inline dim3 row_grid(const Layout& L, bool reducing) {
  const int gx = (L.nx + TB - 1) / TB;
  int gy = L.ny;
  if (reducing && gy > RED_ROWS) gy = RED_ROWS;
  if (gy > 65535) gy = 65535;
  return dim3(gx, gy);
}

#define FOR_ROWS(L)                                                   \
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;             \
  for (int k = blockIdx.y + 1; k <= (L).ny; k += gridDim.y)

// ---------------------------------------------------------------------------
// Epilogues
// ---------------------------------------------------------------------------
template <int NV>
struct EpiMode {
  LoopState* st;
  int mode;
  __device__ void operator()(double (&acc)[NV]) const {
    switch (mode) {
      case RED_INIT_RESIDUAL:
        st->old_error = acc[0];
        st->initial_residual = sqrt(fabs(acc[0]));
        break;
      case RED_RRO:
        st->rro = acc[0];
        break;
      default:
        break;
    }
#pragma unroll
    for (int i = 0; i < NV; ++i) st->red[i] = acc[i];
  }
};

// ---------------------------------------------------------------------------
// tea_leaf_common_init_kernel (kernels/tea_leaf_common_kernel.f90:75-141):
// face coefficients Kx(j,k) j=1..nx+1, k=1..ny and Ky(j,k) j=1..nx, k=1..ny+1, from
// w = density (CONDUCTIVITY) or 1/density (RECIP_CONDUCTIVITY); external faces zero
// unless reflective.  Also the pre-scaled cx = rx*Kx, cy = ry*Ky.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double coef_w(double rho, int coefficient) {
  return coefficient == 2 ? __ddiv_rn(1.0, rho) : rho;
}

__global__ void k_init_faces(Fields f, Layout L, Geometry g) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  for (int k = blockIdx.y + 1; k <= L.ny + 1; k += gridDim.y) {
    if (j > L.nx + 1) continue;
    const long long c = L.at(j, k);
    const double w0 = coef_w(f.density[c], g.coefficient);
    if (k <= L.ny) {
      const double wl = coef_w(f.density[c - 1], g.coefficient);
      double kx = __ddiv_rn(__dadd_rn(wl, w0), __dmul_rn(__dmul_rn(2.0, wl), w0));
      if (!g.reflective && (j == 1 || j == L.nx + 1)) kx = 0.0;
      f.kx[c] = kx;
      f.cx[c] = __dmul_rn(g.rx, kx);
    }
    if (j <= L.nx) {
      const double wb = coef_w(f.density[c - L.ld], g.coefficient);
      double ky = __ddiv_rn(__dadd_rn(wb, w0), __dmul_rn(__dmul_rn(2.0, wb), w0));
      if (!g.reflective && (k == 1 || k == L.ny + 1)) ky = 0.0;
      f.ky[c] = ky;
      f.cy[c] = __dmul_rn(g.ry, ky);
    }
  }
}

// common_kernel.f90:67-72 (u = u0 = energy*density), :144-152 (Di, exact operation order),
// :276-307 (Mi = 1/Di for jac_diag), :162-174 (w = A u, r = u - w; dead in tea_leaf() because
// calc_residual overwrites r, so the solve driver skips it).
__global__ void k_init_cells(Fields f, Layout L, Geometry g) {
  FOR_ROWS(L) {
    if (j > L.nx) continue;
    const long long c = L.at(j, k);
    const double u = __dmul_rn(f.energy1[c], f.density[c]);
    f.u[c] = u;
    f.u0[c] = u;
    const double di = __dadd_rn(__dadd_rn(1.0, __dmul_rn(g.ry, __dadd_rn(f.ky[c + L.ld], f.ky[c]))),
                                __dmul_rn(g.rx, __dadd_rn(f.kx[c + 1], f.kx[c])));
    f.di[c] = di;
    if (g.precond == 2) f.mi[c] = (di != 0.0) ? __ddiv_rn(1.0, di) : 0.0;
  }
}

// common_kernel.f90:67-72 alone (u = u0 = energy*density): the set-up of a solve whose face
// coefficients, Di and preconditioner factors are still those of the previous solve (same
// density, same dt), so k_init_faces / the rest of k_init_cells would rewrite the same bits.
__global__ void k_init_state(Fields f, Layout L) {
  FOR_ROWS(L) {
    if (j > L.nx) continue;
    const long long c = L.at(j, k);
    const double u = __dmul_rn(f.energy1[c], f.density[c]);
    f.u[c] = u;
    f.u0[c] = u;
  }
}

__global__ void k_init_residual(Fields f, Layout L) {
  FOR_ROWS(L) {
    if (j > L.nx) continue;
    const long long c = L.at(j, k);
    const double w = apply_A(f.u, f.cx, f.cy, f.di, c, L.ld);
    f.w[c] = w;
    f.r[c] = f.u[c] - w;
  }
}

// tea_block_init (common_kernel.f90:337-376): 4-row tridiagonal factors per column.
__global__ void k_block_init(Fields f, Layout L, Geometry g) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int ko = blockIdx.y * 4 + 1;
  if (j > L.nx || ko > L.ny) return;
  const int top = min(ko + 3, L.ny);
  long long c = L.at(j, ko);
  double cp = __ddiv_rn(__dmul_rn(-f.ky[c + L.ld], g.ry), f.di[c]);
  f.cp[c] = cp;
  for (int k = ko + 1; k <= top; ++k) {
    c = L.at(j, k);
    const double bfp = __ddiv_rn(1.0, __dsub_rn(f.di[c], __dmul_rn(__dmul_rn(-f.ky[c], g.ry), cp)));
    f.bfp[c] = bfp;
    cp = __dmul_rn(__dmul_rn(-f.ky[c + L.ld], g.ry), bfp);
    f.cp[c] = cp;
  }
}

// tea_block_solve (common_kernel.f90:378-468): z = M^-1 r, 4-row blocks (last block may be short).
__global__ void k_block_solve(Fields f, Layout L, Geometry g, const double* __restrict__ r, double* __restrict__ z) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int bottom = blockIdx.y * 4 + 1;
  if (j > L.nx || bottom > L.ny) return;
  const int top = min(bottom + 3, L.ny);
  double dp[4], zl[4];
  long long c = L.at(j, bottom);
  dp[0] = r[c] / f.di[c];
  for (int k = bottom + 1; k <= top; ++k) {
    c = L.at(j, k);
    dp[k - bottom] = (r[c] - (-f.ky[c] * g.ry) * dp[k - bottom - 1]) * f.bfp[c];
  }
  zl[top - bottom] = dp[top - bottom];
  for (int k = top - 1; k >= bottom; --k) zl[k - bottom] = dp[k - bottom] - f.cp[L.at(j, k)] * zl[k - bottom + 1];
  for (int k = bottom; k <= top; ++k) z[L.at(j, k)] = zl[k - bottom];
}

__global__ void k_diag_solve(Layout L, const double* __restrict__ mi, const double* __restrict__ r,
                             double* __restrict__ z) {
  FOR_ROWS(L) {
    if (j > L.nx) continue;
    const long long c = L.at(j, k);
    z[c] = mi[c] * r[c];
  }
}

// generate_chunk_kernel.f90:80-140 (+ set_field: energy1 = energy0 on the interior, and
// u = energy0*density on the full range as generate_chunk.f90 passes field%u).  states:
// [density, energy, xmin, xmax, ymin, ymax, radius, geometry] per state, extents already
// nudged.  All arithmetic uses round-to-nearest intrinsics so that the in/out tests see
// exactly the reference's coordinates.
__global__ void k_generate(Fields f, Layout L, int nstates, const double* __restrict__ st, double xmin, double ymin,
                           double dx, double dy) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;  // 0..nx+1
  for (int k = blockIdx.y; k <= L.ny + 1; k += gridDim.y) {
    if (j > L.nx + 1) continue;
    const long long c = L.at(j, k);
    double den = st[0], en = st[1];
    const double vx0 = __dadd_rn(xmin, __dmul_rn(dx, (double)(float)(j - 1)));
    const double vx1 = __dadd_rn(xmin, __dmul_rn(dx, (double)(float)(j)));
    const double vy0 = __dadd_rn(ymin, __dmul_rn(dy, (double)(float)(k - 1)));
    const double vy1 = __dadd_rn(ymin, __dmul_rn(dy, (double)(float)(k)));
    const double cxj = __dmul_rn(0.5, __dadd_rn(vx0, vx1));
    const double cyk = __dmul_rn(0.5, __dadd_rn(vy0, vy1));
    const bool interior = j >= 1 && j <= L.nx && k >= 1 && k <= L.ny;
    for (int s = 1; s < nstates; ++s) {
      const double* q = st + 8 * s;
      const int geom = (int)q[7];
      bool hit = false;
      if (geom == 1) {
        hit = interior && vx1 >= q[2] && vx0 < q[3] && vy1 >= q[4] && vy0 < q[5];
      } else if (geom == 2) {
        const double ex = __dsub_rn(cxj, q[2]), ey = __dsub_rn(cyk, q[4]);
        const double rad = __dsqrt_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)));
        hit = rad <= q[6];
      } else if (geom == 3) {
        hit = vx0 == q[2] && vy0 == q[4];
      }
      if (hit) {
        den = q[0];
        en = q[1];
      }
    }
    f.density[c] = den;
    f.u[c] = __dmul_rn(en, den);
    f.energy1[c] = interior ? en : 0.0;
  }
}

// field_summary_kernel.f90:44-62: vol, mass, ie, temp.
// One cell's terms of the summary, in the order k_finalise_summary adds them too (same grid,
// same per-thread order: the two kernels give the same bits).
__device__ __forceinline__ void summary_terms(double (&v)[4], double cell_vol, double rho, double e, double u) {
  const double cell_mass = cell_vol * rho;
  v[0] += cell_vol;
  v[1] += cell_mass;
  v[2] = fma(cell_mass, e, v[2]);
  v[3] = fma(cell_mass, u, v[3]);
}

__global__ void k_field_summary(Fields f, Layout L, double cell_vol, Reduce rd) {
  double v[4] = {0.0, 0.0, 0.0, 0.0};
  FOR_ROWS(L) {
    if (j > L.nx) continue;
    const long long c = L.at(j, k);
    summary_terms(v, cell_vol, f.density[c], f.energy1[c], f.u[c]);
  }
  grid_reduce<4>(v, rd, EpiMode<4>{rd.st, RED_STORE});
}

// tea_leaf_kernel_finalise (common_kernel.f90:179-206) fused with field_summary_kernel
// (field_summary_kernel.f90:44-62): energy1 = u / density and vol, mass, ie, temp in one sweep
// (st->red[0..4)).  st non-null: the CG loop's pending deferred u += alpha p is applied first.
__global__ void k_finalise_summary(Fields f, Layout L, double cell_vol, Reduce rd, const LoopState* __restrict__ st) {
  const bool pending = st && st->u_pending != 0;
  const double ua = pending ? st->u_alpha : 0.0;
  const double* __restrict__ p = (pending && st->u_psel) ? f.p2 : f.p;
  double v[4] = {0.0, 0.0, 0.0, 0.0};
  FOR_ROWS(L) {
    if (j > L.nx) continue;
    const long long c = L.at(j, k);
    double u = f.u[c];
    if (pending) {
      u = fma(ua, p[c], u);
      f.u[c] = u;
    }
    const double rho = f.density[c];
    const double e = u / rho;
    f.energy1[c] = e;
    summary_terms(v, cell_vol, rho, e, u);
  }
  grid_reduce<4>(v, rd, EpiMode<4>{rd.st, RED_STORE});
}

// update_halo_cell (update_halo_kernel.f90:136-195) at depth 1: left/right columns first
// (rows 0..ny+1), then bottom/top rows (columns 0..nx+1) in a second launch.
__global__ void k_halo_lr(double* const* fl, int nf, Layout L) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;  // 0..ny+1
  if (k > L.ny + 1) return;
  for (int i = 0; i < nf; ++i) {
    double* m = fl[i];
    m[L.at(0, k)] = m[L.at(1, k)];
    m[L.at(L.nx + 1, k)] = m[L.at(L.nx, k)];
  }
}
__global__ void k_halo_bt(double* const* fl, int nf, Layout L) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;  // 0..nx+1
  if (j > L.nx + 1) return;
  for (int i = 0; i < nf; ++i) {
    double* m = fl[i];
    m[L.at(j, 0)] = m[L.at(j, 1)];
    m[L.at(j, L.ny + 1)] = m[L.at(j, L.ny)];
  }
}

// The interior of a field (context layout) from / to a host-layout array whose row k starts at
// (k-1) * ld: the device side of the host transfers, which move the host array with one
// contiguous copy.
__global__ void k_unpack(double* __restrict__ dst, const double* __restrict__ src, long long ld, Layout L) {
  FOR_ROWS(L) {
    if (j > L.nx) continue;
    dst[L.at(j, k)] = src[(long long)(k - 1) * ld + (j - 1)];
  }
}
__global__ void k_pack(double* __restrict__ dst, long long ld, const double* __restrict__ src, Layout L) {
  FOR_ROWS(L) {
    if (j > L.nx) continue;
    dst[(long long)(k - 1) * ld + (j - 1)] = src[L.at(j, k)];
  }
}

__global__ void k_copy_interior(double* __restrict__ dst, const double* __restrict__ src, Layout L) {
  FOR_ROWS(L) {
    if (j > L.nx) continue;
    const long long c = L.at(j, k);
    dst[c] = src[c];
  }
}

// ---------------------------------------------------------------------------
// per-kernel (drop-in) kernels
// ---------------------------------------------------------------------------

// tea_leaf_calc_residual_kernel (common_kernel.f90:208-244), optionally with r.r.
template <bool NORM>
__global__ void k_residual(Fields f, Layout L, Reduce rd, int mode) {
  double v[1] = {0.0};
  FOR_ROWS(L) {
    if (j > L.nx) continue;
    const long long c = L.at(j, k);
    const double r = f.u0[c] - apply_A(f.u, f.cx, f.cy, f.di, c, L.ld);
    f.r[c] = r;
    if (NORM) v[0] = fma(r, r, v[0]);
  }
  if (NORM) grid_reduce<1>(v, rd, EpiMode<1>{rd.st, mode});
}

// tea_leaf_calc_2norm_kernel (common_kernel.f90:246-274)
__global__ void k_norm2(const double* __restrict__ a, Layout L, Reduce rd, int mode) {
  double v[1] = {0.0};
  FOR_ROWS(L) {
    if (j > L.nx) continue;
    const double x = a[L.at(j, k)];
    v[0] = fma(x, x, v[0]);
  }
  grid_reduce<1>(v, rd, EpiMode<1>{rd.st, mode});
}

// sum a.(b - bminus)  (ppcg_calc_zrnorm, ppcg_calc_rrn, cg_init's r.p)
__global__ void k_dot(const double* __restrict__ a, const double* __restrict__ b, const double* __restrict__ bm,
                      Layout L, Reduce rd, int mode) {
  double v[1] = {0.0};
  FOR_ROWS(L) {
    if (j > L.nx) continue;
    const long long c = L.at(j, k);
    const double y = bm ? (b[c] - bm[c]) : b[c];
    v[0] = fma(a[c], y, v[0]);
  }
  grid_reduce<1>(v, rd, EpiMode<1>{rd.st, mode});
}

// tea_leaf_kernel_finalise (common_kernel.f90:179-206)
__global__ void k_finalise(Fields f, Layout L) {
  FOR_ROWS(L) {
    if (j > L.nx) continue;
    const long long c = L.at(j, k);
    f.energy1[c] = f.u[c] / f.density[c];
  }
}

// The start of a CG solve in one sweep: tea_leaf_calc_residual_kernel (common_kernel.f90:208-244,
// r = u0 - A u), tea_leaf_calc_2norm_kernel of r (:246-274; the initial residual and old_error,
// tea_solve.f90:124-130) and tea_leaf_cg_init_kernel (cg_kernel.f90:31-112) without a
// preconditioner (p = r, z = 0, rro = r.p) or with jac_diag (z = Mi r, p = z, rro = r.z).
struct EpiResidualCgInit {
  LoopState* st;
  __device__ void operator()(double (&acc)[2]) const {
    st->old_error = acc[0];
    st->initial_residual = sqrt(fabs(acc[0]));
    st->rro = acc[1];
    st->red[0] = acc[0];
    st->red[1] = acc[1];
  }
};
template <bool DIAG>
__global__ void k_residual_cg_init(Fields f, Layout L, Reduce rd) {
  double v[2] = {0.0, 0.0};
  FOR_ROWS(L) {
    if (j > L.nx) continue;
    const long long c = L.at(j, k);
    const double r = f.u0[c] - apply_A(f.u, f.cx, f.cy, f.di, c, L.ld);
    f.r[c] = r;
    double p = r;
    if (DIAG) {
      p = f.mi[c] * r;
      f.z[c] = p;
    } else {
      f.z[c] = 0.0;
    }
    f.p[c] = p;
    v[0] = fma(r, r, v[0]);
    v[1] = fma(r, p, v[1]);
  }
  grid_reduce<2>(v, rd, EpiResidualCgInit{rd.st});
}

// tea_leaf_kernel_finalise with the CG loop's last deferred u += alpha p (LoopState::u_pending)
// applied in the same sweep: u = u + alpha p, energy1 = u / density.
__global__ void k_finalise_flush(Fields f, Layout L, const LoopState* __restrict__ st) {
  const bool pending = st->u_pending != 0;
  const double ua = st->u_alpha;
  const double* __restrict__ p = st->u_psel ? f.p2 : f.p;
  FOR_ROWS(L) {
    if (j > L.nx) continue;
    const long long c = L.at(j, k);
    double u = f.u[c];
    if (pending) {
      u = fma(ua, p[c], u);
      f.u[c] = u;
    }
    f.energy1[c] = u / f.density[c];
  }
}

// tea_leaf_cg_init_kernel (cg_kernel.f90:31-112), after the preconditioner filled z.
__global__ void k_cg_init(Fields f, Layout L, int precond, Reduce rd, int mode) {
  double v[1] = {0.0};
  FOR_ROWS(L) {
    if (j > L.nx) continue;
    const long long c = L.at(j, k);
    const double p = (precond != 1) ? f.z[c] : f.r[c];
    if (precond == 1) f.z[c] = 0.0;
    f.p[c] = p;
    v[0] = fma(f.r[c], p, v[0]);
  }
  grid_reduce<1>(v, rd, EpiMode<1>{rd.st, mode});
}

// tea_leaf_cg_calc_w_kernel (cg_kernel.f90:114-156)
__global__ void k_cg_calc_w(Fields f, Layout L, Reduce rd) {
  double v[1] = {0.0};
  FOR_ROWS(L) {
    if (j > L.nx) continue;
    const long long c = L.at(j, k);
    const double w = apply_A(f.p, f.cx, f.cy, f.di, c, L.ld);
    f.w[c] = w;
    v[0] = fma(w, f.p[c], v[0]);
  }
  grid_reduce<1>(v, rd, EpiMode<1>{rd.st, RED_STORE});
}

// tea_leaf_cg_calc_ur_kernel (cg_kernel.f90:198-304) for none / jac_diag; for jac_block the
// u/r update runs here (MODE 2) and z and r.z come from k_block_solve + k_dot.
template <int MODE>
__global__ void k_cg_calc_ur(Fields f, Layout L, double alpha, Reduce rd) {
  double v[1] = {0.0};
  FOR_ROWS(L) {
    if (j > L.nx) continue;
    const long long c = L.at(j, k);
    f.u[c] = fma(alpha, f.p[c], f.u[c]);
    const double r = fma(-alpha, f.w[c], f.r[c]);
    f.r[c] = r;
    if (MODE == 0) v[0] = fma(r, r, v[0]);
    if (MODE == 1) {
      const double z = f.mi[c] * r;
      f.z[c] = z;
      v[0] = fma(r, z, v[0]);
    }
  }
  if (MODE != 2) grid_reduce<1>(v, rd, EpiMode<1>{rd.st, RED_STORE});
}

// tea_leaf_cg_calc_p_kernel (cg_kernel.f90:306-347)
__global__ void k_cg_calc_p(Fields f, Layout L, double beta, int use_z) {
  FOR_ROWS(L) {
    if (j > L.nx) continue;
    const long long c = L.at(j, k);
    f.p[c] = fma(beta, f.p[c], use_z ? f.z[c] : f.r[c]);
  }
}

// tea_leaf_kernel_cheby_init (cheby_kernel.f90:30-109), phase 1: w = A u, r = u0 - w
__global__ void k_cheby_wr(Fields f, Layout L) {
  FOR_ROWS(L) {
    if (j > L.nx) continue;
    const long long c = L.at(j, k);
    const double w = apply_A(f.u, f.cx, f.cy, f.di, c, L.ld);
    f.w[c] = w;
    f.r[c] = f.u0[c] - w;
  }
}
// phase 2 (init): p = (r|z)/theta, u += p
__global__ void k_cheby_init_pu(Fields f, Layout L, double theta, int use_z) {
  FOR_ROWS(L) {
    if (j > L.nx) continue;
    const long long c = L.at(j, k);
    const double p = (use_z ? f.z[c] : f.r[c]) / theta;
    f.p[c] = p;
    f.u[c] = f.u[c] + p;
  }
}
// phase 2 (iterate, cheby_kernel.f90:175-197): p = a*p + b*(r|z), u += p
__global__ void k_cheby_iter_pu(Fields f, Layout L, double a, double b, int use_z) {
  FOR_ROWS(L) {
    if (j > L.nx) continue;
    const long long c = L.at(j, k);
    const double p = fma(a, f.p[c], b * (use_z ? f.z[c] : f.r[c]));
    f.p[c] = p;
    f.u[c] = f.u[c] + p;
  }
}

// tea_leaf_kernel_ppcg_init_sd (ppcg_kernel.f90:31-88)
__global__ void k_ppcg_init_sd(Fields f, Layout L, double theta_r, int use_z) {
  FOR_ROWS(L) {
    if (j > L.nx) continue;
    const long long c = L.at(j, k);
    const double sd = (use_z ? f.z[c] : f.r[c]) * theta_r;
    f.sd[c] = sd;
    f.rtemp[c] = f.r[c];
    f.utemp[c] = sd;
  }
}

// tea_leaf_ppcg_init_kernel (ppcg_kernel.f90:90-201) after any preconditioner application.
__global__ void k_ppcg_init(Fields f, Layout L, int step, int pz, int pr, Reduce rd, int mode) {
  // pz: p = z (step 1/3 with precond or ppcg_active at step 3); pr: p = r (step 1, no precond)
  double v[1] = {0.0};
  FOR_ROWS(L) {
    if (j > L.nx) continue;
    const long long c = L.at(j, k);
    double p = f.p[c];
    if (step == 1) {
      p = 0.0;
      f.z[c] = (pz ? f.z[c] : 0.0);
    } else if (step == 3) {
      p = 0.0;
    }
    if (pz) p = f.z[c];
    if (pr) p = f.r[c];
    f.p[c] = p;
    v[0] = fma(f.r[c], p, v[0]);
  }
  if (step != 2) grid_reduce<1>(v, rd, EpiMode<1>{rd.st, mode});
}

// tea_leaf_kernel_ppcg_inner (ppcg_kernel.f90:204-310), phase 1: rtemp -= A sd
__global__ void k_ppcg_inner_r(Fields f, Layout L) {
  FOR_ROWS(L) {
    if (j > L.nx) continue;
    const long long c = L.at(j, k);
    f.rtemp[c] = f.rtemp[c] - apply_A(f.sd, f.cx, f.cy, f.di, c, L.ld);
  }
}
// phase 2: sd = a*sd + b*(rtemp | Mi*rtemp | z), utemp += sd
__global__ void k_ppcg_inner_s(Fields f, Layout L, double a, double b, int precond) {
  FOR_ROWS(L) {
    if (j > L.nx) continue;
    const long long c = L.at(j, k);
    const double src = precond == 2 ? f.mi[c] * f.rtemp[c] : (precond == 3 ? f.z[c] : f.rtemp[c]);
    const double sd = fma(a, f.sd[c], b * src);
    f.sd[c] = sd;
    f.utemp[c] = f.utemp[c] + sd;
  }
}

// tea_leaf_jacobi_solve_kernel (jacobi_kernel.f90:26-77), un = r (copied first); off-domain
// neighbours of un read its halo, which the reference never writes (zero).
__global__ void k_jacobi(Fields f, Layout L, Reduce rd, double rx, double ry) {
  double v[1] = {0.0};
  FOR_ROWS(L) {
    if (j > L.nx) continue;
    const long long c = L.at(j, k);
    const double* un = f.r;
    const double u = jacobi_cell(f.u0[c], f.kx[c], f.kx[c + 1], f.ky[c], f.ky[c + L.ld], un[c - 1], un[c + 1],
                                 un[c - L.ld], un[c + L.ld], f.jden[c], f.jinv[c], rx, ry);
    f.u[c] = u;
    v[0] += fabs(u - un[c]);
  }
  grid_reduce<1>(v, rd, EpiMode<1>{rd.st, RED_STORE});
}

// the Jacobi denominator (jacobi_kernel.f90:67-69, exact operation order) and its reciprocal
__global__ void k_jacobi_den(Fields f, Layout L, Geometry g) {
  FOR_ROWS(L) {
    if (j > L.nx) continue;
    const long long c = L.at(j, k);
    const double den = __dadd_rn(__dadd_rn(1.0, __dmul_rn(g.rx, __dadd_rn(f.kx[c], f.kx[c + 1]))),
                                 __dmul_rn(g.ry, __dadd_rn(f.ky[c], f.ky[c + L.ld])));
    f.jden[c] = den;
    f.jinv[c] = __ddiv_rn(1.0, den);
  }
}

}  // namespace

long long& launch_counter() {
  static thread_local long long n = 0;
  return n;
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
void launch_init_faces(const Fields& f, const Layout& L, const Geometry& g, cudaStream_t s) {
  dim3 grid((L.nx + 1 + TB - 1) / TB, L.ny + 1 > 65535 ? 65535 : L.ny + 1);
  { ++launch_counter(); k_init_faces<<<grid, TB, 0, s>>>(f, L, g); }
}
void launch_init_cells(const Fields& f, const Layout& L, const Geometry& g, bool with_residual, cudaStream_t s) {
  { ++launch_counter(); k_init_cells<<<row_grid(L, false), TB, 0, s>>>(f, L, g); }
  if (g.precond == 3) launch_block_init(f, L, g, s);
  if (with_residual) { ++launch_counter(); k_init_residual<<<row_grid(L, false), TB, 0, s>>>(f, L); }
}
void launch_init_state(const Fields& f, const Layout& L, cudaStream_t s) {
  { ++launch_counter(); k_init_state<<<row_grid(L, false), TB, 0, s>>>(f, L); }
}
void launch_block_init(const Fields& f, const Layout& L, const Geometry& g, cudaStream_t s) {
  dim3 grid((L.nx + TB - 1) / TB, (L.ny + 3) / 4);
  { ++launch_counter(); k_block_init<<<grid, TB, 0, s>>>(f, L, g); }
}
void launch_generate(const Fields& f, const Layout& L, int nstates, const double* states, double xmin, double ymin,
                     double dx, double dy, cudaStream_t s) {
  dim3 grid((L.nx + 2 + TB - 1) / TB, L.ny + 2 > 65535 ? 65535 : L.ny + 2);
  { ++launch_counter(); k_generate<<<grid, TB, 0, s>>>(f, L, nstates, states, xmin, ymin, dx, dy); }
}
void launch_field_summary(const Fields& f, const Layout& L, double cell_vol, const Reduce& rd, cudaStream_t s) {
  { ++launch_counter(); k_field_summary<<<row_grid(L, true), TB, 0, s>>>(f, L, cell_vol, rd); }
}
void launch_update_halo(double* const* fields, int nfields, const Layout& L, cudaStream_t s) {
  { ++launch_counter(); k_halo_lr<<<(L.ny + 2 + TB - 1) / TB, TB, 0, s>>>(fields, nfields, L); }
  { ++launch_counter(); k_halo_bt<<<(L.nx + 2 + TB - 1) / TB, TB, 0, s>>>(fields, nfields, L); }
}
void launch_unpack(double* dst, const double* src, long long ld, const Layout& L, cudaStream_t s) {
  { ++launch_counter(); k_unpack<<<row_grid(L, false), TB, 0, s>>>(dst, src, ld, L); }
}
void launch_pack(double* dst, long long ld, const double* src, const Layout& L, cudaStream_t s) {
  { ++launch_counter(); k_pack<<<row_grid(L, false), TB, 0, s>>>(dst, ld, src, L); }
}
void launch_copy_interior(double* dst, const double* src, const Layout& L, cudaStream_t s) {
  { ++launch_counter(); k_copy_interior<<<row_grid(L, false), TB, 0, s>>>(dst, src, L); }
}
void launch_copy_all(double* dst, const double* src, const Layout& L, cudaStream_t s) {
  cudaMemcpyAsync(dst, src, (size_t)L.elems() * sizeof(double), cudaMemcpyDeviceToDevice, s);
}
void launch_residual(const Fields& f, const Layout& L, const Reduce* rd, int mode, cudaStream_t s) {
  if (rd)
    { ++launch_counter(); k_residual<true><<<row_grid(L, true), TB, 0, s>>>(f, L, *rd, mode); }
  else
    { ++launch_counter(); k_residual<false><<<row_grid(L, false), TB, 0, s>>>(f, L, Reduce{}, mode); }
}
void launch_norm2(const double* a, const Layout& L, const Reduce& rd, int mode, cudaStream_t s) {
  { ++launch_counter(); k_norm2<<<row_grid(L, true), TB, 0, s>>>(a, L, rd, mode); }
}
void launch_finalise(const Fields& f, const Layout& L, cudaStream_t s) {
  { ++launch_counter(); k_finalise<<<row_grid(L, false), TB, 0, s>>>(f, L); }
}
void launch_precond(const Fields& f, const Layout& L, const Geometry& g, const double* src, double* dst,
                    cudaStream_t s) {
  if (g.precond == 3) {
    dim3 grid((L.nx + TB - 1) / TB, (L.ny + 3) / 4);
    { ++launch_counter(); k_block_solve<<<grid, TB, 0, s>>>(f, L, g, src, dst); }
  } else if (g.precond == 2) {
    { ++launch_counter(); k_diag_solve<<<row_grid(L, false), TB, 0, s>>>(L, f.mi, src, dst); }
  }
}
void launch_residual_cg_init(const Fields& f, const Layout& L, const Geometry& g, const Reduce& rd, cudaStream_t s) {
  if (g.precond == 2)
    { ++launch_counter(); k_residual_cg_init<true><<<row_grid(L, true), TB, 0, s>>>(f, L, rd); }
  else
    { ++launch_counter(); k_residual_cg_init<false><<<row_grid(L, true), TB, 0, s>>>(f, L, rd); }
}
void launch_finalise_summary(const Fields& f, const Layout& L, double cell_vol, const Reduce& rd, LoopState* flush_st,
                             cudaStream_t s) {
  { ++launch_counter(); k_finalise_summary<<<row_grid(L, true), TB, 0, s>>>(f, L, cell_vol, rd, flush_st); }
  if (flush_st) cudaMemsetAsync(&flush_st->u_pending, 0, sizeof(int), s);
}
void launch_finalise_flush(const Fields& f, const Layout& L, LoopState* st, cudaStream_t s) {
  { ++launch_counter(); k_finalise_flush<<<row_grid(L, false), TB, 0, s>>>(f, L, st); }
  cudaMemsetAsync(&st->u_pending, 0, sizeof(int), s);
}
void launch_cg_init(const Fields& f, const Layout& L, const Geometry& g, const Reduce& rd, int mode, cudaStream_t s) {
  if (g.precond != 1) launch_precond(f, L, g, f.r, f.z, s);
  { ++launch_counter(); k_cg_init<<<row_grid(L, true), TB, 0, s>>>(f, L, g.precond, rd, mode); }
}
void launch_cg_calc_w(const Fields& f, const Layout& L, const Reduce& rd, cudaStream_t s) {
  { ++launch_counter(); k_cg_calc_w<<<row_grid(L, true), TB, 0, s>>>(f, L, rd); }
}
void launch_cg_calc_ur(const Fields& f, const Layout& L, const Geometry& g, double alpha, const Reduce& rd,
                       cudaStream_t s) {
  if (g.precond == 3) {
    { ++launch_counter(); k_cg_calc_ur<2><<<row_grid(L, true), TB, 0, s>>>(f, L, alpha, rd); }
    launch_precond(f, L, g, f.r, f.z, s);
    launch_dot(f.r, f.z, nullptr, L, rd, RED_STORE, s);
  } else if (g.precond == 2) {
    { ++launch_counter(); k_cg_calc_ur<1><<<row_grid(L, true), TB, 0, s>>>(f, L, alpha, rd); }
  } else {
    { ++launch_counter(); k_cg_calc_ur<0><<<row_grid(L, true), TB, 0, s>>>(f, L, alpha, rd); }
  }
}
void launch_cg_calc_p(const Fields& f, const Layout& L, double beta, bool use_z, cudaStream_t s) {
  { ++launch_counter(); k_cg_calc_p<<<row_grid(L, false), TB, 0, s>>>(f, L, beta, use_z ? 1 : 0); }
}
void launch_cheby_init(const Fields& f, const Layout& L, const Geometry& g, double theta, cudaStream_t s) {
  { ++launch_counter(); k_cheby_wr<<<row_grid(L, false), TB, 0, s>>>(f, L); }
  if (g.precond != 1) launch_precond(f, L, g, f.r, f.z, s);
  { ++launch_counter(); k_cheby_init_pu<<<row_grid(L, false), TB, 0, s>>>(f, L, theta, g.precond != 1); }
}
void launch_cheby_wr(const Fields& f, const Layout& L, cudaStream_t s) {
  { ++launch_counter(); k_cheby_wr<<<row_grid(L, false), TB, 0, s>>>(f, L); }
}
void launch_cheby_iterate(const Fields& f, const Layout& L, const Geometry& g, double a, double b, cudaStream_t s) {
  { ++launch_counter(); k_cheby_wr<<<row_grid(L, false), TB, 0, s>>>(f, L); }
  if (g.precond != 1) launch_precond(f, L, g, f.r, f.z, s);
  { ++launch_counter(); k_cheby_iter_pu<<<row_grid(L, false), TB, 0, s>>>(f, L, a, b, g.precond != 1); }
}
void launch_ppcg_init_sd(const Fields& f, const Layout& L, const Geometry& g, double theta, cudaStream_t s) {
  { ++launch_counter(); k_ppcg_init_sd<<<row_grid(L, false), TB, 0, s>>>(f, L, 1.0 / theta, g.precond != 1); }
}
void launch_ppcg_init(const Fields& f, const Layout& L, const Geometry& g, int step, bool ppcg_active,
                      const Reduce& rd, int mode, cudaStream_t s) {
  const bool pre = g.precond != 1 || (ppcg_active && step == 3);
  if (pre && (step == 1 || step == 2) && g.precond != 1) launch_precond(f, L, g, f.r, f.z, s);
  const int pz = pre && (step == 1 || step == 3);
  const int pr = !pre && step == 1;
  { ++launch_counter(); k_ppcg_init<<<row_grid(L, step != 2), TB, 0, s>>>(f, L, step, pz, pr, rd, mode); }
}
void launch_ppcg_inner(const Fields& f, const Layout& L, const Geometry& g, double a, double b, cudaStream_t s) {
  { ++launch_counter(); k_ppcg_inner_r<<<row_grid(L, false), TB, 0, s>>>(f, L); }
  if (g.precond == 3) launch_precond(f, L, g, f.rtemp, f.z, s);
  { ++launch_counter(); k_ppcg_inner_s<<<row_grid(L, false), TB, 0, s>>>(f, L, a, b, g.precond); }
}
void launch_dot(const double* a, const double* b, const double* bminus, const Layout& L, const Reduce& rd, int mode,
                cudaStream_t s) {
  { ++launch_counter(); k_dot<<<row_grid(L, true), TB, 0, s>>>(a, b, bminus, L, rd, mode); }
}
void launch_jacobi(const Fields& f, const Layout& L, const Geometry& g, const Reduce& rd, cudaStream_t s) {
  launch_copy_interior(f.r, f.u, L, s);
  { ++launch_counter(); k_jacobi<<<row_grid(L, true), TB, 0, s>>>(f, L, rd, g.rx, g.ry); }
}
void launch_jacobi_denominator(const Fields& f, const Layout& L, const Geometry& g, cudaStream_t s) {
  { ++launch_counter(); k_jacobi_den<<<row_grid(L, false), TB, 0, s>>>(f, L, g); }
}

}  // namespace tl
