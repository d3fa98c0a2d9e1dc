// tl_device.cuh -- device-side layout, solver state and reduction helpers shared by the
// TeaLeaf GB300 kernels.
//
// Field layout in HBM: every field is a (y_cells + 2) x ld array of FP64, x fastest.
// Row 0 and row y_cells+1 are the bottom/top halo rows; in each row the interior cell
// j = 1 sits at column XOFF, so interior rows start on a 128-byte boundary and ld is a
// multiple of 16 doubles.  Column XOFF-1 is the left halo cell, column XOFF+x_cells the
// right one.  The one-cell halo holds the reference's reflective-boundary copies
// (update_halo_kernel.f90:136-195); without reflective_boundary it stays zero and the
// boundary face coefficients are zero, so halo values never reach the operator.
#pragma once

#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>

#include "tl_fp64emu.cuh"

namespace tl {

constexpr int XOFF = 16;  // column of interior cell j = 1

struct Layout {
  int nx, ny;  // interior cells
  int ld;      // row stride (doubles)
  __host__ __device__ __forceinline__ long long at(int j, int k) const {
    return (long long)k * ld + (XOFF - 1) + j;
  }
  __host__ __device__ __forceinline__ long long elems() const { return (long long)(ny + 2) * ld; }
};

// Solver fields.  cx = rx*Kx and cy = ry*Ky are the face coefficients pre-scaled once per
// solve; kx/ky keep the reference's unscaled values.  p2 is the ping-pong partner of p in
// the fused CG loop; u1 is the partner of u for kernels that read u's neighbours while
// producing a new u (Chebyshev, Jacobi); sd1 is the partner of sd for the PPCG inner
// sweeps; jden = the Jacobi denominator, jinv = RN(1/jden).
struct Fields {
  double *density, *energy1, *u, *u0, *r, *w, *p, *p2, *kx, *ky, *cx, *cy, *di, *z, *mi, *sd, *utemp, *rtemp,
      *r_store, *cp, *bfp, *u1, *sd1, *jinv, *jden;
};

// One Jacobi update (tea_leaf_jacobi_kernel.f90:64-68) with the reference's bits: every
// product and sum in the reference's order, rounded on its own (no contraction), and the
// quotient num/den correctly rounded from the stored y = RN(1/den) by one remainder
// correction, q = RN(num y), q + (num - den q) y (P. Markstein, "Computation of elementary
// functions on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1), 1990): three
// FP64 operations instead of a division.  kx0/kx1 are Kx(j)/Kx(j+1), ky0/ky1 Ky(k)/Ky(k+1).
// Bit i of INT computes the i-th of the seven products (kx1 ur, kx0 ul, rx (..), ky1 ut,
// ky0 ub, ry (..), num y) on the integer pipes (dmul_int: the same bits).
template <int INT = 0>
__device__ __forceinline__ double jacobi_cell(double u0, double kx0, double kx1, double ky0, double ky1, double ul,
                                              double ur, double ub, double ut, double den, double y, double rx,
                                              double ry) {
  auto mul = [](auto bit, double a, double b) { return (INT & decltype(bit)::value) ? dmul_int(a, b) : __dmul_rn(a, b); };
  using B0 = std::integral_constant<int, 1>;
  using B1 = std::integral_constant<int, 2>;
  using B2 = std::integral_constant<int, 4>;
  using B3 = std::integral_constant<int, 8>;
  using B4 = std::integral_constant<int, 16>;
  using B5 = std::integral_constant<int, 32>;
  using B6 = std::integral_constant<int, 64>;
  const double sx = mul(B2{}, rx, __dadd_rn(mul(B0{}, kx1, ur), mul(B1{}, kx0, ul)));
  const double sy = mul(B5{}, ry, __dadd_rn(mul(B3{}, ky1, ut), mul(B4{}, ky0, ub)));
  const double num = __dadd_rn(__dadd_rn(u0, sx), sy);
  const double q = mul(B6{}, num, y);
  return __fma_rn(__fma_rn(-q, den, num), y, q);
}

// Exit / stop codes written by the device epilogues.
enum : int {
  RUN = 0,
  EXIT_CONVERGED = 1,
  EXIT_BREAKDOWN = 2,
  EXIT_MAX_ITERS = 3,
  STOP_SWITCH = 4,  // CG presteps done: host computes eigenvalues / coefficients
  EXIT_TIMEOUT = 5, // a bounded grid-barrier wait of the persistent CG kernel expired
};

// Device-resident state of one tea_leaf() solve (tea_solve.f90:42-68).  Written only by
// the single last-arriving CTA of a reducing kernel (or by the host between launches).
struct LoopState {
  double red[4];  // raw results of the last reduction (per-kernel entry points)
  double rro, pw, rrn, alpha, beta;
  double error, old_error, initial_residual, eps;
  double epslim;
  double theta;
  int n;           // tea_leaf loop index of the iteration about to run / running
  int max_iters;
  int status;      // RUN or an EXIT_* / STOP_* code
  int n_exit;
  int p_pending;   // 1: the next CG matvec first applies p = src + beta*p
  int presteps;
  int first;       // reference 'first' flag (eigenvalues not yet estimated)
  int use_ppcg;    // switch rule for PPCG (tea_solve.f90:164)
  int cheby_step;  // cheby_calc_steps
  int est_itc;
  int cg_calc_steps;
  int check_switch;  // evaluate the CG->Chebyshev/PPCG switch in the CG epilogue
  // Deferred solution update u += u_alpha * P[u_psel] (cg_kernel.f90:286-291 of the previous
  // iteration): applied by the next matvec sweep, which reads that p anyway, or by the
  // flush kernel when the CG phase ends.  The same operands, so the same bits.
  int u_pending;
  int u_psel;
  double u_alpha;
};

// Word of the context's counter buffer that a blocked FP32 sweep of the precision form sets
// when a bounded wait for a staged row expired (1) or its shared memory was misaligned (2):
// MixFields::err points here, and the PPCG loop's epilogue turns it into EXIT_TIMEOUT.
constexpr int MIX_ERR_WORD = 8;

// Launch-independent pointers handed to every kernel that reduces.
struct Reduce {
  double* partials;    // [gridDim.x * gridDim.y][NV]
  unsigned* counter;   // arrival ticket, reset to 0 by the last CTA
  LoopState* st;
  double* hist_a;      // cg_alphas(1:max_iters), 1-based
  double* hist_b;      // cg_betas
  const double* ch_a;  // Chebyshev / PPCG coefficients, 1-based
  const double* ch_b;
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Largest CTA of a kernel that reduces (block_sum's shared scratch is sized for it).
constexpr int MAX_REDUCE_THREADS = 256;

// Block sum of NV values in fixed order; result valid in thread 0.  scratch: NV *
// MAX_REDUCE_THREADS doubles.  Every thread parks its values in shared memory and the first warp
// adds them (a column sum, then a shuffle tree): blockDim/32 + 4 FP64 additions per value, in
// one warp.  A shuffle tree in every warp would cost 5 per warp -- FP64 instructions are what
// the reducing sweeps are short of on this GPU.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* scratch) {
  const int t = threadIdx.x, nt = blockDim.x;
  __syncthreads();  // an earlier use of scratch in this CTA is complete
#pragma unroll
  for (int i = 0; i < NV; ++i) scratch[i * MAX_REDUCE_THREADS + t] = v[i];
  __syncthreads();
  if (t < 32) {
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      const double* s = scratch + i * MAX_REDUCE_THREADS;
      double x = t < nt ? s[t] : 0.0;
      for (int k = t + 32; k < nt; k += 32) x += s[k];
      v[i] = warp_sum(x);
    }
  }
}

// Two-level deterministic grid reduction: every CTA publishes its block sum; the CTA
// that arrives last sums all partials in block order (thread t takes t, t+T, ...; then a
// fixed tree), runs epi(total) in thread 0 and re-arms the ticket.  The result does not
// depend on which CTA arrives last.
// scratch: MAX_REDUCE_THREADS * NV doubles of shared memory the block no longer uses otherwise
// (the caller has synchronised the block after its last use)
template <int NV, typename Epi>
__device__ __forceinline__ void grid_reduce_in(double (&v)[NV], const Reduce& rd, Epi epi, double* scratch) {
  __shared__ int is_last;
  block_sum<NV>(v, scratch);
  const unsigned nblk = gridDim.x * gridDim.y;
  const unsigned bid = blockIdx.y * gridDim.x + blockIdx.x;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int i = 0; i < NV; ++i) rd.partials[(size_t)bid * NV + i] = v[i];
    __threadfence();
    const unsigned ticket = atomicAdd(rd.counter, 1u);
    is_last = (ticket == nblk - 1);
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  double acc[NV];
#pragma unroll
  for (int i = 0; i < NV; ++i) acc[i] = 0.0;
  for (unsigned b = threadIdx.x; b < nblk; b += blockDim.x) {
#pragma unroll
    for (int i = 0; i < NV; ++i) acc[i] += __ldcg(rd.partials + (size_t)b * NV + i);
  }
  block_sum<NV>(acc, scratch);
  if (threadIdx.x == 0) {
    epi(acc);
    *rd.counter = 0u;
    __threadfence();
  }
}

template <int NV, typename Epi>
__device__ __forceinline__ void grid_reduce(double (&v)[NV], const Reduce& rd, Epi epi) {
  __shared__ double scratch[MAX_REDUCE_THREADS * NV];
  grid_reduce_in<NV>(v, rd, epi, scratch);
}

}  // namespace tl
