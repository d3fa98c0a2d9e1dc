// tl_mixed_poly.cu -- FP32 polynomial sweeps of the precision form of the Chebyshev and PPCG
// solvers: the PPCG inner Chebyshev steps (the preconditioner z = p(A) r) and the Chebyshev
// iteration on a correction inside FP64 iterative refinement.  The FP64 outer parts (PPCG's
// w = A p, u/r updates, dot products, p update; Chebyshev's residual u0 - A u and u += d) are
// the FP64 kernels of tl_kernels.cu and tl_mixed.cu.
//
// Fields (MixFields, FP32, the context layout): cx, cy, di are the FP32 operator (k_mix_prep);
// PPCG uses r = rtemp, p / p2 = sd (ping-pong), w = utemp; Chebyshev uses r = its right-hand
// side, p = its direction, d / p2 = the correction (ping-pong, ending in d).  Off-domain
// neighbours: see apply_a32 (with zero boundary coefficients either choice gives the same).
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>

#include "tl_kernels.cuh"

namespace tl {

namespace {

constexpr int PT = 256;

inline dim3 poly_grid(const Layout& L) {
  const int gy = L.ny < 4096 ? L.ny : 4096;
  return dim3((L.nx + PT - 1) / PT, gy);
}

// MIRROR: off-domain neighbours take the cell's own value (PPCG's sd, whose halo the reference
// exchanges between inner steps); otherwise they are zero (Chebyshev's correction d: the
// reference does not exchange u's halo after the switch, so a correction leaves it unchanged).
template <bool MIRROR>
__device__ __forceinline__ float apply_a32(const float* __restrict__ v, const MixFields& m, long long c, int j, int k,
                                           const Layout& L) {
  const float vc = v[c];
  const float off = MIRROR ? vc : 0.f;
  const float vl = (j > 1) ? v[c - 1] : off;
  const float vr = (j < L.nx) ? v[c + 1] : off;
  const float vb = (k > 1) ? v[c - L.ld] : off;
  const float vt = (k < L.ny) ? v[c + L.ld] : off;
  float a = m.di[c] * vc;
  a = fmaf(-m.cy[c + L.ld], vt, a);
  a = fmaf(-m.cy[c], vb, a);
  a = fmaf(-m.cx[c + 1], vr, a);
  a = fmaf(-m.cx[c], vl, a);
  return a;
}

// The preconditioner's z of a residual value: Mi32 x with jac_diag (m.mi non-null), else x.
__device__ __forceinline__ float prec32(const MixFields& m, long long c, float x) { return m.mi ? m.mi[c] * x : x; }

// tea_leaf_kernel_ppcg_init_sd (tea_leaf_ppcg_kernel.f90:31-88) in FP32: rtemp = r, sd = z / theta
// (z = r, or Mi r with jac_diag; as z * (1/theta) in FP32: a per-cell FP64 division would make
// this copy FP64-bound), utemp = sd.
__global__ void k_poly_ppcg_init(const double* __restrict__ r, MixFields m, Layout L, float inv_theta) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (j > L.nx) return;
  for (int k = blockIdx.y + 1; k <= L.ny; k += gridDim.y) {
    const long long c = L.at(j, k);
    const float rv = (float)r[c];
    const float sd = prec32(m, c, rv) * inv_theta;
    m.r[c] = rv;
    m.p[c] = sd;
    m.w[c] = sd;
  }
}

// One inner step (tea_leaf_kernel_ppcg_inner, ppcg_kernel.f90:204-310) in FP32:
// rtemp -= A sd; sd' = a sd + b rtemp (b Mi rtemp with jac_diag); utemp += sd'.  z (nullable,
// FP64): z = utemp after the
// last step (tea_leaf_ppcg_update_z_kernel, :453-477).
__global__ void k_poly_ppcg_step(MixFields m, const float* __restrict__ sd_in, float* __restrict__ sd_out, Layout L,
                                 float a, float b, double* __restrict__ z) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (j > L.nx) return;
  for (int k = blockIdx.y + 1; k <= L.ny; k += gridDim.y) {
    const long long c = L.at(j, k);
    const float rt = m.r[c] - apply_a32<true>(sd_in, m, c, j, k, L);
    m.r[c] = rt;
    const float sd = fmaf(a, sd_in[c], b * prec32(m, c, rt));
    sd_out[c] = sd;
    const float ut = m.w[c] + sd;
    m.w[c] = ut;
    if (z) z[c] = (double)ut;
  }
}

// z = utemp (FP64) when the inner loop has no steps.
__global__ void k_poly_to_z(MixFields m, Layout L, double* __restrict__ z) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (j > L.nx) return;
  for (int k = blockIdx.y + 1; k <= L.ny; k += gridDim.y) {
    const long long c = L.at(j, k);
    z[c] = (double)m.w[c];
  }
}

// Chebyshev on A d = r from d = 0 (tea_leaf_kernel_cheby_init, tea_leaf_cheby_kernel.f90:30-109,
// with u = 0, u0 = r): p = z / theta (z = r, or Mi r with jac_diag), d = p.
__global__ void k_poly_cheby_start(MixFields m, float* __restrict__ d, Layout L, float inv_theta) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (j > L.nx) return;
  for (int k = blockIdx.y + 1; k <= L.ny; k += gridDim.y) {
    const long long c = L.at(j, k);
    const float p = prec32(m, c, m.r[c]) * inv_theta;
    m.p[c] = p;
    d[c] = p;
  }
}

// One Chebyshev iteration on the correction (tea_leaf_kernel_cheby_iterate, :111-200):
// res = r - A d; p = a p + b res (b Mi res with jac_diag); d' = d + p.
__global__ void k_poly_cheby_step(MixFields m, const float* __restrict__ d_in, float* __restrict__ d_out, Layout L,
                                  float a, float b) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (j > L.nx) return;
  for (int k = blockIdx.y + 1; k <= L.ny; k += gridDim.y) {
    const long long c = L.at(j, k);
    const float res = m.r[c] - apply_a32<false>(d_in, m, c, j, k, L);
    const float p = fmaf(a, m.p[c], b * prec32(m, c, res));
    m.p[c] = p;
    d_out[c] = d_in[c] + p;
  }
}

// Clear the correction buffers (m.d is read by the FP64 residual of u + d).
__global__ void k_poly_clear(MixFields m, Layout L) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (j > L.nx) return;
  for (int k = blockIdx.y + 1; k <= L.ny; k += gridDim.y) {
    const long long c = L.at(j, k);
    m.d[c] = 0.f;
    m.p2[c] = 0.f;
  }
}

// ---- temporal blocking: up to TB_S polynomial steps per sweep ----------------------------
// Each warp owns a strip of 32*CPL columns (CPL columns per lane: 2, with 8-byte accesses, or
// 4, with 16-byte accesses) with a TB_HX-column halo on each side, 32*CPL - 2*TB_HX output
// columns, and marches up a range of rows.  At march position m, level 0 loads row m and level
// t = 1..S computes step t at row m - t from level t-1's rows m-t-1 .. m-t+1 (a three-row
// register window per level) and level t-1's cell values of row m-t (its output one march
// position earlier).  Horizontal neighbours come from the adjacent lanes by shuffles.  Level
// 0's rows (coefficients and input state) are staged TB_P rows ahead into per-warp
// shared-memory rings by TMA tensor copies (or cp.async), so a march step does not wait for a
// load; every level reads the coefficients from the ring.  Warps never wait for one another.
// Level t is exact on local columns [t, 32*CPL-t): with S <= TB_HX the output columns are
// exact.  Every cell runs the one-step kernels' arithmetic in the same order, so S steps here
// give the bits of S one-step sweeps, whatever CPL.  Traffic per S steps: the state and the
// coefficients read once (x 32*CPL / output width, for the halo), the state written once.
// CPL 2 halves the register windows and the shared memory of a warp (more resident warps)
// for twice the halo overhead of CPL 4; CPL 4 is the faster (see POLY_CPL).  PRE (jac_diag):
// the preconditioner Mi32 is one more staged coefficient array, applied to the residual of
// every step (and of the start) as in the one-step kernels.
constexpr int TB_S = 4;      // steps per sweep at most
constexpr int TB_HX = 4;     // halo columns on each side of a warp strip
constexpr int TB_WARPS = 4;  // warps per CTA
constexpr int TB_P = 2;      // rows staged ahead by asynchronous copies
constexpr int TB_PF = 8;     // L2 prefetch distance in rows
constexpr unsigned FULL = 0xffffffffu;

template <int CPL>
struct TbGeom {
  static constexpr int SWX = 32 * CPL;        // strip width, halo included (the TMA box width)
  static constexpr int W = SWX - 2 * TB_HX;   // output columns per strip
};

enum { POLY_PPCG = 0, POLY_CHEBY = 1 };

struct PolyArgs {
  MixFields m;
  Layout L;
  const float* x_in;   // the stencil variable: sd (PPCG) | d (Chebyshev)
  float* x_out;
  const float* c1_in;  // rtemp (PPCG) | p (Chebyshev)
  float* c1_out;
  const float* c2_in;  // utemp (PPCG)
  float* c2_out;
  const double* r64;   // PPCG first sweep: level 0 is init_sd of this FP64 residual
  double* z;           // PPCG last sweep: z = utemp (FP64) is its only output
  float inv_theta;
  int first;           // level 0 synthesised: PPCG init_sd from r64, Chebyshev start from m.r
  int rows, nstrips, ntasks;
  int tx, t1, t2;      // TMA: indices in PolyMaps of the maps of x_in, c1_in, c2_in
  int hold_row;        // test of the bounded wait: task 0 arms this row's mbarrier without issuing
                       // its copies, so the wait for it runs out (-1: off)
  float ca[TB_S], cb[TB_S];
};

// Tensor maps (TMA descriptors) of the fields a blocked sweep reads: each a 2-D view
// (ld x (ny+2)) with a (32*CPL)-element by 1-row box.
enum { PM_P = 0, PM_P2, PM_R, PM_W, PM_D, PM_E, PM_CX, PM_CY, PM_DI, PM_MI, PM_R64, PM_N };
struct PolyMaps {
  CUtensorMap t[PM_N];
};

__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// columns j+i with lo <= j+i <= hi: one vector store when all CPL lie there
template <int CPL>
__device__ __forceinline__ void store_cols(float* __restrict__ p, long long c, const float (&v)[CPL], int lo, int hi,
                                           int j) {
  if (j >= lo && j + CPL - 1 <= hi) {
    if constexpr (CPL == 4)
      *reinterpret_cast<float4*>(p + c) = make_float4(v[0], v[1], v[2], v[3]);
    else
      *reinterpret_cast<float2*>(p + c) = make_float2(v[0], v[1]);
  } else {
#pragma unroll
    for (int i = 0; i < CPL; ++i)
      if (j + i >= lo && j + i <= hi) p[c + i] = v[i];
  }
}

// Per-warp shared memory of the blocked sweep: a ring of RING coefficient rows (di, cx, cy,
// Chebyshev's right-hand side, and Mi with jac_diag; CP floats per array row) and a ring of
// TB_P+1 input-state rows.
// With TMA the array rows are 32*CPL floats apart (every TMA destination 128-byte aligned; the
// lane that reads column j+CPL past its warp's strip is a halo lane) and TB_P+1 mbarriers follow.
enum { CA_DI = 0, CA_CX = 1, CA_CY = 2, CA_RHS = 3 };  // coefficient arrays; Mi follows the last
template <int MODE, int S, bool TMA, int CPL, bool PRE>
struct TbSmem {
  static constexpr int SWX = TbGeom<CPL>::SWX;
  static constexpr int NC = (MODE == POLY_PPCG ? 3 : 4) + (PRE ? 1 : 0);
  static constexpr int MI = NC - 1;  // Mi's array (PRE only)
  static constexpr int RING = S + 1 + TB_P;
  static constexpr int CP = TMA ? SWX : SWX + 4;                 // floats per coefficient array row
  static constexpr int SSLOT = (MODE == POLY_PPCG ? 3 : 2) * SWX;  // floats (PPCG: or SWX doubles)
  static constexpr int BAR = TMA ? 32 : 0;                        // floats: the mbarriers (128 B)
  static constexpr int WARP_FLOATS = RING * NC * CP + (TB_P + 1) * SSLOT + BAR;
  static constexpr int BYTES = TB_WARPS * WARP_FLOATS * 4;
};

constexpr unsigned long long TB_WAIT_LIMIT = 1ull << 24;  // polls of a staged row (>= 32 ns each)

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// bounded wait for the phase with the given parity to complete; false if it did not
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity) {
  const unsigned a = smem_u32(bar);
  for (unsigned long long i = 0; i < TB_WAIT_LIMIT; ++i) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    __nanosleep(32);
  }
  return false;
}
// one row box of a 2-D tensor map into shared memory, completing on bar
__device__ __forceinline__ void tma_row(void* dst, const CUtensorMap* map, int x, int y, unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

template <int BYTES>
__device__ __forceinline__ void cp_async(void* dst, const void* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  if constexpr (BYTES == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src));
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N)); }

// columns j .. j+CPL-1 of a float row into shared memory: one asynchronous copy when all lie in
// [lo, hi], else guarded loads (zero outside)
template <int CPL>
__device__ __forceinline__ void stage_cols(float* dst, const float* __restrict__ src, int j, int lo, int hi) {
  if (j >= lo && j + CPL - 1 <= hi) {
    cp_async<4 * CPL>(dst, src);
  } else {
#pragma unroll
    for (int i = 0; i < CPL; ++i) dst[i] = (j + i >= lo && j + i <= hi) ? __ldg(src + i) : 0.f;
  }
}
template <int CPL>
__device__ __forceinline__ void stage_cols_d(double* dst, const double* __restrict__ src, int j, int lo, int hi) {
  if (j >= lo && j + CPL - 1 <= hi) {
#pragma unroll
    for (int i = 0; i < CPL; i += 2) cp_async<16>(dst + i, src + i);
  } else {
#pragma unroll
    for (int i = 0; i < CPL; ++i) dst[i] = (j + i >= lo && j + i <= hi) ? __ldg(src + i) : 0.0;
  }
}

template <int MODE, int S, bool TMA, int CPL, bool PRE>
__global__ void __launch_bounds__(32 * TB_WARPS) k_poly_tb(PolyArgs a, const __grid_constant__ PolyMaps pm) {
  constexpr bool PPCG = MODE == POLY_PPCG;
  using SM = TbSmem<MODE, S, TMA, CPL, PRE>;
  constexpr int NC = SM::NC, RING = SM::RING, CP = SM::CP, SWX = SM::SWX, W = TbGeom<CPL>::W;
  const int lane = threadIdx.x & 31;
  const int task = blockIdx.x * TB_WARPS + (threadIdx.x >> 5);
  if (task >= a.ntasks) return;  // whole warps only
  // an earlier sweep of this solve gave up on a staged row: its results are void, and so would
  // this sweep's be; the solve reports TL_ERR_TIMEOUT
  if (*reinterpret_cast<volatile const unsigned*>(a.m.err) != 0u) return;
  const Layout L = a.L;
  const MixFields& m = a.m;
  const int x0 = 1 + (task % a.nstrips) * W;
  const int k0 = 1 + (task / a.nstrips) * a.rows;
  const int k1 = min(k0 + a.rows - 1, L.ny);
  const int j = x0 - TB_HX + CPL * lane;  // this lane's first column
  const int out0 = x0, out1 = min(x0 + W - 1, L.nx);
  const int lc = CPL * lane;
  extern __shared__ __align__(128) float tb_smem[];
  float* const wbase = tb_smem + (threadIdx.x >> 5) * SM::WARP_FLOATS;
  // ring slots: row r sits in coefficient slot (r - mstart) mod RING and state slot
  // (r - mstart) mod (TB_P+1); the march keeps the slots of row mm in running counters
  auto coef = [&](int slot, int arr) { return wbase + (slot * NC + arr) * CP; };
  auto state = [&](int slot, int arr) { return wbase + RING * NC * CP + slot * SM::SSLOT + arr * SWX; };
  constexpr int SR = TB_P + 1;
  unsigned long long* const bars =
      reinterpret_cast<unsigned long long*>(wbase + RING * NC * CP + SR * SM::SSLOT);  // TMA: one per state slot
  const int crow_max = min(L.ny + 1, k1 + S);  // coefficient rows (cy also of the boundary row ny+1)
  const int srow_max = min(L.ny, k1 + S);      // input-state rows
  const int tmx = (XOFF - 1) + (x0 - TB_HX);  // TMA: first element of the warp's strip in a row
  if (TMA) {
    if (smem_u32(tb_smem) & 127u) {  // TMA destinations must be 128-byte aligned
      if (lane == 0) atomicExch(a.m.err, 2u);
      return;
    }
    if (lane == 0)
      for (int b = 0; b < SR; ++b) mbar_init(&bars[b], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    __syncwarp();
  }
  // TMA: one lane arms the row's mbarrier with the byte count and issues the row's tensor copies
  // (columns past the field's rows read as zero); an empty row only arrives
  auto issue_row_tma = [&](int row, int cs, int ss) {
    if (lane != 0) return;
    constexpr unsigned RB = 4u * SWX;  // bytes of one float row box
    unsigned bytes = 0;
    if (row <= crow_max) bytes += (row <= L.ny ? NC : 1) * RB;
    if (row <= srow_max) bytes += a.first ? (PPCG ? 2 * RB : 0) : (PPCG ? 3 : 2) * RB;
    unsigned long long* bar = &bars[ss];
    if (bytes == 0) {
      mbar_arrive(bar);
      return;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the lanes' reads of these slots come first
    mbar_expect_tx(bar, bytes);
    if (row == a.hold_row && task == 0) return;  // the test's row: armed, never copied
    if (row <= crow_max) {
      tma_row(coef(cs, 2), &pm.t[PM_CY], tmx, row, bar);
      if (row <= L.ny) {
        tma_row(coef(cs, CA_DI), &pm.t[PM_DI], tmx, row, bar);
        tma_row(coef(cs, CA_CX), &pm.t[PM_CX], tmx, row, bar);
        if (!PPCG) tma_row(coef(cs, CA_RHS), &pm.t[PM_R], tmx, row, bar);
        if (PRE) tma_row(coef(cs, SM::MI), &pm.t[PM_MI], tmx, row, bar);
      }
    }
    if (row <= srow_max) {
      if (a.first) {
        if (PPCG) tma_row(state(ss, 0), &pm.t[PM_R64], tmx, row, bar);
      } else {
        tma_row(state(ss, 0), &pm.t[a.tx], tmx, row, bar);
        tma_row(state(ss, 1), &pm.t[a.t1], tmx, row, bar);
        if (PPCG) tma_row(state(ss, 2), &pm.t[a.t2], tmx, row, bar);
      }
    }
  };
  unsigned parity = 0;  // TMA: bit b = phase parity of mbarrier b's next completion
  bool stalled = false;
  // stage row `row` (coefficients and input state) into the rings; one commit group per row
  auto issue_row = [&](int row, int cs, int ss) {
    if (TMA) {
      issue_row_tma(row, cs, ss);
      return;
    }
    if (row <= crow_max) {
      const long long c = L.at(j, row);
      stage_cols<CPL>(coef(cs, 2) + lc, m.cy + c, j, 1, L.nx);
      if (row <= L.ny) {
        stage_cols<CPL>(coef(cs, CA_DI) + lc, m.di + c, j, 1, L.nx);
        stage_cols<CPL>(coef(cs, CA_CX) + lc, m.cx + c, j, 1, L.nx + 1);
        if (!PPCG) stage_cols<CPL>(coef(cs, CA_RHS) + lc, m.r + c, j, 1, L.nx);
        if (PRE) stage_cols<CPL>(coef(cs, SM::MI) + lc, m.mi + c, j, 1, L.nx);
      }
    }
    if (row <= srow_max) {
      const long long c = L.at(j, row);
      if (a.first) {
        if (PPCG) stage_cols_d<CPL>(reinterpret_cast<double*>(state(ss, 0)) + lc, a.r64 + c, j, 1, L.nx);
      } else {
        stage_cols<CPL>(state(ss, 0) + lc, a.x_in + c, j, 1, L.nx);
        stage_cols<CPL>(state(ss, 1) + lc, a.c1_in + c, j, 1, L.nx);
        if (PPCG) stage_cols<CPL>(state(ss, 2) + lc, a.c2_in + c, j, 1, L.nx);
      }
    }
    cp_async_commit();
  };
  float X[S][3][CPL];   // level t < S: stencil variable of rows (newest-2, newest-1, newest)
  float C1[S][2][CPL];  // level t < S: rtemp | p of rows (newest-1, newest)
  float C2[S][2][CPL];  // level t < S: utemp of rows (newest-1, newest)
#pragma unroll
  for (int t = 0; t < S; ++t)
#pragma unroll
    for (int i = 0; i < CPL; ++i) {
      X[t][0][i] = X[t][1][i] = X[t][2][i] = 0.f;
      C1[t][0][i] = C1[t][1][i] = C2[t][0][i] = C2[t][1][i] = 0.f;
    }
  const int mstart = max(1, k0 - S), mend = k1 + S;
#pragma unroll
  for (int r = 0; r < TB_P; ++r) issue_row(mstart + r, r % RING, r % SR);
  int cslot = 0, sslot = 0;  // slots of row mm
  for (int mm = mstart; mm <= mend; ++mm) {
    __syncwarp();  // every lane is done with the slots the next copies overwrite
    {
      int cs = cslot + TB_P, ss = sslot + TB_P;
      if (cs >= RING) cs -= RING;
      if (ss >= SR) ss -= SR;
      issue_row(mm + TB_P, cs, ss);
    }
    const int pf = mm + TB_PF;  // L2 prefetch further ahead, one lane per 32-float stretch
    if (pf <= srow_max && (lc & 31) == 0 && j >= 1 && j + CPL - 1 <= L.nx) {
      const long long c = L.at(j, pf);
      if (!a.first) {
        prefetch_l2(a.x_in + c);
        prefetch_l2(a.c1_in + c);
        if (PPCG) prefetch_l2(a.c2_in + c);
      } else if (PPCG) {
        prefetch_l2(a.r64 + c);
      }
      prefetch_l2(m.di + c);
      prefetch_l2(m.cx + c);
      prefetch_l2(m.cy + c);
      if (!PPCG) prefetch_l2(m.r + c);
      if (PRE) prefetch_l2(m.mi + c);
    }
    if (TMA) {
      // row mm has landed: lane 0 polls (bounded) and tells the warp, so the warp stays
      // converged whatever happens; each lane then observes the completed phase itself
      int ok = lane == 0 ? (int)mbar_wait(&bars[sslot], (parity >> sslot) & 1u) : 0;
      ok = __shfl_sync(FULL, ok, 0);
      if (!ok) {
        stalled = true;
        if (lane == 0) atomicExch(a.m.err, 1u);
        break;
      }
      mbar_wait(&bars[sslot], (parity >> sslot) & 1u);  // completes at the first poll
      parity ^= 1u << sslot;
    } else {
      cp_async_wait<TB_P>();  // row mm has landed
    }
    __syncwarp();
    // ---- level 0: the sweep's input at row mm ----
    float nx[CPL], n1[CPL], n2[CPL];
#pragma unroll
    for (int i = 0; i < CPL; ++i) nx[i] = n1[i] = n2[i] = 0.f;
    if (mm <= srow_max) {
      if (a.first) {
        const float* rm = coef(cslot, SM::MI) + lc;  // Mi of row mm (PRE)
        if (PPCG) {
          const double* rs = reinterpret_cast<const double*>(state(sslot, 0)) + lc;
#pragma unroll
          for (int i = 0; i < CPL; ++i) {
            const float rv = (float)rs[i];
            n1[i] = rv;
            nx[i] = (PRE ? rm[i] * rv : rv) * a.inv_theta;
            n2[i] = nx[i];
          }
        } else {
          const float* rs = coef(cslot, CA_RHS) + lc;
#pragma unroll
          for (int i = 0; i < CPL; ++i) {
            nx[i] = (PRE ? rm[i] * rs[i] : rs[i]) * a.inv_theta;
            n1[i] = nx[i];
          }
        }
      } else {
#pragma unroll
        for (int i = 0; i < CPL; ++i) {
          nx[i] = state(sslot, 0)[lc + i];
          n1[i] = state(sslot, 1)[lc + i];
          if (PPCG) n2[i] = state(sslot, 2)[lc + i];
        }
      }
    }
#pragma unroll
    for (int i = 0; i < CPL; ++i) {
      X[0][0][i] = X[0][1][i];
      X[0][1][i] = X[0][2][i];
      X[0][2][i] = nx[i];
      C1[0][0][i] = C1[0][1][i];
      C1[0][1][i] = n1[i];
      C2[0][0][i] = C2[0][1][i];
      C2[0][1][i] = n2[i];
    }
    // ---- levels 1..S: step t at row mm - t ----
#pragma unroll
    for (int t = 1; t <= S; ++t) {
      const int q = mm - t;
      const bool act = q >= max(1, k0 - (S - t)) && q <= min(L.ny, k1 + (S - t));  // uniform per warp
      float ox[CPL], o1[CPL], o2[CPL];
#pragma unroll
      for (int i = 0; i < CPL; ++i) ox[i] = o1[i] = o2[i] = 0.f;
      if (act) {
        int qs = cslot - t, qs1 = cslot - t + 1;  // slots of rows q and q+1
        if (qs < 0) qs += RING;
        if (qs1 < 0) qs1 += RING;
        const float* rdi = coef(qs, CA_DI) + lc;
        const float* rcx = coef(qs, CA_CX) + lc;
        const float* rcy = coef(qs, CA_CY) + lc;
        const float* rcy1 = coef(qs1, CA_CY) + lc;
        float di[CPL], cxv[CPL], cyb[CPL], cyt[CPL], rhs[CPL], mi[CPL];
#pragma unroll
        for (int i = 0; i < CPL; ++i) {
          di[i] = rdi[i];
          cxv[i] = rcx[i];
          cyb[i] = rcy[i];
          cyt[i] = rcy1[i];
          rhs[i] = PPCG ? 0.f : coef(qs, CA_RHS)[lc + i];
          mi[i] = PRE ? coef(qs, SM::MI)[lc + i] : 1.f;
        }
        const float cxn = rcx[CPL];                                          // cx at column j+CPL
        const float left = __shfl_up_sync(FULL, X[t - 1][1][CPL - 1], 1);  // column j-1
        const float right = __shfl_down_sync(FULL, X[t - 1][1][0], 1);     // column j+CPL
#pragma unroll
        for (int i = 0; i < CPL; ++i) {
          const float vc = X[t - 1][1][i];
          const float off = PPCG ? vc : 0.f;  // mirror (PPCG's sd) or zero (Chebyshev's d)
          float vl = (i == 0) ? left : X[t - 1][1][i - 1];
          float vr = (i == CPL - 1) ? right : X[t - 1][1][i + 1];
          if (j + i == 1) vl = off;
          if (j + i == L.nx) vr = off;
          const float vb = (q > 1) ? X[t - 1][0][i] : off;
          const float vt = (q < L.ny) ? X[t - 1][2][i] : off;
          const float cr1 = (i == CPL - 1) ? cxn : cxv[i + 1];
          float av = di[i] * vc;
          av = fmaf(-cyt[i], vt, av);
          av = fmaf(-cyb[i], vb, av);
          av = fmaf(-cr1, vr, av);
          av = fmaf(-cxv[i], vl, av);
          if (PPCG) {
            const float rt = C1[t - 1][0][i] - av;
            const float sd = fmaf(a.ca[t - 1], vc, a.cb[t - 1] * (PRE ? mi[i] * rt : rt));
            o1[i] = rt;
            ox[i] = sd;
            o2[i] = C2[t - 1][0][i] + sd;
          } else {
            const float res = rhs[i] - av;
            const float pn = fmaf(a.ca[t - 1], C1[t - 1][0][i], a.cb[t - 1] * (PRE ? mi[i] * res : res));
            o1[i] = pn;
            ox[i] = vc + pn;
          }
        }
      }
      if (t < S) {
#pragma unroll
        for (int i = 0; i < CPL; ++i) {
          X[t][0][i] = X[t][1][i];
          X[t][1][i] = X[t][2][i];
          X[t][2][i] = ox[i];
          C1[t][0][i] = C1[t][1][i];
          C1[t][1][i] = o1[i];
          C2[t][0][i] = C2[t][1][i];
          C2[t][1][i] = o2[i];
        }
      } else if (act) {  // rows k0 .. k1 of the last level: the sweep's output
        const long long c = L.at(j, q);
        if (PPCG && a.z) {
#pragma unroll
          for (int i = 0; i < CPL; ++i)
            if (j + i >= out0 && j + i <= out1) a.z[c + i] = (double)o2[i];
        } else {
          store_cols<CPL>(a.x_out, c, ox, out0, out1, j);
          store_cols<CPL>(a.c1_out, c, o1, out0, out1, j);
          if (PPCG) store_cols<CPL>(a.c2_out, c, o2, out0, out1, j);
        }
      }
    }
    if (++cslot == RING) cslot = 0;
    if (++sslot == SR) sslot = 0;
  }
  if (TMA) {
    // every copy issued was for a row the march waited for, unless a wait expired: then give
    // the others in flight a bounded time to land before the warp's shared memory is released
    if (stalled && lane == 0)
      for (int b = 0; b < SR; ++b) mbar_wait(&bars[b], (parity >> b) & 1u);
  } else {
    cp_async_wait<0>();  // no copy outstanding when the warp exits
  }
}

// TL_POLY_TEST_HOLD=1: every blocked sweep launched makes warp 0 wait for a row whose copy is
// never issued (the test of the bounded wait and of TL_ERR_TIMEOUT; TMA staging only).
bool poly_test_hold() {
  const char* e = getenv("TL_POLY_TEST_HOLD");
  return e && e[0] == '1';
}

// Steps per blocked sweep: TB_S, or TL_POLY_STEPS_PER_SWEEP (1 .. TB_S) from the environment;
// 1 selects the one-step kernels above (same results, bit for bit).
int poly_steps_per_sweep() {
  const char* e = getenv("TL_POLY_STEPS_PER_SWEEP");
  const int v = e ? atoi(e) : TB_S;
  return v < 1 ? 1 : (v > TB_S ? TB_S : v);
}

// Columns per lane of the blocked sweeps: POLY_CPL, or TL_POLY_COLS (2 or 4) from the
// environment (same results, bit for bit).  At 4096^2 the 2-column strips (79-96 registers,
// 20-24 resident warps per SM instead of 12) measured slower: 53.1 against 49.1 us per FP32
// PPCG step and 47.0 against 39.9 us per Chebyshev step -- the doubled halo costs more than
// the occupancy gains.
constexpr int POLY_CPL = 4;
int poly_cols() {
  const char* e = getenv("TL_POLY_COLS");
  if (e && (e[0] == '2' || e[0] == '4')) return e[0] - '0';
  return POLY_CPL;
}

// Warp tasks: strips x row ranges, about two waves of the resident warps (warps_per_sm),
// at least 32 rows per task (the warm-up of the levels costs ~S rows per task).
void tb_tasks(PolyArgs& a, const Layout& L, int cpl, int warps_per_sm) {
  const int w = cpl == 4 ? TbGeom<4>::W : TbGeom<2>::W;
  a.nstrips = (L.nx + w - 1) / w;
  const long long target = 152LL * warps_per_sm * 2;
  int rows = (int)(((long long)L.ny * a.nstrips + target - 1) / target);
  rows = rows < 32 ? 32 : (rows > 256 ? 256 : rows);
  a.rows = rows;
  a.ntasks = a.nstrips * ((L.ny + rows - 1) / rows);
}

template <int MODE, int S, bool TMA, int CPL, bool PRE>
void launch_tb_s(const PolyArgs& a, const PolyMaps& pm, dim3 grid, cudaStream_t s) {
  constexpr int bytes = TbSmem<MODE, S, TMA, CPL, PRE>::BYTES;
  // above the 48 KB default: the attribute is set on the current device before each launch
  cudaFuncSetAttribute(k_poly_tb<MODE, S, TMA, CPL, PRE>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  k_poly_tb<MODE, S, TMA, CPL, PRE><<<grid, 32 * TB_WARPS, bytes, s>>>(a, pm);
}

// resident warps per SM of the S = TB_S instance (the one most sweeps use)
template <int MODE, bool TMA, int CPL, bool PRE>
int tb_resident_warps() {
  static const int w = [] {
    constexpr int bytes = TbSmem<MODE, TB_S, TMA, CPL, PRE>::BYTES;
    cudaFuncSetAttribute(k_poly_tb<MODE, TB_S, TMA, CPL, PRE>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_poly_tb<MODE, TB_S, TMA, CPL, PRE>, 32 * TB_WARPS,
                                                      bytes) !=
            cudaSuccess ||
        per_sm < 1) {
      cudaGetLastError();
      per_sm = 3;
    }
    return per_sm * TB_WARPS;
  }();
  return w;
}

// ---- tensor maps ----
// TL_POLY_TMA=0 stages with cp.async instead of TMA (same results, bit for bit).
bool poly_use_tma() {
  const char* e = getenv("TL_POLY_TMA");
  return !(e && e[0] == '0');
}

PFN_cuTensorMapEncodeTiled_v12000 tmap_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// a (ld x (ny+2)) view of one field with a box_w x 1 box; cached per (address, layout, type, box)
bool tmap_of(const void* base, const Layout& L, bool f64, int box_w, CUtensorMap* out) {
  static std::mutex mu;
  static std::map<std::tuple<const void*, int, int, bool, int>, CUtensorMap> cache;
  std::lock_guard<std::mutex> lock(mu);
  const auto key = std::make_tuple(base, L.ld, L.ny, f64, box_w);
  auto it = cache.find(key);
  if (it != cache.end()) {
    *out = it->second;
    return true;
  }
  auto enc = tmap_encoder();
  if (!enc) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)L.ld, (cuuint64_t)L.ny + 2};
  const cuuint64_t strides[1] = {(cuuint64_t)L.ld * (f64 ? 8 : 4)};
  const cuuint32_t box[2] = {(cuuint32_t)box_w, 1};
  const cuuint32_t estr[2] = {1, 1};
  CUtensorMap m;
  if (enc(&m, f64 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base), dims,
          strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return false;
  cache[key] = m;
  *out = m;
  return true;
}

// the maps of every field a blocked sweep may read; false if TMA is off or unavailable
bool poly_maps(const MixFields& m, const Layout& L, const double* r64, int box_w, PolyMaps* pm) {
  if (!poly_use_tma()) return false;
  const float* f[PM_R64] = {m.p, m.p2, m.r, m.w, m.d, m.e, m.cx, m.cy, m.di, m.mi ? m.mi : m.di};
  for (int i = 0; i < PM_R64; ++i)
    if (!tmap_of(f[i], L, false, box_w, &pm->t[i])) return false;
  if (r64) {
    if (!tmap_of(r64, L, true, box_w, &pm->t[PM_R64])) return false;
  } else {
    pm->t[PM_R64] = pm->t[PM_R];  // not read
  }
  return true;
}

int map_index(const MixFields& m, const float* p) {
  if (p == m.p) return PM_P;
  if (p == m.p2) return PM_P2;
  if (p == m.r) return PM_R;
  if (p == m.w) return PM_W;
  if (p == m.d) return PM_D;
  if (p == m.e) return PM_E;
  return PM_R;  // (the first sweep reads no state map)
}

template <int MODE, bool TMA, int CPL, bool PRE>
void launch_tb_cpl(const PolyArgs& a, int steps, const PolyMaps& pm, dim3 grid, cudaStream_t s) {
  switch (steps) {
    case 1: launch_tb_s<MODE, 1, TMA, CPL, PRE>(a, pm, grid, s); break;
    case 2: launch_tb_s<MODE, 2, TMA, CPL, PRE>(a, pm, grid, s); break;
    case 3: launch_tb_s<MODE, 3, TMA, CPL, PRE>(a, pm, grid, s); break;
    default: launch_tb_s<MODE, 4, TMA, CPL, PRE>(a, pm, grid, s); break;
  }
}
template <int MODE, bool TMA, int CPL>
void launch_tb_pre(const PolyArgs& a, int steps, const PolyMaps& pm, dim3 grid, cudaStream_t s) {
  if (a.m.mi)
    launch_tb_cpl<MODE, TMA, CPL, true>(a, steps, pm, grid, s);
  else
    launch_tb_cpl<MODE, TMA, CPL, false>(a, steps, pm, grid, s);
}

template <int MODE>
void launch_tb(PolyArgs a, int steps, bool tma, int cpl, const PolyMaps& pm, cudaStream_t s) {
  const dim3 grid((a.ntasks + TB_WARPS - 1) / TB_WARPS);
  a.tx = map_index(a.m, a.x_in);
  a.t1 = map_index(a.m, a.c1_in);
  a.t2 = map_index(a.m, a.c2_in);
  a.hold_row = poly_test_hold() ? 1 + TB_P : -1;  // task 0 starts its march at row 1
  ++launch_counter();
  if (cpl == 4) {
    if (tma) launch_tb_pre<MODE, true, 4>(a, steps, pm, grid, s);
    else launch_tb_pre<MODE, false, 4>(a, steps, pm, grid, s);
  } else {
    if (tma) launch_tb_pre<MODE, true, 2>(a, steps, pm, grid, s);
    else launch_tb_pre<MODE, false, 2>(a, steps, pm, grid, s);
  }
}

template <int MODE>
int tb_warps(bool tma, int cpl, bool pre) {
  if (pre) {
    if (cpl == 4) return tma ? tb_resident_warps<MODE, true, 4, true>() : tb_resident_warps<MODE, false, 4, true>();
    return tma ? tb_resident_warps<MODE, true, 2, true>() : tb_resident_warps<MODE, false, 2, true>();
  }
  if (cpl == 4) return tma ? tb_resident_warps<MODE, true, 4, false>() : tb_resident_warps<MODE, false, 4, false>();
  return tma ? tb_resident_warps<MODE, true, 2, false>() : tb_resident_warps<MODE, false, 2, false>();
}

}  // namespace

void launch_poly_ppcg_inner(const Fields& f, const MixFields& m, const Layout& L, double theta, int inner_steps,
                            const double* ch_a, const double* ch_b, cudaStream_t s) {
  const int blk = poly_steps_per_sweep();
  if (blk > 1 && inner_steps > 0) {
    // state ping-pong between (p, r, w) and (p2, d, e); the first sweep starts from the FP64 r
    PolyArgs a{};
    a.m = m;
    a.L = L;
    a.r64 = f.r;
    a.inv_theta = (float)(1.0 / theta);
    const int cpl = poly_cols();
    PolyMaps pm;
    const bool tma = poly_maps(m, L, f.r, 32 * cpl, &pm);
    tb_tasks(a, L, cpl, tb_warps<POLY_PPCG>(tma, cpl, m.mi != nullptr));
    int done = 0, par = 0;
    while (done < inner_steps) {
      const int st = inner_steps - done < blk ? inner_steps - done : blk;
      a.first = done == 0;
      a.x_in = par ? m.p2 : m.p;
      a.x_out = par ? m.p : m.p2;
      a.c1_in = par ? m.d : m.r;
      a.c1_out = par ? m.r : m.d;
      a.c2_in = par ? m.e : m.w;
      a.c2_out = par ? m.w : m.e;
      for (int i = 0; i < TB_S; ++i) {
        a.ca[i] = i < st ? (float)ch_a[done + 1 + i] : 0.f;
        a.cb[i] = i < st ? (float)ch_b[done + 1 + i] : 0.f;
      }
      a.z = done + st == inner_steps ? f.z : nullptr;
      launch_tb<POLY_PPCG>(a, st, tma, cpl, pm, s);
      done += st;
      par ^= 1;
    }
    return;
  }
  const dim3 g = poly_grid(L);
  { ++launch_counter(); k_poly_ppcg_init<<<g, PT, 0, s>>>(f.r, m, L, (float)(1.0 / theta)); }
  if (inner_steps <= 0) {
    { ++launch_counter(); k_poly_to_z<<<g, PT, 0, s>>>(m, L, f.z); }
    return;
  }
  for (int step = 1; step <= inner_steps; ++step) {
    const float* in = (step & 1) ? m.p : m.p2;
    float* out = (step & 1) ? m.p2 : m.p;
    double* z = step == inner_steps ? f.z : nullptr;
    ++launch_counter();
    k_poly_ppcg_step<<<g, PT, 0, s>>>(m, in, out, L, (float)ch_a[step], (float)ch_b[step], z);
  }
}

void launch_poly_cheby(const MixFields& m, const Layout& L, double theta, int steps, const double* ch_a,
                       const double* ch_b, cudaStream_t s) {
  const int blk = poly_steps_per_sweep();
  const int iters = steps - 1;
  if (blk > 1 && iters >= 1) {
    // d ping-pong (d, p2) and p ping-pong (p, w), arranged so that the last sweep writes d into
    // m.d; the first sweep starts from m.r (the start step)
    PolyArgs a{};
    a.m = m;
    a.L = L;
    a.inv_theta = (float)(1.0 / theta);
    const int cpl = poly_cols();
    PolyMaps pm;
    const bool tma = poly_maps(m, L, nullptr, 32 * cpl, &pm);
    tb_tasks(a, L, cpl, tb_warps<POLY_CHEBY>(tma, cpl, m.mi != nullptr));
    const int nb = (iters + blk - 1) / blk;
    const float* din = nullptr;
    const float* pin = nullptr;
    for (int b = 0; b < nb; ++b) {
      const int st = iters - b * blk < blk ? iters - b * blk : blk;
      const bool to_d = (nb - 1 - b) % 2 == 0;
      a.first = b == 0;
      a.x_in = din;
      a.c1_in = pin;
      a.x_out = to_d ? m.d : m.p2;
      a.c1_out = to_d ? m.p : m.w;
      for (int i = 0; i < TB_S; ++i) {
        a.ca[i] = i < st ? (float)ch_a[b * blk + 1 + i] : 0.f;
        a.cb[i] = i < st ? (float)ch_b[b * blk + 1 + i] : 0.f;
      }
      launch_tb<POLY_CHEBY>(a, st, tma, cpl, pm, s);
      din = a.x_out;
      pin = a.c1_out;
    }
    return;
  }
  const dim3 g = poly_grid(L);
  // the start writes d into the buffer that makes the last iteration's output m.d
  float* first = ((steps - 1) % 2 == 0) ? m.d : m.p2;
  { ++launch_counter(); k_poly_cheby_start<<<g, PT, 0, s>>>(m, first, L, (float)(1.0 / theta)); }
  const float* cur = first;
  for (int i = 1; i < steps; ++i) {
    float* out = (cur == m.d) ? m.p2 : m.d;
    ++launch_counter();
    k_poly_cheby_step<<<g, PT, 0, s>>>(m, cur, out, L, (float)ch_a[i], (float)ch_b[i]);
    cur = out;
  }
}

void launch_poly_clear(const MixFields& m, const Layout& L, cudaStream_t s) {
  { ++launch_counter(); k_poly_clear<<<poly_grid(L), PT, 0, s>>>(m, L); }
}

}  // namespace tl
