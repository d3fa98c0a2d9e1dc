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
#include <cstdlib>

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

// tea_leaf_kernel_ppcg_init_sd (tea_leaf_ppcg_kernel.f90:31-88, no preconditioner) in FP32:
// rtemp = r, sd = r / theta (as r * (1/theta) in FP32: a per-cell FP64 division would make this
// copy FP64-bound), utemp = sd.
__global__ void k_poly_ppcg_init(const double* __restrict__ r, MixFields m, Layout L, float inv_theta) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (j > L.nx) return;
  for (int k = blockIdx.y + 1; k <= L.ny; k += gridDim.y) {
    const long long c = L.at(j, k);
    const float rv = (float)r[c];
    const float sd = rv * inv_theta;
    m.r[c] = rv;
    m.p[c] = sd;
    m.w[c] = sd;
  }
}

// One inner step (tea_leaf_kernel_ppcg_inner, ppcg_kernel.f90:204-310) in FP32:
// rtemp -= A sd; sd' = a sd + b rtemp; utemp += sd'.  z (nullable, FP64): z = utemp after the
// last step (tea_leaf_ppcg_update_z_kernel, :453-477).
__global__ void k_poly_ppcg_step(MixFields m, const float* __restrict__ sd_in, float* __restrict__ sd_out, Layout L,
                                 float a, float b, double* __restrict__ z) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (j > L.nx) return;
  for (int k = blockIdx.y + 1; k <= L.ny; k += gridDim.y) {
    const long long c = L.at(j, k);
    const float rt = m.r[c] - apply_a32<true>(sd_in, m, c, j, k, L);
    m.r[c] = rt;
    const float sd = fmaf(a, sd_in[c], b * rt);
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
// with u = 0, u0 = r): p = r / theta, d = p.
__global__ void k_poly_cheby_start(MixFields m, float* __restrict__ d, Layout L, float inv_theta) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (j > L.nx) return;
  for (int k = blockIdx.y + 1; k <= L.ny; k += gridDim.y) {
    const long long c = L.at(j, k);
    const float p = m.r[c] * inv_theta;
    m.p[c] = p;
    d[c] = p;
  }
}

// One Chebyshev iteration on the correction (tea_leaf_kernel_cheby_iterate, :111-200):
// res = r - A d; p = a p + b res; d' = d + p.
__global__ void k_poly_cheby_step(MixFields m, const float* __restrict__ d_in, float* __restrict__ d_out, Layout L,
                                  float a, float b) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (j > L.nx) return;
  for (int k = blockIdx.y + 1; k <= L.ny; k += gridDim.y) {
    const long long c = L.at(j, k);
    const float res = m.r[c] - apply_a32<false>(d_in, m, c, j, k, L);
    const float p = fmaf(a, m.p[c], b * res);
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
// Each warp owns a strip of 128 columns (four per lane, 16-byte loads) with a TB_HX-column
// halo on each side, TB_W output columns, and marches up a range of rows.  At march position
// m, level 0 loads row m and level t = 1..S computes step t at row m - t from level t-1's rows
// m-t-1 .. m-t+1 (a three-row register window per level) and level t-1's cell values of row m-t
// (its output one march position earlier).  Horizontal neighbours come from the adjacent
// lanes by shuffles; the coefficient rows sit in a per-warp shared-memory ring, loaded once
// at level 0.  Warps never wait for one another.  Level t is exact on local columns
// [t, 128-t): with S <= TB_HX the output columns are exact.  Every cell runs the one-step
// kernels' arithmetic in the same order, so S steps here give the bits of S one-step sweeps.
// Traffic per S steps: the state and the coefficients read once (x 128/TB_W for the halo),
// the state written once.
constexpr int TB_S = 4;                // steps per sweep at most
constexpr int TB_HX = 4;               // halo columns on each side of a warp strip
constexpr int TB_W = 128 - 2 * TB_HX;  // output columns per warp strip
constexpr int TB_WARPS = 4;            // warps per CTA
constexpr int TB_PF = 8;               // L2 prefetch distance in rows
constexpr unsigned FULL = 0xffffffffu;

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
  float ca[TB_S], cb[TB_S];
};

__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// columns j .. j+3 (j = 1 mod 4, so 16-byte aligned) where lo <= column <= hi, else 0
__device__ __forceinline__ void load4(const float* __restrict__ p, long long c, int j, int lo, int hi,
                                      float (&v)[4]) {
  if (j >= lo && j + 3 <= hi) {
    const float4 q = __ldg(reinterpret_cast<const float4*>(p + c));
    v[0] = q.x, v[1] = q.y, v[2] = q.z, v[3] = q.w;
  } else {
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] = (j + i >= lo && j + i <= hi) ? __ldg(p + c + i) : 0.f;
  }
}

// columns j+i with lo <= j+i <= hi
__device__ __forceinline__ void store4(float* __restrict__ p, long long c, const float (&v)[4], int lo, int hi,
                                       int j) {
  if (j >= lo && j + 3 <= hi) {
    *reinterpret_cast<float4*>(p + c) = make_float4(v[0], v[1], v[2], v[3]);
  } else {
#pragma unroll
    for (int i = 0; i < 4; ++i)
      if (j + i >= lo && j + i <= hi) p[c + i] = v[i];
  }
}

template <int MODE, int S>
__global__ void __launch_bounds__(32 * TB_WARPS) k_poly_tb(PolyArgs a) {
  constexpr bool PPCG = MODE == POLY_PPCG;
  const int lane = threadIdx.x & 31;
  const int task = blockIdx.x * TB_WARPS + (threadIdx.x >> 5);
  if (task >= a.ntasks) return;  // whole warps only
  const Layout L = a.L;
  const MixFields& m = a.m;
  const int x0 = 1 + (task % a.nstrips) * TB_W;
  const int k0 = 1 + (task / a.nstrips) * a.rows;
  const int k1 = min(k0 + a.rows - 1, L.ny);
  const int j = x0 - TB_HX + 4 * lane;  // this lane's first column
  const int out0 = x0, out1 = min(x0 + TB_W - 1, L.nx);
  float X[S][3][4];   // level t < S: stencil variable of rows (newest-2, newest-1, newest)
  float C1[S][2][4];  // level t < S: rtemp | p of rows (newest-1, newest)
  float C2[S][2][4];  // level t < S: utemp of rows (newest-1, newest)
#pragma unroll
  for (int t = 0; t < S; ++t)
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      X[t][0][i] = X[t][1][i] = X[t][2][i] = 0.f;
      C1[t][0][i] = C1[t][1][i] = C2[t][0][i] = C2[t][1][i] = 0.f;
    }
  // per-warp ring of coefficient rows (di, cx, cy, and Chebyshev's right-hand side): row q in
  // slot q mod (S+1), loaded once at level 0 and read by every level from shared memory
  constexpr int NC = PPCG ? 3 : 4;
  constexpr int RING = S + 1;
  __shared__ __align__(16) float ring[TB_WARPS][RING][NC][132];
  float(*cr)[NC][132] = ring[threadIdx.x >> 5];
  const int lc = 4 * lane;
  const int mstart = max(1, k0 - S), mend = k1 + S;
  for (int mm = mstart; mm <= mend; ++mm) {
    // L2 prefetch of the rows the march reaches TB_PF positions later
    const int pf = mm + TB_PF;
    if (pf <= min(L.ny, k1 + S) && j >= 1 && j + 3 <= L.nx) {
      const long long c = L.at(j, pf);
      if (a.first) {
        if (PPCG) prefetch_l2(a.r64 + c);
      } else {
        prefetch_l2(a.x_in + c);
        prefetch_l2(a.c1_in + c);
        if (PPCG) prefetch_l2(a.c2_in + c);
      }
      prefetch_l2(m.di + c);
      prefetch_l2(m.cx + c);
      prefetch_l2(m.cy + c);
      if (!PPCG) prefetch_l2(m.r + c);
    }
    // ---- level 0: coefficient row mm into the ring (cy also for the boundary row ny+1) ----
    __syncwarp();  // every lane is done with the slot's previous row
    if (mm <= min(L.ny + 1, k1 + S)) {
      const long long c = L.at(j, mm);
      float(*slot)[132] = cr[mm % RING];
      float v0[4], v1[4], v2[4], v3[4];
      load4(m.cy, c, j, 1, L.nx, v2);
      if (mm <= L.ny) {
        load4(m.di, c, j, 1, L.nx, v0);
        load4(m.cx, c, j, 1, L.nx + 1, v1);
        if (!PPCG) load4(m.r, c, j, 1, L.nx, v3);
        *reinterpret_cast<float4*>(&slot[0][lc]) = make_float4(v0[0], v0[1], v0[2], v0[3]);
        *reinterpret_cast<float4*>(&slot[1][lc]) = make_float4(v1[0], v1[1], v1[2], v1[3]);
        if (!PPCG) *reinterpret_cast<float4*>(&slot[NC - 1][lc]) = make_float4(v3[0], v3[1], v3[2], v3[3]);
      }
      *reinterpret_cast<float4*>(&slot[2][lc]) = make_float4(v2[0], v2[1], v2[2], v2[3]);
    }
    // ---- level 0: the sweep's input at row mm ----
    float nx[4] = {0.f, 0.f, 0.f, 0.f}, n1[4] = {0.f, 0.f, 0.f, 0.f}, n2[4] = {0.f, 0.f, 0.f, 0.f};
    if (mm <= min(L.ny, k1 + S)) {
      const long long c = L.at(j, mm);
      if (a.first) {
        if (PPCG) {
#pragma unroll
          for (int i = 0; i < 4; ++i)
            if (j + i >= 1 && j + i <= L.nx) {
              const float rv = (float)a.r64[c + i];
              n1[i] = rv;
              nx[i] = rv * a.inv_theta;
              n2[i] = nx[i];
            }
        } else {
          float rr[4];
          load4(m.r, c, j, 1, L.nx, rr);
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            nx[i] = rr[i] * a.inv_theta;
            n1[i] = nx[i];
          }
        }
      } else {
        load4(a.x_in, c, j, 1, L.nx, nx);
        load4(a.c1_in, c, j, 1, L.nx, n1);
        if (PPCG) load4(a.c2_in, c, j, 1, L.nx, n2);
      }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      X[0][0][i] = X[0][1][i];
      X[0][1][i] = X[0][2][i];
      X[0][2][i] = nx[i];
      C1[0][0][i] = C1[0][1][i];
      C1[0][1][i] = n1[i];
      C2[0][0][i] = C2[0][1][i];
      C2[0][1][i] = n2[i];
    }
    __syncwarp();  // the ring row is visible to the whole warp
    // ---- levels 1..S: step t at row mm - t ----
#pragma unroll
    for (int t = 1; t <= S; ++t) {
      const int q = mm - t;
      const bool act = q >= max(1, k0 - (S - t)) && q <= min(L.ny, k1 + (S - t));  // uniform per warp
      float ox[4] = {0.f, 0.f, 0.f, 0.f}, o1[4] = {0.f, 0.f, 0.f, 0.f}, o2[4] = {0.f, 0.f, 0.f, 0.f};
      if (act) {
        const float(*rq)[132] = cr[q % RING];
        const float(*rq1)[132] = cr[(q + 1) % RING];
        float di[4], cxv[4], cyb[4], cyt[4], rhs[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          di[i] = rq[0][lc + i];
          cxv[i] = rq[1][lc + i];
          cyb[i] = rq[2][lc + i];
          cyt[i] = rq1[2][lc + i];
          rhs[i] = PPCG ? 0.f : rq[NC - 1][lc + i];
        }
        const float cx4 = rq[1][lc + 4];                                // cx at column j+4
        const float left = __shfl_up_sync(FULL, X[t - 1][1][3], 1);     // column j-1
        const float right = __shfl_down_sync(FULL, X[t - 1][1][0], 1);  // column j+4
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const float vc = X[t - 1][1][i];
          const float off = PPCG ? vc : 0.f;  // mirror (PPCG's sd) or zero (Chebyshev's d)
          float vl = (i == 0) ? left : X[t - 1][1][i - 1];
          float vr = (i == 3) ? right : X[t - 1][1][i + 1];
          if (j + i == 1) vl = off;
          if (j + i == L.nx) vr = off;
          const float vb = (q > 1) ? X[t - 1][0][i] : off;
          const float vt = (q < L.ny) ? X[t - 1][2][i] : off;
          const float cr1 = (i == 3) ? cx4 : cxv[i + 1];
          float av = di[i] * vc;
          av = fmaf(-cyt[i], vt, av);
          av = fmaf(-cyb[i], vb, av);
          av = fmaf(-cr1, vr, av);
          av = fmaf(-cxv[i], vl, av);
          if (PPCG) {
            const float rt = C1[t - 1][0][i] - av;
            const float sd = fmaf(a.ca[t - 1], vc, a.cb[t - 1] * rt);
            o1[i] = rt;
            ox[i] = sd;
            o2[i] = C2[t - 1][0][i] + sd;
          } else {
            const float res = rhs[i] - av;
            const float pn = fmaf(a.ca[t - 1], C1[t - 1][0][i], a.cb[t - 1] * res);
            o1[i] = pn;
            ox[i] = vc + pn;
          }
        }
      }
      if (t < S) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
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
          for (int i = 0; i < 4; ++i)
            if (j + i >= out0 && j + i <= out1) a.z[c + i] = (double)o2[i];
        } else {
          store4(a.x_out, c, ox, out0, out1, j);
          store4(a.c1_out, c, o1, out0, out1, j);
          if (PPCG) store4(a.c2_out, c, o2, out0, out1, j);
        }
      }
    }
  }
}

// Steps per blocked sweep: TB_S, or TL_POLY_STEPS_PER_SWEEP (1 .. TB_S) from the environment;
// 1 selects the one-step kernels above (same results, bit for bit).
int poly_steps_per_sweep() {
  const char* e = getenv("TL_POLY_STEPS_PER_SWEEP");
  const int v = e ? atoi(e) : TB_S;
  return v < 1 ? 1 : (v > TB_S ? TB_S : v);
}

void tb_tasks(PolyArgs& a, const Layout& L) {
  a.nstrips = (L.nx + TB_W - 1) / TB_W;
  // about two waves of 12 resident warps per SM, at least 32 rows per task (the warm-up of the
  // levels costs ~S rows per task)
  const long long target = 152LL * 12 * 2;
  int rows = (int)(((long long)L.ny * a.nstrips + target - 1) / target);
  rows = rows < 32 ? 32 : (rows > 256 ? 256 : rows);
  a.rows = rows;
  a.ntasks = a.nstrips * ((L.ny + rows - 1) / rows);
}

template <int MODE>
void launch_tb(const PolyArgs& a, int steps, cudaStream_t s) {
  const dim3 grid((a.ntasks + TB_WARPS - 1) / TB_WARPS);
  const int nt = 32 * TB_WARPS;
  ++launch_counter();
  switch (steps) {
    case 1: k_poly_tb<MODE, 1><<<grid, nt, 0, s>>>(a); break;
    case 2: k_poly_tb<MODE, 2><<<grid, nt, 0, s>>>(a); break;
    case 3: k_poly_tb<MODE, 3><<<grid, nt, 0, s>>>(a); break;
    default: k_poly_tb<MODE, 4><<<grid, nt, 0, s>>>(a); break;
  }
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
    tb_tasks(a, L);
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
      launch_tb<POLY_PPCG>(a, st, s);
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
    tb_tasks(a, L);
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
      launch_tb<POLY_CHEBY>(a, st, s);
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
