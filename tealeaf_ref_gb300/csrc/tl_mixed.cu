// tl_mixed.cu -- the mixed-precision form of the CG solve: FP32 inner CG on FP32 copies of
// the operator, wrapped in FP64 iterative refinement.
//
// Outer loop (FP64): r = u0 - A u (true residual, tea_leaf_common_kernel.f90:208-244
// arithmetic in FP64), ||r||^2 in FP64; stop when sqrt(||r||^2) < eps * initial residual
// (the reference's test, tea_solve.f90:410) or when the true residual no longer falls (the
// FP64 accuracy floor of b - A u).  Inner loop (FP32 vectors): CG on A d = r, d0 = 0, to a
// relative reduction `inner_tol` of its recursively updated residual; then u += d in FP64.
//
// The inner sweeps are the FP64 fused CG sweeps (tl_fused.cu) on float data: p update +
// 5-point matvec + p.w with the deferred d += alpha p, and r -= alpha w + r.r.  They move 48
// bytes per cell-iteration and do no FP64 arithmetic per cell: the dot products are summed
// per thread with the compensated FP32 algorithm Dot2 (TwoProduct via FMA + TwoSum; Ogita,
// Rump & Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput. 26, 2005), whose result
// is as accurate as a dot product in twice the working precision; the per-thread (sum,
// error) pairs, the block and grid sums and the step coefficients alpha, beta are FP64.
#include <cmath>
#include <vector>

#include "tl_kernels.cuh"

namespace tl {

namespace {

constexpr int MT = 128;     // threads per CTA
constexpr int MSW = 2 * MT; // strip width

// ---- error-free transformations (Knuth's TwoSum; TwoProduct with FMA) ----
struct Dot2 {
  float s = 0.f, c = 0.f;  // running sum and accumulated error terms
  __device__ __forceinline__ void add(float a, float b) {
    const float p = a * b;
    const float pe = fmaf(a, b, -p);  // a*b = p + pe exactly
    const float t = s + p;
    const float z = t - s;
    const float se = (s - (t - z)) + (p - z);  // s + p = t + se exactly
    s = t;
    c += pe + se;
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

__device__ __forceinline__ void mix_finish(MixState* ms) {
  // inner CG convergence on its recursively updated residual, or the iteration cap
  if (!(ms->rr > ms->tol2) || ms->n >= ms->max_n) {
    ms->status = EXIT_CONVERGED;
  } else {
    ms->n += 1;
  }
}

struct EpiMixResidual {
  MixState* ms;
  __device__ void operator()(double (&acc)[2]) const {
    ms->outer_rr = acc[0];
    ms->rro = acc[1];
    ms->rr0 = acc[1];
    ms->rr = acc[1];
    ms->tol2 = ms->inner_tol * ms->inner_tol * acc[1];
    ms->n = 1;
    ms->status = (acc[1] > 0.0 && isfinite(acc[1])) ? RUN : EXIT_CONVERGED;
    ms->p_pending = 0;
    ms->d_pending = 0;
  }
};

struct EpiMixW {
  MixState* ms;
  __device__ void operator()(double (&acc)[1]) const {
    ms->d_pending = 0;
    ms->pw = acc[0];
    const double alpha = ms->rro / ms->pw;
    ms->alpha = alpha;
    if (!isfinite(alpha)) ms->status = EXIT_BREAKDOWN;
  }
};

struct EpiMixUr {
  MixState* ms;
  __device__ void operator()(double (&acc)[1]) const {
    ms->rr = acc[0];
    ms->beta = acc[0] / ms->rro;
    ms->rro = acc[0];
    ms->p_pending = 1;
    ms->d_pending = 1;
    ms->d_alpha = ms->alpha;
    ms->d_psel = ms->n & 1;
    if (!isfinite(ms->beta)) {
      ms->status = EXIT_BREAKDOWN;
      return;
    }
    mix_finish(ms);
  }
};

// FP32 copies of the pre-scaled face coefficients and the diagonal.
__global__ void k_mix_prep(Fields f, MixFields m, Layout L) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  for (int k = blockIdx.y + 1; k <= L.ny + 1; k += gridDim.y) {
    if (j > L.nx + 1) continue;
    const long long c = L.at(j, k);
    m.cx[c] = (float)f.cx[c];
    m.cy[c] = (float)f.cy[c];
    if (j <= L.nx && k <= L.ny) m.di[c] = (float)f.di[c];
  }
}

// Outer residual in FP64: r = u0 - A u; ||r||^2 (FP64) and the inner start r32 = p32 = r,
// ||r32||^2, d32 = 0.
__global__ void k_mix_residual(Fields f, MixFields m, Layout L, Reduce rd, MixState* ms) {
  double acc[2] = {0.0, 0.0};
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  for (int k = blockIdx.y + 1; k <= L.ny; k += gridDim.y) {
    if (j > L.nx) continue;
    const long long c = L.at(j, k);
    double a = f.di[c] * f.u[c];
    a = fma(-f.cy[c + L.ld], f.u[c + L.ld], a);
    a = fma(-f.cy[c], f.u[c - L.ld], a);
    a = fma(-f.cx[c + 1], f.u[c + 1], a);
    a = fma(-f.cx[c], f.u[c - 1], a);
    const double r = f.u0[c] - a;
    acc[0] = fma(r, r, acc[0]);
    const float r32 = (float)r;
    m.r[c] = r32;
    m.p[c] = r32;
    m.d[c] = 0.f;
    acc[1] = fma((double)r32, (double)r32, acc[1]);
  }
  grid_reduce<2>(acc, rd, EpiMixResidual{ms});
}

// p_n = r + beta p_{n-1} (FP32), w = A p_n (FP32), p.w (Dot2), deferred d += alpha p_{n-1}.
__global__ void __launch_bounds__(MT) k_mix_w(MixFields m, Layout L, Reduce rd, MixState* ms, int rows_per_cta) {
  if (ms->status != RUN) return;
  const int n = ms->n;
  const float beta = (float)ms->beta;
  const bool upd = ms->p_pending != 0;
  const bool upd_d = ms->d_pending != 0;
  const float da = (float)ms->d_alpha;
  const float* __restrict__ pold = (n & 1) ? m.p : m.p2;
  float* __restrict__ pout = (n & 1) ? m.p2 : m.p;
  const float* __restrict__ r = m.r;
  __shared__ float buf[2][MSW + 2];
  const int t = threadIdx.x;
  const int js = blockIdx.x * MSW + 1;
  const int ja = js + 2 * t;
  const bool active = ja <= L.nx, has_b = ja + 1 <= L.nx;
  const int k0 = blockIdx.y * rows_per_cta + 1;
  const int k1 = min(k0 + rows_per_cta - 1, L.ny);
  auto pnew = [&](long long c, float2& old) {
    old = *reinterpret_cast<const float2*>(pold + c);
    float2 q = old;
    if (upd) {
      const float2 s = *reinterpret_cast<const float2*>(r + c);
      q.x = fmaf(beta, q.x, s.x);
      q.y = fmaf(beta, q.y, s.y);
    }
    return q;
  };
  auto pnew1 = [&](long long c) { return upd ? fmaf(beta, pold[c], r[c]) : pold[c]; };
  Dot2 dot;
  float2 pm = make_float2(0.f, 0.f), pc = pm, pnx = pm, cyc = pm, oc = pm, onx = pm, junk;
  if (active) {
    pc = pnew(L.at(ja, k0), oc);
    pm = (k0 == 1) ? pc : pnew(L.at(ja, k0 - 1), junk);
    cyc = *reinterpret_cast<const float2*>(m.cy + L.at(ja, k0));
  }
  for (int k = k0; k <= k1; ++k) {
    const int b = k & 1;
    if (active) {
      pnx = (k == L.ny) ? pc : pnew(L.at(ja, k + 1), onx);
      buf[b][2 * t + 1] = pc.x;
      buf[b][2 * t + 2] = pc.y;
    }
    if (t == 0 && js > 1) buf[b][0] = pnew1(L.at(js - 1, k));
    if (t == MT - 1 && js + MSW <= L.nx) buf[b][MSW + 1] = pnew1(L.at(js + MSW, k));
    __syncthreads();
    if (active) {
      const long long c = L.at(ja, k);
      const float2 cyn = *reinterpret_cast<const float2*>(m.cy + c + L.ld);
      const float2 cxa = *reinterpret_cast<const float2*>(m.cx + c);
      const float2 dd = *reinterpret_cast<const float2*>(m.di + c);
      const float left_a = (ja == 1) ? pc.x : buf[b][ja - js];
      const float right_a = has_b ? pc.y : pc.x;
      float wa = dd.x * pc.x;
      wa = fmaf(-cyn.x, pnx.x, wa);
      wa = fmaf(-cyc.x, pm.x, wa);
      wa = fmaf(-cxa.y, right_a, wa);
      wa = fmaf(-cxa.x, left_a, wa);
      dot.add(wa, pc.x);
      if (has_b) {
        const float cxr = m.cx[c + 2];
        const float right_b = (ja + 1 == L.nx) ? pc.y : buf[b][ja - js + 3];
        float wb = dd.y * pc.y;
        wb = fmaf(-cyn.y, pnx.y, wb);
        wb = fmaf(-cyc.y, pm.y, wb);
        wb = fmaf(-cxr, right_b, wb);
        wb = fmaf(-cxa.y, pc.x, wb);
        dot.add(wb, pc.y);
        *reinterpret_cast<float2*>(m.w + c) = make_float2(wa, wb);
        *reinterpret_cast<float2*>(pout + c) = pc;
        if (upd_d) {
          float2 dv = *reinterpret_cast<const float2*>(m.d + c);
          dv.x = fmaf(da, oc.x, dv.x);
          dv.y = fmaf(da, oc.y, dv.y);
          *reinterpret_cast<float2*>(m.d + c) = dv;
        }
      } else {
        m.w[c] = wa;
        pout[c] = pc.x;
        if (upd_d) m.d[c] = fmaf(da, oc.x, m.d[c]);
      }
      cyc = cyn;
    }
    pm = pc;
    pc = pnx;
    oc = onx;
  }
  double acc[1] = {dot.value()};
  grid_reduce<1>(acc, rd, EpiMixW{ms});
}

// r -= alpha w (FP32), r.r (Dot2), inner epilogue.
__global__ void __launch_bounds__(MT) k_mix_ur(MixFields m, Layout L, Reduce rd, MixState* ms) {
  if (ms->status != RUN) return;
  const float alpha = (float)ms->alpha;
  const int ja = blockIdx.x * MSW + 1 + 2 * threadIdx.x;
  const bool has_b = ja + 1 <= L.nx;
  Dot2 dot;
  if (ja <= L.nx) {
    for (int k = blockIdx.y + 1; k <= L.ny; k += gridDim.y) {
      const long long c = L.at(ja, k);
      const float2 ww = *reinterpret_cast<const float2*>(m.w + c);
      float2 rr = *reinterpret_cast<const float2*>(m.r + c);
      rr.x = fmaf(-alpha, ww.x, rr.x);
      rr.y = fmaf(-alpha, ww.y, rr.y);
      dot.add(rr.x, rr.x);
      if (has_b) {
        dot.add(rr.y, rr.y);
        *reinterpret_cast<float2*>(m.r + c) = rr;
      } else {
        m.r[c] = rr.x;
      }
    }
  }
  double acc[1] = {dot.value()};
  grid_reduce<1>(acc, rd, EpiMixUr{ms});
}

// pending d += alpha p, then u += d in FP64 (one pass per outer iteration)
__global__ void k_mix_apply(Fields f, MixFields m, Layout L, MixState* ms) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (j > L.nx) return;
  const bool pend = ms->d_pending != 0;
  const float da = (float)ms->d_alpha;
  const float* __restrict__ p = ms->d_psel ? m.p2 : m.p;
  for (int k = blockIdx.y + 1; k <= L.ny; k += gridDim.y) {
    const long long c = L.at(j, k);
    float d = m.d[c];
    if (pend) d = fmaf(da, p[c], d);
    f.u[c] = f.u[c] + (double)d;
  }
}

inline int mstrips(const Layout& L) { return (L.nx + MSW - 1) / MSW; }

}  // namespace

void launch_mix_prep(const Fields& f, const MixFields& m, const Layout& L, cudaStream_t s) {
  dim3 grid((L.nx + 1 + 255) / 256, L.ny + 1 > 65535 ? 65535 : L.ny + 1);
  { ++launch_counter(); k_mix_prep<<<grid, 256, 0, s>>>(f, m, L); }
}

void launch_mix_residual(const Fields& f, const MixFields& m, const Layout& L, const Reduce& rd, MixState* ms,
                         cudaStream_t s) {
  dim3 grid((L.nx + 255) / 256, L.ny < 256 ? L.ny : 256);
  { ++launch_counter(); k_mix_residual<<<grid, 256, 0, s>>>(f, m, L, rd, ms); }
}

void launch_mix_iteration(const MixFields& m, const Layout& L, const Reduce& rd, MixState* ms, cudaStream_t s) {
  const int ns = mstrips(L);
  int rows = (int)(((long long)L.ny * ns) / (152 * 8));
  rows = rows < 8 ? 8 : (rows > 64 ? 64 : rows);
  const int min_rows = (int)(((long long)L.ny * ns + MAX_REDUCE_BLOCKS - 1) / MAX_REDUCE_BLOCKS);
  if (rows < min_rows) rows = min_rows;
  { ++launch_counter(); k_mix_w<<<dim3(ns, (L.ny + rows - 1) / rows), MT, 0, s>>>(m, L, rd, ms, rows); }
  int gy = L.ny < 512 ? L.ny : 512;
  if ((long long)gy * ns > MAX_REDUCE_BLOCKS) gy = MAX_REDUCE_BLOCKS / ns;
  { ++launch_counter(); k_mix_ur<<<dim3(ns, gy), MT, 0, s>>>(m, L, rd, ms); }
}

void launch_mix_apply(const Fields& f, const MixFields& m, const Layout& L, MixState* ms, cudaStream_t s) {
  dim3 grid((L.nx + 255) / 256, L.ny < 4096 ? L.ny : 4096);
  { ++launch_counter(); k_mix_apply<<<grid, 256, 0, s>>>(f, m, L, ms); }
}

}  // namespace tl
