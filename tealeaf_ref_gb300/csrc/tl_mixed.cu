// tl_mixed.cu -- the mixed-precision form of the CG solve: CG on FP32 vectors and FP32
// copies of the operator, with the solution accumulated and the residual periodically
// recomputed in FP64 ("reliable updates": van der Vorst & Ye, SIAM J. Sci. Comput. 22,
// 2000; Clark et al., Comput. Phys. Commun. 181, 2010).
//
// The FP32 CG process runs on the correction d (u = u_64 + d).  When its recursively
// updated residual has fallen by `delta` (tl_solve_opts.inner_tol) since the last
// replacement, or a phase has used its step budget, the true residual of u + d is computed
// in FP64 (tea_leaf_common_kernel.f90:208-244 arithmetic) without touching u.  If it is
// lower than the last accepted one, the correction is folded into u in FP64, the true
// residual replaces the FP32 residual and the CG process continues with its search
// direction kept -- unlike a restarted refinement, the Krylov process is not thrown away.
// Otherwise the correction is dropped and u stays the best iterate.  The solve stops when the
// true residual satisfies the reference's test sqrt(r.r) < eps * initial residual
// (tea_solve.f90:410) or stops falling (the FP64 accuracy floor of u0 - A u).
//
// With the jac_diag preconditioner (MixFields::mi non-null) the FP32 process is preconditioned
// CG: the update sweep (and a trial) also writes z = Mi32 r (Mi32 = the FP32 rounding of the
// FP64 Mi = 1/Di) and reduces r.z; the matvec sweep stages z in place of r for p = z + beta p.
// The trial residual also reduces r.(Mi r) in FP64, the norm the reference's preconditioned CG
// tests (error = rrn = r.z, tea_leaf_cg_kernel.f90:256-283).
//
// The FP32 sweeps are the FP64 fused CG sweeps (tl_fused.cu) on float data: p update +
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

constexpr int MT = 128;      // threads per CTA
constexpr int MSW = 4 * MT;  // strip width (four columns per thread)

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
  ms->n += 1;
  if (ms->switch_rr > 0.0 && ms->n >= ms->presteps && ms->rr <= ms->switch_rr) {
    ms->status = STOP_SWITCH;
    return;
  }
  // hand over to the host for a residual replacement (the recursive residual fell by delta,
  // or this phase used up its step budget), or stop at the overall cap
  if (!(ms->rr > ms->delta2 * ms->rr_max) || ms->n > ms->max_n || ms->n >= ms->phase_end)
    ms->status = EXIT_CONVERGED;
}

// Records the norms of a trial residual; the host decides whether to accept the correction.
// The pending d update was flushed before the trial (k_mix_flush_d), so it is cleared here.
struct EpiMixTrial {
  MixState* ms;
  __device__ void operator()(double (&acc)[5]) const {
    ms->trial_rr = acc[0];
    ms->trial_rr32 = acc[1];
    ms->trial_scale = acc[2];
    ms->trial_rz = acc[3];
    ms->trial_rz32 = acc[4];
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
    if (ms->hist_a) ms->hist_a[ms->n] = alpha;
    if (!isfinite(alpha)) ms->status = EXIT_BREAKDOWN;
  }
};

struct EpiMixUr {
  MixState* ms;
  __device__ void operator()(double (&acc)[1]) const {
    ms->rr = acc[0];
    ms->beta = acc[0] / ms->rro;
    if (ms->hist_b) ms->hist_b[ms->n] = ms->beta;
    ms->rro_prev = ms->rro;
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

// FP32 copies of the pre-scaled face coefficients, the diagonal and the jac_diag Mi.
__global__ void k_mix_prep(Fields f, MixFields m, Layout L) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  for (int k = blockIdx.y + 1; k <= L.ny + 1; k += gridDim.y) {
    if (j > L.nx + 1) continue;
    const long long c = L.at(j, k);
    m.cx[c] = (float)f.cx[c];
    m.cy[c] = (float)f.cy[c];
    if (j <= L.nx && k <= L.ny) {
      m.di[c] = (float)f.di[c];
      if (m.mi) m.mi[c] = (float)f.mi[c];
    }
  }
}

// Trial residual in FP64 of the corrected solution: r = u0 - A (u + d), with off-domain
// neighbours mirrored (the reflective halo copy, or a value multiplied by a zero boundary
// coefficient), so u's halo is not needed.  r32 = r; ||r||^2 and ||r32||^2 in FP64, and the
// squared norm of the per-cell magnitude sum |u0| + |Di u| + sum |c u_nb|: FP64 rounding of u
// and of the residual arithmetic leaves r uncertain by a small multiple of eps_64 times it,
// the level below which no correction can lower the true residual.
// With jac_diag also r.(Mi r) and r32.(Mi32 r32).
// first: the start of the CG process, p32 = r32 (z32 = Mi32 r32 with jac_diag) in the buffer the
// next k_mix_w reads as its previous direction.  mirror = false: off-domain neighbours are read from the halo cells as
// they are (u's halo as last exchanged, d's halo zero) -- the operator the reference's
// Chebyshev iteration applies, whose u halo is not exchanged after the switch
// (tea_solve.f90:246-250).
__global__ void k_mix_trial(Fields f, MixFields m, Layout L, Reduce rd, MixState* ms, bool first, bool mirror) {
  double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  float* __restrict__ p0 = (ms->n & 1) ? m.p : m.p2;
  const float* __restrict__ mi32 = m.mi;
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  for (int k = blockIdx.y + 1; k <= L.ny; k += gridDim.y) {
    if (j > L.nx) continue;
    const long long c = L.at(j, k);
    const long long cl = (j > 1 || !mirror) ? c - 1 : c, cr = (j < L.nx || !mirror) ? c + 1 : c;
    const long long cb = (k > 1 || !mirror) ? c - L.ld : c, ct = (k < L.ny || !mirror) ? c + L.ld : c;
    const double uc = f.u[c] + (double)m.d[c];
    const double ul = f.u[cl] + (double)m.d[cl], ur = f.u[cr] + (double)m.d[cr];
    const double ub = f.u[cb] + (double)m.d[cb], ut = f.u[ct] + (double)m.d[ct];
    double a = f.di[c] * uc;
    a = fma(-f.cy[c + L.ld], ut, a);
    a = fma(-f.cy[c], ub, a);
    a = fma(-f.cx[c + 1], ur, a);
    a = fma(-f.cx[c], ul, a);
    const double r = f.u0[c] - a;
    acc[0] = fma(r, r, acc[0]);
    const float r32 = (float)r;
    m.r[c] = r32;
    acc[1] = fma((double)r32, (double)r32, acc[1]);
    if (mi32) {
      const float z32 = mi32[c] * r32;
      m.z[c] = z32;
      if (first) p0[c] = z32;
      acc[3] = fma(r, f.mi[c] * r, acc[3]);
      acc[4] = fma((double)r32, (double)z32, acc[4]);
    } else if (first) {
      p0[c] = r32;
    }
    const double s = fabs(f.u0[c]) + fabs(f.di[c] * uc) + fabs(f.cy[c + L.ld] * ut) + fabs(f.cy[c] * ub) +
                     fabs(f.cx[c + 1] * ur) + fabs(f.cx[c] * ul);
    acc[2] = fma(s, s, acc[2]);
  }
  if (!mi32) {
    acc[3] = acc[0];
    acc[4] = acc[1];
  }
  grid_reduce<5>(acc, rd, EpiMixTrial{ms});
}


// Four adjacent columns (ja .. ja+3) per thread: 16-byte loads of every FP32 stream.
struct F4 {
  float v[4];
  __device__ __forceinline__ void load(const float* __restrict__ p, long long c) {
    const float4 q = *reinterpret_cast<const float4*>(p + c);
    v[0] = q.x, v[1] = q.y, v[2] = q.z, v[3] = q.w;
  }
  __device__ __forceinline__ void store(float* __restrict__ p, long long c, int nv) const {
    if (nv == 4) {
      *reinterpret_cast<float4*>(p + c) = make_float4(v[0], v[1], v[2], v[3]);
    } else {
      for (int i = 0; i < nv; ++i) p[c + i] = v[i];
    }
  }
};

// Rows of the FP32 sweep's inputs are staged into a shared-memory ring MP rows ahead by
// asynchronous copies (cp.async); a staged row holds p_old, r (with the strip's two halo
// columns), cy, cx (with the strip's right face), Di and d.  Column col of a strip starting at
// js sits at index col - js + 4, so interior columns are 16-byte aligned.
constexpr int MP = 2;               // rows staged ahead
constexpr int MNS = MP + 3;         // ring slots: rows k-1 .. k+1+MP
constexpr int MRW = MSW + 8;        // floats per staged array row
constexpr int MARR = 6;             // staged arrays: p_old, r, cy, cx, di, d
constexpr int MIX_W_SMEM = (MNS * MARR * MRW + 2 * (MSW + 2)) * 4;

__device__ __forceinline__ void mix_cp16(float* dst, const float* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src));
}
__device__ __forceinline__ void mix_cp4(float* dst, const float* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(src));
}
__device__ __forceinline__ void mix_commit() { asm volatile("cp.async.commit_group;"); }
template <int N>
__device__ __forceinline__ void mix_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N)); }

// p_n = r + beta p_{n-1} (z in place of r with jac_diag; FP32), w = A p_n (FP32), p.w (Dot2),
// deferred d += alpha p_{n-1}.
// Same row march as the FP64 sweep (tl_fused.cu), four columns per thread, with the inputs of
// row k+1+MP staged while row k is computed.
__global__ void __launch_bounds__(MT) k_mix_w(MixFields m, Layout L, Reduce rd, MixState* ms, int rows_per_cta) {
  if (ms->status != RUN) return;
  const int n = ms->n;
  const float beta = (float)ms->beta;
  const bool upd = ms->p_pending != 0;
  const bool upd_d = ms->d_pending != 0;
  const float da = (float)ms->d_alpha;
  const float* __restrict__ pold = (n & 1) ? m.p : m.p2;
  float* __restrict__ pout = (n & 1) ? m.p2 : m.p;
  const float* __restrict__ r = m.mi ? m.z : m.r;  // the source of the p update: z with jac_diag
  extern __shared__ __align__(16) float mix_smem[];
  float(*buf)[MSW + 2] = reinterpret_cast<float(*)[MSW + 2]>(mix_smem + MNS * MARR * MRW);
  const int t = threadIdx.x;
  const int js = blockIdx.x * MSW + 1;
  const int ja = js + 4 * t;
  const int nv = min(4, L.nx - ja + 1);  // interior columns this thread owns
  const bool active = nv > 0;
  const int k0 = blockIdx.y * rows_per_cta + 1;
  const int k1 = min(k0 + rows_per_cta - 1, L.ny);
  const int o = 4 * t + 4;  // this thread's first column in a staged row
  auto arr = [&](int row, int a) { return mix_smem + ((row - k0 + 1) % MNS * MARR + a) * MRW; };
  enum { A_P = 0, A_R = 1, A_CY = 2, A_CX = 3, A_DI = 4, A_D = 5 };
  // four columns ja.. of a row of src into dst + o (16-byte copy when all are interior)
  auto stage4 = [&](float* dst, const float* src, long long c, int hi) {
    if (ja + 3 <= hi) {
      mix_cp16(dst + o, src + c);
    } else {
      for (int i = 0; i < 4; ++i)
        if (ja + i <= hi) dst[o + i] = src[c + i];
    }
  };
  // stage row `row` (rows k0-1 .. k1+1; what each array needs of it); one commit group
  auto stage_row = [&](int row) {
    if (row >= 1 && row <= L.ny + 1 && row >= k0 - 1 && row <= k1 + 1) {
      const long long c = L.at(ja, row);
      if (row <= L.ny) {
        if (active) {
          stage4(arr(row, A_P), pold, c, L.nx);
          if (upd) stage4(arr(row, A_R), r, c, L.nx);
        }
        if (t == 0 && js > 1) {  // left halo column js-1
          const long long ch = L.at(js - 1, row);
          mix_cp4(arr(row, A_P) + 3, pold + ch);
          if (upd) mix_cp4(arr(row, A_R) + 3, r + ch);
        }
        if (t == MT - 1 && js + MSW <= L.nx) {  // right halo column js+MSW
          const long long ch = L.at(js + MSW, row);
          mix_cp4(arr(row, A_P) + MSW + 4, pold + ch);
          if (upd) mix_cp4(arr(row, A_R) + MSW + 4, r + ch);
        }
      }
      if (row >= k0) {
        if (active) stage4(arr(row, A_CY), m.cy, c, L.nx);
        if (row <= k1) {
          // cx up to the boundary face nx+1: a thread's column ja+4 is staged by the next
          // thread (also when that one owns no interior column), the strip's last by the last
          if (ja <= L.nx + 1) stage4(arr(row, A_CX), m.cx, c, L.nx + 1);
          if (t == MT - 1 && js + MSW <= L.nx + 1) mix_cp4(arr(row, A_CX) + MSW + 4, m.cx + L.at(js + MSW, row));
          if (active) {
            stage4(arr(row, A_DI), m.di, c, L.nx);
            if (upd_d) stage4(arr(row, A_D), m.d, c, L.nx);
          }
        }
      }
    }
    mix_commit();
  };
  // p_n of four columns of a staged row (old: p_{n-1} there)
  auto pnew = [&](int row, F4& q, F4& old) {
    const float* sp = arr(row, A_P) + o;
    const float* sr = arr(row, A_R) + o;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      old.v[i] = sp[i];
      q.v[i] = upd ? fmaf(beta, sp[i], sr[i]) : sp[i];
    }
  };
  auto pnew1 = [&](int row, int idx) {
    const float po = arr(row, A_P)[idx];
    return upd ? fmaf(beta, po, arr(row, A_R)[idx]) : po;
  };
  // prologue: rows k0-1 .. k0+MP
  for (int rr = k0 - 1; rr <= k0 + MP; ++rr) stage_row(rr);
  mix_wait<MP>();  // rows k0-1 and k0 have landed
  __syncthreads();
  Dot2 dot;
  F4 pm{}, pc{}, pnx{}, cyc{}, oc{}, onx{}, junk{};
  if (active) {
    pnew(k0, pc, oc);
    if (k0 == 1)
      pm = pc;
    else
      pnew(k0 - 1, pm, junk);
    const float* sc = arr(k0, A_CY) + o;
#pragma unroll
    for (int i = 0; i < 4; ++i) cyc.v[i] = sc[i];
  }
  for (int k = k0; k <= k1; ++k) {
    const int b = k & 1;
    const long long c = L.at(ja, k);
    stage_row(k + 1 + MP);
    if (active) {
#pragma unroll
      for (int i = 0; i < 4; ++i) buf[b][4 * t + 1 + i] = pc.v[i];
    }
    if (t == 0 && js > 1) buf[b][0] = pnew1(k, 3);
    if (t == MT - 1 && js + MSW <= L.nx) buf[b][MSW + 1] = pnew1(k, MSW + 4);
    mix_wait<MP>();  // row k+1 has landed
    __syncthreads();
    if (active) {
      F4 cyn, cx4, dd, dv, w;
      if (k == L.ny)
        pnx = pc;
      else
        pnew(k + 1, pnx, onx);
      const float* scy = arr(k + 1, A_CY) + o;
      const float* scx = arr(k, A_CX) + o;
      const float* sdi = arr(k, A_DI) + o;
      const float* sd = arr(k, A_D) + o;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        cyn.v[i] = scy[i];
        cx4.v[i] = scx[i];
        dd.v[i] = sdi[i];
        dv.v[i] = upd_d ? sd[i] : 0.f;
      }
      const float cxr = (nv == 4) ? scx[4] : 0.f;  // the next thread's first column, or the right face
      const float left0 = (ja == 1) ? pc.v[0] : buf[b][4 * t];
      const float right3 = buf[b][4 * t + 5];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const float left = (i == 0) ? left0 : pc.v[i - 1];
        float right = (i < 3) ? pc.v[i + 1] : right3;
        if (ja + i == L.nx) right = pc.v[i];  // mirror at the domain edge
        const float cright = (i < 3) ? cx4.v[i + 1] : cxr;
        float a = dd.v[i] * pc.v[i];
        a = fmaf(-cyn.v[i], pnx.v[i], a);
        a = fmaf(-cyc.v[i], pm.v[i], a);
        a = fmaf(-cright, right, a);
        a = fmaf(-cx4.v[i], left, a);
        w.v[i] = a;
        if (i < nv) dot.add(a, pc.v[i]);
      }
      w.store(m.w, c, nv);
      pc.store(pout, c, nv);
      if (upd_d) {
#pragma unroll
        for (int i = 0; i < 4; ++i) dv.v[i] = fmaf(da, oc.v[i], dv.v[i]);
        dv.store(m.d, c, nv);
      }
      cyc = cyn;
    }
    pm = pc;
    pc = pnx;
    oc = onx;
  }
  mix_wait<0>();
  double acc[1] = {dot.value()};
  grid_reduce<1>(acc, rd, EpiMixW{ms});
}

// r -= alpha w (FP32), r.r (Dot2; with jac_diag z = Mi32 r written and r.z), inner epilogue.
// Four columns per thread.
template <bool PRE>
__global__ void __launch_bounds__(MT) k_mix_ur(MixFields m, Layout L, Reduce rd, MixState* ms) {
  if (ms->status != RUN) return;
  const float alpha = (float)ms->alpha;
  const int ja = blockIdx.x * MSW + 1 + 4 * threadIdx.x;
  const int nv = min(4, L.nx - ja + 1);
  Dot2 dot;
  if (nv > 0) {
    // four rows per pass with every load issued before any use (memory-level parallelism)
    const int gy = gridDim.y;
    for (int k = blockIdx.y + 1; k <= L.ny; k += 4 * gy) {
      F4 ww[4], rr[4], mm[PRE ? 4 : 1];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (k + u * gy <= L.ny) {
          const long long c = L.at(ja, k + u * gy);
          ww[u].load(m.w, c);
          rr[u].load(m.r, c);
          if constexpr (PRE) mm[u].load(m.mi, c);
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (k + u * gy <= L.ny) {
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            rr[u].v[i] = fmaf(-alpha, ww[u].v[i], rr[u].v[i]);
            if constexpr (PRE) {
              mm[u].v[i] *= rr[u].v[i];  // z = Mi32 r
              if (i < nv) dot.add(rr[u].v[i], mm[u].v[i]);
            } else {
              if (i < nv) dot.add(rr[u].v[i], rr[u].v[i]);
            }
          }
          if constexpr (PRE) mm[u].store(m.z, L.at(ja, k + u * gy), nv);
          rr[u].store(m.r, L.at(ja, k + u * gy), nv);
        }
      }
    }
  }
  double acc[1] = {dot.value()};
  grid_reduce<1>(acc, rd, EpiMixUr{ms});
}


// d += alpha p when the deferred update of the last step is pending.
__global__ void k_mix_flush_d(MixFields m, Layout L, MixState* ms) {
  if (!ms->d_pending) return;
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (j > L.nx) return;
  const float da = (float)ms->d_alpha;
  const float* __restrict__ p = ms->d_psel ? m.p2 : m.p;
  for (int k = blockIdx.y + 1; k <= L.ny; k += gridDim.y) {
    const long long c = L.at(j, k);
    m.d[c] = fmaf(da, p[c], m.d[c]);
  }
}

// Accept the correction: u += d in FP64, d = 0.
__global__ void k_mix_apply(Fields f, MixFields m, Layout L) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (j > L.nx) return;
  for (int k = blockIdx.y + 1; k <= L.ny; k += gridDim.y) {
    const long long c = L.at(j, k);
    f.u[c] = f.u[c] + (double)m.d[c];
    m.d[c] = 0.f;
  }
}


inline int mstrips(const Layout& L) { return (L.nx + MSW - 1) / MSW; }

}  // namespace

void launch_mix_prep(const Fields& f, const MixFields& m, const Layout& L, cudaStream_t s) {
  dim3 grid((L.nx + 1 + 255) / 256, L.ny + 1 > 65535 ? 65535 : L.ny + 1);
  { ++launch_counter(); k_mix_prep<<<grid, 256, 0, s>>>(f, m, L); }
}

void launch_mix_trial(const Fields& f, const MixFields& m, const Layout& L, const Reduce& rd, MixState* ms,
                      bool first, cudaStream_t s, bool mirror) {
  dim3 grid((L.nx + 255) / 256, L.ny < 256 ? L.ny : 256);
  { ++launch_counter(); k_mix_trial<<<grid, 256, 0, s>>>(f, m, L, rd, ms, first, mirror); }
}

void launch_mix_flush_d(const MixFields& m, const Layout& L, MixState* ms, cudaStream_t s) {
  dim3 grid((L.nx + 255) / 256, L.ny < 4096 ? L.ny : 4096);
  { ++launch_counter(); k_mix_flush_d<<<grid, 256, 0, s>>>(m, L, ms); }
}

long long mix_w_slots() {
  static const long long slots = resident_ctas((const void*)k_mix_w, MT, MIX_W_SMEM);
  return slots;
}

int prepare_mix_kernels() {
  if (cudaFuncSetAttribute(k_mix_w, cudaFuncAttributeMaxDynamicSharedMemorySize, MIX_W_SMEM) != cudaSuccess) return -1;
  mix_w_slots();  // the occupancy query needs the attribute above
  return 0;
}

void launch_mix_iteration(const MixFields& m, const Layout& L, const Reduce& rd, MixState* ms, cudaStream_t s,
                          cudaEvent_t between) {
  const int ns = mstrips(L);
  // whole waves of co-resident CTAs (three per SM: the staging ring's shared memory)
  int rows = wave_rows(L.ny, ns, mix_w_slots());
  const int min_rows = (int)(((long long)L.ny * ns + MAX_REDUCE_BLOCKS - 1) / MAX_REDUCE_BLOCKS);
  if (rows < min_rows) rows = min_rows;
  { ++launch_counter(); k_mix_w<<<dim3(ns, (L.ny + rows - 1) / rows), MT, MIX_W_SMEM, s>>>(m, L, rd, ms, rows); }
  if (between) cudaEventRecord(between, s);
  // about 2048 CTAs striding over rows, as the FP64 update sweep (fewer partials to sum)
  int gy = (2048 + ns - 1) / ns;
  if (gy > L.ny) gy = L.ny;
  if ((long long)gy * ns > MAX_REDUCE_BLOCKS) gy = MAX_REDUCE_BLOCKS / ns;
  if (m.mi)
    { ++launch_counter(); k_mix_ur<true><<<dim3(ns, gy), MT, 0, s>>>(m, L, rd, ms); }
  else
    { ++launch_counter(); k_mix_ur<false><<<dim3(ns, gy), MT, 0, s>>>(m, L, rd, ms); }
}

void launch_mix_apply(const Fields& f, const MixFields& m, const Layout& L, cudaStream_t s) {
  dim3 grid((L.nx + 255) / 256, L.ny < 4096 ? L.ny : 4096);
  { ++launch_counter(); k_mix_apply<<<grid, 256, 0, s>>>(f, m, L); }
}

}  // namespace tl
