// tl_fused.cu -- fused solver-loop kernels: the iteration bodies of tea_leaf()
// (tea_solve.f90:152-414) with every solver scalar kept in device memory (LoopState).
//
// FP64 CG, per iteration n (tea_solve.f90:341-369):
//   k_fused_cg_w : p_n = src + beta*p_{n-1} (cg_kernel.f90:306-347, deferred from iteration
//                  n-1), w = A p_n, pw = p_n.w (cg_kernel.f90:114-156); epilogue alpha = rro/pw.
//   k_fused_cg_ur: u += alpha p_n, r -= alpha w, rrn = r.r (cg_kernel.f90:198-304); epilogue
//                  beta = rrn/rro, error = sqrt|rrn|, the EXIT test, n = n+1.
// p_{n-1} and p_n live in two buffers (P[(n-1)&1] -> P[n&1]) so that the CTA computing a
// halo row of p_n never sees a neighbour's already-updated value.
//
// FP64 PPCG outer iteration (tea_solve.f90:289-331): k_fused_cg_w<PPCG> (p = z + beta p,
// w = A p, p.w, r_store = r, z.r, alpha), k_fused_cg_ur in a PPCG mode (u, r updates, init_sd),
// the inner sweeps, then k_fused_ppcg_rrn (z = utemp, (r - r_store).z, beta, the EXIT test).
// Also here: the persistent cooperative CG kernel for small meshes and the device-resident
// Jacobi sweep.
//
// The matvec kernel marches up a strip of 2*FT columns, one row per step: each thread owns
// two adjacent columns (16-byte loads), keeps p of rows k-1, k, k+1 in registers and swaps
// row k through shared memory for the horizontal neighbours; the two strip-edge columns
// and the first/last row of a CTA are recomputed (p = src + beta*p costs one FMA).  Off the
// domain the neighbour is the mirror value (the reference's reflective halo copy of p, or a
// value multiplied by a zero boundary coefficient otherwise).  The form launched by default,
// k_fused_cg_ws, stages each row step's inputs into shared memory one row step ahead.
#include "tl_kernels.cuh"

namespace tl {

namespace {

constexpr int FT = 128;      // threads per CTA
constexpr int SW = 2 * FT;   // strip width (columns)

__device__ __forceinline__ void finish_iteration(LoopState* st, double err_raw) {
  const double err = sqrt(fabs(err_raw));
  st->error = err;
  if (!isfinite(err)) {
    st->status = EXIT_BREAKDOWN;
    st->n_exit = st->n;
    return;
  }
  if (fabs(err) < st->eps * st->initial_residual) {
    st->status = EXIT_CONVERGED;
    st->n_exit = st->n;
    return;
  }
  st->old_error = err;
  st->n += 1;
  if (st->n > st->max_iters) {
    st->status = EXIT_MAX_ITERS;
    st->n_exit = st->n;
    return;
  }
  if (st->check_switch) {
    // tea_solve.f90:160-174 evaluated for the next iteration (cheby_calc_steps == 0 here)
    const bool sw = (!st->first && st->use_ppcg && st->n > 1) ||
                    (fabs(st->old_error) <= st->epslim && st->n >= st->presteps);
    if (sw) st->status = STOP_SWITCH;
  }
}

// the matvec sweep's sums: p.w (CG), and z.r (PPCG)
template <bool PPCG>
struct EpiCgW {
  static constexpr int NV = PPCG ? 2 : 1;
  Reduce rd;
  __device__ void operator()(double (&acc)[NV]) const {
    LoopState* st = rd.st;
    st->u_pending = 0;  // every CTA applied the deferred u update for its cells
    st->pw = acc[0];
    if constexpr (PPCG) st->rro = acc[1];  // tea_leaf_ppcg_calc_zrnorm, allsum2 (tea_solve.f90:300-303)
    const double alpha = st->rro / st->pw;
    st->alpha = alpha;
    if constexpr (!PPCG) rd.hist_a[st->n] = alpha;
    if (!isfinite(alpha)) {
      st->status = EXIT_BREAKDOWN;
      st->n_exit = st->n;
    }
  }
};

struct EpiCgUr {
  Reduce rd;
  __device__ void operator()(double (&acc)[1]) const {
    LoopState* st = rd.st;
    const double rrn = acc[0];
    st->rrn = rrn;
    const double beta = rrn / st->rro;
    st->beta = beta;
    rd.hist_b[st->n] = beta;
    st->p_pending = 1;
    st->u_pending = 1;  // u += alpha_n p_n, applied by the next matvec sweep or the flush
    st->u_alpha = st->alpha;
    st->u_psel = st->n & 1;
    st->rro = rrn;
    st->cg_calc_steps += 1;
    finish_iteration(st, rrn);
  }
};

// p_new for two adjacent columns (ja, ja+1) of row k
struct PNew {
  const double* __restrict__ src;
  const double* __restrict__ pold;
  double beta;
  bool upd;
  __device__ __forceinline__ double2 pair(long long c) const {
    double2 q = __ldg(reinterpret_cast<const double2*>(pold + c));
    if (upd) {
      const double2 s = __ldg(reinterpret_cast<const double2*>(src + c));
      q.x = fma(beta, q.x, s.x);
      q.y = fma(beta, q.y, s.y);
    }
    return q;
  }
  // same, also returning p_old
  __device__ __forceinline__ double2 pair(long long c, double2& old) const {
    old = __ldg(reinterpret_cast<const double2*>(pold + c));
    double2 q = old;
    if (upd) {
      const double2 s = __ldg(reinterpret_cast<const double2*>(src + c));
      q.x = fma(beta, q.x, s.x);
      q.y = fma(beta, q.y, s.y);
    }
    return q;
  }
  __device__ __forceinline__ double one(long long c) const {
    const double q = __ldg(pold + c);
    return upd ? fma(beta, q, __ldg(src + c)) : q;
  }
};

template <bool PPCG>
__global__ void __launch_bounds__(FT) k_fused_cg_w(LoopArgs a, int rows_per_cta) {
  LoopState* st = a.rd.st;
  if (st->status != RUN) return;
  const Layout L = a.L;
  const int n = st->n;
  const bool use_z = PPCG || a.precond != 1;
  PNew pn_{use_z ? a.f.z : a.f.r, (n & 1) ? a.f.p : a.f.p2, st->beta, st->p_pending != 0};
  double* __restrict__ pout = (n & 1) ? a.f.p2 : a.f.p;
  double* __restrict__ w = a.f.w;
  const double* __restrict__ cx = a.f.cx;
  const double* __restrict__ cy = a.f.cy;
  const double* __restrict__ di = a.f.di;

  __shared__ double buf[2][SW + 2];
  const int t = threadIdx.x;
  const int js = blockIdx.x * SW + 1;
  const int ja = js + 2 * t;
  const bool active = ja <= L.nx;
  const bool has_b = ja + 1 <= L.nx;
  const int k0 = blockIdx.y * rows_per_cta + 1;
  const int k1 = min(k0 + rows_per_cta - 1, L.ny);
  const int ld = L.ld;

  // deferred u += alpha_{n-1} p_{n-1} of the previous iteration (p_{n-1} is pold here)
  const bool upd_u = !PPCG && st->u_pending != 0;
  const double ua = st->u_alpha;
  double* __restrict__ u = a.f.u;

  double acc[EpiCgW<PPCG>::NV] = {};
  double acc_b = 0.0;  // second column's p.w chain, kept separate to shorten the FMA dependency chain
  double2 pm = make_double2(0.0, 0.0), pc = pm, pnx = pm, cyc = pm, oc = pm, onx = pm;
  if (active) {
    pc = pn_.pair(L.at(ja, k0), oc);
    pm = (k0 == 1) ? pc : pn_.pair(L.at(ja, k0 - 1));
    cyc = *reinterpret_cast<const double2*>(cy + L.at(ja, k0));
  }
  for (int k = k0; k <= k1; ++k) {
    const int b = k & 1;
    if (active) {
      if (k == L.ny) {
        pnx = pc;
      } else if (k == k1) {
        pnx = pn_.pair(L.at(ja, k + 1));  // halo row of this CTA: p_new only
      } else {
        pnx = pn_.pair(L.at(ja, k + 1), onx);
      }
      buf[b][2 * t + 1] = pc.x;
      buf[b][2 * t + 2] = pc.y;
    }
    if (t == 0 && js > 1) buf[b][0] = pn_.one(L.at(js - 1, k));
    if (t == FT - 1 && js + SW <= L.nx) buf[b][SW + 1] = pn_.one(L.at(js + SW, k));
    __syncthreads();
    if (active) {
      const long long c = L.at(ja, k);
      const double2 cyn = *reinterpret_cast<const double2*>(cy + c + ld);
      const double2 cxa = *reinterpret_cast<const double2*>(cx + c);
      const double2 dd = *reinterpret_cast<const double2*>(di + c);
      const double left_a = (ja == 1) ? pc.x : buf[b][ja - js];
      const double right_a = has_b ? pc.y : pc.x;
      double wa = dd.x * pc.x;
      wa = fma(-cyn.x, pnx.x, wa);
      wa = fma(-cyc.x, pm.x, wa);
      wa = fma(-cxa.y, right_a, wa);
      wa = fma(-cxa.x, left_a, wa);
      acc[0] = fma(wa, pc.x, acc[0]);
      if (has_b) {
        const double cxr = cx[c + 2];
        const double right_b = (ja + 1 == L.nx) ? pc.y : buf[b][ja - js + 3];
        double wb = dd.y * pc.y;
        wb = fma(-cyn.y, pnx.y, wb);
        wb = fma(-cyc.y, pm.y, wb);
        wb = fma(-cxr, right_b, wb);
        wb = fma(-cxa.y, pc.x, wb);
        acc_b = fma(wb, pc.y, acc_b);
        *reinterpret_cast<double2*>(w + c) = make_double2(wa, wb);
        *reinterpret_cast<double2*>(pout + c) = pc;
        if (upd_u) {
          double2 uu = *reinterpret_cast<const double2*>(u + c);
          uu.x = fma(ua, oc.x, uu.x);
          uu.y = fma(ua, oc.y, uu.y);
          *reinterpret_cast<double2*>(u + c) = uu;
        }
      } else {
        w[c] = wa;
        pout[c] = pc.x;
        if (upd_u) u[c] = fma(ua, oc.x, u[c]);
      }
      if constexpr (PPCG) {
        // tea_leaf_ppcg_store_r (ppcg_kernel.f90:507-530) and calc_zrnorm z.r (:411-451)
        const double2 rr = *reinterpret_cast<const double2*>(a.f.r + c);
        const double2 zz = *reinterpret_cast<const double2*>(a.f.z + c);
        a.f.r_store[c] = rr.x;
        acc[1] = fma(zz.x, rr.x, acc[1]);
        if (has_b) {
          a.f.r_store[c + 1] = rr.y;
          acc[1] = fma(zz.y, rr.y, acc[1]);
        }
      }
      cyc = cyn;
    }
    pm = pc;
    pc = pnx;
    oc = onx;
  }
  acc[0] += acc_b;
  grid_reduce<EpiCgW<PPCG>::NV>(acc, a.rd, EpiCgW<PPCG>{a.rd});
}

// ---- the matvec sweep with its input rows staged one row ahead --------------------------------
// Same arithmetic, row march and results (bit for bit) as k_fused_cg_w.  The inputs a row step
// needs -- p_{n-1} and src of row k+1 (with the strip's two halo columns), cy of row k+1, cx,
// Di and u of row k -- are copied into a two-slot shared-memory ring by
// asynchronous copies (cp.async) one row step before they are used, so the loads' latency
// falls under the previous row's arithmetic instead of stalling it.  Every thread stages
// exactly the columns it reads itself into ring entries no other thread writes (its two
// columns; the right face cx(j+2) of its second one, which is also the next thread's first
// column, into an entry of its own; the strip's halo columns in the two edge threads), so the
// ring needs no barrier: a thread waits only for its own copies (cp.async.wait_group).
//
// Unit m of the ring (slot m & 1) holds p_{n-1}, src and cy of row m and cx, Di, u of row
// m-1; row step k consumes unit k+1 and stages unit k+2 into the slot unit k left.  At 8192^2
// the sweep takes 1.002 ms per launch against 1.026 ms with direct loads (7 CTAs per SM
// instead of 9: the ring's 26 KB per CTA bound them; the block sum at the end reuses the ring
// as its scratch); staging all but u took 1.013 ms.
constexpr int SROW = SW + 4;  // doubles per staged array row; column col at index col - js + 2
constexpr int STAGE_ARRAYS = 6;
constexpr int SSLOT = STAGE_ARRAYS * SROW + FT;  // doubles per slot: the arrays, then cx(j+2) per thread
constexpr size_t STAGE_SMEM = (size_t)2 * SSLOT * sizeof(double);

__device__ __forceinline__ void cp16(double* dst, const double* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src));
}
__device__ __forceinline__ void cp8(double* dst, const double* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// EMU: bit 0 (1) / bit 1 (2) computes the product Di p of the thread's first / second column
// on the integer pipes (dmul_int, the same bits as the FP64 multiply).  The ring bounds the
// sweep to 7 CTAs per SM, so __launch_bounds__(FT, 7) gives the compiler up to 72 registers at
// no cost in occupancy: with both products on the integer pipes (the launched form) the sweep
// takes 0.914 ms per 8192^2 launch against 0.986 ms with FP64 products (1.006 ms with the
// default register limit); one product alone, 0.974 / 0.968 ms.
template <bool PPCG, int EMU = 0>
__global__ void __launch_bounds__(FT, 7) k_fused_cg_ws(LoopArgs a, int rows_per_cta) {
  LoopState* st = a.rd.st;
  if (st->status != RUN) return;
  const Layout L = a.L;
  const int n = st->n;
  const bool use_z = PPCG || a.precond != 1;
  const double* __restrict__ src = use_z ? a.f.z : a.f.r;
  const double* __restrict__ pold = (n & 1) ? a.f.p : a.f.p2;
  const double beta = st->beta;
  const bool upd = st->p_pending != 0;
  double* __restrict__ pout = (n & 1) ? a.f.p2 : a.f.p;
  double* __restrict__ w = a.f.w;
  const double* __restrict__ cx = a.f.cx;
  const double* __restrict__ cy = a.f.cy;
  const double* __restrict__ di = a.f.di;
  const bool upd_u = !PPCG && st->u_pending != 0;
  const double ua = st->u_alpha;
  double* __restrict__ u = a.f.u;

  extern __shared__ __align__(16) double ring[];
  __shared__ double buf[2][SW + 2];
  enum { A_P = 0, A_S, A_CY, A_CX, A_DI, A_U };
  auto arr = [&](int m, int a_) { return ring + (m & 1) * SSLOT + a_ * SROW; };
  auto cxr_at = [&](int m) { return ring + (m & 1) * SSLOT + STAGE_ARRAYS * SROW + threadIdx.x; };

  const int t = threadIdx.x;
  const int js = blockIdx.x * SW + 1;
  const int ja = js + 2 * t;
  const int o = 2 * t + 2;  // this thread's first column in a staged row
  const bool active = ja <= L.nx;
  const bool has_b = ja + 1 <= L.nx;
  const bool left_edge = t == 0 && js > 1;
  const bool right_edge = t == FT - 1 && js + SW <= L.nx;
  const int k0 = blockIdx.y * rows_per_cta + 1;
  const int k1 = min(k0 + rows_per_cta - 1, L.ny);
  const int ld = L.ld;

  // unit m: the copies this thread needs of it (none past the CTA's last row step)
  auto stage = [&](int m) {
    if (m <= k1 + 1) {
      if (m <= L.ny) {  // p_{n-1}, src of row m (row k+1 of step k = m-1; none above the domain)
        const long long c = L.at(ja, m);
        if (active) {
          cp16(arr(m, A_P) + o, pold + c);
          if (upd) cp16(arr(m, A_S) + o, src + c);
        }
        if (left_edge) {
          cp8(arr(m, A_P) + 1, pold + L.at(js - 1, m));
          if (upd) cp8(arr(m, A_S) + 1, src + L.at(js - 1, m));
        }
        if (right_edge) {
          cp8(arr(m, A_P) + SW + 2, pold + L.at(js + SW, m));
          if (upd) cp8(arr(m, A_S) + SW + 2, src + L.at(js + SW, m));
        }
      }
      if (active) {
        const long long c = L.at(ja, m - 1);
        cp16(arr(m, A_CY) + o, cy + c + ld);  // cy of row m: the north face of row m-1
        cp16(arr(m, A_CX) + o, cx + c);
        if (has_b) cp8(cxr_at(m), cx + c + 2);
        cp16(arr(m, A_DI) + o, di + c);
        if (upd_u) cp16(arr(m, A_U) + o, u + c);
      }
    }
    cp_commit();
  };
  auto pnew2 = [&](const double* sp, const double* ss) {
    double2 q = *reinterpret_cast<const double2*>(sp);
    if (upd) {
      const double2 r2 = *reinterpret_cast<const double2*>(ss);
      q.x = fma(beta, q.x, r2.x);
      q.y = fma(beta, q.y, r2.y);
    }
    return q;
  };
  auto pnew1 = [&](const double* sp, const double* ss) { return upd ? fma(beta, *sp, *ss) : *sp; };

  double acc[EpiCgW<PPCG>::NV] = {};
  double acc_b = 0.0;
  double2 pm = make_double2(0.0, 0.0), pc = pm, pnx = pm, cyc = pm, oc = pm, onx = pm;
  double hl = 0.0, hr = 0.0;  // p_n of the strip's halo columns in the current row (edge threads)
  {
    PNew pn_{src, pold, beta, upd};
    if (active) {
      pc = pn_.pair(L.at(ja, k0), oc);
      pm = (k0 == 1) ? pc : pn_.pair(L.at(ja, k0 - 1));
      cyc = *reinterpret_cast<const double2*>(cy + L.at(ja, k0));
    }
    if (left_edge) hl = pn_.one(L.at(js - 1, k0));
    if (right_edge) hr = pn_.one(L.at(js + SW, k0));
  }
  stage(k0 + 1);
  for (int k = k0; k <= k1; ++k) {
    const int b = k & 1;
    if (active) {
      buf[b][2 * t + 1] = pc.x;
      buf[b][2 * t + 2] = pc.y;
    }
    if (left_edge) buf[b][0] = hl;
    if (right_edge) buf[b][SW + 1] = hr;
    stage(k + 2);
    cp_wait<1>();  // unit k+1 has landed
    const int m = k + 1;
    if (active) {
      if (k == L.ny) {
        pnx = pc;
      } else {
        pnx = pnew2(arr(m, A_P) + o, arr(m, A_S) + o);
        if (k < k1) onx = *reinterpret_cast<const double2*>(arr(m, A_P) + o);
      }
    }
    if (k < L.ny) {
      if (left_edge) hl = pnew1(arr(m, A_P) + 1, arr(m, A_S) + 1);
      if (right_edge) hr = pnew1(arr(m, A_P) + SW + 2, arr(m, A_S) + SW + 2);
    }
    __syncthreads();
    if (active) {
      const long long c = L.at(ja, k);
      const double2 cyn = *reinterpret_cast<const double2*>(arr(m, A_CY) + o);
      const double2 cxa = *reinterpret_cast<const double2*>(arr(m, A_CX) + o);
      const double2 dd = *reinterpret_cast<const double2*>(arr(m, A_DI) + o);
      const double left_a = (ja == 1) ? pc.x : buf[b][ja - js];
      const double right_a = has_b ? pc.y : pc.x;
      double wa = (EMU & 1) ? dmul_int(dd.x, pc.x) : dd.x * pc.x;
      wa = fma(-cyn.x, pnx.x, wa);
      wa = fma(-cyc.x, pm.x, wa);
      wa = fma(-cxa.y, right_a, wa);
      wa = fma(-cxa.x, left_a, wa);
      acc[0] = fma(wa, pc.x, acc[0]);
      if (has_b) {
        const double cxr = *cxr_at(m);
        const double right_b = (ja + 1 == L.nx) ? pc.y : buf[b][ja - js + 3];
        double wb = (EMU & 2) ? dmul_int(dd.y, pc.y) : dd.y * pc.y;
        wb = fma(-cyn.y, pnx.y, wb);
        wb = fma(-cyc.y, pm.y, wb);
        wb = fma(-cxr, right_b, wb);
        wb = fma(-cxa.y, pc.x, wb);
        acc_b = fma(wb, pc.y, acc_b);
        *reinterpret_cast<double2*>(w + c) = make_double2(wa, wb);
        *reinterpret_cast<double2*>(pout + c) = pc;
        if (upd_u) {
          double2 uu = *reinterpret_cast<const double2*>(arr(m, A_U) + o);
          uu.x = fma(ua, oc.x, uu.x);
          uu.y = fma(ua, oc.y, uu.y);
          *reinterpret_cast<double2*>(u + c) = uu;
        }
      } else {
        w[c] = wa;
        pout[c] = pc.x;
        if (upd_u) u[c] = fma(ua, oc.x, arr(m, A_U)[o]);
      }
      if constexpr (PPCG) {
        const double2 rr = *reinterpret_cast<const double2*>(a.f.r + c);
        const double2 zz = *reinterpret_cast<const double2*>(a.f.z + c);
        a.f.r_store[c] = rr.x;
        acc[1] = fma(zz.x, rr.x, acc[1]);
        if (has_b) {
          a.f.r_store[c + 1] = rr.y;
          acc[1] = fma(zz.y, rr.y, acc[1]);
        }
      }
      cyc = cyn;
    }
    pm = pc;
    pc = pnx;
    oc = onx;
  }
  cp_wait<0>();
  acc[0] += acc_b;
  __syncthreads();  // every thread is done with the ring: it becomes the block sum's scratch
  grid_reduce_in<EpiCgW<PPCG>::NV>(acc, a.rd, EpiCgW<PPCG>{a.rd}, ring);
}

// ---- the FP64 PPCG inner step as one staged sweep ---------------------------------------------
// tea_leaf_kernel_ppcg_inner (ppcg_kernel.f90:204-310) without a preconditioner, in one pass:
//   rtemp -= A sd_in;  sd_out = a sd_in + b rtemp;  utemp += sd_out
// with every product and sum of the two one-step kernels (k_ppcg_inner_r, k_ppcg_inner_s) in
// their order, so the bits are theirs; sd ping-pongs between its two fields (sd_in is read with
// its neighbours while sd_out is written).  The row march, the two-slot shared-memory ring and
// the thread-private staging are those of k_fused_cg_ws: unit m holds sd_in of row m (the
// thread's two columns and, in entries of its own, the columns left and right of them), cy of
// row m and rtemp, utemp, cx (with the thread's cx(j+2)) and Di of row m-1.  Every 5-point
// operand comes from the field, halo included, as in the one-step kernels.  The products Di sd
// and b rtemp run on the integer pipes (dmul_int).  At 4096^2 a step takes 225.5 us against the
// two kernels' 301.4 us.
constexpr int PSLOT = 6 * SROW + 3 * FT;  // doubles per slot: six arrays, then sd(j-1), sd(j+2), cx(j+2)
constexpr size_t PPCG_SMEM = (size_t)2 * PSLOT * sizeof(double);

__global__ void __launch_bounds__(FT, 7) k_ppcg_inner_ws(Fields f, Layout L, const double* __restrict__ sd_in,
                                                         double* __restrict__ sd_out, double ca, double cb,
                                                         int rows_per_cta) {
  extern __shared__ __align__(16) double pring[];
  enum { B_SD = 0, B_CY, B_RT, B_UT, B_CX, B_DI };
  auto arr = [&](int m, int a_) { return pring + (m & 1) * PSLOT + a_ * SROW; };
  auto own = [&](int m, int e) { return pring + (m & 1) * PSLOT + 6 * SROW + e * FT + threadIdx.x; };
  const double* __restrict__ cx = f.cx;
  const double* __restrict__ cy = f.cy;
  const double* __restrict__ di = f.di;
  double* __restrict__ rtemp = f.rtemp;
  double* __restrict__ utemp = f.utemp;

  const int t = threadIdx.x;
  const int js = blockIdx.x * SW + 1;
  const int ja = js + 2 * t;
  const int o = 2 * t + 2;
  const bool active = ja <= L.nx;
  const bool has_b = ja + 1 <= L.nx;
  const int k0 = blockIdx.y * rows_per_cta + 1;
  const int k1 = min(k0 + rows_per_cta - 1, L.ny);
  const int ld = L.ld;

  auto stage = [&](int m) {
    if (m <= k1 + 1 && active) {
      const long long c = L.at(ja, m);  // row m: up to ny + 1, the halo row
      cp16(arr(m, B_SD) + o, sd_in + c);
      cp8(own(m, 0), sd_in + c - 1);
      if (has_b) cp8(own(m, 1), sd_in + c + 2);
      const long long c0 = c - ld;  // row m - 1
      cp16(arr(m, B_CY) + o, cy + c);
      cp16(arr(m, B_RT) + o, rtemp + c0);
      cp16(arr(m, B_UT) + o, utemp + c0);
      cp16(arr(m, B_CX) + o, cx + c0);
      if (has_b) cp8(own(m, 2), cx + c0 + 2);
      cp16(arr(m, B_DI) + o, di + c0);
    }
    cp_commit();
  };

  double2 sm = make_double2(0.0, 0.0), sc = sm, sn = sm, cyc = sm;
  double nl = 0.0, nr = 0.0;  // sd_in of the columns left and right of the thread's two, row k
  if (active) {
    const long long c = L.at(ja, k0);
    sc = *reinterpret_cast<const double2*>(sd_in + c);
    sm = *reinterpret_cast<const double2*>(sd_in + c - ld);
    cyc = *reinterpret_cast<const double2*>(cy + c);
    nl = sd_in[c - 1];
    if (has_b) nr = sd_in[c + 2];
  }
  stage(k0 + 1);
  for (int k = k0; k <= k1; ++k) {
    stage(k + 2);
    cp_wait<1>();  // unit k+1 has landed
    const int m = k + 1;
    double nl_n = nl, nr_n = nr;
    if (active) {
      sn = *reinterpret_cast<const double2*>(arr(m, B_SD) + o);
      nl_n = *own(m, 0);
      if (has_b) nr_n = *own(m, 1);
      const long long c = L.at(ja, k);
      const double2 cyn = *reinterpret_cast<const double2*>(arr(m, B_CY) + o);
      const double2 cxa = *reinterpret_cast<const double2*>(arr(m, B_CX) + o);
      const double2 dd = *reinterpret_cast<const double2*>(arr(m, B_DI) + o);
      double2 rt = *reinterpret_cast<const double2*>(arr(m, B_RT) + o);
      double2 ut = *reinterpret_cast<const double2*>(arr(m, B_UT) + o);
      // apply_A of the one-step kernels: Di v, then north, south, east, west
      double wa = dmul_int(dd.x, sc.x);
      wa = fma(-cyn.x, sn.x, wa);
      wa = fma(-cyc.x, sm.x, wa);
      wa = fma(-cxa.y, sc.y, wa);
      wa = fma(-cxa.x, nl, wa);
      rt.x = rt.x - wa;
      const double sda = fma(ca, sc.x, dmul_int(cb, rt.x));
      ut.x = ut.x + sda;
      if (has_b) {
        double wb = dmul_int(dd.y, sc.y);
        wb = fma(-cyn.y, sn.y, wb);
        wb = fma(-cyc.y, sm.y, wb);
        wb = fma(-*own(m, 2), nr, wb);
        wb = fma(-cxa.y, sc.x, wb);
        rt.y = rt.y - wb;
        const double sdb = fma(ca, sc.y, dmul_int(cb, rt.y));
        ut.y = ut.y + sdb;
        *reinterpret_cast<double2*>(rtemp + c) = rt;
        *reinterpret_cast<double2*>(utemp + c) = ut;
        *reinterpret_cast<double2*>(sd_out + c) = make_double2(sda, sdb);
      } else {
        rtemp[c] = rt.x;
        utemp[c] = ut.x;
        sd_out[c] = sda;
      }
      cyc = cyn;
    }
    sm = sc;
    sc = sn;
    nl = nl_n;
    nr = nr_n;
  }
  cp_wait<0>();
}

// ---- the FP64 Chebyshev iteration as one staged sweep -----------------------------------------
// tea_leaf_kernel_cheby_iterate (cheby_kernel.f90:111-200) without a preconditioner, in one pass:
//   w = A u_in;  r = u0 - w;  p = a p + b r;  u_out = u_in + p
// with every product and sum of the two one-step kernels (k_cheby_wr, k_cheby_iter_pu) in their
// order, so the bits, and the w, r and p the reference leaves behind, are theirs; u ping-pongs
// between its two fields.  Same ring and staging as k_ppcg_inner_ws: unit m holds u_in of row m
// (with the columns left and right of the thread's two), cy of row m and u0, p, cx (with cx(j+2))
// and Di of row m-1.  Di u and b r run on the integer pipes.  WR = false leaves w and r
// unwritten: the solve asks for them only on the iterations whose residual it reads and on its
// last (it forms them afterwards if it stops on another), so the fields it leaves behind are the
// reference's.  At 4096^2 an iteration takes 224 us (254 us writing w and r every time) against
// the two kernels' 302 us.
template <bool WR>
__global__ void __launch_bounds__(FT, 7) k_cheby_iter_ws(Fields f, Layout L, const double* __restrict__ u_in,
                                                         double* __restrict__ u_out, double ca, double cb,
                                                         int rows_per_cta) {
  extern __shared__ __align__(16) double cring[];
  enum { B_U = 0, B_CY, B_U0, B_P, B_CX, B_DI };
  auto arr = [&](int m, int a_) { return cring + (m & 1) * PSLOT + a_ * SROW; };
  auto own = [&](int m, int e) { return cring + (m & 1) * PSLOT + 6 * SROW + e * FT + threadIdx.x; };
  const double* __restrict__ cx = f.cx;
  const double* __restrict__ cy = f.cy;
  const double* __restrict__ di = f.di;
  const double* __restrict__ u0 = f.u0;
  double* __restrict__ pp = f.p;
  double* __restrict__ w = f.w;
  double* __restrict__ r = f.r;

  const int t = threadIdx.x;
  const int js = blockIdx.x * SW + 1;
  const int ja = js + 2 * t;
  const int o = 2 * t + 2;
  const bool active = ja <= L.nx;
  const bool has_b = ja + 1 <= L.nx;
  const int k0 = blockIdx.y * rows_per_cta + 1;
  const int k1 = min(k0 + rows_per_cta - 1, L.ny);
  const int ld = L.ld;

  auto stage = [&](int m) {
    if (m <= k1 + 1 && active) {
      const long long c = L.at(ja, m);  // row m: up to ny + 1, the halo row
      cp16(arr(m, B_U) + o, u_in + c);
      cp8(own(m, 0), u_in + c - 1);
      if (has_b) cp8(own(m, 1), u_in + c + 2);
      const long long c0 = c - ld;  // row m - 1
      cp16(arr(m, B_CY) + o, cy + c);
      cp16(arr(m, B_U0) + o, u0 + c0);
      cp16(arr(m, B_P) + o, pp + c0);
      cp16(arr(m, B_CX) + o, cx + c0);
      if (has_b) cp8(own(m, 2), cx + c0 + 2);
      cp16(arr(m, B_DI) + o, di + c0);
    }
    cp_commit();
  };

  double2 um = make_double2(0.0, 0.0), uc = um, un = um, cyc = um;
  double nl = 0.0, nr = 0.0;  // u_in of the columns left and right of the thread's two, row k
  if (active) {
    const long long c = L.at(ja, k0);
    uc = *reinterpret_cast<const double2*>(u_in + c);
    um = *reinterpret_cast<const double2*>(u_in + c - ld);
    cyc = *reinterpret_cast<const double2*>(cy + c);
    nl = u_in[c - 1];
    if (has_b) nr = u_in[c + 2];
  }
  stage(k0 + 1);
  for (int k = k0; k <= k1; ++k) {
    stage(k + 2);
    cp_wait<1>();  // unit k+1 has landed
    const int m = k + 1;
    double nl_n = nl, nr_n = nr;
    if (active) {
      un = *reinterpret_cast<const double2*>(arr(m, B_U) + o);
      nl_n = *own(m, 0);
      if (has_b) nr_n = *own(m, 1);
      const long long c = L.at(ja, k);
      const double2 cyn = *reinterpret_cast<const double2*>(arr(m, B_CY) + o);
      const double2 cxa = *reinterpret_cast<const double2*>(arr(m, B_CX) + o);
      const double2 dd = *reinterpret_cast<const double2*>(arr(m, B_DI) + o);
      const double2 u0v = *reinterpret_cast<const double2*>(arr(m, B_U0) + o);
      const double2 pv = *reinterpret_cast<const double2*>(arr(m, B_P) + o);
      // apply_A of the one-step kernels: Di v, then north, south, east, west
      double wa = dmul_int(dd.x, uc.x);
      wa = fma(-cyn.x, un.x, wa);
      wa = fma(-cyc.x, um.x, wa);
      wa = fma(-cxa.y, uc.y, wa);
      wa = fma(-cxa.x, nl, wa);
      const double ra = u0v.x - wa;
      const double pa = fma(ca, pv.x, dmul_int(cb, ra));
      const double ua = uc.x + pa;
      if (has_b) {
        double wb = dmul_int(dd.y, uc.y);
        wb = fma(-cyn.y, un.y, wb);
        wb = fma(-cyc.y, um.y, wb);
        wb = fma(-*own(m, 2), nr, wb);
        wb = fma(-cxa.y, uc.x, wb);
        const double rb = u0v.y - wb;
        const double pb = fma(ca, pv.y, dmul_int(cb, rb));
        const double ub = uc.y + pb;
        if (WR) {
          *reinterpret_cast<double2*>(w + c) = make_double2(wa, wb);
          *reinterpret_cast<double2*>(r + c) = make_double2(ra, rb);
        }
        *reinterpret_cast<double2*>(pp + c) = make_double2(pa, pb);
        *reinterpret_cast<double2*>(u_out + c) = make_double2(ua, ub);
      } else {
        if (WR) {
          w[c] = wa;
          r[c] = ra;
        }
        pp[c] = pa;
        u_out[c] = ua;
      }
      cyc = cyn;
    }
    um = uc;
    uc = un;
    nl = nl_n;
    nr = nr_n;
  }
  cp_wait<0>();
}

// ---- persistent cooperative CG (small meshes) ----------------------------------------------
// One cooperative launch runs up to `max_run` iterations of the CG loop (tea_solve.f90:341-369)
// with grid barriers instead of kernel boundaries; the launch and reduction latency of two
// kernels per iteration dominates below about a million cells.  Per iteration:
//   phase A  p_n = src + beta p_{n-1} (neighbours' p_n recomputed in place), w = A p_n, p.w;
//   barrier; every CTA sums the per-CTA partials in the same fixed order -> alpha;
//   phase B  u += alpha p_n, r -= alpha w (z = Mi r for jac_diag), r.z;
//   barrier; every CTA sums -> beta, error, the EXIT / switch tests of finish_iteration.
// Each CTA runs the epilogues on its own shared-memory copy of the loop state (the sums are
// identical, so are the decisions); CTA 0 writes the alpha/beta history and, at the end, the
// state.  u is updated in phase B, so no update is left pending.
// The grid barrier is an arrival counter and a generation word; a wait gives up after
// PB_SPIN_LIMIT polls (about a second), sets the error word, and every CTA returns with
// status EXIT_TIMEOUT instead of waiting longer.
constexpr int PB_T = 256;
constexpr unsigned long long PB_SPIN_LIMIT = 1ull << 22;  // polls of >= 64 ns plus two L2 atomics each

__device__ __forceinline__ bool pb_barrier(unsigned* arrive, unsigned* gen, unsigned* err, unsigned nblocks) {
  __shared__ int failed;
  __syncthreads();
  if (threadIdx.x == 0) {
    failed = 0;
    const unsigned g = atomicAdd(gen, 0u);
    __threadfence();
    if (atomicAdd(arrive, 1u) == nblocks - 1) {
      atomicExch(arrive, 0u);
      __threadfence();
      atomicAdd(gen, 1u);
    } else {
      unsigned long long spins = 0;
      while (atomicAdd(gen, 0u) == g) {
        if (atomicAdd(err, 0u) != 0u || ++spins > PB_SPIN_LIMIT) {
          atomicExch(err, 1u);
          failed = 1;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return failed == 0;
}

// sum of partials[0 .. nb) in a fixed order; the same bits in every CTA
__device__ __forceinline__ double pb_total(const double* partials, int nb, double* scratch, double* bcast) {
  double v[1] = {0.0};
  for (int b = threadIdx.x; b < nb; b += PB_T) v[0] += __ldcg(partials + b);
  block_sum<1>(v, scratch);
  if (threadIdx.x == 0) *bcast = v[0];
  __syncthreads();
  return *bcast;
}

// extra_arrivals: arrivals the barriers wait for beyond the grid's CTAs -- 0, except in the test
// of the bounded wait (an arrival that never comes)
__global__ void __launch_bounds__(PB_T) k_persistent_cg(LoopArgs a, int max_run, unsigned* bar, int extra_arrivals) {
  __shared__ LoopState S;
  __shared__ double scratch[MAX_REDUCE_THREADS];
  __shared__ double bcast;
  const Layout L = a.L;
  const unsigned nb = gridDim.x;
  const unsigned nwait = nb + (unsigned)extra_arrivals;
  unsigned* arrive = bar;
  unsigned* gen = bar + 1;
  unsigned* err = bar + 2;
  if (threadIdx.x == 0) S = *a.rd.st;
  __syncthreads();
  const bool use_z = a.precond != 1;
  const double* __restrict__ src = use_z ? a.f.z : a.f.r;
  const long long ncell = (long long)L.nx * L.ny;
  const long long stride = (long long)nb * PB_T;
  double* partA = a.rd.partials;
  double* partB = a.rd.partials + nb;
  int done = 0;
  bool ok = true;
  while (S.status == RUN && done < max_run) {
    const int n = S.n;
    const double* __restrict__ pold = (n & 1) ? a.f.p : a.f.p2;
    double* __restrict__ pout = (n & 1) ? a.f.p2 : a.f.p;
    const bool upd = S.p_pending != 0;
    const double beta = S.beta;
    auto pn = [&](long long c) { return upd ? fma(beta, pold[c], src[c]) : pold[c]; };
    // ---- phase A: p_n, w = A p_n, p.w ----
    double acc[1] = {0.0};
    for (long long i = (long long)blockIdx.x * PB_T + threadIdx.x; i < ncell; i += stride) {
      const int j = (int)(i % L.nx) + 1, k = (int)(i / L.nx) + 1;
      const long long c = L.at(j, k);
      const double pc = pn(c);
      // off the domain the neighbour is the mirror value (tl_fused.cu's matvec)
      const double pt = k < L.ny ? pn(c + L.ld) : pc, pb = k > 1 ? pn(c - L.ld) : pc;
      const double pr = j < L.nx ? pn(c + 1) : pc, pl = j > 1 ? pn(c - 1) : pc;
      double wv = a.f.di[c] * pc;
      wv = fma(-a.f.cy[c + L.ld], pt, wv);
      wv = fma(-a.f.cy[c], pb, wv);
      wv = fma(-a.f.cx[c + 1], pr, wv);
      wv = fma(-a.f.cx[c], pl, wv);
      a.f.w[c] = wv;
      pout[c] = pc;
      acc[0] = fma(wv, pc, acc[0]);
    }
    block_sum<1>(acc, scratch);
    if (threadIdx.x == 0) partA[blockIdx.x] = acc[0];
    __threadfence();
    if (!(ok = pb_barrier(arrive, gen, err, nwait))) break;
    const double pw = pb_total(partA, nb, scratch, &bcast);
    // EpiCgW
    const double alpha = S.rro / pw;
    if (threadIdx.x == 0) {
      S.u_pending = 0;
      S.pw = pw;
      S.alpha = alpha;
      if (blockIdx.x == 0) a.rd.hist_a[n] = alpha;
      if (!isfinite(alpha)) {
        S.status = EXIT_BREAKDOWN;
        S.n_exit = n;
      }
    }
    __syncthreads();
    if (S.status != RUN) break;
    // ---- phase B: u += alpha p_n, r -= alpha w, r.z ----
    acc[0] = 0.0;
    for (long long i = (long long)blockIdx.x * PB_T + threadIdx.x; i < ncell; i += stride) {
      const int j = (int)(i % L.nx) + 1, k = (int)(i / L.nx) + 1;
      const long long c = L.at(j, k);
      a.f.u[c] = fma(alpha, pout[c], a.f.u[c]);
      const double rv = fma(-alpha, a.f.w[c], a.f.r[c]);
      a.f.r[c] = rv;
      double zv = rv;
      if (use_z) {
        zv = a.f.mi[c] * rv;
        a.f.z[c] = zv;
      }
      acc[0] = fma(rv, zv, acc[0]);
    }
    block_sum<1>(acc, scratch);
    if (threadIdx.x == 0) partB[blockIdx.x] = acc[0];
    __threadfence();
    if (!(ok = pb_barrier(arrive, gen, err, nwait))) break;
    const double rrn = pb_total(partB, nb, scratch, &bcast);
    // EpiCgUr (u already updated)
    if (threadIdx.x == 0) {
      S.rrn = rrn;
      const double b = rrn / S.rro;
      S.beta = b;
      if (blockIdx.x == 0) a.rd.hist_b[n] = b;
      S.p_pending = 1;
      S.rro = rrn;
      S.cg_calc_steps += 1;
      finish_iteration(&S, rrn);
    }
    __syncthreads();
    ++done;
  }
  if (!ok && threadIdx.x == 0) S.status = EXIT_TIMEOUT;
  __syncthreads();
  // every CTA's copy is the same; CTA 0 publishes it (after all CTAs read the state at entry)
  if (blockIdx.x == 0 && threadIdx.x == 0) *a.rd.st = S;
}

// Applies a pending deferred u update (LoopState::u_pending) when the CG loop stops.
__global__ void __launch_bounds__(FT) k_flush_u(LoopArgs a) {
  const LoopState* st = a.rd.st;
  if (!st->u_pending) return;
  const Layout L = a.L;
  const double* __restrict__ p = st->u_psel ? a.f.p2 : a.f.p;
  const double ua = st->u_alpha;
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (j > L.nx) return;
  for (int k = blockIdx.y + 1; k <= L.ny; k += gridDim.y) {
    const long long c = L.at(j, k);
    a.f.u[c] = fma(ua, p[c], a.f.u[c]);
  }
}

// r -= alpha w (and u += alpha p_n for PPCG), then by MODE:
//   UR_CG    r.r (or r.z with z = Mi r for jac_diag) and the CG epilogue; u += alpha p_n is
//            left pending for the next matvec sweep (LoopState::u_pending);
//   UR_PPCG  u updated here, no reduction (rrn is discarded, tea_solve.f90:309-311), fused
//            init_sd of the inner sweeps;
//   UR_PPCG_NOSD  as UR_PPCG without init_sd (the FP32 inner sweeps start from r themselves);
//   UR_ONLY  as UR_CG without the reduction: the block-Jacobi solve and r.z follow in
//            k_fused_block_rz.
enum { UR_CG = 0, UR_PPCG = 1, UR_ONLY = 2, UR_PPCG_NOSD = 3 };
template <int MODE>
__global__ void __launch_bounds__(FT) k_fused_cg_ur(LoopArgs a) {
  constexpr bool PPCG = MODE == UR_PPCG || MODE == UR_PPCG_NOSD;
  LoopState* st = a.rd.st;
  if (st->status != RUN) return;
  const Layout L = a.L;
  const int n = st->n;
  const double alpha = st->alpha;
  const double* __restrict__ p = (n & 1) ? a.f.p2 : a.f.p;
  const int ja = blockIdx.x * SW + 1 + 2 * threadIdx.x;
  const bool has_b = ja + 1 <= L.nx;
  const double theta_r = PPCG ? 1.0 / st->theta : 0.0;
  double acc[1] = {0.0};
  if (ja <= L.nx) {
    for (int k = blockIdx.y + 1; k <= L.ny; k += gridDim.y) {
      const long long c = L.at(ja, k);
      const double2 ww = *reinterpret_cast<const double2*>(a.f.w + c);
      double2 rr = *reinterpret_cast<const double2*>(a.f.r + c);
      if (PPCG) {
        const double2 pp = *reinterpret_cast<const double2*>(p + c);
        double2 uu = *reinterpret_cast<const double2*>(a.f.u + c);
        uu.x = fma(alpha, pp.x, uu.x);
        uu.y = fma(alpha, pp.y, uu.y);
        if (has_b)
          *reinterpret_cast<double2*>(a.f.u + c) = uu;
        else
          a.f.u[c] = uu.x;
      }
      rr.x = fma(-alpha, ww.x, rr.x);
      rr.y = fma(-alpha, ww.y, rr.y);
      double2 zz = rr;
      if (a.precond == 2) {
        const double2 mi = *reinterpret_cast<const double2*>(a.f.mi + c);
        zz.x = mi.x * rr.x;
        zz.y = mi.y * rr.y;
      }
      if (has_b) {
        *reinterpret_cast<double2*>(a.f.r + c) = rr;
        if (a.precond == 2) *reinterpret_cast<double2*>(a.f.z + c) = zz;
      } else {
        a.f.r[c] = rr.x;
        if (a.precond == 2) a.f.z[c] = zz.x;
      }
      if (MODE == UR_CG) {
        acc[0] = fma(rr.x, zz.x, acc[0]);
        if (has_b) acc[0] = fma(rr.y, zz.y, acc[0]);
      } else if (MODE == UR_PPCG) {
        // tea_leaf_kernel_ppcg_init_sd (ppcg_kernel.f90:31-88): sd = (z|r)/theta, rtemp = r, utemp = sd
        const double2 s = make_double2(zz.x * theta_r, zz.y * theta_r);
        if (has_b) {
          *reinterpret_cast<double2*>(a.f.sd + c) = s;
          *reinterpret_cast<double2*>(a.f.rtemp + c) = rr;
          *reinterpret_cast<double2*>(a.f.utemp + c) = s;
        } else {
          a.f.sd[c] = s.x;
          a.f.rtemp[c] = rr.x;
          a.f.utemp[c] = s.x;
        }
      }
    }
  }
  if (MODE == UR_CG) grid_reduce<1>(acc, a.rd, EpiCgUr{a.rd});
}

// Block-Jacobi CG tail (cg_kernel.f90:256-283): z = M^-1 r with the 4-row tridiagonal
// blocks of tea_block_solve (common_kernel.f90:378-468), r.z, and the CG epilogue.
// One thread per column and 4-row block; blocks of rows strided over gridDim.y.
__global__ void __launch_bounds__(FT) k_fused_block_rz(LoopArgs a, double ry) {
  LoopState* st = a.rd.st;
  if (st->status != RUN) return;
  const Layout L = a.L;
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  double acc[1] = {0.0};
  if (j <= L.nx) {
    for (int bottom = blockIdx.y * 4 + 1; bottom <= L.ny; bottom += gridDim.y * 4) {
      const int top = min(bottom + 3, L.ny);
      double dp[4], zl[4], rv[4];
      long long c = L.at(j, bottom);
      rv[0] = a.f.r[c];
      dp[0] = rv[0] / a.f.di[c];
      for (int k = bottom + 1; k <= top; ++k) {
        c = L.at(j, k);
        rv[k - bottom] = a.f.r[c];
        dp[k - bottom] = (rv[k - bottom] - (-a.f.ky[c] * ry) * dp[k - bottom - 1]) * a.f.bfp[c];
      }
      zl[top - bottom] = dp[top - bottom];
      for (int k = top - 1; k >= bottom; --k) zl[k - bottom] = dp[k - bottom] - a.f.cp[L.at(j, k)] * zl[k - bottom + 1];
      for (int k = bottom; k <= top; ++k) {
        a.f.z[L.at(j, k)] = zl[k - bottom];
        acc[0] = fma(rv[k - bottom], zl[k - bottom], acc[0]);
      }
    }
  }
  grid_reduce<1>(acc, a.rd, EpiCgUr{a.rd});
}

// End of a PPCG outer iteration (tea_solve.f90:320-330): z = utemp (tea_leaf_ppcg_update_z,
// when the FP64 inner sweeps left their result in utemp), rrn = (r - r_store).z
// (tea_leaf_ppcg_calc_rrn, ppcg_kernel.f90:532-561), and on the device beta = rrn/rro,
// p pending as z + beta p for the next matvec sweep, rro = rrn, error = rrn and the loop's
// EXIT test.
struct EpiPpcgRrn {
  Reduce rd;
  __device__ void operator()(double (&acc)[1]) const {
    LoopState* st = rd.st;
    const double rrn = acc[0];
    st->rrn = rrn;
    st->beta = rrn / st->rro;
    st->p_pending = 1;
    st->rro = rrn;
    finish_iteration(st, rrn);
    // a blocked FP32 inner sweep of this iteration gave up waiting for a staged row: stop here
    if (rd.counter[MIX_ERR_WORD] != 0u) {
      st->status = EXIT_TIMEOUT;
      st->n_exit = st->n;
    }
  }
};

template <bool COPY_Z>
__global__ void __launch_bounds__(FT) k_fused_ppcg_rrn(LoopArgs a) {
  LoopState* st = a.rd.st;
  if (st->status != RUN) return;
  const Layout L = a.L;
  const int ja = blockIdx.x * SW + 1 + 2 * threadIdx.x;
  const bool has_b = ja + 1 <= L.nx;
  double acc[1] = {0.0};
  if (ja <= L.nx) {
    for (int k = blockIdx.y + 1; k <= L.ny; k += gridDim.y) {
      const long long c = L.at(ja, k);
      double2 zz;
      if (COPY_Z) {
        zz = *reinterpret_cast<const double2*>(a.f.utemp + c);
        if (has_b)
          *reinterpret_cast<double2*>(a.f.z + c) = zz;
        else
          a.f.z[c] = zz.x;
      } else {
        zz = *reinterpret_cast<const double2*>(a.f.z + c);
      }
      const double2 rr = *reinterpret_cast<const double2*>(a.f.r + c);
      const double2 rs = *reinterpret_cast<const double2*>(a.f.r_store + c);
      acc[0] = fma(rr.x - rs.x, zz.x, acc[0]);
      if (has_b) acc[0] = fma(rr.y - rs.y, zz.y, acc[0]);
    }
  }
  grid_reduce<1>(acc, a.rd, EpiPpcgRrn{a.rd});
}

inline int strips(const Layout& L) { return (L.nx + SW - 1) / SW; }

}  // namespace

// Rows per CTA of a row-marching sweep: the grid is the fewest whole waves of co-resident CTAs
// with at most WAVE_ROWS_MAX rows each.  For the staged CG sweep at 8192^2 (7 CTAs per SM) a
// cap of 256 gives one wave of 249-row CTAs: 0.8985 ms per launch, against 0.9011 with 83-row
// CTAs over three waves and 0.9027 with 62-row CTAs over four (a cap of 64).
constexpr long long WAVE_ROWS_MAX = 256;
int wave_rows(int ny, int ns, long long slots) {
  if (slots < 1) slots = 1;
  const long long cap = WAVE_ROWS_MAX;
  const long long work = (long long)ny * ns;            // strip-rows to sweep
  long long waves = (work + slots * cap - 1) / (slots * cap);  // fewest waves with <= cap rows per CTA
  if (waves < 1) waves = 1;
  long long blocks = waves * slots / ns;                 // row blocks per strip
  if (blocks < 1) blocks = 1;
  long long rows = (ny + blocks - 1) / blocks;
  return (int)(rows < 8 ? 8 : (rows > cap ? cap : rows));
}

long long resident_ctas(const void* kernel, int threads, size_t smem) {
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    return 152LL * 8;
  }
  return (long long)sms * per_sm;
}

// TL_CG_STAGE=0 selects the matvec sweep with direct loads (same bits as the staged one)
int cg_stage_mode() {
  const char* e = getenv("TL_CG_STAGE");
  return (e && e[0] == '0') ? 0 : 1;
}

// TL_CG_EMU=0 keeps the staged sweep's products Di p on the FP64 pipe (same bits)
template <bool PPCG>
const void* cg_w_kernel(int mode) {
  const char* e = getenv("TL_CG_EMU");
  const bool emu = !(e && e[0] == '0');
  if (mode == 0) return (const void*)k_fused_cg_w<PPCG>;
  return emu ? (const void*)k_fused_cg_ws<PPCG, 3> : (const void*)k_fused_cg_ws<PPCG, 0>;
}
size_t cg_w_smem(int mode) { return mode == 0 ? 0 : STAGE_SMEM; }

// Co-resident CTAs of the staged sweep.  Both forms size their grid from it, so that they
// split the p.w sum into the same partials and give the same bits.
long long cg_w_slots() {
  static const long long slots = resident_ctas((const void*)k_fused_cg_ws<false, 0>, FT, STAGE_SMEM);
  return slots;
}

void launch_fused_cg_w(const LoopArgs& a, bool ppcg, cudaStream_t s) {
  const int ns = strips(a.L);
  // Whole waves of co-resident CTAs, 8..256 rows each.  With the staged sweep's 7 CTAs per SM,
  // 8192^2 gives one wave of 249-row CTAs and 4096^2 63-row CTAs in 0.99 of a wave.  (For the
  // direct-load sweep at 9 CTAs per SM, 64-row CTAs over three waves took 1.031 ms at 8192^2 and
  // one resident wave of ~196-row CTAs 1.055 ms.)
  int rows = wave_rows(a.L.ny, ns, cg_w_slots());
  const int min_rows = (int)(((long long)a.L.ny * ns + MAX_REDUCE_BLOCKS - 1) / MAX_REDUCE_BLOCKS);
  if (rows < min_rows) rows = min_rows;  // keep the CTA count within the partials buffer
  dim3 grid(ns, (a.L.ny + rows - 1) / rows);
  const int mode = cg_stage_mode();
  const void* k = ppcg ? cg_w_kernel<true>(mode) : cg_w_kernel<false>(mode);
  LoopArgs aa = a;
  void* args[] = {&aa, &rows};
  ++launch_counter();
  cudaLaunchKernel(k, grid, dim3(FT), args, cg_w_smem(mode), s);
}

int persistent_cg_grid() {
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_persistent_cg, PB_T, 0) != cudaSuccess) return 0;
  return sms * per_sm;
}

cudaError_t launch_persistent_cg(const LoopArgs& a, int max_run, unsigned* bar, int grid, cudaStream_t s,
                                 int extra_arrivals) {
  const long long ncell = (long long)a.L.nx * a.L.ny;
  long long need = (ncell + PB_T - 1) / PB_T;
  int g = (int)(need < grid ? need : grid);
  if (g < 1) g = 1;
  LoopArgs aa = a;
  void* args[] = {&aa, &max_run, &bar, &extra_arrivals};
  ++launch_counter();
  return cudaLaunchCooperativeKernel((const void*)k_persistent_cg, dim3(g), dim3(PB_T), args, 0, s);
}

// Update sweeps: 12 CTAs of 128 threads per SM (1824 on 152 SMs), each striding over rows.
// At 8192^2 the r -= alpha w, r.r sweep took 0.2514 ms with 1824 CTAs, against 0.2645 with
// 1696 (11 per SM, rounded to whole strips), 0.2640 with 1984, 0.259 with 2048, 0.266 with
// 2144 and 2432 (16 per SM), 0.2678 with 1520, 0.279 with 1216 and 0.317 with 16384: fewer
// CTAs mean fewer partials for the last CTA to sum and fewer arrivals on the ticket, until too
// few rows are in flight, and a grid of whole CTAs per SM keeps every SM's share equal.
int sm_count() {
  static const int n = [] {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
      cudaGetLastError();
      return 152;
    }
    return sms;
  }();
  return n;
}

inline dim3 ur_grid(const Layout& L) {
  const int ns = strips(L);
  int gy = (12 * sm_count() + ns - 1) / ns;
  if (gy > L.ny) gy = L.ny;
  if ((long long)gy * ns > MAX_REDUCE_BLOCKS) gy = MAX_REDUCE_BLOCKS / ns;
  return dim3(ns, gy);
}

void launch_fused_ppcg_ur(const LoopArgs& a, bool init_sd, cudaStream_t s) {
  const dim3 grid = ur_grid(a.L);
  if (init_sd)
    { ++launch_counter(); k_fused_cg_ur<UR_PPCG><<<grid, FT, 0, s>>>(a); }
  else
    { ++launch_counter(); k_fused_cg_ur<UR_PPCG_NOSD><<<grid, FT, 0, s>>>(a); }
}

void launch_fused_ppcg_rrn(const LoopArgs& a, bool copy_z, cudaStream_t s) {
  const dim3 grid = ur_grid(a.L);
  if (copy_z)
    { ++launch_counter(); k_fused_ppcg_rrn<true><<<grid, FT, 0, s>>>(a); }
  else
    { ++launch_counter(); k_fused_ppcg_rrn<false><<<grid, FT, 0, s>>>(a); }
}

void launch_fused_cg_ur(const LoopArgs& a, cudaStream_t s) {
  const dim3 grid = ur_grid(a.L);
  if (a.precond == 3) {
    { ++launch_counter(); k_fused_cg_ur<UR_ONLY><<<grid, FT, 0, s>>>(a); }
    const int gx = (a.L.nx + FT - 1) / FT;
    int by = (a.L.ny + 3) / 4;
    if (by > 1024) by = 1024;
    if ((long long)by * gx > MAX_REDUCE_BLOCKS) by = MAX_REDUCE_BLOCKS / gx;
    { ++launch_counter(); k_fused_block_rz<<<dim3(gx, by), FT, 0, s>>>(a, a.ry); }
  } else {
    { ++launch_counter(); k_fused_cg_ur<UR_CG><<<grid, FT, 0, s>>>(a); }
  }
}

namespace {

struct EpiJacobi {
  LoopState* st;
  __device__ void operator()(double (&acc)[1]) const { finish_iteration(st, acc[0]); }
};

// Jacobi iteration n (tea_leaf_jacobi_solve_kernel, jacobi_kernel.f90:26-77) with un and u in
// two buffers swapped every iteration instead of the copy un = u: u_out = (u0 + rx(Kx(j+1)
// un(j+1) + Kx(j) un(j-1)) + ry(Ky(k+1) un(k+1) + Ky(k) un(k-1))) / denominator, error =
// sum |u_out - un|; the epilogue applies the loop's test (error = sqrt|error|) and n = n+1.
// Off-domain neighbours of un are zero: the reference never writes un's halo.  The same
// operation order as k_jacobi, so the same bits.
template <int INT>
__global__ void k_fused_jacobi(Fields f, Layout L, Reduce rd, const double* __restrict__ un, double* __restrict__ u_out,
                               double rx, double ry) {
  if (rd.st->status != RUN) return;
  double v[1] = {0.0};
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  for (int k = blockIdx.y + 1; k <= L.ny; k += gridDim.y) {
    if (j > L.nx) continue;
    const long long c = L.at(j, k);
    const double ur = j < L.nx ? un[c + 1] : 0.0, ul = j > 1 ? un[c - 1] : 0.0;
    const double ut = k < L.ny ? un[c + L.ld] : 0.0, ub = k > 1 ? un[c - L.ld] : 0.0;
    const double u = jacobi_cell<INT>(f.u0[c], f.kx[c], f.kx[c + 1], f.ky[c], f.ky[c + L.ld], ul, ur, ub, ut,
                                      f.jden[c], f.jinv[c], rx, ry);
    u_out[c] = u;
    v[0] += fabs(u - un[c]);
  }
  grid_reduce<1>(v, rd, EpiJacobi{rd.st});
}

}  // namespace

// Which of the Jacobi update's seven products run on the integer pipes (bits of jacobi_cell's
// INT; TL_JACOBI_INT overrides: 0, 0x40, 0x1b, 0x3f or 0x7f).  The default, 0x3f, moves the
// six flux products (kx1 ur, kx0 ul, rx (..), ky1 ut, ky0 ub, ry (..)) off the FP64 pipe and
// keeps the quotient's num y, which starts the dependent tail of the update, on it: at 4096^2
// the sweep takes 0.338 ms per launch against 0.494 ms with FP64 multiplies only (0x1b: 0.372,
// 0x7f: 0.361, 0x40: 0.462).  The bits are the same in every variant.
int jacobi_int_mask() {
  const char* e = getenv("TL_JACOBI_INT");
  return e ? (int)strtol(e, nullptr, 0) : 0x3f;
}

void launch_fused_jacobi(const LoopArgs& a, const double* un, double* u_out, cudaStream_t s) {
  const int gy = a.L.ny < 256 ? a.L.ny : 256;
  const dim3 grid((a.L.nx + 255) / 256, gy);
  ++launch_counter();
  switch (jacobi_int_mask()) {
    case 0x1b: k_fused_jacobi<0x1b><<<grid, 256, 0, s>>>(a.f, a.L, a.rd, un, u_out, a.rx, a.ry); break;
    case 0x3f: k_fused_jacobi<0x3f><<<grid, 256, 0, s>>>(a.f, a.L, a.rd, un, u_out, a.rx, a.ry); break;
    case 0x7f: k_fused_jacobi<0x7f><<<grid, 256, 0, s>>>(a.f, a.L, a.rd, un, u_out, a.rx, a.ry); break;
    case 0x40: k_fused_jacobi<0x40><<<grid, 256, 0, s>>>(a.f, a.L, a.rd, un, u_out, a.rx, a.ry); break;
    default: k_fused_jacobi<0><<<grid, 256, 0, s>>>(a.f, a.L, a.rd, un, u_out, a.rx, a.ry); break;
  }
}

long long ppcg_ws_slots() {
  static const long long slots = resident_ctas((const void*)k_ppcg_inner_ws, FT, PPCG_SMEM);
  return slots;
}

void launch_ppcg_inner_fused(const Fields& f, const Layout& L, const double* sd_in, double* sd_out, double a,
                             double b, cudaStream_t s) {
  const int ns = strips(L);
  const int rows = wave_rows(L.ny, ns, ppcg_ws_slots());
  const dim3 grid(ns, (L.ny + rows - 1) / rows);
  ++launch_counter();
  k_ppcg_inner_ws<<<grid, FT, PPCG_SMEM, s>>>(f, L, sd_in, sd_out, a, b, rows);
}

long long cheby_ws_slots() {
  static const long long slots = resident_ctas((const void*)k_cheby_iter_ws<true>, FT, PPCG_SMEM);
  return slots;
}

void launch_cheby_iterate_fused(const Fields& f, const Layout& L, const double* u_in, double* u_out, double a,
                                double b, bool write_wr, cudaStream_t s) {
  const int ns = strips(L);
  const int rows = wave_rows(L.ny, ns, cheby_ws_slots());
  const dim3 grid(ns, (L.ny + rows - 1) / rows);
  ++launch_counter();
  if (write_wr)
    k_cheby_iter_ws<true><<<grid, FT, PPCG_SMEM, s>>>(f, L, u_in, u_out, a, b, rows);
  else
    k_cheby_iter_ws<false><<<grid, FT, PPCG_SMEM, s>>>(f, L, u_in, u_out, a, b, rows);
}

void launch_flush_u(const LoopArgs& a, cudaStream_t s) {
  dim3 grid((a.L.nx + FT - 1) / FT, a.L.ny < 4096 ? a.L.ny : 4096);
  { ++launch_counter(); k_flush_u<<<grid, FT, 0, s>>>(a); }
  cudaMemsetAsync(&a.rd.st->u_pending, 0, sizeof(int), s);
}

}  // namespace tl
