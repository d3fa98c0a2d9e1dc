// tl_kernels.cuh -- host-side launchers of the TeaLeaf GB300 kernels (defined in
// tl_kernels.cu, tl_fused.cu).  All launchers are asynchronous on the given stream.
#pragma once

#include <string>

#include "tl_device.cuh"

namespace tl {

struct Geometry {
  double rx, ry;   // dt/dx^2, dt/dy^2
  double dx, dy;   // cell widths
  int coefficient, precond, reflective;
};

// Capacity of the per-CTA partials buffer (CTAs x 4 lanes).
constexpr int MAX_REDUCE_BLOCKS = 65536;

// Number of kernels the launchers below have launched on the calling thread.
long long& launch_counter();

// Sets the message tl_last_error() returns on the calling thread.
void set_last_error(const std::string& msg);

// ---- set-up, summary, generation, halo ----------------------------------
void launch_init_faces(const Fields& f, const Layout& L, const Geometry& g, cudaStream_t s);
void launch_init_cells(const Fields& f, const Layout& L, const Geometry& g, bool with_residual, cudaStream_t s);
void launch_init_state(const Fields& f, const Layout& L, cudaStream_t s);
void launch_block_init(const Fields& f, const Layout& L, const Geometry& g, cudaStream_t s);
void launch_generate(const Fields& f, const Layout& L, int nstates, const double* states /*device, 8*nstates*/,
                     double xmin, double ymin, double dx, double dy, cudaStream_t s);
void launch_field_summary(const Fields& f, const Layout& L, double cell_vol, const Reduce& rd, cudaStream_t s);
void launch_update_halo(double* const* fields, int nfields, const Layout& L, cudaStream_t s);
void launch_copy_interior(double* dst, const double* src, const Layout& L, cudaStream_t s);
// interior of a field <- / -> a host-layout array (row k at (k-1)*ld) already on the device
void launch_unpack(double* dst, const double* src, long long ld, const Layout& L, cudaStream_t s);
void launch_pack(double* dst, long long ld, const double* src, const Layout& L, cudaStream_t s);
void launch_copy_all(double* dst, const double* src, const Layout& L, cudaStream_t s);

// ---- per-kernel entry points (reference semantics) ----------------------
// Reduction epilogue modes
enum RedMode : int {
  RED_STORE = 0,          // st->red[0..NV) = totals
  RED_INIT_RESIDUAL = 1,  // old_error = rr, initial_residual = sqrt(|rr|)
  RED_RRO = 2,            // st->rro = total
  RED_EXACT = 3,          // st->red[0] = total (exact residual)
};
void launch_residual(const Fields& f, const Layout& L, const Reduce* rd /*null: no norm*/, int mode, cudaStream_t s);
void launch_norm2(const double* a, const Layout& L, const Reduce& rd, int mode, cudaStream_t s);
void launch_finalise(const Fields& f, const Layout& L, cudaStream_t s);
void launch_precond(const Fields& f, const Layout& L, const Geometry& g, const double* src, double* dst,
                    cudaStream_t s);
void launch_cg_init(const Fields& f, const Layout& L, const Geometry& g, const Reduce& rd, int mode, cudaStream_t s);
// residual + its norm + cg_init in one sweep (precond none or jac_diag): r, p (z), old_error,
// initial_residual, rro
void launch_residual_cg_init(const Fields& f, const Layout& L, const Geometry& g, const Reduce& rd, cudaStream_t s);
// finalise with the pending deferred u update of the CG loop applied first
void launch_finalise_flush(const Fields& f, const Layout& L, LoopState* st, cudaStream_t s);
// finalise fused with field_summary (sums in st->red[0..4)); flush_st non-null: apply the
// pending deferred u update first
void launch_finalise_summary(const Fields& f, const Layout& L, double cell_vol, const Reduce& rd, LoopState* flush_st,
                             cudaStream_t s);
void launch_cg_calc_w(const Fields& f, const Layout& L, const Reduce& rd, cudaStream_t s);
void launch_cg_calc_ur(const Fields& f, const Layout& L, const Geometry& g, double alpha, const Reduce& rd,
                       cudaStream_t s);
void launch_cg_calc_p(const Fields& f, const Layout& L, double beta, bool use_z, cudaStream_t s);
void launch_cheby_init(const Fields& f, const Layout& L, const Geometry& g, double theta, cudaStream_t s);
void launch_cheby_iterate(const Fields& f, const Layout& L, const Geometry& g, double a, double b, cudaStream_t s);
void launch_ppcg_init_sd(const Fields& f, const Layout& L, const Geometry& g, double theta, cudaStream_t s);
void launch_ppcg_init(const Fields& f, const Layout& L, const Geometry& g, int step, bool ppcg_active,
                      const Reduce& rd, int mode, cudaStream_t s);
void launch_ppcg_inner(const Fields& f, const Layout& L, const Geometry& g, double a, double b, cudaStream_t s);
// w = A u, r = u0 - w (the first half of a Chebyshev iteration, cheby_kernel.f90:111-174)
void launch_cheby_wr(const Fields& f, const Layout& L, cudaStream_t s);
// one FP64 Chebyshev iteration (no preconditioner) as one sweep: u_in -> u_out, p in place, and
// w and r when write_wr
void launch_cheby_iterate_fused(const Fields& f, const Layout& L, const double* u_in, double* u_out, double a,
                                double b, bool write_wr, cudaStream_t s);
// one FP64 PPCG inner step (no preconditioner) as one sweep: sd_in -> sd_out, rtemp, utemp in place
void launch_ppcg_inner_fused(const Fields& f, const Layout& L, const double* sd_in, double* sd_out, double a,
                             double b, cudaStream_t s);
void launch_dot(const double* a, const double* b, const double* bminus /*nullable*/, const Layout& L,
                const Reduce& rd, int mode, cudaStream_t s);
void launch_jacobi(const Fields& f, const Layout& L, const Geometry& g, const Reduce& rd, cudaStream_t s);

// ---- fused solver loop (device-resident scalars) ------------------------
struct LoopArgs {
  Fields f;
  Layout L;
  Reduce rd;
  int precond;
  int reflective;
  double ry;  // dt/dy^2 (block-Jacobi tridiagonal coefficients)
  double rx;  // dt/dx^2
};
// Rows per CTA of a row-marching sweep over ns strips: whole waves of `slots` co-resident CTAs
// (SMs x CTAs per SM), 8..64 rows per CTA.
int wave_rows(int ny, int ns, long long slots);
// SMs x co-resident CTAs per SM of `kernel` at `threads` threads and `smem` dynamic shared
// memory (fallback 152 x 8 if the occupancy query fails)
long long resident_ctas(const void* kernel, int threads, size_t smem);
// resident CTAs of the FP64 matvec sweep / the FP32 one (queried once; first called outside
// any stream capture: at context creation / in prepare_mix_kernels)
long long cg_w_slots();
int sm_count();  // multiprocessors of the current device (queried once)
long long mix_w_slots();
void launch_fused_cg_w(const LoopArgs& a, bool ppcg, cudaStream_t s);
void launch_fused_cg_ur(const LoopArgs& a, cudaStream_t s);
// PPCG outer iteration pieces (with launch_fused_cg_w(a, true, s)): u += alpha p, r -= alpha w
// (+ init_sd of the FP64 inner sweeps); then z = utemp (copy_z) and rrn = (r - r_store).z with
// the iteration's epilogue and EXIT test
void launch_fused_ppcg_ur(const LoopArgs& a, bool init_sd, cudaStream_t s);
void launch_fused_ppcg_rrn(const LoopArgs& a, bool copy_z, cudaStream_t s);
// u += alpha p of the last CG iteration when it is still pending (end of a CG phase)
void launch_flush_u(const LoopArgs& a, cudaStream_t s);
// persistent cooperative CG (no preconditioner or jac_diag): up to max_run iterations in one
// launch; bar = three zeroed words (barrier counter, generation, error); grid = the co-resident
// CTA count from persistent_cg_grid() (0 if it cannot be determined)
int persistent_cg_grid();
cudaError_t launch_persistent_cg(const LoopArgs& a, int max_run, unsigned* bar, int grid, cudaStream_t s,
                                 int extra_arrivals = 0);
// one Jacobi iteration from un into u_out (the two swap every iteration), error and the loop's
// test in the epilogue
void launch_fused_jacobi(const LoopArgs& a, const double* un, double* u_out, cudaStream_t s);
void launch_jacobi_denominator(const Fields& f, const Layout& L, const Geometry& g, cudaStream_t s);

// ---- mixed precision: FP32 inner CG inside FP64 iterative refinement (tl_mixed.cu) ----
struct MixFields {
  float *cx, *cy, *di;  // FP32 copies of the pre-scaled operator
  float *r, *p, *p2, *w, *d;
  float* e;             // second buffer of the blocked polynomial sweeps' ping-pong
  unsigned* err;        // set by a blocked sweep whose bounded wait for a staged row expired
  float* mi;            // FP32 copy of the jac_diag preconditioner Mi = 1/Di (null: no preconditioner)
  float* z;             // jac_diag: z = Mi r of the FP32 CG process (null: no preconditioner)
};
struct MixState {
  double rro, rro_prev, pw, rr, alpha, beta;  // FP32-vector CG scalars (FP64)
  double rr_max;                              // r.r at the last residual replacement
  double delta2;                              // replace when r.r < delta2 * rr_max
  double trial_rr;                            // ||u0 - A (u + d)||^2 in FP64 (last trial)
  double trial_rr32;                          // r.r of its FP32 rounding
  double trial_scale;                         // sum of (|u0| + |Di u| + sum |c u_nb|)^2 (last trial)
  double trial_rz;                            // r.(Mi r) in FP64 of the last trial (= trial_rr without
                                              // a preconditioner): the reference's error norm
  double trial_rz32;                          // r32.(Mi32 r32) of its FP32 rounding (the FP32 process's r.z)
  double d_alpha;
  int n, max_n, phase_end, status, p_pending, d_pending, d_psel;
  // CG presteps of the mixed Chebyshev form: stop with STOP_SWITCH once step n >= presteps
  // and r.r <= switch_rr (the reference's switch rule, tea_solve.f90:167); record alpha/beta
  // of every step for the eigenvalue estimate (null: not recorded)
  double switch_rr;
  int presteps;
  double *hist_a, *hist_b;
};
// once per context (device), before any launch or capture: the FP32 matvec sweep's dynamic
// shared memory above the 48 KB default; 0 on success
int prepare_mix_kernels();
void launch_mix_prep(const Fields& f, const MixFields& m, const Layout& L, cudaStream_t s);
// d += alpha p if an update is pending (the host clears MixState::d_pending afterwards)
void launch_mix_flush_d(const MixFields& m, const Layout& L, MixState* ms, cudaStream_t s);
// trial residual r = u0 - A (u + d) in FP64 (u unchanged), r32 = r; first: also p32 = r.
// mirror: off-domain neighbours mirrored (CG); else read from the halo cells (Chebyshev)
void launch_mix_trial(const Fields& f, const MixFields& m, const Layout& L, const Reduce& rd, MixState* ms,
                      bool first, cudaStream_t s, bool mirror = true);
// one FP32 CG step: k_mix_w then k_mix_ur; `between` (nullable) is recorded between them
void launch_mix_iteration(const MixFields& m, const Layout& L, const Reduce& rd, MixState* ms, cudaStream_t s,
                          cudaEvent_t between = nullptr);
// accept the correction: u += d (FP64), d = 0
void launch_mix_apply(const Fields& f, const MixFields& m, const Layout& L, cudaStream_t s);

// ---- FP32 polynomial sweeps of the precision form of Chebyshev / PPCG (tl_mixed_poly.cu) ----
// PPCG inner loop in FP32 from the FP64 r: inner_steps Chebyshev steps with ch_a/ch_b[1..],
// z (FP64) = utemp at the end
void launch_poly_ppcg_inner(const Fields& f, const MixFields& m, const Layout& L, double theta, int inner_steps,
                            const double* ch_a, const double* ch_b, cudaStream_t s);
// `steps` Chebyshev steps (start + steps-1 iterations with ch_a/ch_b[1..]) on A d = m.r from
// d = 0; d ends in m.d
void launch_poly_cheby(const MixFields& m, const Layout& L, double theta, int steps, const double* ch_a,
                       const double* ch_b, cudaStream_t s);
// m.d = m.p2 = 0
void launch_poly_clear(const MixFields& m, const Layout& L, cudaStream_t s);

// ---- adjoint of a time step (tl_adjoint.cu) ----
// rhs = u_bar_ext (nullable) + e_bar / rho;  rho_bar -= e_bar u / rho^2
void launch_adj_rhs(const double* u_bar_ext, const double* e_bar, const double* u, const double* rho, double* rhs,
                    double* rho_bar, const Layout& L, cudaStream_t s);
// rho_bar += lambda e + dA/dK terms chained to rho;  e_bar = lambda rho
void launch_adj_accumulate(const double* lam, const double* u, const double* e, const double* rho, double* rho_bar,
                           double* e_bar, const Layout& L, double rx, double ry, int coefficient, cudaStream_t s);

}  // namespace tl
