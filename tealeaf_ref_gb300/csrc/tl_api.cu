// tl_api.cu -- the C ABI (include/tealeaf_gb300.h): context, host<->device copies, the
// per-kernel drop-in entry points and tl_tea_leaf(), a C++ restatement of the control flow
// of tea_leaf() (tea_solve.f90:37-503) over the GPU kernels.
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/tealeaf_gb300.h"
#include "tl_kernels.cuh"

using namespace tl;

namespace {

thread_local std::string g_err;

int fail(int code, const char* msg) {
  g_err = msg;
  return code;
}
int cuda_fail(cudaError_t e, const char* where) {
  g_err = std::string(where) + ": " + cudaGetErrorString(e);
  return TL_ERR_CUDA;
}

#define CK(call)                                   \
  do {                                             \
    cudaError_t e_ = (call);                       \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

// field order inside the slab
enum Slot {
  S_DENSITY, S_ENERGY1, S_U, S_U0, S_R, S_W, S_P, S_P2, S_KX, S_KY, S_CX, S_CY, S_DI, S_Z, S_MI, S_SD, S_SD1,
  S_UTEMP, S_RTEMP, S_RSTORE, S_CP, S_BFP, S_U1, S_JINV, S_JDEN, S_COUNT
};

}  // namespace

// Lets the library's other translation units report through tl_last_error().
void tl::set_last_error(const std::string& msg) { g_err = msg; }

struct tl_ctx {
  int device = 0;
  Layout L{};
  Geometry g{};
  int halo_depth = 1;
  cudaStream_t stream = nullptr;
  char* slab = nullptr;
  size_t slab_bytes = 0;
  size_t field_stride = 0;  // bytes between fields in the slab
  Fields f{};
  double* partials = nullptr;
  unsigned* counter = nullptr;
  LoopState* st = nullptr;
  LoopState* st_host = nullptr;  // pinned mirror
  double* hist_a = nullptr;
  double* hist_b = nullptr;
  int hist_cap = 0;
  double* ch_a = nullptr;
  double* ch_b = nullptr;
  int ch_cap = 0;
  double* states_dev = nullptr;
  int states_cap = 0;
  double** halo_list = nullptr;  // device array of field pointers for halo updates
  // reference SAVE variables (tea_solve.f90:55,58)
  int first = 1;
  double eigmin = 0, eigmax = 0, theta = 0, cn = 0;
  bool have_coefs = false;
  // Set-up cache: Kx, Ky, cx, cy, Di, Mi and the block factors depend only on density and dt
  // (and the chunk's fixed geometry, coefficient keyword and boundary type).  They are valid
  // for setup_dt while setup_valid; every entry point that can write density, Kx, Ky, Di or
  // Mi clears the flag, so a solve rebuilds them exactly when the reference's per-step
  // tea_leaf_common_init would produce different values.
  bool setup_valid = false;
  double setup_dt = 0.0;
  // tl_tea_leaf_summary: the solve's finalise sweep also forms the field summary (st->red)
  bool want_summary = false;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // per-launch timers of the fused loop kernels (tl_profile)
  static constexpr int BATCH = 16;
  bool prof = false;
  cudaEvent_t pev[3 * BATCH] = {};
  // timed launches of the host-driven loops: event pairs recorded around each launch and read
  // once QCAP are pending or the solve ends, so the host never waits for a single launch
  static constexpr int QCAP = 256;
  cudaEvent_t qev[2 * QCAP] = {};
  int qid[QCAP] = {}, qcount[QCAP] = {};
  int qn = 0;
  // CUDA graphs of one batch of the device-resident loops (captured once per set of kernel
  // arguments): the fused CG batch and the mixed-precision CG batch
  cudaGraphExec_t cg_exec = nullptr, mix_exec = nullptr;
  // the fused CG batch with events recorded around the two kernels of its second iteration
  // (tl_profile on): one sampled iteration per batch, so the events (graph nodes) hardly
  // perturb the timed launches
  cudaGraphExec_t cg_prof_exec = nullptr;
  LoopArgs cg_prof_key{};
  long long cg_prof_nk = 0;
  int pgrid = -1;  // co-resident CTAs of the persistent CG kernel (-1: not yet queried)
  // host transfers: an upload and a download stream (tl_stage_state, tl_fetch_field) and
  // XFER_FIELDS staging fields -- two staged (density, energy1) pairs, the fetch snapshot, and
  // two for the synchronous uploads / downloads.  A host array moves as one contiguous copy
  // (copy engines) and is unpacked / packed on the device; st_ld[slot] is the host row stride of
  // a staged pair in that form, 0 for one copied row by row into the context layout.
  static constexpr int XFER_FIELDS = 7;
  cudaStream_t up = nullptr, down = nullptr;
  char* xfer = nullptr;
  bool xfer_failed = false;
  int st_ld[2] = {0, 0};
  cudaEvent_t st_done[2] = {}, st_used[2] = {}, fe_snap = nullptr, fe_done = nullptr;
  bool st_used_rec[2] = {false, false}, fe_done_rec = false;
  int st_head = 0, st_count = 0;
  double* xfield(int i) const { return reinterpret_cast<double*>(xfer + (size_t)i * field_stride); }
  LoopArgs cg_key{};
  long long cg_nk = 0, mix_nk = 0;
  double prof_ms[TL_NUM_KERNEL_TIMERS] = {};
  long long prof_n[TL_NUM_KERNEL_TIMERS] = {};
  long long nlaunch = 0;  // kernels launched by the current tl_tea_leaf call
  // mixed-precision form: FP32 fields (allocated on first use) and the inner-loop state
  char* mix_slab = nullptr;
  size_t mix_bytes = 0, tape_bytes = 0;  // sizes of the FP32 slab and the adjoint tape (0: none)
  MixFields mix{};
  MixState* mst = nullptr;
  MixState* mst_host = nullptr;
  // adjoint tape (tl_adjoint_*): per recorded step its input energy1 (and, when storing
  // solutions, its u), plus four work fields: rhs, rho_bar, e_bar, recomputed u
  char* tape = nullptr;
  int tape_max = 0, tape_n = 0, tape_store_u = 0;
  std::vector<double> tape_dt;
  std::vector<tl_solve_opts> tape_opts;
  double* tape_field(int i) const { return reinterpret_cast<double*>(tape + (size_t)i * field_stride); }

  double* slot(int s) const { return reinterpret_cast<double*>(slab + (size_t)s * field_stride); }
  Reduce rd() const { return Reduce{partials, counter, st, hist_a, hist_b, ch_a, ch_b}; }
  LoopArgs loop() const { return LoopArgs{f, L, rd(), g.precond, g.reflective, g.ry, g.rx}; }
};

namespace {

double* field_ptr(tl_ctx* c, int id) {
  switch (id) {
    case TL_FIELD_DENSITY: return c->f.density;
    case TL_FIELD_ENERGY0:
    case TL_FIELD_ENERGY1: return c->f.energy1;
    case TL_FIELD_U: return c->f.u;
    case TL_FIELD_P: return c->f.p;
    case TL_FIELD_SD: return c->f.sd;
    case TL_FIELD_R: return c->f.r;
    case TL_FIELD_Z: return c->f.z;
    case TL_FIELD_KX: return c->f.kx;
    case TL_FIELD_KY: return c->f.ky;
    case TL_FIELD_DI: return c->f.di;
    case TL_FIELD_U0: return c->f.u0;
    case TL_FIELD_W: return c->f.w;
    case TL_FIELD_MI: return c->f.mi;
    case TL_FIELD_UTEMP: return c->f.utemp;
    case TL_FIELD_RTEMP: return c->f.rtemp;
    case TL_FIELD_R_STORE: return c->f.r_store;
    default: return nullptr;
  }
}

// update_halo field binding (update_halo.f90:64-80): FIELD_R is vector_rtemp there.
double* halo_field_ptr(tl_ctx* c, int id) {
  if (id == TL_FIELD_R) return c->f.rtemp;
  if (id == TL_FIELD_ENERGY0) return nullptr;  // energy0 is not held on the device
  return field_ptr(c, id);
}

int sync_state(tl_ctx* c) {
  CK(cudaMemcpyAsync(c->st_host, c->st, sizeof(LoopState), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return TL_OK;
}

int push_state(tl_ctx* c) {
  CK(cudaMemcpyAsync(c->st, c->st_host, sizeof(LoopState), cudaMemcpyHostToDevice, c->stream));
  return TL_OK;
}

int reduce_result(tl_ctx* c, double* out, int lanes = 1) {
  int rc = sync_state(c);
  if (rc) return rc;
  for (int i = 0; i < lanes; ++i) out[i] = c->st_host->red[i];
  return TL_OK;
}

int check_launch(const char* where) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, where);
  return TL_OK;
}

int ensure_hist(tl_ctx* c, int n) {
  if (n <= c->hist_cap) return TL_OK;
  if (c->hist_a) cudaFree(c->hist_a);
  if (c->hist_b) cudaFree(c->hist_b);
  c->hist_a = c->hist_b = nullptr;
  CK(cudaMalloc(&c->hist_a, sizeof(double) * n));
  CK(cudaMalloc(&c->hist_b, sizeof(double) * n));
  c->hist_cap = n;
  return TL_OK;
}

int ensure_ch(tl_ctx* c, int n) {
  if (n <= c->ch_cap) return TL_OK;
  if (c->ch_a) cudaFree(c->ch_a);
  if (c->ch_b) cudaFree(c->ch_b);
  c->ch_a = c->ch_b = nullptr;
  CK(cudaMalloc(&c->ch_a, sizeof(double) * n));
  CK(cudaMalloc(&c->ch_b, sizeof(double) * n));
  c->ch_cap = n;
  return TL_OK;
}

// Timers of the host-driven loops: prof_begin before a launch and prof_end after it record an
// event pair on the solve stream; prof_flush (when QCAP pairs are pending, at the end of a
// solve and in tl_profile_read) waits for the last one and adds each launch's time to its
// TL_KERNEL id (count units).  No-ops unless tl_profile is on.
int prof_flush(tl_ctx* c) {
  if (c->qn == 0) return TL_OK;
  CK(cudaEventSynchronize(c->qev[2 * c->qn - 1]));
  for (int i = 0; i < c->qn; ++i) {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, c->qev[2 * i], c->qev[2 * i + 1]));
    c->prof_ms[c->qid[i]] += ms;
    c->prof_n[c->qid[i]] += c->qcount[i];
  }
  c->qn = 0;
  return TL_OK;
}
int prof_begin(tl_ctx* c) {
  if (!c->prof) return TL_OK;
  if (c->qn == tl_ctx::QCAP) {
    int rc = prof_flush(c);
    if (rc) return rc;
  }
  CK(cudaEventRecord(c->qev[2 * c->qn], c->stream));
  return TL_OK;
}
int prof_end(tl_ctx* c, int id, int count) {
  if (!c->prof) return TL_OK;
  CK(cudaEventRecord(c->qev[2 * c->qn + 1], c->stream));
  c->qid[c->qn] = id;
  c->qcount[c->qn] = count;
  c->qn += 1;
  return TL_OK;
}

// Batches of the device-resident loops as CUDA graphs.  All loop state (iteration index, alpha,
// beta, status, which p buffer is current) lives in device memory, so one batch of launches
// has the same arguments every time and is captured once; a launch of the graph replaces
// 2 x BATCH kernel launches.  Recaptured when an argument changes (dt changes ry; a larger
// max_iters reallocates the history buffers).
bool same_loop_args(const LoopArgs& a, const LoopArgs& b) {
  return memcmp(&a.f, &b.f, sizeof(Fields)) == 0 && a.L.nx == b.L.nx && a.L.ny == b.L.ny && a.L.ld == b.L.ld &&
         memcmp(&a.rd, &b.rd, sizeof(Reduce)) == 0 && a.precond == b.precond && a.reflective == b.reflective &&
         a.ry == b.ry;
}

template <typename F>
int capture_batch(tl_ctx* c, cudaGraphExec_t* exec, long long* nk, F&& launches) {
  if (*exec) {
    cudaGraphExecDestroy(*exec);
    *exec = nullptr;
  }
  const long long before = launch_counter();
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  launches();
  const cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  *nk = launch_counter() - before;
  launch_counter() = before;
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
  const cudaError_t ei = cudaGraphInstantiate(exec, g, 0);
  cudaGraphDestroy(g);
  if (ei != cudaSuccess) {
    *exec = nullptr;
    return cuda_fail(ei, "cudaGraphInstantiate");
  }
  return TL_OK;
}

// TL_NO_GRAPHS=1 in the environment: launch the batches kernel by kernel (same kernels, same
// results), e.g. under tools that do not follow graph launches.
bool use_graphs() {
  const char* e = getenv("TL_NO_GRAPHS");
  return !(e && e[0] == '1');
}

// TL_MIXED_PRESTEPS=0: the precision form of Chebyshev runs its CG presteps in FP64 (as the
// reference does) instead of as the mixed CG.
bool use_mixed_presteps() {
  const char* e = getenv("TL_MIXED_PRESTEPS");
  return !(e && e[0] == '0');
}

// TL_PPCG_FUSED=0: run the PPCG outer iterations over the per-kernel path (three scalar round
// trips per iteration) instead of the fused sweeps with device scalars.
bool use_fused_ppcg() {
  const char* e = getenv("TL_PPCG_FUSED");
  return !(e && e[0] == '0');
}

// The last sweep of a solve: energy1 = u / density (tea_leaf_kernel_finalise), with the CG
// loop's pending deferred u update applied first when `flush`, and fused with the field summary
// when the caller asked for one (tl_tea_leaf_summary).
void finalise_sweep(tl_ctx* c, bool flush) {
  if (c->want_summary)
    launch_finalise_summary(c->f, c->L, c->g.dx * c->g.dy, c->rd(), flush ? c->st : nullptr, c->stream);
  else if (flush)
    launch_finalise_flush(c->f, c->L, c->st, c->stream);
  else
    launch_finalise(c->f, c->L, c->stream);
}

// TL_SETUP_CACHE=0: rebuild Kx, Ky, Di (and the preconditioner set-up) in every solve even when
// density and dt are those of the previous solve (same results; for checking the cache).
bool use_setup_cache() {
  const char* e = getenv("TL_SETUP_CACHE");
  return !(e && e[0] == '0');
}

// Fields whose upload (or halo update) changes an input of the set-up cache.
bool writes_setup_input(int field) {
  return field == TL_FIELD_DENSITY || field == TL_FIELD_KX || field == TL_FIELD_KY || field == TL_FIELD_DI ||
         field == TL_FIELD_MI;
}

// The persistent CG kernel replaces the batched kernels up to this many cells (plain or
// jac_diag preconditioner): per iteration it measured 13.8 / 16.9 / 27.6 / 49.5 us at 128^2 /
// 256^2 / 512^2 / 1024^2 against 25.6 / 26.2 / 32.3 / 47.6 us for the batched kernels (CUDA
// graphs), so it stops paying near 800^2.  TL_CG_PERSISTENT=0 / 1 forces it off / on.
constexpr long long PERSIST_MAX_CELLS = 640LL * 1024;
constexpr int PERSIST_RUN = 256;  // iterations per launch at most (the host reads the status between)

// TL_CHEBY_SWEEP=0: the FP64 Chebyshev iterations as the two one-step kernels instead of one
// staged sweep (same bits)
bool use_cheby_sweep() {
  const char* e = getenv("TL_CHEBY_SWEEP");
  return !(e && e[0] == '0');
}

// TL_PPCG_INNER_SWEEP=0: the FP64 PPCG inner steps as the two one-step kernels instead of one
// staged sweep (same bits)
bool use_ppcg_inner_sweep() {
  const char* e = getenv("TL_PPCG_INNER_SWEEP");
  return !(e && e[0] == '0');
}

bool use_persistent(tl_ctx* c) {
  if (c->prof || c->g.precond == TL_PREC_JAC_BLOCK) return false;
  const char* e = getenv("TL_CG_PERSISTENT");
  const bool forced_on = e && e[0] == '1', forced_off = e && e[0] == '0';
  if (forced_off) return false;
  if (!forced_on && (long long)c->L.nx * c->L.ny > PERSIST_MAX_CELLS) return false;
  if (c->pgrid < 0) c->pgrid = persistent_cg_grid();
  return c->pgrid > 0;
}

int run_cg_batch(tl_ctx* c, const LoopArgs& la) {
  if (!c->cg_exec || !same_loop_args(c->cg_key, la)) {
    int rc = capture_batch(c, &c->cg_exec, &c->cg_nk, [&] {
      for (int i = 0; i < tl_ctx::BATCH; ++i) {
        launch_fused_cg_w(la, false, c->stream);
        launch_fused_cg_ur(la, c->stream);
      }
    });
    if (rc) return rc;
    c->cg_key = la;
  }
  CK(cudaGraphLaunch(c->cg_exec, c->stream));
  launch_counter() += c->cg_nk;
  return TL_OK;
}

// The same batch with the per-kernel timer events of its sampled iteration TIMED_ITER recorded
// as graph nodes: pev[0] before that iteration's matvec sweep, pev[1] between the sweeps, pev[2]
// after the update sweep.
constexpr int TIMED_ITER = 1;
int run_cg_batch_timed(tl_ctx* c, const LoopArgs& la) {
  if (!c->cg_prof_exec || !same_loop_args(c->cg_prof_key, la)) {
    cudaError_t rec = cudaSuccess;
    int rc = capture_batch(c, &c->cg_prof_exec, &c->cg_prof_nk, [&] {
      for (int i = 0; i < tl_ctx::BATCH; ++i) {
        const bool t = i == TIMED_ITER;
        if (t && rec == cudaSuccess) rec = cudaEventRecordWithFlags(c->pev[0], c->stream, cudaEventRecordExternal);
        launch_fused_cg_w(la, false, c->stream);
        if (t && rec == cudaSuccess) rec = cudaEventRecordWithFlags(c->pev[1], c->stream, cudaEventRecordExternal);
        launch_fused_cg_ur(la, c->stream);
        if (t && rec == cudaSuccess) rec = cudaEventRecordWithFlags(c->pev[2], c->stream, cudaEventRecordExternal);
      }
    });
    if (rc) return rc;
    if (rec != cudaSuccess) {
      cudaGraphExecDestroy(c->cg_prof_exec);
      c->cg_prof_exec = nullptr;
      return cuda_fail(rec, "cudaEventRecordWithFlags (capture)");
    }
    c->cg_prof_key = la;
  }
  CK(cudaGraphLaunch(c->cg_prof_exec, c->stream));
  launch_counter() += c->cg_prof_nk;
  return TL_OK;
}

int run_mix_batch(tl_ctx* c, const Reduce& rd) {
  // the mixed batch's arguments (FP32 fields, layout, reduction buffers, state) are fixed for
  // a context, except the reduction's history pointers, which the FP32 kernels do not use
  if (!c->mix_exec) {
    int rc = capture_batch(c, &c->mix_exec, &c->mix_nk, [&] {
      for (int i = 0; i < tl_ctx::BATCH; ++i) launch_mix_iteration(c->mix, c->L, rd, c->mst, c->stream);
    });
    if (rc) return rc;
  }
  CK(cudaGraphLaunch(c->mix_exec, c->stream));
  launch_counter() += c->mix_nk;
  return TL_OK;
}

int do_halo(tl_ctx* c, int mask, int depth) {
  (void)depth;  // a single chunk reads only the first halo layer
  if (!c->g.reflective) return TL_OK;
  double* ptrs[TL_FIELD_DI + 1];
  int n = 0;
  for (int id = 1; id <= TL_FIELD_DI; ++id)
    if (mask & (1 << id)) {
      double* p = halo_field_ptr(c, id);
      if (p) ptrs[n++] = p;
    }
  if (!n) return TL_OK;
  CK(cudaMemcpyAsync(c->halo_list, ptrs, sizeof(double*) * n, cudaMemcpyHostToDevice, c->stream));
  launch_update_halo(c->halo_list, n, c->L, c->stream);
  return check_launch("update_halo");
}

constexpr int M(int id) { return 1 << id; }

// ---------------------------------------------------------------------------
// Host scalar math: eigenvalues of the Lanczos tridiagonal built from the CG
// coefficients (tea_leaf_cheby.f90:142-176) and the Chebyshev coefficients (:178-205).
// Extreme eigenvalues by bisection on the Sturm sequence of T - x I (Golub & Van Loan,
// Matrix Computations, 4th ed., sec. 8.4.1).
// ---------------------------------------------------------------------------
int sturm_below(const std::vector<double>& d, const std::vector<double>& e2, double x) {
  const double tiny = 1e-300;
  int neg = 0;
  double q = 1.0;
  for (size_t i = 0; i < d.size(); ++i) {
    q = d[i] - x - (i ? e2[i - 1] / q : 0.0);
    if (q == 0.0) q = -tiny;
    if (q < 0.0) ++neg;
  }
  return neg;
}

double bisect_eigen(const std::vector<double>& d, const std::vector<double>& e2, int which, double lo, double hi) {
  for (int it = 0; it < 4000; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (mid <= lo || mid >= hi) break;
    if (sturm_below(d, e2, mid) > which)
      hi = mid;
    else
      lo = mid;
  }
  return 0.5 * (lo + hi);
}

int calc_eigenvalues(const std::vector<double>& alphas, const std::vector<double>& betas, int nsteps, double* eigmin,
                     double* eigmax) {
  // alphas[i], betas[i] hold cg_alphas(i+1), cg_betas(i+1)
  if (nsteps <= 0) return 1;
  std::vector<double> d(nsteps), off(nsteps > 1 ? nsteps - 1 : 0), e2(off.size());
  for (int n = 0; n < nsteps; ++n) {
    d[n] = 1.0 / alphas[n];
    if (n > 0) d[n] = d[n] + betas[n - 1] / alphas[n - 1];
    if (n < nsteps - 1) off[n] = std::sqrt(betas[n]) / alphas[n];
  }
  double lo = d[0], hi = d[0];
  for (int i = 0; i < nsteps; ++i) {
    const double rad = (i > 0 ? std::fabs(off[i - 1]) : 0.0) + (i < nsteps - 1 ? std::fabs(off[i]) : 0.0);
    lo = std::fmin(lo, d[i] - rad);
    hi = std::fmax(hi, d[i] + rad);
  }
  const double pad = 4.0 * 2.220446049250313e-16 * std::fmax(std::fabs(lo), std::fabs(hi)) + 1e-300;
  lo -= pad;
  hi += pad;
  for (size_t i = 0; i < off.size(); ++i) e2[i] = off[i] * off[i];
  *eigmin = bisect_eigen(d, e2, 0, lo, hi);
  *eigmax = bisect_eigen(d, e2, nsteps - 1, lo, hi);
  if (!(std::isfinite(*eigmin) && std::isfinite(*eigmax))) return 1;
  if (*eigmin < 0.0 || *eigmax < 0.0) return 1;
  return 0;
}

void calc_ch_coefs(std::vector<double>& a, std::vector<double>& b, double eigmin, double eigmax, double* theta, int n) {
  *theta = (eigmax + eigmin) / 2;
  const double delta = (eigmax - eigmin) / 2;
  const double sigma = *theta / delta;
  double rho_old = 1.0 / sigma;
  a.assign(n + 1, 0.0);
  b.assign(n + 1, 0.0);
  for (int i = 1; i <= n; ++i) {
    const double rho_new = 1.0 / (2.0 * sigma - rho_old);
    a[i] = rho_new * rho_old;
    b[i] = 2.0 * rho_new / delta;
    rho_old = rho_new;
  }
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char* tl_last_error(void) { return g_err.c_str(); }

int tl_set_device(int device) {
  int n = 0;
  CK(cudaGetDeviceCount(&n));
  if (device < 0 || device >= n) return fail(TL_ERR_ARG, "tl_set_device: no such device");
  CK(cudaSetDevice(device));
  return TL_OK;
}

int tl_create(int x_cells, int y_cells, int halo_depth, int coefficient, int preconditioner, int reflective_boundary,
              double dx, double dy, tl_ctx** out) {
  if (!out) return fail(TL_ERR_ARG, "tl_create: out is null");
  *out = nullptr;
  if (x_cells < 1 || y_cells < 1 || x_cells > 65536 || y_cells > 65536)
    return fail(TL_ERR_ARG, "tl_create: x_cells and y_cells must be in 1..65536");
  if (halo_depth < 1) return fail(TL_ERR_ARG, "tl_create: Invalid halo exchange depth specified");
  if (coefficient != TL_CONDUCTIVITY && coefficient != TL_RECIP_CONDUCTIVITY)
    return fail(TL_ERR_ARG, "tl_create: unknown coefficient option");
  if (preconditioner < TL_PREC_NONE || preconditioner > TL_PREC_JAC_BLOCK)
    return fail(TL_ERR_ARG, "tl_create: Invalid preconditioner type specified");
  if (halo_depth > 1 && preconditioner == TL_PREC_JAC_BLOCK)
    return fail(TL_ERR_ARG, "tl_create: Unable to use nonstandard halo depth with block jacobi preconditioner");
  if (!(dx > 0.0) || !(dy > 0.0)) return fail(TL_ERR_ARG, "tl_create: dx and dy must be positive");

  tl_ctx* c = new tl_ctx();
  cudaGetDevice(&c->device);
  c->halo_depth = halo_depth;
  c->L.nx = x_cells;
  c->L.ny = y_cells;
  // room after the right halo cell for a 4-wide (FP32) or 2-wide (FP64) vector load that starts
  // at the last interior column
  c->L.ld = ((XOFF + x_cells + 4 + 15) / 16) * 16;
  c->g.dx = dx;
  c->g.dy = dy;
  c->g.coefficient = coefficient;
  c->g.precond = preconditioner;
  c->g.reflective = reflective_boundary ? 1 : 0;

  const size_t field_bytes = ((size_t)c->L.elems() * sizeof(double) + 4 * 256 + 255) / 256 * 256;
  c->field_stride = field_bytes;
  c->slab_bytes = field_bytes * S_COUNT;
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&c->slab, c->slab_bytes);
  if (e == cudaSuccess) e = cudaMemsetAsync(c->slab, 0, c->slab_bytes, c->stream);
  if (e == cudaSuccess) e = cudaMalloc(&c->partials, sizeof(double) * 4 * MAX_REDUCE_BLOCKS);
  if (e == cudaSuccess) e = cudaMalloc(&c->counter, 256);
  if (e == cudaSuccess) e = cudaMemsetAsync(c->counter, 0, 256, c->stream);
  if (e == cudaSuccess) e = cudaMalloc(&c->st, sizeof(LoopState));
  if (e == cudaSuccess) e = cudaMemsetAsync(c->st, 0, sizeof(LoopState), c->stream);
  if (e == cudaSuccess) e = cudaMallocHost(&c->st_host, sizeof(LoopState));
  if (e == cudaSuccess) e = cudaMalloc(&c->halo_list, sizeof(double*) * 16);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
  for (int i = 0; i < 3 * tl_ctx::BATCH && e == cudaSuccess; ++i) e = cudaEventCreate(&c->pev[i]);
  for (int i = 0; i < 2 * tl_ctx::QCAP && e == cudaSuccess; ++i) e = cudaEventCreate(&c->qev[i]);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess) {  // queried outside any capture
    cg_w_slots();  // occupancy of the matvec sweep
    sm_count();    // the update sweeps' grid
  }
  if (e != cudaSuccess) {
    int rc = (e == cudaErrorMemoryAllocation) ? TL_ERR_ALLOC : TL_ERR_CUDA;
    g_err = std::string("tl_create: ") + cudaGetErrorString(e);
    cudaGetLastError();
    tl_destroy(c);
    return rc;
  }
  memset(c->st_host, 0, sizeof(LoopState));
  Fields& f = c->f;
  f.density = c->slot(S_DENSITY);
  f.energy1 = c->slot(S_ENERGY1);
  f.u = c->slot(S_U);
  f.u0 = c->slot(S_U0);
  f.r = c->slot(S_R);
  f.w = c->slot(S_W);
  f.p = c->slot(S_P);
  f.p2 = c->slot(S_P2);
  f.kx = c->slot(S_KX);
  f.ky = c->slot(S_KY);
  f.cx = c->slot(S_CX);
  f.cy = c->slot(S_CY);
  f.di = c->slot(S_DI);
  f.z = c->slot(S_Z);
  f.mi = c->slot(S_MI);
  f.sd = c->slot(S_SD);
  f.sd1 = c->slot(S_SD1);
  f.utemp = c->slot(S_UTEMP);
  f.rtemp = c->slot(S_RTEMP);
  f.r_store = c->slot(S_RSTORE);
  f.cp = c->slot(S_CP);
  f.bfp = c->slot(S_BFP);
  f.u1 = c->slot(S_U1);
  f.jinv = c->slot(S_JINV);
  f.jden = c->slot(S_JDEN);
  *out = c;
  return TL_OK;
}

int tl_destroy(tl_ctx* c) {
  if (!c) return fail(TL_ERR_ARG, "tl_destroy: null context");
  if (c->stream) cudaStreamSynchronize(c->stream);
  cudaFree(c->slab);
  cudaFree(c->partials);
  cudaFree(c->counter);
  cudaFree(c->st);
  if (c->st_host) cudaFreeHost(c->st_host);
  cudaFree(c->hist_a);
  cudaFree(c->hist_b);
  cudaFree(c->ch_a);
  cudaFree(c->ch_b);
  cudaFree(c->states_dev);
  cudaFree(c->halo_list);
  cudaFree(c->mix_slab);
  cudaFree(c->mst);
  if (c->mst_host) cudaFreeHost(c->mst_host);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  for (int i = 0; i < 3 * tl_ctx::BATCH; ++i)
    if (c->pev[i]) cudaEventDestroy(c->pev[i]);
  for (int i = 0; i < 2 * tl_ctx::QCAP; ++i)
    if (c->qev[i]) cudaEventDestroy(c->qev[i]);
  if (c->up) cudaStreamSynchronize(c->up);
  if (c->down) cudaStreamSynchronize(c->down);
  cudaFree(c->xfer);
  for (int i = 0; i < 2; ++i) {
    if (c->st_done[i]) cudaEventDestroy(c->st_done[i]);
    if (c->st_used[i]) cudaEventDestroy(c->st_used[i]);
  }
  if (c->fe_snap) cudaEventDestroy(c->fe_snap);
  if (c->fe_done) cudaEventDestroy(c->fe_done);
  if (c->up) cudaStreamDestroy(c->up);
  if (c->down) cudaStreamDestroy(c->down);
  if (c->cg_exec) cudaGraphExecDestroy(c->cg_exec);
  if (c->cg_prof_exec) cudaGraphExecDestroy(c->cg_prof_exec);
  if (c->mix_exec) cudaGraphExecDestroy(c->mix_exec);
  cudaFree(c->tape);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return TL_OK;
}

int tl_host_register(void* host, unsigned long long bytes) {
  if (!host || bytes == 0) return fail(TL_ERR_ARG, "tl_host_register: null pointer or zero size");
  CK(cudaHostRegister(host, (size_t)bytes, cudaHostRegisterDefault));
  return TL_OK;
}

int tl_host_unregister(void* host) {
  if (!host) return fail(TL_ERR_ARG, "tl_host_unregister: null pointer");
  CK(cudaHostUnregister(host));
  return TL_OK;
}

int tl_host_alloc(unsigned long long bytes, void** host) {
  if (!host || bytes == 0) return fail(TL_ERR_ARG, "tl_host_alloc: null pointer or zero size");
  *host = nullptr;
  const cudaError_t e = cudaHostAlloc(host, (size_t)bytes, cudaHostAllocDefault);
  if (e != cudaSuccess) {
    *host = nullptr;
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? fail(TL_ERR_ALLOC, "tl_host_alloc: cudaHostAlloc failed")
                                          : cuda_fail(e, "tl_host_alloc");
  }
  return TL_OK;
}

int tl_host_free(void* host) {
  if (!host) return fail(TL_ERR_ARG, "tl_host_free: null pointer");
  CK(cudaFreeHost(host));
  return TL_OK;
}

int tl_device_bytes(const tl_ctx* c, unsigned long long* bytes) {
  if (!c || !bytes) return fail(TL_ERR_ARG, "tl_device_bytes: null argument");
  *bytes = c->slab_bytes + sizeof(double) * 4 * MAX_REDUCE_BLOCKS + 256 + sizeof(LoopState) +
           sizeof(double) * 2 * ((size_t)c->hist_cap + c->ch_cap) + c->mix_bytes + (c->tape ? c->tape_bytes : 0) +
           (c->xfer ? (size_t)tl_ctx::XFER_FIELDS * c->field_stride : 0);
  return TL_OK;
}

}  // extern "C"

namespace {
int ensure_xfer(tl_ctx* c) {
  if (c->xfer) return TL_OK;
  // each handle is made once, so a retry after a failed allocation leaks nothing
  if (!c->up) CK(cudaStreamCreateWithFlags(&c->up, cudaStreamNonBlocking));
  if (!c->down) CK(cudaStreamCreateWithFlags(&c->down, cudaStreamNonBlocking));
  for (int i = 0; i < 2; ++i) {
    if (!c->st_done[i]) CK(cudaEventCreateWithFlags(&c->st_done[i], cudaEventDisableTiming));
    if (!c->st_used[i]) CK(cudaEventCreateWithFlags(&c->st_used[i], cudaEventDisableTiming));
  }
  if (!c->fe_snap) CK(cudaEventCreateWithFlags(&c->fe_snap, cudaEventDisableTiming));
  if (!c->fe_done) CK(cudaEventCreateWithFlags(&c->fe_done, cudaEventDisableTiming));
  if (cudaMalloc(&c->xfer, tl_ctx::XFER_FIELDS * c->field_stride) != cudaSuccess) {
    cudaGetLastError();
    c->xfer = nullptr;
    return fail(TL_ERR_ALLOC, "cannot allocate the staging fields of the host transfers");
  }
  CK(cudaMemsetAsync(c->xfer, 0, tl_ctx::XFER_FIELDS * c->field_stride, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return TL_OK;
}

// One contiguous copy of a host array of x_cells x y_cells with row stride ld spans this many
// doubles; it is used when that fits a staging field (always when ld <= the context's stride).
long long host_span(const Layout& L, int ld) { return (long long)(L.ny - 1) * ld + L.nx; }
bool span_fits(const tl_ctx* c, int ld) { return host_span(c->L, ld) * (long long)sizeof(double) <= (long long)c->field_stride; }

// the staging fields, allocated on first use; false (and the row-by-row copies) if they cannot be
bool staging(tl_ctx* c) {
  if (c->xfer) return true;
  if (c->xfer_failed) return false;
  if (ensure_xfer(c) != TL_OK) {
    c->xfer_failed = true;
    cudaGetLastError();
    return false;
  }
  return true;
}
}  // namespace

extern "C" {

int tl_upload_field(tl_ctx* c, int field, const double* host, int ld) {
  if (!c || !host) return fail(TL_ERR_ARG, "tl_upload_field: null argument");
  double* d = field_ptr(c, field);
  if (!d) return fail(TL_ERR_ARG, "tl_upload_field: unknown field id");
  if (ld < c->L.nx) return fail(TL_ERR_ARG, "tl_upload_field: ld < x_cells");
  if (writes_setup_input(field)) c->setup_valid = false;
  if (span_fits(c, ld) && staging(c)) {
    CK(cudaMemcpyAsync(c->xfield(5), host, sizeof(double) * host_span(c->L, ld), cudaMemcpyHostToDevice,
                       c->stream));
    launch_unpack(d, c->xfield(5), ld, c->L, c->stream);
    int rc = check_launch("upload_field");
    if (rc) return rc;
  } else {
    CK(cudaMemcpy2DAsync(d + c->L.at(1, 1), sizeof(double) * c->L.ld, host, sizeof(double) * ld,
                         sizeof(double) * c->L.nx, c->L.ny, cudaMemcpyHostToDevice, c->stream));
  }
  CK(cudaStreamSynchronize(c->stream));
  return TL_OK;
}

int tl_download_field(tl_ctx* c, int field, double* host, int ld) {
  if (!c || !host) return fail(TL_ERR_ARG, "tl_download_field: null argument");
  double* d = field_ptr(c, field);
  if (!d) return fail(TL_ERR_ARG, "tl_download_field: unknown field id");
  if (ld < c->L.nx) return fail(TL_ERR_ARG, "tl_download_field: ld < x_cells");
  // a dense host array (ld == x_cells) takes one contiguous copy; with ld > x_cells the copy
  // goes row by row so that the host's columns beyond x_cells are left as they are
  if (ld == c->L.nx && staging(c)) {
    launch_pack(c->xfield(5), ld, d, c->L, c->stream);
    int rc = check_launch("download_field");
    if (rc) return rc;
    CK(cudaMemcpyAsync(host, c->xfield(5), sizeof(double) * host_span(c->L, ld), cudaMemcpyDeviceToHost,
                       c->stream));
  } else {
    CK(cudaMemcpy2DAsync(host, sizeof(double) * ld, d + c->L.at(1, 1), sizeof(double) * c->L.ld,
                         sizeof(double) * c->L.nx, c->L.ny, cudaMemcpyDeviceToHost, c->stream));
  }
  CK(cudaStreamSynchronize(c->stream));
  return TL_OK;
}

int tl_upload_state(tl_ctx* c, const double* density, const double* energy1, int ld) {
  if (!c || !density || !energy1) return fail(TL_ERR_ARG, "tl_upload_state: null argument");
  if (ld < c->L.nx) return fail(TL_ERR_ARG, "tl_upload_state: ld < x_cells");
  c->setup_valid = false;
  // Work fields need no clearing: every solve initialises what it reads, and halo cells stay
  // finite (zero from tl_create, or the generator's / reflective copies).
  if (span_fits(c, ld) && staging(c)) {
    const size_t bytes = sizeof(double) * host_span(c->L, ld);
    CK(cudaMemcpyAsync(c->xfield(5), density, bytes, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->xfield(6), energy1, bytes, cudaMemcpyHostToDevice, c->stream));
    launch_unpack(c->f.density, c->xfield(5), ld, c->L, c->stream);
    launch_unpack(c->f.energy1, c->xfield(6), ld, c->L, c->stream);
    int rc = check_launch("upload_state");
    if (rc) return rc;
  } else {
    CK(cudaMemcpy2DAsync(c->f.density + c->L.at(1, 1), sizeof(double) * c->L.ld, density, sizeof(double) * ld,
                         sizeof(double) * c->L.nx, c->L.ny, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpy2DAsync(c->f.energy1 + c->L.at(1, 1), sizeof(double) * c->L.ld, energy1, sizeof(double) * ld,
                         sizeof(double) * c->L.nx, c->L.ny, cudaMemcpyHostToDevice, c->stream));
  }
  if (c->g.reflective) {
    int rc = do_halo(c, M(TL_FIELD_DENSITY) | M(TL_FIELD_ENERGY1), c->halo_depth);
    if (rc) return rc;
  }
  CK(cudaStreamSynchronize(c->stream));
  return TL_OK;
}


int tl_stage_state(tl_ctx* c, const double* density, const double* energy1, int ld) {
  if (!c || !density || !energy1) return fail(TL_ERR_ARG, "tl_stage_state: null argument");
  if (ld < c->L.nx) return fail(TL_ERR_ARG, "tl_stage_state: ld < x_cells");
  int rc;
  if ((rc = ensure_xfer(c))) return rc;
  if (c->st_count == 2) return fail(TL_ERR_STATE, "tl_stage_state: two states are staged already");
  const int slot = c->st_head;
  if (c->st_used_rec[slot]) CK(cudaStreamWaitEvent(c->up, c->st_used[slot], 0));  // the slot's last take is done
  if (span_fits(c, ld)) {
    // one contiguous copy per array; tl_take_staged unpacks on the device
    const size_t bytes = sizeof(double) * host_span(c->L, ld);
    CK(cudaMemcpyAsync(c->xfield(2 * slot), density, bytes, cudaMemcpyHostToDevice, c->up));
    CK(cudaMemcpyAsync(c->xfield(2 * slot + 1), energy1, bytes, cudaMemcpyHostToDevice, c->up));
    c->st_ld[slot] = ld;
  } else {
    const size_t dp = sizeof(double) * c->L.ld, sp = sizeof(double) * ld, w = sizeof(double) * c->L.nx;
    CK(cudaMemcpy2DAsync(c->xfield(2 * slot) + c->L.at(1, 1), dp, density, sp, w, c->L.ny,
                         cudaMemcpyHostToDevice, c->up));
    CK(cudaMemcpy2DAsync(c->xfield(2 * slot + 1) + c->L.at(1, 1), dp, energy1, sp, w, c->L.ny,
                         cudaMemcpyHostToDevice, c->up));
    c->st_ld[slot] = 0;
  }
  CK(cudaEventRecord(c->st_done[slot], c->up));
  c->st_head ^= 1;
  c->st_count += 1;
  return TL_OK;
}

int tl_take_staged(tl_ctx* c) {
  if (!c) return fail(TL_ERR_ARG, "tl_take_staged: null context");
  if (c->st_count == 0) return fail(TL_ERR_STATE, "tl_take_staged: no state is staged");
  const int slot = (c->st_head + c->st_count) & 1;  // the oldest
  c->setup_valid = false;
  CK(cudaStreamWaitEvent(c->stream, c->st_done[slot], 0));
  if (c->st_ld[slot]) {
    launch_unpack(c->f.density, c->xfield(2 * slot), c->st_ld[slot], c->L, c->stream);
    launch_unpack(c->f.energy1, c->xfield(2 * slot + 1), c->st_ld[slot], c->L, c->stream);
    int rc = check_launch("take_staged");
    if (rc) return rc;
  } else {
    const size_t dp = sizeof(double) * c->L.ld, w = sizeof(double) * c->L.nx;
    CK(cudaMemcpy2DAsync(c->f.density + c->L.at(1, 1), dp, c->xfield(2 * slot) + c->L.at(1, 1), dp, w, c->L.ny,
                         cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemcpy2DAsync(c->f.energy1 + c->L.at(1, 1), dp, c->xfield(2 * slot + 1) + c->L.at(1, 1), dp, w,
                         c->L.ny, cudaMemcpyDeviceToDevice, c->stream));
  }
  if (c->g.reflective) {
    int rc = do_halo(c, M(TL_FIELD_DENSITY) | M(TL_FIELD_ENERGY1), c->halo_depth);
    if (rc) return rc;
  }
  CK(cudaEventRecord(c->st_used[slot], c->stream));
  c->st_used_rec[slot] = true;
  c->st_count -= 1;
  return TL_OK;
}

int tl_fetch_field(tl_ctx* c, int field, double* host, int ld) {
  if (!c || !host) return fail(TL_ERR_ARG, "tl_fetch_field: null argument");
  double* d = field_ptr(c, field);
  if (!d) return fail(TL_ERR_ARG, "tl_fetch_field: unknown field id");
  if (ld < c->L.nx) return fail(TL_ERR_ARG, "tl_fetch_field: ld < x_cells");
  int rc;
  if ((rc = ensure_xfer(c))) return rc;
  if (c->fe_done_rec) CK(cudaStreamWaitEvent(c->stream, c->fe_done, 0));  // the snapshot is free again
  const bool dense = ld == c->L.nx;  // one contiguous copy (else row by row: host columns beyond x_cells kept)
  if (dense) {
    launch_pack(c->xfield(4), ld, d, c->L, c->stream);
    if ((rc = check_launch("fetch_field"))) return rc;
  } else {
    CK(cudaMemcpyAsync(c->xfield(4), d, (size_t)c->L.elems() * sizeof(double), cudaMemcpyDeviceToDevice,
                       c->stream));
  }
  CK(cudaEventRecord(c->fe_snap, c->stream));
  CK(cudaStreamWaitEvent(c->down, c->fe_snap, 0));
  if (dense) {
    CK(cudaMemcpyAsync(host, c->xfield(4), sizeof(double) * host_span(c->L, ld), cudaMemcpyDeviceToHost, c->down));
  } else {
    CK(cudaMemcpy2DAsync(host, sizeof(double) * ld, c->xfield(4) + c->L.at(1, 1), sizeof(double) * c->L.ld,
                         sizeof(double) * c->L.nx, c->L.ny, cudaMemcpyDeviceToHost, c->down));
  }
  CK(cudaEventRecord(c->fe_done, c->down));
  c->fe_done_rec = true;
  return TL_OK;
}

int tl_wait_transfers(tl_ctx* c) {
  if (!c) return fail(TL_ERR_ARG, "tl_wait_transfers: null context");
  if (c->up) CK(cudaStreamSynchronize(c->up));
  if (c->down) CK(cudaStreamSynchronize(c->down));
  return TL_OK;
}

int tl_generate_chunk(tl_ctx* c, int nstates, const double* density, const double* energy, const double* xmin,
                      const double* xmax, const double* ymin, const double* ymax, const double* radius,
                      const int* geometry, double domain_xmin, double domain_ymin) {
  if (!c || nstates < 1 || !density || !energy || !xmin || !xmax || !ymin || !ymax || !radius || !geometry)
    return fail(TL_ERR_ARG, "tl_generate_chunk: invalid argument");
  std::vector<double> st(8 * (size_t)nstates);
  for (int s = 0; s < nstates; ++s) {
    // read_input.f90:352-359: states 2.. are nudged by a hundredth of a cell
    const double nx = s ? c->g.dx / 100.0 : 0.0, ny = s ? c->g.dy / 100.0 : 0.0;
    st[8 * s + 0] = density[s];
    st[8 * s + 1] = energy[s];
    st[8 * s + 2] = xmin[s] + nx;
    st[8 * s + 3] = xmax[s] - nx;
    st[8 * s + 4] = ymin[s] + ny;
    st[8 * s + 5] = ymax[s] - ny;
    st[8 * s + 6] = radius[s];
    st[8 * s + 7] = (double)geometry[s];
  }
  if (nstates > c->states_cap) {
    cudaFree(c->states_dev);
    c->states_dev = nullptr;
    CK(cudaMalloc(&c->states_dev, st.size() * sizeof(double)));
    c->states_cap = nstates;
  }
  c->setup_valid = false;
  CK(cudaMemsetAsync(c->slab, 0, c->slab_bytes, c->stream));
  CK(cudaMemcpyAsync(c->states_dev, st.data(), st.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  launch_generate(c->f, c->L, nstates, c->states_dev, domain_xmin, domain_ymin, c->g.dx, c->g.dy, c->stream);
  int rc = check_launch("generate_chunk");
  if (rc) return rc;
  // start.f90:113-118: prime density / energy halos (reflective only)
  rc = do_halo(c, M(TL_FIELD_DENSITY) | M(TL_FIELD_ENERGY1), c->halo_depth);
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream));  // states_dev is host-synchronous input
  return TL_OK;
}

int tl_field_summary(tl_ctx* c, double* vol, double* mass, double* ie, double* temp) {
  if (!c || !vol || !mass || !ie || !temp) return fail(TL_ERR_ARG, "tl_field_summary: null argument");
  launch_field_summary(c->f, c->L, c->g.dx * c->g.dy, c->rd(), c->stream);
  int rc = check_launch("field_summary");
  if (rc) return rc;
  double out[4];
  rc = reduce_result(c, out, 4);
  if (rc) return rc;
  *vol = out[0];
  *mass = out[1];
  *ie = out[2];
  *temp = out[3];
  return TL_OK;
}

// ---- per-kernel entry points ---------------------------------------------

int tl_common_init(tl_ctx* c, double dt) {
  if (!c) return fail(TL_ERR_ARG, "tl_common_init: null context");
  c->g.rx = dt / (c->g.dx * c->g.dx);
  c->g.ry = dt / (c->g.dy * c->g.dy);
  launch_init_faces(c->f, c->L, c->g, c->stream);
  launch_init_cells(c->f, c->L, c->g, true, c->stream);
  int rc = check_launch("common_init");
  if (rc) return rc;
  c->setup_valid = true;
  c->setup_dt = dt;
  CK(cudaStreamSynchronize(c->stream));
  return TL_OK;
}

int tl_calc_residual(tl_ctx* c) {
  if (!c) return fail(TL_ERR_ARG, "tl_calc_residual: null context");
  launch_residual(c->f, c->L, nullptr, RED_STORE, c->stream);
  int rc = check_launch("calc_residual");
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream));
  return TL_OK;
}

int tl_calc_2norm(tl_ctx* c, int norm_array, double* norm) {
  if (!c || !norm) return fail(TL_ERR_ARG, "tl_calc_2norm: null argument");
  if (norm_array != 0 && norm_array != 1) return fail(TL_ERR_ARG, "tl_calc_2norm: Invalid value for norm_array");
  launch_norm2(norm_array == 0 ? c->f.u0 : c->f.r, c->L, c->rd(), RED_STORE, c->stream);
  int rc = check_launch("calc_2norm");
  if (rc) return rc;
  return reduce_result(c, norm);
}

int tl_finalise(tl_ctx* c) {
  if (!c) return fail(TL_ERR_ARG, "tl_finalise: null context");
  launch_finalise(c->f, c->L, c->stream);
  int rc = check_launch("finalise");
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream));
  return TL_OK;
}

int tl_cg_init(tl_ctx* c, double* rro) {
  if (!c || !rro) return fail(TL_ERR_ARG, "tl_cg_init: null argument");
  launch_cg_init(c->f, c->L, c->g, c->rd(), RED_STORE, c->stream);
  int rc = check_launch("cg_init");
  if (rc) return rc;
  return reduce_result(c, rro);
}

int tl_cg_calc_w(tl_ctx* c, double* pw) {
  if (!c || !pw) return fail(TL_ERR_ARG, "tl_cg_calc_w: null argument");
  launch_cg_calc_w(c->f, c->L, c->rd(), c->stream);
  int rc = check_launch("cg_calc_w");
  if (rc) return rc;
  return reduce_result(c, pw);
}

int tl_cg_calc_ur(tl_ctx* c, double alpha, double* rrn) {
  if (!c || !rrn) return fail(TL_ERR_ARG, "tl_cg_calc_ur: null argument");
  launch_cg_calc_ur(c->f, c->L, c->g, alpha, c->rd(), c->stream);
  int rc = check_launch("cg_calc_ur");
  if (rc) return rc;
  return reduce_result(c, rrn);
}

int tl_cg_calc_p(tl_ctx* c, double beta, int ppcg_active) {
  if (!c) return fail(TL_ERR_ARG, "tl_cg_calc_p: null context");
  launch_cg_calc_p(c->f, c->L, beta, c->g.precond != TL_PREC_NONE || ppcg_active, c->stream);
  int rc = check_launch("cg_calc_p");
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream));
  return TL_OK;
}

int tl_cheby_init(tl_ctx* c, double theta) {
  if (!c) return fail(TL_ERR_ARG, "tl_cheby_init: null context");
  launch_cheby_init(c->f, c->L, c->g, theta, c->stream);
  int rc = check_launch("cheby_init");
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream));
  return TL_OK;
}

int tl_cheby_iterate(tl_ctx* c, double a, double b) {
  if (!c) return fail(TL_ERR_ARG, "tl_cheby_iterate: null context");
  launch_cheby_iterate(c->f, c->L, c->g, a, b, c->stream);
  int rc = check_launch("cheby_iterate");
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream));
  return TL_OK;
}

int tl_ppcg_init_sd(tl_ctx* c, double theta) {
  if (!c) return fail(TL_ERR_ARG, "tl_ppcg_init_sd: null context");
  launch_ppcg_init_sd(c->f, c->L, c->g, theta, c->stream);
  int rc = check_launch("ppcg_init_sd");
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream));
  return TL_OK;
}

int tl_ppcg_init(tl_ctx* c, int step, int ppcg_active, double* rro) {
  if (!c || !rro) return fail(TL_ERR_ARG, "tl_ppcg_init: null argument");
  if (step < 1 || step > 3) return fail(TL_ERR_ARG, "tl_ppcg_init: step must be 1, 2 or 3");
  launch_ppcg_init(c->f, c->L, c->g, step, ppcg_active != 0, c->rd(), RED_STORE, c->stream);
  int rc = check_launch("ppcg_init");
  if (rc) return rc;
  if (step == 2) {
    CK(cudaStreamSynchronize(c->stream));
    *rro = 0.0;
    return TL_OK;
  }
  return reduce_result(c, rro);
}

int tl_ppcg_inner(tl_ctx* c, double a, double b) {
  if (!c) return fail(TL_ERR_ARG, "tl_ppcg_inner: null context");
  launch_ppcg_inner(c->f, c->L, c->g, a, b, c->stream);
  int rc = check_launch("ppcg_inner");
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream));
  return TL_OK;
}

int tl_ppcg_calc_zrnorm(tl_ctx* c, int ppcg_active, double* rrn) {
  if (!c || !rrn) return fail(TL_ERR_ARG, "tl_ppcg_calc_zrnorm: null argument");
  const double* a = (c->g.precond != TL_PREC_NONE || ppcg_active) ? c->f.z : c->f.r;
  launch_dot(a, c->f.r, nullptr, c->L, c->rd(), RED_STORE, c->stream);
  int rc = check_launch("ppcg_calc_zrnorm");
  if (rc) return rc;
  return reduce_result(c, rrn);
}

int tl_ppcg_update_z(tl_ctx* c) {
  if (!c) return fail(TL_ERR_ARG, "tl_ppcg_update_z: null context");
  launch_copy_interior(c->f.z, c->f.utemp, c->L, c->stream);
  int rc = check_launch("ppcg_update_z");
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream));
  return TL_OK;
}

int tl_ppcg_store_r(tl_ctx* c) {
  if (!c) return fail(TL_ERR_ARG, "tl_ppcg_store_r: null context");
  launch_copy_interior(c->f.r_store, c->f.r, c->L, c->stream);
  int rc = check_launch("ppcg_store_r");
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream));
  return TL_OK;
}

int tl_ppcg_calc_rrn(tl_ctx* c, double* rrn) {
  if (!c || !rrn) return fail(TL_ERR_ARG, "tl_ppcg_calc_rrn: null argument");
  launch_dot(c->f.z, c->f.r, c->f.r_store, c->L, c->rd(), RED_STORE, c->stream);
  int rc = check_launch("ppcg_calc_rrn");
  if (rc) return rc;
  return reduce_result(c, rrn);
}

int tl_jacobi_solve(tl_ctx* c, double* error) {
  if (!c || !error) return fail(TL_ERR_ARG, "tl_jacobi_solve: null argument");
  launch_jacobi_denominator(c->f, c->L, c->g, c->stream);
  launch_jacobi(c->f, c->L, c->g, c->rd(), c->stream);
  int rc = check_launch("jacobi_solve");
  if (rc) return rc;
  return reduce_result(c, error);
}

int tl_update_halo(tl_ctx* c, int field_mask, int depth) {
  if (!c) return fail(TL_ERR_ARG, "tl_update_halo: null context");
  if (depth < 1) return fail(TL_ERR_ARG, "tl_update_halo: depth must be >= 1");
  for (int id = 1; id <= TL_FIELD_DI; ++id)
    if ((field_mask & (1 << id)) && writes_setup_input(id)) c->setup_valid = false;
  int rc = do_halo(c, field_mask, depth);
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream));
  return TL_OK;
}

int tl_reset_eigen(tl_ctx* c) {
  if (!c) return fail(TL_ERR_ARG, "tl_reset_eigen: null context");
  c->first = 1;
  c->have_coefs = false;
  return TL_OK;
}

int tl_cg_eigenvalues(const double* cg_alphas, const double* cg_betas, int nsteps, double* eigmin, double* eigmax) {
  if (!cg_alphas || !cg_betas || !eigmin || !eigmax || nsteps < 1)
    return fail(TL_ERR_ARG, "tl_cg_eigenvalues: null argument or nsteps < 1");
  const std::vector<double> a(cg_alphas, cg_alphas + nsteps), b(cg_betas, cg_betas + nsteps);
  if (calc_eigenvalues(a, b, nsteps, eigmin, eigmax)) return fail(TL_ERR_EIGEN, "Error in calculating eigenvalues");
  return TL_OK;
}

int tl_cheby_coefficients(double eigmin, double eigmax, int n, double* ch_alphas, double* ch_betas, double* theta) {
  if (!ch_alphas || !ch_betas || !theta || n < 1) return fail(TL_ERR_ARG, "tl_cheby_coefficients: null argument or n < 1");
  if (!(eigmax > eigmin)) return fail(TL_ERR_ARG, "tl_cheby_coefficients: eigmax must exceed eigmin");
  std::vector<double> a, b;
  calc_ch_coefs(a, b, eigmin, eigmax, theta, n);
  for (int i = 1; i <= n; ++i) {
    ch_alphas[i - 1] = a[i];
    ch_betas[i - 1] = b[i];
  }
  return TL_OK;
}

int tl_profile(tl_ctx* c, int enable) {
  if (!c) return fail(TL_ERR_ARG, "tl_profile: null context");
  int rc = prof_flush(c);
  if (rc) return rc;
  c->prof = enable != 0;
  if (c->prof)
    for (int i = 0; i < TL_NUM_KERNEL_TIMERS; ++i) {
      c->prof_ms[i] = 0.0;
      c->prof_n[i] = 0;
    }
  return TL_OK;
}

int tl_profile_read(tl_ctx* c, int kernel_id, double* total_ms, long long* launches) {
  if (!c || !total_ms || !launches) return fail(TL_ERR_ARG, "tl_profile_read: null argument");
  if (kernel_id < 0 || kernel_id >= TL_NUM_KERNEL_TIMERS) return fail(TL_ERR_ARG, "tl_profile_read: bad kernel id");
  int rc = prof_flush(c);
  if (rc) return rc;
  *total_ms = c->prof_ms[kernel_id];
  *launches = c->prof_n[kernel_id];
  return TL_OK;
}

}  // extern "C"

// ===========================================================================
// tl_tea_leaf
// ===========================================================================
namespace {

int ensure_mix(tl_ctx* c) {
  if (c->mix_slab) return TL_OK;
  const size_t fb = ((size_t)c->L.elems() * sizeof(float) + 4 * 256 + 255) / 256 * 256;
  const int nf = c->g.precond == TL_PREC_JAC_DIAG ? 11 : 9;  // + the FP32 Mi and z for jac_diag
  CK(cudaMalloc(&c->mix_slab, fb * nf));
  c->mix_bytes = fb * nf;
  CK(cudaMemsetAsync(c->mix_slab, 0, fb * nf, c->stream));
  float* b = reinterpret_cast<float*>(c->mix_slab);
  const size_t step = fb / sizeof(float);
  c->mix = MixFields{b,            b + step,     b + 2 * step, b + 3 * step, b + 4 * step,
                     b + 5 * step, b + 6 * step, b + 7 * step, b + 8 * step, c->counter + MIX_ERR_WORD,
                     nf == 11 ? b + 9 * step : nullptr, nf == 11 ? b + 10 * step : nullptr};
  CK(cudaMalloc(&c->mst, sizeof(MixState)));
  CK(cudaMallocHost(&c->mst_host, sizeof(MixState)));
  if (prepare_mix_kernels() != 0) return fail(TL_ERR_CUDA, "cannot set the mixed-precision kernels' shared memory");
  return TL_OK;
}

int sync_mix(tl_ctx* c) {
  CK(cudaMemcpyAsync(c->mst_host, c->mst, sizeof(MixState), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return TL_OK;
}

// TL_ERR_TIMEOUT (the word cleared) if a blocked FP32 sweep set the error word: a staged row did
// not arrive within its bounded wait (1), or its shared memory was misaligned for TMA (2).
int check_mix_err(tl_ctx* c) {
  unsigned werr = 0;
  CK(cudaMemcpyAsync(&werr, c->mix.err, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (!werr) return TL_OK;
  CK(cudaMemsetAsync(c->mix.err, 0, sizeof(unsigned), c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return fail(TL_ERR_TIMEOUT, werr == 1 ? "tl_tea_leaf: a staged row of a blocked FP32 sweep did not arrive in time"
                                        : "tl_tea_leaf: shared memory misaligned for the blocked FP32 sweep");
}

// Starts a fresh FP32 CG process on the correction (d must be zero): r = p = u0 - A u.
int mix_restart(tl_ctx* c, const Reduce& rd, double* floor_est) {
  MixState& H = *c->mst_host;
  // a fresh direction: the recorded CG process restarts (beta of the previous step = 0)
  if (H.hist_b && H.n > 1) CK(cudaMemsetAsync(H.hist_b + (H.n - 1), 0, sizeof(double), c->stream));
  launch_mix_trial(c->f, c->mix, c->L, rd, c->mst, true, c->stream);
  int rc;
  if ((rc = check_launch("mixed restart"))) return rc;
  if ((rc = sync_mix(c))) return rc;
  *floor_est = DBL_EPSILON * std::sqrt(H.trial_scale);
  H.rro = H.rr = H.rr_max = H.trial_rz32;
  H.p_pending = 0;
  H.status = RUN;
  return TL_OK;
}

// The CG presteps of the mixed Chebyshev form, as run by mixed_cg: where they stopped.
struct MixedPresteps {
  bool switched = false;     // the switch rule fired (else the CG solve finished the time step)
  int n = 0;                 // loop index of the first Chebyshev iteration
  double initial_residual = 0.0, residual = 0.0, floor_est = 0.0;
  int outer = 0;
};

// Mixed-precision CG (tl_mixed.cu): FP64 refinement loop around FP32 inner CG solves.
// Called by tl_tea_leaf after the set-up kernels; finishes the solve (finalise included).
// pre (non-null): the CG presteps of the mixed Chebyshev form -- the FP32 steps also stop at
// the reference's switch rule and record their alpha/beta for the eigenvalue estimate; on a
// switch the last correction is folded into u and the function returns without finalising.
int mixed_cg(tl_ctx* c, const tl_solve_opts* o, tl_solve_info* info, long long launches0,
             MixedPresteps* pre = nullptr) {
  int rc;
  if ((rc = ensure_mix(c))) return rc;
  MixState& H = *c->mst_host;
  memset(&H, 0, sizeof(H));
  if (pre) {
    H.switch_rr = o->ch_cg_epslim * o->ch_cg_epslim;
    H.presteps = o->ch_cg_presteps;
    H.hist_a = c->hist_a;
    H.hist_b = c->hist_b;
  }
  const double delta = o->inner_tol > 0.0 ? o->inner_tol : 0.5;
  H.delta2 = delta * delta;
  H.max_n = o->max_inner_iters > 0 ? std::min(o->max_inner_iters, o->max_iters) : o->max_iters;
  H.phase_end = 0x7fffffff;
  H.n = 1;  // step counter; the set-up trial puts p in the buffer step 1 reads
  const Reduce rd = c->rd();
  const size_t fbytes = (size_t)c->L.elems() * sizeof(float);
  CK(cudaMemsetAsync(c->mix.d, 0, fbytes, c->stream));  // a rejected correction may remain
  CK(cudaMemcpyAsync(c->mst, &H, sizeof(MixState), cudaMemcpyHostToDevice, c->stream));
  launch_mix_prep(c->f, c->mix, c->L, c->stream);
  launch_mix_trial(c->f, c->mix, c->L, rd, c->mst, true, c->stream);  // r = p = u0 - A u
  if ((rc = check_launch("mixed set-up"))) return rc;
  if ((rc = sync_mix(c))) return rc;
  // initial residual: the 2-norm of r as the reference's calc_2norm gives it; the loop's error
  // is sqrt(r.z) (= that norm without a preconditioner; tea_solve.f90:124-130,402-410)
  const double initial_residual = std::sqrt(std::fabs(H.trial_rr));
  H.rro = H.rr = H.rr_max = H.trial_rz32;
  H.n = 1;
  H.p_pending = 0;
  H.d_pending = 0;
  H.status = (H.trial_rz32 > 0.0 && std::isfinite(H.trial_rz32)) ? RUN : EXIT_CONVERGED;
  double res = std::sqrt(std::fabs(H.trial_rz)), prev = res;
  double true_res = initial_residual;  // ||u0 - A u||, the rounding-floor test's measure
  double floor_est = DBL_EPSILON * std::sqrt(H.trial_scale);
  int outer = 0, stalled = 0, stop = TL_STOP_EPS;
  bool rejected = false, stall_restarted = false;
  const int batch = tl_ctx::BATCH;
  while (H.status == RUN) {
    if (res < o->eps * initial_residual) {  // the reference's convergence test
      stop = TL_STOP_EPS;
      break;
    }
    if (true_res <= TL_FLOOR_FACTOR * floor_est) {  // no correction can lower it much further
      stop = TL_STOP_FLOOR;
      break;
    }
    // FP32 CG steps until the recursive residual has fallen by delta since the last
    // replacement (or the overall step cap)
    H.phase_end = 0x7fffffff;
    CK(cudaMemcpyAsync(c->mst, &H, sizeof(MixState), cudaMemcpyHostToDevice, c->stream));
    while (H.status == RUN) {
      const int n_before = H.n;
      if (!c->prof && use_graphs()) {
        if ((rc = run_mix_batch(c, rd))) return rc;
      } else {
        for (int i = 0; i < batch; ++i) {
          if (c->prof) CK(cudaEventRecord(c->pev[3 * i], c->stream));
          launch_mix_iteration(c->mix, c->L, rd, c->mst, c->stream, c->prof ? c->pev[3 * i + 1] : nullptr);
          if (c->prof) CK(cudaEventRecord(c->pev[3 * i + 2], c->stream));
        }
      }
      if ((rc = check_launch("mixed batch"))) return rc;
      if ((rc = sync_mix(c))) return rc;
      if (c->prof) {
        const int ran = std::min(std::max(H.n - n_before, 0), batch);
        for (int i = 0; i < ran; ++i) {
          float a = 0.f, b = 0.f;
          CK(cudaEventElapsedTime(&a, c->pev[3 * i], c->pev[3 * i + 1]));
          CK(cudaEventElapsedTime(&b, c->pev[3 * i + 1], c->pev[3 * i + 2]));
          c->prof_ms[TL_KERNEL_MIX_MATVEC] += a;
          c->prof_ms[TL_KERNEL_MIX_UPDATE] += b;
        }
        c->prof_n[TL_KERNEL_MIX_MATVEC] += ran;
        c->prof_n[TL_KERNEL_MIX_UPDATE] += ran;
      }
    }
    if (H.status == EXIT_BREAKDOWN) return fail(TL_ERR_BREAKDOWN, "tl_tea_leaf: non-finite FP32 CG scalar");
    const bool switching = pre && H.status == STOP_SWITCH;
    const bool capped = H.n > H.max_n;
    // trial replacement: true FP64 residual of u + d, u itself untouched
    launch_mix_flush_d(c->mix, c->L, c->mst, c->stream);  // the trial's epilogue clears d_pending
    launch_mix_trial(c->f, c->mix, c->L, rd, c->mst, false, c->stream);
    if ((rc = check_launch("mixed trial residual"))) return rc;
    if ((rc = sync_mix(c))) return rc;
    const double res_t = std::sqrt(std::fabs(H.trial_rz));
    if (!std::isfinite(res_t)) return fail(TL_ERR_BREAKDOWN, "tl_tea_leaf: non-finite residual");
    if (switching && !(res_t < prev)) {
      CK(cudaMemsetAsync(c->mix.d, 0, fbytes, c->stream));  // keep u, drop the correction
      pre->switched = true;
      break;
    }
    if (!(res_t < prev)) {
      // no gain: keep u and drop the correction.  Restart the FP32 process from the true
      // residual of u with a fresh direction; a second failure in a row means u sits at the
      // FP64 accuracy floor of u0 - A u.
      if (rejected || capped) {
        stop = capped ? TL_STOP_CAP : TL_STOP_REJECT;
        break;
      }
      rejected = true;
      CK(cudaMemsetAsync(c->mix.d, 0, fbytes, c->stream));
      if ((rc = mix_restart(c, rd, &floor_est))) return rc;
      continue;
    }
    launch_mix_apply(c->f, c->mix, c->L, c->stream);  // accept: u += d, d = 0
    ++outer;
    rejected = false;
    floor_est = DBL_EPSILON * std::sqrt(H.trial_scale);
    // replacements that keep gaining less than 10% each: restart the FP32 process once with a
    // fresh direction; if that does not bring back a 10% gain, u has reached the floor
    stalled = (res_t > 0.9 * prev) ? stalled + 1 : 0;
    if (stalled == 0) stall_restarted = false;
    res = prev = res_t;
    true_res = std::sqrt(std::fabs(H.trial_rr));
    if (switching) {
      pre->switched = true;
      break;
    }
    if (capped) {
      stop = TL_STOP_CAP;
      break;
    }
    if (stalled >= 3) {
      if (stall_restarted) {
        stop = TL_STOP_STALL;
        break;
      }
      stall_restarted = true;
      stalled = 0;
      if ((rc = mix_restart(c, rd, &floor_est))) return rc;  // d was zeroed by the apply
      continue;
    }
    // continue the CG process with r replaced by the true residual, search direction kept
    H.beta = H.trial_rz32 / H.rro_prev;
    if (H.hist_b) CK(cudaMemcpyAsync(H.hist_b + (H.n - 1), &H.beta, sizeof(double), cudaMemcpyHostToDevice, c->stream));
    H.rro = H.rr = H.rr_max = H.trial_rz32;
    H.p_pending = 1;
    H.status = RUN;
  }
  if (pre && pre->switched) {
    pre->n = H.n;
    pre->initial_residual = initial_residual;
    pre->residual = res;
    pre->floor_est = floor_est;
    pre->outer = outer;
    return check_launch("mixed CG presteps");
  }
  if (res < o->eps * initial_residual) stop = TL_STOP_EPS;
  const int inner_total = H.n - 1;
  finalise_sweep(c, false);
  if ((rc = do_halo(c, M(TL_FIELD_ENERGY1), 1))) return rc;
  if ((rc = check_launch("finalise"))) return rc;
  CK(cudaEventRecord(c->ev1, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if ((rc = prof_flush(c))) return rc;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  info->n_exit = inner_total;
  info->reported_iterations = inner_total;
  info->cg_calc_steps = inner_total;
  info->initial_residual = initial_residual;
  info->error = res;
  info->exact_error = true_res;
  info->true_residual = true_res;
  info->residual_floor = floor_est;
  info->stop_reason = stop;
  info->outer_iterations = outer;
  info->solve_seconds = ms * 1e-3;
  info->kernel_launches = launch_counter() - launches0;
  return TL_OK;
}

struct Solver {
  tl_ctx* c;
  const tl_solve_opts* o;
  int use_cg, use_cheby, use_ppcg, use_jacobi;
  std::vector<double> ch_a, ch_b;

  // reductions through the per-kernel path, result on the host
  int norm(const double* a, double* out) {
    launch_norm2(a, c->L, c->rd(), RED_STORE, c->stream);
    int rc = check_launch("norm2");
    if (rc) return rc;
    return reduce_result(c, out);
  }

  // Precision form: the inner steps in FP32 (tl_mixed_poly.cu), z = utemp in FP64.
  int run_ppcg_inner_steps32(int inner_steps) {
    if (inner_steps < 0) return TL_OK;
    int rc;
    if ((rc = prof_begin(c))) return rc;
    launch_poly_ppcg_inner(c->f, c->mix, c->L, c->theta, inner_steps, ch_a.data(), ch_b.data(), c->stream);
    if ((rc = prof_end(c, TL_KERNEL_POLY_STEP, std::max(inner_steps, 1)))) return rc;
    return check_launch("ppcg_inner_steps (FP32)");
  }

  // Chebyshev phase of the precision form, from the switch to the end of the solve: FP64
  // refinement cycles, each an FP32 Chebyshev solve of A d = r (the FP64 residual of u,
  // rounded) with the eigenvalue bounds and coefficients of the FP64 form, accepted (u += d in
  // FP64) only if the FP64 residual of u + d is lower.  The cycle length makes the Chebyshev
  // error bound fall by 1e-4 (gamma = (sqrt(cn)-1)/(sqrt(cn)+1), as est_itc uses).  Stops at
  // the reference's test on the FP64 residual, at its rounding floor, on a rejected or
  // stalled cycle, or when max_iters steps are used.  Returns the steps taken.
  int run_mixed_cheby(int budget, double initial_residual, double* error, int* steps, int* stop,
                      double* floor_out = nullptr) {
    const Reduce rd = c->rd();
    MixState& H = *c->mst_host;
    const double gamma = (std::sqrt(c->cn) - 1.0) / (std::sqrt(c->cn) + 1.0);
    int m = (gamma > 0.0 && gamma < 1.0) ? (int)std::ceil(std::log(1e-4) / std::log(gamma)) : 16;
    m = std::max(8, std::min(m, (int)ch_a.size() - 1));
    launch_poly_clear(c->mix, c->L, c->stream);
    // the residual with u's halo as it stands (not exchanged after the switch)
    launch_mix_trial(c->f, c->mix, c->L, rd, c->mst, false, c->stream, false);  // m.r = u0 - A u
    int rc;
    if ((rc = check_launch("mixed chebyshev residual"))) return rc;
    if ((rc = sync_mix(c))) return rc;
    double res = std::sqrt(std::fabs(H.trial_rr));
    double floor_est = DBL_EPSILON * std::sqrt(H.trial_scale);
    int total = 0, stalled = 0;
    *stop = TL_STOP_CAP;
    while (true) {
      if (res < o->eps * initial_residual) {
        *stop = TL_STOP_EPS;
        break;
      }
      if (res <= TL_FLOOR_FACTOR * floor_est) {
        *stop = TL_STOP_FLOOR;
        break;
      }
      const int len = std::min(m, budget - total);
      if (len < 1) break;
      if ((rc = prof_begin(c))) return rc;
      launch_poly_cheby(c->mix, c->L, c->theta, len, ch_a.data(), ch_b.data(), c->stream);
      if ((rc = prof_end(c, TL_KERNEL_POLY_STEP, len))) return rc;
      launch_mix_trial(c->f, c->mix, c->L, rd, c->mst, false, c->stream, false);  // m.r = u0 - A (u + d)
      if ((rc = check_launch("mixed chebyshev cycle"))) return rc;
      if ((rc = sync_mix(c))) return rc;
      if ((rc = check_mix_err(c))) return rc;
      total += len;
      const double res_t = std::sqrt(std::fabs(H.trial_rr));
      if (!std::isfinite(res_t)) return fail(TL_ERR_BREAKDOWN, "tl_tea_leaf: non-finite residual");
      if (!(res_t < res)) {
        *stop = TL_STOP_REJECT;  // d dropped; m.r already holds the residual of u + d, not needed
        break;
      }
      launch_mix_apply(c->f, c->mix, c->L, c->stream);  // u += d (FP64), d = 0
      stalled = (res_t > 0.5 * res) ? stalled + 1 : 0;
      res = res_t;
      floor_est = DBL_EPSILON * std::sqrt(H.trial_scale);
      if (stalled >= 3) {
        *stop = TL_STOP_STALL;
        break;
      }
    }
    *error = res;
    *steps = total;
    if (floor_out) *floor_out = floor_est;
    return check_launch("mixed chebyshev");
  }

  // fused: init_sd already ran in the outer update sweep, and z = utemp is left to the rrn sweep
  int run_ppcg_inner_steps(int inner_steps, bool fused = false) {
    // tea_leaf_ppcg.f90:211-431 on one chunk (every face external: bounds = interior)
    if (inner_steps < 0) return TL_OK;
    if (!fused) launch_ppcg_init_sd(c->f, c->L, c->g, c->theta, c->stream);
    const int h = c->halo_depth;
    int rc;
    if (!c->g.reflective && c->g.precond == TL_PREC_NONE && use_ppcg_inner_sweep()) {
      // one sweep per step, sd ping-ponging between its two fields (the halo exchanges are
      // no-ops without reflective boundaries)
      const double* sd_in = c->f.sd;
      double* sd_out = c->f.sd1;
      for (int step = 1; step <= inner_steps; ++step) {
        if ((rc = prof_begin(c))) return rc;
        launch_ppcg_inner_fused(c->f, c->L, sd_in, sd_out, ch_a[step], ch_b[step], c->stream);
        if ((rc = prof_end(c, TL_KERNEL_PPCG_INNER, 1))) return rc;
        const double* nx_in = sd_out;
        sd_out = const_cast<double*>(sd_in);
        sd_in = nx_in;
      }
      // no solver step reads sd again, but the field the solve leaves behind is the last step's
      if (sd_in != c->f.sd) launch_copy_interior(c->f.sd, c->f.sd1, c->L, c->stream);
      if (!fused) launch_copy_interior(c->f.z, c->f.utemp, c->L, c->stream);
      return check_launch("ppcg_inner_steps");
    }
    for (int cur = 1; cur <= inner_steps; cur += h) {
      if ((rc = do_halo(c, M(TL_FIELD_SD) | M(TL_FIELD_R), h))) return rc;
      for (int be = h - 1; be >= 0; --be) {
        const int step = cur + h - 1 - be;
        if ((rc = prof_begin(c))) return rc;
        launch_ppcg_inner(c->f, c->L, c->g, ch_a[step], ch_b[step], c->stream);
        if ((rc = prof_end(c, TL_KERNEL_PPCG_INNER, 1))) return rc;
        if (c->g.reflective && (rc = do_halo(c, M(TL_FIELD_SD), 1))) return rc;
        if (step == inner_steps) break;
      }
    }
    if (!fused) launch_copy_interior(c->f.z, c->f.utemp, c->L, c->stream);
    return check_launch("ppcg_inner_steps");
  }

  // The PPCG outer iterations from the one after the switch set-up to the end of the solve
  // (tea_solve.f90:289-331), the scalars on the device: the matvec sweep (p = z + beta p,
  // w = A p, p.w, r_store = r, z.r, alpha), the update sweep (u += alpha p, r -= alpha w,
  // init_sd), the inner sweeps, and the rrn sweep (z = utemp, (r - r_store).z, beta, the EXIT
  // test).  One status read per outer iteration instead of three scalar round trips.  p (from
  // ppcg_init step 3) is in the p field on entry.  Precondition: no preconditioner or jac_diag.
  int run_fused_ppcg(int n, double rro, double old_error, bool mixed, int inner, int* n_out, double* error,
                     bool* exited, int* outer_done, int* inner_done) {
    LoopState& H = *c->st_host;
    LoopArgs la = c->loop();
    int rc;
    // iteration n reads p_{n-1} from (n odd ? p : p2)
    if (!(n & 1)) launch_copy_all(c->f.p2, c->f.p, c->L, c->stream);
    H.n = n;
    H.status = RUN;
    H.p_pending = 0;
    H.u_pending = 0;
    H.check_switch = 0;
    H.rro = rro;
    H.old_error = old_error;
    H.theta = c->theta;
    if ((rc = push_state(c))) return rc;
    *outer_done = 0;
    *inner_done = 0;
    while (true) {
      launch_fused_cg_w(la, true, c->stream);
      launch_fused_ppcg_ur(la, !mixed, c->stream);
      if ((rc = mixed ? run_ppcg_inner_steps32(inner) : run_ppcg_inner_steps(inner, true))) return rc;
      launch_fused_ppcg_rrn(la, !mixed, c->stream);
      if ((rc = check_launch("ppcg outer iteration"))) return rc;
      if ((rc = sync_state(c))) return rc;
      *outer_done += 1;
      *inner_done += inner;
      if (H.status == EXIT_BREAKDOWN) {
        // a blocked FP32 inner sweep that gave up waiting leaves void values behind, which can
        // break the outer iteration down before the rrn sweep reports the timeout
        if (mixed && (rc = check_mix_err(c))) return rc;
        return fail(TL_ERR_BREAKDOWN, "tl_tea_leaf: non-finite PPCG scalar");
      }
      if (H.status == EXIT_TIMEOUT) {
        const int e = check_mix_err(c);
        return e ? e : fail(TL_ERR_TIMEOUT, "tl_tea_leaf: a blocked FP32 sweep gave up waiting");
      }
      if (H.status != RUN) break;
    }
    *error = H.error;
    *exited = H.status == EXIT_CONVERGED;
    *n_out = *exited ? H.n_exit : H.n;
    return TL_OK;
  }
};


}  // namespace

namespace {

int check_opts(const tl_ctx* c, const tl_solve_opts* o) {
  if (o->solver < TL_SOLVER_JACOBI || o->solver > TL_SOLVER_PPCG) return fail(TL_ERR_ARG, "tl_tea_leaf: bad solver");
  if (o->max_iters < 1) return fail(TL_ERR_ARG, "tl_tea_leaf: max_iters must be >= 1");
  if (o->precision != TL_PRECISION_FP64 && o->precision != TL_PRECISION_MIXED)
    return fail(TL_ERR_ARG, "tl_tea_leaf: unknown precision form");
  if (o->precision == TL_PRECISION_MIXED && (o->solver == TL_SOLVER_JACOBI || c->g.precond == TL_PREC_JAC_BLOCK))
    return fail(TL_ERR_ARG,
                "tl_tea_leaf: the mixed-precision form is implemented for CG, Chebyshev and PPCG without a "
                "preconditioner or with jac_diag");
  return TL_OK;
}

// One implicit solve (tea_solve.f90:37-503).  rhs (device, context layout; FP64 form only):
// solve A u = rhs from the initial guess u = rhs instead of A u = energy1 * density.
// finalise: energy1 = u / density at the end (tea_leaf_kernel_finalise).
int solve(tl_ctx* c, const tl_solve_opts* o, double dt, tl_solve_info* info, const double* rhs, bool finalise) {
  memset(info, 0, sizeof(*info));
  Solver S{c, o, o->solver == TL_SOLVER_CG, o->solver == TL_SOLVER_CHEBY, o->solver == TL_SOLVER_PPCG,
           o->solver == TL_SOLVER_JACOBI, {}, {}};
  int rc;
  const int max_iters = o->max_iters;
  if ((rc = ensure_hist(c, max_iters + 2))) return rc;
  const int inner = o->ppcg_inner_steps;
  if ((rc = ensure_ch(c, std::max(max_iters + 2, inner + 2)))) return rc;
  const long long launches0 = launch_counter();
  CK(cudaEventRecord(c->ev0, c->stream));

  // ---- INIT (tea_solve.f90:86-146) ----
  if ((rc = do_halo(c, M(TL_FIELD_ENERGY1) | M(TL_FIELD_DENSITY), c->halo_depth))) return rc;
  c->g.rx = dt / (c->g.dx * c->g.dx);
  c->g.ry = dt / (c->g.dy * c->g.dy);
  if (c->setup_valid && c->setup_dt == dt && use_setup_cache()) {
    launch_init_state(c->f, c->L, c->stream);  // u = u0 = energy1*density; the rest is unchanged
  } else {
    launch_init_faces(c->f, c->L, c->g, c->stream);
    launch_init_cells(c->f, c->L, c->g, false, c->stream);
    c->setup_valid = true;
    c->setup_dt = dt;
  }
  if (rhs) {
    launch_copy_interior(c->f.u0, rhs, c->L, c->stream);
    launch_copy_interior(c->f.u, rhs, c->L, c->stream);
  }
  if ((rc = do_halo(c, M(TL_FIELD_U), 1))) return rc;
  const bool mixed = o->precision == TL_PRECISION_MIXED;
  if (mixed && S.use_cg) return mixed_cg(c, o, info, launches0);
  if (mixed) {
    // FP32 copies of the operator for the Chebyshev / PPCG polynomial sweeps
    if ((rc = ensure_mix(c))) return rc;
    launch_mix_prep(c->f, c->mix, c->L, c->stream);
  }
  LoopState& H = *c->st_host;
  memset(&H, 0, sizeof(H));
  H.eps = o->eps;
  H.epslim = o->ch_cg_epslim;
  H.presteps = o->ch_cg_presteps;
  H.max_iters = max_iters;
  H.first = c->first;
  H.use_ppcg = S.use_ppcg;
  H.check_switch = (S.use_cheby || S.use_ppcg) ? 1 : 0;
  H.n = 1;
  H.status = RUN;
  H.theta = c->theta;
  if ((rc = push_state(c))) return rc;
  const bool cg_family = S.use_cg || S.use_cheby || S.use_ppcg;
  if (cg_family && c->g.precond != TL_PREC_JAC_BLOCK) {
    // calc_residual, its 2-norm and cg_init in one sweep
    launch_residual_cg_init(c->f, c->L, c->g, c->rd(), c->stream);
  } else {
    Reduce rd = c->rd();
    launch_residual(c->f, c->L, &rd, RED_INIT_RESIDUAL, c->stream);
  }
  if (cg_family) {
    if (c->g.precond == TL_PREC_JAC_BLOCK) launch_cg_init(c->f, c->L, c->g, c->rd(), RED_RRO, c->stream);
    if ((rc = do_halo(c, M(TL_FIELD_U) | M(TL_FIELD_P), 1))) return rc;
  } else if (S.use_jacobi) {
    launch_jacobi_denominator(c->f, c->L, c->g, c->stream);
  }
  if ((rc = check_launch("tea_leaf init"))) return rc;
  if ((rc = sync_state(c))) return rc;
  const double initial_residual = H.initial_residual;

  // ---- iteration (tea_solve.f90:152-414) ----
  int n = 1;
  double error = 0.0, old_error = H.old_error, rro = H.rro;
  int cheby_calc_steps = 0, est_itc = 0, ppcg_inner_iters = 0, cg_calc_steps = 0, max_cheby_iters = 0;
  bool ch_switch_check = false, ppcg_active = false, exited = false;
  int fields_mask = S.use_jacobi ? M(TL_FIELD_U) : M(TL_FIELD_P);
  const int batch = tl_ctx::BATCH;
  bool flush_in_finalise = false;  // the CG loop's last u update is left to the finalise sweep
  // FP64 Chebyshev iterations as one staged sweep each (no preconditioner, no reflective
  // boundaries): u ping-pongs between u and u1, u_alt when the latest is in u1
  const bool cheby_sweep = !c->g.reflective && c->g.precond == TL_PREC_NONE && use_cheby_sweep();
  bool u_alt = false;
  bool wr_stale = false;  // the last sweep left w and r unwritten
  // write_wr: the iteration's w and r are read (its residual is checked) or left behind (the last)
  auto cheby_iterate = [&](double a, double b, bool write_wr) {
    if (cheby_sweep) {
      launch_cheby_iterate_fused(c->f, c->L, u_alt ? c->f.u1 : c->f.u, u_alt ? c->f.u : c->f.u1, a, b, write_wr,
                                 c->stream);
      u_alt = !u_alt;
      wr_stale = !write_wr;
    } else {
      launch_cheby_iterate(c->f, c->L, c->g, a, b, c->stream);
    }
  };

  // Precision form without reflective boundaries: the CG presteps before the Chebyshev / PPCG
  // switch (tea_solve.f90:160-174) run as the mixed CG -- FP32 steps with FP64 residual
  // replacement, stopping at the reference's switch rule and recording their alpha/beta for
  // the eigenvalue estimate.  Chebyshev needs them every time step, PPCG only until the
  // eigenvalues are known.  The switch then proceeds from the FP64 residual of u.
  const bool mixed_presteps = mixed && !c->g.reflective && use_mixed_presteps() &&
                              (S.use_cheby || (S.use_ppcg && c->first));
  int presteps_outer = 0;
  if (mixed_presteps) {
    MixedPresteps pre;
    if ((rc = mixed_cg(c, o, info, launches0, &pre))) return rc;
    if (!pre.switched) return TL_OK;  // the CG steps finished the time step (finalised)
    launch_residual(c->f, c->L, nullptr, RED_STORE, c->stream);  // r = u0 - A u in FP64
    n = pre.n;
    cg_calc_steps = n - 1;
    old_error = pre.residual;
    ch_switch_check = true;
    presteps_outer = pre.outer;
  }

  while (n <= max_iters) {
    if (!ch_switch_check) {
      if (cheby_calc_steps > 0)
        ch_switch_check = true;
      else if (!c->first && S.use_ppcg && n > 1)
        ch_switch_check = true;
      else if (std::fabs(old_error) <= o->ch_cg_epslim && n >= o->ch_cg_presteps)
        ch_switch_check = true;
    }
    const bool cg_phase = (S.use_cg || S.use_cheby || S.use_ppcg) && !((S.use_cheby || S.use_ppcg) && ch_switch_check);

    if (cg_phase) {
      // device-resident CG loop, batches of iterations, one status read per batch
      LoopArgs la = c->loop();
      const int n_before = n;
      bool sampled = false;  // the timed graph form: only iteration TIMED_ITER of the batch is timed
      if (use_persistent(c)) {
        launch_flush_u(la, c->stream);  // a pending update of the batched kernels (none normally)
        unsigned* bar = c->counter + 4;  // barrier counter, generation, error word
        CK(cudaMemsetAsync(bar, 0, 3 * sizeof(unsigned), c->stream));
        // TL_CG_BARRIER_EXTRA=1: the barriers wait for one arrival that never comes, so every
        // wait runs out (about a second) and the solve reports TL_ERR_TIMEOUT -- the test of the
        // bounded wait
        const char* ex = getenv("TL_CG_BARRIER_EXTRA");
        CK(launch_persistent_cg(la, PERSIST_RUN, bar, c->pgrid, c->stream, ex && ex[0] == '1' ? 1 : 0));
      } else if (!c->prof && use_graphs()) {
        if ((rc = run_cg_batch(c, la))) return rc;
      } else if (use_graphs()) {
        if ((rc = run_cg_batch_timed(c, la))) return rc;
        sampled = true;
      } else {
        for (int i = 0; i < batch; ++i) {
          if (c->prof) CK(cudaEventRecord(c->pev[3 * i], c->stream));
          launch_fused_cg_w(la, false, c->stream);
          if (c->prof) CK(cudaEventRecord(c->pev[3 * i + 1], c->stream));
          launch_fused_cg_ur(la, c->stream);
          if (c->prof) CK(cudaEventRecord(c->pev[3 * i + 2], c->stream));
        }
      }
      if ((rc = check_launch("cg batch"))) return rc;
      if ((rc = sync_state(c))) return rc;
      if (c->prof) {
        // iterations of this batch that did work (the rest returned on the status word); the
        // graph form times its sampled iteration only
        int ran = (H.status == EXIT_CONVERGED || H.status == EXIT_BREAKDOWN) ? H.n_exit - n_before + 1
                                                                               : H.n - n_before;
        ran = std::min(std::max(ran, 0), batch);
        if (sampled) ran = ran > TIMED_ITER ? 1 : 0;
        for (int i = 0; i < ran; ++i) {
          float a = 0.f, b = 0.f;
          CK(cudaEventElapsedTime(&a, c->pev[3 * i], c->pev[3 * i + 1]));
          CK(cudaEventElapsedTime(&b, c->pev[3 * i + 1], c->pev[3 * i + 2]));
          c->prof_ms[TL_KERNEL_CG_MATVEC] += a;
          c->prof_ms[TL_KERNEL_CG_UPDATE] += b;
        }
        c->prof_n[TL_KERNEL_CG_MATVEC] += ran;
        c->prof_n[TL_KERNEL_CG_UPDATE] += ran;
      }
      cg_calc_steps = H.cg_calc_steps;
      if (H.status == EXIT_BREAKDOWN) return fail(TL_ERR_BREAKDOWN, "tl_tea_leaf: non-finite CG scalar");
      if (H.status == EXIT_TIMEOUT)
        return fail(TL_ERR_TIMEOUT, "tl_tea_leaf: a grid-barrier wait of the persistent CG kernel expired");
      if (H.status != RUN) {
        // the CG phase stops here: apply the deferred u += alpha p of its last iteration -- in
        // the finalise sweep when nothing reads u before it (a CG solve without check_result)
        if (S.use_cg && finalise && !o->check_result) {
          flush_in_finalise = true;
        } else {
          launch_flush_u(la, c->stream);
          H.u_pending = 0;
        }
      }
      error = H.error;
      old_error = H.old_error;
      rro = H.rro;
      if (H.status == EXIT_CONVERGED) {
        n = H.n_exit;
        exited = true;
        break;
      }
      n = H.n;
      if (H.status == EXIT_MAX_ITERS) break;
      if (H.status == STOP_SWITCH) {
        H.status = RUN;
        if ((rc = push_state(c))) return rc;
      }
      continue;
    }

    if (S.use_jacobi) {
      // device-resident Jacobi loop: un and u swap between the u and r fields; iteration m
      // reads (m odd ? u : r) and writes the other
      LoopArgs la = c->loop();
      while (H.status == RUN) {
        const int n_before = H.n;
        for (int i = 0; i < batch; ++i) {
          const int m = n_before + i;
          const double* un = (m & 1) ? c->f.u : c->f.r;
          double* uo = (m & 1) ? c->f.r : c->f.u;
          if (c->prof) CK(cudaEventRecord(c->pev[2 * i], c->stream));
          launch_fused_jacobi(la, un, uo, c->stream);
          if (c->prof) CK(cudaEventRecord(c->pev[2 * i + 1], c->stream));
        }
        if ((rc = check_launch("jacobi batch"))) return rc;
        if ((rc = sync_state(c))) return rc;
        if (c->prof) {
          int ran = (H.status == EXIT_CONVERGED || H.status == EXIT_BREAKDOWN) ? H.n_exit - n_before + 1
                                                                                 : H.n - n_before;
          ran = std::min(std::max(ran, 0), batch);
          for (int i = 0; i < ran; ++i) {
            float a = 0.f;
            CK(cudaEventElapsedTime(&a, c->pev[2 * i], c->pev[2 * i + 1]));
            c->prof_ms[TL_KERNEL_JACOBI] += a;
          }
          c->prof_n[TL_KERNEL_JACOBI] += ran;
        }
      }
      if (H.status == EXIT_BREAKDOWN) return fail(TL_ERR_BREAKDOWN, "tl_tea_leaf: non-finite Jacobi error");
      // the last iteration computed: n_exit when converged, max_iters otherwise
      const int last = H.status == EXIT_CONVERGED ? H.n_exit : H.n - 1;
      if (last >= 1 && (last & 1)) launch_copy_interior(c->f.u, c->f.r, c->L, c->stream);
      if ((rc = do_halo(c, M(TL_FIELD_U), 1))) return rc;
      error = H.error;
      n = H.status == EXIT_CONVERGED ? H.n_exit : H.n;
      exited = H.status == EXIT_CONVERGED;
      break;
    }

    // ---- Chebyshev / PPCG from iteration n: the switch set-up over the per-kernel path, then
    // Chebyshev iterations launched one by one, or the PPCG outer iterations as fused sweeps
    // (run_fused_ppcg; the per-kernel path for jac_block or TL_PPCG_FUSED=0) ----
    if ((S.use_cheby || S.use_ppcg) && ch_switch_check) {
      if (cheby_calc_steps == 0) {
        max_cheby_iters = max_iters - n + 2;
        if (c->first) {
          std::vector<double> ha(n - 1 > 0 ? n - 1 : 1), hb(ha.size());
          if (n - 1 > 0) {
            CK(cudaMemcpy(ha.data(), c->hist_a + 1, sizeof(double) * (n - 1), cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(hb.data(), c->hist_b + 1, sizeof(double) * (n - 1), cudaMemcpyDeviceToHost));
          }
          const int bad = calc_eigenvalues(ha, hb, n - 1, &c->eigmin, &c->eigmax);
          c->first = 0;
          if (bad) return fail(TL_ERR_EIGEN, "tea_leaf: Error in calculating eigenvalues");
          c->eigmin = c->eigmin * 0.95;
          c->eigmax = c->eigmax * 1.05;
        }
        if (S.use_cheby) {
          calc_ch_coefs(S.ch_a, S.ch_b, c->eigmin, c->eigmax, &c->theta, max_cheby_iters);
          fields_mask = M(TL_FIELD_U);
        } else {
          calc_ch_coefs(S.ch_a, S.ch_b, c->eigmin, c->eigmax, &c->theta, std::max(inner, 0));
          ppcg_active = true;
        }
        if ((int)S.ch_a.size() < inner + 2) {
          S.ch_a.resize(inner + 2, 0.0);
          S.ch_b.resize(inner + 2, 0.0);
        }
        c->cn = c->eigmax / c->eigmin;
        // p currently lives in whichever CG buffer the last iteration wrote; step 3 rebuilds p
        launch_ppcg_init(c->f, c->L, c->g, 2, ppcg_active, c->rd(), RED_STORE, c->stream);
        if ((rc = mixed ? S.run_ppcg_inner_steps32(inner) : S.run_ppcg_inner_steps(inner))) return rc;
        ppcg_inner_iters += inner;
        launch_ppcg_init(c->f, c->L, c->g, 3, ppcg_active, c->rd(), RED_STORE, c->stream);
        if ((rc = check_launch("ppcg_init"))) return rc;
        if ((rc = reduce_result(c, &rro))) return rc;
        if (mixed && (rc = check_mix_err(c))) return rc;  // the set-up's FP32 inner sweeps
        fields_mask = M(TL_FIELD_P);
        if ((rc = do_halo(c, fields_mask, 1))) return rc;
      }
      if (S.use_cheby && mixed) {
        int steps = 0, stop = 0;
        double floor_est = 0.0;
        if ((rc = S.run_mixed_cheby(max_iters - n + 1, initial_residual, &error, &steps, &stop, &floor_est)))
          return rc;
        if (mixed_presteps && (stop == TL_STOP_REJECT || stop == TL_STOP_STALL)) {
          // cycles that ended rejected or stalled: the mixed CG finishes from u (it stops at
          // once if u is already at the rounding floor); it finalises and reports
          const int done = n - 1 + steps;
          if ((rc = mixed_cg(c, o, info, launches0))) return rc;
          info->n_exit += done;
          info->reported_iterations += done;
          info->cg_calc_steps += cg_calc_steps;
          info->cheby_calc_steps = steps;
          info->outer_iterations += presteps_outer;
          info->initial_residual = initial_residual;
          info->eigmin = c->eigmin;
          info->eigmax = c->eigmax;
          return TL_OK;
        }
        cheby_calc_steps = steps;
        n += steps;
        info->stop_reason = stop;
        info->true_residual = error;
        info->residual_floor = floor_est;
        info->outer_iterations = presteps_outer;
        exited = true;
        break;
      }
      if (S.use_cheby) {
        if (cheby_calc_steps == 0) {
          double bb;
          if ((rc = S.norm(c->f.u0, &bb))) return rc;
          launch_cheby_init(c->f, c->L, c->g, c->theta, c->stream);
          if ((rc = do_halo(c, fields_mask, 1))) return rc;
          if ((rc = prof_begin(c))) return rc;
          cheby_iterate(S.ch_a[1], S.ch_b[1], true);
          if ((rc = prof_end(c, TL_KERNEL_CHEBY_ITERATE, 1))) return rc;
          if ((rc = S.norm(c->f.r, &old_error))) return rc;
          const double it_alpha = o->eps / 2.0 * std::sqrt(bb / old_error);
          const double gamm = (std::sqrt(c->cn) - 1.0) / (std::sqrt(c->cn) + 1.0);
          est_itc = (int)std::lround(std::log(it_alpha) / std::log(gamm));
          cheby_calc_steps = 1;
        } else {
          if ((rc = prof_begin(c))) return rc;
          cheby_iterate(S.ch_a[cheby_calc_steps], S.ch_b[cheby_calc_steps],
                        (n >= est_itc && n % 10 == 0) || n >= max_iters);
          if ((rc = prof_end(c, TL_KERNEL_CHEBY_ITERATE, 1))) return rc;
          if (n >= est_itc && n % 10 == 0) {
            if ((rc = S.norm(c->f.r, &error))) return rc;
          }
        }
      } else if (c->g.precond != TL_PREC_JAC_BLOCK && use_fused_ppcg()) {
        int outer = 0, inner_done = 0;
        if ((rc = S.run_fused_ppcg(n, rro, old_error, mixed, inner, &n, &error, &exited, &outer, &inner_done)))
          return rc;
        ppcg_inner_iters += inner_done;
        cheby_calc_steps += outer;
        break;
      } else {
        double pw, rrn;
        launch_cg_calc_w(c->f, c->L, c->rd(), c->stream);
        if ((rc = reduce_result(c, &pw))) return rc;
        launch_copy_interior(c->f.r_store, c->f.r, c->L, c->stream);
        launch_dot(c->f.z, c->f.r, nullptr, c->L, c->rd(), RED_STORE, c->stream);
        if ((rc = reduce_result(c, &rro))) return rc;
        const double alpha = rro / pw;
        launch_cg_calc_ur(c->f, c->L, c->g, alpha, c->rd(), c->stream);
        if ((rc = mixed ? S.run_ppcg_inner_steps32(inner) : S.run_ppcg_inner_steps(inner))) return rc;
        ppcg_inner_iters += inner;
        launch_dot(c->f.z, c->f.r, c->f.r_store, c->L, c->rd(), RED_STORE, c->stream);
        if ((rc = reduce_result(c, &rrn))) return rc;
        const double beta = rrn / rro;
        launch_cg_calc_p(c->f, c->L, beta, true, c->stream);
        error = rrn;
        rro = rrn;
      }
      cheby_calc_steps += 1;
    }
    if ((rc = do_halo(c, fields_mask, 1))) return rc;
    error = std::sqrt(std::fabs(error));
    if (std::fabs(error) < o->eps * initial_residual) {
      exited = true;
      break;
    }
    old_error = error;
    ++n;
  }
  (void)exited;
  if (wr_stale) {
    // the loop ended on an iteration whose w and r were not written (an exit on the stale error,
    // only when tl_eps times the initial residual exceeds 1): form them from that iteration's
    // input u as the sweep would have
    Fields fw = c->f;
    fw.u = u_alt ? c->f.u : c->f.u1;
    launch_cheby_wr(fw, c->L, c->stream);
  }
  if (u_alt) launch_copy_interior(c->f.u, c->f.u1, c->L, c->stream);  // the latest u back into u

  double exact_error = 0.0;
  if (o->check_result) {
    if ((rc = do_halo(c, M(TL_FIELD_U), 1))) return rc;
    Reduce rd = c->rd();
    launch_residual(c->f, c->L, &rd, RED_STORE, c->stream);
    if ((rc = reduce_result(c, &exact_error))) return rc;
    exact_error = std::sqrt(exact_error);
  }
  if (mixed && (rc = check_mix_err(c))) return rc;
  if (finalise) {
    finalise_sweep(c, flush_in_finalise);
    if ((rc = do_halo(c, M(TL_FIELD_ENERGY1), 1))) return rc;
  }
  if ((rc = check_launch("finalise"))) return rc;
  CK(cudaEventRecord(c->ev1, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);

  info->n_exit = n;
  info->reported_iterations = n - 1;
  info->ppcg_inner_iters = ppcg_inner_iters;
  info->cg_calc_steps = cg_calc_steps;
  info->cheby_calc_steps = cheby_calc_steps;
  info->est_itc = est_itc;
  info->initial_residual = initial_residual;
  info->error = error;
  info->exact_error = exact_error;
  info->eigmin = c->eigmin;
  info->eigmax = c->eigmax;
  if (mixed_presteps) info->outer_iterations = presteps_outer;
  info->solve_seconds = ms * 1e-3;
  info->kernel_launches = launch_counter() - launches0;
  return TL_OK;
}

}  // namespace

extern "C" int tl_tea_leaf(tl_ctx* c, const tl_solve_opts* o, double dt, tl_solve_info* info) {
  if (!c || !o || !info) return fail(TL_ERR_ARG, "tl_tea_leaf: null argument");
  int rc;
  if ((rc = check_opts(c, o))) return rc;
  return solve(c, o, dt, info, nullptr, true);
}

extern "C" int tl_tea_leaf_summary(tl_ctx* c, const tl_solve_opts* o, double dt, tl_solve_info* info,
                                   double* summary) {
  if (!c || !o || !info || !summary) return fail(TL_ERR_ARG, "tl_tea_leaf_summary: null argument");
  int rc;
  if ((rc = check_opts(c, o))) return rc;
  c->want_summary = true;
  rc = solve(c, o, dt, info, nullptr, true);
  c->want_summary = false;
  if (rc) return rc;
  return reduce_result(c, summary, 4);
}

extern "C" int tl_finalise_field_summary(tl_ctx* c, double* vol, double* mass, double* ie, double* temp) {
  if (!c || !vol || !mass || !ie || !temp) return fail(TL_ERR_ARG, "tl_finalise_field_summary: null argument");
  launch_finalise_summary(c->f, c->L, c->g.dx * c->g.dy, c->rd(), nullptr, c->stream);
  int rc = check_launch("finalise_field_summary");
  if (rc) return rc;
  double out[4];
  if ((rc = reduce_result(c, out, 4))) return rc;
  *vol = out[0];
  *mass = out[1];
  *ie = out[2];
  *temp = out[3];
  return TL_OK;
}

// ===========================================================================
// Adjoint of a run of time steps (tl_adjoint.cu has the kernels)
// ===========================================================================
extern "C" int tl_adjoint_begin(tl_ctx* c, int max_steps, int store_solutions) {
  if (!c) return fail(TL_ERR_ARG, "tl_adjoint_begin: null context");
  if (max_steps < 1) return fail(TL_ERR_ARG, "tl_adjoint_begin: max_steps must be >= 1");
  if (store_solutions != 0 && store_solutions != 1) return fail(TL_ERR_ARG, "tl_adjoint_begin: store_solutions is 0 or 1");
  CK(cudaStreamSynchronize(c->stream));
  cudaFree(c->tape);
  c->tape = nullptr;
  c->tape_max = c->tape_n = 0;
  const size_t nf = (size_t)max_steps * (1 + store_solutions) + 4;
  if (cudaMalloc(&c->tape, nf * c->field_stride) != cudaSuccess) {
    cudaGetLastError();
    c->tape = nullptr;
    return fail(TL_ERR_ALLOC, "tl_adjoint_begin: cannot allocate the checkpoint fields");
  }
  CK(cudaMemsetAsync(c->tape, 0, nf * c->field_stride, c->stream));
  c->tape_bytes = nf * c->field_stride;
  c->tape_max = max_steps;
  c->tape_store_u = store_solutions;
  c->tape_dt.assign(max_steps, 0.0);
  c->tape_opts.assign(max_steps, tl_solve_opts{});
  return TL_OK;
}

extern "C" int tl_adjoint_record_step(tl_ctx* c, const tl_solve_opts* o, double dt, tl_solve_info* info) {
  if (!c || !o || !info) return fail(TL_ERR_ARG, "tl_adjoint_record_step: null argument");
  if (!c->tape) return fail(TL_ERR_STATE, "tl_adjoint_record_step: no tape (call tl_adjoint_begin)");
  if (c->tape_n >= c->tape_max) return fail(TL_ERR_STATE, "tl_adjoint_record_step: tape full");
  int rc;
  if ((rc = check_opts(c, o))) return rc;
  const size_t fb = (size_t)c->L.elems() * sizeof(double);
  const int t = c->tape_n;
  CK(cudaMemcpyAsync(c->tape_field(t), c->f.energy1, fb, cudaMemcpyDeviceToDevice, c->stream));
  if ((rc = solve(c, o, dt, info, nullptr, true))) return rc;
  if (c->tape_store_u)
    CK(cudaMemcpyAsync(c->tape_field(c->tape_max + t), c->f.u, fb, cudaMemcpyDeviceToDevice, c->stream));
  c->tape_dt[t] = dt;
  c->tape_opts[t] = *o;
  c->tape_n = t + 1;
  CK(cudaStreamSynchronize(c->stream));
  return TL_OK;
}

extern "C" int tl_adjoint_backward(tl_ctx* c, const double* u_bar, const double* e_bar, int ld, double* density_bar,
                                   double* energy0_bar, tl_solve_info* info) {
  if (!c || !density_bar || !info) return fail(TL_ERR_ARG, "tl_adjoint_backward: null argument");
  if (ld < c->L.nx) return fail(TL_ERR_ARG, "tl_adjoint_backward: ld < x_cells");
  if (!c->tape || c->tape_n < 1) return fail(TL_ERR_STATE, "tl_adjoint_backward: no recorded steps");
  const Layout& L = c->L;
  const size_t fb = (size_t)L.elems() * sizeof(double);
  const int T = c->tape_n, base = c->tape_max * (1 + c->tape_store_u);
  double* rhs = c->tape_field(base);
  double* rho_bar = c->tape_field(base + 1);
  double* eb = c->tape_field(base + 2);
  double* u_re = c->tape_field(base + 3);
  const size_t row = sizeof(double) * L.nx, dpitch = sizeof(double) * L.ld, spitch = sizeof(double) * ld;
  CK(cudaMemsetAsync(rhs, 0, fb, c->stream));
  CK(cudaMemsetAsync(rho_bar, 0, fb, c->stream));
  CK(cudaMemsetAsync(eb, 0, fb, c->stream));
  if (u_bar)
    CK(cudaMemcpy2DAsync(rhs + L.at(1, 1), dpitch, u_bar, spitch, row, L.ny, cudaMemcpyHostToDevice, c->stream));
  if (e_bar)
    CK(cudaMemcpy2DAsync(eb + L.at(1, 1), dpitch, e_bar, spitch, row, L.ny, cudaMemcpyHostToDevice, c->stream));
  tl_solve_info total{}, one{};
  int rc;
  for (int t = T - 1; t >= 0; --t) {
    const double* e_t = c->tape_field(t);
    const double* u_t;
    if (c->tape_store_u) {
      u_t = c->tape_field(c->tape_max + t);
    } else {
      // recompute the step's solution from its checkpointed input energy
      CK(cudaMemcpyAsync(c->f.energy1, e_t, fb, cudaMemcpyDeviceToDevice, c->stream));
      if ((rc = solve(c, &c->tape_opts[t], c->tape_dt[t], &one, nullptr, true))) return rc;
      CK(cudaMemcpyAsync(u_re, c->f.u, fb, cudaMemcpyDeviceToDevice, c->stream));
      total.solve_seconds += one.solve_seconds;
      total.kernel_launches += one.kernel_launches;
      u_t = u_re;
    }
    // u_bar of this step: the loss term (last step only) plus e'_bar / rho
    launch_adj_rhs(t == T - 1 ? rhs : nullptr, eb, u_t, c->f.density, rhs, rho_bar, L, c->stream);
    // lambda = A^-1 u_bar by the FP64 CG solve (A is symmetric); lambda = 0 for u_bar = 0
    double nrm = 0.0;
    launch_norm2(rhs, L, c->rd(), RED_STORE, c->stream);
    if ((rc = check_launch("adjoint rhs"))) return rc;
    if ((rc = reduce_result(c, &nrm))) return rc;
    if (nrm > 0.0) {
      tl_solve_opts oc = c->tape_opts[t];
      oc.solver = TL_SOLVER_CG;
      oc.precision = TL_PRECISION_FP64;
      if ((rc = solve(c, &oc, c->tape_dt[t], &one, rhs, false))) return rc;
      total.reported_iterations += one.reported_iterations;
      total.solve_seconds += one.solve_seconds;
      total.kernel_launches += one.kernel_launches;
    } else {
      CK(cudaMemsetAsync(c->f.u, 0, fb, c->stream));
    }
    const double rx = c->tape_dt[t] / (c->g.dx * c->g.dx), ry = c->tape_dt[t] / (c->g.dy * c->g.dy);
    launch_adj_accumulate(c->f.u, u_t, e_t, c->f.density, rho_bar, eb, L, rx, ry, c->g.coefficient, c->stream);
    total.kernel_launches += 1;
    if ((rc = check_launch("adjoint step"))) return rc;
  }
  CK(cudaMemcpy2DAsync(density_bar, spitch, rho_bar + L.at(1, 1), dpitch, row, L.ny, cudaMemcpyDeviceToHost,
                       c->stream));
  if (energy0_bar)
    CK(cudaMemcpy2DAsync(energy0_bar, spitch, eb + L.at(1, 1), dpitch, row, L.ny, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  *info = total;
  return TL_OK;
}

extern "C" int tl_adjoint_end(tl_ctx* c) {
  if (!c) return fail(TL_ERR_ARG, "tl_adjoint_end: null context");
  CK(cudaStreamSynchronize(c->stream));
  cudaFree(c->tape);
  c->tape = nullptr;
  c->tape_max = c->tape_n = 0;
  return TL_OK;
}
