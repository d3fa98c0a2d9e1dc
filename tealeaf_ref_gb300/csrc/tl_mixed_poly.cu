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

}  // namespace

void launch_poly_ppcg_inner(const Fields& f, const MixFields& m, const Layout& L, double theta, int inner_steps,
                            const double* ch_a, const double* ch_b, cudaStream_t s) {
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
