// tl_adjoint.cu -- kernels of the reverse (adjoint) sweep through tea_leaf() time steps.
//
// One forward step (tea_solve.f90 with tea_leaf_common_kernel.f90:67-152 and :179-206):
//   b = e * rho,  A(rho) u = b,  e' = u / rho,
// with A u = u + sum over interior faces f=(L,R) of c_f (u_L - u_R) on both cells,
// c_f = rx Kx_f (x faces) or ry Ky_f (y faces), Kx_f = (w_L + w_R) / (2 w_L w_R),
// w = rho (CONDUCTIVITY) or 1/rho (RECIP_CONDUCTIVITY); external faces are zero (or, with
// reflective boundaries, cancelled by the mirrored halo), so they carry no gradient.
//
// Reverse step, given e'_bar (adjoint of the step's output energy) and u_bar (a loss on u):
//   u_bar += e'_bar / rho;            rho_bar -= e'_bar u / rho^2          (k_adj_rhs)
//   lambda = A^-1 u_bar               (A is symmetric: the forward CG solve, tl_api.cu)
//   rho_bar += lambda e               (b = e rho)
//   Kx_bar_f = -rx (lambda_L - lambda_R)(u_L - u_R), Ky likewise          (dA/dK)
//   w_bar += Kx_bar_f * dKx_f/dw = -Kx_bar_f / (2 w^2) per face side, chained to rho
//   e_bar = lambda rho                (adjoint of the step's input energy) (k_adj_accumulate)
#include "tl_kernels.cuh"

namespace tl {

namespace {

constexpr int AT = 256;

inline dim3 adj_grid(const Layout& L) {
  const int gy = L.ny < 65535 ? L.ny : 65535;
  return dim3((L.nx + AT - 1) / AT, gy);
}

// rhs = u_bar_ext (nullable) + e_bar / rho;  rho_bar -= e_bar u / rho^2.  In place on rhs is
// allowed (u_bar_ext == rhs).
__global__ void k_adj_rhs(const double* u_bar_ext, const double* e_bar, const double* u, const double* rho,
                          double* rhs, double* rho_bar, Layout L) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (j > L.nx) return;
  for (int k = blockIdx.y + 1; k <= L.ny; k += gridDim.y) {
    const long long c = L.at(j, k);
    double r = u_bar_ext ? u_bar_ext[c] : 0.0;
    const double eb = e_bar[c];
    const double inv = 1.0 / rho[c];
    r += eb * inv;
    rho_bar[c] -= eb * u[c] * inv * inv;
    rhs[c] = r;
  }
}

// rho_bar += lambda e + (face terms chained through w to rho);  e_bar = lambda rho.
// Each cell gathers the gradient of its own w from its (up to four) interior faces.
__global__ void k_adj_accumulate(const double* lam, const double* u, const double* e, const double* rho,
                                 double* rho_bar, double* e_bar, Layout L, double rx, double ry, int coefficient) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (j > L.nx) return;
  for (int k = blockIdx.y + 1; k <= L.ny; k += gridDim.y) {
    const long long c = L.at(j, k);
    const double lc = lam[c], uc = u[c];
    double ks = 0.0;  // sum over this cell's interior faces of K_bar_f
    if (j > 1) ks -= rx * (lam[c - 1] - lc) * (u[c - 1] - uc);
    if (j < L.nx) ks -= rx * (lam[c + 1] - lc) * (u[c + 1] - uc);
    if (k > 1) ks -= ry * (lam[c - L.ld] - lc) * (u[c - L.ld] - uc);
    if (k < L.ny) ks -= ry * (lam[c + L.ld] - lc) * (u[c + L.ld] - uc);
    const double r = rho[c];
    // dK_f/dw = -1/(2 w^2); w = rho: dw/drho = 1; w = 1/rho: dw/drho = -1/rho^2 (product 1/2)
    const double dk = coefficient == 2 ? 0.5 * ks : -ks / (2.0 * r * r);
    rho_bar[c] += lc * e[c] + dk;
    e_bar[c] = lc * r;
  }
}

}  // namespace

void launch_adj_rhs(const double* u_bar_ext, const double* e_bar, const double* u, const double* rho, double* rhs,
                    double* rho_bar, const Layout& L, cudaStream_t s) {
  { ++launch_counter(); k_adj_rhs<<<adj_grid(L), AT, 0, s>>>(u_bar_ext, e_bar, u, rho, rhs, rho_bar, L); }
}

void launch_adj_accumulate(const double* lam, const double* u, const double* e, const double* rho, double* rho_bar,
                           double* e_bar, const Layout& L, double rx, double ry, int coefficient, cudaStream_t s) {
  {
    ++launch_counter();
    k_adj_accumulate<<<adj_grid(L), AT, 0, s>>>(lam, u, e, rho, rho_bar, e_bar, L, rx, ry, coefficient);
  }
}

}  // namespace tl
