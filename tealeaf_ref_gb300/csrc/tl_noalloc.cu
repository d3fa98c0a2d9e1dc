// tl_noalloc.cu -- tl_cg_calc_w_noalloc: the CG matvec kernel (w = A p, pw = p.w) on
// caller-owned device arrays, without allocating any device memory.
//
// Who needs it: a caller that owns every byte of device memory itself -- for example a
// Fortran driver that keeps the reference's field arrays resident on the GPU through
// OpenACC or CUDA Fortran, a code running under a fixed device-memory budget, or a time
// loop that must never trigger a cudaMalloc/cudaFree (which can synchronise the device).
// Such a caller cannot use tl_create, whose context allocates the solver fields and the
// reduction buffers.
//
// The reduction needs scratch: one partial sum per interior row plus the final sum.  It
// lives in g_noalloc_scratch, a file-scope __device__ array of NOALLOC_MAX_ROWS + 32
// doubles (about 128 KiB) that every GPU loading this library holds until the process
// exits.  Host code must not pass the symbol itself to a kernel (on the host it is only a
// stand-in, not a device address): every call looks up the device address with
// cudaGetSymbolAddress for the device current at the call.  The first call on a device
// also loads this library's device code there (set-up); make that first call before any
// stream capture.  Looking the address up on every call, rather than caching it, keeps it
// right after the caller resets the device or its primary context (cudaDeviceReset, or a
// reset made by an OpenACC runtime), which can place the array at a new address.
//
// Each call overwrites every partial it reads, so nothing has to be cleared between
// calls; the array keeps the last call's values afterwards.  Calls whose kernels overlap
// on the GPU (different streams or host threads at the same time) share the one array and
// race: serialise them.
//
// Ordering: the two kernels and the copy of pw run on the legacy default stream, which
// waits for work on the caller's blocking streams but not for work on streams created with
// cudaStreamNonBlocking (OpenACC async queues, some framework streams).  The caller must
// finish its own writes of p, Kx, Ky and Di on such streams before the call.
#include <string>

#include "../../include/tealeaf_gb300.h"

namespace tl {
void set_last_error(const std::string& msg);
}

namespace {

constexpr int NOALLOC_MAX_ROWS = 16384;  // largest y_cells the scratch array serves
constexpr int NOALLOC_THREADS = 256;

static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_MAX_ROWS + 32];

int fail(int code, const std::string& msg) {
  tl::set_last_error(msg);
  return code;
}

int cuda_fail(cudaError_t e, const char* where) {
  return fail(TL_ERR_CUDA, std::string("tl_cg_calc_w_noalloc: ") + where + ": " + cudaGetErrorString(e));
}

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ double block_sum(double v) {
  __shared__ double s[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) s[wid] = v;
  __syncthreads();
  v = (threadIdx.x < (blockDim.x >> 5)) ? s[lane] : 0.0;
  return wid == 0 ? warp_sum(v) : 0.0;
}

// tea_leaf_cg_calc_w_kernel (kernels/tea_leaf_cg_kernel.f90:114-156) on arrays dimensioned
// (1-h : nx+h, 1-h : ny+h), x fastest; one CTA per interior row (strided), the row's p.w
// partial goes to scratch[k-1].
__global__ void k_calc_w_rows(int nx, int ny, int h, const double* __restrict__ p, double* __restrict__ w,
                              const double* __restrict__ kx, const double* __restrict__ ky,
                              const double* __restrict__ di, double rx, double ry, double* __restrict__ scratch) {
  const long long ldx = (long long)nx + 2LL * h;
  for (int k = blockIdx.x + 1; k <= ny; k += gridDim.x) {
    double acc = 0.0;
    for (int j = threadIdx.x + 1; j <= nx; j += blockDim.x) {
      const long long c = (long long)(k - 1 + h) * ldx + (j - 1 + h);
      const double v = di[c] * p[c] - ry * (ky[c + ldx] * p[c + ldx] + ky[c] * p[c - ldx]) -
                       rx * (kx[c + 1] * p[c + 1] + kx[c] * p[c - 1]);
      w[c] = v;
      acc = fma(v, p[c], acc);
    }
    acc = block_sum(acc);
    if (threadIdx.x == 0) scratch[k - 1] = acc;
  }
}

// Sums the ny row partials in a fixed order into scratch[NOALLOC_MAX_ROWS].
__global__ void k_sum_rows(int ny, double* __restrict__ scratch) {
  double acc = 0.0;
  for (int i = threadIdx.x; i < ny; i += blockDim.x) acc += scratch[i];
  acc = block_sum(acc);
  if (threadIdx.x == 0) scratch[NOALLOC_MAX_ROWS] = acc;
}

}  // namespace

extern "C" int tl_cg_calc_w_noalloc(int x_cells, int y_cells, int halo_depth, const double* p, double* w,
                                    const double* kx, const double* ky, const double* di, double rx, double ry,
                                    double* pw) {
  if (!p || !w || !kx || !ky || !di || !pw) return fail(TL_ERR_ARG, "tl_cg_calc_w_noalloc: null pointer");
  if (x_cells < 1 || y_cells < 1 || halo_depth < 1)
    return fail(TL_ERR_ARG, "tl_cg_calc_w_noalloc: x_cells, y_cells and halo_depth must be >= 1");
  if (y_cells > NOALLOC_MAX_ROWS)
    return fail(TL_ERR_ARG, "tl_cg_calc_w_noalloc: y_cells exceeds the 16384-row limit of its fixed scratch array");
  const long long dim_x = (long long)x_cells + 2LL * halo_depth, dim_y = (long long)y_cells + 2LL * halo_depth;
  if (dim_x >= (1LL << 31) || dim_y >= (1LL << 31) || dim_x * dim_y >= (1LL << 40))
    return fail(TL_ERR_ARG, "tl_cg_calc_w_noalloc: array too large");
  // device address of the scratch array on the current device (see the file comment)
  void* sym = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&sym, g_noalloc_scratch);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress");
  if (!sym) return fail(TL_ERR_CUDA, "tl_cg_calc_w_noalloc: cudaGetSymbolAddress returned no address");
  double* scratch = static_cast<double*>(sym);
  // Launched through cudaLaunchKernel so that each launch's own status is checked; an error
  // the caller's earlier work left in the runtime's last-error slot is neither reported nor
  // cleared here.
  int nx = x_cells, ny = y_cells, h = halo_depth;
  double rxv = rx, ryv = ry;
  void* w_args[] = {&nx, &ny, &h, (void*)&p, (void*)&w, (void*)&kx, (void*)&ky, (void*)&di, &rxv, &ryv, &scratch};
  const unsigned grid = y_cells < 4096 ? (unsigned)y_cells : 4096u;
  e = cudaLaunchKernel((const void*)k_calc_w_rows, dim3(grid), dim3(NOALLOC_THREADS), w_args, 0, 0);
  if (e != cudaSuccess) return cuda_fail(e, "launch of the matvec kernel");
  void* s_args[] = {&ny, &scratch};
  e = cudaLaunchKernel((const void*)k_sum_rows, dim3(1), dim3(1024), s_args, 0, 0);
  if (e != cudaSuccess) return cuda_fail(e, "launch of the row-sum kernel");
  e = cudaMemcpy(pw, scratch + NOALLOC_MAX_ROWS, sizeof(double), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "copy of pw");
  return TL_OK;
}
