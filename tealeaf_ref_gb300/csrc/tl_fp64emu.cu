// tl_fp64emu.cu -- check entry for the integer-pipe FP64 multiply of tl_fp64emu.cuh.
//
// tl_fp64_emu_check runs dmul_int and the FP64 instruction (mul.rn.f64) on the same operands
// on the GPU and returns both results, so that a test can compare them bit for bit.  It is a
// diagnostic of this library, not part of the reference's interface, and is not declared in
// the public header.
#include <cuda_runtime.h>

#include "tl_fp64emu.cuh"

namespace {

__global__ void k_fp64_emu_check(const double* __restrict__ a, const double* __restrict__ b, long long n,
                                 double* __restrict__ emu, double* __restrict__ hw) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    emu[i] = tl::dmul_int(a[i], b[i]);
    hw[i] = __dmul_rn(a[i], b[i]);
  }
}

}  // namespace

// a*b for host arrays of n elements: emu_out from dmul_int, hw_out from mul.rn.f64.  Returns
// 0, -1 for a bad argument, -2 when a CUDA call fails.
extern "C" int tl_fp64_emu_check(const double* a, const double* b, long long n, double* emu_out, double* hw_out) {
  if (n < 0 || (n > 0 && (!a || !b || !emu_out || !hw_out))) return -1;
  if (n == 0) return 0;
  const size_t bytes = (size_t)n * sizeof(double);
  double* d = nullptr;
  if (cudaMalloc(&d, 4 * bytes) != cudaSuccess) {
    cudaGetLastError();
    return -2;
  }
  double *da = d, *db = d + n, *de = d + 2 * n, *dh = d + 3 * n;
  bool ok = cudaMemcpy(da, a, bytes, cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemcpy(db, b, bytes, cudaMemcpyHostToDevice) == cudaSuccess;
  if (ok) {
    const long long blocks = (n + 255) / 256;
    k_fp64_emu_check<<<(unsigned)(blocks < 4096 ? blocks : 4096), 256>>>(da, db, n, de, dh);
    ok = cudaGetLastError() == cudaSuccess && cudaDeviceSynchronize() == cudaSuccess &&
         cudaMemcpy(emu_out, de, bytes, cudaMemcpyDeviceToHost) == cudaSuccess &&
         cudaMemcpy(hw_out, dh, bytes, cudaMemcpyDeviceToHost) == cudaSuccess;
  }
  cudaFree(d);
  if (!ok) cudaGetLastError();
  return ok ? 0 : -2;
}
