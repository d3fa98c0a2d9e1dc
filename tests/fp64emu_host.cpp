// Host build of the integer-pipe FP64 multiply (tealeaf_ref_gb300/csrc/tl_fp64emu.cuh),
// checked bit for bit against the FPU's multiply on seeded operands of every class: random
// bit patterns (zeros, subnormals, infinities, NaNs), normal operands over a narrow and the
// full exponent range, significands with few bits set (exact products and ties), and
// products at the edges of the normal range (overflow, subnormal results, underflow to zero).
// Usage: fp64emu_host N SEED; prints the mismatch count, exits 1 on any mismatch.
#include "tl_fp64emu.cuh"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

using tl::emu::FRAC;
using tl::emu::SIGN;

static uint64_t bits_of(double x) {
  uint64_t u;
  std::memcpy(&u, &x, 8);
  return u;
}
static double of_bits(uint64_t u) {
  double x;
  std::memcpy(&x, &u, 8);
  return x;
}
static bool same(double a, double b) { return bits_of(a) == bits_of(b) || (std::isnan(a) && std::isnan(b)); }

int main(int argc, char** argv) {
  const long n = argc > 1 ? atol(argv[1]) : 1000000;
  std::mt19937_64 g(argc > 2 ? strtoull(argv[2], nullptr, 10) : 1);
  auto with_exp = [&](int e) { return of_bits((g() & (FRAC | SIGN)) | ((uint64_t)e << 52)); };
  auto draw = [&](int mode) -> double {
    switch (mode) {
      case 0: return of_bits(g());                                  // any class
      case 1: return with_exp(1023 + (int)(g() % 80) - 40);        // normal, narrow range
      case 2: {                                                     // few significand bits
        const uint64_t m = g() & FRAC & ~((1ull << (g() % 53)) - 1);
        return of_bits((g() & SIGN) | m | ((uint64_t)(1018 + g() % 10) << 52));
      }
      case 3: return with_exp((int)(g() % 2047));                   // normal or subnormal, any range
      default: return with_exp((g() & 1) ? 1 + (int)(g() % 40) : 2046 - (int)(g() % 40));  // range edges
    }
  };
  long bad = 0;
  for (long i = 0; i < n; ++i) {
    const int mode = (int)(i % 5);
    double a = draw(mode), b = draw(mode);
    if (mode == 4) b = with_exp(1023 + (int)(g() % 3) - 1);  // keep products near the edges too
    if (i % 17 == 0) a = (g() & 1) ? 0.0 : -0.0;
    volatile double hw = a * b;
    const double em = tl::dmul_int(a, b);
    if (!same(hw, em) && bad++ < 5) printf("mul %a * %a: %a, integer %a\n", a, b, (double)hw, em);
  }
  printf("n %ld mismatch %ld\n", n, bad);
  return bad ? 1 : 0;
}
