// tl_fp64emu.cuh -- the FP64 multiply computed on the integer pipes.
//
// On GB300 the FP64 pipe retires 2 thread-operations per clock per SM (the FP32 pipes 128):
// one warp's FP64 instruction holds its sub-partition's FP64 pipe for 64 cycles, while the
// integer pipes and most issue slots of an FP64-bound sweep sit idle.  A sweep with
// standalone products can move some of them onto integer instructions and shorten the FP64
// pipe's work, as long as the warps have the issue slots and registers to spare.
//
// dmul_int(x, y) returns the IEEE-754 binary64 product rounded to nearest, ties to even --
// the bits of mul.rn.f64 -- from the operands' integer representations: unpack sign, biased
// exponent and 53-bit significand, form the exact 106-bit product (four 32 x 32-bit products),
// round on the guard bit and the sticky bits below it, and pack (IEEE 754-2008 sections 4.3.1
// and 7.4).  Every class of operand is handled in integer arithmetic: zeros, subnormal
// operands (normalised first) and results (the exact product shifted into the subnormal range
// and rounded once), overflow to infinity, infinities and NaNs (a NaN result is the quiet NaN
// 0x7fff...f).
//
// A warp's FP64 instruction that is predicated off still holds the FP64 pipe, and the
// compiler turns integer tests on a double's bits back into FP64 compares unless the bits are
// taken with an opaque move: so no FP64 instruction appears anywhere in dmul_int, and a warp
// enters the general cases only when one of its lanes needs them.
//
// The function also compiles for the host (g++), where a CPU test checks it bit for bit
// against the FPU's multiply.
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define TL_EMU_FN __host__ __device__ __forceinline__
#else
#define TL_EMU_FN inline
#endif

namespace tl {
namespace emu {

constexpr uint64_t SIGN = 0x8000000000000000ull;
constexpr uint64_t FRAC = 0x000fffffffffffffull;
constexpr uint64_t HIDDEN = 0x0010000000000000ull;

// On the device the reinterpretation is an opaque move: the compiler would otherwise turn the
// integer tests on the bits (zero, exponent range) back into floating-point compares, which
// issue on the FP64 pipe.
TL_EMU_FN uint64_t bits(double x) {
#if defined(__CUDA_ARCH__)
  uint64_t u;
  asm("mov.b64 %0, %1;" : "=l"(u) : "d"(x));
  return u;
#else
  uint64_t u;
  std::memcpy(&u, &x, 8);
  return u;
#endif
}

TL_EMU_FN double from_bits(uint64_t u) {
#if defined(__CUDA_ARCH__)
  double x;
  asm("mov.b64 %0, %1;" : "=d"(x) : "l"(u));
  return x;
#else
  double x;
  std::memcpy(&x, &u, 8);
  return x;
#endif
}

TL_EMU_FN int clz64(uint64_t v) {
#if defined(__CUDA_ARCH__)
  return __clzll((long long)v);
#else
  return v ? __builtin_clzll(v) : 64;
#endif
}

// (hi:lo) >> n and the high word of (hi:lo) << n, 0 <= n < 32 (funnel shifts)
TL_EMU_FN uint32_t funnel_r(uint32_t lo, uint32_t hi, uint32_t n) {
#if defined(__CUDA_ARCH__)
  return __funnelshift_r(lo, hi, n);
#else
  return (uint32_t)((((uint64_t)hi << 32) | lo) >> n);
#endif
}
TL_EMU_FN uint32_t funnel_l(uint32_t lo, uint32_t hi, uint32_t n) {
#if defined(__CUDA_ARCH__)
  return __funnelshift_l(lo, hi, n);
#else
  return (uint32_t)(((((uint64_t)hi << 32) | lo) << n) >> 32);
#endif
}

// round-to-nearest-even increment for a significand m whose discarded bits, left-aligned,
// are `rest` (bit 63 the guard bit, the rest sticky)
TL_EMU_FN uint64_t rne_up(uint64_t m, uint64_t rest) {
  return (uint64_t)(rest > SIGN) | ((uint64_t)(rest == SIGN) & m & 1ull);
}

}  // namespace emu

namespace emu {

constexpr uint64_t INF = 0x7ff0000000000000ull;
constexpr uint64_t QNAN = 0x7fffffffffffffffull;

// true when the predicate holds for some lane of the calling threads' warp (on the host: for
// the one caller)
TL_EMU_FN bool any_lane(bool p) {
#if defined(__CUDA_ARCH__)
  return __any_sync(__activemask(), p);
#else
  return p;
#endif
}

// an operand outside the normal range: a subnormal one is normalised (its exponent may go
// below 1); zero, infinity and NaN become 1.0 and are recorded in `kind` (1 zero, 2 infinity,
// 3 NaN), their result being decided by the IEEE rules rather than by the product
TL_EMU_FN void unpack_any(uint64_t X, int& e, uint64_t& m, int& kind) {
  const uint64_t ax = X & ~SIGN;
  kind = 0;
  if (ax == 0 || ax >= INF) {
    kind = ax == 0 ? 1 : (ax == INF ? 2 : 3);
    e = 1023;
    m = HIDDEN;
  } else if (e == 0) {
    const int sh = clz64(ax) - 11;
    m = ax << sh;
    e = 1 - sh;
  }
}

// a product of normalised significands (hi:lo, in [2^104, 2^106); top = its bit 105) whose
// biased exponent e lies below the normal range: the exact product shifted into the
// subnormal range and rounded once (a rounding carry into bit 52 gives the smallest normal)
TL_EMU_FN uint64_t subnormal_bits(uint64_t hi, uint64_t lo, int top, int e) {
  const int t = 52 + top + 1 - e;  // bits below the result's last place
  if (t >= 107) return 0;          // below half the smallest subnormal
  uint64_t m, rest;
  if (t < 64) {
    m = (hi << (64 - t)) | (lo >> t);
    rest = lo << (64 - t);
  } else if (t == 64) {
    m = hi;
    rest = lo;
  } else {
    const int u = t - 64;
    m = hi >> u;
    rest = (hi << (64 - u)) | (lo >> u) | (uint64_t)((lo << (64 - u)) != 0);
  }
  return m + rne_up(m, rest);
}

}  // namespace emu

// x * y rounded to nearest even; the bits of mul.rn.f64 (the quiet NaN 0x7fff...f for a NaN
// result).  Straight-line for normal operands with a normal result; a warp enters the
// general cases (zero, subnormal, infinite or NaN operands; subnormal results; overflow)
// only when one of its lanes needs them.  No FP64 instruction is issued.
TL_EMU_FN double dmul_int(double x, double y) {
  using namespace emu;
  const uint64_t X = bits(x), Y = bits(y);
  const uint64_t sgn = (X ^ Y) & SIGN;
  int ex = (int)(X >> 52) & 0x7ff, ey = (int)(Y >> 52) & 0x7ff;
  uint64_t mx = (X & FRAC) | HIDDEN, my = (Y & FRAC) | HIDDEN;
  const bool ops_normal = (unsigned)(ex - 1) < 2046u && (unsigned)(ey - 1) < 2046u;
  int kx = 0, ky = 0;
  if (any_lane(!ops_normal)) {
    if (!ops_normal) {
      unpack_any(X, ex, mx, kx);
      unpack_any(Y, ey, my, ky);
    }
  }
  // the exact product of the significands, in [2^104, 2^106), as four 32-bit words w3:w2:w1:w0
  // from the 21- and 32-bit halves of each significand (four 32 x 32 -> 64-bit products)
  const uint32_t a0 = (uint32_t)mx, a1 = (uint32_t)(mx >> 32);
  const uint32_t b0 = (uint32_t)my, b1 = (uint32_t)(my >> 32);
  const uint64_t p00 = (uint64_t)a0 * b0;
  const uint64_t mid = (uint64_t)a1 * b0 + (uint64_t)a0 * b1;  // < 2^54
  const uint64_t t1 = (p00 >> 32) + (mid & 0xffffffffull);
  const uint64_t t2 = (mid >> 32) + (uint64_t)a1 * b1 + (t1 >> 32);
  const uint32_t w0 = (uint32_t)p00, w1 = (uint32_t)t1, w2 = (uint32_t)t2, w3 = (uint32_t)(t2 >> 32);
  const int top = (int)(w3 >> 9);  // bit 105: one more bit below the result
  // the significand m = product >> (52 + top) in mh:ml, and the bits below it, left-aligned, in
  // rh:rl (rh's top bit the guard bit, the rest sticky)
  const uint32_t mh = funnel_r(w2, w3, 20 + top), ml = funnel_r(w1, w2, 20 + top);
  const uint32_t rh = funnel_l(w0, w1, 12 - top), rl = w0 << (12 - top);
  const int e = ex + ey - 1023 + top;  // biased exponent of the result
  // round to nearest, ties to even
  const uint32_t up = (uint32_t)(rh > 0x80000000u) | ((uint32_t)(rh == 0x80000000u) & ((uint32_t)(rl != 0u) | (ml & 1u)));
  // m carries the hidden bit into the exponent field; a carry out of rounding moves the
  // result to the next binade (or to infinity) by the same addition
  uint64_t r = (((uint64_t)((uint32_t)(sgn >> 32) + ((uint32_t)(e - 1) << 20) + mh) << 32) | ml) + up;
  const bool res_normal = (unsigned)(e - 1) < 2046u;
  if (any_lane(!res_normal)) {
    if (!res_normal) {
      const uint64_t hi = ((uint64_t)w3 << 32) | w2, lo = ((uint64_t)w1 << 32) | w0;
      r = e >= 2047 ? (sgn | INF) : (sgn | subnormal_bits(hi, lo, top, e));
    }
  }
  if (kx | ky) {
    const int k = kx > ky ? kx : ky;  // NaN, then infinity, then zero decides
    const bool invalid = k == 3 || (kx == 2 && ky == 1) || (kx == 1 && ky == 2);
    r = invalid ? QNAN : (k == 2 ? (sgn | INF) : sgn);
  }
  return from_bits(r);
}

}  // namespace tl

#undef TL_EMU_FN
