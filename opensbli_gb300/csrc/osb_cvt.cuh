// osb_cvt.cuh -- float <-> double conversions on the integer pipes.
//
// On GB300 the FP64 pipe retires about 2 lanes per clock per SM, and conversions between FP32 and
// FP64 run on it.  The mixed-precision RK update converts every residual to FP64 and every new stage
// value back to FP32, which made those conversions the limiter of the fused central/RK kernel.
// These functions give the same results as the IEEE conversions (float -> double is exact;
// double -> float rounds to nearest, ties to even) using 32-bit integer operations, which run at
// the FP32 rate.  Operands whose result is not a normal number (zero, subnormal, infinity, NaN,
// overflow) take the hardware conversion instead.
//
// Layout facts used: binary32 = sign | 8-bit exponent (bias 127) | 23-bit fraction; binary64 =
// sign | 11-bit exponent (bias 1023) | 52-bit fraction.  A normal float's fraction sits in the top
// 23 of the double's 52 fraction bits (shift by 29) and its exponent is rebiased by 1023-127 = 896.
// Plain C++ on 32-bit halves, so the host compiler can check them bit for bit against its own casts.
#pragma once
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define OSB_HD __host__ __device__ __forceinline__
#else
#define OSB_HD inline
#endif

namespace osb {

OSB_HD uint32_t bits_f32(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  uint32_t b;
  std::memcpy(&b, &x, 4);
  return b;
#endif
}
OSB_HD float f32_bits(uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(b);
#else
  float x;
  std::memcpy(&x, &b, 4);
  return x;
#endif
}
OSB_HD double f64_halves(uint32_t hi, uint32_t lo) {
#if defined(__CUDA_ARCH__)
  return __hiloint2double((int)hi, (int)lo);
#else
  const uint64_t b = ((uint64_t)hi << 32) | lo;
  double x;
  std::memcpy(&x, &b, 8);
  return x;
#endif
}
OSB_HD void halves_f64(double x, uint32_t &hi, uint32_t &lo) {
#if defined(__CUDA_ARCH__)
  hi = (uint32_t)__double2hiint(x);
  lo = (uint32_t)__double2loint(x);
#else
  uint64_t b;
  std::memcpy(&b, &x, 8);
  hi = (uint32_t)(b >> 32);
  lo = (uint32_t)b;
#endif
}

// (double)x, exact
OSB_HD double cvt_f32_f64(float x) {
  const uint32_t b = bits_f32(x);
  const uint32_t m = b & 0x7fffffffu;
  if (m - 0x00800000u >= 0x7f000000u) return (double)x;  // zero, subnormal, inf, NaN
  // exponent+fraction (31 bits) shifted left by 29 across the two halves, exponent rebiased
  const uint32_t hi = (b & 0x80000000u) | ((m >> 3) + 0x38000000u);
  const uint32_t lo = m << 29;
  return f64_halves(hi, lo);
}

// (float)x, round to nearest, ties to even
OSB_HD float cvt_f64_f32(double x) {
  uint32_t hi, lo;
  halves_f64(x, hi, lo);
  const uint32_t e = (hi >> 20) & 0x7ffu;
  // normal float results have double exponents 897..1150; the largest of them may still round up
  // to infinity, which the carry below produces correctly
  if (e - 897u >= 254u) return (float)x;
  const uint32_t mh = (hi & 0x7fffffffu) - 0x38000000u;  // rebiased exponent | top 20 fraction bits
  uint32_t r = (mh << 3) | (lo >> 29);                   // exponent | 23-bit fraction, truncated
  const uint32_t rem = lo & 0x1fffffffu;                 // the 29 discarded bits
  r += (rem > 0x10000000u || (rem == 0x10000000u && (r & 1u))) ? 1u : 0u;
  return f32_bits(r | (hi & 0x80000000u));
}

// FP64 value of a state-precision number: the integer-pipe conversion for FP32, identity for FP64
OSB_HD double to_f64(float x) { return cvt_f32_f64(x); }
OSB_HD double to_f64(double x) { return x; }

}  // namespace osb
