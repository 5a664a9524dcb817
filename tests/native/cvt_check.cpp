// Checks osb_cvt.cuh's integer-pipe conversions bit for bit against the host compiler's IEEE casts:
// every float bit pattern for float -> double, and random plus constructed doubles (rounding ties,
// binade edges, overflow and underflow boundaries) for double -> float.  Prints the mismatch count.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <initializer_list>

#include "osb_cvt.cuh"

static uint64_t bits64(double x) {
  uint64_t b;
  std::memcpy(&b, &x, 8);
  return b;
}
static double dbl(uint64_t b) {
  double x;
  std::memcpy(&x, &b, 8);
  return x;
}
static uint32_t bits32(float x) {
  uint32_t b;
  std::memcpy(&b, &x, 4);
  return b;
}

int main() {
  uint64_t bad = 0, n = 0;
  // float -> double: all 2^32 patterns (NaNs compared as NaN)
  for (uint64_t i = 0; i <= 0xffffffffull; ++i) {
    const float x = osb::f32_bits((uint32_t)i);
    const double a = osb::cvt_f32_f64(x), b = (double)x;
    ++n;
    if (std::isnan(b) ? !std::isnan(a) : bits64(a) != bits64(b)) ++bad;
  }
  // double -> float: xorshift random patterns, then constructed cases around every float exponent
  uint64_t s = 0x9e3779b97f4a7c15ull;
  auto next = [&]() {
    s ^= s << 13;
    s ^= s >> 7;
    s ^= s << 17;
    return s;
  };
  auto check = [&](double x) {
    const float a = osb::cvt_f64_f32(x), b = (float)x;
    ++n;
    if (std::isnan(b) ? !std::isnan(a) : bits32(a) != bits32(b)) ++bad;
  };
  for (int i = 0; i < 200000000; ++i) check(dbl(next()));
  for (uint32_t e = 850; e <= 1200; ++e)
    for (uint64_t f : {0ull, 1ull, 0x10000000ull, 0x0fffffffull, 0x10000001ull, 0x30000000ull, 0x20000000ull,
                       0x000fffffffffffffull, 0x000fffffe0000000ull, 0x000fffffefffffffull, 0x000ffffff0000000ull,
                       0x000ffffff0000001ull})
      for (uint64_t sg : {0ull, 1ull})
        for (int k = 0; k < 64; ++k) {
          const uint64_t frac = (f + (uint64_t)k * 0x20000000ull) & 0x000fffffffffffffull;
          check(dbl((sg << 63) | ((uint64_t)e << 52) | frac));
        }
  std::printf("%llu %llu\n", (unsigned long long)bad, (unsigned long long)n);
  return bad != 0;
}
