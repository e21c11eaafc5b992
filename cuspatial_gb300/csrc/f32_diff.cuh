// fl32(x - a) for float64 x and a, rounded once to nearest-even, with 64-bit
// integer arithmetic: on GB300 the float64 pipe (a subtraction and a
// conversion per coordinate) issues at a small fraction of the integer pipe's
// rate.  Plain C++ as well, so that the host tests can check it against exact
// rational arithmetic.
//
// x = mx 2^ex, a = ma 2^ea with 53-bit integer significands.  When both are
// normal and finite and their exponents differ by at most 9, the difference
// D 2^min(ex, ea) is exact in a 64-bit integer (|D| < 2^63); D is then
// rounded to 24 bits and the float's fields are assembled.  Everything else (zeros, subnormal,
// non-finite inputs, exponents further apart, a float result that is not
// normal) returns false, and the caller takes static_cast<float>(x - a).
#pragma once

#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define CSPT_HD __host__ __device__
#else
#define CSPT_HD
#endif

namespace cspt {

CSPT_HD inline int clz64(uint64_t v)
{
#ifdef __CUDA_ARCH__
  return __clzll(static_cast<long long>(v));
#else
  return v ? __builtin_clzll(v) : 64;
#endif
}

CSPT_HD inline uint64_t bits_of(double v)
{
#ifdef __CUDA_ARCH__
  return static_cast<uint64_t>(__double_as_longlong(v));
#else
  uint64_t b;
  std::memcpy(&b, &v, sizeof b);
  return b;
#endif
}

CSPT_HD inline float float_of_bits(uint32_t b)
{
#ifdef __CUDA_ARCH__
  return __uint_as_float(b);
#else
  float f;
  std::memcpy(&f, &b, sizeof f);
  return f;
#endif
}

CSPT_HD inline bool f32_of_difference(double x, double a, float& out)
{
  uint64_t const bx = bits_of(x), ba = bits_of(a);
  int const fx = static_cast<int>((bx >> 52) & 0x7FF), fa = static_cast<int>((ba >> 52) & 0x7FF);
  // both normal and finite
  if (fx == 0 || fa == 0 || fx == 0x7FF || fa == 0x7FF) return false;
  int const lo = fx < fa ? fx : fa;
  int const dx = fx - lo, da = fa - lo;
  if (dx > 9 || da > 9) return false;
  int64_t const mx = static_cast<int64_t>((bx & 0xFFFFFFFFFFFFFull) | (1ull << 52)) << dx;
  int64_t const ma = static_cast<int64_t>((ba & 0xFFFFFFFFFFFFFull) | (1ull << 52)) << da;
  int64_t const sx = (bx >> 63) ? -mx : mx;
  int64_t const sa = (ba >> 63) ? -ma : ma;
  int64_t const d  = sx - sa;  // |d| < 2^63: exact
  if (d == 0) {
    out = 0.0f;  // x - a == +0 in round-to-nearest
    return true;
  }
  uint32_t const sign = d < 0 ? 0x80000000u : 0u;
  uint64_t const m    = d < 0 ? static_cast<uint64_t>(-d) : static_cast<uint64_t>(d);
  int const top       = 63 - clz64(m);  // value = m 2^(lo - 1075), m in [2^top, 2^(top+1))
  int e               = lo - 1075 + top;  // unbiased exponent of the result
  uint64_t q;
  if (top <= 23) {
    q = m << (23 - top);
  } else {
    int const sh       = top - 23;
    q                  = m >> sh;
    uint64_t const rem = m & ((1ull << sh) - 1);
    uint64_t const half = 1ull << (sh - 1);
    if (rem > half || (rem == half && (q & 1u))) ++q;
    if (q == (1ull << 24)) {
      q >>= 1;
      ++e;
    }
  }
  int const biased = e + 127;
  if (biased <= 0 || biased >= 255) return false;  // subnormal or not finite in float
  out = float_of_bits(sign | (static_cast<uint32_t>(biased) << 23) |
                      static_cast<uint32_t>(q & 0x7FFFFFu));
  return true;
}

}  // namespace cspt
