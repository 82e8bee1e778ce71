// Exact conversions between float, double and int64 from integer and FP32
// operations only, for the merges and write-backs of the tensor-core GEMMs
// (gemm_fp64tc.cu, gemm_tf32x3.cu).  The hardware conversion instructions
// between these types issue on the FP64 pipe, which on this part runs about
// two operations per clock per SM: in the merge of a 128 x 96 FP64-accurate
// tile (61k conversions per 256-k chunk) and in the write-back of a short-k
// tile they outlasted the tile's MMAs.  Each function returns exactly what
// the conversion it replaces returns (checked on the host against the C
// library by tests/test_exact_convert.py); compiled for the device and for
// the host.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define GQ_XC __host__ __device__ __forceinline__
#else
#define GQ_XC inline
#endif

namespace gq {
namespace xconv {

GQ_XC uint32_t bits_of(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  uint32_t u;
  std::memcpy(&u, &x, sizeof(u));
  return u;
#endif
}

GQ_XC double double_of(uint64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double d;
  std::memcpy(&d, &b, sizeof(d));
  return d;
#endif
}

GQ_XC int clz32(uint32_t x) {  // x != 0
#ifdef __CUDA_ARCH__
  return __clz((int)x);
#else
  return __builtin_clz(x);
#endif
}

GQ_XC int clz64(uint64_t x) {  // x != 0
#ifdef __CUDA_ARCH__
  return __clzll((long long)x);
#else
  return __builtin_clzll(x);
#endif
}

// x rounded to the nearest integer, ties to even (as a float-to-int64
// conversion in round-to-nearest mode): adding and removing 2^23 with the
// sign of x rounds a float of magnitude below 2^23 (FP32 adds round to
// nearest even); larger floats are integers already.
GQ_XC float round_f32(float x) {
  const float big = 8388608.0f;  // 2^23
  if (!(std::fabs(x) < big)) return x;
  return x >= 0.0f ? (x + big) - big : (x - big) + big;
}

// An integer-valued float (|x| < 2^63) as int64: its significand shifted by
// its exponent.
GQ_XC long long integral_f32_to_i64(float x) {
  const uint32_t u = bits_of(x);
  const int e = (int)((u >> 23) & 0xffu);
  if (e < 127) return 0;  // |x| < 1: zero (x is an integer)
  const uint64_t m = (uint64_t)((u & 0x7fffffu) | 0x800000u);
  const int sh = e - 150;  // x = m 2^sh, sh >= -23
  const uint64_t mag = sh >= 0 ? (m << (sh < 39 ? sh : 39)) : (m >> -sh);
  return (u >> 31) ? -(long long)mag : (long long)mag;
}

// x 2^e as a double, rounded to nearest even: the same value as
// ldexp((double)x, e) whenever that is a normal double; otherwise ok is
// false and the caller takes that expression.
GQ_XC double scaled_i64_to_f64(long long x, int e, bool &ok) {
  ok = true;
  if (x == 0) return 0.0;
  const unsigned long long sign = x < 0 ? 1ull : 0ull;
  const unsigned long long mag = sign ? 0ull - (unsigned long long)x : (unsigned long long)x;
  const int lz = clz64(mag);
  const unsigned long long norm = mag << lz;  // leading one at bit 63
  unsigned long long sig = norm >> 11;        // 53 bits
  const unsigned long long rem = norm & 0x7ffull;
  int biased = 63 - lz + e + 1023;
  if (rem > 0x400ull || (rem == 0x400ull && (sig & 1ull))) {
    sig += 1ull;
    if (sig == (1ull << 53)) {
      sig >>= 1;
      biased += 1;
    }
  }
  if (biased <= 0 || biased >= 2047) {
    ok = false;
    return 0.0;
  }
  return double_of((sign << 63) | ((unsigned long long)biased << 52) |
                   (sig & ((1ull << 52) - 1ull)));
}

// A float (given by its bits) as the double of the same value.
GQ_XC double f32_bits_to_f64(uint32_t u) {
  const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
  const uint32_t e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
  if (e == 0) {
    if (m == 0) return double_of(sign);
    const int sh = clz32(m) - 8;  // leading one of a subnormal to bit 23
    return double_of(sign | ((unsigned long long)(897 - sh) << 52) |
                     ((unsigned long long)((m << sh) & 0x7fffffu) << 29));
  }
  const unsigned long long ex = e == 255u ? 2047ull : (unsigned long long)(e + 896u);
  return double_of(sign | (ex << 52) | ((unsigned long long)m << 29));
}

}  // namespace xconv
}  // namespace gq
