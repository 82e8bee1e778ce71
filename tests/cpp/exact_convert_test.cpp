// Host check of the tensor-core kernels' exact conversions
// (mps2_gb300/csrc/exact_convert.cuh) against the C library, for
// tests/test_exact_convert.py: every function must return exactly what the
// conversion it replaces returns.  Prints the number of mismatches per
// function; exits non-zero on any.
#include "../../mps2_gb300/csrc/exact_convert.cuh"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>

using namespace gq::xconv;

static bool same(double a, double b) { return std::memcmp(&a, &b, sizeof(a)) == 0; }

int main() {
  std::mt19937_64 g(20261204);
  long bad_round = 0, bad_int = 0, bad_scale = 0, bad_f2d = 0, slow = 0;
  // float -> nearest-even integer -> int64, and truncation of integral floats
  for (long i = 0; i < 4000000; ++i) {
    uint32_t u = (uint32_t)g();
    const int e = 100 + (int)(g() % 90);  // |x| from 2^-27 to 2^62
    u = (u & 0x807fffffu) | ((uint32_t)e << 23);
    float x;
    std::memcpy(&x, &u, 4);
    if (integral_f32_to_i64(round_f32(x)) != std::llrint(x)) ++bad_round;
    const float t = std::trunc(x);
    if (integral_f32_to_i64(t) != (long long)t) ++bad_int;
  }
  for (float x : {0.5f, 1.5f, 2.5f, -0.5f, -1.5f, -2.5f, 8388607.5f, -8388607.5f, 0.0f, -0.0f,
                  4194303.5f, 8388608.0f, -8388609.0f})
    if (integral_f32_to_i64(round_f32(x)) != std::llrint(x)) ++bad_round;
  // int64 times 2^e -> double
  for (long i = 0; i < 4000000; ++i) {
    long long x = (long long)g();
    x >>= (int)(g() % 64);
    if (g() & 1) x = -x;
    if (i % 1000 == 0) x = (long long)(g() % 5) - 2;
    if (i % 777 == 0) x = (long long)0x8000000000000000ull;
    const int e = (int)(g() % 2200) - 1100;
    bool ok;
    const double a = scaled_i64_to_f64(x, e, ok);
    if (!ok) {
      ++slow;
      continue;
    }
    if (!same(a, std::ldexp((double)x, e))) ++bad_scale;
  }
  // float bits -> double (every 97th bit pattern, NaNs skipped)
  for (uint64_t v = 0; v < (1ull << 32); v += 97) {
    const uint32_t u = (uint32_t)v;
    float f;
    std::memcpy(&f, &u, 4);
    if (f != f) continue;
    if (!same(f32_bits_to_f64(u), (double)f)) ++bad_f2d;
  }
  for (uint32_t u : {0x00000001u, 0x007fffffu, 0x80000001u, 0x00400000u, 0x7f800000u,
                     0xff800000u, 0x80000000u, 0x00000000u, 0x7f7fffffu}) {
    float f;
    std::memcpy(&f, &u, 4);
    if (!same(f32_bits_to_f64(u), (double)f)) ++bad_f2d;
  }
  std::printf("round %ld int %ld scale %ld (out of normal range %ld) f2d %ld\n", bad_round,
              bad_int, bad_scale, slow, bad_f2d);
  return (bad_round || bad_int || bad_scale || bad_f2d) ? 1 : 0;
}
