// The FP32 running sum s <- fl(s + x) over a sequence, rounded to nearest (ties to even) at every step, reproduced bit
// for bit in bulk (host and device; compiles with nvcc and with a plain C++ compiler).
//
// While s stays inside one binade [2^(e-1), 2^e), every value the sum takes is a multiple of u = 2^(e-24), so a step
// adds the nearest integer to x / u units of u; only an exact half (a tie, which goes to the even total) depends on
// the total so far. Steps whose units keep the total at or below 2^24 - 2 units therefore never leave the binade and
// add up as one integer sum, in any order. Terms that are negative or not finite, ties, running sums that are zero,
// subnormal or not finite, and runs that could reach the next binade are taken one fl(s + x) at a time.
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define THEA_RSUM_HD __host__ __device__ __forceinline__
#else
#define THEA_RSUM_HD inline
#endif

namespace thea {

// Largest total, in units of the binade's ulp, that a run added in bulk may reach (2^24 units would be 2^e itself).
constexpr long long RUNNING_SUM_MAX_UNITS = (1LL << 24) - 2;

THEA_RSUM_HD uint32_t running_sum_bits(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  uint32_t u;
  std::memcpy(&u, &x, 4);
  return u;
#endif
}

THEA_RSUM_HD float running_sum_float(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float x;
  std::memcpy(&x, &u, 4);
  return x;
#endif
}

// e with s in [2^(e-1), 2^e) for a positive normal finite s; false for anything else (the step is then exact only
// when taken on its own). All of the arithmetic below is on the float's bits: integers only.
THEA_RSUM_HD bool running_sum_binade(float s, int & e) {
  uint32_t be = running_sum_bits(s) >> 23;  // biased exponent; the sign bit makes it 256 or more
  if (be < 1 || be > 254) return false;
  e = (int)be - 126;
  return true;
}

// The running sum as a count of units 2^(e-24): its 24-bit significand, in [2^23, 2^24).
THEA_RSUM_HD long long running_sum_units_of(float s, int e) {
  (void)e;
  return (long long)((running_sum_bits(s) & 0x7FFFFFu) | 0x800000u);
}

// The float of a count of units 2^(e-24) in [2^23, 2^24) (exact: the count is the significand).
THEA_RSUM_HD float running_sum_from_units(long long t, int e) {
  return running_sum_float(((uint32_t)(e + 126) << 23) | ((uint32_t)t & 0x7FFFFFu));
}

// Units one step adds to a running sum in binade e: x / u rounded to the nearest integer, or false when the step has to
// be taken on its own (x negative, not finite or of 2^30 units or more, or x / u an exact half). x = m 2^(k - 23) with
// m its significand (subnormals: k = -126, no implicit bit), so x / u = m 2^(k - e + 1).
THEA_RSUM_HD bool running_sum_step_units(int e, float x, long long & d) {
  uint32_t b = running_sum_bits(x);
  d = 0;
  if (b == 0x80000000u) return true;  // -0 adds nothing
  if (b >> 31) return false;          // negative
  uint32_t be = b >> 23;
  if (be == 255) return false;        // infinity or NaN
  uint32_t m = b & 0x7FFFFFu;
  int k = -126;
  if (be != 0) {
    m |= 0x800000u;
    k = (int)be - 127;
  }
  if (m == 0) return true;
  int sh = k - e + 1;
  if (sh >= 0) {
    if (sh >= 30) return false;
    uint64_t y = (uint64_t)m << sh;
    if (y >= (1ull << 30)) return false;
    d = (long long)y;
    return true;
  }
  int r = -sh;
  if (r >= 32) return true;  // m 2^-r < 2^24 2^-32: below half a unit
  uint32_t q = m >> r, rem = m & ((1u << r) - 1u), half = 1u << (r - 1);
  if (rem == half) return false;
  d = (long long)q + (rem > half ? 1 : 0);
  return true;
}

}  // namespace thea
