// Checks the bulk FP32 running sum of thea_gb300/csrc/running_sum.cuh against the plain sequential loop, bit for bit:
// the kernel's windowed algorithm (groups of consecutive terms added as integer multiples of the sum's ulp, the first
// group that cannot be taken one term at a time) is restated here with the group size and group count as parameters,
// on random sequences of many magnitudes, sequences built to hit ties (x / ulp an exact half), binade crossings,
// zeros, subnormals, negative terms and non-finite terms.
#include "../../thea_gb300/csrc/running_sum.cuh"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <random>
#include <vector>

namespace {

volatile float g_sink;

float add_rn(float a, float b) {
  volatile float r = a + b;  // one IEEE single addition, kept out of any wider evaluation
  return r;
}

float naive(std::vector<float> const & x, float s) {
  for (float v : x) s = add_rn(s, v);
  return s;
}

float bulk(std::vector<float> const & x, float s, int threads, int items) {
  int64_t n = (int64_t)x.size(), cur = 0;
  std::vector<long long> units((size_t)threads);
  std::vector<char> ok((size_t)threads);
  while (cur < n) {
    int e = 0;
    bool b = thea::running_sum_binade(s, e);
    for (int t = 0; t < threads; ++t) {
      units[(size_t)t] = 0;
      ok[(size_t)t] = b;
      int64_t g0 = cur + (int64_t)t * items;
      for (int64_t j = g0; b && j < g0 + items && j < n; ++j) {
        long long d = 0;
        if (!thea::running_sum_step_units(e, x[(size_t)j], d)) ok[(size_t)t] = 0;
        units[(size_t)t] += d;
      }
    }
    long long base = b ? thea::running_sum_units_of(s, e) : 0, before = 0;
    int g = threads;
    for (int t = 0; t < threads; ++t) {
      int64_t g0 = cur + (int64_t)t * items;
      if (g0 >= n) break;
      if (!ok[(size_t)t] || base + before + units[(size_t)t] > thea::RUNNING_SUM_MAX_UNITS) {
        g = t;
        break;
      }
      before += units[(size_t)t];
    }
    if (g < threads) {
      if (b && before > 0) s = thea::running_sum_from_units(base + before, e);
      int64_t g0 = cur + (int64_t)g * items, end = std::min<int64_t>(g0 + items, n);
      for (int64_t j = g0; j < end; ++j) s = add_rn(s, x[(size_t)j]);
      cur = end;
    } else {
      if (b) s = thea::running_sum_from_units(base + before, e);
      cur += (int64_t)threads * items;
    }
  }
  return s;
}

bool same(float a, float b) {
  if (std::isnan(a) || std::isnan(b)) return std::isnan(a) && std::isnan(b);
  uint32_t x, y;
  std::memcpy(&x, &a, 4);
  std::memcpy(&y, &b, 4);
  return x == y;
}

int failures = 0, cases = 0;

void check(std::vector<float> const & x, float s0, char const * what) {
  float want = naive(x, s0);
  int const shapes[][2] = {{1, 1}, {4, 1}, {32, 4}, {512, 16}, {7, 3}};
  for (auto const & sh : shapes) {
    float got = bulk(x, s0, sh[0], sh[1]);
    ++cases;
    if (!same(got, want)) {
      if (++failures <= 10)
        std::printf("MISMATCH %s n=%zu threads=%d items=%d: %.9g vs %.9g\n", what, x.size(), sh[0], sh[1], got, want);
    }
  }
}

}  // namespace

int main() {
  std::mt19937_64 rng(12345);
  std::uniform_real_distribution<float> u01(0.f, 1.f);
  std::normal_distribution<double> nrm(0.0, 1.0);
  // separations-like: small positive values, long sums crossing many binades
  for (int trial = 0; trial < 40; ++trial) {
    size_t n = 1 + (size_t)(rng() % 200000);
    std::vector<float> x(n);
    float scale = std::ldexp(1.f, (int)(rng() % 40) - 20);
    for (auto & v : x) v = u01(rng) * scale;
    check(x, 0.f, "uniform");
  }
  // magnitudes spread over many binades (log-normal), some exact zeros, some subnormals
  for (int trial = 0; trial < 40; ++trial) {
    size_t n = 1 + (size_t)(rng() % 50000);
    std::vector<float> x(n);
    for (auto & v : x) {
      int k = (int)(rng() % 20);
      if (k == 0) v = 0.f;
      else if (k == 1) v = std::numeric_limits<float>::denorm_min() * (float)(1 + rng() % 1000);
      else v = (float)std::exp(nrm(rng) * 6.0);
    }
    check(x, 0.f, "lognormal");
  }
  // ties: terms that are odd multiples of half the running sum's ulp, in a sum that stays near a chosen binade
  for (int trial = 0; trial < 200; ++trial) {
    int e = (int)(rng() % 60) - 30;
    float s0 = std::ldexp(1.f, e) * (1.f + u01(rng));  // in [2^e, 2^(e+1))
    float ulp = std::ldexp(1.f, e - 23);
    size_t n = 1 + (size_t)(rng() % 5000);
    std::vector<float> x(n);
    for (auto & v : x) {
      int k = (int)(rng() % 4);
      if (k == 0) v = ulp * (0.5f + (float)(rng() % 8));        // x / u an exact half
      else if (k == 1) v = ulp * 0.5f;                          // the smallest tie
      else if (k == 2) v = ulp * (float)(rng() % 16) * 0.25f;   // quarters
      else v = u01(rng) * ulp * 64.f;
    }
    check(x, s0, "ties");
  }
  // binade crossings: sums that start just below a power of two, big jumps, and sums near FLT_MAX
  for (int trial = 0; trial < 200; ++trial) {
    int e = (int)(rng() % 200) - 100;
    float p = std::ldexp(1.f, e);
    float s0 = std::nextafter(p, 0.f);
    for (int k = 0; k < (int)(rng() % 8); ++k) s0 = std::nextafter(s0, 0.f);
    size_t n = 1 + (size_t)(rng() % 3000);
    std::vector<float> x(n);
    for (auto & v : x) {
      int k = (int)(rng() % 5);
      v = k == 0 ? std::ldexp(1.f, e - 24) : k == 1 ? std::ldexp(u01(rng), e - 20) : k == 2 ? p * u01(rng) * 0.01f
          : k == 3 ? std::ldexp(1.f, e - 25) * 3.f : 0.f;
    }
    check(x, s0, "crossing");
  }
  {
    std::vector<float> x(1000, 1e37f);
    check(x, 3e38f, "overflow");
  }
  // negative and non-finite terms take the one-at-a-time path
  for (int trial = 0; trial < 40; ++trial) {
    size_t n = 1 + (size_t)(rng() % 20000);
    std::vector<float> x(n);
    for (auto & v : x) v = u01(rng);
    for (int k = 0; k < 5; ++k) x[(size_t)(rng() % n)] = -u01(rng);
    check(x, 0.f, "negative");
    if (trial % 4 == 0) {
      x[(size_t)(rng() % n)] = trial % 8 == 0 ? std::numeric_limits<float>::infinity()
                                              : std::numeric_limits<float>::quiet_NaN();
      check(x, 0.f, "nonfinite");
    }
  }
  check(std::vector<float>(), 2.5f, "empty");
  g_sink = 0.f;
  if (failures) {
    std::printf("%d of %d cases differ\n", failures, cases);
    return 1;
  }
  std::printf("running sum matches the sequential loop in %d cases\n", cases);
  return 0;
}
