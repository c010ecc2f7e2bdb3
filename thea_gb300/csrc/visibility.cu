// Any-hit ray queries and the Visibility surface feature.
//
// rayIntersects (BvhN.hpp:1266-1269) is rayIntersectionTime >= 0: whether any element has a hit time in [0, max_time].
// The first-hit kernel answers it too, but an occlusion query can stop at the first accepted element: the any-hit
// kernel here is the persistent-lane loop of the first-hit kernel with a fixed bound (max_time, or +inf) and an exit on
// the first hit. Nearest-first child order is kept (hits tend to lie in near boxes).
//
// Visibility::compute (SurfaceFeatures/Local/Visibility.hpp:104-126) casts, from a point on the surface, rays along
// num_rays directions of Random::common().sphere() from origins pushed out by 0.001 * scale along the direction, and
// returns the fraction of rays with no hit. Random::common() is a process-wide generator; here Random(seed) takes its
// place so that the result is reproducible: point i uses directions [i * num_rays, (i + 1) * num_rays) of the stream.
// Random::sphere (Random.cpp:225-250, Knop's method) draws x = 2 u - 1, y = 2 u - 1 until 1e-10 <= x² + y² <= 1, each
// attempt consuming two uniforms, so the accepted directions are the accepted attempts of the pairwise-grouped uniform
// stream in order: attempts are evaluated in parallel and compacted with a scan.
#include "visibility.hpp"

#include "device_util.cuh"
#include "query.hpp"
#include "transform.hpp"
#include "any_hit.cuh"
#include "traverse_ops.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace thea {
namespace {

constexpr int SPHERE_THREADS = 256;

// Visibility rays: ray r starts at point r / num_rays pushed out along direction r (world space, then mapped)
struct VisibilityRays {
  float const * pos;
  float const * dirs;
  int num_rays;
  float off;  // 0.001f * scale
  Inverse inv;
  __device__ __forceinline__ void get(int64_t r, V3 & ro, V3 & rd) const {
    int64_t i = r / num_rays;
    V3 u = load_v3(dirs + 3 * r);
    V3 p = load_v3(pos + 3 * i);
    // Vector3 offset = 0.001f * scale * u; Ray3(position + offset, u)
    ro = p + off * u;
    rd = u;
    if (inv.on) {
      ro = affine_point(inv.m, ro);
      rd = affine_vector(inv.m, rd);
    }
  }
};

struct EscapeCounts {
  unsigned * count;
  int num_rays;
  __device__ __forceinline__ void put(int64_t r, bool hit) const {
    if (!hit) atomicAdd(count + r / num_rays, 1u);
  }
};

// Attempt a of Random::sphere: uniforms 2a and 2a + 1 of the stream
__device__ __forceinline__ bool sphere_attempt(uint32_t const * __restrict__ words, int64_t a, float & x, float & y,
                                               float & m2) {
  float const NORM = 2.3283064365386963e-10f;  // Random::uniform01: (float)bits() * (1.0f / (float)0xFFFFFFFF)
  x = 2.f * (__uint2float_rn(words[2 * a]) * NORM) - 1.f;
  y = 2.f * (__uint2float_rn(words[2 * a + 1]) * NORM) - 1.f;
  m2 = x * x + y * y;
  return !(m2 > 1.f || (double)m2 < 1e-10);  // the reference compares with the double literal 1e-10
}

__global__ void sphere_accept_kernel(uint32_t const * __restrict__ words, int64_t attempts, uint32_t * __restrict__ flag) {
  int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= attempts) return;
  float x, y, m2;
  flag[a] = sphere_attempt(words, a, x, y, m2) ? 1u : 0u;
}

__global__ void sphere_emit_kernel(uint32_t const * __restrict__ words, int64_t attempts,
                                   uint32_t const * __restrict__ slot, int64_t count, float * __restrict__ dirs) {
  int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= attempts) return;
  float x, y, m2;
  if (!sphere_attempt(words, a, x, y, m2)) return;
  int64_t j = slot[a];
  if (j >= count) return;
  float z = 2.f * m2 - 1.f;
  float sc = 2.f * sqrtf(1.f - m2);
  dirs[3 * j] = x * sc;
  dirs[3 * j + 1] = y * sc;
  dirs[3 * j + 2] = z;
}

__global__ void fraction_kernel(unsigned const * __restrict__ escaped, int64_t n, int num_rays,
                                double * __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (double)escaped[i] / (double)num_rays;
}

}  // namespace

void run_ray_intersects(thea_bvh const * b, float const * o, float const * d, int64_t n, float max_time, uint8_t * hit,
                        cudaStream_t s) {
  if (n <= 0) return;
  dispatch_any(b, RayArrays{o, d, inverse_of(b)}, HitFlags{hit}, n, max_time, s);
}

void run_random_sphere(uint32_t seed, int64_t count, float * dirs, cudaStream_t s) {
  if (count <= 0) return;
  // accepted with probability pi/4 per attempt; draw enough attempts for `count` with a wide margin, and more if short
  int64_t attempts = count + count / 3 + 64 + 16 * (int64_t)std::sqrt((double)count);
  THEA_REQUIRE(attempts < ((int64_t)1 << 32), "random_sphere: too many directions for one call");
  while (true) {
    Scratch words((size_t)attempts * 8, s), slot((size_t)attempts * 4, s);
    run_thea_random_words(seed, 2 * attempts, words.as<uint32_t>(), s);
    unsigned grid = (unsigned)ceil_div(attempts, SPHERE_THREADS);
    THEA_LAUNCH(sphere_accept_kernel, grid, SPHERE_THREADS, 0, s, words.as<uint32_t>(), attempts, slot.as<uint32_t>());
    uint32_t last_flag = 0, last_slot = 0;
    THEA_CUDA_CHECK(cudaMemcpyAsync(&last_flag, slot.as<uint32_t>() + attempts - 1, 4, cudaMemcpyDeviceToHost, s));
    exclusive_scan<uint32_t>(slot.as<uint32_t>(), slot.as<uint32_t>(), attempts, s);
    THEA_CUDA_CHECK(cudaMemcpyAsync(&last_slot, slot.as<uint32_t>() + attempts - 1, 4, cudaMemcpyDeviceToHost, s));
    THEA_CUDA_CHECK(cudaStreamSynchronize(s));
    if ((int64_t)last_slot + last_flag >= count) {
      THEA_LAUNCH(sphere_emit_kernel, grid, SPHERE_THREADS, 0, s, words.as<uint32_t>(), attempts, slot.as<uint32_t>(),
                  count, dirs);
      return;
    }
    attempts *= 2;
    THEA_REQUIRE(attempts < ((int64_t)1 << 32), "random_sphere: too many directions for one call");
  }
}

float visibility_scale(thea_bvh const * b) {
  // AxisAlignedBoxN::scaleCentered(1.05): c = 0.5 (hi + lo); lo' = 1.05 (lo - c) + c; hi' likewise
  float const F = 1.05f;
  float lo[3], hi[3];
  for (int a = 0; a < 3; ++a) {
    float c = 0.5f * (b->hi[a] + b->lo[a]);
    lo[a] = F * (b->lo[a] - c) + c;
    hi[a] = F * (b->hi[a] - c) + c;
  }
  if (b->has_transform) {
    // getBounds() of a transformed BVH: the box of the eight mapped corners (AxisAlignedBoxN::transformAndBound)
    float wl[3] = {INFINITY, INFINITY, INFINITY}, wh[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int c = 0; c < 8; ++c) {
      V3 w = affine_point(b->xf, V3{(c & 1) ? hi[0] : lo[0], (c & 2) ? hi[1] : lo[1], (c & 4) ? hi[2] : lo[2]});
      float wc[3] = {w.x, w.y, w.z};
      for (int a = 0; a < 3; ++a) wl[a] = std::min(wl[a], wc[a]), wh[a] = std::max(wh[a], wc[a]);
    }
    for (int a = 0; a < 3; ++a) lo[a] = wl[a], hi[a] = wh[a];
  }
  // getExtent().norm()
  float e[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
  return std::sqrt(e[0] * e[0] + (e[1] * e[1] + e[2] * e[2]));
}

void run_visibility(thea_bvh const * b, float const * positions, int64_t n, int num_rays, uint32_t seed,
                    double * fraction, cudaStream_t s) {
  if (n <= 0) return;
  int64_t total = n * (int64_t)num_rays;
  Scratch dirs((size_t)total * 12, s), escaped((size_t)n * 4, s);
  run_random_sphere(seed, total, dirs.as<float>(), s);
  THEA_CUDA_CHECK(cudaMemsetAsync(escaped.ptr, 0, (size_t)n * 4, s));
  float off = 0.001f * visibility_scale(b);
  dispatch_any(b, VisibilityRays{positions, dirs.as<float>(), num_rays, off, inverse_of(b)},
               EscapeCounts{escaped.as<unsigned>(), num_rays}, total, -1.f, s);
  THEA_LAUNCH(fraction_kernel, (unsigned)ceil_div(n, 256), 256, 0, s, escaped.as<unsigned>(), n, num_rays, fraction);
  THEA_CUDA_CHECK(cudaStreamSynchronize(s));
}

}  // namespace thea
