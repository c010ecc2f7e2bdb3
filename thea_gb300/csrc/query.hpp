// Host-side launchers of the query and sampling kernels (device pointers only; staging lives in the C ABI layer).
#pragma once

#include "bvh.hpp"

namespace thea {

struct ClosestParams {
  float thresh = INFINITY;  // FP32 mode: accept squared distances <= thresh
  double bound2 = -1.0;     // FP64 mode: accept FP64 squared distances < bound2 (< 0: unbounded)
  int precision = THEA_PRECISION_FP32_REFERENCE;
  float scene_scale = 0.f;  // largest coordinate magnitude of the BVH's elements
  int budget = 0;           // batched search: stack pops per thread before a query moves to a whole warp (0: never)
};

struct RayParams {
  float max_time = -1.f;
  bool recheck = false;
};

bool small_stack_ok(thea_bvh const * b);

void run_closest(thea_bvh const * b, float const * q, int64_t n, ClosestParams const & cp, int32_t * idx, float * dist,
                 float * cpt, float * errout, unsigned * err, cudaStream_t s);
// FP32 first hit with rays and results in pinned host memory accessed by the kernel (device-usable pointers).
void run_ray_stream(thea_bvh const * b, float const * o, float const * d, int64_t n, float max_time, float * t,
                    int32_t * idx, unsigned * err, cudaStream_t s);
void run_ray(thea_bvh const * b, float const * o, float const * d, int64_t n, RayParams const & rp, float * t,
             int32_t * idx, float * nrm, float * t64, int32_t * idx64, int32_t * flags, unsigned * err, cudaStream_t s);
// q == nullptr: self mode over the BVH's own points (n = number of points, rows in element order)
// Points of a point BVH within `radius` of each query, as CSR. idx == nullptr: counting pass, writes offsets[0..n]
// (n + 1 entries, device). Otherwise: filling pass with the offsets of the counting pass; each query's slice holds its
// neighbours in ascending element index, with squared distances in d2 (nullable). Synchronizes in the filling pass.
void run_range(thea_bvh const * b, float const * q, int64_t n, float radius, int32_t const * ex, int64_t * offsets,
               int32_t * idx, float * d2, unsigned * err, cudaStream_t s);
// init_bound (self mode only): per leaf position, an inclusive upper bound on the k-th neighbour's squared distance
void run_knn(thea_bvh const * b, float const * q, int64_t n, int k, float thresh, int32_t const * ex, int32_t * idx,
             float * d2, unsigned * err, cudaStream_t s, float const * init_bound = nullptr);

// `count` tempered words of Random(seed) (Random::Random(seed), then bits() repeatedly), in stream order
void run_thea_random_words(uint32_t seed, int64_t count, uint32_t * out, cudaStream_t s);

// Returns the number of samples written (0 when the total area is not positive); synchronizes the stream.
int64_t run_sample_by_area(float const * V, int64_t nv, int32_t const * F, int64_t nf, int64_t n, uint32_t seed, int rng,
                           float * pos, float * nrm, int32_t * face, cudaStream_t s);

// The same computation with all scratch in a fixed device array (no allocation); device pointers only.
int64_t run_sample_by_area_noalloc(float const * V, int64_t nv, int32_t const * F, int64_t nf, int64_t n,
                                   uint32_t seed, int rng, float * pos, float * nrm, int32_t * face, cudaStream_t s);

// Largest coordinate magnitude of a handle's element bounds
inline float scene_scale_of(thea_bvh const * b) {
  float s = 0.f;
  for (int a = 0; a < 3; ++a) s = fmaxf(s, fmaxf(fabsf(b->lo[a]), fabsf(b->hi[a])));
  return s;
}

}  // namespace thea
