// Host-side launchers of the query and sampling kernels (device pointers only; staging lives in the C ABI layer).
#pragma once

#include "bvh.hpp"

namespace thea {

// thresh: accept squared distances <= thresh (+inf when unbounded)
void run_closest(thea_bvh const * b, float const * q, int64_t n, float thresh, int32_t * idx, float * dist, float * cp,
                 unsigned * err, cudaStream_t s);
void run_ray(thea_bvh const * b, float const * o, float const * d, int64_t n, float max_time, float * t, int32_t * idx,
             float * nrm, unsigned * err, cudaStream_t s);
// q == nullptr: self mode over the BVH's own points (n = number of points, rows in element order)
void run_knn(thea_bvh const * b, float const * q, int64_t n, int k, float thresh, int32_t const * ex, int32_t * idx,
             float * d2, unsigned * err, cudaStream_t s);

// Returns the number of samples written (0 when the total area is not positive); synchronizes the stream.
int64_t run_sample_by_area(float const * V, int64_t nv, int32_t const * F, int64_t nf, int64_t n, uint32_t seed, int rng,
                           float * pos, float * nrm, int32_t * face, cudaStream_t s);

// The same computation with all scratch in a fixed device array (no allocation); device pointers only.
int64_t run_sample_by_area_noalloc(float const * V, int64_t nv, int32_t const * F, int64_t nf, int64_t n,
                                   uint32_t seed, int rng, float * pos, float * nrm, int32_t * face, cudaStream_t s);

}  // namespace thea
