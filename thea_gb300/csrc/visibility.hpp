// Any-hit ray queries (BvhN::rayIntersects) and the Visibility surface feature built on them.
#pragma once

#include "bvh.hpp"

namespace thea {

// BvhN::rayIntersects (BvhN.hpp:1266-1269): hit[i] = 1 iff ray i has a hit at a time in [0, max_time] (any time when
// max_time < 0), i.e. rayIntersectionTime >= 0. Stops at the first accepted element. Device pointers; the rays are in
// the handle's world space (mapped into object space here when a transform is set).
void run_ray_intersects(thea_bvh const * b, float const * o, float const * d, int64_t n, float max_time, uint8_t * hit,
                        cudaStream_t s);

// `count` directions of Random(seed).sphere() (Random.cpp:225-250), in stream order, as float xyz triples
void run_random_sphere(uint32_t seed, int64_t count, float * dirs, cudaStream_t s);

// Visibility::compute (SurfaceFeatures/Local/Visibility.hpp) for n points with Random(seed) in place of
// Random::common(): point i casts rays along directions [i * num_rays, (i + 1) * num_rays) of the sphere stream.
// Device pointers; synchronizes the stream.
void run_visibility(thea_bvh const * b, float const * positions, int64_t n, int num_rays, uint32_t seed,
                    double * fraction, cudaStream_t s);

// The origin offset scale of Visibility: |extent| of the BVH's root box as the reference pads it (scaleCentered by
// 1.05 about its centre, BvhN.hpp:1437, 2458), in FP32
float visibility_scale(thea_bvh const * b);

}  // namespace thea
