// Batched queries over a forest of BVHs (one per mesh or point set).
#pragma once

#include "bvh.hpp"
#include "query.hpp"

namespace thea {

// Device view of a forest passed by value to the persistent kernels
struct BatchForest {
  void const * nodes;
  float4 const * cp_rec;
  float4 const * ray_rec;
  float4 const * pt_rec;
  float4 const * slabs;  // oriented slabs of the child slots (single-mesh BVHs; nullptr otherwise)
  int64_t const * seg_start;
  int32_t const * seg_root;
  int M;
  unsigned * err;
};

BatchForest forest_view(thea_bvh const * b);

// qoff: device array of M + 1 query offsets (queries of segment m are [qoff[m], qoff[m+1])). chunk: queries a warp
// takes per fetch (a multiple of 32).
void run_batch_closest(thea_bvh const * b, float const * q, int64_t const * qoff, int64_t nq, ClosestParams const & cp,
                       int chunk, int32_t * idx, float * dist, float * cpt, float * err, cudaStream_t s);
// FP32 closest point of one BVH with queries and results in pinned host memory accessed by the kernels in place
// (device-usable pointers); cp.budget > 0 enables the warp-per-query second phase.
void run_closest_stream(thea_bvh const * b, float const * q, int64_t nq, ClosestParams const & cp, int32_t * idx,
                        float * dist, float * cpt, cudaStream_t s);
void run_batch_ray(thea_bvh const * b, float const * o, float const * d, int64_t const * qoff, int64_t nq,
                   float max_time, int chunk, float * t, int32_t * idx, cudaStream_t s);
void run_batch_knn(thea_bvh const * b, float const * q, int64_t const * qoff, int64_t nq, int k, float thresh,
                   int chunk, int32_t * idx, float * d2, cudaStream_t s);

}  // namespace thea
