// Closest pairs between the elements of two BVHs (BvhN::closestPair / kClosestPairs with a BVH as the query).
#pragma once

#include "bvh.hpp"

namespace thea {

struct PairResult {
  int32_t query_index = -1, target_index = -1;
  float d2 = -1.f;                   // squared distance (the reference's monotone approximate L2 distance)
  float query_point[3] = {0, 0, 0};  // closest points on the two elements (world space)
  float target_point[3] = {0, 0, 0};
};

// The pair of (query element, target element) at the smallest squared distance d2 <= thresh, lowest query index and
// then lowest target index among equal distances. At least one of the two BVHs holds points (mesh-mesh pairs:
// THEA_ERR_NOT_SUPPORTED). Returns false when no pair qualifies. Synchronizes the stream.
bool run_closest_pair(thea_bvh const * target, thea_bvh const * query, float thresh, PairResult & out, cudaStream_t s);

// The k pairs of two point BVHs with the smallest (d2, query index, target index), d2 <= thresh, in that order, into
// device arrays of k entries (-1 past the count). Returns the count. Synchronizes the stream.
int64_t run_k_closest_pairs(thea_bvh const * target, thea_bvh const * query, int k, float thresh, int32_t * qi,
                            int32_t * ti, float * d2, cudaStream_t s);

}  // namespace thea
