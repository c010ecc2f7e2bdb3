// Sample proximity graph (PointSet3::updateGraph without oversampling).
#pragma once

#include "bvh.hpp"

namespace thea {

struct SampleGraphOut {
  int32_t * neighbors;     // n x max_degree, ascending (separation, index), -1 past the degree
  float * separations;     // n x max_degree (nullable), 0 past the degree
  int32_t * degree;        // n (nullable)
  float avg_separation_estimate = 0.f;  // RMS nearest-neighbour distance of the sampled trials
};

// Device pointers. normals: nullable; surface: nullable mesh BVH (ray layout) for the reachability test, used only with
// normals, as in the reference. Synchronizes the stream.
void run_sample_graph(float const * positions, float const * normals, int64_t n, int max_degree, uint32_t seed,
                      thea_bvh const * surface, SampleGraphOut & out, cudaStream_t s);

}  // namespace thea
