// Sample proximity graph (PointSet3::updateGraph, with or without a dense oversampling).
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

// The same with a dense oversampling (PointSet3::addOversampling + updateGraph, PointSet3.hpp:231-290, 324-391): the
// graph is built over samples + dense samples, then each sample's neighbours are the first max_degree other samples
// reached along shortest paths in it (extractOriginalAdjacencies, PointSet3.cpp:157-176), their separations the path
// lengths. dense_normals are used when normals are. Device pointers; synchronizes the stream. Raises
// THEA_ERR_NOT_SUPPORTED if a shortest-path search needs more than its fixed working set.
void run_sample_graph_oversampled(float const * positions, float const * normals, int64_t n, float const * dense,
                                  float const * dense_normals, int64_t n_dense, int max_degree, uint32_t seed,
                                  thea_bvh const * surface, SampleGraphOut & out, cudaStream_t s);

// updateAverageSeparation (PointSet3.hpp:688-702) on the device: the FP32 sum, in sample order, of each sample's first
// degree[i] separations (rows of max_degree), divided by their count as a float (the sum as it is when there are
// none); one float to `out` (device memory). Asynchronous.
void run_mean_separation(float const * separations, int32_t const * degree, int64_t n, int max_degree, float * out,
                         cudaStream_t s);

// The FP32 running sum fl(... fl(fl(s0 + x[0]) + x[1]) ...) over x[0 .. count), bit for bit the sequential loop's (one
// block, runs of terms added as integer multiples of the sum's ulp: running_sum.cuh). count: device pointer to the
// number of terms, or null for n. One float to `out` (device memory). Asynchronous.
void run_running_sum(float const * x, int64_t const * count, int64_t n, float s0, float * out, cudaStream_t s);

}  // namespace thea
