// The BVH handle shared by the build, the query kernels and the C ABI.
#pragma once

#include "common.cuh"

#include <vector>

// A BVH's root box as the reference's closestPair sees it (the element bounds grown by 1.05 about their centre, mapped
// by the transform if any) and the loosening it adds to a distance bound: max(0.001 |root box extent|, 100 eps)
struct RootCut {
  float lo[3], hi[3];
  double fudge;
};

// Opaque to C callers; immutable once built.
struct thea_bvh {
  int32_t is_mesh = 0;
  int32_t width = 4;
  int32_t leaf_size = 4;
  int32_t depth = 0;
  int32_t device = 0;
  uint32_t layouts = 0;
  int32_t query_order = 0;  // traverse large batches in Morton order of the query point
  int64_t n = 0;          // elements
  int64_t num_nodes = 0;  // wide nodes; node 0 is the root
  void * nodes = nullptr;          // WideNode<width>[num_nodes]
  float4 * cp_rec = nullptr;       // mesh closest-point records, CP_REC_F4 per element, leaf order
  float4 * ray_rec = nullptr;      // mesh ray records, RAY_REC_F4 per element, leaf order
  float4 * pt_rec = nullptr;       // point records, 1 per element, leaf order
  float4 * slabs = nullptr;        // single mesh with the closest layout: one oriented slab per node child slot (width
                                   // per node); recomputed when an image is loaded (not part of it)
  int32_t * leaf_to_elem = nullptr;  // leaf-order position -> element index
  unsigned * err = nullptr;          // device word: error bits raised by query kernels
  unsigned * err_host = nullptr;     // pinned host mirror of *err, refreshed at the end of every query call
  float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  int64_t device_bytes = 0;
  // forest of one BVH per segment (one segment for a single mesh / point set)
  int32_t num_segments = 1;
  int64_t * seg_start = nullptr;     // device, num_segments + 1: first sorted position (= first element) of each segment
  int32_t * seg_root = nullptr;      // device, num_segments: root wide node of each segment
  std::vector<int64_t> seg_start_host;
  std::vector<float> seg_lo, seg_hi;  // per-segment element bounds (3 floats each)
  RootCut * seg_roots = nullptr;      // device, num_segments: per-segment root cuts (distance bounds of closest queries)
  // affine transform (BvhN::setTransform): row-major 3x4 [L | t] and its FP32 inverse; `world` is the world-space copy
  // of the element records that closest-point, k-NN and radius queries read (it shares this handle's error word)
  int32_t has_transform = 0;
  float xf[12] = {0}, xf_inv[12] = {0};
  thea_bvh * world = nullptr;
};

namespace thea {

thea_bvh * build_bvh(bool is_mesh, float const * V, int64_t nv, int32_t const * F, int64_t nf,
                     thea_build_config const & cfg, cudaStream_t stream);

// One BVH per segment of elements [seg_start[s], seg_start[s+1]) (host array of M + 1 entries; segments non-empty).
// Mesh faces index the shared vertex array; element records store indices within their segment.
thea_bvh * build_forest(bool is_mesh, float const * V, int64_t nv, int32_t const * F, int64_t n_elems,
                        int64_t const * seg_start_host, int M, thea_build_config const & cfg, cudaStream_t stream);
void destroy_bvh(thea_bvh * b);

// Fills seg_roots from seg_lo / seg_hi (allocates it; synchronizes the stream)
void init_segment_roots(thea_bvh * b, cudaStream_t stream);
// The oriented slabs of a single-mesh BVH with the closest layout, from its nodes and records (after a build, and after
// loading an image); other handles, and node arrays that do not follow the build's layout, get none.
void init_slabs(thea_bvh * b, cudaStream_t stream);

// Throws INVALID_ARGUMENT unless every face index lies in [0, nv): checked on the device before any kernel loads a
// vertex through the faces (one pass over F and one 4-byte read back, which synchronizes `stream`).
void check_face_indices(int32_t const * F, int64_t nf, int64_t nv, char const * what, cudaStream_t stream);

}  // namespace thea
