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
  struct BoundCut const * seg_cut = nullptr;  // forests: per-mesh thresholds (device array), replacing thresh/bound2
};

// How the reference applies a distance bound to a closest-element query (BvhN::closestPair, BvhN.hpp:1093-1107). With
// dist_bound >= 0: a query whose point is farther from the root box than dist_bound (FP32 box-box squared distance,
// AxisAlignedBoxN::squaredDistance, compared in double with dist_bound^2) gets no element; otherwise the bound is
// loosened (accelerationBound returns it unchanged and closestPair adds max(0.001 |root box extent|, 100 eps)) and the
// search accepts squared distances below the loosened bound squared. The root box is the element bounds grown by 1.05
// about their centre (AxisAlignedBoxN::scaleCentered), mapped through the affine transform if one is set
// (AxisAlignedBoxN::transformAndBound).
struct BoundCut {
  float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};  // root box, world space
  double b2 = -1.0;                            // dist_bound^2 (< 0: no bound, nothing is cut)
  float thresh = INFINITY;                     // FP32 search: accept squared distances <= thresh
  double bound2 = -1.0;                        // FP64 search: accept squared distances < bound2
};

// The part that does not depend on the bound (RootCut, bvh.hpp). elem_lo / elem_hi: the BVH's element bounds (object
// space); xf: row-major 3x4 affine map or nullptr.
RootCut root_cut_of(float const * elem_lo, float const * elem_hi, float const * xf);

__host__ __device__ inline BoundCut make_bound_cut(RootCut const & r, float dist_bound) {
  BoundCut c;
  if (!(dist_bound >= 0.f)) return c;
  for (int a = 0; a < 3; ++a) c.lo[a] = r.lo[a], c.hi[a] = r.hi[a];
  double b = (double)dist_bound + r.fudge;
  c.b2 = (double)dist_bound * (double)dist_bound;
  c.bound2 = b * b;
  // the largest float whose double is below the loosened bound squared
#ifdef __CUDA_ARCH__
  float f = __double2float_rd(c.bound2);
  if ((double)f >= c.bound2) f = nextafterf(f, -INFINITY);
#else
  float f = (float)c.bound2;
  if ((double)f >= c.bound2) f = std::nextafter(f, -INFINITY);
#endif
  c.thresh = f;
  return c;
}

inline BoundCut closest_bound_cut(thea_bvh const * b, float dist_bound) {
  return make_bound_cut(root_cut_of(b->lo, b->hi, b->has_transform ? b->xf : nullptr), dist_bound);
}

// Per-segment cuts of a forest for one bound (device array of num_segments), from the handle's per-segment root cuts
void run_segment_cuts(thea_bvh const * b, float dist_bound, BoundCut * out, cudaStream_t s);

// True when a query at p has no element under the cut's bound (its point is farther than the bound from the root box)
__host__ __device__ __forceinline__ bool bound_cut_out(BoundCut const & c, V3 p) {
  if (c.b2 < 0.0) return false;
  // AxisAlignedBoxN::squaredDistance(box) with the query's point box as "this"
  float dx = fmaxf(fmaxf(p.x, c.lo[0]) - fminf(p.x, c.hi[0]), 0.f);
  float dy = fmaxf(fmaxf(p.y, c.lo[1]) - fminf(p.y, c.hi[1]), 0.f);
  float dz = fmaxf(fmaxf(p.z, c.lo[2]) - fminf(p.z, c.hi[2]), 0.f);
  float lb = dx * dx + (dy * dy + dz * dz);
  return (double)lb > c.b2;
}

// Writes "no element" (index -1, distance -1, closest point 0, error -1) for the queries that a cut removes: `one` for
// every query, or with cuts != nullptr one cut per mesh (device array of M) and queries grouped by mesh through qoff
// (M + 1 entries, device). Device or device-usable host pointers; outputs other than idx nullable.
void run_closest_cut(float const * q, int64_t n, BoundCut const & one, int64_t const * qoff, int M,
                     BoundCut const * cuts, int32_t * idx, float * dist, float * cpt, float * errout, cudaStream_t s);

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
// sorted = false: the filling pass writes each slice in traversal order instead, without the sort and without
// synchronizing (for callers whose use of a slice does not depend on its order).
void run_range(thea_bvh const * b, float const * q, int64_t n, float radius, int32_t const * ex, int64_t * offsets,
               int32_t * idx, float * d2, unsigned * err, cudaStream_t s, bool sorted = true);
// The counting pass that also writes each query's first row_cap neighbours (traversal order) into row q of `rows`
// (n x row_cap) and sets *overflow (device) if a query has more; offsets as the counting pass writes them.
void run_range_rows(thea_bvh const * b, float const * q, int64_t n, float radius, int32_t const * ex,
                    int64_t * offsets, int32_t * rows, int row_cap, unsigned * overflow, unsigned * err, cudaStream_t s);
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
