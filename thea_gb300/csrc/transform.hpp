// Affine transforms of a built BVH (BvhN::setTransform / clearTransform / getTransformInv, BvhN.hpp:903-929).
#pragma once

#include "bvh.hpp"

namespace thea {

// Row-major 3x4 affine map [L | t]: p -> L p + t, evaluated like AffineTransformN::operator* (AffineTransformN.hpp:160,
// `linear * v + trans`): each coordinate is the 3-term product sum in Eigen's order e0 + (e1 + e2), then + t.
__host__ __device__ __forceinline__ V3 affine_point(float const * m, V3 v) {
  return V3{(m[0] * v.x + (m[1] * v.y + m[2] * v.z)) + m[3], (m[4] * v.x + (m[5] * v.y + m[6] * v.z)) + m[7],
            (m[8] * v.x + (m[9] * v.y + m[10] * v.z)) + m[11]};
}
// The linear part alone (ray directions: `getLinear() * dir`, BvhN.hpp:2175-2178)
__host__ __device__ __forceinline__ V3 affine_vector(float const * m, V3 v) {
  return V3{m[0] * v.x + (m[1] * v.y + m[2] * v.z), m[4] * v.x + (m[5] * v.y + m[6] * v.z),
            m[8] * v.x + (m[9] * v.y + m[10] * v.z)};
}
// normalToWorldSpace (BvhN.hpp:2181-2184): (inverse(L)^T n).normalized(), with inv the inverse's 3x4 matrix
__host__ __device__ __forceinline__ V3 normal_to_world(float const * inv, V3 n) {
  V3 w{inv[0] * n.x + (inv[4] * n.y + inv[8] * n.z), inv[1] * n.x + (inv[5] * n.y + inv[9] * n.z),
       inv[2] * n.x + (inv[6] * n.y + inv[10] * n.z)};
  return normalized(w);
}

// AffineTransformN::inverse (AffineTransformN.hpp:133-137) in FP32: L^-1 by cofactors, then t' = L^-1 (-t).
// Returns false (and leaves inv unspecified) when the determinant is zero or not finite.
bool affine_inverse(float const * m, float * inv);

// Validates the map, stores it with its inverse and builds the world-space copy of the element records that closest-point,
// k-NN and radius queries then run against. Rays keep the object-space structure and are moved into object space per
// query. Single BVHs only (not forests). Synchronizes the stream. Must not run concurrently with queries on the handle.
void set_transform(thea_bvh * b, float const * m, cudaStream_t s);
void clear_transform(thea_bvh * b);

// Per-query parts of the ray path: origins and directions into object space, hit normals back to world space
void rays_to_object(thea_bvh const * b, float const * o, float const * d, int64_t n, float * o_obj, float * d_obj,
                    cudaStream_t s);
void normals_to_world(thea_bvh const * b, float * normals, int64_t n, cudaStream_t s);

// The handle that closest-point, k-NN and radius queries read: the world-space copy when a transform is set
inline thea_bvh const * query_target(thea_bvh const * b) { return b && b->world ? b->world : b; }

}  // namespace thea
