// Affine transforms of a built BVH. The reference (BvhN.hpp:903-921, 2027-2062, 2175-2184) keeps its tree in object
// space and, per query, moves rays into object space (toObjectSpace) but evaluates proximity against each element
// transformed into world space (makeTransformedObject -> Transformer::transform -> TriangleN::transform, whose cached
// plane, normal and edges are recomputed from the transformed vertices). Both are kept here:
//  * rays: origins and directions are moved into object space with the FP32 inverse, the object-space structure is
//    traversed unchanged, and normals of hits go back through the inverse transpose;
//  * closest point, k-NN, radius: a world-space copy of the element records (vertices transformed once, records and
//    tree rebuilt from them on the device) answers them; results depend only on the transformed elements, not on a tree.
#include "transform.hpp"

#include "common.cuh"
#include "device_util.cuh"

#include <cmath>
#include <cstring>

namespace thea {
namespace {

struct Affine {
  float m[12];
};

constexpr int XF_THREADS = 256;

// World-space vertices of every triangle, in original face order (face e -> vertices 3e, 3e + 1, 3e + 2), read from
// the closest-point records (vertices stored exactly, leaf order, original index in record 5's w)
__global__ void world_triangles_kernel(float4 const * __restrict__ cp_rec, int64_t n, Affine a, float * __restrict__ V,
                                       int32_t * __restrict__ F) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  float4 const * r = cp_rec + s * CP_REC_F4;
  int64_t e = __float_as_int(__ldg(r + 5).w);
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    V3 w = affine_point(a.m, xyz(__ldg(r + j)));
    V[9 * e + 3 * j] = w.x;
    V[9 * e + 3 * j + 1] = w.y;
    V[9 * e + 3 * j + 2] = w.z;
    F[3 * e + j] = (int32_t)(3 * e + j);
  }
}

__global__ void world_points_kernel(float4 const * __restrict__ pt_rec, int64_t n, Affine a, float * __restrict__ P) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  float4 r = __ldg(pt_rec + s);
  int64_t e = __float_as_int(r.w);
  V3 w = affine_point(a.m, xyz(r));
  P[3 * e] = w.x;
  P[3 * e + 1] = w.y;
  P[3 * e + 2] = w.z;
}

__global__ void rays_to_object_kernel(float const * __restrict__ o, float const * __restrict__ d, int64_t n, Affine inv,
                                      float * __restrict__ o2, float * __restrict__ d2) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  V3 a = affine_point(inv.m, load_v3(o + 3 * i));
  V3 b = affine_vector(inv.m, load_v3(d + 3 * i));
  o2[3 * i] = a.x;
  o2[3 * i + 1] = a.y;
  o2[3 * i + 2] = a.z;
  d2[3 * i] = b.x;
  d2[3 * i + 1] = b.y;
  d2[3 * i + 2] = b.z;
}

// Misses carry a zero normal and keep it (the reference transforms the normal of valid hits only)
__global__ void normals_to_world_kernel(float * __restrict__ nrm, int64_t n, Affine inv) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  V3 v = load_v3(nrm + 3 * i);
  if (v.x == 0.f && v.y == 0.f && v.z == 0.f) return;
  V3 w = normal_to_world(inv.m, v);
  nrm[3 * i] = w.x;
  nrm[3 * i + 1] = w.y;
  nrm[3 * i + 2] = w.z;
}

Affine affine_of(float const * m) {
  Affine a;
  std::memcpy(a.m, m, sizeof(a.m));
  return a;
}

}  // namespace

bool affine_inverse(float const * m, float * inv) {
  // cofactor (i, j) of L: L(i1, j1) L(i2, j2) - L(i1, j2) L(i2, j1) with i1 = i + 1, i2 = i + 2, j1, j2 likewise mod 3
  auto L = [&](int i, int j) { return m[4 * (i % 3) + (j % 3)]; };
  auto cof = [&](int i, int j) { return L(i + 1, j + 1) * L(i + 2, j + 2) - L(i + 1, j + 2) * L(i + 2, j + 1); };
  float c00 = cof(0, 0), c10 = cof(1, 0), c20 = cof(2, 0);
  // determinant: the cofactors of column 0 dotted with column 0 (3-term sum in the order e0 + (e1 + e2))
  float det = c00 * m[0] + (c10 * m[4] + c20 * m[8]);
  if (!(det != 0.f) || !std::isfinite(det)) return false;
  float invdet = 1.0f / det;
  // inverse(j, i) = cofactor(i, j) / det, as cofactor times the reciprocal
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) inv[4 * j + i] = cof(i, j) * invdet;
  // translation: inverse(L) * (-t)
  float nt[3] = {-m[3], -m[7], -m[11]};
  for (int r = 0; r < 3; ++r) inv[4 * r + 3] = inv[4 * r] * nt[0] + (inv[4 * r + 1] * nt[1] + inv[4 * r + 2] * nt[2]);
  for (int k = 0; k < 12; ++k)
    if (!std::isfinite(inv[k])) return false;
  return true;
}

void set_transform(thea_bvh * b, float const * m, cudaStream_t s) {
  THEA_REQUIRE(b && m, "bvh_set_transform: null argument");
  THEA_REQUIRE(b->num_segments == 1, "bvh_set_transform: forests take no transform");
  for (int k = 0; k < 12; ++k) THEA_REQUIRE(std::isfinite(m[k]), "bvh_set_transform: non-finite matrix entry");
  float inv[12];
  THEA_REQUIRE(affine_inverse(m, inv), "bvh_set_transform: the linear part is singular");
  int prev = -1;
  THEA_CUDA_CHECK(cudaGetDevice(&prev));
  THEA_CUDA_CHECK(cudaSetDevice(b->device));
  thea_bvh * world = nullptr;
  try {
    thea_build_config cfg{};
    cfg.width = b->width;
    cfg.max_leaf_size = b->leaf_size;
    cfg.query_order = b->query_order;
    int64_t n = b->n;
    unsigned grid = (unsigned)ceil_div(n, XF_THREADS);
    if (b->is_mesh && b->cp_rec) {
      cfg.layouts = THEA_LAYOUT_CLOSEST;
      Scratch V((size_t)n * 36, s), F((size_t)n * 12, s);
      THEA_LAUNCH(world_triangles_kernel, grid, XF_THREADS, 0, s, b->cp_rec, n, affine_of(m), V.as<float>(),
                  F.as<int32_t>());
      world = build_bvh(true, V.as<float>(), 3 * n, F.as<int32_t>(), n, cfg, s);
    } else if (!b->is_mesh) {
      Scratch P((size_t)n * 12, s);
      THEA_LAUNCH(world_points_kernel, grid, XF_THREADS, 0, s, b->pt_rec, n, affine_of(m), P.as<float>());
      world = build_bvh(false, P.as<float>(), n, nullptr, 0, cfg, s);
    }
    if (world) {
      // the copy reports errors through its parent's word
      THEA_CUDA_CHECK(cudaStreamSynchronize(s));
      THEA_CUDA_CHECK(cudaFree(world->err));
      world->err = b->err;
    }
  } catch (...) {
    if (world) destroy_bvh(world);
    cudaSetDevice(prev);
    throw;
  }
  clear_transform(b);
  b->world = world;
  b->has_transform = 1;
  std::memcpy(b->xf, m, sizeof(b->xf));
  std::memcpy(b->xf_inv, inv, sizeof(b->xf_inv));
  THEA_CUDA_CHECK(cudaSetDevice(prev));
}

void clear_transform(thea_bvh * b) {
  if (b->world) {
    b->world->err = nullptr;  // owned by b
    destroy_bvh(b->world);
    b->world = nullptr;
  }
  b->has_transform = 0;
}

void rays_to_object(thea_bvh const * b, float const * o, float const * d, int64_t n, float * o_obj, float * d_obj,
                    cudaStream_t s) {
  if (n <= 0) return;
  THEA_LAUNCH(rays_to_object_kernel, (unsigned)ceil_div(n, XF_THREADS), XF_THREADS, 0, s, o, d, n,
              affine_of(b->xf_inv), o_obj, d_obj);
}

void normals_to_world(thea_bvh const * b, float * normals, int64_t n, cudaStream_t s) {
  if (n <= 0 || !normals) return;
  THEA_LAUNCH(normals_to_world_kernel, (unsigned)ceil_div(n, XF_THREADS), XF_THREADS, 0, s, normals, n,
              affine_of(b->xf_inv));
}

}  // namespace thea
