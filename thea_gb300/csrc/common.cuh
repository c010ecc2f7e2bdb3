// Shared device definitions of the spatial-query library: exact FP32 geometry in the reference's operation order,
// element record layouts, wide-node layout, and launch bookkeeping.
//
// Every translation unit of this library is compiled with --fmad=false, so no multiply-add below is fused and each
// expression rounds exactly as the reference's FP32 Eigen code does (vectors are Eigen fixed-size 3-vectors; a
// 3-element reduction such as dot() or squaredNorm() evaluates e0 + (e1 + e2)). Division and square root are the
// IEEE-rounded operations (-prec-div / -prec-sqrt defaults) and denormals are kept (no flush-to-zero).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <climits>
#include <cstdio>
#include <stdexcept>
#include <string>

#include "../../include/thea_gpu.h"

namespace thea {

//============================================================================================================================
// Errors and launch bookkeeping (host)
//============================================================================================================================

struct Error : public std::runtime_error {
  thea_status status;
  Error(thea_status s, std::string const & msg) : std::runtime_error(msg), status(s) {}
};

#define THEA_CUDA_CHECK(expr)                                                                                      \
  do {                                                                                                            \
    cudaError_t _e = (expr);                                                                                      \
    if (_e != cudaSuccess) {                                                                                      \
      thea_status _s = (_e == cudaErrorMemoryAllocation) ? THEA_ERR_OUT_OF_MEMORY : THEA_ERR_CUDA;                \
      throw ::thea::Error(_s, std::string(#expr) + ": " + cudaGetErrorString(_e) + " (" + __FILE__ + ":" +        \
                                  std::to_string(__LINE__) + ")");                                                \
    }                                                                                                             \
  } while (0)

#define THEA_REQUIRE(cond, msg)                                                                                    \
  do {                                                                                                            \
    if (!(cond)) throw ::thea::Error(THEA_ERR_INVALID_ARGUMENT, msg);                                             \
  } while (0)

// Counts every kernel launch of the library and, when profiling is on, brackets it with CUDA events on its stream.
void note_launch(char const * kernel_name, cudaStream_t stream, cudaEvent_t * begin_event);
void note_launch_end(char const * kernel_name, cudaStream_t stream, cudaEvent_t begin_event);

// Counts every device or pinned-host allocation the library makes (driver or pool); the allocators below go through it.
void note_allocation();
template <class T> inline cudaError_t thea_malloc(T ** p, size_t n) {
  note_allocation();
  return cudaMalloc((void **)p, n);
}
template <class T> inline cudaError_t thea_malloc_host(T ** p, size_t n) {
  note_allocation();
  return cudaMallocHost((void **)p, n);
}
template <class T> inline cudaError_t thea_malloc_async(T ** p, size_t n, cudaStream_t s) {
  note_allocation();
  return cudaMallocAsync((void **)p, n, s);
}
template <class T> inline cudaError_t thea_malloc_from_pool_async(T ** p, size_t n, cudaMemPool_t pool, cudaStream_t s) {
  note_allocation();
  return cudaMallocFromPoolAsync((void **)p, n, pool, s);
}

struct LaunchScope {
  char const * name;
  cudaStream_t stream;
  cudaEvent_t begin = nullptr;
  LaunchScope(char const * n, cudaStream_t s) : name(n), stream(s) { note_launch(name, stream, &begin); }
  ~LaunchScope() { note_launch_end(name, stream, begin); }
};

// Launch a kernel with bookkeeping, then check the launch itself for errors.
#define THEA_LAUNCH(kernel, grid, block, smem, stream, ...)                                                        \
  THEA_LAUNCH_NAMED(#kernel, kernel, grid, block, smem, stream, __VA_ARGS__)

// The same, with an explicit name for the timing records (for kernels held in a variable).
#define THEA_LAUNCH_NAMED(name, kernel, grid, block, smem, stream, ...)                                            \
  do {                                                                                                            \
    ::thea::LaunchScope _scope(name, stream);                                                                     \
    kernel<<<(grid), (block), (smem), (stream)>>>(__VA_ARGS__);                                                   \
    THEA_CUDA_CHECK(cudaGetLastError());                                                                          \
  } while (0)

__host__ __device__ inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

//============================================================================================================================
// Exact FP32 vector arithmetic (device + host)
//============================================================================================================================

struct V3 {
  float x, y, z;
};

__host__ __device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__host__ __device__ __forceinline__ V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__host__ __device__ __forceinline__ V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__host__ __device__ __forceinline__ V3 operator*(float s, V3 a) { return V3{s * a.x, s * a.y, s * a.z}; }
__host__ __device__ __forceinline__ V3 operator*(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
__host__ __device__ __forceinline__ V3 operator/(V3 a, float s) { return V3{a.x / s, a.y / s, a.z / s}; }
__host__ __device__ __forceinline__ float get(V3 const & v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }

// Eigen's fixed-size 3-element reduction order: e0 + (e1 + e2)
__host__ __device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + (a.y * b.y + a.z * b.z); }
__host__ __device__ __forceinline__ float squared_norm(V3 a) { return a.x * a.x + (a.y * a.y + a.z * a.z); }
__host__ __device__ __forceinline__ V3 cross(V3 a, V3 b) {
  return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// MatrixBase::normalized(): divide by sqrt(squaredNorm) only when it is positive
__host__ __device__ __forceinline__ V3 normalized(V3 a) {
  float z = squared_norm(a);
  return z > 0.f ? a / sqrtf(z) : a;
}
// Math::maxAbsAxis (Code/Source/MatrixUtil.hpp:110-115): first index of the largest |component|
__host__ __device__ __forceinline__ int max_abs_axis(V3 v) {
  float a0 = fabsf(v.x), a1 = fabsf(v.y), a2 = fabsf(v.z);
  int m = 0;
  float best = a0;
  if (a1 > best) { m = 1; best = a1; }
  if (a2 > best) { m = 2; }
  return m;
}

__device__ __forceinline__ V3 load_v3(float const * p) { return V3{p[0], p[1], p[2]}; }
__device__ __forceinline__ V3 xyz(float4 a) { return V3{a.x, a.y, a.z}; }

//============================================================================================================================
// Triangle primitives (Code/Source/Triangle3.hpp, HyperplaneN.hpp, Hyperplane3.hpp)
//============================================================================================================================

// Cached triangle properties as TriangleN<3>::update() computes them (Triangle3.hpp:143-155)
struct TriPlane {
  V3 normal;   // HyperplaneN::fromThreePoints: normalized((v1 - v0) x (v2 - v0)) (Hyperplane3.hpp:34-41)
  float dist;  // normal . v0
  int axis;    // maxAbsAxis(normal)
  float area;  // 0.5 * |normal . (e01 x e02)|
};

__host__ __device__ __forceinline__ TriPlane tri_plane(V3 v0, V3 v1, V3 v2) {
  TriPlane t;
  V3 e01 = v1 - v0, e02 = v2 - v0;
  t.normal = normalized(cross(e01, e02));
  t.dist = dot(t.normal, v0);
  t.axis = max_abs_axis(t.normal);
  t.area = 0.5f * fabsf(dot(t.normal, cross(e01, e02)));
  return t;
}

// Triangle3Internal::isPointInsideTriangle (Triangle3.hpp:1416-1462)
__device__ __forceinline__ bool point_inside_triangle(V3 v0, V3 v1, V3 v2, int axis, V3 p) {
  float v0i, v0j, v1i, v1j, v2i, v2j, pi, pj;
  if (axis == 1) {  // i = 2, j = 0
    v0i = v0.z; v0j = v0.x; v1i = v1.z; v1j = v1.x; v2i = v2.z; v2j = v2.x; pi = p.z; pj = p.x;
  } else if (axis == 2) {  // i = 0, j = 1
    v0i = v0.x; v0j = v0.y; v1i = v1.x; v1j = v1.y; v2i = v2.x; v2j = v2.y; pi = p.x; pj = p.y;
  } else {  // i = 1, j = 2
    v0i = v0.y; v0j = v0.z; v1i = v1.y; v1j = v1.z; v2i = v2.y; v2j = v2.z; pi = p.y; pj = p.z;
  }
  // AREA2(d, e, f) = (e_i - d_i) (f_j - d_j) - (f_i - d_i) (e_j - d_j)
  float area = (v1i - v0i) * (v2j - v0j) - (v2i - v0i) * (v1j - v0j);
  if (area == 0.f) return v0.x == p.x && v0.y == p.y && v0.z == p.z;
  float inv_area = 1.0f / area;
  float b0 = ((v1i - pi) * (v2j - pj) - (v2i - pi) * (v1j - pj)) * inv_area;
  if ((b0 < 0.f) || (b0 > 1.f)) return false;
  float b1 = ((pi - v0i) * (v2j - v0j) - (v2i - v0i) * (pj - v0j)) * inv_area;
  if ((b1 < 0.f) || (b1 > 1.f)) return false;
  float b2 = 1.0f - b0 - b1;
  return (b2 >= 0.f) && (b2 <= 1.f);
}

// Triangle3Internal::closestPointOnLineSegment (Triangle3.hpp:1311-1338) with a precomputed unit direction and length
__device__ __forceinline__ V3 closest_on_segment(V3 a, V3 b, V3 dir, float len, V3 p) {
  V3 c = p - a;
  float t = dot(dir, c);
  if (t <= 0.f) return a;
  if (t >= len) return b;
  return a + dir * t;
}

// Triangle3Internal::closestPointOnTrianglePerimeter (Triangle3.hpp:1342-1412)
__device__ __forceinline__ V3 closest_on_perimeter(V3 v0, V3 v1, V3 v2, V3 d0, float l0, V3 d1, float l1, V3 d2,
                                                   float l2, V3 p) {
  V3 r0 = closest_on_segment(v0, v1, d0, l0, p);
  V3 r1 = closest_on_segment(v1, v2, d1, l1, p);
  V3 r2 = closest_on_segment(v2, v0, d2, l2, p);
  float q0 = squared_norm(r0 - p), q1 = squared_norm(r1 - p), q2 = squared_norm(r2 - p);
  if (q0 < q1) return (q0 < q2) ? r0 : r2;
  return (q1 < q2) ? r1 : r2;
}

// Edge directions and lengths as closestPointOnTrianglePerimeter computes them: dir = (b - a) / |b - a|
__host__ __device__ __forceinline__ void edge_dir(V3 a, V3 b, V3 & dir, float & len) {
  V3 e = b - a;
  len = sqrtf(squared_norm(e));
  dir = e / len;
}

// Triangle3Internal::rayTriangleIntersectionTime (Triangle3.hpp:1466-1524). Returns -1 on a miss.
__device__ __forceinline__ float ray_triangle_time(V3 origin, V3 dir, V3 v0, V3 e01, V3 e02) {
  float const EPS = 1.1920928955078125e-07f;  // FLT_EPSILON, Math::eps<float>()
  V3 diff = origin - v0;
  V3 n = cross(e01, e02);
  float DdN = dot(dir, n);
  float sign;
  if (DdN > EPS) sign = 1.f;
  else if (DdN < -EPS) { sign = -1.f; DdN = -DdN; }
  else return -1.f;
  float DdQxE2 = sign * dot(dir, cross(diff, e02));
  if (DdQxE2 >= 0.f) {
    float DdE1xQ = sign * dot(dir, cross(e01, diff));
    if (DdE1xQ >= 0.f) {
      if (DdQxE2 + DdE1xQ <= DdN) {
        float QdN = (-sign) * dot(diff, n);
        if (QdN >= 0.f) return QdN / DdN;
      }
    }
  }
  return -1.f;
}

//============================================================================================================================
// Element records, stored in leaf order (sorted by Morton code) so that a leaf's elements are contiguous
//============================================================================================================================

// Closest-point record: 8 x float4 = 128 bytes (one cache line). The in-plane test reads r0..r3 only.
//   r0 = (v0, plane dist)   r1 = (v1, edge len 0)   r2 = (v2, edge len 1)   r3 = (normal, primary axis bits)
//   r4 = (edge dir 0, edge len 2)   r5 = (edge dir 1, original index bits)   r6 = (edge dir 2, area)   r7 = unused
// Edge i runs from vertex i to vertex i+1 (mod 3), with unit direction and length as the perimeter search computes them.
constexpr int CP_REC_F4 = 8;
// Ray record: 3 x float4 = 48 bytes: (v0, original index bits), (e01, 0), (e02, 0)
constexpr int RAY_REC_F4 = 3;
// Point record: 1 x float4 = 16 bytes: (p, original index bits)

//============================================================================================================================
// Wide BVH node: W children, boxes in structure-of-arrays order so a node is read with 16-byte vector loads.
//   child[c] >= 0         : index of an internal node
//   child[c] == EMPTY      : unused slot
//   otherwise              : leaf, ~child[c] = (first element << 4) | (count - 1), count in 1..16
//============================================================================================================================

constexpr int CHILD_EMPTY = INT_MIN;
constexpr int LEAF_COUNT_BITS = 4;
constexpr int MAX_LEAF_SIZE = 1 << LEAF_COUNT_BITS;

__host__ __device__ __forceinline__ int encode_leaf(int first, int count) {
  return ~((first << LEAF_COUNT_BITS) | (count - 1));
}
__host__ __device__ __forceinline__ void decode_leaf(int code, int & first, int & count) {
  int v = ~code;
  first = v >> LEAF_COUNT_BITS;
  count = (v & (MAX_LEAF_SIZE - 1)) + 1;
}

template <int W> struct alignas(16) WideNode {
  float lox[W], hix[W], loy[W], hiy[W], loz[W], hiz[W];
  int child[W];
  int pad[W == 4 ? 4 : 8];  // 128 bytes for W = 4, 256 bytes for W = 8
};
static_assert(sizeof(WideNode<4>) == 128, "BVH4 node must be one 128-byte line");
static_assert(sizeof(WideNode<8>) == 256, "BVH8 node must be two 128-byte lines");

// Read-only 16-byte load through the non-coherent path
__device__ __forceinline__ float4 ldg4(float4 const * p) { return __ldg(p); }
__device__ __forceinline__ int4 ldg4i(int4 const * p) { return __ldg(p); }

// Slack applied when comparing a box's lower bound with the best element distance (relative): covers the rounding of
// element distances, so a box holding an element at exactly the best distance is never skipped.
constexpr float PRUNE_SLACK = 1.0f + 1.0f / 262144.0f;  // 1 + 2^-18

}  // namespace thea
