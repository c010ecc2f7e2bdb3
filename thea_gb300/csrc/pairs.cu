// Closest pairs between two BVHs (BvhN::closestPair, BvhN.hpp:1082-1114, and kClosestPairs, :1139-1146, with a BVH as
// the query; the reference descends both trees together, BvhN.hpp:1916-2033).
//
// A pair's distance is the distance between one element of each structure, so the closest pair is the smallest, over
// the elements of one side, of that element's nearest neighbour on the other side: the batched nearest-neighbour kernels
// answer it with one query per element, and a 64-bit atomic minimum of (squared distance bits, query index) picks the
// pair (non-negative floats order like their bit patterns). Point-point pairs query the target's points from the
// query's; point-mesh pairs query the mesh from the points, whichever side the mesh is on. The k closest pairs of two
// point sets are among the k nearest target points of each query point within the k-th smallest of the rows' nearest
// distances: those candidates are compacted in slot order and sorted by (squared distance, query index) with a stable
// radix sort that keeps each row's target order.
//
// Mesh-mesh pairs: one thread per query triangle descends the target BVH with the box-box lower bound and evaluates the
// reference's triangle-triangle distance at the leaves; every thread also prunes against the best distance found by
// any thread so far (a 64-bit atomic minimum of (squared distance bits, query index)), which cannot remove a pair at
// the final minimum distance, so the tie rule still sees all of them.
#include "pairs.hpp"

#include "device_util.cuh"
#include "query.hpp"
#include "transform.hpp"
#include "traverse_ops.cuh"

#include <algorithm>
#include <cstring>

namespace thea {
namespace {

constexpr int PAIR_THREADS = 256;

// coordinates of a point BVH's elements in element order
__global__ void element_points_kernel(float4 const * __restrict__ rec, int32_t const * __restrict__ leaf_to_elem,
                                      int64_t n, float * __restrict__ out) {
  int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= n) return;
  float4 r = rec[p];
  int64_t e = leaf_to_elem[p];
  out[3 * e] = r.x;
  out[3 * e + 1] = r.y;
  out[3 * e + 2] = r.z;
}

__device__ __forceinline__ float row_d2(int64_t r, float const * d2, float const * pts, float const * cp) {
  if (d2) return d2[r];
  V3 a = load_v3(cp + 3 * r), b = load_v3(pts + 3 * r);
  return squared_norm(a - b);  // as the closest-point kernel evaluates it: |closest point - query|^2
}

// per row (one element of the searching side): key = (d2 bits, query index), minimum over rows
__global__ void pair_min_kernel(int32_t const * __restrict__ idx, float const * __restrict__ d2,
                                float const * __restrict__ pts, float const * __restrict__ cp, int64_t n,
                                int rows_are_query, unsigned long long * __restrict__ best) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n || idx[r] < 0) return;
  uint32_t q = rows_are_query ? (uint32_t)r : (uint32_t)idx[r];
  unsigned long long key = ((unsigned long long)__float_as_uint(row_d2(r, d2, pts, cp)) << 32) | q;
  atomicMin(best, key);
}

// among rows holding the best key: the lowest target index
__global__ void pair_tie_kernel(int32_t const * __restrict__ idx, float const * __restrict__ d2,
                                float const * __restrict__ pts, float const * __restrict__ cp, int64_t n,
                                int rows_are_query, unsigned long long const * __restrict__ best,
                                unsigned * __restrict__ best_target) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n || idx[r] < 0) return;
  uint32_t q = rows_are_query ? (uint32_t)r : (uint32_t)idx[r];
  unsigned long long key = ((unsigned long long)__float_as_uint(row_d2(r, d2, pts, cp)) << 32) | q;
  if (key == *best) atomicMin(best_target, rows_are_query ? (unsigned)idx[r] : (unsigned)r);
}

// key of each row's nearest distance for the k-th-smallest selection (all ones for a row without a neighbour)
__global__ void row_min_keys_kernel(int32_t const * __restrict__ idx, float const * __restrict__ d2, int64_t n,
                                    unsigned long long * __restrict__ keys, uint32_t * __restrict__ vals) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  keys[r] = idx[r] < 0 ? 0xffffffffull : (unsigned long long)__float_as_uint(d2[r]);
  vals[r] = (uint32_t)r;
}

__global__ void slot_flag_kernel(int32_t const * __restrict__ idx, int64_t slots, uint32_t * __restrict__ flag) {
  int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c < slots) flag[c] = idx[c] >= 0 ? 1u : 0u;
}

__global__ void slot_total_kernel(uint32_t const * __restrict__ flag, uint32_t const * __restrict__ pos, int64_t slots,
                                  uint32_t * __restrict__ total) {
  *total = pos[slots - 1] + flag[slots - 1];
}

// filled slot c = row * k + j of the k-NN rows, written at its compacted position: key (d2 bits, row), value c
__global__ void pair_candidates_kernel(int32_t const * __restrict__ idx, float const * __restrict__ d2,
                                       uint32_t const * __restrict__ pos, int64_t slots, int k,
                                       unsigned long long * __restrict__ keys, uint32_t * __restrict__ vals) {
  int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= slots || idx[c] < 0) return;
  uint32_t p = pos[c];
  keys[p] = ((unsigned long long)__float_as_uint(d2[c]) << 32) | (uint64_t)(c / k);
  vals[p] = (uint32_t)c;
}

__global__ void pair_take_kernel(unsigned long long const * __restrict__ keys, uint32_t const * __restrict__ vals,
                                 int32_t const * __restrict__ idx, float const * __restrict__ d2, int64_t m, int k,
                                 int32_t * __restrict__ qi, int32_t * __restrict__ ti, float * __restrict__ od2,
                                 unsigned * __restrict__ count) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= k) return;
  bool ok = j < m && keys[j] != ~0ull;
  qi[j] = ok ? (int32_t)(keys[j] & 0xffffffffu) : -1;
  ti[j] = ok ? idx[vals[j]] : -1;
  od2[j] = ok ? d2[vals[j]] : -1.f;
  if (ok) atomicAdd(count, 1u);
}

//============================================================================================================================
// Triangle-triangle distance: TriangleN<3>::squaredDistance(other, this_pt, other_pt) (Triangle3.hpp:314-400, after
// Ericson), with Moller's intersection test returning the intersection segment (tri_tri_intersect_with_isectline,
// Triangle3.hpp:1117-1290; coplanar_tri_tri :730-776) and Internal::closestPtSegmentSegment (LineSegmentN.hpp:262-340).
// The intersection test evaluates the reference's C expressions on coordinate arrays (three-term sums left to right);
// the segment and projection steps use Eigen's e0 + (e1 + e2) reduction (dot, squared_norm). Every FP32 operation is
// the reference's, in its order, so the squared distance is bit-identical with the reference's evaluation for the same
// ("this", "other") roles.
//============================================================================================================================

struct TriRec {
  V3 v[3];
  V3 n;       // unit plane normal
  float dist;  // plane offset
  int axis;    // primary axis
};

__device__ __forceinline__ TriRec load_tri(float4 const * __restrict__ rec, int64_t k) {
  float4 const * r = rec + k * CP_REC_F4;
  float4 a = __ldg(r), b = __ldg(r + 1), c = __ldg(r + 2), nn = __ldg(r + 3);
  TriRec t;
  t.v[0] = xyz(a); t.v[1] = xyz(b); t.v[2] = xyz(c);
  t.n = xyz(nn);
  t.dist = a.w;
  t.axis = __float_as_int(nn.w);
  return t;
}

__device__ __forceinline__ float dot_lr(float const * a, float const * b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
__device__ __forceinline__ void cross_a(float * d, float const * a, float const * b) {
  d[0] = a[1] * b[2] - a[2] * b[1];
  d[1] = a[2] * b[0] - a[0] * b[2];
  d[2] = a[0] * b[1] - a[1] * b[0];
}
__device__ __forceinline__ void sub_a(float * d, float const * a, float const * b) {
  d[0] = a[0] - b[0]; d[1] = a[1] - b[1]; d[2] = a[2] - b[2];
}

// EDGE_EDGE_TEST (Triangle3.hpp:674-693)
__device__ __forceinline__ bool tt_edge_edge(float Ax, float Ay, float const * v0, float const * u0, float const * u1,
                                             int i0, int i1) {
  float Bx = u0[i0] - u1[i0], By = u0[i1] - u1[i1];
  float Cx = v0[i0] - u0[i0], Cy = v0[i1] - u0[i1];
  float f = Ay * Bx - Ax * By;
  float d = By * Cx - Bx * Cy;
  if ((f > 0.f && d >= 0.f && d <= f) || (f < 0.f && d <= 0.f && d >= f)) {
    float e = Ax * Cy - Ay * Cx;
    if (f > 0.f) return e >= 0.f && e <= f;
    return e <= 0.f && e >= f;
  }
  return false;
}

// EDGE_AGAINST_TRI_EDGES (Triangle3.hpp:695-707)
__device__ __forceinline__ bool tt_edge_tri(float const * v0, float const * v1, float const * u0, float const * u1,
                                            float const * u2, int i0, int i1) {
  float Ax = v1[i0] - v0[i0], Ay = v1[i1] - v0[i1];
  return tt_edge_edge(Ax, Ay, v0, u0, u1, i0, i1) || tt_edge_edge(Ax, Ay, v0, u1, u2, i0, i1) ||
         tt_edge_edge(Ax, Ay, v0, u2, u0, i0, i1);
}

// POINT_IN_TRI (Triangle3.hpp:709-728)
__device__ __forceinline__ bool tt_point_in_tri(float const * v0, float const * u0, float const * u1, float const * u2,
                                                int i0, int i1) {
  float a = u1[i1] - u0[i1], b = -(u1[i0] - u0[i0]);
  float c = -a * u0[i0] - b * u0[i1];
  float d0 = a * v0[i0] + b * v0[i1] + c;
  a = u2[i1] - u1[i1]; b = -(u2[i0] - u1[i0]);
  c = -a * u1[i0] - b * u1[i1];
  float d1 = a * v0[i0] + b * v0[i1] + c;
  a = u0[i1] - u2[i1]; b = -(u0[i0] - u2[i0]);
  c = -a * u2[i0] - b * u2[i1];
  float d2 = a * v0[i0] + b * v0[i1] + c;
  return d0 * d1 > 0.f && d0 * d2 > 0.f;
}

// coplanar_tri_tri (Triangle3.hpp:730-776)
__device__ bool tt_coplanar(float const * N, float const * v0, float const * v1, float const * v2, float const * u0,
                            float const * u1, float const * u2) {
  float A0 = fabsf(N[0]), A1 = fabsf(N[1]), A2 = fabsf(N[2]);
  int i0, i1;
  if (A0 > A1) {
    if (A0 > A2) { i0 = 1; i1 = 2; }
    else { i0 = 0; i1 = 1; }
  } else {
    if (A2 > A1) { i0 = 0; i1 = 1; }
    else { i0 = 0; i1 = 2; }
  }
  return tt_edge_tri(v0, v1, u0, u1, u2, i0, i1) || tt_edge_tri(v1, v2, u0, u1, u2, i0, i1) ||
         tt_edge_tri(v2, v0, u0, u1, u2, i0, i1) || tt_point_in_tri(v0, u0, u1, u2, i0, i1) ||
         tt_point_in_tri(u0, v0, v1, v2, i0, i1);
}

// isect2 (Triangle3.hpp:1023-1039)
__device__ __forceinline__ void tt_isect2(float const * x0, float const * x1, float const * x2, float vv0, float vv1,
                                          float vv2, float d0, float d1, float d2, float & is0, float & is1, float * p0,
                                          float * p1) {
  float tmp = d0 / (d0 - d1);
  float diff[3];
  is0 = vv0 + (vv1 - vv0) * tmp;
  sub_a(diff, x1, x0);
#pragma unroll
  for (int k = 0; k < 3; ++k) p0[k] = tmp * diff[k] + x0[k];
  tmp = d0 / (d0 - d2);
  is1 = vv0 + (vv2 - vv0) * tmp;
  sub_a(diff, x2, x0);
#pragma unroll
  for (int k = 0; k < 3; ++k) p1[k] = x0[k] + tmp * diff[k];
}

// compute_intervals_isectline (Triangle3.hpp:1041-1077): true when the triangles are coplanar
__device__ __forceinline__ bool tt_intervals(float const * x0, float const * x1, float const * x2, float vv0, float vv1,
                                             float vv2, float d0, float d1, float d2, float d0d1, float d0d2,
                                             float & is0, float & is1, float * p0, float * p1) {
  if (d0d1 > 0.f) tt_isect2(x2, x0, x1, vv2, vv0, vv1, d2, d0, d1, is0, is1, p0, p1);
  else if (d0d2 > 0.f) tt_isect2(x1, x0, x2, vv1, vv0, vv2, d1, d0, d2, is0, is1, p0, p1);
  else if (d1 * d2 > 0.f || d0 != 0.f) tt_isect2(x0, x1, x2, vv0, vv1, vv2, d0, d1, d2, is0, is1, p0, p1);
  else if (d1 != 0.f) tt_isect2(x1, x0, x2, vv1, vv0, vv2, d1, d0, d2, is0, is1, p0, p1);
  else if (d2 != 0.f) tt_isect2(x2, x0, x1, vv2, vv0, vv1, d2, d0, d1, is0, is1, p0, p1);
  else return true;
  return false;
}

// tri_tri_intersect_with_isectline (Triangle3.hpp:1117-1290)
__device__ bool tt_intersect(float const * V0, float const * V1, float const * V2, float const * U0, float const * U1,
                             float const * U2, bool & coplanar, float * pt1, float * pt2) {
  float const EPS = 1.1920928955078125e-07f;  // Math::eps<float>()
  float E1[3], E2[3], N1[3], N2[3], D[3];
  float isA[2] = {0.f, 0.f}, isB[2] = {0.f, 0.f};
  float pA1[3] = {0.f, 0.f, 0.f}, pA2[3] = {0.f, 0.f, 0.f}, pB1[3] = {0.f, 0.f, 0.f}, pB2[3] = {0.f, 0.f, 0.f};
  sub_a(E1, V1, V0);
  sub_a(E2, V2, V0);
  cross_a(N1, E1, E2);
  float d1 = -dot_lr(N1, V0);
  float du0 = dot_lr(N1, U0) + d1, du1 = dot_lr(N1, U1) + d1, du2 = dot_lr(N1, U2) + d1;
  if (fabsf(du0) < EPS) du0 = 0.f;
  if (fabsf(du1) < EPS) du1 = 0.f;
  if (fabsf(du2) < EPS) du2 = 0.f;
  float du0du1 = du0 * du1, du0du2 = du0 * du2;
  if (du0du1 > 0.f && du0du2 > 0.f) return false;
  sub_a(E1, U1, U0);
  sub_a(E2, U2, U0);
  cross_a(N2, E1, E2);
  float d2 = -dot_lr(N2, U0);
  float dv0 = dot_lr(N2, V0) + d2, dv1 = dot_lr(N2, V1) + d2, dv2 = dot_lr(N2, V2) + d2;
  if (fabsf(dv0) < EPS) dv0 = 0.f;
  if (fabsf(dv1) < EPS) dv1 = 0.f;
  if (fabsf(dv2) < EPS) dv2 = 0.f;
  float dv0dv1 = dv0 * dv1, dv0dv2 = dv0 * dv2;
  if (dv0dv1 > 0.f && dv0dv2 > 0.f) return false;
  cross_a(D, N1, N2);
  float mx = fabsf(D[0]);
  int index = 0;
  float b = fabsf(D[1]), c = fabsf(D[2]);
  if (b > mx) { mx = b; index = 1; }
  if (c > mx) { mx = c; index = 2; }
  coplanar = tt_intervals(V0, V1, V2, V0[index], V1[index], V2[index], dv0, dv1, dv2, dv0dv1, dv0dv2, isA[0], isA[1],
                          pA1, pA2);
  if (coplanar) return tt_coplanar(N1, V0, V1, V2, U0, U1, U2);
  tt_intervals(U0, U1, U2, U0[index], U1[index], U2[index], du0, du1, du2, du0du1, du0du2, isB[0], isB[1], pB1, pB2);
  bool s1 = false, s2 = false;
  if (isA[0] > isA[1]) { float t = isA[0]; isA[0] = isA[1]; isA[1] = t; s1 = true; }
  if (isB[0] > isB[1]) { float t = isB[0]; isB[0] = isB[1]; isB[1] = t; s2 = true; }
  if (isA[1] < isB[0] || isB[1] < isA[0]) return false;
  float const * a_lo = s1 ? pA2 : pA1;
  float const * a_hi = s1 ? pA1 : pA2;
  float const * b_lo = s2 ? pB2 : pB1;
  float const * b_hi = s2 ? pB1 : pB2;
  float const * e1 = isB[0] < isA[0] ? a_lo : b_lo;
  float const * e2 = isB[0] < isA[0] ? (isB[1] < isA[1] ? b_hi : a_hi) : (isB[1] > isA[1] ? a_hi : b_hi);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    pt1[k] = e1[k];
    pt2[k] = e2[k];
  }
  return true;
}

// Math::fuzzyEq(a, 0) (Math.hpp:131-148)
__device__ __forceinline__ bool fuzzy_zero(float a) {
  float const E = 1.1920928955078125e-07f;
  if (isinf(a)) return false;
  float l = fabsf(a);
  float tol = l > 1.f ? l * E : E;
  return a == 0.f || fabsf(a) <= tol;
}

__device__ __forceinline__ float clamp01(float x) { return x < 0.f ? 0.f : (x > 1.f ? 1.f : x); }

// Internal::closestPtSegmentSegment for two segments (LineSegmentN.hpp:262-340)
__device__ float tt_segment_segment(V3 p1, V3 q1, V3 p2, V3 q2, V3 & c1, V3 & c2) {
  V3 d1 = q1 - p1, d2 = q2 - p2, r = p1 - p2;
  float a = squared_norm(d1), e = squared_norm(d2), f = dot(d2, r);
  float s, t;
  if (fuzzy_zero(a)) {
    if (fuzzy_zero(e)) {
      c1 = p1;
      c2 = p2;
      return dot(c1 - c2, c1 - c2);
    }
    s = 0.f;
    t = clamp01(f / e);
  } else {
    float c = dot(d1, r);
    if (fuzzy_zero(e)) {
      t = 0.f;
      s = clamp01(-c / a);
    } else {
      float b = dot(d1, d2);
      float denom = a * e - b * b;
      s = denom != 0.f ? clamp01((b * f - c * e) / denom) : 0.f;
      t = (b * s + f) / e;
      if (t < 0.f) {
        t = 0.f;
        s = clamp01(-c / a);
      } else if (t > 1.f) {
        t = 1.f;
        s = clamp01((b - c) / a);
      }
    }
  }
  c1 = p1 + s * d1;
  c2 = p2 + t * d2;
  return squared_norm(c1 - c2);
}

// TriangleN<3>::squaredDistance(other, this_pt, other_pt) with a = "this", b = "other"
__device__ __noinline__ float tri_tri_sq_distance(TriRec const & a, TriRec const & b, V3 & pa, V3 & pb) {
  V3 c1 = V3{0.f, 0.f, 0.f}, c2 = c1;
  float best = 3.402823466e+38f;  // std::numeric_limits<float>::max()
  float A0[3] = {a.v[0].x, a.v[0].y, a.v[0].z}, A1[3] = {a.v[1].x, a.v[1].y, a.v[1].z};
  float A2[3] = {a.v[2].x, a.v[2].y, a.v[2].z};
  float B0[3] = {b.v[0].x, b.v[0].y, b.v[0].z}, B1[3] = {b.v[1].x, b.v[1].y, b.v[1].z};
  float B2[3] = {b.v[2].x, b.v[2].y, b.v[2].z};
  bool cop = false;
  float i1[3] = {0.f, 0.f, 0.f}, i2[3] = {0.f, 0.f, 0.f};
  if (tt_intersect(A0, A1, A2, B0, B1, B2, cop, i1, i2)) {
    if (cop) {
      V3 ca = (a.v[0] + a.v[1] + a.v[2]) / 3.f, cb = (b.v[0] + b.v[1] + b.v[2]) / 3.f;
      c1 = c2 = 0.5f * (ca + cb);
    } else {
      // LineSegmentN keeps (point, direction); getPoint(t) = point + t * direction
      V3 pt = V3{i1[0], i1[1], i1[2]};
      V3 dir = V3{i2[0], i2[1], i2[2]} - pt;
      c1 = c2 = 0.5f * ((pt + 0.f * dir) + (pt + 1.f * dir));
    }
    best = 0.f;
  } else {
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        V3 p, q;
        float d2 = tt_segment_segment(a.v[i], a.v[i == 2 ? 0 : i + 1], b.v[j], b.v[j == 2 ? 0 : j + 1], p, q);
        if (d2 < best) { best = d2; c1 = p; c2 = q; }
      }
    for (int i = 0; i < 3; ++i) {  // vertices of b projected into a
      V3 q = b.v[i];
      V3 p = q - (dot(q, a.n) - a.dist) * a.n;
      if (point_inside_triangle(a.v[0], a.v[1], a.v[2], a.axis, p)) {
        float d2 = squared_norm(p - q);
        if (d2 < best) { best = d2; c1 = p; c2 = q; }
      }
    }
    for (int i = 0; i < 3; ++i) {  // vertices of a projected into b
      V3 p = a.v[i];
      V3 q = p - (dot(p, b.n) - b.dist) * b.n;
      if (point_inside_triangle(b.v[0], b.v[1], b.v[2], b.axis, q)) {
        float d2 = squared_norm(p - q);
        if (d2 < best) { best = d2; c1 = p; c2 = q; }
      }
    }
  }
  pa = c1;
  pb = c2;
  return best;
}

__device__ __forceinline__ float box_box_d2(float lx, float ly, float lz, float hx, float hy, float hz, V3 qlo, V3 qhi) {
  float dx = fmaxf(fmaxf(lx - qhi.x, qlo.x - hx), 0.f);
  float dy = fmaxf(fmaxf(ly - qhi.y, qlo.y - hy), 0.f);
  float dz = fmaxf(fmaxf(lz - qhi.z, qlo.z - hz), 0.f);
  return __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, dz * dz));
}

__device__ __forceinline__ float key_d2(unsigned long long key) {
  return key == ~0ull ? INFINITY : __uint_as_float((unsigned)(key >> 32));
}

// One thread per query triangle (query sorted position p): its nearest target triangle (smallest d2 <= thresh, lowest
// target index among ties) under a bound that also uses the best key any thread has published. Row arrays are indexed
// by the query element index; a row that finds nothing within the bound gets target -1.
template <int W, int STACK>
__global__ void __launch_bounds__(PAIR_THREADS) mesh_pair_kernel(
    WideNode<W> const * __restrict__ tnodes, float4 const * __restrict__ trec, float4 const * __restrict__ qrec,
    int64_t nq, float thresh, unsigned long long * __restrict__ best_key, int32_t * __restrict__ row_t,
    float * __restrict__ row_d2, int64_t * __restrict__ row_slots, unsigned * __restrict__ err) {
  int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= nq) return;
  TriRec q = load_tri(qrec, p);
  int qe = cp_record_index(qrec, p);
  V3 qlo = V3{fminf(q.v[0].x, fminf(q.v[1].x, q.v[2].x)), fminf(q.v[0].y, fminf(q.v[1].y, q.v[2].y)),
              fminf(q.v[0].z, fminf(q.v[1].z, q.v[2].z))};
  V3 qhi = V3{fmaxf(q.v[0].x, fmaxf(q.v[1].x, q.v[2].x)), fmaxf(q.v[0].y, fmaxf(q.v[1].y, q.v[2].y)),
              fmaxf(q.v[0].z, fmaxf(q.v[1].z, q.v[2].z))};
  float best = thresh;
  int best_t = INT_MAX;
  int64_t best_slot = -1;
  int2 stk[STACK];
  int sp = 0, next = 0;
  while (next != CHILD_EMPTY || sp > 0) {
    float lim = fminf(best, key_d2(*(volatile unsigned long long *)best_key)) * PRUNE_SLACK;
    int code = next;
    if (code == CHILD_EMPTY) {
      --sp;
      code = stk[sp].x;
      if (__int_as_float(stk[sp].y) > lim) continue;
    }
    next = CHILD_EMPTY;
    if (code >= 0) {
      NodeRegs<W> nd;
      load_node(tnodes, code, nd);
      float lb[W];
#pragma unroll
      for (int c = 0; c < W; ++c)
        lb[c] = box_box_d2(nd.lox[c], nd.loy[c], nd.loz[c], nd.hix[c], nd.hiy[c], nd.hiz[c], qlo, qhi);
      push_children_next<W, STACK>(nd, lb, lim, stk, sp, next, err);
    } else {
      int first, count;
      decode_leaf(code, first, count);
      bool improved = false;
      for (int64_t k = first; k < first + count; ++k) {
        TriRec t = load_tri(trec, k);
        V3 pa, pb;
        float d2 = tri_tri_sq_distance(t, q, pa, pb);
        if (d2 <= best) {
          int idx = cp_record_index(trec, k);
          if (d2 < best || idx < best_t) {
            improved = improved || d2 < best || best_t == INT_MAX;
            best = d2;
            best_t = idx;
            best_slot = k;
          }
        }
      }
      if (improved) atomicMin(best_key, ((unsigned long long)__float_as_uint(best) << 32) | (unsigned)qe);
    }
  }
  bool found = best_t != INT_MAX;
  row_t[qe] = found ? best_t : -1;
  row_d2[qe] = found ? best : -1.f;
  row_slots[2 * (int64_t)qe] = p;
  row_slots[2 * (int64_t)qe + 1] = best_slot;
}

// The closest points of one pair (query slot, target slot), target triangle as "this"
__global__ void mesh_pair_points_kernel(float4 const * __restrict__ trec, float4 const * __restrict__ qrec,
                                        int64_t const * __restrict__ slots, unsigned long long const * __restrict__ key,
                                        float * __restrict__ out) {
  if (*key == ~0ull) return;  // no pair
  int64_t qe = (int64_t)(*key & 0xffffffffu);
  TriRec q = load_tri(qrec, slots[2 * qe]), t = load_tri(trec, slots[2 * qe + 1]);
  V3 pa, pb;
  out[6] = tri_tri_sq_distance(t, q, pa, pb);
  out[0] = pb.x; out[1] = pb.y; out[2] = pb.z;
  out[3] = pa.x; out[4] = pa.y; out[5] = pa.z;
}

Scratch element_points(thea_bvh const * b, cudaStream_t s) {
  thea_bvh const * w = query_target(b);  // world-space records when a transform is set
  Scratch out((size_t)w->n * 12, s);
  THEA_LAUNCH(element_points_kernel, (unsigned)ceil_div(w->n, PAIR_THREADS), PAIR_THREADS, 0, s, w->pt_rec,
              w->leaf_to_elem, w->n, out.as<float>());
  return out;
}

void check_single(thea_bvh const * b, char const * what) {
  THEA_REQUIRE(b, std::string(what) + ": null BVH");
  THEA_REQUIRE(b->num_segments == 1, std::string(what) + ": forests are not supported");
  if (b->is_mesh) THEA_REQUIRE(query_target(b)->cp_rec, std::string(what) + ": the mesh BVH needs THEA_LAYOUT_CLOSEST");
}

}  // namespace

// Mesh-mesh closest pair (see the file comment): rows are the query mesh's triangles.
static bool run_mesh_pair(thea_bvh const * target, thea_bvh const * query, float thresh, PairResult & out,
                          cudaStream_t s) {
  thea_bvh const * t = query_target(target);
  thea_bvh const * q = query_target(query);
  int64_t n = q->n;
  if (n == 0 || t->n == 0) return false;
  Scratch rt((size_t)n * 4, s), rd((size_t)n * 4, s), slots((size_t)n * 16, s), best(8, s), best_t(4, s);
  Scratch pts(7 * 4, s);
  THEA_CUDA_CHECK(cudaMemsetAsync(best.ptr, 0xff, 8, s));
  THEA_CUDA_CHECK(cudaMemsetAsync(best_t.ptr, 0xff, 4, s));
  unsigned blocks = (unsigned)ceil_div(n, PAIR_THREADS);
  if (t->width == 4)
    THEA_LAUNCH((mesh_pair_kernel<4, StackSize<4>::value>), blocks, PAIR_THREADS, 0, s,
                (WideNode<4> const *)t->nodes, t->cp_rec, q->cp_rec, n, thresh, best.as<unsigned long long>(),
                rt.as<int32_t>(), rd.as<float>(), slots.as<int64_t>(), target->err);
  else
    THEA_LAUNCH((mesh_pair_kernel<8, StackSize<8>::value>), blocks, PAIR_THREADS, 0, s,
                (WideNode<8> const *)t->nodes, t->cp_rec, q->cp_rec, n, thresh, best.as<unsigned long long>(),
                rt.as<int32_t>(), rd.as<float>(), slots.as<int64_t>(), target->err);
  // the winner: smallest (d2, query index) over the rows, then the lowest target among rows holding it
  THEA_CUDA_CHECK(cudaMemsetAsync(best.ptr, 0xff, 8, s));
  THEA_LAUNCH(pair_min_kernel, blocks, PAIR_THREADS, 0, s, rt.as<int32_t>(), rd.as<float>(), (float const *)nullptr,
              (float const *)nullptr, n, 1, best.as<unsigned long long>());
  THEA_LAUNCH(pair_tie_kernel, blocks, PAIR_THREADS, 0, s, rt.as<int32_t>(), rd.as<float>(), (float const *)nullptr,
              (float const *)nullptr, n, 1, best.as<unsigned long long>(), best_t.as<unsigned>());
  THEA_LAUNCH(mesh_pair_points_kernel, 1, 1, 0, s, t->cp_rec, q->cp_rec, slots.as<int64_t>(),
              best.as<unsigned long long>(), pts.as<float>());
  unsigned long long hb = 0;
  unsigned ht = 0;
  float hp[7];
  THEA_CUDA_CHECK(cudaMemcpyAsync(&hb, best.ptr, 8, cudaMemcpyDeviceToHost, s));
  THEA_CUDA_CHECK(cudaMemcpyAsync(&ht, best_t.ptr, 4, cudaMemcpyDeviceToHost, s));
  THEA_CUDA_CHECK(cudaMemcpyAsync(hp, pts.ptr, sizeof(hp), cudaMemcpyDeviceToHost, s));
  THEA_CUDA_CHECK(cudaStreamSynchronize(s));
  if (hb == ~0ull) return false;
  out.query_index = (int32_t)(hb & 0xffffffffu);
  out.target_index = (int32_t)ht;
  uint32_t bits = (uint32_t)(hb >> 32);
  std::memcpy(&out.d2, &bits, 4);
  std::memcpy(out.query_point, hp, 12);
  std::memcpy(out.target_point, hp + 3, 12);
  return true;
}

bool run_closest_pair(thea_bvh const * target, thea_bvh const * query, float thresh, PairResult & out,
                      cudaStream_t s) {
  check_single(target, "closest_pair");
  check_single(query, "closest_pair");
  out = PairResult();
  if (target->is_mesh && query->is_mesh) return run_mesh_pair(target, query, thresh, out, s);
  // rows: the elements of the point side that searches the other side
  bool rows_are_query = !query->is_mesh;
  thea_bvh const * rows_bvh = rows_are_query ? query : target;
  thea_bvh const * searched = query_target(rows_are_query ? target : query);
  int64_t n = rows_bvh->n;
  if (n == 0 || searched->n == 0) return false;
  Scratch pts = element_points(rows_bvh, s);
  Scratch idx((size_t)n * 4, s), d2, cp, best(8, s), best_t(4, s);
  if (searched->is_mesh) {
    cp = Scratch((size_t)n * 12, s);
    ClosestParams c;
    c.thresh = thresh;
    c.scene_scale = scene_scale_of(searched);
    run_closest(searched, pts.as<float>(), n, c, idx.as<int32_t>(), nullptr, cp.as<float>(), nullptr, searched->err,
                s);
  } else {
    d2 = Scratch((size_t)n * 4, s);
    run_knn(searched, pts.as<float>(), n, 1, thresh, nullptr, idx.as<int32_t>(), d2.as<float>(), searched->err, s);
  }
  THEA_CUDA_CHECK(cudaMemsetAsync(best.ptr, 0xff, 8, s));
  THEA_CUDA_CHECK(cudaMemsetAsync(best_t.ptr, 0xff, 4, s));
  unsigned blocks = (unsigned)ceil_div(n, PAIR_THREADS);
  THEA_LAUNCH(pair_min_kernel, blocks, PAIR_THREADS, 0, s, idx.as<int32_t>(), d2.as<float>(), pts.as<float>(),
              cp.as<float>(), n, rows_are_query ? 1 : 0, best.as<unsigned long long>());
  THEA_LAUNCH(pair_tie_kernel, blocks, PAIR_THREADS, 0, s, idx.as<int32_t>(), d2.as<float>(), pts.as<float>(),
              cp.as<float>(), n, rows_are_query ? 1 : 0, best.as<unsigned long long>(), best_t.as<unsigned>());
  unsigned long long hb = 0;
  unsigned ht = 0;
  THEA_CUDA_CHECK(cudaMemcpyAsync(&hb, best.ptr, 8, cudaMemcpyDeviceToHost, s));
  THEA_CUDA_CHECK(cudaMemcpyAsync(&ht, best_t.ptr, 4, cudaMemcpyDeviceToHost, s));
  THEA_CUDA_CHECK(cudaStreamSynchronize(s));
  if (hb == ~0ull) return false;
  out.query_index = (int32_t)(hb & 0xffffffffu);
  out.target_index = (int32_t)ht;
  uint32_t bits = (uint32_t)(hb >> 32);
  std::memcpy(&out.d2, &bits, 4);
  // the closest points: each point element itself, and on the mesh side the closest point of the row
  int64_t row = rows_are_query ? out.query_index : out.target_index;
  float row_pt[3], other_pt[3];
  THEA_CUDA_CHECK(cudaMemcpyAsync(row_pt, pts.as<float>() + 3 * row, 12, cudaMemcpyDeviceToHost, s));
  Scratch other;
  if (searched->is_mesh) {
    THEA_CUDA_CHECK(cudaMemcpyAsync(other_pt, cp.as<float>() + 3 * row, 12, cudaMemcpyDeviceToHost, s));
  } else {  // point-point: the target point itself
    other = element_points(target, s);
    THEA_CUDA_CHECK(cudaMemcpyAsync(other_pt, other.as<float>() + 3 * (int64_t)out.target_index, 12,
                                    cudaMemcpyDeviceToHost, s));
  }
  THEA_CUDA_CHECK(cudaStreamSynchronize(s));
  std::memcpy(rows_are_query ? out.query_point : out.target_point, row_pt, 12);
  std::memcpy(rows_are_query ? out.target_point : out.query_point, other_pt, 12);
  return true;
}

int64_t run_k_closest_pairs(thea_bvh const * target, thea_bvh const * query, int k, float thresh, int32_t * qi,
                            int32_t * ti, float * d2, cudaStream_t s) {
  check_single(target, "k_closest_pairs");
  check_single(query, "k_closest_pairs");
  THEA_REQUIRE(!target->is_mesh && !query->is_mesh, "k_closest_pairs: two point BVHs are required");
  THEA_REQUIRE(k >= 1 && k <= 32, "k_closest_pairs: k must be in 1..32");
  int64_t n = query->n;
  Scratch count(4, s);
  THEA_CUDA_CHECK(cudaMemsetAsync(count.ptr, 0, 4, s));
  Scratch keys(8, s), vals(4, s), idx(4, s), dd(4, s);
  int64_t m = 0;
  if (n > 0 && target->n > 0) {
    Scratch pts = element_points(query, s);
    thea_bvh const * searched = query_target(target);
    unsigned blocks = (unsigned)ceil_div(n, PAIR_THREADS);
    // 1. every row's nearest target point; the k-th smallest of those distances bounds the k-th closest pair (the k
    //    rows with the smallest minima already give k distinct pairs within it)
    if (n >= k) {
      Scratch idx1((size_t)n * 4, s), d21((size_t)n * 4, s), rk((size_t)n * 8, s), rv((size_t)n * 4, s);
      run_knn(searched, pts.as<float>(), n, 1, thresh, nullptr, idx1.as<int32_t>(), d21.as<float>(), searched->err, s);
      THEA_LAUNCH(row_min_keys_kernel, blocks, PAIR_THREADS, 0, s, idx1.as<int32_t>(), d21.as<float>(), n,
                  rk.as<unsigned long long>(), rv.as<uint32_t>());
      radix_sort_pairs(rk.as<uint64_t>(), rv.as<uint32_t>(), n, 32, s);
      unsigned long long kth = 0;
      THEA_CUDA_CHECK(cudaMemcpyAsync(&kth, rk.as<unsigned long long>() + (k - 1), 8, cudaMemcpyDeviceToHost, s));
      THEA_CUDA_CHECK(cudaStreamSynchronize(s));
      if (kth != 0xffffffffull) {
        float tau;
        uint32_t bits = (uint32_t)kth;
        std::memcpy(&tau, &bits, 4);
        thresh = std::min(thresh, tau);  // both accept squared distances <= the threshold
      }
    }
    // 2. each row's k nearest within the bound; the global k closest pairs are among them
    int64_t slots = n * k;
    idx = Scratch((size_t)slots * 4, s);
    dd = Scratch((size_t)slots * 4, s);
    run_knn(searched, pts.as<float>(), n, k, thresh, nullptr, idx.as<int32_t>(), dd.as<float>(), searched->err, s);
    // 3. compact the filled slots in slot order, then sort them by (squared distance, row), stably
    Scratch flag((size_t)slots * 4, s), pos((size_t)slots * 4, s), total(4, s);
    unsigned sblocks = (unsigned)ceil_div(slots, PAIR_THREADS);
    THEA_LAUNCH(slot_flag_kernel, sblocks, PAIR_THREADS, 0, s, idx.as<int32_t>(), slots, flag.as<uint32_t>());
    exclusive_scan(flag.as<uint32_t>(), pos.as<uint32_t>(), slots, s);
    THEA_LAUNCH(slot_total_kernel, 1, 1, 0, s, flag.as<uint32_t>(), pos.as<uint32_t>(), slots, total.as<uint32_t>());
    uint32_t hm = 0;
    THEA_CUDA_CHECK(cudaMemcpyAsync(&hm, total.ptr, 4, cudaMemcpyDeviceToHost, s));
    THEA_CUDA_CHECK(cudaStreamSynchronize(s));
    m = hm;
    if (m > 0) {
      keys = Scratch((size_t)m * 8, s);
      vals = Scratch((size_t)m * 4, s);
      THEA_LAUNCH(pair_candidates_kernel, sblocks, PAIR_THREADS, 0, s, idx.as<int32_t>(), dd.as<float>(),
                  pos.as<uint32_t>(), slots, k, keys.as<unsigned long long>(), vals.as<uint32_t>());
      radix_sort_pairs(keys.as<uint64_t>(), vals.as<uint32_t>(), m, 64, s);
    }
  }
  THEA_LAUNCH(pair_take_kernel, 1, 32, 0, s, keys.as<unsigned long long>(), vals.as<uint32_t>(), idx.as<int32_t>(),
              dd.as<float>(), m, k, qi, ti, d2, count.as<unsigned>());
  unsigned hc = 0;
  THEA_CUDA_CHECK(cudaMemcpyAsync(&hc, count.ptr, 4, cudaMemcpyDeviceToHost, s));
  THEA_CUDA_CHECK(cudaStreamSynchronize(s));
  return (int64_t)hc;
}

}  // namespace thea
