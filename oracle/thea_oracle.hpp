// TEST INFRASTRUCTURE ONLY -- the CPU oracle for the spatial-query hot path.
//
// This file restates, in plain C++17 without Eigen, the CPU algorithms of Thea's spatial-query path so that the CUDA
// implementation can be checked against them. Only tests, the smoke check and the CPU-baseline legs of bench.py may
// load it; the product library never links it, and nothing here is a fallback for the GPU path.
//
// Parity status: PINNED to the reference's own code. The reference's BvhN, Triangle3, AxisAlignedBoxN, Random and Math
// sources are compiled in this build (oracle/Makefile, target `ref`) with oracle/ref_pin/eigen_subset.hpp standing in for
// Eigen, which is absent here; the reference mode below reproduces their outputs bit for bit (element indices,
// distances, closest points, hit times, normals, k-NN lists, random words: tests/test_oracle_pinned.py against
// tests/golden/reference_outputs.npz). What both share, and what remains assumed, is the order of Eigen's 3-term sums
// (next paragraph).
//
// Arithmetic order. The reference computes in FP32 (Real = float, Code/Source/NumericType.hpp:40) through Eigen
// fixed-size 3-vectors. Eigen reduces a 3-element sum (dot, squaredNorm) as e0 + (e1 + e2) when no SIMD packet fits the
// size (the x86 SSE/AVX case: redux_novec_unroller splits the range in halves). Every reduction below uses that order, and
// this file must be compiled with -ffp-contract=off so that no multiply-add is fused.
//
// Two result conventions are provided:
//   * reference mode: the reference's own kd-tree build and traversal, whose ties go to the element found first in
//     traversal order (strict-less replacement, Code/Source/Algorithms/BvhN.hpp:459-466);
//   * contract mode: the same per-element arithmetic, with ties broken by the lowest element index. This is the
//     structure-independent normalisation that the GPU path implements bit-exactly.
// Each function is templated on the scalar type; instantiating it with double gives the FP64 twin used for error reports.

#pragma once

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <limits>
#include <thread>
#include <vector>

namespace oracle {

//============================================================================================================================
// Vectors (Eigen fixed-size 3-vector semantics, Code/Source/MatVec.hpp:56)
//============================================================================================================================

template <class S> struct V3 {
  S x, y, z;
  V3() : x(0), y(0), z(0) {}
  V3(S a, S b, S c) : x(a), y(b), z(c) {}
  S operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
  S & operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  bool operator==(V3 const & o) const { return x == o.x && y == o.y && z == o.z; }
};

template <class S> inline V3<S> operator+(V3<S> const & a, V3<S> const & b) { return V3<S>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class S> inline V3<S> operator-(V3<S> const & a, V3<S> const & b) { return V3<S>(a.x - b.x, a.y - b.y, a.z - b.z); }
// scalar * vector and vector * scalar are both a per-component product
template <class S> inline V3<S> operator*(S s, V3<S> const & a) { return V3<S>(s * a.x, s * a.y, s * a.z); }
template <class S> inline V3<S> operator*(V3<S> const & a, S s) { return V3<S>(a.x * s, a.y * s, a.z * s); }
template <class S> inline V3<S> operator/(V3<S> const & a, S s) { return V3<S>(a.x / s, a.y / s, a.z / s); }

// Eigen redux order for 3 elements: e0 + (e1 + e2)
template <class S> inline S dot(V3<S> const & a, V3<S> const & b) { return a.x * b.x + (a.y * b.y + a.z * b.z); }
template <class S> inline S squaredNorm(V3<S> const & a) { return a.x * a.x + (a.y * a.y + a.z * a.z); }
template <class S> inline S norm(V3<S> const & a) { return std::sqrt(squaredNorm(a)); }
template <class S> inline V3<S> cross(V3<S> const & a, V3<S> const & b) {
  return V3<S>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
// MatrixBase::normalized(): divide by the norm only if the squared norm is positive
template <class S> inline V3<S> normalized(V3<S> const & a) {
  S z = squaredNorm(a);
  return z > S(0) ? a / std::sqrt(z) : a;
}
template <class S> inline V3<S> cwiseMin(V3<S> const & a, V3<S> const & b) {
  return V3<S>(std::min(a.x, b.x), std::min(a.y, b.y), std::min(a.z, b.z));
}
template <class S> inline V3<S> cwiseMax(V3<S> const & a, V3<S> const & b) {
  return V3<S>(std::max(a.x, b.x), std::max(a.y, b.y), std::max(a.z, b.z));
}
// Math::maxAbsAxis / maxAxis (Code/Source/MatrixUtil.hpp:84-115): first index of the maximum (Eigen visitor uses strict >)
template <class S> inline int maxAbsAxis(V3<S> const & v) {
  S a0 = std::fabs(v.x), a1 = std::fabs(v.y), a2 = std::fabs(v.z);
  int m = 0; S best = a0;
  if (a1 > best) { m = 1; best = a1; }
  if (a2 > best) { m = 2; }
  return m;
}
template <class S> inline int maxAxis(V3<S> const & v) {
  int m = 0; S best = v.x;
  if (v.y > best) { m = 1; best = v.y; }
  if (v.z > best) { m = 2; }
  return m;
}

template <class S> inline V3<S> load3(float const * p) { return V3<S>(S(p[0]), S(p[1]), S(p[2])); }

//============================================================================================================================
// Axis-aligned box (Code/Source/AxisAlignedBoxN.hpp)
//============================================================================================================================

template <class S> struct Box {
  V3<S> lo, hi;
  bool is_null = true;

  // merge(point) / merge(box): AxisAlignedBoxN.hpp:237-271
  void merge(V3<S> const & p) {
    if (is_null) { lo = hi = p; is_null = false; }
    else { lo = cwiseMin(lo, p); hi = cwiseMax(hi, p); }
  }
  void merge(Box const & b) {
    if (!b.is_null) {
      if (is_null) { lo = b.lo; hi = b.hi; is_null = false; }
      else { lo = cwiseMin(lo, b.lo); hi = cwiseMax(hi, b.hi); }
    }
  }
  // getCenter(): 0.5 * (hi + lo)
  V3<S> center() const { return S(0.5) * (hi + lo); }
  V3<S> extent() const { return hi - lo; }
  // scaleCentered(scale): AxisAlignedBoxN.hpp:316-325
  void scaleCentered(S s) {
    if (!is_null) {
      V3<S> c = center();
      lo = s * (lo - c) + c;
      hi = s * (hi - c) + c;
    }
  }
  // squaredDistance(box): AxisAlignedBoxN.hpp:429-442
  S squaredDistance(Box const & o) const {
    if (is_null || o.is_null) return S(0);
    V3<S> vmax = cwiseMin(hi, o.hi);
    V3<S> vmin = cwiseMax(lo, o.lo);
    V3<S> vdiff = vmin - vmax;
    vdiff = cwiseMax(vdiff, V3<S>(0, 0, 0));
    return squaredNorm(vdiff);
  }
  // squaredDistance(point): AxisAlignedBoxN.hpp:448-456
  S squaredDistance(V3<S> const & p) const {
    if (is_null) return S(0);
    V3<S> vmax = cwiseMin(p, hi);
    V3<S> vmin = cwiseMax(p, lo);
    return squaredNorm(vmin - vmax);
  }
};

// Math::eps(a, b) and fuzzyNe(a, 0) (Code/Source/Math.hpp:124-154)
template <class S> inline bool fuzzyNeZero(S a) {
  S const E = std::numeric_limits<S>::epsilon();
  if (std::isinf(a)) return !(a == S(0) || std::fabs(a) <= E);
  S larger = std::fabs(a);
  S tol = larger > S(1) ? larger * E : E;
  return !((a == S(0)) || std::fabs(a) <= tol);
}

// AxisAlignedBoxN::rayIntersection (...)::getTime (AxisAlignedBoxN.hpp:589-658): candidate-plane test; 0 if the origin is
// inside, -1 on a miss.
template <class S> S boxRayIntersectionTime(Box<S> const & b, V3<S> const & origin, V3<S> const & dir, S max_time) {
  if (b.is_null) return S(-1);
  if (max_time >= 0) {
    S ray_sqlen = squaredNorm(dir);
    S origin_sqdist = b.squaredDistance(origin);
    if (origin_sqdist > max_time * max_time * ray_sqlen) return S(-1);
  }
  V3<S> max_t(-1, -1, -1), location;
  bool inside = true;
  for (int i = 0; i < 3; ++i) {
    if (origin[i] < b.lo[i]) {
      location[i] = b.lo[i];
      inside = false;
      if (fuzzyNeZero(dir[i])) max_t[i] = (b.lo[i] - origin[i]) / dir[i];
    } else if (origin[i] > b.hi[i]) {
      location[i] = b.hi[i];
      inside = false;
      if (fuzzyNeZero(dir[i])) max_t[i] = (b.hi[i] - origin[i]) / dir[i];
    }
  }
  if (inside) return S(0);
  int which = 0;
  for (int i = 1; i < 3; ++i)
    if (max_t[i] > max_t[which]) which = i;
  if (max_t[which] < S(-0.5)) return S(-1);
  for (int i = 0; i < 3; ++i) {
    if (i != which) {
      location[i] = origin[i] + max_t[which] * dir[i];
      if (location[i] < b.lo[i] || location[i] > b.hi[i]) return S(-1);
    }
  }
  return max_t[which];
}

//============================================================================================================================
// Triangle (Code/Source/Triangle3.hpp, Code/Source/HyperplaneN.hpp, Code/Source/Hyperplane3.hpp)
//============================================================================================================================

template <class S> struct Tri {
  V3<S> v0, v1, v2;
  V3<S> normal;  // plane normal (unit), Hyperplane3.hpp:34-41
  S dist;        // plane offset: normal . v0
  int primary_axis;
  V3<S> edge01, edge02;
  S area;

  Tri() {}
  Tri(V3<S> a, V3<S> b, V3<S> c) : v0(a), v1(b), v2(c) { update(); }

  // TriangleN<3>::update(): Triangle3.hpp:143-155
  void update() {
    normal = normalized(cross(v1 - v0, v2 - v0));
    dist = dot(normal, v0);
    primary_axis = maxAbsAxis(normal);
    edge01 = v1 - v0;
    edge02 = v2 - v0;
    area = S(0.5) * std::fabs(dot(normal, cross(edge01, edge02)));
  }

  // getBounds(): Triangle3.hpp:215-219
  Box<S> bounds() const {
    Box<S> b;
    b.lo = cwiseMin(v0, cwiseMin(v1, v2));
    b.hi = cwiseMax(v0, cwiseMax(v1, v2));
    b.is_null = false;
    return b;
  }
};

// Triangle3Internal::closestPointOnLineSegment: Triangle3.hpp:1311-1338
template <class S>
V3<S> closestPointOnLineSegment(V3<S> const & v0, V3<S> const & v1, V3<S> const & dir, S len, V3<S> const & p) {
  V3<S> c = p - v0;
  S t = dot(dir, c);
  if (t <= S(0)) return v0;
  else if (t >= len) return v1;
  else return v0 + dir * t;
}

// Triangle3Internal::closestPointOnTrianglePerimeter: Triangle3.hpp:1342-1412
template <class S> V3<S> closestPointOnTrianglePerimeter(V3<S> const & v0, V3<S> const & v1, V3<S> const & v2,
                                                         V3<S> const & p) {
  V3<S> v[3] = {v0, v1, v2};
  V3<S> dir[3] = {v1 - v0, v2 - v1, v0 - v2};
  S len[3];
  for (int i = 0; i < 3; ++i) {
    len[i] = norm(dir[i]);
    dir[i] = dir[i] / len[i];
  }
  static int const next[3] = {1, 2, 0};
  V3<S> r[3];
  S d[3];
  for (int i = 0; i < 3; ++i) {
    r[i] = closestPointOnLineSegment(v[i], v[next[i]], dir[i], len[i], p);
    d[i] = squaredNorm(r[i] - p);
  }
  int e;
  if (d[0] < d[1]) e = (d[0] < d[2]) ? 0 : 2;
  else e = (d[1] < d[2]) ? 1 : 2;
  return r[e];
}

// Triangle3Internal::isPointInsideTriangle: Triangle3.hpp:1416-1462
template <class S>
bool isPointInsideTriangle(V3<S> const & v0, V3<S> const & v1, V3<S> const & v2, int primary_axis, V3<S> const & p) {
  int i, j;
  switch (primary_axis) {
    case 1: i = 2; j = 0; break;
    case 2: i = 0; j = 1; break;
    default: i = 1; j = 2;
  }
  auto area2 = [i, j](V3<S> const & d, V3<S> const & e, V3<S> const & f) {
    return (e[i] - d[i]) * (f[j] - d[j]) - (f[i] - d[i]) * (e[j] - d[j]);
  };
  S area = area2(v0, v1, v2);
  if (area == S(0)) return v0 == p;
  S inv_area = S(1) / area;
  S b0 = area2(p, v1, v2) * inv_area;
  if ((b0 < S(0)) || (b0 > S(1))) return false;
  S b1 = area2(v0, p, v2) * inv_area;
  if ((b1 < S(0)) || (b1 > S(1))) return false;
  S b2 = S(1) - b0 - b1;
  return (b2 >= S(0)) && (b2 <= S(1));
}

// TriangleN<3>::closestPoint: Triangle3.hpp:294-304 with HyperplaneN::closestPoint (HyperplaneN.hpp:145-160)
template <class S> V3<S> triangleClosestPoint(Tri<S> const & t, V3<S> const & p) {
  S sd = dot(p, t.normal) - t.dist;
  V3<S> proj = p - sd * t.normal;
  if (isPointInsideTriangle(t.v0, t.v1, t.v2, t.primary_axis, proj)) return proj;
  return closestPointOnTrianglePerimeter(t.v0, t.v1, t.v2, p);
}

// MetricL2Impl<Triangle, Point>::closestPoints: MetricL2.hpp:209-215 -- squared distance, closest point on the triangle
template <class S> S triangleClosestPoints(Tri<S> const & t, V3<S> const & p, V3<S> & cp) {
  cp = triangleClosestPoint(t, p);
  return squaredNorm(cp - p);
}

// Triangle3Internal::rayTriangleIntersectionTime: Triangle3.hpp:1466-1524 (Eberly). Returns -1 on a miss.
template <class S>
S rayTriangleIntersectionTime(V3<S> const & origin, V3<S> const & dir, V3<S> const & v0, V3<S> const & e01,
                              V3<S> const & e02) {
  S const EPS = std::numeric_limits<S>::epsilon();
  V3<S> diff = origin - v0;
  V3<S> n = cross(e01, e02);
  S DdN = dot(dir, n);
  int sign;
  if (DdN > EPS) sign = 1;
  else if (DdN < -EPS) { sign = -1; DdN = -DdN; }
  else return S(-1);
  S DdQxE2 = S(sign) * dot(dir, cross(diff, e02));
  if (DdQxE2 >= S(0)) {
    S DdE1xQ = S(sign) * dot(dir, cross(e01, diff));
    if (DdE1xQ >= S(0)) {
      if (DdQxE2 + DdE1xQ <= DdN) {
        S QdN = S(-sign) * dot(diff, n);
        if (QdN >= S(0)) return QdN / DdN;
      }
    }
  }
  return S(-1);
}

//============================================================================================================================
// Triangle-triangle distance: TriangleN<3>::squaredDistance(other, this_pt, other_pt) (Triangle3.hpp:314-400, after
// Ericson, "Real-Time Collision Detection"), with Moller's intersection test that also returns the line of intersection
// (Triangle3Internal::tri_tri_intersect_with_isectline, Triangle3.hpp:1117-1290, coplanar_tri_tri :730-776) and the
// segment-segment closest points of Internal::closestPtSegmentSegment (LineSegmentN.hpp:262-340).
//
// Arithmetic order: the intersection test works on raw coordinate arrays with the reference's C expressions, so its
// three-term dot products add left to right ((a0 b0 + a1 b1) + a2 b2); the segment-segment and plane-projection steps
// use Eigen vectors (the e0 + (e1 + e2) reduction of dot() above).
//============================================================================================================================

namespace tritri {

template <class S> inline S dotLR(S const * a, S const * b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
template <class S> inline void crossA(S * d, S const * a, S const * b) {
  d[0] = a[1] * b[2] - a[2] * b[1];
  d[1] = a[2] * b[0] - a[0] * b[2];
  d[2] = a[0] * b[1] - a[1] * b[0];
}
template <class S> inline void subA(S * d, S const * a, S const * b) {
  d[0] = a[0] - b[0]; d[1] = a[1] - b[1]; d[2] = a[2] - b[2];
}

// EDGE_EDGE_TEST (Triangle3.hpp:674-693): edge (v0, v0 + A) against edge (u0, u1) in the projection (i0, i1)
template <class S>
inline bool edgeEdge(S Ax, S Ay, S const * v0, S const * u0, S const * u1, int i0, int i1) {
  S Bx = u0[i0] - u1[i0], By = u0[i1] - u1[i1];
  S Cx = v0[i0] - u0[i0], Cy = v0[i1] - u0[i1];
  S f = Ay * Bx - Ax * By;
  S d = By * Cx - Bx * Cy;
  if ((f > 0 && d >= 0 && d <= f) || (f < 0 && d <= 0 && d >= f)) {
    S e = Ax * Cy - Ay * Cx;
    if (f > 0) {
      if (e >= 0 && e <= f) return true;
    } else {
      if (e <= 0 && e >= f) return true;
    }
  }
  return false;
}

// EDGE_AGAINST_TRI_EDGES (Triangle3.hpp:695-707)
template <class S>
inline bool edgeAgainstTri(S const * v0, S const * v1, S const * u0, S const * u1, S const * u2, int i0, int i1) {
  S Ax = v1[i0] - v0[i0], Ay = v1[i1] - v0[i1];
  return edgeEdge(Ax, Ay, v0, u0, u1, i0, i1) || edgeEdge(Ax, Ay, v0, u1, u2, i0, i1) ||
         edgeEdge(Ax, Ay, v0, u2, u0, i0, i1);
}

// POINT_IN_TRI (Triangle3.hpp:709-728)
template <class S> inline bool pointInTri(S const * v0, S const * u0, S const * u1, S const * u2, int i0, int i1) {
  S a = u1[i1] - u0[i1], b = -(u1[i0] - u0[i0]);
  S c = -a * u0[i0] - b * u0[i1];
  S d0 = a * v0[i0] + b * v0[i1] + c;
  a = u2[i1] - u1[i1]; b = -(u2[i0] - u1[i0]);
  c = -a * u1[i0] - b * u1[i1];
  S d1 = a * v0[i0] + b * v0[i1] + c;
  a = u0[i1] - u2[i1]; b = -(u0[i0] - u2[i0]);
  c = -a * u2[i0] - b * u2[i1];
  S d2 = a * v0[i0] + b * v0[i1] + c;
  return d0 * d1 > 0 && d0 * d2 > 0;
}

// coplanar_tri_tri (Triangle3.hpp:730-776)
template <class S>
bool coplanar(S const * N, S const * v0, S const * v1, S const * v2, S const * u0, S const * u1, S const * u2) {
  S A0 = std::fabs(N[0]), A1 = std::fabs(N[1]), A2 = std::fabs(N[2]);
  int i0, i1;
  if (A0 > A1) {
    if (A0 > A2) { i0 = 1; i1 = 2; }
    else { i0 = 0; i1 = 1; }
  } else {
    if (A2 > A1) { i0 = 0; i1 = 1; }
    else { i0 = 0; i1 = 2; }
  }
  if (edgeAgainstTri(v0, v1, u0, u1, u2, i0, i1)) return true;
  if (edgeAgainstTri(v1, v2, u0, u1, u2, i0, i1)) return true;
  if (edgeAgainstTri(v2, v0, u0, u1, u2, i0, i1)) return true;
  if (pointInTri(v0, u0, u1, u2, i0, i1)) return true;
  if (pointInTri(u0, v0, v1, v2, i0, i1)) return true;
  return false;
}

// isect2 (Triangle3.hpp:1023-1039)
template <class S>
inline void isect2(S const * x0, S const * x1, S const * x2, S vv0, S vv1, S vv2, S d0, S d1, S d2, S & is0, S & is1,
                   S * p0, S * p1) {
  S tmp = d0 / (d0 - d1);
  S diff[3];
  is0 = vv0 + (vv1 - vv0) * tmp;
  subA(diff, x1, x0);
  for (int k = 0; k < 3; ++k) diff[k] = tmp * diff[k];
  for (int k = 0; k < 3; ++k) p0[k] = diff[k] + x0[k];
  tmp = d0 / (d0 - d2);
  is1 = vv0 + (vv2 - vv0) * tmp;
  subA(diff, x2, x0);
  for (int k = 0; k < 3; ++k) diff[k] = tmp * diff[k];
  for (int k = 0; k < 3; ++k) p1[k] = x0[k] + diff[k];
}

// compute_intervals_isectline (Triangle3.hpp:1041-1077); true when the triangles are coplanar
template <class S>
inline bool intervals(S const * x0, S const * x1, S const * x2, S vv0, S vv1, S vv2, S d0, S d1, S d2, S d0d1, S d0d2,
                      S & is0, S & is1, S * p0, S * p1) {
  if (d0d1 > 0) isect2(x2, x0, x1, vv2, vv0, vv1, d2, d0, d1, is0, is1, p0, p1);
  else if (d0d2 > 0) isect2(x1, x0, x2, vv1, vv0, vv2, d1, d0, d2, is0, is1, p0, p1);
  else if (d1 * d2 > 0 || d0 != 0) isect2(x0, x1, x2, vv0, vv1, vv2, d0, d1, d2, is0, is1, p0, p1);
  else if (d1 != 0) isect2(x1, x0, x2, vv1, vv0, vv2, d1, d0, d2, is0, is1, p0, p1);
  else if (d2 != 0) isect2(x2, x0, x1, vv2, vv0, vv1, d2, d0, d1, is0, is1, p0, p1);
  else return true;
  return false;
}

// tri_tri_intersect_with_isectline (Triangle3.hpp:1117-1290): 1 if the triangles intersect; *coplanar_out tells whether
// they are coplanar, and if not, pt1 and pt2 are the ends of the intersection segment
template <class S>
int intersect(S const * V0, S const * V1, S const * V2, S const * U0, S const * U1, S const * U2, int & coplanar_out,
              S * pt1, S * pt2) {
  S const EPS = std::numeric_limits<S>::epsilon();
  S E1[3], E2[3], N1[3], N2[3], D[3];
  S isA[2] = {0, 0}, isB[2] = {0, 0};
  S pA1[3] = {0, 0, 0}, pA2[3] = {0, 0, 0}, pB1[3] = {0, 0, 0}, pB2[3] = {0, 0, 0};
  subA(E1, V1, V0);
  subA(E2, V2, V0);
  crossA(N1, E1, E2);
  S d1 = -dotLR(N1, V0);
  S du0 = dotLR(N1, U0) + d1, du1 = dotLR(N1, U1) + d1, du2 = dotLR(N1, U2) + d1;
  if (std::fabs(du0) < EPS) du0 = 0;
  if (std::fabs(du1) < EPS) du1 = 0;
  if (std::fabs(du2) < EPS) du2 = 0;
  S du0du1 = du0 * du1, du0du2 = du0 * du2;
  if (du0du1 > 0 && du0du2 > 0) return 0;
  subA(E1, U1, U0);
  subA(E2, U2, U0);
  crossA(N2, E1, E2);
  S d2 = -dotLR(N2, U0);
  S dv0 = dotLR(N2, V0) + d2, dv1 = dotLR(N2, V1) + d2, dv2 = dotLR(N2, V2) + d2;
  if (std::fabs(dv0) < EPS) dv0 = 0;
  if (std::fabs(dv1) < EPS) dv1 = 0;
  if (std::fabs(dv2) < EPS) dv2 = 0;
  S dv0dv1 = dv0 * dv1, dv0dv2 = dv0 * dv2;
  if (dv0dv1 > 0 && dv0dv2 > 0) return 0;
  crossA(D, N1, N2);
  S mx = std::fabs(D[0]);
  int index = 0;
  S b = std::fabs(D[1]), c = std::fabs(D[2]);
  if (b > mx) { mx = b; index = 1; }
  if (c > mx) { mx = c; index = 2; }
  S vp0 = V0[index], vp1 = V1[index], vp2 = V2[index];
  S up0 = U0[index], up1 = U1[index], up2 = U2[index];
  coplanar_out = intervals(V0, V1, V2, vp0, vp1, vp2, dv0, dv1, dv2, dv0dv1, dv0dv2, isA[0], isA[1], pA1, pA2) ? 1 : 0;
  if (coplanar_out) return coplanar(N1, V0, V1, V2, U0, U1, U2) ? 1 : 0;
  intervals(U0, U1, U2, up0, up1, up2, du0, du1, du2, du0du1, du0du2, isB[0], isB[1], pB1, pB2);
  int smallest1 = 0, smallest2 = 0;
  if (isA[0] > isA[1]) { std::swap(isA[0], isA[1]); smallest1 = 1; }
  if (isB[0] > isB[1]) { std::swap(isB[0], isB[1]); smallest2 = 1; }
  if (isA[1] < isB[0] || isB[1] < isA[0]) return 0;
  S const * a_lo = smallest1 == 0 ? pA1 : pA2;  // end of A's interval at isA[0]
  S const * a_hi = smallest1 == 0 ? pA2 : pA1;
  S const * b_lo = smallest2 == 0 ? pB1 : pB2;
  S const * b_hi = smallest2 == 0 ? pB2 : pB1;
  if (isB[0] < isA[0]) {
    std::copy(a_lo, a_lo + 3, pt1);
    if (isB[1] < isA[1]) std::copy(b_hi, b_hi + 3, pt2);
    else std::copy(a_hi, a_hi + 3, pt2);
  } else {
    std::copy(b_lo, b_lo + 3, pt1);
    if (isB[1] > isA[1]) std::copy(a_hi, a_hi + 3, pt2);
    else std::copy(b_hi, b_hi + 3, pt2);
  }
  return 1;
}

// Math::fuzzyEq(a, 0) (Math.hpp:131-148)
template <class S> inline bool fuzzyZero(S a) { return !fuzzyNeZero(a); }

// Math::clamp (Math.hpp:249)
template <class S> inline S clamp01(S x) { return x < S(0) ? S(0) : (x > S(1) ? S(1) : x); }

// Internal::closestPtSegmentSegment for two segments (LineSegmentN.hpp:262-340)
template <class S>
S segmentSegment(V3<S> const & p1, V3<S> const & q1, V3<S> const & p2, V3<S> const & q2, V3<S> & c1, V3<S> & c2) {
  V3<S> d1 = q1 - p1, d2 = q2 - p2, r = p1 - p2;
  S a = squaredNorm(d1), e = squaredNorm(d2), f = dot(d2, r);
  S s, t;
  if (fuzzyZero(a)) {
    if (fuzzyZero(e)) {
      c1 = p1;
      c2 = p2;
      return dot(c1 - c2, c1 - c2);
    }
    s = 0;
    t = clamp01(f / e);
  } else {
    S c = dot(d1, r);
    if (fuzzyZero(e)) {
      t = 0;
      s = clamp01(-c / a);
    } else {
      S b = dot(d1, d2);
      S denom = a * e - b * b;
      s = denom != 0 ? clamp01((b * f - c * e) / denom) : S(0);
      t = (b * s + f) / e;
      if (t < 0) {
        t = 0;
        s = clamp01(-c / a);
      } else if (t > 1) {
        t = 1;
        s = clamp01((b - c) / a);
      }
    }
  }
  c1 = p1 + s * d1;
  c2 = p2 + t * d2;
  return squaredNorm(c1 - c2);
}

}  // namespace tritri

// TriangleN<3>::squaredDistance(other, this_pt, other_pt): Triangle3.hpp:314-400. `a` is the triangle whose method runs
// ("this"); pa and pb receive the closest points on a and b.
template <class S> S triangleTriangleSquaredDistance(Tri<S> const & a, Tri<S> const & b, V3<S> & pa, V3<S> & pb) {
  V3<S> c1(0, 0, 0), c2(0, 0, 0);
  S best = std::numeric_limits<S>::max();
  S A0[3] = {a.v0.x, a.v0.y, a.v0.z}, A1[3] = {a.v1.x, a.v1.y, a.v1.z}, A2[3] = {a.v2.x, a.v2.y, a.v2.z};
  S B0[3] = {b.v0.x, b.v0.y, b.v0.z}, B1[3] = {b.v1.x, b.v1.y, b.v1.z}, B2[3] = {b.v2.x, b.v2.y, b.v2.z};
  int cop = 0;
  S i1[3] = {0, 0, 0}, i2[3] = {0, 0, 0};
  if (tritri::intersect(A0, A1, A2, B0, B1, B2, cop, i1, i2)) {
    if (cop) {
      // centroids: (v0 + v1 + v2) / 3 (Triangle3.hpp:149)
      V3<S> ca = (a.v0 + a.v1 + a.v2) / S(3), cb = (b.v0 + b.v1 + b.v2) / S(3);
      c1 = c2 = S(0.5) * (ca + cb);
    } else {
      // LineSegmentN(isectpt1, isectpt2) keeps (point, direction); getPoint(t) = point + t * direction
      V3<S> pt(i1[0], i1[1], i1[2]), dir = V3<S>(i2[0], i2[1], i2[2]) - pt;
      c1 = c2 = S(0.5) * ((pt + S(0) * dir) + (pt + S(1) * dir));
    }
    best = 0;
  } else {
    V3<S> av[3] = {a.v0, a.v1, a.v2}, bv[3] = {b.v0, b.v1, b.v2};
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        V3<S> p, q;
        S d2 = tritri::segmentSegment(av[i], av[(i + 1) % 3], bv[j], bv[(j + 1) % 3], p, q);
        if (d2 < best) { best = d2; c1 = p; c2 = q; }
      }
    for (int i = 0; i < 3; ++i) {  // vertices of b projected into a
      V3<S> q = bv[i];
      V3<S> p = q - (dot(q, a.normal) - a.dist) * a.normal;
      if (isPointInsideTriangle(a.v0, a.v1, a.v2, a.primary_axis, p)) {
        S d2 = squaredNorm(p - q);
        if (d2 < best) { best = d2; c1 = p; c2 = q; }
      }
    }
    for (int i = 0; i < 3; ++i) {  // vertices of a projected into b
      V3<S> p = av[i];
      V3<S> q = p - (dot(p, b.normal) - b.dist) * b.normal;
      if (isPointInsideTriangle(b.v0, b.v1, b.v2, b.primary_axis, q)) {
        S d2 = squaredNorm(p - q);
        if (d2 < best) { best = d2; c1 = p; c2 = q; }
      }
    }
  }
  pa = c1;
  pb = c2;
  return best;
}

// TriangleN<3>::rayIntersection time: Triangle3.hpp:542-552 (hit if t >= 0 and (max_time < 0 or t <= max_time))
template <class S> S triangleRayTime(Tri<S> const & t, V3<S> const & o, V3<S> const & d, S max_time) {
  S time = rayTriangleIntersectionTime(o, d, t.v0, t.edge01, t.edge02);
  if (time >= S(0) && (max_time < S(0) || time <= max_time)) return time;
  return S(-1);
}

//============================================================================================================================
// Median-split kd-tree (BvhN::initTree / createKdTree, BvhN.hpp:1366-1525)
//============================================================================================================================

// Math::treeDepth: Code/Source/Math.cpp:23-36
inline int64_t treeDepth(int64_t n, int max_leaf, float max_child_fraction) {
  if (n <= 0) return 0;
  // the fraction is a Real (float), so the reference takes a float logarithm here
  double log_inv_mcf = -(double)std::log(max_child_fraction);
  int64_t d = (int64_t)std::ceil(std::log(n / (double)max_leaf) / log_inv_mcf);
  return d < 0 ? 0 : d;
}

template <class S> struct KdNode {
  int64_t depth = 0;
  Box<S> bounds;
  int64_t first = 0, count = 0;  // element index range in the tree's index array
  int64_t child[2] = {-1, -1};
  bool isLeaf() const { return child[0] < 0 && child[1] < 0; }
};

// A kd-tree over elements that expose bounds() (triangles) or are points. ElemBounds(i) gives the element's box.
template <class S> struct KdTree {
  std::vector<KdNode<S>> nodes;
  std::vector<int64_t> index;  // element indices; each node owns a contiguous range
  int64_t max_depth = 0;
  int64_t max_leaf = 5;

  // initTree + createKdTree. bounds_of(i) returns the element box, center_of(i) the split key (BoundedTraitsN::getCenter).
  template <class BoundsF, class CenterF>
  void build(int64_t n, BoundsF bounds_of, CenterF center_of, int64_t max_leaf_ = -1) {
    nodes.clear();
    index.resize((size_t)n);
    if (n <= 0) return;
    max_leaf = max_leaf_ <= 0 ? 5 : max_leaf_;
    max_depth = treeDepth(n, (int)max_leaf, 0.5f);
    for (int64_t i = 0; i < n; ++i) index[(size_t)i] = i;
    nodes.reserve((size_t)(4 * n / max_leaf + 16));
    KdNode<S> root;
    root.depth = 0; root.first = 0; root.count = n;
    for (int64_t i = 0; i < n; ++i) root.bounds.merge(bounds_of(i));
    nodes.push_back(root);
    recurse(0, bounds_of, center_of);
    nodes[0].bounds.scaleCentered(S(1.05f));  // BOUNDS_EXPANSION_FACTOR, BvhN.hpp:1437, 2458
  }

  template <class BoundsF, class CenterF> void recurse(int64_t ni, BoundsF & bounds_of, CenterF & center_of) {
    KdNode<S> start = nodes[(size_t)ni];
    if (start.depth >= max_depth || start.count <= max_leaf) return;
    int coord = maxAxis(start.bounds.extent());
    int64_t mid = start.count / 2;
    int64_t * base = index.data() + start.first;
    std::nth_element(base, base + mid, base + start.count, [&](int64_t a, int64_t b) {
      return center_of(a)[coord] < center_of(b)[coord];
    });
    for (int c = 0; c < 2; ++c) {
      KdNode<S> child;
      child.depth = start.depth + 1;
      int64_t b = (c == 0) ? 0 : start.count - mid;
      int64_t e = (c == 0) ? start.count - mid : start.count;
      child.first = start.first + b;
      child.count = e - b;
      for (int64_t k = child.first; k < child.first + child.count; ++k) child.bounds.merge(bounds_of(index[(size_t)k]));
      int64_t ci = (int64_t)nodes.size();
      nodes.push_back(child);
      nodes[(size_t)ni].child[c] = ci;
      recurse(ci, bounds_of, center_of);
      nodes[(size_t)ci].bounds.scaleCentered(S(1.05f));
    }
  }
};

// distanceLessThan: BvhN.hpp:178-181 (negative = "none", greater than any non-negative value)
template <class U, class V> inline bool distanceLessThan(U lhs, V rhs) { return (lhs >= 0 && (rhs < 0 || lhs < rhs)); }

// ChildDistanceArray ordering for two children (BoundedSortedArrayN<2, NodeDistance>::insert, stable on ties)
template <class D> inline void orderTwo(D d0, D d1, int & first, int & second) {
  if (distanceLessThan(d1, d0)) { first = 1; second = 0; }
  else { first = 0; second = 1; }
}

//============================================================================================================================
// Mesh index: triangles + kd-tree
//============================================================================================================================

template <class S> struct MeshIndex {
  std::vector<Tri<S>> tris;
  KdTree<S> tree;

  void init(float const * V, int64_t nv, int32_t const * F, int64_t nf, int64_t max_leaf = -1) {
    (void)nv;
    tris.resize((size_t)nf);
    for (int64_t f = 0; f < nf; ++f)
      tris[(size_t)f] = Tri<S>(load3<S>(V + 3 * (int64_t)F[3 * f]), load3<S>(V + 3 * (int64_t)F[3 * f + 1]),
                               load3<S>(V + 3 * (int64_t)F[3 * f + 2]));
    std::vector<Box<S>> boxes((size_t)nf);
    std::vector<V3<S>> centers((size_t)nf);
    // split key: BoundedTraitsN<TriangleN>::getCenter = the cached centroid (v0 + v1 + v2) / 3 (BoundedTraitsN.hpp:219,
    // Triangle3.hpp:149), not the box centre
    for (size_t f = 0; f < (size_t)nf; ++f) {
      boxes[f] = tris[f].bounds();
      centers[f] = (tris[f].v0 + tris[f].v1 + tris[f].v2) / S(3);
    }
    tree.build(nf, [&](int64_t i) -> Box<S> const & { return boxes[(size_t)i]; },
               [&](int64_t i) -> V3<S> const & { return centers[(size_t)i]; }, max_leaf);
  }

  // ---- closest point, reference mode (closestElement -> closestPair -> processNeighbors, BvhN.hpp:1050-1114,1868-1893,
  //      2038-2089). Returns the element index or -1; mad is the squared distance as stored by the reference (double).
  // BvhN::closestPair with a distance bound (BvhN.hpp:1093-1107): a query farther from the root box than the bound
  // (squared distances, FP32 box distance compared in double) has no element; otherwise accelerationBound returns the
  // bound itself, which is loosened by max(0.001 |root box extent|, 100 eps) before the search. Returns the loosened
  // squared bound, or -2 when the query is cut, -1 when unbounded.
  double closestBound(Box<S> const & qb, double dist_bound) const {
    if (dist_bound < 0) return -1;
    double lb = (double)qb.squaredDistance(tree.nodes[0].bounds);
    if (lb >= 0 && lb > dist_bound * dist_bound) return -2;
    double fudge = std::max((double)(0.001 * (double)norm(tree.nodes[0].bounds.extent())),
                            (double)(S(100) * std::numeric_limits<S>::epsilon()));
    double b = dist_bound + fudge;
    return b * b;
  }

  int64_t closestRef(V3<S> const & q, double dist_bound, double & mad_out, V3<S> & cp_out) const {
    if (tree.nodes.empty()) return -1;
    Box<S> qb; qb.merge(q);
    double mon_bound = closestBound(qb, dist_bound);
    if (mon_bound == -2) return -1;
    int64_t best_idx = -1;
    double best_mad = mon_bound >= 0 ? mon_bound : -1;
    V3<S> best_cp;
    closestRefRec(0, q, qb, best_idx, best_mad, best_cp);
    if (best_idx >= 0) { mad_out = best_mad; cp_out = best_cp; }
    return best_idx;
  }

  void closestRefRec(int64_t ni, V3<S> const & q, Box<S> const & qb, int64_t & best_idx, double & best_mad,
                     V3<S> & best_cp) const {
    KdNode<S> const & n = tree.nodes[(size_t)ni];
    if (n.isLeaf()) {
      for (int64_t k = n.first; k < n.first + n.count; ++k) {
        int64_t idx = tree.index[(size_t)k];
        V3<S> cp;
        double mad = (double)triangleClosestPoints(tris[(size_t)idx], q, cp);
        // allows(NeighborPair(-1, -1, mad)) then operator(): replace on strict less (BvhN.hpp:451-466)
        if (mad < 0 || best_mad < 0 || mad < best_mad) {
          if (best_mad < 0 || mad < best_mad) { best_mad = mad; best_idx = idx; best_cp = cp; }
        }
      }
      return;
    }
    double d[2];
    for (int c = 0; c < 2; ++c) d[c] = (double)qb.squaredDistance(tree.nodes[(size_t)n.child[c]].bounds);
    int o[2];
    orderTwo(d[0], d[1], o[0], o[1]);
    for (int s = 0; s < 2; ++s) {
      double cd = d[o[s]];
      if (cd < 0 || best_mad < 0 || cd < best_mad) closestRefRec(n.child[o[s]], q, qb, best_idx, best_mad, best_cp);
    }
  }

  // ---- closest point, contract mode: lowest index among equal squared distances; elements accepted only if
  //      (double)d2 < dist_bound^2 when dist_bound >= 0 (the reference's strict bound test).
  int64_t closestContract(V3<S> const & q, double dist_bound, S & best_d2, V3<S> & cp_out) const {
    if (tree.nodes.empty()) return -1;
    Box<S> qb; qb.merge(q);
    double mon_bound = closestBound(qb, dist_bound);
    if (mon_bound == -2) return -1;
    int64_t best_idx = -1;
    S bd2 = std::numeric_limits<S>::infinity();
    V3<S> bcp;
    std::vector<int64_t> stack;
    stack.push_back(0);
    while (!stack.empty()) {
      int64_t ni = stack.back(); stack.pop_back();
      KdNode<S> const & n = tree.nodes[(size_t)ni];
      S bd = qb.squaredDistance(n.bounds);
      if (best_idx >= 0 && bd > bd2) continue;
      if (mon_bound >= 0 && (double)bd > mon_bound) continue;
      if (n.isLeaf()) {
        for (int64_t k = n.first; k < n.first + n.count; ++k) {
          int64_t idx = tree.index[(size_t)k];
          V3<S> cp;
          S d2 = triangleClosestPoints(tris[(size_t)idx], q, cp);
          if (!(d2 == d2)) continue;  // a NaN distance (coincident vertices) is never selected
          if (mon_bound >= 0 && !((double)d2 < mon_bound)) continue;
          if (best_idx < 0 || d2 < bd2 || (d2 == bd2 && idx < best_idx)) { bd2 = d2; best_idx = idx; bcp = cp; }
        }
      } else {
        // nearer child on top, so the bound tightens early (the result does not depend on the order: every element
        // whose box is not farther than the best is tested)
        S c0 = qb.squaredDistance(tree.nodes[(size_t)n.child[0]].bounds);
        S c1 = qb.squaredDistance(tree.nodes[(size_t)n.child[1]].bounds);
        if (c1 < c0) {
          stack.push_back(n.child[0]);
          stack.push_back(n.child[1]);
        } else {
          stack.push_back(n.child[1]);
          stack.push_back(n.child[0]);
        }
      }
    }
    if (best_idx >= 0) { best_d2 = bd2; cp_out = bcp; }
    return best_idx;
  }

  // ---- nearest element to a query triangle, contract mode: smallest squared triangle-triangle distance computed with
  //      the element as "this" (TriangleN::squaredDistance, Triangle3.hpp:314-400), lowest index among ties; only
  //      distances with (double)d2 < dist_bound^2 when dist_bound >= 0. Node boxes (padded by the build) prune by the
  //      box-box distance (AxisAlignedBoxN::squaredDistance, AxisAlignedBoxN.hpp:429-442).
  int64_t closestTriangleContract(Tri<S> const & q, double dist_bound, S & best_d2) const {
    if (tree.nodes.empty()) return -1;
    Box<S> qb = q.bounds();
    double mon_bound = dist_bound >= 0 ? dist_bound * dist_bound : -1;
    int64_t best_idx = -1;
    S bd2 = std::numeric_limits<S>::infinity();
    std::vector<int64_t> stack;
    stack.push_back(0);
    while (!stack.empty()) {
      int64_t ni = stack.back(); stack.pop_back();
      KdNode<S> const & n = tree.nodes[(size_t)ni];
      S bd = qb.squaredDistance(n.bounds);
      if (best_idx >= 0 && bd > bd2) continue;
      if (mon_bound >= 0 && (double)bd > mon_bound) continue;
      if (n.isLeaf()) {
        for (int64_t k = n.first; k < n.first + n.count; ++k) {
          int64_t idx = tree.index[(size_t)k];
          V3<S> pa, pb;
          S d2 = triangleTriangleSquaredDistance(tris[(size_t)idx], q, pa, pb);
          if (!(d2 == d2)) continue;
          if (mon_bound >= 0 && !((double)d2 < mon_bound)) continue;
          if (best_idx < 0 || d2 < bd2 || (d2 == bd2 && idx < best_idx)) { bd2 = d2; best_idx = idx; }
        }
      } else {
        S c0 = qb.squaredDistance(tree.nodes[(size_t)n.child[0]].bounds);
        S c1 = qb.squaredDistance(tree.nodes[(size_t)n.child[1]].bounds);
        if (c1 < c0) {
          stack.push_back(n.child[0]);
          stack.push_back(n.child[1]);
        } else {
          stack.push_back(n.child[1]);
          stack.push_back(n.child[0]);
        }
      }
    }
    if (best_idx >= 0) best_d2 = bd2;
    return best_idx;
  }

  // ---- ray first hit, reference mode (rayStructureIntersection, BvhN.hpp:1292-1316, 2241-2291)
  struct RayHit { S t; int64_t idx; };

  RayHit rayRef(V3<S> const & o, V3<S> const & d, S max_time) const {
    RayHit none{S(-1), -1};
    if (tree.nodes.empty()) return none;
    if (!(boxRayIntersectionTime(tree.nodes[0].bounds, o, d, max_time) > S(-0.5))) return none;
    return rayRefRec(0, o, d, max_time);
  }

  RayHit rayRefRec(int64_t ni, V3<S> const & o, V3<S> const & d, S max_time) const {
    KdNode<S> const & n = tree.nodes[(size_t)ni];
    RayHit best{max_time, -1};
    bool found = false;
    if (n.isLeaf()) {
      for (int64_t k = n.first; k < n.first + n.count; ++k) {
        int64_t idx = tree.index[(size_t)k];
        S t = triangleRayTime(tris[(size_t)idx], o, d, best.t);
        if (distanceLessThan(t, best.t)) { best.t = t; best.idx = idx; found = true; }
      }
      return found ? best : RayHit{S(-1), -1};
    }
    S bt[2];
    for (int c = 0; c < 2; ++c) bt[c] = boxRayIntersectionTime(tree.nodes[(size_t)n.child[c]].bounds, o, d, max_time);
    int ord[2];
    orderTwo(bt[0], bt[1], ord[0], ord[1]);
    for (int s = 0; s < 2; ++s) {
      if (distanceLessThan(bt[ord[s]], best.t)) {
        RayHit h = rayRefRec(n.child[ord[s]], o, d, best.t);
        if (distanceLessThan(h.t, best.t)) { best = h; found = true; }
      }
    }
    return found ? best : RayHit{S(-1), -1};
  }
};

// Conservative slab test used only by contract-mode traversal (returns entry time clamped at 0, or -1 on a miss). The
// box is widened by a relative margin so that no triangle hit inside it can be rejected by rounding.
template <class S> S slabEntry(Box<S> const & b, V3<S> const & o, V3<S> const & d) {
  S tmin = S(0), tmax = std::numeric_limits<S>::infinity();
  for (int i = 0; i < 3; ++i) {
    S pad = (std::fabs(b.lo[i]) + std::fabs(b.hi[i]) + (b.hi[i] - b.lo[i])) * S(1e-5) + S(1e-30);
    S lo = b.lo[i] - pad, hi = b.hi[i] + pad;
    if (d[i] == S(0)) {
      if (o[i] < lo || o[i] > hi) return S(-1);
      continue;
    }
    S t0 = (lo - o[i]) / d[i], t1 = (hi - o[i]) / d[i];
    if (t0 > t1) std::swap(t0, t1);
    tmin = std::max(tmin, t0);
    tmax = std::min(tmax, t1);
    if (tmin > tmax) return S(-1);
  }
  return tmin;
}

// ---- ray first hit, contract mode: smallest valid t, lowest index among equal t
template <class S> typename MeshIndex<S>::RayHit rayContract(MeshIndex<S> const & m, V3<S> const & o, V3<S> const & d,
                                                             S max_time) {
  typename MeshIndex<S>::RayHit best{S(-1), -1};
  if (m.tree.nodes.empty()) return best;
  std::vector<int64_t> stack;
  stack.push_back(0);
  while (!stack.empty()) {
    int64_t ni = stack.back(); stack.pop_back();
    KdNode<S> const & n = m.tree.nodes[(size_t)ni];
    S te = slabEntry(n.bounds, o, d);
    if (te < S(0)) continue;
    if (best.idx >= 0 && te > best.t * (S(1) + S(1e-5))) continue;
    if (max_time >= S(0) && te > max_time * (S(1) + S(1e-5))) continue;
    if (n.isLeaf()) {
      for (int64_t k = n.first; k < n.first + n.count; ++k) {
        int64_t idx = m.tree.index[(size_t)k];
        S t = triangleRayTime(m.tris[(size_t)idx], o, d, max_time);
        if (t < S(0)) continue;
        if (best.idx < 0 || t < best.t || (t == best.t && idx < best.idx)) { best.t = t; best.idx = idx; }
      }
    } else {
      stack.push_back(n.child[1]);
      stack.push_back(n.child[0]);
    }
  }
  return best;
}

//============================================================================================================================
// Point index + k nearest neighbours (kClosestPairs + KClosestPairsFunctor + BoundedSortedArrayN, BvhN.hpp:474-500,
// 1139-1146; Code/Source/BoundedSortedArrayN.hpp:137-214; NeighborPair ordering ProximityQueryStructureN.hpp:117-123)
//============================================================================================================================

struct Neighbor { double mad; int64_t idx; };

template <class S> struct PointIndex {
  std::vector<V3<S>> pts;
  std::vector<Box<S>> boxes;
  KdTree<S> tree;

  void init(float const * P, int64_t n, int64_t max_leaf = -1) {
    pts.resize((size_t)n);
    boxes.resize((size_t)n);
    for (int64_t i = 0; i < n; ++i) { pts[(size_t)i] = load3<S>(P + 3 * i); boxes[(size_t)i].merge(pts[(size_t)i]); }
    tree.build(n, [&](int64_t i) -> Box<S> const & { return boxes[(size_t)i]; },
               [&](int64_t i) -> V3<S> const & { return pts[(size_t)i]; }, max_leaf);
  }

  static S pointSqDist(V3<S> const & a, V3<S> const & b) { return squaredNorm(a - b); }

  // reference mode: results sorted by increasing distance; ties keep discovery order. exclude < 0: no filter.
  void knnRef(V3<S> const & q, int k, double dist_bound, int64_t exclude, std::vector<Neighbor> & out) const {
    out.clear();
    if (tree.nodes.empty() || k <= 0) return;
    double mad_bound = dist_bound >= 0 ? dist_bound * dist_bound : -1;
    Box<S> qb; qb.merge(q);
    // root pruning: processNeighbors public (BvhN.hpp:1193-1206)
    double rd = (double)qb.squaredDistance(tree.nodes[0].bounds);
    if (!boxAllows(rd, out, k)) return;
    knnRefRec(0, q, qb, k, mad_bound, exclude, out);
  }

  // KClosestPairsFunctor::allows for an incomplete pair (-1, -1, mad): insertable with query index -1 (<= semantics)
  static bool boxAllows(double mad, std::vector<Neighbor> const & arr, int k) {
    if (mad < 0) return true;
    if ((int)arr.size() < k) return true;
    return mad <= arr.back().mad;
  }

  void knnRefRec(int64_t ni, V3<S> const & q, Box<S> const & qb, int k, double mad_bound, int64_t exclude,
                 std::vector<Neighbor> & arr) const {
    KdNode<S> const & n = tree.nodes[(size_t)ni];
    if (n.isLeaf()) {
      for (int64_t kk = n.first; kk < n.first + n.count; ++kk) {
        int64_t idx = tree.index[(size_t)kk];
        if (idx == exclude) continue;  // FilterSelf (PointSet3.hpp:576-583) via elementPassesFilters
        bool dup = false;
        for (auto const & e : arr) if (e.idx == idx) { dup = true; break; }
        if (dup) continue;
        double mad = (double)pointSqDist(pts[(size_t)idx], q);
        if (!boxAllows(mad, arr, k)) continue;
        // operator(): (mad_bound < 0 || mad < mad_bound) && isInsertable(pair) -- strict for complete pairs
        if ((mad_bound < 0 || mad < mad_bound) && ((int)arr.size() < k || mad < arr.back().mad)) {
          // upperBound: first element strictly greater, i.e. after all equal distances (stable)
          size_t ub = 0;
          while (ub < arr.size() && !(mad < arr[ub].mad)) ++ub;
          arr.insert(arr.begin() + (long)ub, Neighbor{mad, idx});
          if ((int)arr.size() > k) arr.pop_back();
        }
      }
      return;
    }
    double d[2];
    for (int c = 0; c < 2; ++c) d[c] = (double)qb.squaredDistance(tree.nodes[(size_t)n.child[c]].bounds);
    int o[2];
    orderTwo(d[0], d[1], o[0], o[1]);
    for (int s = 0; s < 2; ++s)
      if (boxAllows(d[o[s]], arr, k)) knnRefRec(n.child[o[s]], q, qb, k, mad_bound, exclude, arr);
  }

  // contract mode: the k smallest (d2, index) pairs in lexicographic order
  void knnContract(V3<S> const & q, int k, double dist_bound, int64_t exclude, std::vector<std::pair<S, int64_t>> & out)
      const {
    out.clear();
    if (tree.nodes.empty() || k <= 0) return;
    double mad_bound = dist_bound >= 0 ? dist_bound * dist_bound : -1;
    Box<S> qb; qb.merge(q);
    std::vector<int64_t> stack;
    stack.push_back(0);
    while (!stack.empty()) {
      int64_t ni = stack.back(); stack.pop_back();
      KdNode<S> const & n = tree.nodes[(size_t)ni];
      S bd = qb.squaredDistance(n.bounds);
      if ((int)out.size() == k && bd > out.back().first) continue;
      if (mad_bound >= 0 && (double)bd > mad_bound) continue;
      if (n.isLeaf()) {
        for (int64_t kk = n.first; kk < n.first + n.count; ++kk) {
          int64_t idx = tree.index[(size_t)kk];
          if (idx == exclude) continue;
          S d2 = pointSqDist(pts[(size_t)idx], q);
          if (mad_bound >= 0 && !((double)d2 < mad_bound)) continue;
          std::pair<S, int64_t> cand(d2, idx);
          if ((int)out.size() == k && !(cand < out.back())) continue;
          auto it = std::upper_bound(out.begin(), out.end(), cand);
          out.insert(it, cand);
          if ((int)out.size() > k) out.pop_back();
        }
      } else {
        // nearer child on top (the result does not depend on the order)
        S c0 = qb.squaredDistance(tree.nodes[(size_t)n.child[0]].bounds);
        S c1 = qb.squaredDistance(tree.nodes[(size_t)n.child[1]].bounds);
        if (c1 < c0) {
          stack.push_back(n.child[0]);
          stack.push_back(n.child[1]);
        } else {
          stack.push_back(n.child[1]);
          stack.push_back(n.child[0]);
        }
      }
    }
  }
};

//============================================================================================================================
// Thea's Mersenne-Twister variant (Code/Source/Random.hpp:48-228, Code/Source/Random.cpp:49-157)
//============================================================================================================================

struct TheaRandom {
  static constexpr int N = 624, M = 397, R = 31, U = 11, Sh = 7, T = 15, L = 18;
  static constexpr uint32_t A = 0x9908B0DFu, B = 0x9D2C5680u, C = 0xEFC60000u;
  uint32_t state[N];
  int index;

  // Random(uint32 seed): Random.cpp:49-60 (leaves index == N, so the first draw regenerates)
  explicit TheaRandom(uint32_t seed) {
    state[0] = seed;
    for (index = 1; index < N; ++index)
      state[index] = 1812433253u * (state[index - 1] ^ (state[index - 1] >> 30)) + (uint32_t)index;
  }

  // generate(): Random.cpp:99-132. The second loop starts at N - M + 1, so state[N - M] keeps its old value.
  void generate() {
    uint32_t const LOWER = (1u << R) - 1u, UPPER = 0xFFFFFFFFu << R;
    uint32_t const mag01[2] = {0u, A};
    for (int i = 0; i < N - M; ++i) {
      uint32_t x = (state[i] & UPPER) | (state[i + 1] & LOWER);
      state[i] = state[i + M] ^ (x >> 1) ^ mag01[x & 1u];
    }
    for (int i = N - M + 1; i < N - 1; ++i) {
      uint32_t x = (state[i] & UPPER) | (state[i + 1] & LOWER);
      state[i] = state[i + (M - N)] ^ (x >> 1) ^ mag01[x & 1u];
    }
    uint32_t y = (state[N - 1] & UPPER) | (state[0] & LOWER);
    state[N - 1] = state[M - 1] ^ (y >> 1) ^ mag01[y & 1u];
    index = 0;
  }

  // bits(): Random.cpp:68-97
  uint32_t bits() {
    if ((uint32_t)index >= (uint32_t)N) { generate(); index = 0; }
    uint32_t r = state[index++];
    r ^= r >> U;
    r ^= (r << Sh) & B;
    r ^= (r << T) & C;
    r ^= r >> L;
    return r;
  }

  // integer(low, high): Random.cpp:147-157
  int32_t integer(int32_t low, int32_t high) {
    int32_t r = (int32_t)std::floor(low + (high - low + 1) * (double)bits() / 0xFFFFFFFFUL);
    return r > high ? high : r;
  }

  // uniform01(): Random.hpp:126-131 -- (float)bits() * (1.0f / (float)0xFFFFFFFF)
  float uniform01() {
    static float const NORM = 1.0f / (float)0xFFFFFFFFul;
    return (float)bits() * NORM;
  }
};

//============================================================================================================================
// MeshSampler::sampleEvenlyByArea, EXACT count mode (Code/Source/Algorithms/MeshSampler.hpp:100-204) with
// TriangleN<3>::randomPoint (Triangle3.hpp:179-195), drawing from an explicit TheaRandom instead of Random::common().
//============================================================================================================================

inline int64_t sampleEvenlyByArea(float const * V, int64_t nv, int32_t const * F, int64_t nf, int64_t n, uint32_t seed,
                                  float * pos, float * nrm, int32_t * face) {
  (void)nv;
  if (n <= 0 || nf <= 0) return 0;
  std::vector<Tri<float>> tris((size_t)nf);
  for (int64_t f = 0; f < nf; ++f)
    tris[(size_t)f] = Tri<float>(load3<float>(V + 3 * (int64_t)F[3 * f]), load3<float>(V + 3 * (int64_t)F[3 * f + 1]),
                                 load3<float>(V + 3 * (int64_t)F[3 * f + 2]));
  double total_area = 0;
  for (int64_t i = 0; i < nf; ++i) total_area += tris[(size_t)i].area;
  if (total_area <= 0) return 0;
  std::vector<double> cum((size_t)nf);
  cum[0] = tris[0].area;
  for (size_t i = 1; i < cum.size(); ++i) cum[i] = cum[i - 1] + tris[i].area;
  TheaRandom rng(seed);
  double const * first = cum.data();
  double const * last = first + cum.size();
  for (int64_t i = 0; i < n; ++i) {
    double t = rng.uniform01() * total_area;
    int64_t ti = std::min((int64_t)(std::lower_bound(first, last, t) - first), nf - 1);
    Tri<float> const & tr = tris[(size_t)ti];
    float s = rng.uniform01();
    float u = rng.uniform01();
    if (s + u > 1) { u = 1 - u; s = 1 - s; }
    V3<float> p = s * tr.edge01 + u * tr.edge02 + tr.v0;
    pos[3 * i] = p.x; pos[3 * i + 1] = p.y; pos[3 * i + 2] = p.z;
    if (nrm) { nrm[3 * i] = tr.normal.x; nrm[3 * i + 1] = tr.normal.y; nrm[3 * i + 2] = tr.normal.z; }
    if (face) face[i] = (int32_t)ti;
  }
  return n;
}

//============================================================================================================================
// Thread pool helper for the CPU baseline: static partition of [0, n) over nthreads std::threads.
//============================================================================================================================

template <class F> void parallelFor(int64_t n, int nthreads, F f) {
  if (nthreads <= 1 || n < 2) { f((int64_t)0, n); return; }
  int64_t chunk = (n + nthreads - 1) / nthreads;
  std::vector<std::thread> th;
  for (int t = 0; t < nthreads; ++t) {
    int64_t b = t * chunk, e = std::min(n, b + chunk);
    if (b >= e) break;
    th.emplace_back([=]() { f(b, e); });
  }
  for (auto & x : th) x.join();
}

//============================================================================================================================
// Affine transforms (BvhN::setTransform, BvhN.hpp:903-912; AffineTransformN.hpp:133-137,160; toObjectSpace and
// normalToWorldSpace, BvhN.hpp:2175-2184). Matrices are row-major 3x4 [L | t].
//
// Products follow Eigen's coefficient-wise evaluation of a fixed 3x3 by 3-vector product (row(i) . v, reduced as
// e0 + (e1 + e2)). The inverse restates Eigen 3.4's 3x3 inverse (Eigen/src/LU/InverseImpl.h, compute_inverse for size 3;
// Eigen is not present here, so this step is the published algorithm, unpinned): cofactor(i, j) =
// L(i+1, j+1) L(i+2, j+2) - L(i+1, j+2) L(i+2, j+1) (indices mod 3), det = the cofactors of column 0 dotted with column 0,
// inverse(j, i) = cofactor(i, j) * (1 / det); then the translation L^-1 (-t) (AffineTransformN::inverse).
//============================================================================================================================

template <class S> inline V3<S> affinePoint(S const * m, V3<S> const & v) {
  return V3<S>((m[0] * v.x + (m[1] * v.y + m[2] * v.z)) + m[3], (m[4] * v.x + (m[5] * v.y + m[6] * v.z)) + m[7],
               (m[8] * v.x + (m[9] * v.y + m[10] * v.z)) + m[11]);
}
template <class S> inline V3<S> affineLinear(S const * m, V3<S> const & v) {
  return V3<S>(m[0] * v.x + (m[1] * v.y + m[2] * v.z), m[4] * v.x + (m[5] * v.y + m[6] * v.z),
               m[8] * v.x + (m[9] * v.y + m[10] * v.z));
}
template <class S> inline bool affineInverse(S const * m, S * inv) {
  auto L = [&](int i, int j) { return m[4 * (i % 3) + (j % 3)]; };
  auto cof = [&](int i, int j) { return L(i + 1, j + 1) * L(i + 2, j + 2) - L(i + 1, j + 2) * L(i + 2, j + 1); };
  S det = cof(0, 0) * m[0] + (cof(1, 0) * m[4] + cof(2, 0) * m[8]);
  if (!(det != S(0)) || !std::isfinite(det)) return false;
  S invdet = S(1) / det;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) inv[4 * j + i] = cof(i, j) * invdet;
  S nt[3] = {-m[3], -m[7], -m[11]};
  for (int r = 0; r < 3; ++r) inv[4 * r + 3] = inv[4 * r] * nt[0] + (inv[4 * r + 1] * nt[1] + inv[4 * r + 2] * nt[2]);
  return true;
}
// (L^-1)^T n, normalised; inv is the inverse transform's 3x4 matrix
template <class S> inline V3<S> normalToWorld(S const * inv, V3<S> const & n) {
  return normalized(V3<S>(inv[0] * n.x + (inv[4] * n.y + inv[8] * n.z), inv[1] * n.x + (inv[5] * n.y + inv[9] * n.z),
                          inv[2] * n.x + (inv[6] * n.y + inv[10] * n.z)));
}

//============================================================================================================================
// Random::sphere (Random.cpp:225-250; Knop, CACM 13, 1970) and Visibility::compute
// (Algorithms/SurfaceFeatures/Local/Visibility.hpp:104-126) with a given generator in place of Random::common().
//============================================================================================================================

inline V3<float> theaSphere(TheaRandom & r) {
  float x, y, m2;
  do {
    x = 2 * r.uniform01() - 1;
    y = 2 * r.uniform01() - 1;
    m2 = x * x + y * y;
  } while (m2 > 1 || m2 < 1e-10);
  float z = 2 * m2 - 1;
  float s = 2 * std::sqrt(1 - m2);
  return V3<float>(x * s, y * s, z);
}

// Escaped fraction of the rays along dirs[0 .. num_rays) from `position`, with `scale` the |extent| of the BVH's
// getBounds(); inv (nullable): the inverse of the BVH's transform, which moves each ray into object space
// (toObjectSpace, BvhN.hpp:2175-2178)
inline double visibilityFraction(MeshIndex<float> const & m, V3<float> const & position, V3<float> const * dirs,
                                 int64_t num_rays, float scale, float const * inv) {
  int64_t escaped = 0;
  for (int64_t i = 0; i < num_rays; ++i) {
    V3<float> u = dirs[i];
    V3<float> offset = 0.001f * scale * u;
    V3<float> o = position + offset, d = u;
    if (inv) o = affinePoint(inv, o), d = affineLinear(inv, d);
    bool hit = m.rayRef(o, d, -1.f).idx >= 0;  // rayIntersects = rayIntersectionTime >= 0
    if (!hit) ++escaped;
  }
  return (double)escaped / num_rays;
}

//============================================================================================================================
// ShapeDiameter::compute (Algorithms/SurfaceFeatures/Local/ShapeDiameter.hpp:143-217) for a BVH-backed instance
// (constructor at :94-101). Rays by contract-mode first hit (lowest index among equal times); the median is selected by
// this C++ library's own std::nth_element, which permutes the values but not the weights paired with them afterwards.
//============================================================================================================================

// The reference's 30 cone directions about the local z axis (ShapeDiameter.hpp:163-193)
static float const SDF_CONE_DIRS[30][3] = {
    {0.407497f, 0.134086f, 0.903309f},     {0.128722f, -0.822715f, 0.553688f},   {0.359298f, 0.686129f, 0.632560f},
    {0.813318f, -0.153956f, 0.561081f},    {-0.707169f, 0.296987f, 0.641647f},   {-0.478783f, -0.543441f, 0.689520f},
    {0.561083f, 0.523634f, 0.641087f},     {-0.380898f, -0.655789f, 0.651811f},  {0.722588f, 0.472155f, 0.504912f},
    {-0.535205f, 0.421235f, 0.732200f},    {0.577593f, -0.477896f, 0.661817f},   {0.393652f, -0.144484f, 0.907834f},
    {0.141508f, -0.660777f, 0.737122f},    {-0.274967f, -0.141703f, 0.950954f},  {-0.304935f, 0.474085f, 0.825989f},
    {0.711150f, 0.301383f, 0.635164f},     {-0.696119f, -0.112341f, 0.709082f},  {-0.248327f, 0.381035f, 0.890588f},
    {-0.0772394f, 0.0462501f, 0.995939f},  {0.438024f, 0.656463f, 0.614159f},    {-0.483384f, -0.542477f, 0.687065f},
    {0.498569f, -0.697466f, 0.514752f},    {-0.128902f, -0.0173429f, 0.991506f}, {0.338759f, -0.318772f, 0.885227f},
    {-0.574364f, -0.463887f, 0.674474f},   {-0.459207f, 0.260125f, 0.849390f},   {-0.628057f, -0.528928f, 0.570771f},
    {0.232916f, -0.328273f, 0.915416f},    {0.231667f, -0.796882f, 0.557951f},   {-0.270612f, -0.809654f, 0.520797f},
};

// Math::orthogonalDirection (MatrixUtil.hpp:225-231)
inline V3<float> orthogonalDirection(V3<float> const & v) {
  return maxAbsAxis(v) == 0 ? normalized(V3<float>(v.y, -v.x, 0.f)) : normalized(V3<float>(0.f, v.z, -v.y));
}

// One point with its outward normal; inv (nullable): the inverse of the BVH's transform (rays into object space, hit
// normals back through its transpose)
inline double shapeDiameter(MeshIndex<float> const & m, V3<float> const & position, V3<float> const & normal,
                            float scale, bool only_interior, float const * inv) {
  V3<float> nn = normalized(normal);
  V3<float> in(-nn.x, -nn.y, -nn.z);
  // Math::orthonormalBasis(in) (MatrixUtil.hpp:241-249): columns u, v, w
  V3<float> w = normalized(in);
  V3<float> u = orthogonalDirection(in);
  V3<float> v = cross(w, u);
  V3<float> offset = 0.001f * scale * in;
  double values[30], weights[30];
  int num_values = 0;
  for (int i = 0; i < 30; ++i) {
    float const * c = SDF_CONE_DIRS[i];
    V3<float> dir(u.x * c[0] + (v.x * c[1] + w.x * c[2]), u.y * c[0] + (v.y * c[1] + w.y * c[2]),
                  u.z * c[0] + (v.z * c[1] + w.z * c[2]));
    V3<float> o = position + offset, d = dir;
    if (inv) o = affinePoint(inv, o), d = affineLinear(inv, d);
    auto hit = rayContract(m, o, d, -1.f);
    if (hit.idx < 0) continue;
    V3<float> hn = m.tris[(size_t)hit.idx].normal;
    if (inv) hn = normalToWorld(inv, hn);
    if (!only_interior || dot(hn, dir) >= 0.f) {
      values[num_values] = hit.t;
      weights[num_values] = c[2];
      ++num_values;
    }
  }
  if (num_values <= 0) return -1.0;
  int mid = num_values / 2;
  std::nth_element(values, values + mid, values + num_values);
  double sum_values = 0, sum_squares = 0;
  for (int i = 0; i < num_values; ++i) {
    sum_values += values[i];
    sum_squares += values[i] * values[i];
  }
  double avg = sum_values / num_values;
  double var = sum_squares / num_values - avg * avg;
  sum_values = 0;
  double sum_weights = 0;
  for (int i = 0; i < num_values; ++i)
    if ((values[i] - values[mid]) * (values[i] - values[mid]) <= var) {
      sum_values += weights[i] * values[i];
      sum_weights += weights[i];
    }
  double r = sum_weights > 0 ? sum_values / (sum_weights * scale) : values[mid] / scale;
  return r < 0.0 ? 0.0 : (r > 1.0 ? 1.0 : r);
}

//============================================================================================================================
// Sample proximity graph: PointSet3::updateGraph without oversampling (Algorithms/PointSet3.hpp:324-391), with
// findSampleNeighbors / NeighborFunctor (:586-681) and updateAverageSeparation (:688-702). The separation estimate draws
// from the given generator in place of Random::common(). Candidates by brute force (every other sample inside the
// ball); neighbour sets keep the max_degree smallest (separation, index), SamplePoint3's order.
//============================================================================================================================

// Math::fastRsq (Math.hpp:193-208) and fastSqrt (:218-223)
inline float fastRsq(float x) {
  float x2 = x * 0.5f;
  float y = x;
  int32_t i;
  std::memcpy(&i, &y, 4);
  i = 0x5f3759df - (i >> 1);
  std::memcpy(&y, &i, 4);
  y = y * (1.5f - (x2 * y * y));
  return y;
}
inline float fastSqrt(float x) { return 1.0f / fastRsq(x); }

struct SampleGraphResult {
  std::vector<std::vector<std::pair<float, int32_t>>> nbrs;  // per sample, ascending (separation, index)
  float estimate = 0, final_avg = 0;
};

inline SampleGraphResult sampleGraph(std::vector<V3<float>> const & P, std::vector<V3<float>> const * N, int max_degree,
                                     TheaRandom & rng, MeshIndex<float> const * surface, int nthreads) {
  SampleGraphResult g;
  int64_t n = (int64_t)P.size();
  g.nbrs.resize((size_t)n);
  int64_t trials = std::min<int64_t>(100, n);
  float avg = 0;
  for (int64_t t = 0; t < trials; ++t) {
    int32_t i = rng.integer(0, (int32_t)n - 1);
    float best = std::numeric_limits<float>::infinity();
    for (int64_t j = 0; j < n; ++j)
      if (j != i) best = std::min(best, squaredNorm(P[(size_t)j] - P[(size_t)i]));
    avg += best;
  }
  avg = std::sqrt(avg / (float)trials);
  g.estimate = avg;
  float init_radius = std::sqrt((float)max_degree) * avg;
  int d4 = (int)(0.25 * max_degree);
  int min_degree = d4 < 4 ? 4 : (d4 > max_degree ? max_degree : d4);
  parallelFor(n, nthreads, [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) {
      float radius = init_radius;
      auto & out = g.nbrs[(size_t)i];
      for (int it = 0; it < 3; ++it) {
        out.clear();
        float r2 = radius * radius;
        for (int64_t j = 0; j < n; ++j) {
          if (j == i) continue;
          V3<float> diff = P[(size_t)j] - P[(size_t)i];
          float sq = squaredNorm(diff);
          if (!(sq <= r2)) continue;  // BallN::contains
          if (N && dot((*N)[(size_t)i], (*N)[(size_t)j]) < -0.5f) continue;
          float sep = fastSqrt(sq);
          if (surface && N) {
            V3<float> lift = normalized((*N)[(size_t)i] + (*N)[(size_t)j]);
            V3<float> o = P[(size_t)i] + 5.0f * sep * lift;
            if (surface->rayRef(o, diff, 1.f).idx >= 0) continue;
          }
          std::pair<float, int32_t> c(sep, (int32_t)j);
          auto pos = std::lower_bound(out.begin(), out.end(), c);
          if ((int)out.size() < max_degree) out.insert(pos, c);
          else if (pos != out.end()) { out.insert(pos, c); out.pop_back(); }
        }
        if ((int)out.size() >= min_degree) break;
        radius *= 2.0f;
      }
    }
  });
  float s = 0;
  int64_t edges = 0;
  for (auto const & v : g.nbrs) {
    for (auto const & c : v) s += c.first;
    edges += (int64_t)v.size();
  }
  if (edges > 0) s /= (float)edges;
  g.final_avg = s;
  return g;
}

}  // namespace oracle
