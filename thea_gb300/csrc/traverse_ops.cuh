// Per-query traversal routines shared by the single-BVH kernels and the batched persistent kernels, plus the FP64
// re-check arithmetic.
//
// Each routine walks one BVH of a forest from its root node with a per-thread stack of (node or leaf code, lower bound),
// nearest child first. Leaves hold element positions relative to their segment's first sorted position (elem_base).
#pragma once

#include "traverse.cuh"

namespace thea {

//============================================================================================================================
// FP64 twin of the triangle arithmetic: the same algorithm as the FP32 path (Triangle3.hpp:143-155, 294-304,
// 1311-1462; HyperplaneN.hpp:145-160), evaluated in double from the FP32 vertices, with the same operation order.
//============================================================================================================================

struct D3 {
  double x, y, z;
};
__device__ __forceinline__ D3 operator+(D3 a, D3 b) { return D3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ D3 operator-(D3 a, D3 b) { return D3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ D3 operator*(double s, D3 a) { return D3{s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ D3 operator*(D3 a, double s) { return D3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ D3 operator/(D3 a, double s) { return D3{a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ double dotd(D3 a, D3 b) { return a.x * b.x + (a.y * b.y + a.z * b.z); }
__device__ __forceinline__ double sqnormd(D3 a) { return a.x * a.x + (a.y * a.y + a.z * a.z); }
__device__ __forceinline__ D3 crossd(D3 a, D3 b) {
  return D3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ D3 todd(V3 v) { return D3{(double)v.x, (double)v.y, (double)v.z}; }

__device__ __forceinline__ bool inside_d(D3 v0, D3 v1, D3 v2, int axis, D3 p) {
  double v0i, v0j, v1i, v1j, v2i, v2j, pi, pj;
  if (axis == 1) {
    v0i = v0.z; v0j = v0.x; v1i = v1.z; v1j = v1.x; v2i = v2.z; v2j = v2.x; pi = p.z; pj = p.x;
  } else if (axis == 2) {
    v0i = v0.x; v0j = v0.y; v1i = v1.x; v1j = v1.y; v2i = v2.x; v2j = v2.y; pi = p.x; pj = p.y;
  } else {
    v0i = v0.y; v0j = v0.z; v1i = v1.y; v1j = v1.z; v2i = v2.y; v2j = v2.z; pi = p.y; pj = p.z;
  }
  double area = (v1i - v0i) * (v2j - v0j) - (v2i - v0i) * (v1j - v0j);
  if (area == 0.0) return v0.x == p.x && v0.y == p.y && v0.z == p.z;
  double inv_area = 1.0 / area;
  double b0 = ((v1i - pi) * (v2j - pj) - (v2i - pi) * (v1j - pj)) * inv_area;
  if ((b0 < 0.0) || (b0 > 1.0)) return false;
  double b1 = ((pi - v0i) * (v2j - v0j) - (v2i - v0i) * (pj - v0j)) * inv_area;
  if ((b1 < 0.0) || (b1 > 1.0)) return false;
  double b2 = 1.0 - b0 - b1;
  return (b2 >= 0.0) && (b2 <= 1.0);
}

__device__ __forceinline__ D3 seg_d(D3 a, D3 b, D3 dir, double len, D3 p) {
  D3 c = p - a;
  double t = dotd(dir, c);
  if (t <= 0.0) return a;
  if (t >= len) return b;
  return a + dir * t;
}

// Squared distance (and closest point) from p to the triangle, in FP64
__device__ __forceinline__ double closest_point_f64(V3 fv0, V3 fv1, V3 fv2, V3 fp, D3 & cp) {
  D3 v0 = todd(fv0), v1 = todd(fv1), v2 = todd(fv2), p = todd(fp);
  D3 n = crossd(v1 - v0, v2 - v0);
  double z = sqnormd(n);
  if (z > 0.0) n = n / sqrt(z);
  double dist = dotd(n, v0);
  double a0 = fabs(n.x), a1 = fabs(n.y), a2 = fabs(n.z);
  int axis = 0;
  double best = a0;
  if (a1 > best) { axis = 1; best = a1; }
  if (a2 > best) axis = 2;
  double sd = dotd(p, n) - dist;
  D3 proj = p - sd * n;
  if (inside_d(v0, v1, v2, axis, proj)) {
    cp = proj;
  } else {
    D3 e[3] = {v1 - v0, v2 - v1, v0 - v2};
    double len[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      len[i] = sqrt(sqnormd(e[i]));
      e[i] = e[i] / len[i];
    }
    D3 r0 = seg_d(v0, v1, e[0], len[0], p), r1 = seg_d(v1, v2, e[1], len[1], p), r2 = seg_d(v2, v0, e[2], len[2], p);
    double q0 = sqnormd(r0 - p), q1 = sqnormd(r1 - p), q2 = sqnormd(r2 - p);
    if (q0 < q1) cp = (q0 < q2) ? r0 : r2;
    else cp = (q1 < q2) ? r1 : r2;
  }
  return sqnormd(cp - p);
}

// Watertight ray/triangle test in FP64 (Woop, Benthin, Wald, "Watertight Ray/Triangle Intersection", JCGT 2013):
// shear the triangle into the ray's frame, evaluate the three edge functions, accept points on edges. Returns the hit
// time (>= 0) or -1.
__device__ __forceinline__ double ray_triangle_watertight_f64(V3 fo, V3 fd, V3 fv0, V3 fe01, V3 fe02) {
  D3 o = todd(fo), d = todd(fd);
  D3 v0 = todd(fv0);
  D3 v1 = v0 + todd(fe01), v2 = v0 + todd(fe02);
  double ad[3] = {fabs(d.x), fabs(d.y), fabs(d.z)};
  int kz = (ad[0] > ad[1]) ? ((ad[0] > ad[2]) ? 0 : 2) : ((ad[1] > ad[2]) ? 1 : 2);
  int kx = kz == 2 ? 0 : kz + 1;
  int ky = kx == 2 ? 0 : kx + 1;
  double dd[3] = {d.x, d.y, d.z};
  if (dd[kz] < 0.0) { int t = kx; kx = ky; ky = t; }
  if (dd[kz] == 0.0) return -1.0;
  double Sx = dd[kx] / dd[kz], Sy = dd[ky] / dd[kz], Sz = 1.0 / dd[kz];
  D3 A = v0 - o, B = v1 - o, C = v2 - o;
  double a[3] = {A.x, A.y, A.z}, b[3] = {B.x, B.y, B.z}, c[3] = {C.x, C.y, C.z};
  double Ax = a[kx] - Sx * a[kz], Ay = a[ky] - Sy * a[kz];
  double Bx = b[kx] - Sx * b[kz], By = b[ky] - Sy * b[kz];
  double Cx = c[kx] - Sx * c[kz], Cy = c[ky] - Sy * c[kz];
  double U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
  if ((U < 0.0 || V < 0.0 || W < 0.0) && (U > 0.0 || V > 0.0 || W > 0.0)) return -1.0;
  double det = U + V + W;
  if (det == 0.0) return -1.0;
  double T = U * (Sz * a[kz]) + V * (Sz * b[kz]) + W * (Sz * c[kz]);
  double t = T / det;
  return t >= 0.0 ? t : -1.0;
}

//============================================================================================================================
// Closest element
//============================================================================================================================

// Squared distance and closest point of the record at sorted position k (FP32, reference arithmetic)
__device__ __forceinline__ float cp_record_test(float4 const * __restrict__ rec, int64_t k, V3 p, V3 & cp) {
  float4 const * r = rec + k * CP_REC_F4;
  float4 a = __ldg(r), b = __ldg(r + 1), c = __ldg(r + 2), nn = __ldg(r + 3);
  V3 v0 = xyz(a), v1 = xyz(b), v2 = xyz(c), nrm = xyz(nn);
  // HyperplaneN::closestPoint: p - signedDistance(p) * normal, signedDistance = p . normal - dist
  float sd = dot(p, nrm) - a.w;
  V3 proj = p - sd * nrm;
  if (point_inside_triangle(v0, v1, v2, __float_as_int(nn.w), proj)) {
    cp = proj;
  } else {
    float4 e0 = __ldg(r + 4), e1 = __ldg(r + 5), e2 = __ldg(r + 6);
    cp = closest_on_perimeter(v0, v1, v2, xyz(e0), b.w, xyz(e1), c.w, xyz(e2), e0.w, p);
  }
  return squared_norm(cp - p);
}

__device__ __forceinline__ int cp_record_index(float4 const * __restrict__ rec, int64_t k) {
  return __float_as_int(__ldg(rec + k * CP_REC_F4 + 5).w);
}

__device__ __forceinline__ float l1(V3 a) { return fabsf(a.x) + fabsf(a.y) + fabsf(a.z); }

// FP64 squared distance and closest point of one closest-point record: the result of closest_point_f64 on the record's
// vertices, bit for bit, with less FP64 work. The record's FP32 data decide, with error margins, which branch
// closest_point_f64 takes: whether the plane projection is inside the triangle (then only the normalised normal and the
// projection are computed), and on the perimeter path, for each edge, whether the segment search clamps to an endpoint
// (then the endpoint is the result with no square root or division) and whether the edge can be the nearest at all
// (if its distance provably exceeds another edge's, it is left out: it cannot be the minimum, and ties are only
// resolved among minima). Every FP64 value that is computed uses closest_point_f64's own operations; where the margins
// do not decide a branch, closest_point_f64 itself runs. The margins are 2^5 or more times an FP32 rounding bound.
__device__ __forceinline__ double cp_record_f64_fast(float4 const * __restrict__ r, V3 fp, D3 & out_cp) {
  float4 a0 = __ldg(r), a1 = __ldg(r + 1), a2 = __ldg(r + 2), a3 = __ldg(r + 3);
  float4 a4 = __ldg(r + 4), a5 = __ldg(r + 5), a6 = __ldg(r + 6);
  V3 fv0 = xyz(a0), fv1 = xyz(a1), fv2 = xyz(a2), n32 = xyz(a3);
  int axis = __float_as_int(a3.w);
  // region of the plane projection, in FP32: 1 inside, 2 outside, 0 undecided
  float sd32 = dot(fp, n32) - a0.w;
  V3 pr = fp - sd32 * n32;
  float v0i, v0j, v1i, v1j, v2i, v2j, pi, pj;
  if (axis == 1) {
    v0i = fv0.z; v0j = fv0.x; v1i = fv1.z; v1j = fv1.x; v2i = fv2.z; v2j = fv2.x; pi = pr.z; pj = pr.x;
  } else if (axis == 2) {
    v0i = fv0.x; v0j = fv0.y; v1i = fv1.x; v1j = fv1.y; v2i = fv2.x; v2j = fv2.y; pi = pr.x; pj = pr.y;
  } else {
    v0i = fv0.y; v0j = fv0.z; v1i = fv1.y; v1j = fv1.z; v2i = fv2.y; v2j = fv2.z; pi = pr.y; pj = pr.z;
  }
  float area = (v1i - v0i) * (v2j - v0j) - (v2i - v0i) * (v1j - v0j);
  float len[3] = {a1.w, a2.w, a4.w};
  int region = 0;
  if (area != 0.f) {
    float b0 = ((v1i - pi) * (v2j - pj) - (v2i - pi) * (v1j - pj)) / area;
    float b1 = ((pi - v0i) * (v2j - v0j) - (v2i - v0i) * (pj - v0j)) / area;
    float b2 = 1.0f - b0 - b1;
    float S = fmaxf(fmaxf(fmaxf(fabsf(fp.x), fabsf(fp.y)), fabsf(fp.z)),
                    fmaxf(fmaxf(l1(fv0), l1(fv1)), l1(fv2)));
    float R = fmaxf(fmaxf(l1(fv0 - pr), l1(fv1 - pr)), l1(fv2 - pr));
    float L = fmaxf(fmaxf(len[0], len[1]), len[2]);
    float tau = (1.0f / 4096.0f) + (1.0f / 65536.0f) * (S + R) * (R + L) / fabsf(area);
    float bmin = fminf(fminf(b0, b1), b2);
    if (bmin >= tau) region = 1;
    else if (bmin <= -tau) region = 2;
  }
  if (region == 0) return closest_point_f64(fv0, fv1, fv2, fp, out_cp);
  D3 v0 = todd(fv0), v1 = todd(fv1), v2 = todd(fv2), p = todd(fp);
  if (region == 1) {
    D3 n = crossd(v1 - v0, v2 - v0);
    double z = sqnormd(n);
    if (z > 0.0) n = n / sqrt(z);
    double dist = dotd(n, v0);
    double sd = dotd(p, n) - dist;
    D3 proj = p - sd * n;
    out_cp = proj;
    return sqnormd(proj - p);
  }
  // perimeter: edge i runs from vertex i to vertex i + 1
  V3 fa[3] = {fv0, fv1, fv2}, fb[3] = {fv1, fv2, fv0}, fdir[3] = {xyz(a4), xyz(a5), xyz(a6)};
  D3 da[3] = {v0, v1, v2}, db[3] = {v1, v2, v0};
  float q32[3], qerr[3];
  int kind[3];  // 0: clamps to the edge's start, 1: to its end, 2: undecided (closest_point_f64's segment search)
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    V3 c = fp - fa[i];
    float t = dot(fdir[i], c);
    float D = l1(c) + len[i];
    float dl = (1.0f / 65536.0f) * D;
    kind[i] = t <= -dl ? 0 : (t >= len[i] + dl ? 1 : 2);
    V3 rr = t <= 0.f ? fa[i] : (t >= len[i] ? fb[i] : fa[i] + fdir[i] * t);
    q32[i] = squared_norm(rr - fp);
    qerr[i] = (1.0f / 16384.0f) * D * D;
  }
  float qmin = fminf(fminf(q32[0] + qerr[0], q32[1] + qerr[1]), q32[2] + qerr[2]);
  double q[3];
  D3 rr[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    rr[i] = da[i];
    if (q32[i] - qerr[i] > qmin) {
      q[i] = INFINITY;  // provably farther than another edge
      continue;
    }
    if (kind[i] == 1) {
      rr[i] = db[i];
    } else if (kind[i] == 2) {
      D3 e = db[i] - da[i];
      double l = sqrt(sqnormd(e));
      rr[i] = seg_d(da[i], db[i], e / l, l, p);
    }
    q[i] = sqnormd(rr[i] - p);
  }
  D3 cp;
  if (q[0] < q[1]) cp = (q[0] < q[2]) ? rr[0] : rr[2];
  else cp = (q[1] < q[2]) ? rr[1] : rr[2];
  out_cp = cp;
  return sqnormd(cp - p);
}

// Out of line: every caller shares one copy of the FP64 sequence, which matters on a GPU whose FP64 pipe is narrow.
static __device__ __noinline__ double cp_record_f64_call(float4 const * __restrict__ rec, int64_t k, V3 p, D3 * cp) {
  return cp_record_f64_fast(rec + k * CP_REC_F4, p, *cp);
}

__device__ __forceinline__ float cp_record_f64(float4 const * __restrict__ rec, int64_t k, V3 p, D3 & cp, double & d2) {
  d2 = cp_record_f64_call(rec, k, p, &cp);
  return (float)d2;
}

struct ClosestOut {
  int idx;      // element index within its mesh, INT_MAX if none
  float d2;     // FP32 squared distance (reference mode) or the FP64 squared distance rounded (re-check mode)
  V3 cp;
  double d2_64;  // FP64 squared distance of the chosen element (re-check mode, or when an error estimate is wanted)
  int64_t slot;  // sorted position of the chosen element
  float best32;  // re-check mode: smallest FP32 squared distance of an accepted element (an upper bound), +inf if none
  bool done;     // false when the pop budget ran out before the search finished
};

// Children of a node whose lower bound passes `lim` (misses carry a NaN bound and never pass), in ascending bound
// order: the nearest is returned in `next` (the
// next step visits it without a stack round trip) and the others are pushed farthest first as packed (code, bound bits)
// entries, one 8-byte access each. `next` is CHILD_EMPTY when no child is kept.
template <int W, int STACK>
__device__ __forceinline__ void push_children_next(NodeRegs<W> const & nd, float const (&lb)[W], float lim,
                                                   int2 (&stk)[STACK], int & sp, int & next, unsigned * err) {
  uint32_t key[W];
  int cc[W];
#pragma unroll
  for (int c = 0; c < W; ++c) {
    bool keep = nd.child[c] != CHILD_EMPTY && lb[c] <= lim;
    key[c] = keep ? __float_as_uint(lb[c]) : 0xffffffffu;
    cc[c] = nd.child[c];
  }
  sort_children<W>(key, cc);
  next = key[0] != 0xffffffffu ? cc[0] : CHILD_EMPTY;
#pragma unroll
  for (int c = W - 1; c >= 1; --c) {
    if (key[c] != 0xffffffffu) {
      if (sp < STACK) {
        stk[sp] = make_int2(cc[c], (int)key[c]);
        ++sp;
      } else {
        atomicOr(err, ERR_STACK_OVERFLOW);
      }
    }
  }
}

template <int W>
__device__ __forceinline__ void point_child_bounds(NodeRegs<W> const & nd, V3 p, float (&lb)[W]) {
#pragma unroll
  for (int c = 0; c < W; ++c)
    lb[c] = point_box_d2(p.x, p.y, p.z, nd.lox[c], nd.loy[c], nd.loz[c], nd.hix[c], nd.hiy[c], nd.hiz[c]);
}

// Oriented slab of a child slot: float4 (nx, ny, dmin, dmax). The unit normal n has nz = +-sqrt(1 - nx^2 - ny^2), its
// sign in the lowest bit of nx's encoding; every vertex v of the child's triangles satisfies dmin <= n . v <= dmax for
// the decoded n. An empty slot has dmin = +inf, dmax = -inf.
__host__ __device__ __forceinline__ uint32_t slab_bits(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  uint32_t u;
  memcpy(&u, &x, 4);
  return u;
#endif
}

__host__ __device__ __forceinline__ float slab_float(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float x;
  memcpy(&x, &u, 4);
  return x;
#endif
}

__host__ __device__ __forceinline__ V3 slab_normal(float4 s) {
  float nz = sqrtf(fmaxf(0.f, 1.f - (s.x * s.x + s.y * s.y)));
  return V3{s.x, s.y, (slab_bits(s.x) & 1u) ? -nz : nz};
}

__host__ __device__ __forceinline__ float4 slab_encode(V3 n) {
  float x = slab_float((slab_bits(n.x) & ~1u) | (n.z < 0.f ? 1u : 0u));
  return make_float4(x, n.y, 0.f, 0.f);
}

// Squared lower bound on the distance from q to a child's triangles by its slab, with d = n . q in FP32 (q1 = |q.x| +
// |q.y| + |q.z|). A triangle lies between the slab's planes, so its distance to q is at least the distance from q to
// the slab, |n . q - n . v| / |n| over its points v. The decoded |n| is 1 to within a few ulps; the margin subtracted
// (2^-20 of the magnitudes involved) covers that and the FP32 rounding of n . q and of the difference.
__device__ __forceinline__ float slab_lower_bound(float4 s, V3 q, float q1, float & d) {
  V3 n = slab_normal(s);
  d = n.x * q.x + (n.y * q.y + n.z * q.z);
  float margin = (q1 + fabsf(s.z) + fabsf(s.w)) * (1.0f / 1048576.0f);
  float g = fmaxf(d - s.w, s.z - d) - margin;
  return g > 0.f ? g * g : 0.f;
}

// Raises the box bounds `lb` of a node's children to their slab bounds where those are larger. `order` is the visiting
// key: the box bound, except where q lies on the inner side of every child's slab (below dmin: inside a closed
// surface), where the slabs separate the children better than their boxes and the raised bound orders them.
template <int W>
__device__ __forceinline__ void slab_child_bounds(NodeRegs<W> const & nd, float4 const * __restrict__ slabs, int node,
                                                  V3 p, float q1, float (&lb)[W], float (&order)[W]) {
#pragma unroll
  for (int c = 0; c < W; ++c) order[c] = lb[c];
  float4 const * sp = slabs + (int64_t)node * W;
  bool inner = true;
#pragma unroll
  for (int c = 0; c < W; ++c) {
    float4 sl = __ldg(sp + c);
    float d;
    lb[c] = fmaxf(lb[c], slab_lower_bound(sl, p, q1, d));
    inner = inner && (nd.child[c] == CHILD_EMPTY || d < sl.z);
  }
  if (inner) {
#pragma unroll
    for (int c = 0; c < W; ++c) order[c] = lb[c];
  }
}

// push_children_next with a visiting key apart from the pruning bound: the children whose bound passes `lim` are kept,
// the one with the smallest key goes to `next`, the others are pushed with their bounds, largest key first.
template <int W, int STACK>
__device__ __forceinline__ void push_children_ordered(NodeRegs<W> const & nd, float const (&lb)[W],
                                                      float const (&order)[W], float lim, int2 (&stk)[STACK], int & sp,
                                                      int & next, unsigned * err) {
  uint32_t key[W];
  int slot[W];
#pragma unroll
  for (int c = 0; c < W; ++c) {
    bool keep = nd.child[c] != CHILD_EMPTY && lb[c] <= lim;
    key[c] = keep ? __float_as_uint(order[c]) : 0xffffffffu;
    slot[c] = c;
  }
  sort_children<W>(key, slot);
  // the arrays stay in registers: a slot's code and bound are picked by select loops, not by dynamic indexing
  int code0 = CHILD_EMPTY;
#pragma unroll
  for (int u = 0; u < W; ++u) code0 = u == slot[0] ? nd.child[u] : code0;
  next = key[0] != 0xffffffffu ? code0 : CHILD_EMPTY;
#pragma unroll
  for (int c = W - 1; c >= 1; --c) {
    if (key[c] != 0xffffffffu) {
      if (sp < STACK) {
        int code = CHILD_EMPTY;
        float bound = 0.f;
#pragma unroll
        for (int u = 0; u < W; ++u) {
          code = u == slot[c] ? nd.child[u] : code;
          bound = u == slot[c] ? lb[u] : bound;
        }
        stk[sp] = make_int2(code, __float_as_int(bound));
        ++sp;
      } else {
        atomicOr(err, ERR_STACK_OVERFLOW);
      }
    }
  }
}

// Element tests of one leaf (segment-relative elements [first, first + count)), FP32 reference arithmetic: keeps the
// smallest (d2, index) with d2 <= best.
__device__ __forceinline__ void cp_leaf_fp32(float4 const * __restrict__ rec, int64_t elem_base, int first, int count,
                                             V3 p, float & best, int & best_idx, int64_t & best_slot, V3 & best_cp) {
  int64_t k0 = elem_base + first;
  for (int64_t k = k0; k < k0 + count; ++k) {
    V3 cp;
    float d2 = cp_record_test(rec, k, p, cp);
    if (d2 <= best) {
      int idx = cp_record_index(rec, k);
      if (d2 < best || idx < best_idx) {
        best = d2;
        best_idx = idx;
        best_cp = cp;
        best_slot = k;
      }
    }
  }
}

// FP32 reference-arithmetic search: smallest (d2, index), accepting d2 <= thresh. With budget > 0 the search stops
// after that many stack pops (done = false), leaving the best found so far. With the BVH's oriented slabs (single
// mesh BVHs) the children's bounds are raised to their slab bounds; the result is the same, the search shorter.
template <int W, int STACK>
__device__ __forceinline__ ClosestOut closest_query(WideNode<W> const * __restrict__ nodes,
                                                    float4 const * __restrict__ rec, int root, int64_t elem_base, V3 p,
                                                    float thresh, unsigned * err, int budget = 0,
                                                    float4 const * __restrict__ slabs = nullptr) {
  float q1 = fabsf(p.x) + fabsf(p.y) + fabsf(p.z);
  bool done = true;
  float best = thresh;
  int best_idx = INT_MAX;
  int64_t best_slot = -1;
  V3 best_cp = V3{0.f, 0.f, 0.f};
  int2 stk[STACK];  // (child code, bound bits)
  int sp = 0;
  int next = root;  // nearest child of the last node, visited without a stack round trip
  int pops = 0;
  while (next != CHILD_EMPTY || sp > 0) {
    if (budget > 0 && ++pops > budget) {
      done = false;
      break;
    }
    int code = next;
    if (code == CHILD_EMPTY) {
      --sp;
      code = stk[sp].x;
      if (__int_as_float(stk[sp].y) > best * PRUNE_SLACK) continue;
    }
    next = CHILD_EMPTY;
    if (code >= 0) {
      NodeRegs<W> nd;
      load_node(nodes, code, nd);
      float lb[W];
      point_child_bounds<W>(nd, p, lb);
      if (slabs) {
        float order[W];
        slab_child_bounds<W>(nd, slabs, code, p, q1, lb, order);
        push_children_ordered<W, STACK>(nd, lb, order, best * PRUNE_SLACK, stk, sp, next, err);
      } else {
        push_children_next<W, STACK>(nd, lb, best * PRUNE_SLACK, stk, sp, next, err);
      }
    } else {
      int first, count;
      decode_leaf(code, first, count);
      cp_leaf_fp32(rec, elem_base, first, count, p, best, best_idx, best_slot, best_cp);
    }
  }
  ClosestOut o;
  o.idx = best_idx;
  o.d2 = best;
  o.cp = best_cp;
  o.d2_64 = 0.0;
  o.slot = best_slot;
  o.best32 = best;
  o.done = done;
  return o;
}

// Mixed-precision search, in two steps. closest_search_f64 runs the FP32 traversal and element tests of one query and
// collects every element whose FP32 distance lies within a band of the FP32 best; f64_resolve_warp then evaluates the
// collected elements of all 32 lanes of a warp in FP64 together and picks, per query, the FP64 minimum (ties: lowest
// index) with its FP64 distance and closest point. FP64 arithmetic is a narrow pipe on this GPU and a warp instruction
// costs the same whether one lane or 32 take part, so the evaluations are gathered into full-warp rounds instead of
// running inside each lane's divergent traversal.
//
// The band is relative 2^-14 of the distance plus 2^-18 of the coordinate scale `scale` (the largest coordinate
// magnitude of the query and the mesh): FP32 closest-point arithmetic is accurate to about 8 ulps of that scale, so the
// element that is nearest in FP64 always falls inside the band of the FP32 best. A relative band alone would not do:
// near the surface the FP32 error is absolute, not relative to the distance. Accepts elements with FP64 d2 < bound2
// (bound2 < 0: unbounded).
constexpr int F64_CAND = 8;  // band entries a lane keeps for the warp-wide FP64 step

struct F64Search {
  float cand_d[F64_CAND];  // FP32 squared distances of the kept entries (+inf: empty slot)
  int cand_k[F64_CAND];    // their sorted positions relative to the segment start (-1: empty slot)
  float lim;               // final band limit on FP32 squared distances
  float best32;            // smallest FP32 squared distance of an accepted element (+inf if none)
  // best of the entries already evaluated in FP64 by the lane itself (entries pushed out of a full list)
  double best64;
  int best_idx;
  int64_t best_slot;
  float cpx, cpy, cpz;
  bool done;               // false when the pop budget ran out before the traversal finished
};

__device__ __forceinline__ void f64_search_init(F64Search & s) {
#pragma unroll
  for (int j = 0; j < F64_CAND; ++j) {
    s.cand_d[j] = INFINITY;
    s.cand_k[j] = -1;
  }
  s.lim = INFINITY;
  s.best32 = INFINITY;
  s.best64 = INFINITY;
  s.best_idx = INT_MAX;
  s.best_slot = -1;
  s.cpx = s.cpy = s.cpz = 0.f;
  s.done = true;
}

// Folds one FP64 evaluation into the lane's best (FP64 squared distance d64, closest point cp, sorted position k)
__device__ __forceinline__ void f64_take(F64Search & s, float4 const * __restrict__ rec, int64_t k, double d64, float cx,
                                         float cy, float cz, double bound2) {
  if (bound2 >= 0.0 && !(d64 < bound2)) return;
  int idx = cp_record_index(rec, k);
  if (d64 < s.best64 || (d64 == s.best64 && idx < s.best_idx)) {
    s.best64 = d64;
    s.best_idx = idx;
    s.best_slot = k;
    s.cpx = cx;
    s.cpy = cy;
    s.cpz = cz;
  }
}

// Element tests of one leaf for the mixed-precision search: FP32 distances, band limit `lim` and FP32 best `best32`
// updated, band entries kept in s (an entry pushed out of a full list is evaluated in FP64 at once).
__device__ __forceinline__ void cp_leaf_f64(float4 const * __restrict__ rec, int64_t elem_base, int first, int count,
                                            V3 p, double bound2, float abs_tol, float & lim, float & best32,
                                            F64Search & s) {
  float const REL = 1.0f + 1.0f / 16384.0f;
  for (int kr = first; kr < first + count; ++kr) {
    V3 cp;
    float d2 = cp_record_test(rec, elem_base + kr, p, cp);
    if (!(d2 <= lim)) continue;
    if (d2 < best32) {
      best32 = d2;
      float lb1 = sqrtf(best32) * REL + abs_tol;
      lim = fminf(lim, lb1 * lb1);
    }
    // the entry takes a slot that has left the band, else the farthest slot if that is farther than it
    int slot_j = -1;
    float worst = d2;
#pragma unroll
    for (int j = 0; j < F64_CAND; ++j)
      if (slot_j < 0 && !(s.cand_k[j] >= 0 && s.cand_d[j] <= lim)) slot_j = j;
    if (slot_j < 0) {
#pragma unroll
      for (int j = 0; j < F64_CAND; ++j)
        if (s.cand_d[j] > worst) { worst = s.cand_d[j]; slot_j = j; }
    }
    int evict = slot_j < 0 ? kr : -1;
#pragma unroll
    for (int j = 0; j < F64_CAND; ++j) {
      if (j == slot_j) {
        if (s.cand_k[j] >= 0 && s.cand_d[j] <= lim) evict = s.cand_k[j];
        s.cand_d[j] = d2;
        s.cand_k[j] = kr;
      }
    }
    if (evict >= 0) {
      // more band entries than slots (rare): this one is evaluated by the lane alone
      D3 c64;
      double d64 = cp_record_f64_call(rec, elem_base + evict, p, &c64);
      f64_take(s, rec, elem_base + evict, d64, (float)c64.x, (float)c64.y, (float)c64.z, bound2);
    }
  }
}

// Band limit before any element is seen: from the distance bound (or +inf), and the band's absolute term
__device__ __forceinline__ float f64_band_start(double bound2, float scale, float & abs_tol) {
  float const REL = 1.0f + 1.0f / 16384.0f;
  abs_tol = scale * (1.0f / 262144.0f);
  float lim = bound2 >= 0.0 ? __double2float_ru(bound2) : INFINITY;
  if (bound2 >= 0.0) {
    float lb0 = sqrtf(lim) * REL + abs_tol;
    lim = lb0 * lb0;
  }
  return lim;
}

template <int W, int STACK>
__device__ __forceinline__ void closest_search_f64(WideNode<W> const * __restrict__ nodes,
                                                   float4 const * __restrict__ rec, int root, int64_t elem_base, V3 p,
                                                   double bound2, float scale, unsigned * err, F64Search & s,
                                                   int budget = 0, float4 const * __restrict__ slabs = nullptr) {
  float q1 = fabsf(p.x) + fabsf(p.y) + fabsf(p.z);
  f64_search_init(s);
  int pops = 0;
  float abs_tol;
  float lim = f64_band_start(bound2, scale, abs_tol);
  float best32 = INFINITY;
  int2 stk[STACK];  // (child code, bound bits)
  int sp = 0;
  int next = root;  // nearest child of the last node, visited without a stack round trip
  while (next != CHILD_EMPTY || sp > 0) {
    if (budget > 0 && ++pops > budget) {
      s.done = false;
      break;
    }
    int code = next;
    if (code == CHILD_EMPTY) {
      --sp;
      code = stk[sp].x;
      if (__int_as_float(stk[sp].y) > lim * PRUNE_SLACK) continue;
    }
    next = CHILD_EMPTY;
    if (code >= 0) {
      NodeRegs<W> nd;
      load_node(nodes, code, nd);
      float lb[W];
      point_child_bounds<W>(nd, p, lb);
      if (slabs) {
        float order[W];
        slab_child_bounds<W>(nd, slabs, code, p, q1, lb, order);
        push_children_ordered<W, STACK>(nd, lb, order, lim * PRUNE_SLACK, stk, sp, next, err);
      } else {
        push_children_next<W, STACK>(nd, lb, lim * PRUNE_SLACK, stk, sp, next, err);
      }
    } else {
      int first, count;
      decode_leaf(code, first, count);
      cp_leaf_f64(rec, elem_base, first, count, p, bound2, abs_tol, lim, best32, s);
    }
  }
  s.lim = lim;
  s.best32 = best32;
}

// Shared-memory work list of one warp for f64_resolve_warp
struct F64WarpBuf {
  float4 const * r[32 * F64_CAND];  // record of each entry (lanes may query different meshes)
  double d[32 * F64_CAND];
  float cp[32 * F64_CAND][3];
  float p[32][3];
  unsigned char owner[32 * F64_CAND];
};

// Evaluates in FP64 the band entries of every lane of the warp, in full-warp rounds, and folds each lane's results
// into its own F64Search. All 32 lanes call it together; `active` is false for a lane without a query (or with a
// query that is not finished), whose entries are ignored. `rec` and `elem_base` are the lane's own (lanes of one warp
// may query different meshes).
__device__ __forceinline__ void f64_resolve_warp(F64Search & s, bool active, float4 const * __restrict__ rec,
                                                 int64_t elem_base, V3 p, double bound2, F64WarpBuf & b) {
  unsigned const FULL = 0xffffffffu;
  int lane = threadIdx.x & 31;
  bool keep[F64_CAND];
  int c = 0;
#pragma unroll
  for (int j = 0; j < F64_CAND; ++j) {
    keep[j] = active && s.cand_k[j] >= 0 && s.cand_d[j] <= s.lim;
    c += keep[j] ? 1 : 0;
  }
  int incl = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(FULL, incl, o);
    if (lane >= o) incl += t;
  }
  int total = __shfl_sync(FULL, incl, 31);
  int off = incl - c;
  b.p[lane][0] = p.x;
  b.p[lane][1] = p.y;
  b.p[lane][2] = p.z;
  int w = off;
#pragma unroll
  for (int j = 0; j < F64_CAND; ++j) {
    if (keep[j]) {
      b.r[w] = rec + (elem_base + s.cand_k[j]) * CP_REC_F4;
      b.owner[w] = (unsigned char)lane;
      ++w;
    }
  }
  __syncwarp();
  for (int i = lane; i < total; i += 32) {
    int o = b.owner[i];
    V3 q = V3{b.p[o][0], b.p[o][1], b.p[o][2]};
    D3 c64;
    b.d[i] = cp_record_f64_call(b.r[i], 0, q, &c64);
    b.cp[i][0] = (float)c64.x;
    b.cp[i][1] = (float)c64.y;
    b.cp[i][2] = (float)c64.z;
  }
  __syncwarp();
  for (int i = off; i < off + c; ++i)
    f64_take(s, rec, (b.r[i] - rec) / CP_REC_F4, b.d[i], b.cp[i][0], b.cp[i][1], b.cp[i][2], bound2);
  __syncwarp();
}

__device__ __forceinline__ ClosestOut f64_result(F64Search const & s) {
  ClosestOut o;
  o.idx = s.best_idx;
  o.d2_64 = s.best64;
  o.d2 = (float)s.best64;
  o.cp = V3{s.cpx, s.cpy, s.cpz};
  o.slot = s.best_slot;
  o.best32 = s.best32;
  o.done = s.done;
  return o;
}

//============================================================================================================================
// First ray hit
//============================================================================================================================

struct RayOut {
  float t;       // FP32 reference verdict: hit time, or the initial bound when nothing was hit
  int idx;       // INT_MAX if none
  int64_t slot;
};

static __device__ __noinline__ double watertight_f64_call(V3 o, V3 d, float4 a, float4 b, float4 c) {
  return ray_triangle_watertight_f64(o, d, xyz(a), xyz(b), xyz(c));
}

// The reference's verdict: FP32 Eberly test with its parallel threshold (TriangleN<3>::rayIntersection), nearest hit
// with t >= 0 and, with a bound, t <= max_time; ties to the lowest index. (The FP64 watertight verdict is
// ray_search_f64 + ray_resolve_warp below.) The template flag is kept for the callers' signatures and must be false.
template <int W, int STACK, bool RECHECK>
__device__ __forceinline__ RayOut ray_query(WideNode<W> const * __restrict__ nodes, float4 const * __restrict__ rec,
                                            int root, int64_t elem_base, V3 o, V3 d, float max_time, unsigned * err) {
  static_assert(!RECHECK, "the FP64 re-test is ray_search_f64 + ray_resolve_warp");
  float ix = 1.0f / (fabsf(d.x) > 1e-30f ? d.x : copysignf(1e-30f, d.x));
  float iy = 1.0f / (fabsf(d.y) > 1e-30f ? d.y : copysignf(1e-30f, d.y));
  float iz = 1.0f / (fabsf(d.z) > 1e-30f ? d.z : copysignf(1e-30f, d.z));
  float ox = -o.x * ix, oy = -o.y * iy, oz = -o.z * iz;
  float best = max_time >= 0.f ? max_time : INFINITY;
  int best_idx = INT_MAX;
  int64_t best_slot = -1;
  int2 stk[STACK];  // (child code, bound bits)
  int sp = 0;
  int next = root;  // nearest child of the last node, visited without a stack round trip
  while (next != CHILD_EMPTY || sp > 0) {
    int code = next;
    if (code == CHILD_EMPTY) {
      --sp;
      code = stk[sp].x;
      if (__int_as_float(stk[sp].y) > best * PRUNE_SLACK) continue;
    }
    next = CHILD_EMPTY;
    if (code >= 0) {
      NodeRegs<W> nd;
      load_node(nodes, code, nd);
      float lb[W];
#pragma unroll
      for (int c = 0; c < W; ++c) {
        float tx0 = __fmaf_rn(nd.lox[c], ix, ox), tx1 = __fmaf_rn(nd.hix[c], ix, ox);
        float ty0 = __fmaf_rn(nd.loy[c], iy, oy), ty1 = __fmaf_rn(nd.hiy[c], iy, oy);
        float tz0 = __fmaf_rn(nd.loz[c], iz, oz), tz1 = __fmaf_rn(nd.hiz[c], iz, oz);
        float tmin = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), 0.f));
        float tmax = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fmaxf(tz0, tz1));
        lb[c] = tmin <= tmax ? tmin : __int_as_float(0x7fffffff);  // a miss: NaN passes no bound
      }
      push_children_next<W, STACK>(nd, lb, best * PRUNE_SLACK, stk, sp, next, err);
    } else {
      int first, count;
      decode_leaf(code, first, count);
      int64_t k0 = elem_base + first;
      for (int64_t k = k0; k < k0 + count; ++k) {
        float4 const * r = rec + k * RAY_REC_F4;
        float4 a = __ldg(r), b = __ldg(r + 1), c = __ldg(r + 2);
        float t = ray_triangle_time(o, d, xyz(a), xyz(b), xyz(c));
        int idx = __float_as_int(a.w);
        if (t >= 0.f && t <= best && (t < best || idx < best_idx)) {
          best = t;
          best_idx = idx;
          best_slot = k;
        }
      }
    }
  }
  RayOut out;
  out.t = best;
  out.idx = best_idx;
  out.slot = best_slot;
  return out;
}

//============================================================================================================================
// First ray hit with the FP64 watertight re-test, in two steps (the closest-point scheme above, for rays):
// ray_search_f64 runs the FP32 traversal, keeps the reference's FP32 verdict, and collects the elements whose FP64
// watertight verdict could be the nearest hit; ray_resolve_warp evaluates the collected elements of all 32 lanes in FP64
// together.
//
// Which elements are collected. Every element the FP32 test accepts or rejects within an error allowance of an edge
// (edge functions within 2^-12 of the determinant plus a bound on their FP32 rounding), every near-parallel element,
// and nothing farther than the band B. B comes from "certain" FP32 hits: accepted with every edge function at least
// 2^-10 of the determinant plus the rounding bound inside, and not grazing (angle between ray and plane above ~1.8
// degrees). The FP64 test accepts a certain hit too, at a time within relative 2^-10 plus 2^-11 |o - v0|_1 / |d|_1 of
// the FP32 time, so no element beyond B can be the FP64 nearest hit, and the traversal prunes with B.
//============================================================================================================================

constexpr int RAY_CAND = 6;

struct RaySearch64 {
  float ct[RAY_CAND];   // lower bound on each collected element's FP64 time: its FP32 hit or plane time less the
                        // time allowance (+inf: empty)
  int ck[RAY_CAND];     // sorted position relative to the segment start (-1: empty)
  unsigned keep;        // bit j: entry j is grazing and kept whatever its time estimate
  float B;              // band from certain hits (+inf if none)
  float tcap;           // max_time with its allowance (+inf if unbounded)
  // FP64 best of entries evaluated by the lane alone (a full list)
  double best64;
  int idx64;
  int64_t slot64;
  // the reference's FP32 verdict
  float t;
  int idx;
  int64_t slot;
};


__device__ __forceinline__ void ray_f64_take(RaySearch64 & s, int64_t k, int idx, double t64, float max_time) {
  if (!(t64 >= 0.0) || (max_time >= 0.f && t64 > (double)max_time)) return;
  if (t64 < s.best64 || (t64 == s.best64 && idx < s.idx64)) {
    s.best64 = t64;
    s.idx64 = idx;
    s.slot64 = k;
  }
}

__device__ __forceinline__ void ray_search_init(RaySearch64 & s, float max_time) {
#pragma unroll
  for (int j = 0; j < RAY_CAND; ++j) {
    s.ct[j] = INFINITY;
    s.ck[j] = -1;
  }
  s.keep = 0;
  s.B = INFINITY;
  s.tcap = max_time >= 0.f ? max_time + max_time * (1.0f / 1024.0f) : INFINITY;
  s.best64 = INFINITY;
  s.idx64 = INT_MAX;
  s.slot64 = -1;
  s.t = max_time >= 0.f ? max_time : INFINITY;
  s.idx = INT_MAX;
  s.slot = -1;
}

template <int W, int STACK>
__device__ __forceinline__ void ray_search_f64(WideNode<W> const * __restrict__ nodes, float4 const * __restrict__ rec,
                                               int root, int64_t elem_base, V3 o, V3 d, float max_time, unsigned * err,
                                               RaySearch64 & s) {
  float const EPS = 1.1920928955078125e-07f;
  ray_search_init(s, max_time);
  float ix = 1.0f / (fabsf(d.x) > 1e-30f ? d.x : copysignf(1e-30f, d.x));
  float iy = 1.0f / (fabsf(d.y) > 1e-30f ? d.y : copysignf(1e-30f, d.y));
  float iz = 1.0f / (fabsf(d.z) > 1e-30f ? d.z : copysignf(1e-30f, d.z));
  float ox = -o.x * ix, oy = -o.y * iy, oz = -o.z * iz;
  float nd = l1(d);
  float dd = dot(d, d);
  int2 stk[STACK];  // (child code, bound bits)
  int sp = 0;
  int next = root;  // nearest child of the last node, visited without a stack round trip
  while (next != CHILD_EMPTY || sp > 0) {
    // the FP32 verdict needs everything up to its best; the FP64 one everything up to B
    float bound = fminf(fmaxf(s.t, s.B), s.tcap);
    int code = next;
    if (code == CHILD_EMPTY) {
      --sp;
      code = stk[sp].x;
      if (__int_as_float(stk[sp].y) > bound * PRUNE_SLACK) continue;
    }
    next = CHILD_EMPTY;
    if (code >= 0) {
      NodeRegs<W> nd4;
      load_node(nodes, code, nd4);
      float lb[W];
#pragma unroll
      for (int c = 0; c < W; ++c) {
        float tx0 = __fmaf_rn(nd4.lox[c], ix, ox), tx1 = __fmaf_rn(nd4.hix[c], ix, ox);
        float ty0 = __fmaf_rn(nd4.loy[c], iy, oy), ty1 = __fmaf_rn(nd4.hiy[c], iy, oy);
        float tz0 = __fmaf_rn(nd4.loz[c], iz, oz), tz1 = __fmaf_rn(nd4.hiz[c], iz, oz);
        float tmin = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), 0.f));
        float tmax = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fmaxf(tz0, tz1));
        lb[c] = tmin <= tmax ? tmin : __int_as_float(0x7fffffff);  // a miss: NaN passes no bound
      }
      push_children_next<W, STACK>(nd4, lb, bound * PRUNE_SLACK, stk, sp, next, err);
      continue;
    }
    int first, count;
    decode_leaf(code, first, count);
    for (int kr = first; kr < first + count; ++kr) {
      int64_t k = elem_base + kr;
      float4 const * r = rec + k * RAY_REC_F4;
      float4 a = __ldg(r), b = __ldg(r + 1), c = __ldg(r + 2);
      V3 v0 = xyz(a), e01 = xyz(b), e02 = xyz(c);
      int idx = __float_as_int(a.w);
      // The reference's test (Triangle3.hpp:1466-1524: the same operations as ray_triangle_time, without its early
      // exits, whose intermediate values the classification below reuses) ...
      V3 diff = o - v0;
      V3 n = cross(e01, e02);
      float DdN = dot(d, n);
      float sg = DdN < 0.f ? -1.f : 1.f;
      float adn = fabsf(DdN);
      float e1 = sg * dot(d, cross(diff, e02));
      float e2 = sg * dot(d, cross(e01, diff));
      float t = -1.f;
      if (adn > EPS && e1 >= 0.f && e2 >= 0.f && e1 + e2 <= adn) {
        float QdN = (-sg) * dot(diff, n);
        if (QdN >= 0.f) t = QdN / adn;
      }
      // ... and its verdict (TriangleN<3>::rayIntersection: t >= 0 and, with a bound, t <= max_time)
      if (t >= 0.f && t <= s.t && (t < s.t || idx < s.idx)) {
        s.t = t;
        s.idx = idx;
        s.slot = k;
      }
      // classification for the FP64 verdict, from the same FP32 quantities. The reference's parallel threshold
      // (|D.N| <= FLT_EPSILON with N unnormalised) is a property of its FP32 test only: a small triangle seen at a
      // moderate angle is classified here by its geometry like any other.
      float nn2 = dot(n, n);
      if (!(nn2 > 0.f)) continue;  // degenerate triangle: the watertight test has no hit either
      float e3 = adn - e1 - e2;
      float ndiff = l1(diff);
      // FP32 rounding allowance of an edge function (D.(diff x e), D.(e x diff) and D.N - both)
      float le1 = l1(e01), le2 = l1(e02);
      float E = (1.0f / 262144.0f) * nd * (ndiff * (le1 + le2) + le1 * le2);
      bool grazing = DdN * DdN < (1.0f / 1024.0f) * dd * nn2;
      float emin = fminf(fminf(e1, e2), e3);
      float tabs = (1.0f / 2048.0f) * ndiff / nd;
      float te;
      if (grazing) {
        te = 0.f;  // the FP32 time is unreliable: kept whatever the band
      } else {
        float tp = t >= 0.f ? t : (-sg * dot(diff, n)) / adn;  // plane time (the reference's formula)
        if (tp < -tabs) continue;                             // behind the origin in FP64 too
        if (emin >= adn * (1.0f / 1024.0f) + E && tp >= tabs) {
          // certain: the FP64 test hits this element too, within the time allowance
          s.B = fminf(s.B, tp + tp * (1.0f / 1024.0f) + tabs);
        }
        if (!(emin >= -(adn * (1.0f / 4096.0f) + E))) continue;  // clearly outside: no FP64 hit
        te = tp - tabs;
      }
      float lim = fminf(s.B, s.tcap);
      if (!grazing && te > lim) continue;
      // the entry takes a slot that has left the band, else the farthest non-grazing slot if that is farther
      int slot_j = -1;
#pragma unroll
      for (int j = 0; j < RAY_CAND; ++j)
        if (slot_j < 0 && (s.ck[j] < 0 || (!((s.keep >> j) & 1u) && s.ct[j] > lim))) slot_j = j;
      float worst = grazing ? INFINITY : te;
      if (slot_j < 0) {
        float wv = -INFINITY;
#pragma unroll
        for (int j = 0; j < RAY_CAND; ++j)
          if (!((s.keep >> j) & 1u) && s.ct[j] > wv) { wv = s.ct[j]; slot_j = j; }
        if (slot_j >= 0 && !(wv > worst)) slot_j = -1;
      }
      int evict = slot_j < 0 ? kr : -1;
#pragma unroll
      for (int j = 0; j < RAY_CAND; ++j) {
        if (j == slot_j) {
          if (s.ck[j] >= 0 && (((s.keep >> j) & 1u) || s.ct[j] <= lim)) evict = s.ck[j];
          s.ct[j] = te;
          s.ck[j] = kr;
          s.keep = grazing ? (s.keep | (1u << j)) : (s.keep & ~(1u << j));
        }
      }
      if (evict >= 0) {
        // more entries than slots (rare): this one is evaluated by the lane alone
        float4 const * er = rec + (elem_base + evict) * RAY_REC_F4;
        float4 ea = __ldg(er), eb = __ldg(er + 1), ec = __ldg(er + 2);
        double t64 = watertight_f64_call(o, d, ea, eb, ec);
        ray_f64_take(s, elem_base + evict, __float_as_int(ea.w), t64, max_time);
      }
    }
  }
}

// Shared-memory work list of one warp for ray_resolve_warp
struct RayWarpBuf {
  float4 const * r[32 * RAY_CAND];
  double t[32 * RAY_CAND];
  float o[32][3], d[32][3];
  unsigned char owner[32 * RAY_CAND];
};

// FP64 watertight verdict over every lane's kept entries, in full-warp rounds; all 32 lanes call it together.
__device__ __forceinline__ void ray_resolve_warp(RaySearch64 & s, bool active, float4 const * __restrict__ rec,
                                                 int64_t elem_base, V3 o, V3 d, float max_time, RayWarpBuf & b) {
  unsigned const FULL = 0xffffffffu;
  int lane = threadIdx.x & 31;
  float lim = fminf(s.B, s.tcap);
  bool keepj[RAY_CAND];
  int c = 0;
#pragma unroll
  for (int j = 0; j < RAY_CAND; ++j) {
    keepj[j] = active && s.ck[j] >= 0 && (((s.keep >> j) & 1u) || s.ct[j] <= lim);
    c += keepj[j] ? 1 : 0;
  }
  int incl = c;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    int v = __shfl_up_sync(FULL, incl, off);
    if (lane >= off) incl += v;
  }
  int total = __shfl_sync(FULL, incl, 31);
  int base = incl - c;
  b.o[lane][0] = o.x;
  b.o[lane][1] = o.y;
  b.o[lane][2] = o.z;
  b.d[lane][0] = d.x;
  b.d[lane][1] = d.y;
  b.d[lane][2] = d.z;
  int w = base;
#pragma unroll
  for (int j = 0; j < RAY_CAND; ++j) {
    if (keepj[j]) {
      b.r[w] = rec + (elem_base + s.ck[j]) * RAY_REC_F4;
      b.owner[w] = (unsigned char)lane;
      ++w;
    }
  }
  __syncwarp();
  for (int i = lane; i < total; i += 32) {
    int ow = b.owner[i];
    float4 const * r = b.r[i];
    V3 oo = V3{b.o[ow][0], b.o[ow][1], b.o[ow][2]}, dd = V3{b.d[ow][0], b.d[ow][1], b.d[ow][2]};
    b.t[i] = watertight_f64_call(oo, dd, __ldg(r), __ldg(r + 1), __ldg(r + 2));
  }
  __syncwarp();
  for (int i = base; i < base + c; ++i)
    ray_f64_take(s, (b.r[i] - rec) / RAY_REC_F4, __float_as_int(__ldg(b.r[i]).w), b.t[i], max_time);
  __syncwarp();
}

//============================================================================================================================
// k nearest points
//============================================================================================================================

// Insert (d, i) into sorted register arrays, lexicographic (distance, index); the last entry falls off.
template <int K> __device__ __forceinline__ void knn_insert(float (&bd)[K], int (&bi)[K], float d, int i) {
#pragma unroll
  for (int j = 0; j < K; ++j) {
    bool lt = (d < bd[j]) || (d == bd[j] && i < bi[j]);
    float td = bd[j];
    int ti = bi[j];
    bd[j] = lt ? d : td;
    bi[j] = lt ? i : ti;
    d = lt ? td : d;
    i = lt ? ti : i;
  }
}

template <int W, int K, int STACK>
__device__ __forceinline__ void knn_query(WideNode<W> const * __restrict__ nodes, float4 const * __restrict__ pts,
                                          int root, int64_t elem_base, V3 p, int excl, float (&bd)[K], int (&bi)[K],
                                          unsigned * err) {
  int2 stk[STACK];  // (child code, bound bits)
  int sp = 0;
  int next = root;  // nearest child of the last node, visited without a stack round trip
  while (next != CHILD_EMPTY || sp > 0) {
    int code = next;
    if (code == CHILD_EMPTY) {
      --sp;
      code = stk[sp].x;
      if (__int_as_float(stk[sp].y) > bd[K - 1] * PRUNE_SLACK) continue;
    }
    next = CHILD_EMPTY;
    if (code >= 0) {
      NodeRegs<W> nd;
      load_node(nodes, code, nd);
      float lb[W];
      point_child_bounds<W>(nd, p, lb);
      push_children_next<W, STACK>(nd, lb, bd[K - 1] * PRUNE_SLACK, stk, sp, next, err);
    } else {
      int first, count;
      decode_leaf(code, first, count);
      int64_t k0 = elem_base + first;
      for (int64_t k = k0; k < k0 + count; ++k) {
        float4 a = __ldg(pts + k);
        int idx = __float_as_int(a.w);
        if (idx == excl) continue;
        // MetricL2Impl<point, point>::closestPoints: (element - query).squaredNorm()
        float d2 = squared_norm(xyz(a) - p);
        if (d2 < bd[K - 1] || (d2 == bd[K - 1] && idx < bi[K - 1])) knn_insert<K>(bd, bi, d2, idx);
      }
    }
  }
}

// knn_query with the sorted list in shared memory instead of registers: sd / si are [K][B] arrays of the block (B
// threads, entry j of thread t at [j][t], so a warp's accesses fall in distinct banks) and the k-th entry is mirrored in
// kth / kth_i for the reject test. An insertion shifts the larger entries up one place (the same (distance, index)
// order as knn_insert). Holding the lists out of registers lets twice as many warps stay resident. `elem(k, idx, d2)`
// gives element k's index and squared distance (false: skip it).
template <int W, int K, int STACK, int B, class Elem>
__device__ __forceinline__ void knn_search_shared(WideNode<W> const * __restrict__ nodes, int root, int64_t elem_base,
                                                  V3 p, int excl, float (*sd)[B], int (*si)[B], float & kth,
                                                  int & kth_i, unsigned * err, Elem elem) {
  int t = threadIdx.x;
  int2 stk[STACK];  // (child code, bound bits)
  int sp = 0;
  int next = root;
  while (next != CHILD_EMPTY || sp > 0) {
    int code = next;
    if (code == CHILD_EMPTY) {
      --sp;
      code = stk[sp].x;
      if (__int_as_float(stk[sp].y) > kth * PRUNE_SLACK) continue;
    }
    next = CHILD_EMPTY;
    if (code >= 0) {
      NodeRegs<W> nd;
      load_node(nodes, code, nd);
      float lb[W];
      point_child_bounds<W>(nd, p, lb);
      push_children_next<W, STACK>(nd, lb, kth * PRUNE_SLACK, stk, sp, next, err);
    } else {
      int first, count;
      decode_leaf(code, first, count);
      int64_t k0 = elem_base + first;
      for (int64_t k = k0; k < k0 + count; ++k) {
        int idx;
        float d2;
        if (!elem(k, idx, d2) || idx == excl) continue;
        if (d2 < kth || (d2 == kth && idx < kth_i)) {
          int j = K - 1;
          while (j > 0) {
            float dj = sd[j - 1][t];
            int ij = si[j - 1][t];
            if (dj < d2 || (dj == d2 && ij < idx)) break;
            sd[j][t] = dj;
            si[j][t] = ij;
            --j;
          }
          sd[j][t] = d2;
          si[j][t] = idx;
          kth = sd[K - 1][t];
          kth_i = si[K - 1][t];
        }
      }
    }
  }
}

// Points: MetricL2Impl<point, point>::closestPoints, (element - query).squaredNorm()
template <int W, int K, int STACK, int B>
__device__ __forceinline__ void knn_query_shared(WideNode<W> const * __restrict__ nodes,
                                                 float4 const * __restrict__ pts, int root, int64_t elem_base, V3 p,
                                                 int excl, float (*sd)[B], int (*si)[B], float & kth, int & kth_i,
                                                 unsigned * err) {
  knn_search_shared<W, K, STACK, B>(nodes, root, elem_base, p, excl, sd, si, kth, kth_i, err,
                                    [&](int64_t k, int & idx, float & d2) {
                                      float4 a = __ldg(pts + k);
                                      idx = __float_as_int(a.w);
                                      d2 = squared_norm(xyz(a) - p);
                                      return true;
                                    });
}

// Triangles: the closest-point record test (FP32 reference arithmetic); a NaN distance is never kept
template <int W, int K, int STACK, int B>
__device__ __forceinline__ void knn_mesh_query_shared(WideNode<W> const * __restrict__ nodes,
                                                      float4 const * __restrict__ rec, int root, int64_t elem_base,
                                                      V3 p, int excl, float (*sd)[B], int (*si)[B], float & kth,
                                                      int & kth_i, unsigned * err) {
  knn_search_shared<W, K, STACK, B>(nodes, root, elem_base, p, excl, sd, si, kth, kth_i, err,
                                    [&](int64_t k, int & idx, float & d2) {
                                      idx = cp_record_index(rec, k);
                                      if (idx == excl) return false;
                                      V3 cp;
                                      d2 = cp_record_test(rec, k, p, cp);
                                      return true;
                                    });
}

// k nearest triangles of a mesh BVH: the same search with the closest-point record test (FP32 reference arithmetic);
// a NaN distance (coincident vertices) is never kept
template <int W, int K, int STACK>
__device__ __forceinline__ void knn_mesh_query(WideNode<W> const * __restrict__ nodes, float4 const * __restrict__ rec,
                                               int root, int64_t elem_base, V3 p, int excl, float (&bd)[K],
                                               int (&bi)[K], unsigned * err) {
  int2 stk[STACK];  // (child code, bound bits)
  int sp = 0;
  int next = root;
  while (next != CHILD_EMPTY || sp > 0) {
    int code = next;
    if (code == CHILD_EMPTY) {
      --sp;
      code = stk[sp].x;
      if (__int_as_float(stk[sp].y) > bd[K - 1] * PRUNE_SLACK) continue;
    }
    next = CHILD_EMPTY;
    if (code >= 0) {
      NodeRegs<W> nd;
      load_node(nodes, code, nd);
      float lb[W];
      point_child_bounds<W>(nd, p, lb);
      push_children_next<W, STACK>(nd, lb, bd[K - 1] * PRUNE_SLACK, stk, sp, next, err);
    } else {
      int first, count;
      decode_leaf(code, first, count);
      int64_t k0 = elem_base + first;
      for (int64_t k = k0; k < k0 + count; ++k) {
        int idx = cp_record_index(rec, k);
        if (idx == excl) continue;
        V3 cp;
        float d2 = cp_record_test(rec, k, p, cp);
        if (d2 < bd[K - 1] || (d2 == bd[K - 1] && idx < bi[K - 1])) knn_insert<K>(bd, bi, d2, idx);
      }
    }
  }
}

}  // namespace thea
