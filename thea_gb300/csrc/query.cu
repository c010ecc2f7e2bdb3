// Query kernels: closest element of a mesh, first ray hit, k nearest points. One thread per query walks the wide BVH
// with a per-thread stack of (node or leaf code, lower bound), nearest-first; each element test reproduces the
// reference's FP32 arithmetic and the best element is kept under the lowest-index tie rule.
#include "bvh.hpp"
#include "query.hpp"
#include "traverse.cuh"

namespace thea {
namespace {

constexpr int QUERY_THREADS = 128;

//============================================================================================================================
// Closest element (BvhN::closestPair -> processNeighbors -> TriangleN<3>::closestPoint; BvhN.hpp:1082-1114, 1868-1893,
// 2038-2089; Triangle3.hpp:294-304)
//============================================================================================================================

// Squared distance and closest point of record k; `idx` receives the element index only when it is needed for a tie.
__device__ __forceinline__ float cp_record_test(float4 const * __restrict__ rec, int k, V3 p, V3 & cp) {
  float4 const * r = rec + (int64_t)k * CP_REC_F4;
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

template <int W, int STACK>
__global__ void __launch_bounds__(QUERY_THREADS)
closest_kernel(WideNode<W> const * __restrict__ nodes, float4 const * __restrict__ rec, float const * __restrict__ queries,
               int64_t n, float thresh, int32_t * __restrict__ out_index, float * __restrict__ out_dist,
               float * __restrict__ out_cp, unsigned * __restrict__ err) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  V3 p = load_v3(queries + 3 * q);
  float best = thresh;  // accept d2 <= thresh (thresh = +inf when unbounded)
  int best_idx = INT_MAX;
  V3 best_cp = V3{0.f, 0.f, 0.f};
  int stk[STACK];
  float stkd[STACK];
  int sp = 0;
  stk[sp] = 0;
  stkd[sp] = 0.f;
  ++sp;
  while (sp > 0) {
    --sp;
    int code = stk[sp];
    if (stkd[sp] > best * PRUNE_SLACK) continue;
    if (code >= 0) {
      NodeRegs<W> nd;
      load_node(nodes, code, nd);
      uint32_t key[W];
      int cc[W];
#pragma unroll
      for (int c = 0; c < W; ++c) {
        float d2 = point_box_d2(p.x, p.y, p.z, nd.lox[c], nd.loy[c], nd.loz[c], nd.hix[c], nd.hiy[c], nd.hiz[c]);
        bool keep = nd.child[c] != CHILD_EMPTY && d2 <= best * PRUNE_SLACK;
        key[c] = keep ? __float_as_uint(d2) : 0xffffffffu;
        cc[c] = nd.child[c];
      }
      sort_children<W>(key, cc);
#pragma unroll
      for (int c = W - 1; c >= 0; --c) {
        if (key[c] != 0xffffffffu) {
          if (sp < STACK) {
            stk[sp] = cc[c];
            stkd[sp] = __uint_as_float(key[c]);
            ++sp;
          } else {
            atomicOr(err, ERR_STACK_OVERFLOW);
          }
        }
      }
    } else {
      int first, count;
      decode_leaf(code, first, count);
      for (int k = first; k < first + count; ++k) {
        V3 cp;
        float d2 = cp_record_test(rec, k, p, cp);
        if (d2 <= best) {
          int idx = __float_as_int(__ldg(rec + (int64_t)k * CP_REC_F4 + 5).w);
          if (d2 < best || idx < best_idx) {
            best = d2;
            best_idx = idx;
            best_cp = cp;
          }
        }
      }
    }
  }
  bool found = best_idx != INT_MAX;
  out_index[q] = found ? best_idx : -1;
  if (out_dist) out_dist[q] = found ? sqrtf(best) : -1.f;
  if (out_cp) {
    out_cp[3 * q] = found ? best_cp.x : 0.f;
    out_cp[3 * q + 1] = found ? best_cp.y : 0.f;
    out_cp[3 * q + 2] = found ? best_cp.z : 0.f;
  }
}

//============================================================================================================================
// First ray hit (BvhN::rayStructureIntersection, BvhN.hpp:1292-1316, 2241-2291; TriangleN<3>::rayIntersection,
// Triangle3.hpp:542-552 -> rayTriangleIntersectionTime, Triangle3.hpp:1466-1524)
//============================================================================================================================

template <int W, int STACK>
__global__ void __launch_bounds__(QUERY_THREADS)
ray_kernel(WideNode<W> const * __restrict__ nodes, float4 const * __restrict__ rec, float const * __restrict__ origins,
           float const * __restrict__ dirs, int64_t n, float max_time, float * __restrict__ out_time,
           int32_t * __restrict__ out_index, float * __restrict__ out_normal, unsigned * __restrict__ err) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  V3 o = load_v3(origins + 3 * q);
  V3 d = load_v3(dirs + 3 * q);
  // slab test on padded boxes with a finite inverse direction
  float ix = 1.0f / (fabsf(d.x) > 1e-30f ? d.x : copysignf(1e-30f, d.x));
  float iy = 1.0f / (fabsf(d.y) > 1e-30f ? d.y : copysignf(1e-30f, d.y));
  float iz = 1.0f / (fabsf(d.z) > 1e-30f ? d.z : copysignf(1e-30f, d.z));
  float ox = -o.x * ix, oy = -o.y * iy, oz = -o.z * iz;
  float best = max_time >= 0.f ? max_time : INFINITY;
  int best_idx = INT_MAX;
  int best_slot = -1;
  int stk[STACK];
  float stkd[STACK];
  int sp = 0;
  stk[sp] = 0;
  stkd[sp] = 0.f;
  ++sp;
  while (sp > 0) {
    --sp;
    int code = stk[sp];
    if (stkd[sp] > best * PRUNE_SLACK) continue;
    if (code >= 0) {
      NodeRegs<W> nd;
      load_node(nodes, code, nd);
      uint32_t key[W];
      int cc[W];
#pragma unroll
      for (int c = 0; c < W; ++c) {
        float tx0 = __fmaf_rn(nd.lox[c], ix, ox), tx1 = __fmaf_rn(nd.hix[c], ix, ox);
        float ty0 = __fmaf_rn(nd.loy[c], iy, oy), ty1 = __fmaf_rn(nd.hiy[c], iy, oy);
        float tz0 = __fmaf_rn(nd.loz[c], iz, oz), tz1 = __fmaf_rn(nd.hiz[c], iz, oz);
        float tmin = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), 0.f));
        float tmax = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fmaxf(tz0, tz1));
        bool keep = nd.child[c] != CHILD_EMPTY && tmin <= tmax && tmin <= best * PRUNE_SLACK;
        key[c] = keep ? __float_as_uint(tmin) : 0xffffffffu;
        cc[c] = nd.child[c];
      }
      sort_children<W>(key, cc);
#pragma unroll
      for (int c = W - 1; c >= 0; --c) {
        if (key[c] != 0xffffffffu) {
          if (sp < STACK) {
            stk[sp] = cc[c];
            stkd[sp] = __uint_as_float(key[c]);
            ++sp;
          } else {
            atomicOr(err, ERR_STACK_OVERFLOW);
          }
        }
      }
    } else {
      int first, count;
      decode_leaf(code, first, count);
      for (int k = first; k < first + count; ++k) {
        float4 const * r = rec + (int64_t)k * RAY_REC_F4;
        float4 a = __ldg(r), b = __ldg(r + 1), c = __ldg(r + 2);
        float t = ray_triangle_time(o, d, xyz(a), xyz(b), xyz(c));
        // TriangleN<3>::rayIntersection accepts t >= 0 and, with a bound, t <= max_time
        if (t >= 0.f && t <= best) {
          int idx = __float_as_int(a.w);
          if (t < best || idx < best_idx) {
            best = t;
            best_idx = idx;
            best_slot = k;
          }
        }
      }
    }
  }
  bool found = best_idx != INT_MAX;
  out_time[q] = found ? best : -1.f;
  if (out_index) out_index[q] = found ? best_idx : -1;
  if (out_normal) {
    V3 nn = V3{0.f, 0.f, 0.f};
    if (found) {
      float4 const * r = rec + (int64_t)best_slot * RAY_REC_F4;
      nn = normalized(cross(xyz(__ldg(r + 1)), xyz(__ldg(r + 2))));
    }
    out_normal[3 * q] = nn.x;
    out_normal[3 * q + 1] = nn.y;
    out_normal[3 * q + 2] = nn.z;
  }
}

//============================================================================================================================
// k nearest points (BvhN::kClosestPairs + KClosestPairsFunctor + BoundedSortedArrayN; BvhN.hpp:474-500, 1139-1146;
// BoundedSortedArrayN.hpp:137-214)
//============================================================================================================================

// Insert (d, i) into the sorted register arrays, lexicographic (distance, index); the last entry falls off.
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
__global__ void __launch_bounds__(QUERY_THREADS)
knn_kernel(WideNode<W> const * __restrict__ nodes, float4 const * __restrict__ pts, float const * __restrict__ queries,
           int64_t n, int k_out, float thresh, int32_t const * __restrict__ exclude, int32_t * __restrict__ out_index,
           float * __restrict__ out_d2, unsigned * __restrict__ err) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  V3 p;
  int excl;
  int64_t row;
  if (queries) {
    p = load_v3(queries + 3 * q);
    excl = exclude ? exclude[q] : -1;
    row = q;
  } else {
    // self mode: query q is the point at leaf position q, excluding itself; its row is its element index
    float4 a = __ldg(pts + q);
    p = xyz(a);
    excl = __float_as_int(a.w);
    row = excl;
  }
  float bd[K];
  int bi[K];
#pragma unroll
  for (int j = 0; j < K; ++j) { bd[j] = thresh; bi[j] = INT_MAX; }
  int stk[STACK];
  float stkd[STACK];
  int sp = 0;
  stk[sp] = 0;
  stkd[sp] = 0.f;
  ++sp;
  while (sp > 0) {
    --sp;
    int code = stk[sp];
    if (stkd[sp] > bd[K - 1] * PRUNE_SLACK) continue;
    if (code >= 0) {
      NodeRegs<W> nd;
      load_node(nodes, code, nd);
      uint32_t key[W];
      int cc[W];
      float lim = bd[K - 1] * PRUNE_SLACK;
#pragma unroll
      for (int c = 0; c < W; ++c) {
        float d2 = point_box_d2(p.x, p.y, p.z, nd.lox[c], nd.loy[c], nd.loz[c], nd.hix[c], nd.hiy[c], nd.hiz[c]);
        bool keep = nd.child[c] != CHILD_EMPTY && d2 <= lim;
        key[c] = keep ? __float_as_uint(d2) : 0xffffffffu;
        cc[c] = nd.child[c];
      }
      sort_children<W>(key, cc);
#pragma unroll
      for (int c = W - 1; c >= 0; --c) {
        if (key[c] != 0xffffffffu) {
          if (sp < STACK) {
            stk[sp] = cc[c];
            stkd[sp] = __uint_as_float(key[c]);
            ++sp;
          } else {
            atomicOr(err, ERR_STACK_OVERFLOW);
          }
        }
      }
    } else {
      int first, count;
      decode_leaf(code, first, count);
      for (int k = first; k < first + count; ++k) {
        float4 a = __ldg(pts + k);
        int idx = __float_as_int(a.w);
        if (idx == excl) continue;
        // MetricL2Impl<point, point>::closestPoints: (element - query).squaredNorm()
        float d2 = squared_norm(xyz(a) - p);
        if (d2 < bd[K - 1] || (d2 == bd[K - 1] && idx < bi[K - 1])) knn_insert<K>(bd, bi, d2, idx);
      }
    }
  }
  for (int j = 0; j < k_out; ++j) {
    bool v = bi[j] != INT_MAX;
    out_index[row * k_out + j] = v ? bi[j] : -1;
    out_d2[row * k_out + j] = v ? bd[j] : -1.f;
  }
}

template <int W, int STACK>
void launch_closest(thea_bvh const * b, float const * q, int64_t n, float thresh, int32_t * idx, float * dist,
                    float * cp, unsigned * err, cudaStream_t s) {
  THEA_LAUNCH((closest_kernel<W, STACK>), (unsigned)ceil_div(n, QUERY_THREADS), QUERY_THREADS, 0, s,
              (WideNode<W> const *)b->nodes, b->cp_rec, q, n, thresh, idx, dist, cp, err);
}

template <int W, int STACK>
void launch_ray(thea_bvh const * b, float const * o, float const * d, int64_t n, float max_time, float * t,
                int32_t * idx, float * nrm, unsigned * err, cudaStream_t s) {
  THEA_LAUNCH((ray_kernel<W, STACK>), (unsigned)ceil_div(n, QUERY_THREADS), QUERY_THREADS, 0, s,
              (WideNode<W> const *)b->nodes, b->ray_rec, o, d, n, max_time, t, idx, nrm, err);
}

template <int W, int K, int STACK>
void launch_knn_k(thea_bvh const * b, float const * q, int64_t n, int k, float thresh, int32_t const * ex,
                  int32_t * idx, float * d2, unsigned * err, cudaStream_t s) {
  THEA_LAUNCH((knn_kernel<W, K, STACK>), (unsigned)ceil_div(n, QUERY_THREADS), QUERY_THREADS, 0, s,
              (WideNode<W> const *)b->nodes, b->pt_rec, q, n, k, thresh, ex, idx, d2, err);
}

template <int W, int STACK>
void launch_knn(thea_bvh const * b, float const * q, int64_t n, int k, float thresh, int32_t const * ex, int32_t * idx,
                float * d2, unsigned * err, cudaStream_t s) {
  if (k <= 1) launch_knn_k<W, 1, STACK>(b, q, n, k, thresh, ex, idx, d2, err, s);
  else if (k <= 2) launch_knn_k<W, 2, STACK>(b, q, n, k, thresh, ex, idx, d2, err, s);
  else if (k <= 4) launch_knn_k<W, 4, STACK>(b, q, n, k, thresh, ex, idx, d2, err, s);
  else if (k <= 8) launch_knn_k<W, 8, STACK>(b, q, n, k, thresh, ex, idx, d2, err, s);
  else if (k <= 16) launch_knn_k<W, 16, STACK>(b, q, n, k, thresh, ex, idx, d2, err, s);
  else launch_knn_k<W, 32, STACK>(b, q, n, k, thresh, ex, idx, d2, err, s);
}

}  // namespace

// Stack entries needed by a tree of the handle's depth: D * (W - 1) + 1
static bool small_stack_ok(thea_bvh const * b) {
  int need = b->depth * (b->width - 1) + 1;
  return need <= (b->width == 4 ? 64 : 128);
}

void run_closest(thea_bvh const * b, float const * q, int64_t n, float thresh, int32_t * idx, float * dist, float * cp,
                 unsigned * err, cudaStream_t s) {
  if (n <= 0) return;
  bool sm = small_stack_ok(b);
  if (b->width == 4) sm ? launch_closest<4, 64>(b, q, n, thresh, idx, dist, cp, err, s)
                        : launch_closest<4, 256>(b, q, n, thresh, idx, dist, cp, err, s);
  else sm ? launch_closest<8, 128>(b, q, n, thresh, idx, dist, cp, err, s)
          : launch_closest<8, 512>(b, q, n, thresh, idx, dist, cp, err, s);
}

void run_ray(thea_bvh const * b, float const * o, float const * d, int64_t n, float max_time, float * t, int32_t * idx,
             float * nrm, unsigned * err, cudaStream_t s) {
  if (n <= 0) return;
  bool sm = small_stack_ok(b);
  if (b->width == 4) sm ? launch_ray<4, 64>(b, o, d, n, max_time, t, idx, nrm, err, s)
                        : launch_ray<4, 256>(b, o, d, n, max_time, t, idx, nrm, err, s);
  else sm ? launch_ray<8, 128>(b, o, d, n, max_time, t, idx, nrm, err, s)
          : launch_ray<8, 512>(b, o, d, n, max_time, t, idx, nrm, err, s);
}

void run_knn(thea_bvh const * b, float const * q, int64_t n, int k, float thresh, int32_t const * ex, int32_t * idx,
             float * d2, unsigned * err, cudaStream_t s) {
  if (n <= 0) return;
  bool sm = small_stack_ok(b);
  if (b->width == 4) sm ? launch_knn<4, 64>(b, q, n, k, thresh, ex, idx, d2, err, s)
                        : launch_knn<4, 256>(b, q, n, k, thresh, ex, idx, d2, err, s);
  else sm ? launch_knn<8, 128>(b, q, n, k, thresh, ex, idx, d2, err, s)
          : launch_knn<8, 512>(b, q, n, k, thresh, ex, idx, d2, err, s);
}

}  // namespace thea
