// The any-hit ray loop (BvhN::rayIntersects) as a template over where rays come from and where verdicts go, shared by
// the occlusion query, Visibility and the sample graph's reachability test. Instantiated per translation unit.
#pragma once

#include "device_util.cuh"
#include "query.hpp"
#include "transform.hpp"
#include "traverse_ops.cuh"

#include <algorithm>
#include <cstring>

namespace thea {
namespace {

constexpr int ANY_THREADS = 128;
constexpr int ANY_WARP_BLOCK = 64;

struct Inverse {
  float m[12];
  int on;
};

// rays given as arrays (optionally mapped into object space)
struct RayArrays {
  float const * o;
  float const * d;
  Inverse inv;
  __device__ __forceinline__ void get(int64_t r, V3 & ro, V3 & rd) const {
    ro = load_v3(o + 3 * r);
    rd = load_v3(d + 3 * r);
    if (inv.on) {
      ro = affine_point(inv.m, ro);
      rd = affine_vector(inv.m, rd);
    }
  }
};

struct HitFlags {
  uint8_t * out;
  __device__ __forceinline__ void put(int64_t r, bool hit) const { out[r] = hit ? 1 : 0; }
};

template <int W, int STACK, class Src, class Sink>
__global__ void __launch_bounds__(ANY_THREADS)
any_hit_kernel(WideNode<W> const * __restrict__ nodes, float4 const * __restrict__ rec, Src src, Sink sink, int64_t n,
               float max_time, unsigned * __restrict__ err, unsigned long long * __restrict__ counter) {
  unsigned const FULL = 0xffffffffu;
  int lane = threadIdx.x & 31;
  int64_t qb = 0, qe = 0;  // warp-local block of ray ids, warp-uniform
  bool exhausted = false;  // warp-uniform
  int64_t q = -1;          // this lane's ray (-1: idle)
  V3 o = V3{0.f, 0.f, 0.f}, d = V3{0.f, 0.f, 1.f};
  float ix = 0.f, iy = 0.f, iz = 0.f, ox = 0.f, oy = 0.f, oz = 0.f;
  float const bound = max_time >= 0.f ? max_time : INFINITY;
  bool hit = false;
  int2 stk[STACK];
  int sp = 0;
  int next = CHILD_EMPTY;
  while (true) {
    unsigned idle = __ballot_sync(FULL, q < 0);
    if (idle && !exhausted) {
      if (qb >= qe) {
        unsigned long long b = 0;
        if (lane == 0) b = atomicAdd(counter, (unsigned long long)ANY_WARP_BLOCK);
        b = __shfl_sync(FULL, b, 0);
        qb = (int64_t)b;
        qe = qb + ANY_WARP_BLOCK < n ? qb + ANY_WARP_BLOCK : n;
        if (qb >= n) exhausted = true;
      }
      if (!exhausted) {
        int rank = __popc(idle & ((1u << lane) - 1));
        int take = __popc(idle);
        int64_t avail = qe - qb;
        if (q < 0 && rank < avail) {
          q = qb + rank;
          src.get(q, o, d);
          ix = 1.0f / (fabsf(d.x) > 1e-30f ? d.x : copysignf(1e-30f, d.x));
          iy = 1.0f / (fabsf(d.y) > 1e-30f ? d.y : copysignf(1e-30f, d.y));
          iz = 1.0f / (fabsf(d.z) > 1e-30f ? d.z : copysignf(1e-30f, d.z));
          ox = -o.x * ix;
          oy = -o.y * iy;
          oz = -o.z * iz;
          hit = false;
          sp = 0;
          next = 0;
        }
        qb += take < avail ? take : avail;
      }
    }
    if (__ballot_sync(FULL, q >= 0) == 0) break;
    if (q < 0) continue;
    int code = next;
    if (hit || (code == CHILD_EMPTY && sp == 0)) {
      sink.put(q, hit);
      q = -1;
      continue;
    }
    if (code == CHILD_EMPTY) code = stk[--sp].x;  // entries were pushed within the fixed bound
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
      push_children_next<W, STACK>(nd, lb, bound * PRUNE_SLACK, stk, sp, next, err);
    } else {
      int first, count;
      decode_leaf(code, first, count);
      for (int64_t k = first; k < first + count; ++k) {
        float4 const * r = rec + k * RAY_REC_F4;
        float t = ray_triangle_time(o, d, xyz(__ldg(r)), xyz(__ldg(r + 1)), xyz(__ldg(r + 2)));
        // TriangleN<3>::rayIntersection: a hit at t >= 0, and t <= max_time when bounded
        if (t >= 0.f && t <= bound) {
          hit = true;
          break;
        }
      }
    }
  }
}

template <int W, int STACK, class Src, class Sink>
void launch_any(thea_bvh const * b, Src const & src, Sink const & sink, int64_t n, float max_time, cudaStream_t s) {
  auto k = any_hit_kernel<W, STACK, Src, Sink>;
  int per_sm = 0;
  THEA_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, ANY_THREADS, 0));
  int64_t need = ceil_div(ceil_div(n, ANY_WARP_BLOCK) * 32, ANY_THREADS);
  unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((int64_t)std::max(1, per_sm) * sm_count(), need));
  Scratch counter(sizeof(unsigned long long), s);
  THEA_CUDA_CHECK(cudaMemsetAsync(counter.ptr, 0, sizeof(unsigned long long), s));
  THEA_LAUNCH_NAMED("any_hit_kernel", k, grid, ANY_THREADS, 0, s, (WideNode<W> const *)b->nodes, b->ray_rec, src, sink,
                    n, max_time, b->err, counter.as<unsigned long long>());
}

template <class Src, class Sink>
void dispatch_any(thea_bvh const * b, Src const & src, Sink const & sink, int64_t n, float max_time, cudaStream_t s) {
  bool sm = small_stack_ok(b);
  if (b->width == 4) sm ? launch_any<4, 64>(b, src, sink, n, max_time, s) : launch_any<4, 256>(b, src, sink, n, max_time, s);
  else sm ? launch_any<8, 128>(b, src, sink, n, max_time, s) : launch_any<8, 512>(b, src, sink, n, max_time, s);
}

Inverse inverse_of(thea_bvh const * b) {
  Inverse v;
  std::memcpy(v.m, b->xf_inv, sizeof(v.m));
  v.on = b->has_transform;
  return v;
}

}  // namespace
}  // namespace thea
