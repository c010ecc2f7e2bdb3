// Single-BVH query kernels: closest element of a mesh, first ray hit, k nearest points. One thread per query; the
// traversal routines live in traverse_ops.cuh and are shared with the batched kernels.
#include "bvh.hpp"
#include "device_util.cuh"
#include "query.hpp"
#include "transform.hpp"
#include "traverse_ops.cuh"
#include "batch.hpp"

#include <algorithm>

namespace thea {
namespace {

constexpr int QUERY_THREADS = 128;

//============================================================================================================================
// Closest element (BvhN::closestPair -> processNeighbors -> TriangleN<3>::closestPoint; BvhN.hpp:1082-1114, 1868-1893,
// 2038-2089; Triangle3.hpp:294-304)
//============================================================================================================================

template <int W, int STACK, int PREC>
__global__ void __launch_bounds__(QUERY_THREADS)
closest_kernel(WideNode<W> const * __restrict__ nodes, float4 const * __restrict__ rec, float const * __restrict__ queries,
               int64_t n, float thresh, double bound2, float scene_scale, int32_t * __restrict__ out_index,
               float * __restrict__ out_dist, float * __restrict__ out_cp, float * __restrict__ out_err,
               unsigned * __restrict__ err, uint32_t const * __restrict__ order, float4 const * __restrict__ slabs) {
  // no early exit: the FP64 step and the error estimate run with the warp's lanes together
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool active = q < n;
  if (active && order) q = order[q];
  V3 p = active ? load_v3(queries + 3 * q) : V3{0.f, 0.f, 0.f};
  ClosestOut r;
  r.idx = INT_MAX;
  r.d2 = 0.f;
  r.d2_64 = 0.0;
  r.slot = -1;
  float dist = 0.f;
  if constexpr (PREC == THEA_PRECISION_FP64_RECHECK) {
    __shared__ F64WarpBuf buf[QUERY_THREADS / 32];
    float scale = fmaxf(scene_scale, fmaxf(fabsf(p.x), fmaxf(fabsf(p.y), fabsf(p.z))));
    F64Search s;
    if (active) closest_search_f64<W, STACK>(nodes, rec, 0, 0, p, bound2, scale, err, s, 0, slabs);
    else f64_search_init(s);
    f64_resolve_warp(s, active, rec, 0, p, bound2, buf[threadIdx.x >> 5]);
    r = f64_result(s);
    dist = (float)sqrt(r.d2_64);
  } else {
    if (active) r = closest_query<W, STACK>(nodes, rec, 0, 0, p, thresh, err, 0, slabs);
    dist = sqrtf(r.d2);
  }
  bool found = r.idx != INT_MAX;
  double d64 = r.d2_64;
  if (PREC != THEA_PRECISION_FP64_RECHECK && out_err) {
    // FP64 distance of the returned element, evaluated with the warp's lanes together
    __syncwarp();
    if (active && found) {
      D3 cp64;
      cp_record_f64(rec, r.slot, p, cp64, d64);
    }
  }
  if (!active) return;
  out_index[q] = found ? r.idx : -1;
  if (out_dist) out_dist[q] = found ? dist : -1.f;
  if (out_cp) {
    out_cp[3 * q] = found ? r.cp.x : 0.f;
    out_cp[3 * q + 1] = found ? r.cp.y : 0.f;
    out_cp[3 * q + 2] = found ? r.cp.z : 0.f;
  }
  // |returned distance - FP64 distance of the returned element|
  if (out_err) out_err[q] = found ? (float)fabs((double)dist - sqrt(d64)) : -1.f;
}

//============================================================================================================================
// First ray hit (BvhN::rayStructureIntersection, BvhN.hpp:1292-1316, 2241-2291; TriangleN<3>::rayIntersection,
// Triangle3.hpp:542-552 -> rayTriangleIntersectionTime, Triangle3.hpp:1466-1524)
//============================================================================================================================

template <int W, int STACK, bool RECHECK>
__device__ __forceinline__ void ray_body(WideNode<W> const * __restrict__ nodes, float4 const * __restrict__ rec, float const * __restrict__ origins,
           float const * __restrict__ dirs, int64_t n, float max_time, float * __restrict__ out_time,
           int32_t * __restrict__ out_index, float * __restrict__ out_normal, float * __restrict__ out_time64,
           int32_t * __restrict__ out_index64, int32_t * __restrict__ out_flags, unsigned * __restrict__ err,
           uint32_t const * __restrict__ order) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float t;
  int idx;
  int64_t slot;
  double t64 = 0.0;
  int idx64 = INT_MAX;
  if constexpr (RECHECK) {
    // no early exit: the FP64 step runs with the warp's lanes together
    __shared__ RayWarpBuf buf[QUERY_THREADS / 32];
    bool active = q < n;
    if (active && order) q = order[q];
    V3 o = active ? load_v3(origins + 3 * q) : V3{0.f, 0.f, 1.f};
    V3 d = active ? load_v3(dirs + 3 * q) : V3{0.f, 0.f, 1.f};
    RaySearch64 s;
    if (active) ray_search_f64<W, STACK>(nodes, rec, 0, 0, o, d, max_time, err, s);
    else ray_search_init(s, max_time);
    ray_resolve_warp(s, active, rec, 0, o, d, max_time, buf[threadIdx.x >> 5]);
    if (!active) return;
    t = s.t;
    idx = s.idx;
    slot = s.slot;
    t64 = s.best64;
    idx64 = s.idx64;
  } else {
    if (q >= n) return;
    if (order) q = order[q];
    RayOut r = ray_query<W, STACK, false>(nodes, rec, 0, 0, load_v3(origins + 3 * q), load_v3(dirs + 3 * q), max_time,
                                          err);
    t = r.t;
    idx = r.idx;
    slot = r.slot;
  }
  bool found = idx != INT_MAX;
  out_time[q] = found ? t : -1.f;
  if (out_index) out_index[q] = found ? idx : -1;
  if (out_normal) {
    V3 nn = V3{0.f, 0.f, 0.f};
    if (found) {
      float4 const * rr = rec + slot * RAY_REC_F4;
      nn = normalized(cross(xyz(__ldg(rr + 1)), xyz(__ldg(rr + 2))));
    }
    out_normal[3 * q] = nn.x;
    out_normal[3 * q + 1] = nn.y;
    out_normal[3 * q + 2] = nn.z;
  }
  if (RECHECK) {
    bool f64 = idx64 != INT_MAX;
    if (out_time64) out_time64[q] = f64 ? (float)t64 : -1.f;
    if (out_index64) out_index64[q] = f64 ? idx64 : -1;
    if (out_flags) out_flags[q] = (found != f64 ? THEA_RAY_FLAG_HIT_DIFFERS : 0) |
                                  (found && f64 && idx != idx64 ? THEA_RAY_FLAG_ELEMENT_DIFFERS : 0);
  }
}

template <int W, int STACK, bool RECHECK>
__global__ void __launch_bounds__(QUERY_THREADS)
ray_kernel(WideNode<W> const * __restrict__ nodes, float4 const * __restrict__ rec, float const * __restrict__ origins,
           float const * __restrict__ dirs, int64_t n, float max_time, float * __restrict__ out_time,
           int32_t * __restrict__ out_index, float * __restrict__ out_normal, float * __restrict__ out_time64,
           int32_t * __restrict__ out_index64, int32_t * __restrict__ out_flags, unsigned * __restrict__ err,
           uint32_t const * __restrict__ order) {
  ray_body<W, STACK, false>(nodes, rec, origins, dirs, n, max_time, out_time, out_index, out_normal, out_time64,
                            out_index64, out_flags, err, order);
}

// The FP64 re-check form: register use capped so that five blocks of 128 threads fit on an SM
template <int W, int STACK>
__global__ void __launch_bounds__(QUERY_THREADS, 5)
ray_recheck_kernel(WideNode<W> const * __restrict__ nodes, float4 const * __restrict__ rec,
                   float const * __restrict__ origins, float const * __restrict__ dirs, int64_t n, float max_time,
                   float * __restrict__ out_time, int32_t * __restrict__ out_index, float * __restrict__ out_normal,
                   float * __restrict__ out_time64, int32_t * __restrict__ out_index64, int32_t * __restrict__ out_flags,
                   unsigned * __restrict__ err, uint32_t const * __restrict__ order) {
  ray_body<W, STACK, true>(nodes, rec, origins, dirs, n, max_time, out_time, out_index, out_normal, out_time64,
                           out_index64, out_flags, err, order);
}

// Persistent form of ray_kernel for large batches (FP32 verdict only). Rays that leave the mesh after a few nodes and
// rays that traverse deep share warps; with one ray per thread the finished lanes idle until their warp's last ray is
// done. Here each lane takes a new ray as soon as its ray finishes: every loop iteration advances each busy lane by one
// stack entry, and idle lanes are refilled from a warp-local block of 64 rays (one atomic per block). Results are the
// same as ray_kernel's: each ray's traversal is the same sequence of steps. (Measured on the 2 M-triangle heightfield:
// skipping pruned entries in an inner loop, or postponing leaves so that node steps run converged, were both slower,
// since a lane's extra steps then stall its whole warp; keeping the nearest child in a register and packing stack
// entries into 8 bytes gained 4.5 %.)
constexpr int RAY_WARP_BLOCK = 64;
constexpr int64_t RAY_PERSISTENT_MIN = 1 << 16;

template <int W, int STACK>
__global__ void __launch_bounds__(QUERY_THREADS)
ray_persistent_kernel(WideNode<W> const * __restrict__ nodes, float4 const * __restrict__ rec,
                      float const * __restrict__ origins, float const * __restrict__ dirs, int64_t n, float max_time,
                      float * __restrict__ out_time, int32_t * __restrict__ out_index, float * __restrict__ out_normal,
                      unsigned * __restrict__ err, uint32_t const * __restrict__ order,
                      unsigned long long * __restrict__ counter) {
  unsigned const FULL = 0xffffffffu;
  int lane = threadIdx.x & 31;
  int64_t qb = 0, qe = 0;  // warp-local block of ray ids [qb, qe), warp-uniform
  bool exhausted = false;  // warp-uniform
  int64_t q = -1;          // this lane's ray (-1: idle)
  V3 o = V3{0.f, 0.f, 0.f};
  float ix = 0.f, iy = 0.f, iz = 0.f, ox = 0.f, oy = 0.f, oz = 0.f;
  V3 d = V3{0.f, 0.f, 1.f};
  float best = 0.f;
  int best_idx = INT_MAX;
  int64_t best_slot = -1;
  int2 stk[STACK];  // (child code, bit pattern of its entry-time lower bound): one 8-byte access per push and pop
  int sp = 0;
  int next = CHILD_EMPTY;  // the nearest child of the last node: visited next without a stack round trip
  while (true) {
    unsigned idle = __ballot_sync(FULL, q < 0);
    if (idle && !exhausted) {
      if (qb >= qe) {
        unsigned long long b = 0;
        if (lane == 0) b = atomicAdd(counter, (unsigned long long)RAY_WARP_BLOCK);
        b = __shfl_sync(FULL, b, 0);
        qb = (int64_t)b;
        qe = qb + RAY_WARP_BLOCK < n ? qb + RAY_WARP_BLOCK : n;
        if (qb >= n) exhausted = true;
      }
      if (!exhausted) {
        int rank = __popc(idle & ((1u << lane) - 1));
        int take = __popc(idle);
        int64_t avail = qe - qb;
        if (q < 0 && rank < avail) {
          q = qb + rank;
          int64_t r = order ? (int64_t)order[q] : q;
          q = r;
          o = load_v3(origins + 3 * r);
          d = load_v3(dirs + 3 * r);
          ix = 1.0f / (fabsf(d.x) > 1e-30f ? d.x : copysignf(1e-30f, d.x));
          iy = 1.0f / (fabsf(d.y) > 1e-30f ? d.y : copysignf(1e-30f, d.y));
          iz = 1.0f / (fabsf(d.z) > 1e-30f ? d.z : copysignf(1e-30f, d.z));
          ox = -o.x * ix;
          oy = -o.y * iy;
          oz = -o.z * iz;
          best = max_time >= 0.f ? max_time : INFINITY;
          best_idx = INT_MAX;
          best_slot = -1;
          sp = 0;
          next = 0;  // the root
        }
        qb += take < avail ? take : avail;
      }
    }
    if (__ballot_sync(FULL, q >= 0) == 0) break;
    if (q < 0) continue;
    int code = next;
    if (code == CHILD_EMPTY) {
      if (sp == 0) {
        // finished: the same outputs as ray_kernel
        bool found = best_idx != INT_MAX;
        out_time[q] = found ? best : -1.f;
        if (out_index) out_index[q] = found ? best_idx : -1;
        if (out_normal) {
          V3 nn = V3{0.f, 0.f, 0.f};
          if (found) {
            float4 const * rr = rec + best_slot * RAY_REC_F4;
            nn = normalized(cross(xyz(__ldg(rr + 1)), xyz(__ldg(rr + 2))));
          }
          out_normal[3 * q] = nn.x;
          out_normal[3 * q + 1] = nn.y;
          out_normal[3 * q + 2] = nn.z;
        }
        q = -1;
        continue;
      }
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
      // nearest child next (it would be on top of the stack), the others pushed farthest first
      push_children_next<W, STACK>(nd, lb, best * PRUNE_SLACK, stk, sp, next, err);
    } else {
      int first, count;
      decode_leaf(code, first, count);
      for (int64_t k = first; k < first + count; ++k) {
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
}

// Host-resident form of ray_persistent_kernel, for rays and results in pinned host memory read and written by the
// kernel itself (Grace-Blackwell reaches host memory coherently over NVLink-C2C). Instead of staging the batch through
// device buffers in chunks (each launch then ends with its own tail of long rays), one launch covers the batch: a warp
// copies each 64-ray block into shared memory once when it takes the block (one wait per block instead of one per ray),
// and results go to a per-warp ring of block buffers in shared memory that are written out, in ray order and with
// coalesced stores, once every ray of the block is done. A warp takes a new block only when a ring slot is free; the
// lanes then idle until their warp's oldest block completes, which always happens because its rays are in flight on
// lanes of the same warp. Time and index only (the normal variant keeps the staged path).
constexpr int STREAM_RING = 4;
constexpr int STREAM_WARPS = QUERY_THREADS / 32;

template <int W, int STACK>
__global__ void __launch_bounds__(QUERY_THREADS)
ray_stream_kernel(WideNode<W> const * __restrict__ nodes, float4 const * __restrict__ rec,
                  float const * __restrict__ origins, float const * __restrict__ dirs, int64_t n, float max_time,
                  float * __restrict__ out_time, int32_t * __restrict__ out_index, unsigned * __restrict__ err,
                  unsigned long long * __restrict__ counter) {
  __shared__ float s_in[STREAM_WARPS][RAY_WARP_BLOCK * 6];
  __shared__ float s_t[STREAM_WARPS][STREAM_RING][RAY_WARP_BLOCK];
  __shared__ int s_i[STREAM_WARPS][STREAM_RING][RAY_WARP_BLOCK];
  __shared__ int s_left[STREAM_WARPS][STREAM_RING];
  __shared__ long long s_base[STREAM_WARPS][STREAM_RING];
  __shared__ int s_cnt[STREAM_WARPS][STREAM_RING];
  unsigned const FULL = 0xffffffffu;
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float * in = s_in[warp];
  int64_t qb = 0, qe = 0;   // rays of the current block not yet handed out, warp-uniform
  bool exhausted = false;   // warp-uniform
  long long taken = 0;      // blocks taken by this warp, warp-uniform
  long long oldest = 0;     // oldest block not written out yet, warp-uniform
  int64_t q = -1;           // this lane's ray (-1: idle)
  int slot = 0;             // ring slot of this lane's ray
  int64_t qbase = 0;        // first ray of that slot's block
  V3 o = V3{0.f, 0.f, 0.f};
  float ix = 0.f, iy = 0.f, iz = 0.f, ox = 0.f, oy = 0.f, oz = 0.f;
  V3 d = V3{0.f, 0.f, 1.f};
  float best = 0.f;
  int best_idx = INT_MAX;
  int2 stk[STACK];
  int sp = 0;
  int next = CHILD_EMPTY;
  while (true) {
    __syncwarp();
    // write out completed blocks, oldest first
    while (oldest < taken && s_left[warp][oldest % STREAM_RING] == 0) {
      int sl = (int)(oldest % STREAM_RING);
      long long base = s_base[warp][sl];
      int cnt = s_cnt[warp][sl];
      for (int j = lane; j < cnt; j += 32) {
        out_time[base + j] = s_t[warp][sl][j];
        if (out_index) out_index[base + j] = s_i[warp][sl][j];
      }
      ++oldest;
    }
    __syncwarp();
    unsigned idle = __ballot_sync(FULL, q < 0);
    if (idle && !exhausted) {
      if (qb >= qe && taken - oldest < STREAM_RING) {
        unsigned long long b = 0;
        if (lane == 0) b = atomicAdd(counter, (unsigned long long)RAY_WARP_BLOCK);
        b = __shfl_sync(FULL, b, 0);
        if ((int64_t)b >= n) {
          exhausted = true;
        } else {
          qb = (int64_t)b;
          qe = qb + RAY_WARP_BLOCK < n ? qb + RAY_WARP_BLOCK : n;
          int cnt = (int)(qe - qb);
          // one coalesced copy of the block's origins and directions
          for (int k = lane; k < 3 * cnt; k += 32) {
            in[(k / 3) * 6 + k % 3] = origins[3 * qb + k];
            in[(k / 3) * 6 + 3 + k % 3] = dirs[3 * qb + k];
          }
          int sl = (int)(taken % STREAM_RING);
          if (lane == 0) {
            s_base[warp][sl] = qb;
            s_cnt[warp][sl] = cnt;
            s_left[warp][sl] = cnt;
          }
          ++taken;
          __syncwarp();
        }
      }
      if (!exhausted && qb < qe) {
        int rank = __popc(idle & ((1u << lane) - 1));
        int take = __popc(idle);
        int64_t avail = qe - qb;
        if (q < 0 && rank < avail) {
          q = qb + rank;
          slot = (int)((taken - 1) % STREAM_RING);
          qbase = s_base[warp][slot];
          float const * r = in + (q - qbase) * 6;
          o = V3{r[0], r[1], r[2]};
          d = V3{r[3], r[4], r[5]};
          ix = 1.0f / (fabsf(d.x) > 1e-30f ? d.x : copysignf(1e-30f, d.x));
          iy = 1.0f / (fabsf(d.y) > 1e-30f ? d.y : copysignf(1e-30f, d.y));
          iz = 1.0f / (fabsf(d.z) > 1e-30f ? d.z : copysignf(1e-30f, d.z));
          ox = -o.x * ix;
          oy = -o.y * iy;
          oz = -o.z * iz;
          best = max_time >= 0.f ? max_time : INFINITY;
          best_idx = INT_MAX;
          sp = 0;
          next = 0;
        }
        qb += take < avail ? take : avail;
      }
    }
    bool busy = __ballot_sync(FULL, q >= 0) != 0;
    if (!busy && oldest == taken && (exhausted || qb >= qe)) {
      if (exhausted) break;
      continue;  // every block written out and no ray in flight: take the next block
    }
    if (q < 0) continue;
    int code = next;
    if (code == CHILD_EMPTY) {
      if (sp == 0) {
        bool found = best_idx != INT_MAX;
        int j = (int)(q - qbase);
        s_t[warp][slot][j] = found ? best : -1.f;
        s_i[warp][slot][j] = found ? best_idx : -1;
        atomicSub(&s_left[warp][slot], 1);
        q = -1;
        continue;
      }
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
        lb[c] = tmin <= tmax ? tmin : __int_as_float(0x7fffffff);
      }
      push_children_next<W, STACK>(nd, lb, best * PRUNE_SLACK, stk, sp, next, err);
    } else {
      int first, count;
      decode_leaf(code, first, count);
      for (int64_t k = first; k < first + count; ++k) {
        float4 const * r = rec + k * RAY_REC_F4;
        float4 a = __ldg(r), b = __ldg(r + 1), c = __ldg(r + 2);
        float t = ray_triangle_time(o, d, xyz(a), xyz(b), xyz(c));
        int idx = __float_as_int(a.w);
        if (t >= 0.f && t <= best && (t < best || idx < best_idx)) {
          best = t;
          best_idx = idx;
        }
      }
    }
  }
}

template <int W, int STACK>
void launch_ray_stream(thea_bvh const * b, float const * o, float const * d, int64_t n, float max_time, float * t,
                       int32_t * idx, unsigned * err, cudaStream_t s) {
  auto k = ray_stream_kernel<W, STACK>;
  int per_sm = 0;
  THEA_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, QUERY_THREADS, 0));
  int64_t need = ceil_div(ceil_div(n, RAY_WARP_BLOCK) * 32, QUERY_THREADS);
  unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((int64_t)std::max(1, per_sm) * sm_count(), need));
  Scratch counter(sizeof(unsigned long long), s);
  THEA_CUDA_CHECK(cudaMemsetAsync(counter.ptr, 0, sizeof(unsigned long long), s));
  THEA_LAUNCH_NAMED("ray_stream_kernel", k, grid, QUERY_THREADS, 0, s, (WideNode<W> const *)b->nodes, b->ray_rec, o, d,
                    n, max_time, t, idx, err, counter.as<unsigned long long>());
}

//============================================================================================================================
// k nearest points (BvhN::kClosestPairs + KClosestPairsFunctor + BoundedSortedArrayN; BvhN.hpp:474-500, 1139-1146;
// BoundedSortedArrayN.hpp:137-214)
//============================================================================================================================

// The k-NN kernels keep lists of K >= 8 in shared memory (knn_search_shared): 48-56 registers for K = 16, and the
// register allocator is asked for eight resident blocks of 128 threads (four for K = 32, whose lists take 32 KB)
template <int K> __host__ __device__ constexpr bool knn_lists_shared() { return K >= 8; }
template <int K> constexpr int knn_point_min_blocks() { return knn_lists_shared<K>() ? (K <= 16 ? 8 : 4) : 8; }

// Row `row` of the k-NN outputs from a K-entry list read through gd(j) / gi(j) (registers or shared memory): -1 for
// empty entries. Whole rows go out as 16-byte stores when they can: rows land at scattered element indices (self
// mode), and full-sector writes keep the L2 from sending partial sectors to DRAM.
template <int K, class GD, class GI>
__device__ __forceinline__ void write_knn_row(int32_t * __restrict__ out_index, float * __restrict__ out_d2, int64_t row,
                                              int k_out, GD gd, GI gi) {
  uintptr_t outs = reinterpret_cast<uintptr_t>(out_index) | reinterpret_cast<uintptr_t>(out_d2);
  if (K % 4 == 0 && k_out == K && (outs & 15) == 0) {
    int4 * oi = reinterpret_cast<int4 *>(out_index + row * K);
    float4 * od = reinterpret_cast<float4 *>(out_d2 + row * K);
#pragma unroll
    for (int j = 0; j < K; j += 4) {
      int i0 = gi(j), i1 = gi(j + 1), i2 = gi(j + 2), i3 = gi(j + 3);
      i0 = i0 != INT_MAX ? i0 : -1;
      i1 = i1 != INT_MAX ? i1 : -1;
      i2 = i2 != INT_MAX ? i2 : -1;
      i3 = i3 != INT_MAX ? i3 : -1;
      oi[j / 4] = make_int4(i0, i1, i2, i3);
      od[j / 4] = make_float4(i0 >= 0 ? gd(j) : -1.f, i1 >= 0 ? gd(j + 1) : -1.f, i2 >= 0 ? gd(j + 2) : -1.f,
                              i3 >= 0 ? gd(j + 3) : -1.f);
    }
    return;
  }
  for (int j = 0; j < k_out; ++j) {
    int i = gi(j);
    bool v = i != INT_MAX;
    out_index[row * k_out + j] = v ? i : -1;
    out_d2[row * k_out + j] = v ? gd(j) : -1.f;
  }
}

template <int W, int K, int STACK>
__global__ void __launch_bounds__(QUERY_THREADS, knn_point_min_blocks<K>())
knn_kernel(WideNode<W> const * __restrict__ nodes, float4 const * __restrict__ pts, float const * __restrict__ queries,
           int64_t n, int k_out, float thresh, int32_t const * __restrict__ exclude, int32_t * __restrict__ out_index,
           float * __restrict__ out_d2, unsigned * __restrict__ err, uint32_t const * __restrict__ order,
           float const * __restrict__ init_bound) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  if (order) q = order[q];
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
  // init_bound (self mode, per leaf position): an upper bound on the k-th neighbour's squared distance, inclusive, from
  // actual points; the search keeps every point within it, so the result is the same as without it
  float start = init_bound ? fminf(thresh, init_bound[q]) : thresh;
  if constexpr (knn_lists_shared<K>()) {
    __shared__ float s_d[K][QUERY_THREADS];
    __shared__ int s_i[K][QUERY_THREADS];
    int t = threadIdx.x;
#pragma unroll
    for (int j = 0; j < K; ++j) {
      s_d[j][t] = start;
      s_i[j][t] = INT_MAX;
    }
    float kth = start;
    int kth_i = INT_MAX;
    knn_query_shared<W, K, STACK, QUERY_THREADS>(nodes, pts, 0, 0, p, excl, s_d, s_i, kth, kth_i, err);
    // the row straight from shared memory (no register copy, which the dynamic row length would put in local memory)
    write_knn_row<K>(out_index, out_d2, row, k_out, [&](int j) { return s_d[j][t]; }, [&](int j) { return s_i[j][t]; });
  } else {
    float bd[K];
    int bi[K];
#pragma unroll
    for (int j = 0; j < K; ++j) { bd[j] = start; bi[j] = INT_MAX; }
    knn_query<W, K, STACK>(nodes, pts, 0, 0, p, excl, bd, bi, err);
    write_knn_row<K>(out_index, out_d2, row, k_out, [&](int j) { return bd[j]; }, [&](int j) { return bi[j]; });
  }
}

// k nearest triangles of a mesh BVH to each query point (kClosestPairs on a MeshBvh)
template <int W, int K, int STACK>
__global__ void __launch_bounds__(QUERY_THREADS, knn_point_min_blocks<K>())
knn_mesh_kernel(WideNode<W> const * __restrict__ nodes, float4 const * __restrict__ rec,
                float const * __restrict__ queries, int64_t n, int k_out, float thresh,
                int32_t const * __restrict__ exclude, int32_t * __restrict__ out_index, float * __restrict__ out_d2,
                unsigned * __restrict__ err, uint32_t const * __restrict__ order) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  if (order) q = order[q];
  V3 p = load_v3(queries + 3 * q);
  int excl = exclude ? exclude[q] : -1;
  if constexpr (knn_lists_shared<K>()) {
    __shared__ float s_d[K][QUERY_THREADS];
    __shared__ int s_i[K][QUERY_THREADS];
    int t = threadIdx.x;
#pragma unroll
    for (int j = 0; j < K; ++j) {
      s_d[j][t] = thresh;
      s_i[j][t] = INT_MAX;
    }
    float kth = thresh;
    int kth_i = INT_MAX;
    knn_mesh_query_shared<W, K, STACK, QUERY_THREADS>(nodes, rec, 0, 0, p, excl, s_d, s_i, kth, kth_i, err);
    write_knn_row<K>(out_index, out_d2, q, k_out, [&](int j) { return s_d[j][t]; }, [&](int j) { return s_i[j][t]; });
  } else {
    float bd[K];
    int bi[K];
#pragma unroll
    for (int j = 0; j < K; ++j) { bd[j] = thresh; bi[j] = INT_MAX; }
    knn_mesh_query<W, K, STACK>(nodes, rec, 0, 0, p, excl, bd, bi, err);
    write_knn_row<K>(out_index, out_d2, q, k_out, [&](int j) { return bd[j]; }, [&](int j) { return bi[j]; });
  }
}

// FP32 calls on one BVH by size (config-0 sweep of 1,024 .. 262,144 queries, event-timed):
//  * fewer than CLOSEST_WARP_MAX queries: two kernels with a 16-step budget, so nearly every query runs as one warp
//    over up to 8 nodes a step (4,096 queries: 0.19 ms against 0.59 ms one per thread, whose time is the longest
//    query's chain of dependent loads);
//  * up to CLOSEST_TWO_PHASE_MIN: one query per thread (65,536 queries: 0.71 ms; 0.72 with a 16-step budget);
//  * from there: two kernels with a 256-step budget (persistent lanes, then a warp per query past it; 262,144 queries:
//    1.30 ms against 1.84 one per thread).
constexpr int64_t CLOSEST_WARP_MAX = 57344;
constexpr int CLOSEST_WARP_BUDGET = 16;
constexpr int64_t CLOSEST_TWO_PHASE_MIN = 98304;
constexpr int CLOSEST_TWO_PHASE_BUDGET = 256;

__global__ void query_range_kernel(int64_t * qoff, int64_t n) {
  qoff[0] = 0;
  qoff[1] = n;
}

//============================================================================================================================
// Points within a radius (BvhN::rangeQueryIndices with a Ball3 range, BvhN.hpp:1208-1219, 2118-2171; BallN::contains,
// BallN.hpp:83: (p - center).squaredNorm() <= radius * radius, inclusive, FP32). Counting pass, then a filling pass into
// each query's slice of a CSR list; the slices are then put in ascending element order by one key sort.
//============================================================================================================================

// MODE 0: count each query's neighbours; 1: write (query, element) keys and squared distances at the query's offset,
// for the sort into ascending element order; 2: write the elements (and squared distances, if asked) directly, in
// traversal order.
template <int W, int STACK, int MODE>
__global__ void __launch_bounds__(QUERY_THREADS)
range_kernel(WideNode<W> const * __restrict__ nodes, float4 const * __restrict__ pts, float const * __restrict__ queries,
             int64_t n, float r2, int32_t const * __restrict__ exclude, int64_t * __restrict__ count_or_offset,
             uint64_t * __restrict__ keys, float * __restrict__ out_d2, unsigned * __restrict__ err,
             int32_t * __restrict__ out_idx = nullptr, int row_cap = 0, unsigned * __restrict__ overflow = nullptr) {
  constexpr bool FILL = MODE == 1 || MODE == 2;  // MODE 3: count, and write the first row_cap into row q of out_idx
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  V3 p = load_v3(queries + 3 * q);
  int ex = exclude ? exclude[q] : -1;
  int64_t w = FILL ? count_or_offset[q] : 0;
  int64_t c = 0;
  // every child within the radius is visited whatever the order, so children are pushed unsorted
  int stk[STACK];
  int sp = 0;
  stk[sp++] = 0;
  float lim = r2 * PRUNE_SLACK;
  while (sp > 0) {
    int code = stk[--sp];
    if (code >= 0) {
      NodeRegs<W> nd;
      load_node(nodes, code, nd);
      float lb[W];
      point_child_bounds<W>(nd, p, lb);
#pragma unroll
      for (int c = 0; c < W; ++c) {
        if (nd.child[c] != CHILD_EMPTY && lb[c] <= lim) {
          if (sp < STACK) stk[sp++] = nd.child[c];
          else atomicOr(err, ERR_STACK_OVERFLOW);
        }
      }
    } else {
      int first, count;
      decode_leaf(code, first, count);
      for (int64_t k = first; k < first + count; ++k) {
        float4 a = __ldg(pts + k);
        int idx = __float_as_int(a.w);
        if (idx == ex) continue;
        float d2 = squared_norm(xyz(a) - p);
        if (d2 <= r2) {
          if (MODE == 1) {
            keys[w + c] = ((uint64_t)q << 32) | (uint32_t)idx;
            out_d2[w + c] = d2;
          } else if (MODE == 2) {
            out_idx[w + c] = idx;
            if (out_d2) out_d2[w + c] = d2;
          } else if (MODE == 3) {
            if (c < row_cap) out_idx[q * row_cap + c] = idx;
          }
          ++c;
        }
      }
    }
  }
  if (!FILL) count_or_offset[q] = c;
  if (MODE == 3 && c > row_cap) atomicOr(overflow, 1u);
}

__global__ void range_total_kernel(int64_t const * __restrict__ counts, int64_t n, int64_t * __restrict__ offsets) {
  offsets[n] = offsets[n - 1] + counts[n - 1];
}

__global__ void range_iota_kernel(int64_t total, uint32_t * __restrict__ v) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < total) v[i] = (uint32_t)i;
}

// After the key sort: element index from the low key bits, squared distance gathered through the permutation
__global__ void range_emit_kernel(uint64_t const * __restrict__ keys, uint32_t const * __restrict__ perm,
                                  float const * __restrict__ d2_unsorted, int64_t total, int32_t * __restrict__ out_idx,
                                  float * __restrict__ out_d2) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  out_idx[i] = (int32_t)(uint32_t)(keys[i] & 0xffffffffu);
  if (out_d2) out_d2[i] = d2_unsorted[perm[i]];
}

template <int W, int STACK>
void launch_range(thea_bvh const * b, float const * q, int64_t n, float r2, int32_t const * ex, int64_t * offsets,
                  int32_t * out_idx, float * out_d2, unsigned * err, bool sorted, cudaStream_t s) {
  unsigned grid = (unsigned)ceil_div(n, QUERY_THREADS);
  if (out_idx && !sorted) {
    THEA_LAUNCH((range_kernel<W, STACK, 2>), grid, QUERY_THREADS, 0, s, (WideNode<W> const *)b->nodes, b->pt_rec, q,
                n, r2, ex, offsets, (uint64_t *)nullptr, out_d2, err, out_idx);
    return;
  }
  if (!out_idx) {
    Scratch counts((size_t)n * sizeof(int64_t), s);
    THEA_LAUNCH((range_kernel<W, STACK, 0>), grid, QUERY_THREADS, 0, s, (WideNode<W> const *)b->nodes, b->pt_rec,
                q, n, r2, ex, counts.as<int64_t>(), (uint64_t *)nullptr, (float *)nullptr, err);
    exclusive_scan<int64_t>(counts.as<int64_t>(), offsets, n, s);
    THEA_LAUNCH(range_total_kernel, 1, 1, 0, s, counts.as<int64_t>(), n, offsets);
    return;
  }
  int64_t total = 0;
  THEA_CUDA_CHECK(cudaMemcpyAsync(&total, offsets + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  THEA_CUDA_CHECK(cudaStreamSynchronize(s));
  if (total <= 0) return;
  THEA_REQUIRE(total < (int64_t(1) << 32), "radius_neighbors: more than 2^32 neighbours in one call");
  Scratch keys((size_t)total * sizeof(uint64_t), s), d2((size_t)total * sizeof(float), s);
  Scratch perm((size_t)total * sizeof(uint32_t), s);
  THEA_LAUNCH((range_kernel<W, STACK, 1>), grid, QUERY_THREADS, 0, s, (WideNode<W> const *)b->nodes, b->pt_rec, q,
              n, r2, ex, offsets, keys.as<uint64_t>(), d2.as<float>(), err);
  THEA_LAUNCH(range_iota_kernel, (unsigned)ceil_div(total, 256), 256, 0, s, total, perm.as<uint32_t>());
  int qbits = 1;
  while ((int64_t(1) << qbits) < n) ++qbits;
  radix_sort_pairs(keys.as<uint64_t>(), perm.as<uint32_t>(), total, 32 + qbits, s);
  THEA_LAUNCH(range_emit_kernel, (unsigned)ceil_div(total, 256), 256, 0, s, keys.as<uint64_t>(), perm.as<uint32_t>(),
              d2.as<float>(), total, out_idx, out_d2);
}

template <int W, int STACK>
void launch_range_rows(thea_bvh const * b, float const * q, int64_t n, float r2, int32_t const * ex, int64_t * offsets,
                       int32_t * rows, int row_cap, unsigned * overflow, unsigned * err, cudaStream_t s) {
  unsigned grid = (unsigned)ceil_div(n, QUERY_THREADS);
  Scratch counts((size_t)n * sizeof(int64_t), s);
  THEA_LAUNCH((range_kernel<W, STACK, 3>), grid, QUERY_THREADS, 0, s, (WideNode<W> const *)b->nodes, b->pt_rec, q, n,
              r2, ex, counts.as<int64_t>(), (uint64_t *)nullptr, (float *)nullptr, err, rows, row_cap, overflow);
  exclusive_scan<int64_t>(counts.as<int64_t>(), offsets, n, s);
  THEA_LAUNCH(range_total_kernel, 1, 1, 0, s, counts.as<int64_t>(), n, offsets);
}

//============================================================================================================================
// Distance bounds of closest-element queries (BoundCut in query.hpp)
//============================================================================================================================

}  // namespace

RootCut root_cut_of(float const * elem_lo, float const * elem_hi, float const * xf) {
  RootCut r;
  float lo[3], hi[3];
  for (int a = 0; a < 3; ++a) {
    // scaleCentered(1.05f): centre = 0.5 (hi + lo); lo = 1.05 (lo - centre) + centre, hi likewise
    float ctr = 0.5f * (elem_hi[a] + elem_lo[a]);
    lo[a] = 1.05f * (elem_lo[a] - ctr) + ctr;
    hi[a] = 1.05f * (elem_hi[a] - ctr) + ctr;
  }
  if (xf) {
    // transformAndBound: the box of the eight mapped corners
    float wlo[3] = {INFINITY, INFINITY, INFINITY}, whi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int k = 0; k < 8; ++k) {
      V3 w = affine_point(xf, V3{(k & 1) ? hi[0] : lo[0], (k & 2) ? hi[1] : lo[1], (k & 4) ? hi[2] : lo[2]});
      float wc[3] = {w.x, w.y, w.z};
      for (int a = 0; a < 3; ++a) {
        wlo[a] = std::min(wlo[a], wc[a]);
        whi[a] = std::max(whi[a], wc[a]);
      }
    }
    for (int a = 0; a < 3; ++a) lo[a] = wlo[a], hi[a] = whi[a];
  }
  for (int a = 0; a < 3; ++a) r.lo[a] = lo[a], r.hi[a] = hi[a];
  V3 ext = V3{hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
  float nrm = std::sqrt(squared_norm(ext));
  r.fudge = std::max(0.001 * (double)nrm, (double)(100.0f * 1.1920928955078125e-07f));
  return r;
}

namespace {

__global__ void closest_cut_kernel(float const * __restrict__ q, int64_t n, int64_t const * __restrict__ qoff, int M,
                                   BoundCut one, BoundCut const * __restrict__ cuts, int32_t * __restrict__ idx,
                                   float * __restrict__ dist, float * __restrict__ cpt, float * __restrict__ errout) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  BoundCut c = one;
  if (cuts) {
    int lo = 0, hi = M - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (__ldg(qoff + mid) <= i) lo = mid;
      else hi = mid - 1;
    }
    c = cuts[lo];
  }
  if (!bound_cut_out(c, load_v3(q + 3 * i))) return;
  idx[i] = -1;
  if (dist) dist[i] = -1.f;
  if (cpt) cpt[3 * i] = cpt[3 * i + 1] = cpt[3 * i + 2] = 0.f;
  if (errout) errout[i] = -1.f;
}

}  // namespace

namespace {
__global__ void segment_cuts_kernel(RootCut const * __restrict__ roots, int M, float dist_bound,
                                    BoundCut * __restrict__ out) {
  int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m < M) out[m] = make_bound_cut(roots[m], dist_bound);
}
}  // namespace

void run_segment_cuts(thea_bvh const * b, float dist_bound, BoundCut * out, cudaStream_t s) {
  THEA_REQUIRE(b->seg_roots, "segment cuts: the forest has no per-segment root boxes");
  THEA_LAUNCH(segment_cuts_kernel, (unsigned)ceil_div(b->num_segments, 256), 256, 0, s, b->seg_roots,
              b->num_segments, dist_bound, out);
}

void run_closest_cut(float const * q, int64_t n, BoundCut const & one, int64_t const * qoff, int M,
                     BoundCut const * cuts, int32_t * idx, float * dist, float * cpt, float * errout, cudaStream_t s) {
  if (n <= 0 || (!cuts && one.b2 < 0.0)) return;
  THEA_LAUNCH(closest_cut_kernel, (unsigned)ceil_div(n, 256), 256, 0, s, q, n, qoff, M, one, cuts, idx, dist, cpt,
              errout);
}

namespace {

//============================================================================================================================
// Query ordering: large batches can be traversed in the order of a Morton code of the query point (rays: of the
// origin, with the direction octant as the top bits). Results are written to each query's own slot.
//============================================================================================================================

constexpr int64_t ORDER_MIN_QUERIES = 1 << 15;

__device__ __forceinline__ uint32_t expand10(uint32_t x) {
  x &= 0x3ffu;
  x = (x | x << 16) & 0x030000FFu;
  x = (x | x << 8) & 0x0300F00Fu;
  x = (x | x << 4) & 0x030C30C3u;
  x = (x | x << 2) & 0x09249249u;
  return x;
}

__global__ void query_key_kernel(float const * __restrict__ p, float const * __restrict__ dir, int64_t n, float lx,
                                 float ly, float lz, float sx, float sy, float sz, uint64_t * __restrict__ keys,
                                 uint32_t * __restrict__ vals) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int bits = dir ? 9 : 10;
  float cells = (float)(1 << bits);
  float c[3] = {(p[3 * i] - lx) * sx, (p[3 * i + 1] - ly) * sy, (p[3 * i + 2] - lz) * sz};
  uint32_t q[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float t = fminf(fmaxf(c[a], 0.f), 1.f);  // NaN-safe: fminf/fmaxf drop a NaN operand
    q[a] = min((uint32_t)(t * cells), (uint32_t)(1 << bits) - 1u);
  }
  uint32_t key = (expand10(q[0]) << 2) | (expand10(q[1]) << 1) | expand10(q[2]);
  if (dir) {
    uint32_t oct = (dir[3 * i] < 0.f ? 4u : 0u) | (dir[3 * i + 1] < 0.f ? 2u : 0u) | (dir[3 * i + 2] < 0.f ? 1u : 0u);
    key |= oct << 27;
  }
  keys[i] = key;
  vals[i] = (uint32_t)i;
}

struct QueryOrder {
  Scratch keys, vals;
  uint32_t const * order = nullptr;
  QueryOrder(thea_bvh const * b, float const * p, float const * dir, int64_t n, cudaStream_t s, bool always = false) {
    if ((!b->query_order && !always) || n < ORDER_MIN_QUERIES) return;
    keys = Scratch((size_t)n * sizeof(uint64_t), s);
    vals = Scratch((size_t)n * sizeof(uint32_t), s);
    float sc[3];
    for (int a = 0; a < 3; ++a) {
      float ext = b->hi[a] - b->lo[a];
      sc[a] = ext > 0.f ? 1.0f / ext : 0.f;
    }
    THEA_LAUNCH(query_key_kernel, (unsigned)ceil_div(n, 256), 256, 0, s, p, dir, n, b->lo[0], b->lo[1], b->lo[2],
                sc[0], sc[1], sc[2], keys.as<uint64_t>(), vals.as<uint32_t>());
    radix_sort_pairs(keys.as<uint64_t>(), vals.as<uint32_t>(), n, 30, s, /*probe_passes=*/false);
    order = vals.as<uint32_t>();
  }
};

template <int W, int STACK>
void launch_closest(thea_bvh const * b, float const * q, int64_t n, ClosestParams const & cp, int32_t * idx,
                    float * dist, float * cpt, float * errout, unsigned * err, uint32_t const * order, cudaStream_t s) {
  unsigned grid = (unsigned)ceil_div(n, QUERY_THREADS);
  if (cp.precision == THEA_PRECISION_FP64_RECHECK)
    THEA_LAUNCH((closest_kernel<W, STACK, THEA_PRECISION_FP64_RECHECK>), grid, QUERY_THREADS, 0, s,
                (WideNode<W> const *)b->nodes, b->cp_rec, q, n, cp.thresh, cp.bound2, cp.scene_scale, idx, dist, cpt,
                errout, err, order, b->slabs);
  else
    THEA_LAUNCH((closest_kernel<W, STACK, THEA_PRECISION_FP32_REFERENCE>), grid, QUERY_THREADS, 0, s,
                (WideNode<W> const *)b->nodes, b->cp_rec, q, n, cp.thresh, cp.bound2, cp.scene_scale, idx, dist, cpt,
                errout, err, order, b->slabs);
}

template <int W, int STACK>
void launch_ray(thea_bvh const * b, float const * o, float const * d, int64_t n, RayParams const & rp, float * t,
                int32_t * idx, float * nrm, float * t64, int32_t * idx64, int32_t * flags, unsigned * err,
                uint32_t const * order, cudaStream_t s) {
  unsigned grid = (unsigned)ceil_div(n, QUERY_THREADS);
  if (!rp.recheck && n >= RAY_PERSISTENT_MIN) {
    auto k = ray_persistent_kernel<W, STACK>;
    int sms = sm_count();
    int per_sm = 0;
    THEA_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, QUERY_THREADS, 0));
    unsigned pgrid = (unsigned)std::min<int64_t>((int64_t)std::max(1, per_sm) * sms, grid);
    Scratch counter(sizeof(unsigned long long), s);
    THEA_CUDA_CHECK(cudaMemsetAsync(counter.ptr, 0, sizeof(unsigned long long), s));
    THEA_LAUNCH_NAMED("ray_kernel_persistent", k, pgrid, QUERY_THREADS, 0, s, (WideNode<W> const *)b->nodes,
                      b->ray_rec, o, d, n, rp.max_time, t, idx, nrm, err, order, counter.as<unsigned long long>());
    return;
  }
  if (rp.recheck)
    THEA_LAUNCH((ray_recheck_kernel<W, STACK>), grid, QUERY_THREADS, 0, s, (WideNode<W> const *)b->nodes, b->ray_rec,
                o, d, n, rp.max_time, t, idx, nrm, t64, idx64, flags, err, order);
  else
    THEA_LAUNCH((ray_kernel<W, STACK, false>), grid, QUERY_THREADS, 0, s, (WideNode<W> const *)b->nodes, b->ray_rec, o,
                d, n, rp.max_time, t, idx, nrm, t64, idx64, flags, err, order);
}

template <int W, int K, int STACK>
void launch_knn_k(thea_bvh const * b, float const * q, int64_t n, int k, float thresh, int32_t const * ex,
                  int32_t * idx, float * d2, unsigned * err, uint32_t const * order, float const * ib, cudaStream_t s) {
  THEA_LAUNCH((knn_kernel<W, K, STACK>), (unsigned)ceil_div(n, QUERY_THREADS), QUERY_THREADS, 0, s,
              (WideNode<W> const *)b->nodes, b->pt_rec, q, n, k, thresh, ex, idx, d2, err, order, ib);
}

template <int W, int K, int STACK>
void launch_knn_mesh_k(thea_bvh const * b, float const * q, int64_t n, int k, float thresh, int32_t const * ex,
                       int32_t * idx, float * d2, unsigned * err, uint32_t const * order, cudaStream_t s) {
  THEA_LAUNCH((knn_mesh_kernel<W, K, STACK>), (unsigned)ceil_div(n, QUERY_THREADS), QUERY_THREADS, 0, s,
              (WideNode<W> const *)b->nodes, b->cp_rec, q, n, k, thresh, ex, idx, d2, err, order);
}

template <int W, int STACK>
void launch_knn_mesh(thea_bvh const * b, float const * q, int64_t n, int k, float thresh, int32_t const * ex,
                     int32_t * idx, float * d2, unsigned * err, uint32_t const * order, cudaStream_t s) {
  if (k <= 1) launch_knn_mesh_k<W, 1, STACK>(b, q, n, k, thresh, ex, idx, d2, err, order, s);
  else if (k <= 4) launch_knn_mesh_k<W, 4, STACK>(b, q, n, k, thresh, ex, idx, d2, err, order, s);
  else if (k <= 8) launch_knn_mesh_k<W, 8, STACK>(b, q, n, k, thresh, ex, idx, d2, err, order, s);
  else if (k <= 16) launch_knn_mesh_k<W, 16, STACK>(b, q, n, k, thresh, ex, idx, d2, err, order, s);
  else launch_knn_mesh_k<W, 32, STACK>(b, q, n, k, thresh, ex, idx, d2, err, order, s);
}

template <int W, int STACK>
void launch_knn(thea_bvh const * b, float const * q, int64_t n, int k, float thresh, int32_t const * ex, int32_t * idx,
                float * d2, unsigned * err, uint32_t const * order, float const * ib, cudaStream_t s) {
  if (b->is_mesh) {
    launch_knn_mesh<W, STACK>(b, q, n, k, thresh, ex, idx, d2, err, order, s);
    return;
  }
  if (k <= 1) launch_knn_k<W, 1, STACK>(b, q, n, k, thresh, ex, idx, d2, err, order, ib, s);
  else if (k <= 2) launch_knn_k<W, 2, STACK>(b, q, n, k, thresh, ex, idx, d2, err, order, ib, s);
  else if (k <= 4) launch_knn_k<W, 4, STACK>(b, q, n, k, thresh, ex, idx, d2, err, order, ib, s);
  else if (k <= 8) launch_knn_k<W, 8, STACK>(b, q, n, k, thresh, ex, idx, d2, err, order, ib, s);
  else if (k <= 16) launch_knn_k<W, 16, STACK>(b, q, n, k, thresh, ex, idx, d2, err, order, ib, s);
  else launch_knn_k<W, 32, STACK>(b, q, n, k, thresh, ex, idx, d2, err, order, ib, s);
}

}  // namespace

bool small_stack_ok(thea_bvh const * b) {
  int need = b->depth * (b->width - 1) + 1;
  return need <= (b->width == 4 ? 64 : 128);
}

void run_closest(thea_bvh const * b, float const * q, int64_t n, ClosestParams const & cp, int32_t * idx, float * dist,
                 float * cpt, float * errout, unsigned * err, cudaStream_t s) {
  if (n <= 0) return;
  if (cp.precision == THEA_PRECISION_FP32_REFERENCE && !errout && !b->query_order &&
      (n < CLOSEST_WARP_MAX || n >= CLOSEST_TWO_PHASE_MIN)) {
    // Persistent lanes with a step budget, then one warp per query over budget (the BVH is a one-mesh forest). The
    // same searches, so the same results.
    Scratch qoff(2 * sizeof(int64_t), s);
    THEA_LAUNCH(query_range_kernel, 1, 1, 0, s, qoff.as<int64_t>(), n);
    ClosestParams c2 = cp;
    c2.budget = n < CLOSEST_WARP_MAX ? CLOSEST_WARP_BUDGET : CLOSEST_TWO_PHASE_BUDGET;
    run_batch_closest(b, q, qoff.as<int64_t>(), n, c2, 64, idx, dist, cpt, nullptr, s);
    return;
  }
  // FP64 re-check: warps of Morton-ordered queries share band candidates (config 0: 2.64 -> 2.26 ms), so the order is
  // taken whatever the BVH's query_order option says
  QueryOrder ord(b, q, nullptr, n, s, cp.precision == THEA_PRECISION_FP64_RECHECK);
  uint32_t const * o = ord.order;
  bool sm = small_stack_ok(b);
  if (b->width == 4) sm ? launch_closest<4, 64>(b, q, n, cp, idx, dist, cpt, errout, err, o, s)
                        : launch_closest<4, 256>(b, q, n, cp, idx, dist, cpt, errout, err, o, s);
  else sm ? launch_closest<8, 128>(b, q, n, cp, idx, dist, cpt, errout, err, o, s)
          : launch_closest<8, 512>(b, q, n, cp, idx, dist, cpt, errout, err, o, s);
}

void run_ray(thea_bvh const * b, float const * o, float const * d, int64_t n, RayParams const & rp, float * t,
             int32_t * idx, float * nrm, float * t64, int32_t * idx64, int32_t * flags, unsigned * err, cudaStream_t s) {
  if (n <= 0) return;
  QueryOrder ord(b, o, d, n, s);
  uint32_t const * od = ord.order;
  bool sm = small_stack_ok(b);
  if (b->width == 4) sm ? launch_ray<4, 64>(b, o, d, n, rp, t, idx, nrm, t64, idx64, flags, err, od, s)
                        : launch_ray<4, 256>(b, o, d, n, rp, t, idx, nrm, t64, idx64, flags, err, od, s);
  else sm ? launch_ray<8, 128>(b, o, d, n, rp, t, idx, nrm, t64, idx64, flags, err, od, s)
          : launch_ray<8, 512>(b, o, d, n, rp, t, idx, nrm, t64, idx64, flags, err, od, s);
}

void run_ray_stream(thea_bvh const * b, float const * o, float const * d, int64_t n, float max_time, float * t,
                    int32_t * idx, unsigned * err, cudaStream_t s) {
  if (n <= 0) return;
  bool sm = small_stack_ok(b);
  if (b->width == 4) sm ? launch_ray_stream<4, 64>(b, o, d, n, max_time, t, idx, err, s)
                        : launch_ray_stream<4, 256>(b, o, d, n, max_time, t, idx, err, s);
  else sm ? launch_ray_stream<8, 128>(b, o, d, n, max_time, t, idx, err, s)
          : launch_ray_stream<8, 512>(b, o, d, n, max_time, t, idx, err, s);
}

void run_range(thea_bvh const * b, float const * q, int64_t n, float radius, int32_t const * ex, int64_t * offsets,
               int32_t * idx, float * d2, unsigned * err, cudaStream_t s, bool sorted) {
  if (n <= 0) return;
  float r2 = radius * radius;  // BallN::contains compares with radius * radius in FP32
  bool sm = small_stack_ok(b);
  if (b->width == 4) sm ? launch_range<4, 64>(b, q, n, r2, ex, offsets, idx, d2, err, sorted, s)
                        : launch_range<4, 256>(b, q, n, r2, ex, offsets, idx, d2, err, sorted, s);
  else sm ? launch_range<8, 128>(b, q, n, r2, ex, offsets, idx, d2, err, sorted, s)
          : launch_range<8, 512>(b, q, n, r2, ex, offsets, idx, d2, err, sorted, s);
}

void run_range_rows(thea_bvh const * b, float const * q, int64_t n, float radius, int32_t const * ex,
                    int64_t * offsets, int32_t * rows, int row_cap, unsigned * overflow, unsigned * err, cudaStream_t s) {
  if (n <= 0) return;
  float r2 = radius * radius;
  bool sm = small_stack_ok(b);
  if (b->width == 4) sm ? launch_range_rows<4, 64>(b, q, n, r2, ex, offsets, rows, row_cap, overflow, err, s)
                        : launch_range_rows<4, 256>(b, q, n, r2, ex, offsets, rows, row_cap, overflow, err, s);
  else sm ? launch_range_rows<8, 128>(b, q, n, r2, ex, offsets, rows, row_cap, overflow, err, s)
          : launch_range_rows<8, 512>(b, q, n, r2, ex, offsets, rows, row_cap, overflow, err, s);
}

void run_knn(thea_bvh const * b, float const * q, int64_t n, int k, float thresh, int32_t const * ex, int32_t * idx,
             float * d2, unsigned * err, cudaStream_t s, float const * init_bound) {
  if (n <= 0) return;
  // self mode already runs in leaf order
  QueryOrder ord(b, q, nullptr, q ? n : 0, s);
  uint32_t const * o = ord.order;
  float const * ib = q ? nullptr : init_bound;
  bool sm = small_stack_ok(b);
  if (b->width == 4) sm ? launch_knn<4, 64>(b, q, n, k, thresh, ex, idx, d2, err, o, ib, s)
                        : launch_knn<4, 256>(b, q, n, k, thresh, ex, idx, d2, err, o, ib, s);
  else sm ? launch_knn<8, 128>(b, q, n, k, thresh, ex, idx, d2, err, o, ib, s)
          : launch_knn<8, 512>(b, q, n, k, thresh, ex, idx, d2, err, o, ib, s);
}

}  // namespace thea
