// Batched queries over a forest (one BVH per mesh or point set, built together by build_forest).
//
// One persistent launch serves every mesh: the grid is sized to fill the GPU once (blocks per SM x SMs), and each warp
// repeatedly takes the next chunk of queries from a global counter, so meshes with 1k or 100k queries and 320 or
// 327,680 triangles share the SMs without a tail of idle blocks. Queries are grouped by mesh (query_offsets, M + 1
// entries); a lane finds its query's mesh by binary search and starts from that mesh's root node. The whole call is
// asynchronous and allocation-stable, so it can be captured once into a CUDA graph and replayed.
#include "batch.hpp"
#include "device_util.cuh"
#include "traverse_ops.cuh"
#include "warp_traverse.cuh"

#include <algorithm>
#include <chrono>
#include <vector>

namespace thea {
namespace {

constexpr int BATCH_THREADS = 128;

__device__ __forceinline__ int mesh_of_query(int64_t const * __restrict__ qoff, int M, int64_t q) {
  int lo = 0, hi = M - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (__ldg(qoff + mid) <= q) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Each warp takes `chunk` consecutive queries per fetch; lanes stride through them.
__device__ __forceinline__ bool next_chunk(unsigned long long * counter, int chunk, int64_t nq, int64_t & base) {
  unsigned long long b = 0;
  if ((threadIdx.x & 31) == 0) b = atomicAdd(counter, (unsigned long long)chunk);
  b = __shfl_sync(0xffffffffu, b, 0);
  base = (int64_t)b;
  return base < nq;
}

//============================================================================================================================
// Closest element. Each warp works in rounds of 32 queries, one per lane; every lane of the warp takes part in every
// round (lanes past the end of the chunk carry no query), so the warp-wide FP64 step of the mixed-precision search and
// the FP64 error estimate run with all lanes together.
//
// Two-phase form: with budget > 0, phase 1 stops a query after that many stack pops and queues it with the best
// element found so far (a valid upper bound); phase 2 finishes the queued queries with one warp per query.
//============================================================================================================================

struct HardQueue {
  int64_t * q;
  float * bound;  // FP32 squared distance of the best element found so far (+inf if none)
  int32_t * idx;
  int64_t * slot;
  unsigned long long * count;
};

// d64: FP64 squared distance of the returned element (for the error estimate)
__device__ __forceinline__ void write_closest(int64_t q, bool found, float dist, V3 cp, int idx, double d64,
                                              int32_t * out_index, float * out_dist, float * out_cp, float * out_err) {
  out_index[q] = found ? idx : -1;
  if (out_dist) out_dist[q] = found ? dist : -1.f;
  if (out_cp) {
    out_cp[3 * q] = found ? cp.x : 0.f;
    out_cp[3 * q + 1] = found ? cp.y : 0.f;
    out_cp[3 * q + 2] = found ? cp.z : 0.f;
  }
  if (out_err) out_err[q] = found ? (float)fabs((double)dist - sqrt(d64)) : -1.f;
}

struct ClosestArgs {
  float const * queries;
  int64_t const * qoff;
  float thresh;
  double bound2;
  float scene_scale;
  int32_t * out_index;
  float * out_dist;
  float * out_cp;
  float * out_err;
  BoundCut const * seg_cut = nullptr;  // per mesh: thresh and bound2 of that mesh (nullptr: the scalars for all)
};

__device__ __forceinline__ float thresh_of(ClosestArgs const & a, int m) {
  return a.seg_cut ? a.seg_cut[m].thresh : a.thresh;
}
__device__ __forceinline__ double bound2_of(ClosestArgs const & a, int m) {
  return a.seg_cut ? a.seg_cut[m].bound2 : a.bound2;
}

// One round: lane query q when active. Called by all 32 lanes of the warp together.
template <int W, int STACK, int PREC>
__device__ __forceinline__ void closest_round(BatchForest const & f, ClosestArgs const & a, int64_t q, bool active,
                                              int budget, HardQueue const & hq, F64WarpBuf * buf) {
  WideNode<W> const * nodes = (WideNode<W> const *)f.nodes;
  int root = 0;
  int64_t ebase = 0;
  V3 p = V3{0.f, 0.f, 0.f};
  float thresh = a.thresh;
  double bound2 = a.bound2;
  if (active) {
    int m = mesh_of_query(a.qoff, f.M, q);
    root = __ldg(f.seg_root + m);
    ebase = __ldg(f.seg_start + m);
    p = load_v3(a.queries + 3 * q);
    thresh = thresh_of(a, m);
    bound2 = bound2_of(a, m);
  }
  ClosestOut r;
  r.idx = INT_MAX;
  r.d2 = 0.f;
  r.d2_64 = 0.0;
  r.slot = -1;
  r.best32 = INFINITY;
  r.done = true;
  float dist = 0.f;
  if constexpr (PREC == THEA_PRECISION_FP64_RECHECK) {
    float scale = fmaxf(a.scene_scale, fmaxf(fabsf(p.x), fmaxf(fabsf(p.y), fabsf(p.z))));
    F64Search s;
    if (active) closest_search_f64<W, STACK>(nodes, f.cp_rec, root, ebase, p, bound2, scale, f.err, s, budget);
    else f64_search_init(s);
    f64_resolve_warp(s, active && s.done, f.cp_rec, ebase, p, bound2, *buf);
    r = f64_result(s);
    dist = (float)sqrt(r.d2_64);
  } else {
    if (active) r = closest_query<W, STACK>(nodes, f.cp_rec, root, ebase, p, thresh, f.err, budget);
    dist = sqrtf(r.d2);
  }
  if (active && !r.done) {
    unsigned long long pos = atomicAdd(hq.count, 1ull);
    hq.q[pos] = q;
    hq.bound[pos] = r.best32;
    hq.idx[pos] = PREC == THEA_PRECISION_FP64_RECHECK ? INT_MAX : r.idx;
    hq.slot[pos] = r.slot;
  }
  bool fin = active && r.done;
  bool found = r.idx != INT_MAX;
  double d64 = r.d2_64;
  if (PREC != THEA_PRECISION_FP64_RECHECK && a.out_err) {
    __syncwarp();
    if (fin && found) {
      D3 cp64;
      cp_record_f64(f.cp_rec, r.slot, p, cp64, d64);
    }
  }
  if (fin) write_closest(q, found, dist, r.cp, r.idx, d64, a.out_index, a.out_dist, a.out_cp, a.out_err);
}

template <int W, int STACK, int PREC>
__global__ void __launch_bounds__(BATCH_THREADS)
batch_closest_kernel(BatchForest f, ClosestArgs a, int64_t nq, unsigned long long * counter, int chunk, int budget,
                     HardQueue hq) {
  F64WarpBuf * buf = nullptr;
  if constexpr (PREC == THEA_PRECISION_FP64_RECHECK) {
    __shared__ F64WarpBuf s_buf[BATCH_THREADS / 32];
    buf = &s_buf[threadIdx.x >> 5];
  }
  int lane = threadIdx.x & 31;
  int64_t base;
  while (next_chunk(counter, chunk, nq, base)) {
    int64_t end = base + chunk < nq ? base + chunk : nq;
    for (int64_t r0 = base; r0 < end; r0 += 32)
      closest_round<W, STACK, PREC>(f, a, r0 + lane, r0 + lane < end, budget, hq, buf);
  }
}

// Persistent-lane form of batch_closest_kernel: each lane takes a new query as soon as its query is done, instead of
// idling until the slowest query of its warp's round (the queries deep inside a mesh take ten times the steps of the
// others). Every loop iteration advances each busy lane by one stack entry; idle lanes are refilled from a warp-local
// block of 64 query indices. In the mixed-precision mode a lane whose traversal is done waits, its band entries kept,
// until 8 lanes of its warp are waiting (or nothing else is left), and the warp then evaluates all their entries in FP64
// together (f64_resolve_warp). Results are the round-based kernel's: each query's search is the same sequence of steps.
constexpr int REFILL_BLOCK = 64;
constexpr int REFILL_RESOLVE_AT = 8;

template <int W, int STACK, int PREC>
__global__ void __launch_bounds__(BATCH_THREADS)
batch_closest_refill_kernel(BatchForest f, ClosestArgs a, int64_t nq, unsigned long long * counter, int budget,
                            HardQueue hq) {
  F64WarpBuf * buf = nullptr;
  if constexpr (PREC == THEA_PRECISION_FP64_RECHECK) {
    __shared__ F64WarpBuf s_buf[BATCH_THREADS / 32];
    buf = &s_buf[threadIdx.x >> 5];
  }
  unsigned const FULL = 0xffffffffu;
  int lane = threadIdx.x & 31;
  WideNode<W> const * nodes = (WideNode<W> const *)f.nodes;
  int64_t qb = 0, qe = 0;  // warp-local block of query indices, warp-uniform
  bool exhausted = false;  // warp-uniform
  int64_t q = -1;          // this lane's query (-1: idle)
  bool pending = false;    // mixed precision: traversal done, waiting for the warp's FP64 step
  int64_t ebase = 0;
  V3 p = V3{0.f, 0.f, 0.f};
  int2 stk[STACK];  // (child code, bound bits)
  int sp = 0;
  int next = CHILD_EMPTY;  // nearest child of the last node, visited next without a stack round trip
  float best = 0.f;  // FP32 mode: best squared distance; mixed mode: band limit
  int best_idx = INT_MAX;
  int64_t best_slot = -1;
  V3 best_cp = V3{0.f, 0.f, 0.f};
  F64Search s;
  float best32 = INFINITY, abs_tol = 0.f;
  int pops = 0;  // stack entries taken by this lane's query (two-phase form: budget > 0)
  double bound2 = a.bound2;  // this lane's mesh's FP64 bound
  if constexpr (PREC == THEA_PRECISION_FP64_RECHECK) f64_search_init(s);
  while (true) {
    unsigned idle = __ballot_sync(FULL, q < 0);
    if (idle && !exhausted) {
      if (qb >= qe) {
        unsigned long long b = 0;
        if (lane == 0) b = atomicAdd(counter, (unsigned long long)REFILL_BLOCK);
        b = __shfl_sync(FULL, b, 0);
        qb = (int64_t)b;
        qe = qb + REFILL_BLOCK < nq ? qb + REFILL_BLOCK : nq;
        if (qb >= nq) exhausted = true;
      }
      if (!exhausted) {
        int rank = __popc(idle & ((1u << lane) - 1));
        int64_t avail = qe - qb;
        int64_t take = __popc(idle);
        if (q < 0 && rank < avail) {
          q = qb + rank;
          int m = mesh_of_query(a.qoff, f.M, q);
          ebase = __ldg(f.seg_start + m);
          p = load_v3(a.queries + 3 * q);
          sp = 0;
          next = __ldg(f.seg_root + m);
          pops = 0;
          bound2 = bound2_of(a, m);
          if constexpr (PREC == THEA_PRECISION_FP64_RECHECK) {
            f64_search_init(s);
            float scale = fmaxf(a.scene_scale, fmaxf(fabsf(p.x), fmaxf(fabsf(p.y), fabsf(p.z))));
            best = f64_band_start(bound2, scale, abs_tol);
            best32 = INFINITY;
          } else {
            best = thresh_of(a, m);
            best_idx = INT_MAX;
            best_slot = -1;
          }
        }
        qb += take < avail ? take : avail;
      }
    }
    if constexpr (PREC == THEA_PRECISION_FP64_RECHECK) {
      unsigned pend = __ballot_sync(FULL, pending);
      unsigned trav = __ballot_sync(FULL, q >= 0 && !pending);
      if (pend && (__popc(pend) >= REFILL_RESOLVE_AT || trav == 0)) {
        f64_resolve_warp(s, pending, f.cp_rec, ebase, p, bound2, *buf);
        if (pending) {
          ClosestOut r = f64_result(s);
          write_closest(q, r.idx != INT_MAX, (float)sqrt(r.d2_64), r.cp, r.idx, r.d2_64, a.out_index, a.out_dist,
                        a.out_cp, a.out_err);
          q = -1;
          pending = false;
        }
        continue;
      }
    }
    if (__ballot_sync(FULL, q >= 0) == 0) break;
    if (q < 0 || pending) continue;
    if (next == CHILD_EMPTY && sp == 0) {
      if constexpr (PREC == THEA_PRECISION_FP64_RECHECK) {
        s.lim = best;
        s.best32 = best32;
        pending = true;
      } else {
        write_closest(q, best_idx != INT_MAX, sqrtf(best), best_cp, best_idx, 0.0, a.out_index, a.out_dist, a.out_cp,
                      nullptr);
        q = -1;
      }
      continue;
    }
    if (budget > 0 && ++pops > budget) {
      // over budget (steps taken, the register-held child included): queued with the best element so far, finished
      // by a warp of its own in the second kernel
      unsigned long long pos = atomicAdd(hq.count, 1ull);
      hq.q[pos] = q;
      if constexpr (PREC == THEA_PRECISION_FP64_RECHECK) {
        hq.bound[pos] = best32;
        hq.idx[pos] = INT_MAX;
        hq.slot[pos] = -1;
      } else {
        hq.bound[pos] = best;
        hq.idx[pos] = best_idx;
        hq.slot[pos] = best_slot;
      }
      q = -1;
      continue;
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
      push_children_next<W, STACK>(nd, lb, best * PRUNE_SLACK, stk, sp, next, f.err);
    } else {
      int first, count;
      decode_leaf(code, first, count);
      if constexpr (PREC == THEA_PRECISION_FP64_RECHECK)
        cp_leaf_f64(f.cp_rec, ebase, first, count, p, bound2, abs_tol, best, best32, s);
      else
        cp_leaf_fp32(f.cp_rec, ebase, first, count, p, best, best_idx, best_slot, best_cp);
    }
  }
}

constexpr int PHASE2_WARPS = BATCH_THREADS / 32;

template <int W, int PREC>
__global__ void __launch_bounds__(BATCH_THREADS)
batch_closest_phase2_kernel(BatchForest f, ClosestArgs a, HardQueue hq, unsigned long long * counter) {
  __shared__ int s_code[PHASE2_WARPS][WARP_STACK];
  __shared__ float s_lb[PHASE2_WARPS][WARP_STACK];
  __shared__ float s_cd[PHASE2_WARPS][PREC == THEA_PRECISION_FP64_RECHECK ? WARP_CAND : 1];
  __shared__ int64_t s_ck[PHASE2_WARPS][PREC == THEA_PRECISION_FP64_RECHECK ? WARP_CAND : 1];
  WideNode<W> const * nodes = (WideNode<W> const *)f.nodes;
  int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned long long total = *hq.count;
  while (true) {
    unsigned long long j = 0;
    if (lane == 0) j = atomicAdd(counter, 1ull);
    j = __shfl_sync(0xffffffffu, j, 0);
    if (j >= total) break;
    int64_t q = hq.q[j];
    int m = mesh_of_query(a.qoff, f.M, q);
    int root = __ldg(f.seg_root + m);
    int64_t ebase = __ldg(f.seg_start + m);
    V3 p = load_v3(a.queries + 3 * q);
    if (PREC == THEA_PRECISION_FP64_RECHECK) {
      float scale = fmaxf(a.scene_scale, fmaxf(fabsf(p.x), fmaxf(fabsf(p.y), fabsf(p.z))));
      WarpBest64 b = closest_warp_query_f64<W>(nodes, f.cp_rec, root, ebase, p, bound2_of(a, m), scale, hq.bound[j],
                                               s_code[warp], s_lb[warp], s_cd[warp], s_ck[warp], f.err);
      if (lane == 0) {
        bool found = b.idx != INT_MAX;
        V3 cp = V3{0.f, 0.f, 0.f};
        if (found) {
          D3 cp64;
          double d64;
          cp_record_f64(f.cp_rec, b.slot, p, cp64, d64);
          cp = V3{(float)cp64.x, (float)cp64.y, (float)cp64.z};
        }
        write_closest(q, found, (float)sqrt(b.d2), cp, b.idx, b.d2, a.out_index, a.out_dist, a.out_cp, a.out_err);
      }
    } else {
      WarpBest init;
      init.idx = hq.idx[j];
      init.d2 = init.idx != INT_MAX ? hq.bound[j] : thresh_of(a, m);
      init.slot = hq.slot[j];
      // the queries over budget are the long searches (deep inside closed surfaces), which the slabs cut most
      WarpBest b = closest_warp_query<W>(nodes, f.cp_rec, root, ebase, p, init, s_code[warp], s_lb[warp], f.err,
                                         f.slabs);
      if (lane == 0) {
        bool found = b.idx != INT_MAX;
        V3 cp = V3{0.f, 0.f, 0.f};
        double d64 = 0.0;
        if (found) {
          cp_record_test(f.cp_rec, b.slot, p, cp);
          if (a.out_err) {
            D3 cp64;
            cp_record_f64(f.cp_rec, b.slot, p, cp64, d64);
          }
        }
        write_closest(q, found, sqrtf(b.d2), cp, b.idx, d64, a.out_index, a.out_dist, a.out_cp, a.out_err);
      }
    }
    __syncwarp();
  }
}

// Closest point of one BVH with queries and results in pinned host memory, read and written by the kernel (the
// in-place form of the first phase above, FP32 reference arithmetic): a warp copies each 64-query block into shared
// memory once, results collect in a per-warp ring of block buffers and are written out in query order with coalesced
// stores once the block is done. A query over the step budget is queued as in the first phase and counts as done for
// its block; the warp-per-query kernel then writes its result over the block's placeholder.
constexpr int CP_STREAM_RING = 4;
constexpr int CP_STREAM_WARPS = BATCH_THREADS / 32;

template <int W, int STACK>
__global__ void __launch_bounds__(BATCH_THREADS)
closest_stream_kernel(BatchForest f, ClosestArgs a, int64_t nq, unsigned long long * counter, int budget,
                      HardQueue hq) {
  __shared__ float s_in[CP_STREAM_WARPS][REFILL_BLOCK * 3];
  __shared__ int s_i[CP_STREAM_WARPS][CP_STREAM_RING][REFILL_BLOCK];
  __shared__ float s_d[CP_STREAM_WARPS][CP_STREAM_RING][REFILL_BLOCK];
  __shared__ float s_c[CP_STREAM_WARPS][CP_STREAM_RING][REFILL_BLOCK * 3];
  __shared__ int s_left[CP_STREAM_WARPS][CP_STREAM_RING];
  __shared__ long long s_base[CP_STREAM_WARPS][CP_STREAM_RING];
  __shared__ int s_cnt[CP_STREAM_WARPS][CP_STREAM_RING];
  unsigned const FULL = 0xffffffffu;
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  WideNode<W> const * nodes = (WideNode<W> const *)f.nodes;
  int const root = __ldg(f.seg_root);
  float * in = s_in[warp];
  int64_t qb = 0, qe = 0;  // queries of the current block not yet handed out, warp-uniform
  bool exhausted = false;  // warp-uniform
  long long taken = 0, oldest = 0;  // blocks taken / oldest block not written out, warp-uniform
  int64_t q = -1;
  int slot = 0;
  int64_t qbase = 0;
  V3 p = V3{0.f, 0.f, 0.f};
  int2 stk[STACK];
  int sp = 0;
  int next = CHILD_EMPTY;
  float best = 0.f;
  int best_idx = INT_MAX;
  int64_t best_slot = -1;
  V3 best_cp = V3{0.f, 0.f, 0.f};
  int pops = 0;
  while (true) {
    __syncwarp();
    while (oldest < taken && s_left[warp][oldest % CP_STREAM_RING] == 0) {
      int sl = (int)(oldest % CP_STREAM_RING);
      long long base = s_base[warp][sl];
      int cnt = s_cnt[warp][sl];
      for (int j = lane; j < cnt; j += 32) {
        a.out_index[base + j] = s_i[warp][sl][j];
        if (a.out_dist) a.out_dist[base + j] = s_d[warp][sl][j];
      }
      if (a.out_cp)
        for (int j = lane; j < 3 * cnt; j += 32) a.out_cp[3 * base + j] = s_c[warp][sl][j];
      ++oldest;
    }
    __syncwarp();
    unsigned idle = __ballot_sync(FULL, q < 0);
    if (idle && !exhausted) {
      if (qb >= qe && taken - oldest < CP_STREAM_RING) {
        unsigned long long b = 0;
        if (lane == 0) b = atomicAdd(counter, (unsigned long long)REFILL_BLOCK);
        b = __shfl_sync(FULL, b, 0);
        if ((int64_t)b >= nq) {
          exhausted = true;
        } else {
          qb = (int64_t)b;
          qe = qb + REFILL_BLOCK < nq ? qb + REFILL_BLOCK : nq;
          int cnt = (int)(qe - qb);
          for (int k = lane; k < 3 * cnt; k += 32) in[k] = a.queries[3 * qb + k];
          int sl = (int)(taken % CP_STREAM_RING);
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
          slot = (int)((taken - 1) % CP_STREAM_RING);
          qbase = s_base[warp][slot];
          float const * r = in + (q - qbase) * 3;
          p = V3{r[0], r[1], r[2]};
          best = a.thresh;
          best_idx = INT_MAX;
          best_slot = -1;
          sp = 0;
          next = root;
          pops = 0;
        }
        qb += take < avail ? take : avail;
      }
    }
    bool busy = __ballot_sync(FULL, q >= 0) != 0;
    if (!busy && oldest == taken && (exhausted || qb >= qe)) {
      if (exhausted) break;
      continue;
    }
    if (q < 0) continue;
    if (next == CHILD_EMPTY && sp == 0) {
      bool found = best_idx != INT_MAX;
      int j = (int)(q - qbase);
      s_i[warp][slot][j] = found ? best_idx : -1;
      s_d[warp][slot][j] = found ? sqrtf(best) : -1.f;
      s_c[warp][slot][3 * j] = found ? best_cp.x : 0.f;
      s_c[warp][slot][3 * j + 1] = found ? best_cp.y : 0.f;
      s_c[warp][slot][3 * j + 2] = found ? best_cp.z : 0.f;
      atomicSub(&s_left[warp][slot], 1);
      q = -1;
      continue;
    }
    if (budget > 0 && ++pops > budget) {
      // over budget: queued with its best element; the warp-per-query kernel writes its result in place later
      unsigned long long pos = atomicAdd(hq.count, 1ull);
      hq.q[pos] = q;
      hq.bound[pos] = best;
      hq.idx[pos] = best_idx;
      hq.slot[pos] = best_slot;
      atomicSub(&s_left[warp][slot], 1);
      q = -1;
      continue;
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
      push_children_next<W, STACK>(nd, lb, best * PRUNE_SLACK, stk, sp, next, f.err);
    } else {
      int first, count;
      decode_leaf(code, first, count);
      cp_leaf_fp32(f.cp_rec, 0, first, count, p, best, best_idx, best_slot, best_cp);
    }
  }
}

template <int W, int STACK>
__global__ void __launch_bounds__(BATCH_THREADS)
batch_ray_kernel(BatchForest f, float const * __restrict__ origins, float const * __restrict__ dirs,
                 int64_t const * __restrict__ qoff, int64_t nq, float max_time, float * __restrict__ out_time,
                 int32_t * __restrict__ out_index, unsigned long long * counter, int chunk) {
  WideNode<W> const * nodes = (WideNode<W> const *)f.nodes;
  int64_t base;
  while (next_chunk(counter, chunk, nq, base)) {
    int64_t end = base + chunk < nq ? base + chunk : nq;
    for (int64_t q = base + (threadIdx.x & 31); q < end; q += 32) {
      int m = mesh_of_query(qoff, f.M, q);
      RayOut r = ray_query<W, STACK, false>(nodes, f.ray_rec, __ldg(f.seg_root + m), __ldg(f.seg_start + m),
                                            load_v3(origins + 3 * q), load_v3(dirs + 3 * q), max_time, f.err);
      bool found = r.idx != INT_MAX;
      out_time[q] = found ? r.t : -1.f;
      if (out_index) out_index[q] = found ? r.idx : -1;
    }
  }
}

template <int W, int K, int STACK>
__global__ void __launch_bounds__(BATCH_THREADS)
batch_knn_kernel(BatchForest f, float const * __restrict__ queries, int64_t const * __restrict__ qoff, int64_t nq,
                 int k_out, float thresh, int32_t * __restrict__ out_index, float * __restrict__ out_d2,
                 unsigned long long * counter, int chunk) {
  WideNode<W> const * nodes = (WideNode<W> const *)f.nodes;
  int64_t base;
  while (next_chunk(counter, chunk, nq, base)) {
    int64_t end = base + chunk < nq ? base + chunk : nq;
    for (int64_t q = base + (threadIdx.x & 31); q < end; q += 32) {
      int m = mesh_of_query(qoff, f.M, q);
      float bd[K];
      int bi[K];
      if constexpr (K >= 8) {
        // the K-best list in shared memory, as the point k-NN kernel keeps it (more warps resident)
        __shared__ float s_d[K][BATCH_THREADS];
        __shared__ int s_i[K][BATCH_THREADS];
        int th = threadIdx.x;
#pragma unroll
        for (int j = 0; j < K; ++j) {
          s_d[j][th] = thresh;
          s_i[j][th] = INT_MAX;
        }
        float kth = thresh;
        int kth_i = INT_MAX;
        knn_query_shared<W, K, STACK, BATCH_THREADS>(nodes, f.pt_rec, __ldg(f.seg_root + m), __ldg(f.seg_start + m),
                                                     load_v3(queries + 3 * q), -1, s_d, s_i, kth, kth_i, f.err);
        // the row from shared memory
        for (int j = 0; j < k_out; ++j) {
          int bij = s_i[j][th];
          bool v = bij != INT_MAX;
          out_index[q * k_out + j] = v ? bij : -1;
          out_d2[q * k_out + j] = v ? s_d[j][th] : -1.f;
        }
        continue;
      } else {
#pragma unroll
        for (int j = 0; j < K; ++j) { bd[j] = thresh; bi[j] = INT_MAX; }
        knn_query<W, K, STACK>(nodes, f.pt_rec, __ldg(f.seg_root + m), __ldg(f.seg_start + m),
                               load_v3(queries + 3 * q), -1, bd, bi, f.err);
      }
      for (int j = 0; j < k_out; ++j) {
        bool v = bi[j] != INT_MAX;
        out_index[q * k_out + j] = v ? bi[j] : -1;
        out_d2[q * k_out + j] = v ? bd[j] : -1.f;
      }
    }
  }
}

int persistent_grid(void const * kernel) {
  int sms = sm_count();
  int per_sm = 0;
  THEA_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, BATCH_THREADS, 0));
  return std::max(1, per_sm) * sms;
}

template <int W, int STACK, int PREC>
void launch_closest_prec(BatchForest const & f, ClosestArgs const & a, int64_t nq, int budget,
                         unsigned long long * counters, int chunk, HardQueue const & hq, cudaStream_t s) {
  auto k1 = batch_closest_kernel<W, STACK, PREC>;
  // FP32 without error estimates: persistent lanes (1.5x on the 256-mesh case), also as the first phase of the
  // two-phase form. The mixed-precision search stays on rounds: it is bound by the FP64 pipe, and rounds fill the FP64
  // step better (27.5 against 25.7 ms measured).
  bool refill = PREC != THEA_PRECISION_FP64_RECHECK && !a.out_err;
  if (budget <= 0) {
    if (refill) {
      auto kr = batch_closest_refill_kernel<W, STACK, PREC>;
      THEA_LAUNCH_NAMED("batch_closest_kernel_fp32", kr, persistent_grid((void const *)kr), BATCH_THREADS, 0, s, f, a,
                        nq, counters, 0, hq);
      return;
    }
    THEA_LAUNCH_NAMED(PREC == THEA_PRECISION_FP64_RECHECK ? "batch_closest_kernel_fp64" : "batch_closest_kernel_fp32",
                      k1, persistent_grid((void const *)k1), BATCH_THREADS, 0, s, f, a, nq, counters, chunk, 0, hq);
    return;
  }
  if (refill) {
    auto kr = batch_closest_refill_kernel<W, STACK, PREC>;
    THEA_LAUNCH_NAMED("batch_closest_phase1_kernel", kr, persistent_grid((void const *)kr), BATCH_THREADS, 0, s, f, a,
                      nq, counters, budget, hq);
  } else {
    THEA_LAUNCH_NAMED("batch_closest_phase1_kernel", k1, persistent_grid((void const *)k1), BATCH_THREADS, 0, s, f, a,
                      nq, counters, chunk, budget, hq);
  }
  auto k2 = batch_closest_phase2_kernel<W, PREC>;
  THEA_LAUNCH_NAMED("batch_closest_phase2_kernel", k2, persistent_grid((void const *)k2), BATCH_THREADS, 0, s, f, a, hq,
                    counters + 1);
}

template <int W, int STACK>
void launch_batch_closest(BatchForest const & f, ClosestArgs const & a, int64_t nq, int prec, int budget,
                          unsigned long long * counters, int chunk, HardQueue const & hq, cudaStream_t s) {
  if (prec == THEA_PRECISION_FP64_RECHECK)
    launch_closest_prec<W, STACK, THEA_PRECISION_FP64_RECHECK>(f, a, nq, budget, counters, chunk, hq, s);
  else
    launch_closest_prec<W, STACK, THEA_PRECISION_FP32_REFERENCE>(f, a, nq, budget, counters, chunk, hq, s);
}

template <int W, int STACK>
void launch_batch_ray(BatchForest const & f, float const * o, float const * d, int64_t const * qoff, int64_t nq,
                      float max_time, float * t, int32_t * idx, unsigned long long * counter, int chunk,
                      cudaStream_t s) {
  auto k = batch_ray_kernel<W, STACK>;
  THEA_LAUNCH_NAMED("batch_ray_kernel", k, persistent_grid((void const *)k), BATCH_THREADS, 0, s, f, o, d, qoff, nq, max_time, t, idx, counter,
              chunk);
}

template <int W, int K, int STACK>
void launch_batch_knn_k(BatchForest const & f, float const * q, int64_t const * qoff, int64_t nq, int k, float thresh,
                        int32_t * idx, float * d2, unsigned long long * counter, int chunk, cudaStream_t s) {
  auto kern = batch_knn_kernel<W, K, STACK>;
  THEA_LAUNCH_NAMED("batch_knn_kernel", kern, persistent_grid((void const *)kern), BATCH_THREADS, 0, s, f, q, qoff, nq, k, thresh, idx, d2,
              counter, chunk);
}

template <int W, int STACK>
void launch_batch_knn(BatchForest const & f, float const * q, int64_t const * qoff, int64_t nq, int k, float thresh,
                      int32_t * idx, float * d2, unsigned long long * counter, int chunk, cudaStream_t s) {
  if (k <= 1) launch_batch_knn_k<W, 1, STACK>(f, q, qoff, nq, k, thresh, idx, d2, counter, chunk, s);
  else if (k <= 2) launch_batch_knn_k<W, 2, STACK>(f, q, qoff, nq, k, thresh, idx, d2, counter, chunk, s);
  else if (k <= 4) launch_batch_knn_k<W, 4, STACK>(f, q, qoff, nq, k, thresh, idx, d2, counter, chunk, s);
  else if (k <= 8) launch_batch_knn_k<W, 8, STACK>(f, q, qoff, nq, k, thresh, idx, d2, counter, chunk, s);
  else if (k <= 16) launch_batch_knn_k<W, 16, STACK>(f, q, qoff, nq, k, thresh, idx, d2, counter, chunk, s);
  else launch_batch_knn_k<W, 32, STACK>(f, q, qoff, nq, k, thresh, idx, d2, counter, chunk, s);
}

}  // namespace

BatchForest forest_view(thea_bvh const * b) {
  BatchForest f;
  f.nodes = b->nodes;
  f.cp_rec = b->cp_rec;
  f.ray_rec = b->ray_rec;
  f.pt_rec = b->pt_rec;
  f.slabs = b->slabs;
  f.seg_start = b->seg_start;
  f.seg_root = b->seg_root;
  f.M = b->num_segments;
  f.err = b->err;
  return f;
}

namespace {

// FP64 re-check batches take their queries in (mesh, Morton code) order: a warp's round of 32 queries then holds
// neighbours, whose searches take similar paths and share band candidates (256 config-3 meshes: 24.9 -> 20.8 ms). The
// FP32 kernels refill lanes one query at a time and ran slower on sorted queries (11.2 -> 12.4 ms), so they keep the
// caller's order. Results do not depend on the order.
constexpr int64_t SORTED_QUERIES_MIN = 1 << 15;

__device__ __forceinline__ uint32_t spread10(uint32_t x) {
  x &= 0x3ffu;
  x = (x | (x << 16)) & 0x030000ffu;
  x = (x | (x << 8)) & 0x0300f00fu;
  x = (x | (x << 4)) & 0x030c30c3u;
  x = (x | (x << 2)) & 0x09249249u;
  return x;
}

__global__ void sorted_query_keys_kernel(float const * __restrict__ q, int64_t const * __restrict__ qoff, int M,
                                         int64_t nq, float lx, float ly, float lz, float sx, float sy, float sz,
                                         uint64_t * __restrict__ keys, uint32_t * __restrict__ vals) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nq) return;
  int m = mesh_of_query(qoff, M, i);
  float c[3] = {(q[3 * i] - lx) * sx, (q[3 * i + 1] - ly) * sy, (q[3 * i + 2] - lz) * sz};
  uint32_t g[3];
#pragma unroll
  for (int t = 0; t < 3; ++t) {
    float u = fminf(fmaxf(c[t], 0.f), 1.f);  // NaN-safe: fminf/fmaxf drop a NaN operand
    g[t] = min((uint32_t)(u * 1024.f), 1023u);
  }
  keys[i] = ((uint64_t)m << 30) | (spread10(g[0]) << 2) | (spread10(g[1]) << 1) | spread10(g[2]);
  vals[i] = (uint32_t)i;
}

__global__ void gather_queries_kernel(float const * __restrict__ q, uint32_t const * __restrict__ order, int64_t nq,
                                      float * __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nq) return;
  int64_t j = order[i];
  out[3 * i] = q[3 * j];
  out[3 * i + 1] = q[3 * j + 1];
  out[3 * i + 2] = q[3 * j + 2];
}

__global__ void scatter_closest_kernel(uint32_t const * __restrict__ order, int64_t nq, int32_t const * __restrict__ si,
                                       float const * __restrict__ sd, float const * __restrict__ sc,
                                       float const * __restrict__ se, int32_t * __restrict__ idx,
                                       float * __restrict__ dist, float * __restrict__ cpt, float * __restrict__ err) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nq) return;
  int64_t j = order[i];
  idx[j] = si[i];
  if (dist) dist[j] = sd[i];
  if (cpt) {
    cpt[3 * j] = sc[3 * i];
    cpt[3 * j + 1] = sc[3 * i + 1];
    cpt[3 * j + 2] = sc[3 * i + 2];
  }
  if (err) err[j] = se[i];
}

// One batched closest-point search of `a` (queries, offsets, outputs) over the forest
void batch_closest_core(thea_bvh const * b, ClosestArgs const & a, int64_t nq, ClosestParams const & cp, int chunk,
                        cudaStream_t s) {
  BatchForest f = forest_view(b);
  bool sm = small_stack_ok(b);
  int budget = cp.budget > 0 ? cp.budget : 0;
  Scratch counters(3 * sizeof(unsigned long long), s);
  THEA_CUDA_CHECK(cudaMemsetAsync(counters.ptr, 0, 3 * sizeof(unsigned long long), s));
  auto * c = counters.as<unsigned long long>();
  size_t hq_n = budget > 0 ? (size_t)nq : 0;
  Scratch hq_q(hq_n * sizeof(int64_t), s), hq_b(hq_n * sizeof(float), s);
  Scratch hq_i(hq_n * sizeof(int32_t), s), hq_s(hq_n * sizeof(int64_t), s);
  HardQueue hq{hq_q.as<int64_t>(), hq_b.as<float>(), hq_i.as<int32_t>(), hq_s.as<int64_t>(), c + 2};
  if (b->width == 4) sm ? launch_batch_closest<4, 64>(f, a, nq, cp.precision, budget, c, chunk, hq, s)
                        : launch_batch_closest<4, 256>(f, a, nq, cp.precision, budget, c, chunk, hq, s);
  else sm ? launch_batch_closest<8, 128>(f, a, nq, cp.precision, budget, c, chunk, hq, s)
          : launch_batch_closest<8, 512>(f, a, nq, cp.precision, budget, c, chunk, hq, s);
}

// batch_closest_core on the queries in (mesh, Morton code) order: keys, a stable radix sort, the permuted copy, the
// search into scratch outputs, then the results scattered back to the caller's order
void batch_closest_sorted(thea_bvh const * b, float const * q, int64_t const * qoff, int64_t nq,
                          ClosestParams const & cp, int chunk, int32_t * idx, float * dist, float * cpt, float * err,
                          cudaStream_t s) {
  float sc[3];
  for (int t = 0; t < 3; ++t) {
    float ext = b->hi[t] - b->lo[t];
    sc[t] = ext > 0.f ? 1.0f / ext : 0.f;
  }
  Scratch keys((size_t)nq * sizeof(uint64_t), s), order((size_t)nq * sizeof(uint32_t), s);
  unsigned grid = (unsigned)ceil_div(nq, 256);
  THEA_LAUNCH(sorted_query_keys_kernel, grid, 256, 0, s, q, qoff, b->num_segments, nq, b->lo[0], b->lo[1], b->lo[2],
              sc[0], sc[1], sc[2], keys.as<uint64_t>(), order.as<uint32_t>());
  int seg_bits = 0;
  while ((1 << seg_bits) < b->num_segments) ++seg_bits;
  radix_sort_pairs(keys.as<uint64_t>(), order.as<uint32_t>(), nq, 30 + seg_bits, s, /*probe_passes=*/false);
  keys = Scratch();
  Scratch qs((size_t)nq * 12, s), si((size_t)nq * 4, s), sd(dist ? (size_t)nq * 4 : 0, s);
  Scratch scp(cpt ? (size_t)nq * 12 : 0, s), se(err ? (size_t)nq * 4 : 0, s);
  THEA_LAUNCH(gather_queries_kernel, grid, 256, 0, s, q, order.as<uint32_t>(), nq, qs.as<float>());
  ClosestArgs a{qs.as<float>(), qoff, cp.thresh, cp.bound2, cp.scene_scale, si.as<int32_t>(),
                dist ? sd.as<float>() : nullptr, cpt ? scp.as<float>() : nullptr, err ? se.as<float>() : nullptr,
                cp.seg_cut};
  batch_closest_core(b, a, nq, cp, chunk, s);
  THEA_LAUNCH(scatter_closest_kernel, grid, 256, 0, s, order.as<uint32_t>(), nq, si.as<int32_t>(),
              dist ? sd.as<float>() : nullptr, cpt ? scp.as<float>() : nullptr, err ? se.as<float>() : nullptr, idx,
              dist, cpt, err);
}

}  // namespace

void run_batch_closest(thea_bvh const * b, float const * q, int64_t const * qoff, int64_t nq, ClosestParams const & cp,
                       int chunk, int32_t * idx, float * dist, float * cpt, float * err, cudaStream_t s) {
  if (nq <= 0) return;
  if (cp.precision == THEA_PRECISION_FP64_RECHECK && nq >= SORTED_QUERIES_MIN && nq < ((int64_t)1 << 32) &&
      b->num_segments <= (1 << 20)) {
    batch_closest_sorted(b, q, qoff, nq, cp, chunk, idx, dist, cpt, err, s);
    return;
  }
  ClosestArgs a{q, qoff, cp.thresh, cp.bound2, cp.scene_scale, idx, dist, cpt, err, cp.seg_cut};
  batch_closest_core(b, a, nq, cp, chunk, s);
}

template <int W, int STACK>
void launch_closest_stream(BatchForest const & f, ClosestArgs const & a, int64_t nq, int budget,
                           unsigned long long * counters, HardQueue const & hq, cudaStream_t s) {
  auto k1 = closest_stream_kernel<W, STACK>;
  int64_t need = ceil_div(ceil_div(nq, REFILL_BLOCK) * 32, BATCH_THREADS);
  unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(persistent_grid((void const *)k1), need));
  THEA_LAUNCH_NAMED("closest_stream_kernel", k1, grid, BATCH_THREADS, 0, s, f, a, nq, counters, budget, hq);
  auto k2 = batch_closest_phase2_kernel<W, THEA_PRECISION_FP32_REFERENCE>;
  THEA_LAUNCH_NAMED("batch_closest_phase2_kernel", k2, persistent_grid((void const *)k2), BATCH_THREADS, 0, s, f, a, hq,
                    counters + 1);
}

void run_closest_stream(thea_bvh const * b, float const * q, int64_t nq, ClosestParams const & cp, int32_t * idx,
                        float * dist, float * cpt, cudaStream_t s) {
  if (nq <= 0) return;
  THEA_REQUIRE(b->num_segments == 1, "closest_stream: one BVH only");
  BatchForest f = forest_view(b);
  bool sm = small_stack_ok(b);
  ClosestArgs a{q, nullptr, cp.thresh, cp.bound2, cp.scene_scale, idx, dist, cpt, nullptr};
  int budget = cp.budget > 0 ? cp.budget : 0;
  Scratch counters(3 * sizeof(unsigned long long), s);
  THEA_CUDA_CHECK(cudaMemsetAsync(counters.ptr, 0, 3 * sizeof(unsigned long long), s));
  auto * c = counters.as<unsigned long long>();
  size_t hq_n = budget > 0 ? (size_t)nq : 1;
  Scratch hq_q(hq_n * sizeof(int64_t), s), hq_b(hq_n * sizeof(float), s);
  Scratch hq_i(hq_n * sizeof(int32_t), s), hq_s(hq_n * sizeof(int64_t), s);
  HardQueue hq{hq_q.as<int64_t>(), hq_b.as<float>(), hq_i.as<int32_t>(), hq_s.as<int64_t>(), c + 2};
  if (b->width == 4) sm ? launch_closest_stream<4, 64>(f, a, nq, budget, c, hq, s)
                        : launch_closest_stream<4, 256>(f, a, nq, budget, c, hq, s);
  else sm ? launch_closest_stream<8, 128>(f, a, nq, budget, c, hq, s)
          : launch_closest_stream<8, 512>(f, a, nq, budget, c, hq, s);
}

void run_batch_ray(thea_bvh const * b, float const * o, float const * d, int64_t const * qoff, int64_t nq,
                   float max_time, int chunk, float * t, int32_t * idx, cudaStream_t s) {
  if (nq <= 0) return;
  BatchForest f = forest_view(b);
  Scratch counter(sizeof(unsigned long long), s);
  THEA_CUDA_CHECK(cudaMemsetAsync(counter.ptr, 0, sizeof(unsigned long long), s));
  auto * c = counter.as<unsigned long long>();
  bool sm = small_stack_ok(b);
  if (b->width == 4) sm ? launch_batch_ray<4, 64>(f, o, d, qoff, nq, max_time, t, idx, c, chunk, s)
                        : launch_batch_ray<4, 256>(f, o, d, qoff, nq, max_time, t, idx, c, chunk, s);
  else sm ? launch_batch_ray<8, 128>(f, o, d, qoff, nq, max_time, t, idx, c, chunk, s)
          : launch_batch_ray<8, 512>(f, o, d, qoff, nq, max_time, t, idx, c, chunk, s);
}

void run_batch_knn(thea_bvh const * b, float const * q, int64_t const * qoff, int64_t nq, int k, float thresh,
                   int chunk, int32_t * idx, float * d2, cudaStream_t s) {
  if (nq <= 0) return;
  BatchForest f = forest_view(b);
  Scratch counter(sizeof(unsigned long long), s);
  THEA_CUDA_CHECK(cudaMemsetAsync(counter.ptr, 0, sizeof(unsigned long long), s));
  auto * c = counter.as<unsigned long long>();
  bool sm = small_stack_ok(b);
  if (b->width == 4) sm ? launch_batch_knn<4, 64>(f, q, qoff, nq, k, thresh, idx, d2, c, chunk, s)
                        : launch_batch_knn<4, 256>(f, q, qoff, nq, k, thresh, idx, d2, c, chunk, s);
  else sm ? launch_batch_knn<8, 128>(f, q, qoff, nq, k, thresh, idx, d2, c, chunk, s)
          : launch_batch_knn<8, 512>(f, q, qoff, nq, k, thresh, idx, d2, c, chunk, s);
}

}  // namespace thea
