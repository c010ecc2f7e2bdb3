// Warp-cooperative closest-element search for the queries that one thread cannot finish cheaply (points deep inside a
// closed mesh, where thousands of nodes lie within the pruning bound).
//
// A whole warp serves one query. Each step pops up to 32 / W internal nodes from a per-warp stack in shared memory; lane
// l tests child (l mod W) of node (l / W): its box against the current best, and, for a leaf child, the leaf's elements
// with the reference's FP32 arithmetic. The warp then agrees on the best (d2, index) by a shuffle reduction, sorts the
// surviving internal children by their lower bound with a bitonic network across the lanes, and pushes them with the
// nearest on top, so the search stays close to nearest-first while keeping all 32 lanes busy.
#pragma once

#include "traverse_ops.cuh"

namespace thea {

constexpr int WARP_STACK = 1024;  // entries per warp (code + bound = 8 KB)

// Lexicographic (d2, index) key: non-negative float bits order like unsigned integers.
__device__ __forceinline__ unsigned long long best_key(float d2, int idx) {
  return ((unsigned long long)__float_as_uint(d2) << 32) | (unsigned)idx;
}

__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long u = __shfl_xor_sync(0xffffffffu, v, o);
    v = u < v ? u : v;
  }
  return v;
}

// Ascending bitonic sort of one (key, code) pair per lane.
__device__ __forceinline__ void warp_sort_pairs(uint32_t & key, int & code) {
  int lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      uint32_t pk = __shfl_xor_sync(0xffffffffu, key, j);
      int pc = __shfl_xor_sync(0xffffffffu, code, j);
      bool ascending = (lane & k) == 0;
      bool lower = (lane & j) == 0;
      bool take = (lower == ascending) ? (pk < key) : (pk > key);
      if (take) {
        key = pk;
        code = pc;
      }
    }
  }
}

// Reads the box and code of child c of node `idx` (one lane per child; the lanes of a node read one 128-byte line).
template <int W>
__device__ __forceinline__ void load_child(WideNode<W> const * __restrict__ nodes, int idx, int c, float & lx, float & hx,
                                           float & ly, float & hy, float & lz, float & hz, int & child) {
  float const * f = reinterpret_cast<float const *>(nodes + idx);
  lx = __ldg(f + 0 * W + c);
  hx = __ldg(f + 1 * W + c);
  ly = __ldg(f + 2 * W + c);
  hy = __ldg(f + 3 * W + c);
  lz = __ldg(f + 4 * W + c);
  hz = __ldg(f + 5 * W + c);
  child = __ldg(reinterpret_cast<int const *>(f + 6 * W) + c);
}

struct WarpBest {
  float d2;
  int idx;
  int64_t slot;
};

// FP32 search from `root` with an initial best (d2, idx, slot) that is a valid element (or +inf / INT_MAX / -1).
// s_code / s_lb: this warp's shared-memory stack. Returns the warp-uniform best.
template <int W>
__device__ WarpBest closest_warp_query(WideNode<W> const * __restrict__ nodes, float4 const * __restrict__ rec,
                                       int root, int64_t elem_base, V3 p, WarpBest best, int * s_code, float * s_lb,
                                       unsigned * err, float4 const * __restrict__ slabs = nullptr) {
  float q1 = fabsf(p.x) + fabsf(p.y) + fabsf(p.z);
  constexpr int NPOP = 32 / W;
  int lane = threadIdx.x & 31;
  int e = lane / W, c = lane % W;
  int sp = 1;
  if (lane == 0) {
    s_code[0] = root;
    s_lb[0] = 0.f;
  }
  __syncwarp();
  unsigned long long bkey = best_key(best.d2, best.idx);
  while (sp > 0) {
    int npop = sp < NPOP ? sp : NPOP;
    int base = sp - npop;
    int code = CHILD_EMPTY;
    float lbe = 0.f;
    if (e < npop) {
      code = s_code[base + e];
      lbe = s_lb[base + e];
    }
    __syncwarp();
    sp = base;
    float bd = __uint_as_float((unsigned)(bkey >> 32));
    float lim = bd * PRUNE_SLACK;
    uint32_t key = 0xffffffffu;
    int push_code = CHILD_EMPTY;
    unsigned long long my_key = ~0ull;
    int64_t my_slot = -1;
    if (code != CHILD_EMPTY && lbe <= lim) {
      float lx, hx, ly, hy, lz, hz;
      int child;
      load_child<W>(nodes, code, c, lx, hx, ly, hy, lz, hz, child);
      float d2b = point_box_d2(p.x, p.y, p.z, lx, ly, lz, hx, hy, hz);
      if (slabs && child != CHILD_EMPTY) {
        // the child's oriented slab raises its bound (single-mesh BVHs)
        float d;
        d2b = fmaxf(d2b, slab_lower_bound(__ldg(slabs + (int64_t)code * W + c), p, q1, d));
      }
      if (child != CHILD_EMPTY && d2b <= lim) {
        if (child >= 0) {
          key = __float_as_uint(d2b);
          push_code = child;
        } else {
          int first, count;
          decode_leaf(child, first, count);
          int64_t k0 = elem_base + first;
          for (int64_t k = k0; k < k0 + count; ++k) {
            V3 cp;
            float d2 = cp_record_test(rec, k, p, cp);
            if (d2 <= bd) {
              unsigned long long kk = best_key(d2, cp_record_index(rec, k));
              if (kk < my_key) {
                my_key = kk;
                my_slot = k;
              }
            }
          }
        }
      }
    }
    // agree on the best element
    unsigned long long wmin = warp_min_u64(my_key);
    if (wmin < bkey) {
      unsigned who = __ballot_sync(0xffffffffu, my_key == wmin);
      int src = __ffs(who) - 1;
      best.slot = __shfl_sync(0xffffffffu, my_slot, src);
      bkey = wmin;
    }
    // push surviving internal children, nearest on top
    warp_sort_pairs(key, push_code);
    unsigned valid = __ballot_sync(0xffffffffu, key != 0xffffffffu);
    int m = __popc(valid);
    if (sp + m > WARP_STACK) {
      if (lane == 0) atomicOr(err, ERR_STACK_OVERFLOW);
      m = WARP_STACK - sp;
    }
    if (lane < m) {
      int pos = sp + (m - 1 - lane);
      s_code[pos] = push_code;
      s_lb[pos] = __uint_as_float(key);
    }
    __syncwarp();
    sp += m;
  }
  best.d2 = __uint_as_float((unsigned)(bkey >> 32));
  best.idx = (int)(unsigned)(bkey & 0xffffffffu);
  return best;
}

constexpr int WARP_CAND = 64;  // FP64 candidates per warp

struct WarpBest64 {
  double d2;
  int idx;
  int64_t slot;
};

// Mixed-precision form of closest_warp_query (the band rule of closest_query_f64): FP32 traversal and tests; elements
// within the band of the FP32 best are collected in a per-warp list and evaluated in FP64 at the end (or at once when
// the list is full). init_best32: FP32 squared distance of a known element (a valid upper bound) or +inf.
template <int W>
__device__ WarpBest64 closest_warp_query_f64(WideNode<W> const * __restrict__ nodes, float4 const * __restrict__ rec,
                                             int root, int64_t elem_base, V3 p, double bound2, float scale,
                                             float init_best32, int * s_code, float * s_lb, float * s_cd,
                                             int64_t * s_ck, unsigned * err) {
  constexpr int NPOP = 32 / W;
  float const REL = 1.0f + 1.0f / 16384.0f;
  float abs_tol = scale * (1.0f / 262144.0f);
  int lane = threadIdx.x & 31;
  int e = lane / W, c = lane % W;
  auto band = [&](float b32) {
    float lb = sqrtf(b32) * REL + abs_tol;
    return lb * lb;
  };
  float lim = INFINITY;
  if (bound2 >= 0.0) lim = band(__double2float_ru(bound2));
  if (init_best32 < INFINITY) lim = fminf(lim, band(init_best32));
  double my64 = INFINITY;
  int my_idx = INT_MAX;
  int64_t my_slot = -1;
  auto eval64 = [&](int64_t k) {
    D3 cp64;
    double d64;
    cp_record_f64(rec, k, p, cp64, d64);
    if (bound2 >= 0.0 && !(d64 < bound2)) return;
    int idx = cp_record_index(rec, k);
    if (d64 < my64 || (d64 == my64 && idx < my_idx)) {
      my64 = d64;
      my_idx = idx;
      my_slot = k;
    }
  };
  int ncand = 0;
  int sp = 1;
  if (lane == 0) {
    s_code[0] = root;
    s_lb[0] = 0.f;
  }
  __syncwarp();
  while (sp > 0) {
    int npop = sp < NPOP ? sp : NPOP;
    int base = sp - npop;
    int code = CHILD_EMPTY;
    float lbe = 0.f;
    if (e < npop) {
      code = s_code[base + e];
      lbe = s_lb[base + e];
    }
    __syncwarp();
    sp = base;
    float plim = lim * PRUNE_SLACK;
    uint32_t key = 0xffffffffu;
    int push_code = CHILD_EMPTY;
    float my_best32 = INFINITY;
    // up to MAX_LEAF_SIZE candidates per lane this step; kept in registers until appended
    float cd[MAX_LEAF_SIZE];
    int64_t ck[MAX_LEAF_SIZE];
    int nc = 0;
    if (code != CHILD_EMPTY && lbe <= plim) {
      float lx, hx, ly, hy, lz, hz;
      int child;
      load_child<W>(nodes, code, c, lx, hx, ly, hy, lz, hz, child);
      float d2b = point_box_d2(p.x, p.y, p.z, lx, ly, lz, hx, hy, hz);
      if (child != CHILD_EMPTY && d2b <= plim) {
        if (child >= 0) {
          key = __float_as_uint(d2b);
          push_code = child;
        } else {
          int first, count;
          decode_leaf(child, first, count);
          int64_t k0 = elem_base + first;
          for (int j = 0; j < count; ++j) {
            V3 cp;
            float d2 = cp_record_test(rec, k0 + j, p, cp);
            if (d2 <= lim) {
              my_best32 = fminf(my_best32, d2);
#pragma unroll
              for (int t = 0; t < MAX_LEAF_SIZE; ++t)
                if (t == nc) { cd[t] = d2; ck[t] = k0 + j; }
              ++nc;
            }
          }
        }
      }
    }
    // tighten the band with the warp's best FP32 distance
    float wb = my_best32;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) wb = fminf(wb, __shfl_xor_sync(0xffffffffu, wb, o));
    if (wb < INFINITY) lim = fminf(lim, band(wb));
    // append this step's candidates that are still in the band; compact or evaluate when the list is full
    int nmax = (int)__reduce_max_sync(0xffffffffu, (unsigned)nc);
    for (int t = 0; t < nmax; ++t) {
      bool have = t < nc && cd[t] <= lim;
      unsigned ball = __ballot_sync(0xffffffffu, have);
      if (!ball) continue;
      int cnt = __popc(ball);
      if (ncand + cnt > WARP_CAND) {
        // drop entries that left the band
        int keep_n = 0;
        for (int b = 0; b < ncand; b += 32) {
          int j = b + lane;
          bool keep = j < ncand && s_cd[j] <= lim;
          float kd = keep ? s_cd[j] : 0.f;
          int64_t kk = keep ? s_ck[j] : 0;
          unsigned kb = __ballot_sync(0xffffffffu, keep);
          __syncwarp();
          if (keep) {
            int pos = keep_n + __popc(kb & ((1u << lane) - 1u));
            s_cd[pos] = kd;
            s_ck[pos] = kk;
          }
          keep_n += __popc(kb);
          __syncwarp();
        }
        ncand = keep_n;
      }
      if (ncand + cnt > WARP_CAND) {
        if (have) eval64(ck[t]);  // no room: evaluate now
      } else {
        if (have) {
          int pos = ncand + __popc(ball & ((1u << lane) - 1u));
          s_cd[pos] = cd[t];
          s_ck[pos] = ck[t];
        }
        ncand += cnt;
      }
      __syncwarp();
    }
    // push surviving internal children, nearest on top
    warp_sort_pairs(key, push_code);
    unsigned valid = __ballot_sync(0xffffffffu, key != 0xffffffffu);
    int m = __popc(valid);
    if (sp + m > WARP_STACK) {
      if (lane == 0) atomicOr(err, ERR_STACK_OVERFLOW);
      m = WARP_STACK - sp;
    }
    if (lane < m) {
      int pos = sp + (m - 1 - lane);
      s_code[pos] = push_code;
      s_lb[pos] = __uint_as_float(key);
    }
    __syncwarp();
    sp += m;
  }
  // FP64 evaluation of the final band
  for (int j = lane; j < ncand; j += 32)
    if (s_cd[j] <= lim) eval64(s_ck[j]);
  double wmin = my64;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double u = __shfl_xor_sync(0xffffffffu, wmin, o);
    wmin = u < wmin ? u : wmin;
  }
  unsigned cand_idx = (my64 == wmin) ? (unsigned)my_idx : 0xffffffffu;
  unsigned widx = __reduce_min_sync(0xffffffffu, cand_idx);
  unsigned who = __ballot_sync(0xffffffffu, my64 == wmin && (unsigned)my_idx == widx);
  WarpBest64 out;
  out.d2 = wmin;
  out.idx = (int)widx;
  out.slot = who ? __shfl_sync(0xffffffffu, my_slot, __ffs(who) - 1) : -1;
  if (!(wmin < INFINITY)) out.idx = INT_MAX;
  return out;
}

}  // namespace thea
