// LBVH build of a forest: one BVH per segment of elements (one segment for a single mesh or point set; one per mesh
// for a batch), all built together in one pass: element boxes -> per-segment 3D Morton codes with the segment id in the
// top bits -> one stable radix sort -> Karras binary radix trees that never cross a segment boundary -> bottom-up box
// refit -> top-down collapse into W-wide trees whose leaves are contiguous runs of sorted elements -> element records in
// leaf order.
//
// Replaces BvhN::init / initTree / createKdTree (Code/Source/Algorithms/BvhN.hpp:705-794, 1366-1525). The reference
// builds a median-split kd-tree with leaves of at most 5 elements and pads every node box by 5%; this build produces a
// different tree over the same elements. Query results do not depend on the tree: every query returns the element with
// the smallest distance or hit time, ties to the lowest index, and node boxes are padded so that no element at the best
// distance can be pruned by rounding.
//
// Index conventions: elements are addressed by their global sorted position; a leaf stores its first element relative to
// its segment's first sorted position (so one segment may hold up to 2^27 - 1 elements while a forest may hold more),
// and element records store the element's index within its segment (the face index within its mesh).
#include "bvh.hpp"
#include "device_util.cuh"
#include "query.hpp"
#include "traverse_ops.cuh"

#include <algorithm>
#include <vector>

namespace thea {
namespace {

constexpr int BUILD_THREADS = 256;

__device__ __forceinline__ int f2ord(float f) {
  int i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7fffffff;
}
__host__ __device__ __forceinline__ float ord2f(int i) {
#ifdef __CUDA_ARCH__
  return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff);
#else
  int j = i >= 0 ? i : i ^ 0x7fffffff;
  float f;
  memcpy(&f, &j, 4);
  return f;
#endif
}

// Segment of element i: largest s with start[s] <= i (start has M + 1 entries, start[0] = 0)
__device__ __forceinline__ int segment_of(int64_t const * __restrict__ start, int M, int64_t i) {
  int lo = 0, hi = M - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (start[mid] <= i) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Per-segment bounds, 12 ordered ints per segment: [0..2] min of box centres, [3..5] max of box centres,
// [6..8] min of box lo, [9..11] max of box hi. A warp whose lanes share one segment reduces before its atomics, and a
// block whose warps all share one segment reduces once more, so a single large segment takes 12 atomics per block
// rather than per warp (the per-warp form spent 0.5 ms of contended atomics on 2 M triangles).
__global__ void elem_box_kernel(float const * __restrict__ V, int32_t const * __restrict__ F, int64_t n, int is_mesh,
                                int64_t const * __restrict__ seg_start, int M, float4 * __restrict__ elo,
                                float4 * __restrict__ ehi, int * __restrict__ bounds) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool ok = i < n;
  int v[12];
  int seg = 0;
  if (ok) {
    V3 lo, hi;
    if (is_mesh) {
      V3 a = load_v3(V + 3 * (int64_t)F[3 * i]);
      V3 b = load_v3(V + 3 * (int64_t)F[3 * i + 1]);
      V3 c = load_v3(V + 3 * (int64_t)F[3 * i + 2]);
      lo = V3{fminf(a.x, fminf(b.x, c.x)), fminf(a.y, fminf(b.y, c.y)), fminf(a.z, fminf(b.z, c.z))};
      hi = V3{fmaxf(a.x, fmaxf(b.x, c.x)), fmaxf(a.y, fmaxf(b.y, c.y)), fmaxf(a.z, fmaxf(b.z, c.z))};
    } else {
      lo = hi = load_v3(V + 3 * i);
    }
    elo[i] = make_float4(lo.x, lo.y, lo.z, 0.f);
    ehi[i] = make_float4(hi.x, hi.y, hi.z, 0.f);
    V3 c = 0.5f * (hi + lo);
    v[0] = v[3] = f2ord(c.x); v[1] = v[4] = f2ord(c.y); v[2] = v[5] = f2ord(c.z);
    v[6] = f2ord(lo.x); v[7] = f2ord(lo.y); v[8] = f2ord(lo.z);
    v[9] = f2ord(hi.x); v[10] = f2ord(hi.y); v[11] = f2ord(hi.z);
    seg = M > 1 ? segment_of(seg_start, M, i) : 0;
  } else {
#pragma unroll
    for (int t = 0; t < 12; ++t) v[t] = ((t < 3) || (t >= 6 && t < 9)) ? INT_MAX : INT_MIN;
    seg = -1;
  }
  int seg0 = __shfl_sync(0xffffffffu, seg, 0);
  bool uniform = __all_sync(0xffffffffu, seg == seg0 || seg < 0) && seg0 >= 0;
  if (uniform) {
#pragma unroll
    for (int t = 0; t < 12; ++t) {
      bool is_min = (t < 3) || (t >= 6 && t < 9);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        int u = __shfl_xor_sync(0xffffffffu, v[t], o);
        v[t] = is_min ? min(v[t], u) : max(v[t], u);
      }
    }
  }
  // block level: warps that reduced for the same segment combine in shared memory
  __shared__ int s_v[BUILD_THREADS / 32][12];
  __shared__ int s_seg[BUILD_THREADS / 32];
  int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) s_seg[warp] = uniform ? seg0 : -1;
  if (uniform && lane < 12) s_v[warp][lane] = v[lane];
  __syncthreads();
  int bseg = s_seg[0];
  bool block_uniform = bseg >= 0;
  for (int w = 1; w < BUILD_THREADS / 32; ++w) block_uniform = block_uniform && s_seg[w] == bseg;
  if (block_uniform) {
    if (threadIdx.x < 12) {
      int t = threadIdx.x;
      bool is_min = (t < 3) || (t >= 6 && t < 9);
      int r = s_v[0][t];
      for (int w = 1; w < BUILD_THREADS / 32; ++w) r = is_min ? min(r, s_v[w][t]) : max(r, s_v[w][t]);
      if (is_min) atomicMin(&bounds[12 * bseg + t], r);
      else atomicMax(&bounds[12 * bseg + t], r);
    }
    return;
  }
  if (uniform) {
    if (lane == 0) {
#pragma unroll
      for (int t = 0; t < 12; ++t) {
        bool is_min = (t < 3) || (t >= 6 && t < 9);
        if (is_min) atomicMin(&bounds[12 * seg0 + t], v[t]);
        else atomicMax(&bounds[12 * seg0 + t], v[t]);
      }
    }
  } else if (ok) {
#pragma unroll
    for (int t = 0; t < 12; ++t) {
      bool is_min = (t < 3) || (t >= 6 && t < 9);
      if (is_min) atomicMin(&bounds[12 * seg + t], v[t]);
      else atomicMax(&bounds[12 * seg + t], v[t]);
    }
  }
}

// Sets *bad when any of the 3 * nf face indices lies outside [0, nv).
__global__ void face_range_kernel(int32_t const * __restrict__ F, int64_t count, int64_t nv, int * __restrict__ bad) {
  bool out = false;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
    int32_t f = F[i];
    out |= f < 0 || (int64_t)f >= nv;
  }
  if (__any_sync(0xffffffffu, out) && (threadIdx.x & 31) == 0) atomicOr(bad, 1);
}

__global__ void init_bounds_kernel(int * __restrict__ bounds, int M) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 12 * (int64_t)M) return;
  int t = (int)(i % 12);
  bounds[i] = ((t < 3) || (t >= 6 && t < 9)) ? INT_MAX : INT_MIN;
}

__device__ __forceinline__ uint64_t expand21(uint32_t v) {
  uint64_t x = v & 0x1fffffull;
  x = (x | x << 32) & 0x1f00000000ffffull;
  x = (x | x << 16) & 0x1f0000ff0000ffull;
  x = (x | x << 8) & 0x100f00f00f00f00full;
  x = (x | x << 4) & 0x10c30c30c30c30c3ull;
  x = (x | x << 2) & 0x1249249249249249ull;
  return x;
}

// key = (segment << 3 bpa) | Morton code with bpa bits per axis of the box centre within its segment's centre bounds
__global__ void morton_kernel(float4 const * __restrict__ elo, float4 const * __restrict__ ehi, int64_t n,
                              int64_t const * __restrict__ seg_start, int M, int const * __restrict__ bounds, int bpa,
                              uint64_t * __restrict__ keys, uint32_t * __restrict__ vals) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int seg = M > 1 ? segment_of(seg_start, M, i) : 0;
  float4 l = elo[i], h = ehi[i];
  float c[3] = {0.5f * (h.x + l.x), 0.5f * (h.y + l.y), 0.5f * (h.z + l.z)};
  float cells = (float)(1u << bpa);
  uint32_t q[3];
  // One scale for all axes (the largest extent), so that the implicit split planes are spatial medians of a cube: a
  // flat or elongated segment gets few splits across its thin axes. (Per-axis scaling gave the 2 M-triangle heightfield,
  // 0.3 units thick over 1 x 1, as many splits in z as in x and y, whose children overlap in x and y: 12 % slower rays.)
  float ext = 0.f;
#pragma unroll
  for (int a = 0; a < 3; ++a) ext = fmaxf(ext, ord2f(bounds[12 * seg + 3 + a]) - ord2f(bounds[12 * seg + a]));
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float lo = ord2f(bounds[12 * seg + a]);
    float t = ext > 0.f ? (c[a] - lo) / ext : 0.f;
    t = fminf(fmaxf(t, 0.f), 1.f);
    q[a] = min((uint32_t)(t * cells), (1u << bpa) - 1u);
  }
  uint64_t code = (expand21(q[0]) << 2) | (expand21(q[1]) << 1) | expand21(q[2]);
  keys[i] = ((uint64_t)seg << (3 * bpa)) | code;
  vals[i] = (uint32_t)i;
}

// Common-prefix length of sorted keys i and j inside [a, b), extended by the positions when the keys are equal
// (Karras 2012); -1 outside the segment.
__device__ __forceinline__ int kdelta(uint64_t const * __restrict__ codes, int64_t a, int64_t b, int64_t i, int64_t j) {
  if (j < a || j >= b) return -1;
  uint64_t x = codes[i], y = codes[j];
  if (x == y) return 64 + __clzll((long long)(i ^ j));
  return __clzll((long long)(x ^ y));
}

// Binary radix trees, one per segment. The internal node at sorted position i of segment s lives in slot i - s.
// Child codes: >= 0 an internal slot, < 0 a leaf at sorted position ~code.
__global__ void karras_kernel(uint64_t const * __restrict__ codes, int64_t n, int64_t const * __restrict__ seg_start,
                              int M, int mbits, int * __restrict__ left, int * __restrict__ right,
                              int * __restrict__ first, int * __restrict__ last, int * __restrict__ parent,
                              int * __restrict__ leaf_parent) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int s = M > 1 ? (int)(codes[i] >> mbits) : 0;
  int64_t a = M > 1 ? seg_start[s] : 0, b = M > 1 ? seg_start[s + 1] : n;
  if (i >= b - 1) return;  // a segment of m elements has m - 1 internal nodes, at positions a .. b - 2
  int d = (kdelta(codes, a, b, i, i + 1) - kdelta(codes, a, b, i, i - 1)) >= 0 ? 1 : -1;
  int dmin = kdelta(codes, a, b, i, i - d);
  int64_t lmax = 2;
  while (kdelta(codes, a, b, i, i + lmax * d) > dmin) lmax <<= 1;
  int64_t l = 0;
  for (int64_t t = lmax >> 1; t >= 1; t >>= 1)
    if (kdelta(codes, a, b, i, i + (l + t) * d) > dmin) l += t;
  int64_t j = i + l * d;
  int dnode = kdelta(codes, a, b, i, j);
  int64_t sp = 0, t = l;
  do {
    t = (t + 1) >> 1;
    if (kdelta(codes, a, b, i, i + (sp + t) * d) > dnode) sp += t;
  } while (t > 1);
  int64_t gamma = i + sp * d + (d < 0 ? -1 : 0);
  int64_t lo = i < j ? i : j, hi = i < j ? j : i;
  int slot = (int)(i - s);
  int lc = (lo == gamma) ? ~(int)gamma : (int)(gamma - s);
  int rc = (hi == gamma + 1) ? ~(int)(gamma + 1) : (int)(gamma + 1 - s);
  left[slot] = lc;
  right[slot] = rc;
  first[slot] = (int)lo;
  last[slot] = (int)hi;
  if (lc < 0) leaf_parent[~lc] = slot; else parent[lc] = slot;
  if (rc < 0) leaf_parent[~rc] = slot; else parent[rc] = slot;
}

__device__ __forceinline__ void child_box(int code, float4 const * __restrict__ elo, float4 const * __restrict__ ehi,
                                          uint32_t const * __restrict__ sorted, float4 const * ilo, float4 const * ihi,
                                          float4 & lo, float4 & hi) {
  if (code < 0) {
    uint32_t e = sorted[~code];
    lo = elo[e];
    hi = ehi[e];
  } else {
    lo = __ldcg(ilo + code);
    hi = __ldcg(ihi + code);
  }
}

// Bottom-up refit: the second thread to reach a node merges its two children and continues upwards.
__global__ void refit_kernel(int64_t n, int const * __restrict__ left, int const * __restrict__ right,
                             int const * __restrict__ parent, int const * __restrict__ leaf_parent,
                             float4 const * __restrict__ elo, float4 const * __restrict__ ehi,
                             uint32_t const * __restrict__ sorted, float4 * ilo, float4 * ihi,
                             unsigned * __restrict__ visits) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  int p = leaf_parent[s];
  while (p >= 0) {
    __threadfence();
    unsigned old = atomicAdd(&visits[p], 1u);
    if (old == 0) return;
    float4 al, ah, bl, bh;
    child_box(left[p], elo, ehi, sorted, ilo, ihi, al, ah);
    child_box(right[p], elo, ehi, sorted, ilo, ihi, bl, bh);
    __stcg(ilo + p, make_float4(fminf(al.x, bl.x), fminf(al.y, bl.y), fminf(al.z, bl.z), 0.f));
    __stcg(ihi + p, make_float4(fmaxf(ah.x, bh.x), fmaxf(ah.y, bh.y), fmaxf(ah.z, bh.z), 0.f));
    p = parent[p];
  }
}

struct CollapseArgs {
  int const * left;
  int const * right;
  int const * first;
  int const * last;
  float4 const * elo;
  float4 const * ehi;
  uint32_t const * sorted;
  float4 const * ilo;
  float4 const * ihi;
  int64_t const * seg_start;  // sorted position where each segment starts (nullptr: one segment)
  int M;
  int leaf_size;
};

__device__ __forceinline__ int code_count(CollapseArgs const & a, int code) {
  return code < 0 ? 1 : a.last[code] - a.first[code] + 1;
}
__device__ __forceinline__ int code_first(CollapseArgs const & a, int code) { return code < 0 ? ~code : a.first[code]; }

__device__ __forceinline__ float half_area(float4 lo, float4 hi) {
  float x = hi.x - lo.x, y = hi.y - lo.y, z = hi.z - lo.z;
  return x * y + y * z + z * x;
}

// For each frontier binary node, choose the W binary subtrees that become the children of its wide node: starting from
// the two children, repeatedly open the subtree with the largest surface area among those too big to be a leaf.
// Frontier of the level being collapsed, kept on the device so that several levels run between host synchronisations:
// its size, the wide index of its first node, and the number of levels emitted so far.
struct CollapseLevel {
  int64_t fsize;
  int64_t base;
  int64_t levels;
  int64_t overflow;  // set if a node would have landed past the node bound (never, by the bound's construction)
  int64_t parity;    // which of the two frontier buffers holds the current frontier
};

// The W binary subtrees that become the children of frontier node f's wide node; returns how many are internal
template <int W>
__device__ __forceinline__ int collapse_decide_one(CollapseArgs const & a, int const * __restrict__ frontier, int64_t f,
                                                   int * __restrict__ chosen) {
  int b = frontier[f];
  int codes[W];
  int ne = 2;
  codes[0] = a.left[b];
  codes[1] = a.right[b];
#pragma unroll
  for (int e = 2; e < W; ++e) codes[e] = CHILD_EMPTY;
  while (ne < W) {
    int best = -1;
    float best_sa = -1.f;
    for (int e = 0; e < ne; ++e) {
      int c = codes[e];
      if (c >= 0 && code_count(a, c) > a.leaf_size) {
        float sa = half_area(a.ilo[c], a.ihi[c]);
        if (sa > best_sa) { best_sa = sa; best = e; }
      }
    }
    if (best < 0) break;
    int c = codes[best];
    codes[best] = a.left[c];
    codes[ne++] = a.right[c];
  }
  int nint = 0;
  for (int e = 0; e < W; ++e) {
    chosen[f * W + e] = codes[e];
    if (codes[e] != CHILD_EMPTY && code_count(a, codes[e]) > a.leaf_size) ++nint;
  }
  return nint;
}

template <int W>
__global__ void collapse_decide_kernel(CollapseArgs a, int const * __restrict__ fa, int const * __restrict__ fb,
                                       CollapseLevel const * __restrict__ lv, int64_t bound,
                                       int * __restrict__ chosen, int * __restrict__ num_internal) {
  int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= bound) return;
  int64_t fsize = lv->fsize;
  num_internal[f] = f < fsize ? collapse_decide_one<W>(a, lv->parity ? fb : fa, f, chosen) : 0;  // the scan covers
                                                                                                   // the host's bound
}

// Pad a box outwards by a relative margin of its coordinates' magnitude, so that rounding in element distances and hit
// times can never make an element that lies inside the box look closer than the box.
__device__ __forceinline__ void pad_box(float4 & lo, float4 & hi) {
  float const R = 1.0f / 1048576.0f;  // 2^-20
  float px = (fabsf(lo.x) + fabsf(hi.x)) * R, py = (fabsf(lo.y) + fabsf(hi.y)) * R, pz = (fabsf(lo.z) + fabsf(hi.z)) * R;
  lo.x -= px; lo.y -= py; lo.z -= pz;
  hi.x += px; hi.y += py; hi.z += pz;
}

template <int W> __device__ __forceinline__ void clear_node(WideNode<W> & node) {
#pragma unroll
  for (int e = 0; e < W; ++e) {
    node.lox[e] = node.loy[e] = node.loz[e] = INFINITY;
    node.hix[e] = node.hiy[e] = node.hiz[e] = -INFINITY;
    node.child[e] = CHILD_EMPTY;
  }
#pragma unroll
  for (int e = 0; e < (W == 4 ? 4 : 8); ++e) node.pad[e] = 0;
}

// Writes frontier node f's wide node (level_base + f) and appends its internal children to the next frontier at
// offset `off` (their wide indices next_base + off + k); false if a node would land past the node bound
template <int W>
__device__ __forceinline__ bool collapse_emit_one(CollapseArgs const & a, int const * __restrict__ frontier, int64_t f,
                                                  int const * __restrict__ chosen, int off, int64_t level_base,
                                                  int64_t next_base, int64_t cap, WideNode<W> * __restrict__ nodes,
                                                  int * __restrict__ next_frontier) {
  if (level_base + f >= cap) return false;
  WideNode<W> node;
  clear_node(node);
  int k = 0;
  // leaves store their first element relative to the segment's first sorted position
  int64_t seg_base = 0;
  if (a.M > 1) {
    int64_t pos = a.first[frontier[f]];
    seg_base = a.seg_start[segment_of(a.seg_start, a.M, pos)];
  }
#pragma unroll
  for (int e = 0; e < W; ++e) {
    int code = chosen[f * W + e];
    if (code == CHILD_EMPTY) continue;
    float4 lo, hi;
    child_box(code, a.elo, a.ehi, a.sorted, a.ilo, a.ihi, lo, hi);
    pad_box(lo, hi);
    node.lox[e] = lo.x; node.loy[e] = lo.y; node.loz[e] = lo.z;
    node.hix[e] = hi.x; node.hiy[e] = hi.y; node.hiz[e] = hi.z;
    int cnt = code_count(a, code);
    if (cnt <= a.leaf_size) {
      node.child[e] = encode_leaf((int)(code_first(a, code) - seg_base), cnt);
    } else {
      if (next_base + off + k >= cap) return false;
      node.child[e] = (int)(next_base + off + k);
      next_frontier[off + k] = code;
      ++k;
    }
  }
  nodes[level_base + f] = node;
  return true;
}

template <int W>
__global__ void collapse_emit_kernel(CollapseArgs a, int * __restrict__ fa, int * __restrict__ fb,
                                     CollapseLevel * __restrict__ lv, int64_t bound, int const * __restrict__ chosen,
                                     int const * __restrict__ offsets, int64_t cap, WideNode<W> * __restrict__ nodes) {
  int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t fsize = lv->fsize;
  if (f >= fsize || f >= bound) return;
  int64_t level_base = lv->base;
  bool par = lv->parity != 0;
  if (!collapse_emit_one<W>(a, par ? fb : fa, f, chosen, offsets[f], level_base, level_base + fsize, cap, nodes,
                            par ? fa : fb))
    lv->overflow = 1;
}

// Levels whose frontier fits in one block, one after another in one launch (the top of the tree and its tail): thread f
// decides and emits frontier node f, a block scan places the internal children. Returns when the frontier is empty or
// outgrows the block.
constexpr int COLLAPSE_BLOCK = 1024;

template <int W>
__global__ void __launch_bounds__(COLLAPSE_BLOCK)
collapse_small_levels_kernel(CollapseArgs a, int * __restrict__ fa, int * __restrict__ fb,
                             CollapseLevel * __restrict__ lv, int * __restrict__ chosen, int64_t cap,
                             WideNode<W> * __restrict__ nodes) {
  __shared__ int64_t s_fsize, s_base, s_parity;
  __shared__ int s_bad;
  int t = threadIdx.x;
  if (t == 0) {
    s_fsize = lv->fsize;
    s_base = lv->base;
    s_parity = lv->parity;
    s_bad = 0;
  }
  __syncthreads();
  int64_t levels = 0;
  while (true) {
    int64_t fsize = s_fsize;
    if (fsize <= 0 || fsize > COLLAPSE_BLOCK || s_bad) break;
    bool par = s_parity != 0;
    int * cur = par ? fb : fa;
    int * nxt = par ? fa : fb;
    int nint = t < fsize ? collapse_decide_one<W>(a, cur, t, chosen) : 0;
    int total = 0;
    int off = block_exclusive_scan<int>(nint, total);
    if (t < fsize && !collapse_emit_one<W>(a, cur, t, chosen, off, s_base, s_base + fsize, cap, nodes, nxt))
      s_bad = 1;
    __syncthreads();
    if (t == 0) {
      s_base += fsize;
      s_fsize = total;
      s_parity = !par;
    }
    ++levels;
    __syncthreads();
  }
  if (t == 0) {
    lv->fsize = s_bad ? 0 : s_fsize;
    lv->base = s_base;
    lv->parity = s_parity;
    lv->levels += levels;
    if (s_bad) lv->overflow = 1;
  }
}

// Moves the device state to the next level: the emitted children form the next frontier
__global__ void collapse_advance_kernel(CollapseLevel * __restrict__ lv, int64_t bound, int const * __restrict__ offsets,
                                        int const * __restrict__ num_internal) {
  int64_t fsize = lv->fsize;
  if (fsize <= 0) return;
  if (fsize > bound) {  // the host's bound did not hold: stop, reported as an overflow
    lv->overflow = 1;
    lv->fsize = 0;
    return;
  }
  lv->base += fsize;
  lv->fsize = (int64_t)offsets[fsize - 1] + num_internal[fsize - 1];
  lv->levels += 1;
  lv->parity = !lv->parity;
}

// Segment roots: big segments (more elements than a leaf) become level-0 frontier entries; small non-empty segments get
// a single-leaf root node. Small roots take wide indices [0, num_small), big roots [num_small, num_small + num_big).
__global__ void segment_flags_kernel(int64_t const * __restrict__ seg_start, int M, int64_t n, int leaf_size,
                                     int * __restrict__ is_small, int * __restrict__ is_big) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= M) return;
  int64_t a = seg_start ? seg_start[s] : 0, b = seg_start ? seg_start[s + 1] : n;
  int64_t cnt = b - a;
  is_small[s] = (cnt >= 1 && cnt <= leaf_size) ? 1 : 0;
  is_big[s] = cnt > leaf_size ? 1 : 0;
}

template <int W>
__global__ void segment_roots_kernel(CollapseArgs a, int64_t n, int const * __restrict__ is_small,
                                     int const * __restrict__ small_rank, int const * __restrict__ is_big,
                                     int const * __restrict__ big_rank, int num_small, int const * __restrict__ bounds,
                                     WideNode<W> * __restrict__ nodes, int * __restrict__ frontier,
                                     int * __restrict__ seg_root) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= a.M) return;
  int64_t sa = a.seg_start ? a.seg_start[s] : 0, sb = a.seg_start ? a.seg_start[s + 1] : n;
  if (is_big[s]) {
    // the Karras root of the segment is the internal node at its first position, slot sa - s
    frontier[big_rank[s]] = (int)(sa - s);
    seg_root[s] = num_small + big_rank[s];
  } else if (is_small[s]) {
    WideNode<W> node;
    clear_node(node);
    float4 lo = make_float4(ord2f(bounds[12 * s + 6]), ord2f(bounds[12 * s + 7]), ord2f(bounds[12 * s + 8]), 0.f);
    float4 hi = make_float4(ord2f(bounds[12 * s + 9]), ord2f(bounds[12 * s + 10]), ord2f(bounds[12 * s + 11]), 0.f);
    pad_box(lo, hi);
    node.lox[0] = lo.x; node.loy[0] = lo.y; node.loz[0] = lo.z;
    node.hix[0] = hi.x; node.hiy[0] = hi.y; node.hiz[0] = hi.z;
    node.child[0] = encode_leaf(0, (int)(sb - sa));
    nodes[small_rank[s]] = node;
    seg_root[s] = small_rank[s];
  } else {
    seg_root[s] = -1;  // empty segment
  }
}

__global__ void count_big_kernel(int const * __restrict__ first, int const * __restrict__ last, int64_t m, int leaf_size,
                                 unsigned long long * __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool big = i < m && (last[i] - first[i] + 1) > leaf_size;
  unsigned b = __ballot_sync(0xffffffffu, big);
  if ((threadIdx.x & 31) == 0 && b) atomicAdd(out, (unsigned long long)__popc(b));
}

// Element records in sorted order; the stored index is the element's index within its segment.
__global__ void mesh_records_kernel(float const * __restrict__ V, int32_t const * __restrict__ F, int64_t n,
                                    int64_t const * __restrict__ seg_start, int M, uint32_t const * __restrict__ sorted,
                                    float4 * __restrict__ cp_rec, float4 * __restrict__ ray_rec,
                                    int32_t * __restrict__ leaf_to_elem) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  int64_t ge = (int64_t)sorted[s];
  int e = (int)(M > 1 ? ge - seg_start[segment_of(seg_start, M, ge)] : ge);
  leaf_to_elem[s] = e;
  V3 v0 = load_v3(V + 3 * (int64_t)F[3 * ge]);
  V3 v1 = load_v3(V + 3 * (int64_t)F[3 * ge + 1]);
  V3 v2 = load_v3(V + 3 * (int64_t)F[3 * ge + 2]);
  if (cp_rec) {
    TriPlane pl = tri_plane(v0, v1, v2);
    V3 d0, d1, d2;
    float l0, l1, l2;
    edge_dir(v0, v1, d0, l0);
    edge_dir(v1, v2, d1, l1);
    edge_dir(v2, v0, d2, l2);
    float4 * r = cp_rec + s * CP_REC_F4;
    r[0] = make_float4(v0.x, v0.y, v0.z, pl.dist);
    r[1] = make_float4(v1.x, v1.y, v1.z, l0);
    r[2] = make_float4(v2.x, v2.y, v2.z, l1);
    r[3] = make_float4(pl.normal.x, pl.normal.y, pl.normal.z, __int_as_float(pl.axis));
    r[4] = make_float4(d0.x, d0.y, d0.z, l2);
    r[5] = make_float4(d1.x, d1.y, d1.z, __int_as_float(e));
    r[6] = make_float4(d2.x, d2.y, d2.z, pl.area);
    r[7] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  if (ray_rec) {
    V3 e01 = v1 - v0, e02 = v2 - v0;
    float4 * r = ray_rec + s * RAY_REC_F4;
    r[0] = make_float4(v0.x, v0.y, v0.z, __int_as_float(e));
    r[1] = make_float4(e01.x, e01.y, e01.z, 0.f);
    r[2] = make_float4(e02.x, e02.y, e02.z, 0.f);
  }
}

__global__ void point_records_kernel(float const * __restrict__ P, int64_t n, int64_t const * __restrict__ seg_start,
                                     int M, uint32_t const * __restrict__ sorted, float4 * __restrict__ pt_rec,
                                     int32_t * __restrict__ leaf_to_elem) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  int64_t ge = (int64_t)sorted[s];
  int e = (int)(M > 1 ? ge - seg_start[segment_of(seg_start, M, ge)] : ge);
  leaf_to_elem[s] = e;
  V3 p = load_v3(P + 3 * ge);
  pt_rec[s] = make_float4(p.x, p.y, p.z, __int_as_float(e));
}

// Oriented slab of every child slot (slab_normal / slab_lower_bound in traverse_ops.cuh): n = the area-weighted mean of
// the slot's triangle normals (triangles with a non-finite normal or area left out; +z if the mean vanishes), encoded
// and decoded as the searches decode it, and the range of n . v over the slot's vertices, accumulated in double
// (products of floats are exact in double) and rounded outwards to float. One block per slot, slots taken in a
// grid-stride loop; slots with no elements get an empty slab.
constexpr int SLAB_THREADS = 128;

__global__ void __launch_bounds__(SLAB_THREADS)
slab_kernel(int2 const * __restrict__ ranges, int64_t slots, float4 const * __restrict__ rec, float4 * __restrict__ out) {
  __shared__ float s_n[3][SLAB_THREADS / 32];
  __shared__ double s_d[2][SLAB_THREADS / 32];
  __shared__ float4 s_enc;
  int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  for (int64_t slot = blockIdx.x; slot < slots; slot += gridDim.x) {
    int2 r = ranges[slot];
    if (r.y <= 0) {
      if (t == 0) out[slot] = make_float4(0.f, 0.f, INFINITY, -INFINITY);
      continue;
    }
    int64_t k0 = r.x, k1 = (int64_t)r.x + r.y;
    float nx = 0.f, ny = 0.f, nz = 0.f;
    for (int64_t k = k0 + t; k < k1; k += SLAB_THREADS) {
      float4 nn = __ldg(rec + k * CP_REC_F4 + 3);
      float area = __ldg(rec + k * CP_REC_F4 + 6).w;
      if (isfinite(nn.x) && isfinite(nn.y) && isfinite(nn.z) && isfinite(area)) {
        nx += nn.x * area;
        ny += nn.y * area;
        nz += nn.z * area;
      }
    }
    for (int o = 16; o; o >>= 1) {
      nx += __shfl_xor_sync(0xffffffffu, nx, o);
      ny += __shfl_xor_sync(0xffffffffu, ny, o);
      nz += __shfl_xor_sync(0xffffffffu, nz, o);
    }
    if (lane == 0) s_n[0][warp] = nx, s_n[1][warp] = ny, s_n[2][warp] = nz;
    __syncthreads();
    if (t == 0) {
      float x = 0.f, y = 0.f, z = 0.f;
      for (int w = 0; w < SLAB_THREADS / 32; ++w) x += s_n[0][w], y += s_n[1][w], z += s_n[2][w];
      float l = sqrtf(x * x + y * y + z * z);
      if (!(l > 0.f) || !isfinite(l)) x = 0.f, y = 0.f, z = 1.f, l = 1.f;
      s_enc = slab_encode(V3{x / l, y / l, z / l});
    }
    __syncthreads();
    float4 enc = s_enc;
    V3 n = slab_normal(enc);
    double lo = INFINITY, hi = -INFINITY;
    for (int64_t k = k0 + t; k < k1; k += SLAB_THREADS) {
#pragma unroll
      for (int v = 0; v < 3; ++v) {
        float4 q = __ldg(rec + k * CP_REC_F4 + v);
        double d = (double)n.x * (double)q.x + (double)n.y * (double)q.y + (double)n.z * (double)q.z;
        lo = fmin(lo, d);
        hi = fmax(hi, d);
      }
    }
    for (int o = 16; o; o >>= 1) {
      lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
      hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if (lane == 0) s_d[0][warp] = lo, s_d[1][warp] = hi;
    __syncthreads();
    if (t == 0) {
      for (int w = 1; w < SLAB_THREADS / 32; ++w) lo = fmin(lo, s_d[0][w]), hi = fmax(hi, s_d[1][w]);
      enc.z = __double2float_rd(lo);
      enc.w = __double2float_ru(hi);
      out[slot] = enc;
    }
    __syncthreads();
  }
}

constexpr int COLLAPSE_LEVELS_PER_SYNC = 6;

template <int W>
void collapse(thea_bvh * b, CollapseArgs const & a, int64_t n, int const * d_bounds, cudaStream_t stream) {
  int M = a.M;
  // segment roots
  Scratch is_small((size_t)M * sizeof(int), stream), is_big((size_t)M * sizeof(int), stream);
  Scratch small_rank((size_t)M * sizeof(int), stream), big_rank((size_t)M * sizeof(int), stream);
  THEA_LAUNCH(segment_flags_kernel, (unsigned)ceil_div(M, BUILD_THREADS), BUILD_THREADS, 0, stream, a.seg_start, M, n,
              a.leaf_size, is_small.as<int>(), is_big.as<int>());
  exclusive_scan<int>(is_small.as<int>(), small_rank.as<int>(), M, stream);
  exclusive_scan<int>(is_big.as<int>(), big_rank.as<int>(), M, stream);
  int tails[4];
  THEA_CUDA_CHECK(cudaMemcpyAsync(&tails[0], small_rank.as<int>() + M - 1, sizeof(int), cudaMemcpyDeviceToHost, stream));
  THEA_CUDA_CHECK(cudaMemcpyAsync(&tails[1], is_small.as<int>() + M - 1, sizeof(int), cudaMemcpyDeviceToHost, stream));
  THEA_CUDA_CHECK(cudaMemcpyAsync(&tails[2], big_rank.as<int>() + M - 1, sizeof(int), cudaMemcpyDeviceToHost, stream));
  THEA_CUDA_CHECK(cudaMemcpyAsync(&tails[3], is_big.as<int>() + M - 1, sizeof(int), cudaMemcpyDeviceToHost, stream));
  // every other wide node corresponds to a distinct binary node with more elements than a leaf holds
  int64_t m = n - M;  // binary internal nodes in the forest (segments are non-empty)
  Scratch cnt(sizeof(unsigned long long), stream);
  THEA_CUDA_CHECK(cudaMemsetAsync(cnt.ptr, 0, cnt.bytes, stream));
  if (m > 0)
    THEA_LAUNCH(count_big_kernel, (unsigned)ceil_div(m, BUILD_THREADS), BUILD_THREADS, 0, stream, a.first, a.last, m,
                a.leaf_size, cnt.as<unsigned long long>());
  unsigned long long nbig = 0;
  THEA_CUDA_CHECK(cudaMemcpyAsync(&nbig, cnt.ptr, sizeof(nbig), cudaMemcpyDeviceToHost, stream));
  THEA_CUDA_CHECK(cudaStreamSynchronize(stream));
  int num_small = tails[0] + tails[1], num_big = tails[2] + tails[3];
  int64_t cap = (int64_t)num_small + (int64_t)std::max<unsigned long long>(nbig, 1);

  WideNode<W> * nodes = nullptr;
  THEA_CUDA_CHECK(thea_malloc_async((void **)&nodes, (size_t)cap * sizeof(WideNode<W>), stream));
  THEA_CUDA_CHECK(thea_malloc_async((void **)&b->seg_root, (size_t)M * sizeof(int32_t), stream));
  Scratch fa((size_t)std::max<int64_t>(cap, 1) * sizeof(int), stream), fb((size_t)std::max<int64_t>(cap, 1) * sizeof(int), stream);
  THEA_LAUNCH((segment_roots_kernel<W>), (unsigned)ceil_div(M, BUILD_THREADS), BUILD_THREADS, 0, stream, a, n,
              is_small.as<int>(), small_rank.as<int>(), is_big.as<int>(), big_rank.as<int>(), num_small, d_bounds,
              nodes, fa.as<int>(), b->seg_root);
  Scratch chosen((size_t)std::max<int64_t>(cap, 1) * W * sizeof(int), stream);
  Scratch nint((size_t)std::max<int64_t>(cap, 1) * sizeof(int), stream);
  Scratch offs((size_t)std::max<int64_t>(cap, 1) * sizeof(int), stream);
  int depth = num_small > 0 ? 1 : 0;
  // Levels whose frontier fits in one block run in one launch (collapse_small_levels_kernel); larger ones run
  // COLLAPSE_LEVELS_PER_SYNC at a time, a few launches each, on the device state, with the host bounding each frontier
  // (a frontier node has at most W internal children, and no level holds more than the nbig wide internal nodes) to
  // size the launches and the scan. Levels past the last one find an empty frontier and do nothing.
  CollapseLevel h{num_big, num_small, 0, 0, 0};
  Scratch lv(sizeof(CollapseLevel), stream);
  THEA_CUDA_CHECK(cudaMemcpyAsync(lv.ptr, &h, sizeof(h), cudaMemcpyHostToDevice, stream));
  int64_t limit = std::max<int64_t>((int64_t)nbig, 1);
  while (h.fsize > 0) {
    int64_t bound = h.fsize;
    if (bound <= COLLAPSE_BLOCK) {
      THEA_LAUNCH(collapse_small_levels_kernel<W>, 1, COLLAPSE_BLOCK, 0, stream, a, fa.as<int>(), fb.as<int>(),
                  lv.as<CollapseLevel>(), chosen.as<int>(), cap, nodes);
      bound = 0;  // read the state back before choosing the next step
    }
    for (int l = 0; l < COLLAPSE_LEVELS_PER_SYNC && bound > 0; ++l) {
      unsigned grid = (unsigned)ceil_div(bound, BUILD_THREADS);
      THEA_LAUNCH(collapse_decide_kernel<W>, grid, BUILD_THREADS, 0, stream, a, fa.as<int>(), fb.as<int>(),
                  lv.as<CollapseLevel>(), bound, chosen.as<int>(), nint.as<int>());
      exclusive_scan<int>(nint.as<int>(), offs.as<int>(), bound, stream);
      THEA_LAUNCH(collapse_emit_kernel<W>, grid, BUILD_THREADS, 0, stream, a, fa.as<int>(), fb.as<int>(),
                  lv.as<CollapseLevel>(), bound, chosen.as<int>(), offs.as<int>(), cap, nodes);
      THEA_LAUNCH(collapse_advance_kernel, 1, 1, 0, stream, lv.as<CollapseLevel>(), bound, offs.as<int>(),
                  nint.as<int>());
      bound = std::min<int64_t>(bound * W, limit);
    }
    THEA_CUDA_CHECK(cudaMemcpyAsync(&h, lv.ptr, sizeof(h), cudaMemcpyDeviceToHost, stream));
    THEA_CUDA_CHECK(cudaStreamSynchronize(stream));
    THEA_REQUIRE(!h.overflow, "BVH collapse exceeded its node bound");
  }
  b->nodes = nodes;
  b->num_nodes = h.base;
  b->depth = std::max<int>(depth, (int)h.levels);
}

}  // namespace

thea_bvh * build_forest(bool is_mesh, float const * V, int64_t nv, int32_t const * F, int64_t n_elems,
                        int64_t const * seg_start_host, int M, thea_build_config const & cfg, cudaStream_t stream) {
  int64_t n = is_mesh ? n_elems : nv;
  THEA_REQUIRE(M >= 1, "build: at least one segment is required");
  THEA_REQUIRE(n >= 1, "build: at least one element is required");
  THEA_REQUIRE(n < (int64_t(1) << 31) - 1, "build: at most 2^31 - 2 elements per forest");
  int width = cfg.width == 0 ? 4 : cfg.width;
  THEA_REQUIRE(width == 4 || width == 8, "build: width must be 4 or 8");
  int leaf = cfg.max_leaf_size == 0 ? (is_mesh ? 2 : 1) : cfg.max_leaf_size;
  THEA_REQUIRE(leaf >= 1 && leaf <= MAX_LEAF_SIZE, "build: max_leaf_size must be in 1..16");
  uint32_t layouts = is_mesh ? (cfg.layouts == 0 ? (THEA_LAYOUT_CLOSEST | THEA_LAYOUT_RAY) : cfg.layouts) : 0u;
  THEA_REQUIRE((layouts & ~3u) == 0, "build: unknown layout bits");
  std::vector<int64_t> starts;
  if (M > 1) {
    THEA_REQUIRE(seg_start_host, "build: segment starts are required for more than one segment");
    starts.assign(seg_start_host, seg_start_host + M + 1);
    THEA_REQUIRE(starts[0] == 0 && starts[M] == n, "build: segment starts must run from 0 to the element count");
    for (int s = 0; s < M; ++s) {
      THEA_REQUIRE(starts[s + 1] > starts[s], "build: every segment must hold at least one element");
      THEA_REQUIRE(starts[s + 1] - starts[s] < (int64_t(1) << 27), "build: at most 2^27 - 1 elements per segment");
    }
  } else {
    THEA_REQUIRE(n < (int64_t(1) << 27), "build: at most 2^27 - 1 elements per BVH");
    starts = {0, n};
  }

  if (is_mesh) check_face_indices(F, n_elems, nv, "build", stream);

  thea_bvh * b = new thea_bvh;
  try {
    THEA_CUDA_CHECK(cudaGetDevice(&b->device));
    b->is_mesh = is_mesh ? 1 : 0;
    b->width = width;
    b->leaf_size = leaf;
    b->layouts = layouts;
    b->query_order = cfg.query_order;
    b->n = n;
    b->num_segments = M;
    b->seg_start_host = starts;

    THEA_CUDA_CHECK(thea_malloc_async((void **)&b->seg_start, (size_t)(M + 1) * sizeof(int64_t), stream));
    THEA_CUDA_CHECK(cudaMemcpyAsync(b->seg_start, starts.data(), (size_t)(M + 1) * sizeof(int64_t),
                                    cudaMemcpyHostToDevice, stream));
    int64_t const * seg = b->seg_start;

    Scratch elo((size_t)n * sizeof(float4), stream), ehi((size_t)n * sizeof(float4), stream);
    Scratch bounds((size_t)12 * M * sizeof(int), stream);
    THEA_LAUNCH(init_bounds_kernel, (unsigned)ceil_div(12 * (int64_t)M, BUILD_THREADS), BUILD_THREADS, 0, stream,
                bounds.as<int>(), M);
    unsigned grid = (unsigned)ceil_div(n, BUILD_THREADS);
    THEA_LAUNCH(elem_box_kernel, grid, BUILD_THREADS, 0, stream, V, F, n, is_mesh ? 1 : 0, seg, M, elo.as<float4>(),
                ehi.as<float4>(), bounds.as<int>());

    int segbits = 0;
    while ((int64_t(1) << segbits) < M) ++segbits;
    int bpa = std::min(21, (63 - segbits) / 3);
    int mbits = 3 * bpa;
    Scratch keys((size_t)n * sizeof(uint64_t), stream), vals((size_t)n * sizeof(uint32_t), stream);
    THEA_LAUNCH(morton_kernel, grid, BUILD_THREADS, 0, stream, elo.as<float4>(), ehi.as<float4>(), n, seg, M,
                bounds.as<int>(), bpa, keys.as<uint64_t>(), vals.as<uint32_t>());
    radix_sort_pairs(keys.as<uint64_t>(), vals.as<uint32_t>(), n, mbits + segbits, stream);

    int64_t m = n - M;  // binary internal nodes
    size_t mm = (size_t)std::max<int64_t>(m, 1);
    Scratch left(mm * sizeof(int), stream), right(mm * sizeof(int), stream);
    Scratch first(mm * sizeof(int), stream), last(mm * sizeof(int), stream);
    Scratch parent(mm * sizeof(int), stream), leaf_parent((size_t)n * sizeof(int), stream);
    Scratch ilo(mm * sizeof(float4), stream), ihi(mm * sizeof(float4), stream);
    Scratch visits(mm * sizeof(unsigned), stream);
    if (m >= 1) {
      THEA_CUDA_CHECK(cudaMemsetAsync(parent.ptr, 0xff, (size_t)m * sizeof(int), stream));
      THEA_CUDA_CHECK(cudaMemsetAsync(leaf_parent.ptr, 0xff, (size_t)n * sizeof(int), stream));
      THEA_CUDA_CHECK(cudaMemsetAsync(visits.ptr, 0, (size_t)m * sizeof(unsigned), stream));
      THEA_LAUNCH(karras_kernel, grid, BUILD_THREADS, 0, stream, keys.as<uint64_t>(), n, seg, M, mbits,
                  left.as<int>(), right.as<int>(), first.as<int>(), last.as<int>(), parent.as<int>(),
                  leaf_parent.as<int>());
      THEA_LAUNCH(refit_kernel, grid, BUILD_THREADS, 0, stream, n, left.as<int>(), right.as<int>(), parent.as<int>(),
                  leaf_parent.as<int>(), elo.as<float4>(), ehi.as<float4>(), vals.as<uint32_t>(), ilo.as<float4>(),
                  ihi.as<float4>(), visits.as<unsigned>());
    }
    CollapseArgs a{left.as<int>(), right.as<int>(), first.as<int>(), last.as<int>(), elo.as<float4>(),
                   ehi.as<float4>(), vals.as<uint32_t>(), ilo.as<float4>(), ihi.as<float4>(),
                   M > 1 ? seg : nullptr, M, leaf};
    if (width == 4) collapse<4>(b, a, n, bounds.as<int>(), stream);
    else collapse<8>(b, a, n, bounds.as<int>(), stream);
    int64_t node_bytes = b->num_nodes * (width == 4 ? (int64_t)sizeof(WideNode<4>) : (int64_t)sizeof(WideNode<8>));

    int need = b->depth * (width - 1) + 1;
    if (need > (width == 4 ? 256 : 512))
      throw Error(THEA_ERR_NOT_SUPPORTED, "build: tree too deep for the traversal stack (depth " +
                                              std::to_string(b->depth) + ")");
    THEA_CUDA_CHECK(thea_malloc_async((void **)&b->err, sizeof(unsigned), stream));
    THEA_CUDA_CHECK(cudaMemsetAsync(b->err, 0, sizeof(unsigned), stream));
    THEA_CUDA_CHECK(thea_malloc_host(&b->err_host, sizeof(unsigned)));
    *b->err_host = 0;
    THEA_CUDA_CHECK(thea_malloc_async((void **)&b->leaf_to_elem, (size_t)n * sizeof(int32_t), stream));
    int64_t rec_bytes = n * (int64_t)sizeof(int32_t);
    if (is_mesh) {
      if (layouts & THEA_LAYOUT_CLOSEST) {
        THEA_CUDA_CHECK(thea_malloc_async((void **)&b->cp_rec, (size_t)n * CP_REC_F4 * sizeof(float4), stream));
        rec_bytes += n * CP_REC_F4 * (int64_t)sizeof(float4);
      }
      if (layouts & THEA_LAYOUT_RAY) {
        THEA_CUDA_CHECK(thea_malloc_async((void **)&b->ray_rec, (size_t)n * RAY_REC_F4 * sizeof(float4), stream));
        rec_bytes += n * RAY_REC_F4 * (int64_t)sizeof(float4);
      }
      THEA_LAUNCH(mesh_records_kernel, grid, BUILD_THREADS, 0, stream, V, F, n, seg, M, vals.as<uint32_t>(),
                  b->cp_rec, b->ray_rec, b->leaf_to_elem);
    } else {
      THEA_CUDA_CHECK(thea_malloc_async((void **)&b->pt_rec, (size_t)n * sizeof(float4), stream));
      rec_bytes += n * (int64_t)sizeof(float4);
      THEA_LAUNCH(point_records_kernel, grid, BUILD_THREADS, 0, stream, V, n, seg, M, vals.as<uint32_t>(), b->pt_rec,
                  b->leaf_to_elem);
    }
    std::vector<int> hb((size_t)12 * M);
    THEA_CUDA_CHECK(cudaMemcpyAsync(hb.data(), bounds.ptr, hb.size() * sizeof(int), cudaMemcpyDeviceToHost, stream));
    THEA_CUDA_CHECK(cudaStreamSynchronize(stream));
    b->seg_lo.resize((size_t)3 * M);
    b->seg_hi.resize((size_t)3 * M);
    for (int s = 0; s < M; ++s)
      for (int t = 0; t < 3; ++t) {
        b->seg_lo[3 * s + t] = ord2f(hb[12 * s + 6 + t]);
        b->seg_hi[3 * s + t] = ord2f(hb[12 * s + 9 + t]);
      }
    for (int t = 0; t < 3; ++t) {
      b->lo[t] = b->seg_lo[t];
      b->hi[t] = b->seg_hi[t];
      for (int s = 1; s < M; ++s) {
        b->lo[t] = std::min(b->lo[t], b->seg_lo[3 * s + t]);
        b->hi[t] = std::max(b->hi[t], b->seg_hi[3 * s + t]);
      }
    }
    b->device_bytes = node_bytes + rec_bytes;
    init_segment_roots(b, stream);
    init_slabs(b, stream);
    if (b->slabs) b->device_bytes += b->num_nodes * width * (int64_t)sizeof(float4);
    return b;
  } catch (...) {
    cudaStreamSynchronize(stream);
    destroy_bvh(b);
    throw;
  }
}

// Element range [first, end) of every node's subtree, from its children's: leaves carry their run, internal children
// follow their parent in the node array (the collapse emits level by level). One pass settles every node whose
// children are settled; a node array that breaks those rules (an image written by another build) sets `bad`.
template <int W>
__global__ void subtree_range_kernel(WideNode<W> const * __restrict__ nodes, int64_t num_nodes, int64_t n,
                                     int2 * __restrict__ range, int * __restrict__ changed, int * __restrict__ bad) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < num_nodes; i += (int64_t)gridDim.x * blockDim.x) {
    if (range[i].y >= 0) continue;
    int lo = INT_MAX, hi = -1;
    bool ready = true;
#pragma unroll
    for (int c = 0; c < W; ++c) {
      int code = nodes[i].child[c];
      if (code == CHILD_EMPTY) continue;
      if (code < 0) {
        int first, count;
        decode_leaf(code, first, count);
        if (first < 0 || count <= 0 || (int64_t)first + count > n) {
          atomicOr(bad, 1);
          ready = false;
          break;
        }
        lo = min(lo, first);
        hi = max(hi, first + count);
      } else {
        if ((int64_t)code >= num_nodes || (int64_t)code <= i) {
          atomicOr(bad, 1);
          ready = false;
          break;
        }
        int2 r = range[code];
        if (r.y < 0) {
          ready = false;
          continue;
        }
        lo = min(lo, r.x);
        hi = max(hi, r.y);
      }
    }
    if (!ready) continue;
    range[i] = hi >= 0 ? make_int2(lo, hi) : make_int2(0, 0);
    *changed = 1;
  }
}

// Run of sorted element positions (first, count) under each child slot
template <int W>
__global__ void slot_range_kernel(WideNode<W> const * __restrict__ nodes, int64_t num_nodes,
                                  int2 const * __restrict__ range, int2 * __restrict__ slot) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < num_nodes * W;
       k += (int64_t)gridDim.x * blockDim.x) {
    int code = nodes[k / W].child[k % W];
    int2 r = make_int2(0, 0);
    if (code != CHILD_EMPTY && code < 0) {
      int first, count;
      decode_leaf(code, first, count);
      r = make_int2(first, count);
    } else if (code >= 0) {
      int2 sub = range[code];
      r = make_int2(sub.x, sub.y - sub.x);
    }
    slot[k] = r;
  }
}

template <int W>
bool slot_ranges(thea_bvh const * b, Scratch & slots, cudaStream_t stream) {
  WideNode<W> const * nodes = (WideNode<W> const *)b->nodes;
  int64_t nn = b->num_nodes;
  Scratch range((size_t)nn * sizeof(int2), stream), flags(2 * sizeof(int), stream);
  THEA_CUDA_CHECK(cudaMemsetAsync(range.ptr, 0xff, range.bytes, stream));
  THEA_CUDA_CHECK(cudaMemsetAsync(flags.ptr, 0, flags.bytes, stream));
  unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(nn, BUILD_THREADS), 152 * 8));
  // every pass settles at least the deepest unsettled level; a pass that settles nothing ends the loop, and any node
  // still unsettled then (or after the pass limit) means the array is not a tree of this build's layout
  // Passes run four at a time between reads of the flags (a pass after the one that settled the last node changes
  // nothing, so the extra passes are no-ops); the flags are those of the group's last pass, `bad` accumulates.
  bool settled = false;
  int limit = 2 * b->depth + 4;
  int2 root = make_int2(-1, -1);
  for (int pass = 0; pass < limit && !settled;) {
    for (int k = 0; k < 4 && pass < limit; ++k, ++pass) {
      THEA_CUDA_CHECK(cudaMemsetAsync(flags.ptr, 0, sizeof(int), stream));
      THEA_LAUNCH(subtree_range_kernel<W>, grid, BUILD_THREADS, 0, stream, nodes, nn, b->n, range.as<int2>(),
                  flags.as<int>(), flags.as<int>() + 1);
    }
    int h[2];
    THEA_CUDA_CHECK(cudaMemcpyAsync(h, flags.ptr, sizeof(h), cudaMemcpyDeviceToHost, stream));
    THEA_CUDA_CHECK(cudaMemcpyAsync(&root, range.ptr, sizeof(root), cudaMemcpyDeviceToHost, stream));
    THEA_CUDA_CHECK(cudaStreamSynchronize(stream));
    if (h[1]) return false;
    settled = !h[0];
  }
  if (!settled) return false;
  // the root (node 0) must cover every element once settled
  if (root.x != 0 || (int64_t)root.y != b->n) return false;
  slots = Scratch((size_t)nn * W * sizeof(int2), stream);
  unsigned sgrid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(nn * W, BUILD_THREADS), 152 * 8));
  THEA_LAUNCH(slot_range_kernel<W>, sgrid, BUILD_THREADS, 0, stream, nodes, nn, range.as<int2>(), slots.as<int2>());
  return true;
}

// Oriented slabs go with single-mesh BVHs that have the closest layout: they shorten the longest searches of the
// one-query-per-thread kernels (small batches, serving), whose warps wait for their slowest lane. The persistent
// batched kernels, which refill a lane as soon as its query ends, ran faster with boxes alone, so forests have none.
void init_slabs(thea_bvh * b, cudaStream_t stream) {
  if (!b->is_mesh || b->num_segments != 1 || !b->cp_rec || b->slabs) return;
  Scratch slots;
  bool ok = b->width == 4 ? slot_ranges<4>(b, slots, stream) : slot_ranges<8>(b, slots, stream);
  if (!ok) return;  // searches use boxes alone
  int64_t n_slots = b->num_nodes * b->width;
  THEA_CUDA_CHECK(thea_malloc_async((void **)&b->slabs, (size_t)n_slots * sizeof(float4), stream));
  unsigned grid = (unsigned)std::min<int64_t>(n_slots, (int64_t)sm_count() * 16);
  THEA_LAUNCH(slab_kernel, grid, SLAB_THREADS, 0, stream, slots.as<int2>(), n_slots, b->cp_rec, b->slabs);
  THEA_CUDA_CHECK(cudaStreamSynchronize(stream));
}

void init_segment_roots(thea_bvh * b, cudaStream_t stream) {
  int M = b->num_segments;
  std::vector<RootCut> h((size_t)M);
  for (int s = 0; s < M; ++s) h[(size_t)s] = root_cut_of(&b->seg_lo[3 * (size_t)s], &b->seg_hi[3 * (size_t)s], nullptr);
  if (b->seg_roots) cudaFree(b->seg_roots);
  b->seg_roots = nullptr;
  THEA_CUDA_CHECK(thea_malloc(&b->seg_roots, (size_t)M * sizeof(RootCut)));
  THEA_CUDA_CHECK(cudaMemcpyAsync(b->seg_roots, h.data(), (size_t)M * sizeof(RootCut), cudaMemcpyHostToDevice, stream));
  THEA_CUDA_CHECK(cudaStreamSynchronize(stream));
}

void check_face_indices(int32_t const * F, int64_t nf, int64_t nv, char const * what, cudaStream_t stream) {
  if (nf <= 0) return;
  Scratch bad(sizeof(int), stream);
  THEA_CUDA_CHECK(cudaMemsetAsync(bad.ptr, 0, sizeof(int), stream));
  int64_t count = 3 * nf;
  unsigned grid = (unsigned)std::min<int64_t>(ceil_div(count, BUILD_THREADS), 152 * 8);
  THEA_LAUNCH(face_range_kernel, grid, BUILD_THREADS, 0, stream, F, count, nv, bad.as<int>());
  int h = 0;
  THEA_CUDA_CHECK(cudaMemcpyAsync(&h, bad.ptr, sizeof(int), cudaMemcpyDeviceToHost, stream));
  THEA_CUDA_CHECK(cudaStreamSynchronize(stream));
  THEA_REQUIRE(h == 0, std::string(what) + ": a face index lies outside [0, num_vertices)");
}

thea_bvh * build_bvh(bool is_mesh, float const * V, int64_t nv, int32_t const * F, int64_t nf,
                     thea_build_config const & cfg, cudaStream_t stream) {
  return build_forest(is_mesh, V, nv, F, nf, nullptr, 1, cfg, stream);
}

void destroy_bvh(thea_bvh * b) {
  if (!b) return;
  if (b->world) {
    b->world->err = nullptr;  // shared with b
    destroy_bvh(b->world);
    b->world = nullptr;
  }
  int prev = -1;
  cudaGetDevice(&prev);
  cudaSetDevice(b->device);
  cudaDeviceSynchronize();
  if (b->nodes) cudaFree(b->nodes);
  if (b->cp_rec) cudaFree(b->cp_rec);
  if (b->slabs) cudaFree(b->slabs);
  if (b->ray_rec) cudaFree(b->ray_rec);
  if (b->pt_rec) cudaFree(b->pt_rec);
  if (b->leaf_to_elem) cudaFree(b->leaf_to_elem);
  if (b->err) cudaFree(b->err);
  if (b->err_host) cudaFreeHost(b->err_host);
  if (b->seg_start) cudaFree(b->seg_start);
  if (b->seg_root) cudaFree(b->seg_root);
  if (b->seg_roots) cudaFree(b->seg_roots);
  if (prev >= 0) cudaSetDevice(prev);
  delete b;
}

}  // namespace thea
