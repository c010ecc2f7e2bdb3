// Wide-node access and the per-query traversal stack shared by the query kernels.
#pragma once

#include "common.cuh"

namespace thea {

template <int W> struct NodeRegs {
  float lox[W], hix[W], loy[W], hiy[W], loz[W], hiz[W];
  int child[W];
};

// A node is W*6 box floats followed by W child codes, read as 16-byte vector loads through the read-only path.
template <int W> __device__ __forceinline__ void load_node(WideNode<W> const * __restrict__ nodes, int idx,
                                                           NodeRegs<W> & r) {
  float4 const * p = reinterpret_cast<float4 const *>(nodes + idx);
  constexpr int Q = W / 4;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    float4 a = __ldg(p + 0 * Q + q), b = __ldg(p + 1 * Q + q), c = __ldg(p + 2 * Q + q);
    float4 d = __ldg(p + 3 * Q + q), e = __ldg(p + 4 * Q + q), f = __ldg(p + 5 * Q + q);
    int4 g = __ldg(reinterpret_cast<int4 const *>(p + 6 * Q + q));
    r.lox[4 * q] = a.x; r.lox[4 * q + 1] = a.y; r.lox[4 * q + 2] = a.z; r.lox[4 * q + 3] = a.w;
    r.hix[4 * q] = b.x; r.hix[4 * q + 1] = b.y; r.hix[4 * q + 2] = b.z; r.hix[4 * q + 3] = b.w;
    r.loy[4 * q] = c.x; r.loy[4 * q + 1] = c.y; r.loy[4 * q + 2] = c.z; r.loy[4 * q + 3] = c.w;
    r.hiy[4 * q] = d.x; r.hiy[4 * q + 1] = d.y; r.hiy[4 * q + 2] = d.z; r.hiy[4 * q + 3] = d.w;
    r.loz[4 * q] = e.x; r.loz[4 * q + 1] = e.y; r.loz[4 * q + 2] = e.z; r.loz[4 * q + 3] = e.w;
    r.hiz[4 * q] = f.x; r.hiz[4 * q + 1] = f.y; r.hiz[4 * q + 2] = f.z; r.hiz[4 * q + 3] = f.w;
    r.child[4 * q] = g.x; r.child[4 * q + 1] = g.y; r.child[4 * q + 2] = g.z; r.child[4 * q + 3] = g.w;
  }
}

// Ascending odd-even transposition sort of W (key, code) pairs held in registers. Keys are non-negative float bit
// patterns or 0xFFFFFFFF for "do not visit".
template <int W> __device__ __forceinline__ void sort_children(uint32_t (&key)[W], int (&code)[W]) {
#pragma unroll
  for (int pass = 0; pass < W; ++pass) {
#pragma unroll
    for (int i = pass & 1; i + 1 < W; i += 2) {
      bool sw = key[i + 1] < key[i];
      uint32_t k0 = sw ? key[i + 1] : key[i], k1 = sw ? key[i] : key[i + 1];
      int c0 = sw ? code[i + 1] : code[i], c1 = sw ? code[i] : code[i + 1];
      key[i] = k0; key[i + 1] = k1;
      code[i] = c0; code[i + 1] = c1;
    }
  }
}

// Squared distance from a point to a box (any order of evaluation gives a valid bound thanks to the box padding)
__device__ __forceinline__ float point_box_d2(float px, float py, float pz, float lx, float ly, float lz, float hx,
                                              float hy, float hz) {
  float dx = fmaxf(fmaxf(lx - px, px - hx), 0.f);
  float dy = fmaxf(fmaxf(ly - py, py - hy), 0.f);
  float dz = fmaxf(fmaxf(lz - pz, pz - hz), 0.f);
  return __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, dz * dz));
}

// Stack depth bound: a W-wide tree of depth D needs at most D * (W - 1) + 1 entries
template <int W> struct StackSize { static constexpr int value = W == 4 ? 64 : 128; };

// Device-side error bits reported through the handle's error word
constexpr unsigned ERR_STACK_OVERFLOW = 1u;
// a bounded wait of the tensor-core k-NN candidate kernel gave up (its queries fell back to the plain search)
constexpr unsigned ERR_GRAM_TIMEOUT = 2u;

}  // namespace thea
