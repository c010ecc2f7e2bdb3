// k-NN candidates from tensor-core Gram tiles (tcgen05), re-ranked exactly in FP32, then finished by a BVH traversal
// bounded by the re-ranked k-th distance.
//
// Points are taken in the point BVH's leaf order (a Morton order), so a block of 128 consecutive points and the 512
// points around it are spatial neighbours. One CTA scores its 128 query points against that 512-point window with four
// tcgen05.mma (M = 128, N = 128, K = 16, FP16 operands, FP32 accumulators in tensor memory):
//   A row r = (a_r, 1, 0, ...)          B row j = (-2 b_j, |b_j|^2, 0, ...)        (A B^T)[r][j] = |b_j|^2 - 2 a_r . b_j
// with coordinates taken relative to the block's first point and scaled to the window's extent. Per row that is
// |a_r - b_j|^2 - |a_r|^2, so the row's order of the keys is the order of the squared distances (up to FP16 rounding).
// Each thread owns one row (one tensor-memory lane), keeps the KP smallest keys, re-computes those candidates' squared
// distances with the reference's FP32 arithmetic and outputs the k-th smallest as an upper bound on the query's k-th
// neighbour distance. The exact search (knn_query, seeded with that bound) then returns the same neighbours as the
// plain traversal; the Gram tile only tightens its pruning from the first node on.
//
// Every wait on the MMA's completion barrier is bounded; on expiry the kernel records THEA_ERR_BIT_GRAM_TIMEOUT in the
// BVH's error word, leaves the bound at +inf (the plain search), waits once more (bounded) and frees its tensor memory.
#include "gram.hpp"

#include "device_util.cuh"
#include "query.hpp"
#include "traverse_ops.cuh"

#include <cuda_fp16.h>
#include <algorithm>
#include <cstdint>

namespace thea {
namespace {

constexpr int GRAM_M = 128;      // query rows per CTA (tensor-memory lanes)
constexpr int GRAM_N = 128;      // candidates per MMA
constexpr int GRAM_PASSES = 4;
constexpr int GRAM_WINDOW = GRAM_N * GRAM_PASSES;
constexpr int GRAM_K = 16;       // K of one f16 MMA; coordinates use 4 of it
constexpr int GRAM_THREADS = 128;
constexpr uint32_t GRAM_TMEM_COLS = 128;
constexpr int GRAM_SPIN_LIMIT = 1 << 20;  // try_wait rounds before a wait is declared failed

// Operand tiles in the no-swizzle K-major core-matrix layout: 8 rows x 16 bytes per core matrix (128 B contiguous), the
// two core matrices of a row group along K 128 B apart (leading byte offset), row groups 256 B apart (stride byte
// offset).
constexpr uint32_t GRAM_LBO = 128;
constexpr uint32_t GRAM_SBO = 256;

__device__ __forceinline__ int core_off(int r, int k) {  // in f16 elements
  return (r >> 3) * (GRAM_SBO / 2) + (k >> 3) * (GRAM_LBO / 2) + (r & 7) * 8 + (k & 7);
}

struct __align__(1024) GramSmem {
  uint16_t a[GRAM_M * GRAM_K];       // FP16 bits, 4 KB
  uint16_t b[GRAM_WINDOW * GRAM_K];  // 16 KB
  unsigned long long mbar;
  uint32_t tmem_base;
  unsigned maxabs_bits;
  int failed;
  uint32_t failed_parity;
};

__device__ __forceinline__ uint32_t smem_addr(void const * p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start address, leading / stride byte offsets (all >> 4), descriptor version 1,
// base offset 0, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(void const * p) {
  uint64_t d = 0;
  d |= (uint64_t)((smem_addr(p) >> 4) & 0x3fffu);
  d |= (uint64_t)((GRAM_LBO >> 4) & 0x3fffu) << 16;
  d |= (uint64_t)((GRAM_SBO >> 4) & 0x3fffu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator, FP16 A and B, both K-major, N and M
constexpr uint32_t GRAM_IDESC =
    (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(GRAM_N >> 3) << 17) | ((uint32_t)(GRAM_M >> 4) << 24);

__device__ __forceinline__ void tmem_alloc(uint32_t * dst_smem) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst_smem)),
               "r"(GRAM_TMEM_COLS)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t base) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(base), "r"(GRAM_TMEM_COLS) : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc) {
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "setp.ne.b32 p, 0, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
      "}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc)
      : "memory");
}

__device__ __forceinline__ void mma_commit(unsigned long long * bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

// Bounded wait for the barrier phase `parity`; false if it did not complete within `limit` rounds.
__device__ __forceinline__ bool mbar_wait(unsigned long long * bar, uint32_t parity, int limit = GRAM_SPIN_LIMIT) {
  uint32_t a = smem_addr(bar);
  for (int i = 0; i < limit; ++i) {
    uint32_t ok;
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// 32 consecutive accumulator columns of this thread's lane (row)
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Stages the A block (rows a_pts[0..GRAM_M)) and the B window (b_pts[0..GRAM_WINDOW)) relative to `c`, scaled by the
// window's extent; missing rows (count < tile) are zero. One call per CTA, all threads.
__device__ void stage_tiles(GramSmem & s, float4 const * __restrict__ a_pts, int a_count,
                            float4 const * __restrict__ b_pts, int b_count, V3 c) {
  int t = threadIdx.x;
  if (t == 0) s.maxabs_bits = 0;
  __syncthreads();
  float m = 0.f;
  if (t < a_count) {
    V3 p = xyz(__ldg(a_pts + t)) - c;
    m = fmaxf(m, fmaxf(fabsf(p.x), fmaxf(fabsf(p.y), fabsf(p.z))));
  }
  for (int j = t; j < b_count; j += GRAM_THREADS) {
    V3 p = xyz(__ldg(b_pts + j)) - c;
    m = fmaxf(m, fmaxf(fabsf(p.x), fmaxf(fabsf(p.y), fabsf(p.z))));
  }
  atomicMax(&s.maxabs_bits, __float_as_uint(m));
  __syncthreads();
  float ext = __uint_as_float(s.maxabs_bits);
  float inv = ext > 0.f ? 1.f / ext : 1.f;
  for (int r = t; r < GRAM_M; r += GRAM_THREADS) {
    float v[4] = {0.f, 0.f, 0.f, 0.f};
    if (r < a_count) {
      V3 p = xyz(__ldg(a_pts + r)) - c;
      v[0] = p.x * inv;
      v[1] = p.y * inv;
      v[2] = p.z * inv;
      v[3] = 1.f;
    }
#pragma unroll
    for (int k = 0; k < GRAM_K; ++k) s.a[core_off(r, k)] = __half_as_ushort(__float2half_rn(k < 4 ? v[k] : 0.f));
  }
  for (int j = t; j < GRAM_WINDOW; j += GRAM_THREADS) {
    float v[4] = {0.f, 0.f, 0.f, 0.f};
    if (j < b_count) {
      V3 p = xyz(__ldg(b_pts + j)) - c;
      float x = p.x * inv, y = p.y * inv, z = p.z * inv;
      v[0] = -2.f * x;
      v[1] = -2.f * y;
      v[2] = -2.f * z;
      v[3] = x * x + y * y + z * z;
    } else {
      v[3] = 65504.f;  // padding rows score worst
    }
#pragma unroll
    for (int k = 0; k < GRAM_K; ++k) s.b[core_off(j, k)] = __half_as_ushort(__float2half_rn(k < 4 ? v[k] : 0.f));
  }
  // make the tiles visible to the tensor core (async proxy) before the MMA is issued
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();
}

// Allocates tensor memory (warp 0) and initialises the completion barrier (thread 0).
__device__ void gram_setup(GramSmem & s) {
  if (threadIdx.x < 32) tmem_alloc(&s.tmem_base);
  if (threadIdx.x == 0) {
    s.failed = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&s.mbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
}

// One MMA pass over window half `pass`; returns false (and flags the CTA) if its completion was not observed.
// `phase` counts the CTA's MMA commits so far (the barrier's phase parity alternates with each).
__device__ bool gram_pass(GramSmem & s, int pass, uint32_t phase) {
  if (threadIdx.x == 0) {
    mma_f16(s.tmem_base, smem_desc(s.a), smem_desc(s.b + pass * GRAM_N * GRAM_K), GRAM_IDESC);
    mma_commit(&s.mbar);
  }
  bool ok = mbar_wait(&s.mbar, phase & 1u);
  if (!ok) {
    atomicOr(&s.failed, 1);
    s.failed_parity = phase & 1u;
  }
  __syncthreads();  // the verdict is the CTA's, so the warp-collective loads below are taken by all lanes or none
  fence_after_sync();
  return s.failed == 0;
}

// Before the next pass overwrites the accumulators, or before the tensor memory is freed
__device__ void gram_pass_end(GramSmem & s) {
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
}

__device__ void gram_teardown(GramSmem & s, unsigned * err) {
  __syncthreads();
  if (s.failed) {
    // the MMA of the failed pass may still be running: one more bounded wait on its phase before the tensor memory is
    // released (no MMA is issued after a failure)
    if (threadIdx.x == 0) {
      mbar_wait(&s.mbar, s.failed_parity);
      if (err) atomicOr(err, ERR_GRAM_TIMEOUT);
    }
    __syncthreads();
  }
  if (threadIdx.x < 32) tmem_dealloc(s.tmem_base);
}

// Keeps the KP smallest (key, position) pairs, sorted ascending; position -1 = empty.
template <int KP> __device__ __forceinline__ void cand_insert(float (&ck)[KP], int (&cp)[KP], float key, int pos) {
#pragma unroll
  for (int j = 0; j < KP; ++j) {
    bool lt = key < ck[j];
    float tk = ck[j];
    int tp = cp[j];
    ck[j] = lt ? key : tk;
    cp[j] = lt ? pos : tp;
    key = lt ? tk : key;
    pos = lt ? tp : pos;
  }
}

// Bound kernel: persistent CTAs (tensor memory allocated once per CTA) take blocks of GRAM_M consecutive leaf positions
// from a global counter. bound[q] = k-th smallest exact FP32 squared distance among the query's KP best-scoring window
// candidates (+inf if fewer than k), excluding the point itself.
//
// Selection cost is dominated by insertions into the per-row candidate list, and a warp pays for an insertion whenever
// any of its lanes makes one. Each warp therefore reads its accumulator columns starting from the 32 candidates around
// its own rows (their Morton neighbours) and moving outward, so the list holds near neighbours early and later
// candidates rarely pass its threshold.
template <int KP, int KX>
__global__ void __launch_bounds__(GRAM_THREADS)
gram_bound_kernel(float4 const * __restrict__ pts, int64_t n, int k, float * __restrict__ bound,
                  unsigned long long * __restrict__ next_block, unsigned * err) {
  __shared__ GramSmem s;
  __shared__ long long s_blk;
  int64_t nblocks = ceil_div(n, GRAM_M);
  gram_setup(s);
  int warp = threadIdx.x >> 5;
  uint32_t lane_base = s.tmem_base + ((uint32_t)(warp * 32) << 16);
  uint32_t phase = 0;
  while (true) {
    if (threadIdx.x == 0) s_blk = (long long)atomicAdd(next_block, 1ull);
    __syncthreads();
    int64_t blk = s_blk;
    if (blk >= nblocks) break;
    int64_t q0 = blk * GRAM_M;
    int64_t w0 = q0 + GRAM_M / 2 - GRAM_WINDOW / 2;
    w0 = w0 < 0 ? 0 : (w0 + GRAM_WINDOW > n ? n - GRAM_WINDOW : w0);
    int a_count = (int)(n - q0 < GRAM_M ? n - q0 : GRAM_M);
    bool live = s.failed == 0;
    if (live) stage_tiles(s, pts + q0, a_count, pts + w0, GRAM_WINDOW, xyz(__ldg(pts + q0)));
    int64_t q = q0 + threadIdx.x;
    int64_t self = q - w0;
    float ck[KP];
    int cpos[KP];
#pragma unroll
    for (int j = 0; j < KP; ++j) {
      ck[j] = INFINITY;
      cpos[j] = -1;
    }
    // the warp's own 32 rows sit in window chunk (q0 + 32 warp - w0) / 32
    int own = (int)((q0 + 32 * warp - w0) >> 5);
    for (int pass = 0; pass < GRAM_PASSES && live; ++pass) {
      bool ok = gram_pass(s, pass, phase++);
      if (ok) {
        int first = own - pass * (GRAM_N / 32);
        first = first < 0 ? 0 : (first > GRAM_N / 32 - 1 ? GRAM_N / 32 - 1 : first);
        int done = 0;
#pragma unroll 1
        for (int t = 0; done < GRAM_N / 32; ++t) {
          int ch = first + ((t + 1) >> 1) * ((t & 1) ? 1 : -1);
          if (ch < 0 || ch >= GRAM_N / 32) continue;
          ++done;
          float v[32];
          tmem_ld32(lane_base + (uint32_t)(ch * 32), v);
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            int pos = pass * GRAM_N + ch * 32 + j;
            if (v[j] < ck[KP - 1] && pos != self) cand_insert<KP>(ck, cpos, v[j], pos);
          }
        }
      }
      gram_pass_end(s);
      live = s.failed == 0;
    }
    if (q < n) {
      // exact re-rank: the reference's FP32 squared distance, lowest index on ties
      V3 p = xyz(__ldg(pts + q));
      float bd[KX];
      int bi[KX];
#pragma unroll
      for (int j = 0; j < KX; ++j) {
        bd[j] = INFINITY;
        bi[j] = INT_MAX;
      }
#pragma unroll
      for (int j = 0; j < KP; ++j) {
        if (cpos[j] < 0 || !live) continue;
        float4 b = __ldg(pts + w0 + cpos[j]);
        float d2 = squared_norm(xyz(b) - p);
        int idx = __float_as_int(b.w);
        if (d2 < bd[KX - 1] || (d2 == bd[KX - 1] && idx < bi[KX - 1])) knn_insert<KX>(bd, bi, d2, idx);
      }
      float kth = INFINITY;
#pragma unroll
      for (int j = 0; j < KX; ++j)
        if (j == k - 1) kth = bd[j];
      bound[q] = live ? kth : INFINITY;
    }
    __syncthreads();  // s_blk and the tiles are rewritten by the next block
  }
  gram_teardown(s, err);
}

// Raw Gram tile of two point sets (the candidate score above, for tests): keys[r][j] = |b_j|^2 - 2 a_r . b_j in the
// tile's normalised FP16 frame (relative to a[0], scaled to the tiles' extent), FP32 accumulation.
__global__ void __launch_bounds__(GRAM_THREADS)
gram_tile_kernel(float4 const * __restrict__ a, int na, float4 const * __restrict__ b, int nb, float * __restrict__ keys,
                 unsigned * err) {
  __shared__ GramSmem s;
  V3 c = xyz(__ldg(a));
  gram_setup(s);
  stage_tiles(s, a, na, b, nb, c);
  uint32_t lane_base = s.tmem_base + ((uint32_t)((threadIdx.x >> 5) * 32) << 16);
  int row = threadIdx.x;
  for (int pass = 0; pass < GRAM_PASSES; ++pass) {
    bool ok = gram_pass(s, pass, (uint32_t)pass);
#pragma unroll 1
    for (int c0 = 0; c0 < GRAM_N; c0 += 32) {
      float v[32];
      if (ok) tmem_ld32(lane_base + (uint32_t)c0, v);
#pragma unroll
      for (int j = 0; j < 32; ++j) keys[(int64_t)row * GRAM_WINDOW + pass * GRAM_N + c0 + j] = ok ? v[j] : NAN;
    }
    gram_pass_end(s);
  }
  gram_teardown(s, err);
}

// Self-test of the bounded wait above: one warp waits on a barrier phase that nothing completes. The wait must give up
// after `limit` rounds and report it (out = 1), leaving the context usable.
__global__ void wait_probe_kernel(int limit, int * out) {
  __shared__ unsigned long long bar;
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  bool ok = mbar_wait(&bar, 0u, limit);
  if (threadIdx.x == 0) *out = ok ? 0 : 1;
}

__global__ void to_float4_kernel(float const * __restrict__ p, int n, float4 * __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = make_float4(p[3 * i], p[3 * i + 1], p[3 * i + 2], __int_as_float(i));
}

}  // namespace

bool run_wait_probe(int limit, cudaStream_t s) {
  Scratch flag(sizeof(int), s);
  THEA_LAUNCH(wait_probe_kernel, 1, 32, 0, s, limit, flag.as<int>());
  int h = 0;
  THEA_CUDA_CHECK(cudaMemcpyAsync(&h, flag.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
  THEA_CUDA_CHECK(cudaStreamSynchronize(s));
  return h != 0;
}

int gram_tile_rows() { return GRAM_M; }
int gram_tile_cols() { return GRAM_WINDOW; }

bool gram_supported(int64_t n) { return n >= GRAM_WINDOW; }

void run_gram_bounds(thea_bvh const * b, int k, float * bound, cudaStream_t s) {
  int64_t n = b->n;
  float4 const * pts = b->pt_rec;
  // four CTAs per SM: each holds a quarter of the SM's tensor memory (128 of 512 columns) for its whole life
  int sms = sm_count();
  int blocks = (int)std::min<int64_t>(ceil_div(n, GRAM_M), 4 * (int64_t)sms);
  Scratch counter(sizeof(unsigned long long), s);
  THEA_CUDA_CHECK(cudaMemsetAsync(counter.ptr, 0, sizeof(unsigned long long), s));
  unsigned long long * next = counter.as<unsigned long long>();
  // KP = the k bucket: the selection's cost grows with the square of the list length, and the re-rank of the k best
  // scored candidates already gives a bound close to the k-th neighbour distance
  auto k8 = gram_bound_kernel<8, 8>;
  auto k16 = gram_bound_kernel<16, 16>;
  auto k32 = gram_bound_kernel<32, 32>;
  auto kern = k <= 8 ? k8 : k <= 16 ? k16 : k32;
  THEA_LAUNCH_NAMED("gram_bound_kernel", kern, blocks, GRAM_THREADS, 0, s, pts, n, k, bound, next, b->err);
}

void run_gram_tile(float const * a, int na, float const * b, int nb, float * keys, unsigned * err, cudaStream_t s) {
  Scratch a4((size_t)GRAM_M * sizeof(float4), s), b4((size_t)GRAM_WINDOW * sizeof(float4), s);
  THEA_LAUNCH(to_float4_kernel, 1, GRAM_M, 0, s, a, na, a4.as<float4>());
  THEA_LAUNCH(to_float4_kernel, (int)ceil_div(nb, 128), 128, 0, s, b, nb, b4.as<float4>());
  THEA_LAUNCH(gram_tile_kernel, 1, GRAM_THREADS, 0, s, a4.as<float4>(), na, b4.as<float4>(), nb, keys, err);
}

}  // namespace thea
