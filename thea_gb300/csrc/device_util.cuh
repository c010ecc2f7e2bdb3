// Device-wide building blocks used by the BVH build and the sampler: stream-ordered scratch buffers, an exclusive scan,
// and a stable LSD radix sort of (64-bit key, 32-bit value) pairs.
//
// The radix sort is reduce-then-scan: per 8-bit digit pass, an upsweep kernel counts digits per tile, one exclusive scan
// over the digit-major [256][tiles] count matrix gives every (digit, tile) its output offset, and a downsweep kernel
// ranks keys inside each tile with warp match/ballot and scatters them. No CTA ever waits on another CTA.
#pragma once

#include "common.cuh"

#include <mutex>

#include <algorithm>
#include <cstring>

namespace thea {

// The library's own stream-ordered memory pool on the current device (created once per device, with a release
// threshold high enough that freed scratch stays mapped for the next call instead of going back to the driver).
cudaMemPool_t scratch_pool();

// A device buffer taken from the library's stream-ordered pool and returned to it when the owner goes out of scope.
// Multiprocessor count of the current device (cached per device; safe to call from several threads)
inline int sm_count() {
  static std::mutex m;
  static int counts[64] = {0};
  int dev = 0;
  THEA_CUDA_CHECK(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(m);
  if (dev < 0 || dev >= 64) dev = 0;
  if (!counts[dev]) THEA_CUDA_CHECK(cudaDeviceGetAttribute(&counts[dev], cudaDevAttrMultiProcessorCount, dev));
  return counts[dev];
}

struct Scratch {
  void * ptr = nullptr;
  size_t bytes = 0;
  cudaStream_t stream = nullptr;
  Scratch() {}
  Scratch(size_t n, cudaStream_t s) : bytes(n), stream(s) {
    if (n) THEA_CUDA_CHECK(thea_malloc_from_pool_async(&ptr, n, scratch_pool(), s));
  }
  Scratch(Scratch const &) = delete;
  Scratch & operator=(Scratch const &) = delete;
  Scratch(Scratch && o) noexcept : ptr(o.ptr), bytes(o.bytes), stream(o.stream) { o.ptr = nullptr; }
  Scratch & operator=(Scratch && o) noexcept {
    release();
    ptr = o.ptr; bytes = o.bytes; stream = o.stream; o.ptr = nullptr;
    return *this;
  }
  ~Scratch() { release(); }
  void release() {
    if (ptr) cudaFreeAsync(ptr, stream);
    ptr = nullptr;
  }
  template <class T> T * as() const { return static_cast<T *>(ptr); }
};

//============================================================================================================================
// Exclusive scan (uint32 or uint64 elements)
//============================================================================================================================

constexpr int SCAN_THREADS = 512;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

template <class T> __device__ __forceinline__ T warp_inclusive_scan(T v) {
  int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += u;
  }
  return v;
}

// Block-wide exclusive scan of one value per thread; returns the exclusive prefix and writes the block total.
template <class T> __device__ __forceinline__ T block_exclusive_scan(T v, T & total) {
  __shared__ T warp_sums[32];
  __shared__ T tot;
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int nw = (int)(blockDim.x >> 5);
  T inc = warp_inclusive_scan(v);
  if (lane == 31) warp_sums[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    T w = lane < nw ? warp_sums[lane] : T(0);
    T wi = warp_inclusive_scan(w);
    if (lane < nw) warp_sums[lane] = wi - w;
    if (lane == nw - 1) tot = wi;
  }
  __syncthreads();
  T excl = warp_sums[warp] + inc - v;
  total = tot;
  __syncthreads();  // warp_sums and tot are reused by the next call
  return excl;
}

template <class T> __global__ void scan_reduce_kernel(T const * __restrict__ in, int64_t n, T * __restrict__ partials) {
  int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
  T s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    int64_t i = base + (int64_t)k * SCAN_THREADS + threadIdx.x;
    if (i < n) s += in[i];
  }
  T total;
  block_exclusive_scan(s, total);
  if (threadIdx.x == 0) partials[blockIdx.x] = total;
}

template <class T>
__global__ void scan_downsweep_kernel(T const * __restrict__ in, int64_t n, T const * __restrict__ block_offsets,
                                      T * __restrict__ out) {
  __shared__ T tile[SCAN_TILE];
  int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    int idx = k * SCAN_THREADS + threadIdx.x;
    int64_t i = base + idx;
    tile[idx] = i < n ? in[i] : T(0);
  }
  __syncthreads();
  T v[SCAN_ITEMS];
  T s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    v[k] = tile[threadIdx.x * SCAN_ITEMS + k];
    s += v[k];
  }
  T total;
  T excl = block_exclusive_scan(s, total);
  T run = excl + (block_offsets ? block_offsets[blockIdx.x] : T(0));
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    tile[threadIdx.x * SCAN_ITEMS + k] = run;
    run += v[k];
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    int idx = k * SCAN_THREADS + threadIdx.x;
    int64_t i = base + idx;
    if (i < n) out[i] = tile[idx];
  }
}

// out[i] = sum(in[0..i)); in and out may alias. Returns nothing; the total can be read as out[n-1] + in[n-1].
template <class T> void exclusive_scan(T const * in, T * out, int64_t n, cudaStream_t stream) {
  if (n <= 0) return;
  int64_t blocks = ceil_div(n, SCAN_TILE);
  if (blocks == 1) {
    THEA_LAUNCH(scan_downsweep_kernel<T>, 1, SCAN_THREADS, 0, stream, in, n, (T const *)nullptr, out);
    return;
  }
  Scratch partials((size_t)blocks * sizeof(T), stream);
  THEA_LAUNCH(scan_reduce_kernel<T>, (unsigned)blocks, SCAN_THREADS, 0, stream, in, n, partials.as<T>());
  exclusive_scan<T>(partials.as<T>(), partials.as<T>(), blocks, stream);
  THEA_LAUNCH(scan_downsweep_kernel<T>, (unsigned)blocks, SCAN_THREADS, 0, stream, in, n,
              (T const *)partials.as<T>(), out);
}

//============================================================================================================================
// Stable LSD radix sort of (uint64 key, uint32 value)
//============================================================================================================================

constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_ITEMS = 8;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;
constexpr int RS_BINS = 256;

// Item j of lane l in warp w of a tile sits at tile offset w * 32 * RS_ITEMS + j * 32 + l (warp-striped)
__device__ __forceinline__ int64_t rs_item_index(int64_t tile, int warp, int j, int lane) {
  return tile * RS_TILE + (int64_t)warp * (32 * RS_ITEMS) + j * 32 + lane;
}

static __global__ void rs_upsweep_kernel(uint64_t const * __restrict__ keys, int64_t n, int shift, uint32_t * __restrict__ counts,
                                  int64_t num_tiles) {
  __shared__ uint32_t hist[RS_BINS];
  for (int d = threadIdx.x; d < RS_BINS; d += RS_THREADS) hist[d] = 0;
  __syncthreads();
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t tile = blockIdx.x;
#pragma unroll
  for (int j = 0; j < RS_ITEMS; ++j) {
    int64_t i = rs_item_index(tile, warp, j, lane);
    if (i < n) atomicAdd(&hist[(uint32_t)(keys[i] >> shift) & 0xffu], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < RS_BINS; d += RS_THREADS) counts[(int64_t)d * num_tiles + tile] = hist[d];
}

static __global__ void rs_downsweep_kernel(uint64_t const * __restrict__ keys_in, uint32_t const * __restrict__ vals_in,
                                    uint64_t * __restrict__ keys_out, uint32_t * __restrict__ vals_out, int64_t n,
                                    int shift, uint32_t const * __restrict__ offsets, int64_t num_tiles) {
  __shared__ uint32_t wc[RS_WARPS][RS_BINS];
  __shared__ uint32_t base[RS_BINS];
  for (int t = threadIdx.x; t < RS_WARPS * RS_BINS; t += RS_THREADS) (&wc[0][0])[t] = 0;
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t tile = blockIdx.x;
  uint64_t k[RS_ITEMS];
  uint32_t v[RS_ITEMS];
  uint32_t dig[RS_ITEMS];
  uint32_t rank[RS_ITEMS];
#pragma unroll
  for (int j = 0; j < RS_ITEMS; ++j) {
    int64_t i = rs_item_index(tile, warp, j, lane);
    bool ok = i < n;
    k[j] = ok ? keys_in[i] : 0ull;
    v[j] = ok ? vals_in[i] : 0u;
    // invalid items get a per-lane sentinel that matches no digit and no other lane
    dig[j] = ok ? (uint32_t)(k[j] >> shift) & 0xffu : (0x10000u | (uint32_t)lane);
  }
  __syncthreads();
  unsigned lt_mask = (1u << lane) - 1u;
#pragma unroll
  for (int j = 0; j < RS_ITEMS; ++j) {
    bool ok = dig[j] < RS_BINS;
    unsigned peers = __match_any_sync(0xffffffffu, dig[j]);
    uint32_t prior = ok ? wc[warp][dig[j]] : 0u;
    __syncwarp();
    if (ok && lane == __ffs(peers) - 1) wc[warp][dig[j]] = prior + (uint32_t)__popc(peers);
    __syncwarp();
    rank[j] = prior + (uint32_t)__popc(peers & lt_mask);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < RS_BINS; d += RS_THREADS) {
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < RS_WARPS; ++w) {
      uint32_t t = wc[w][d];
      wc[w][d] = run;
      run += t;
    }
    base[d] = offsets[(int64_t)d * num_tiles + tile];
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < RS_ITEMS; ++j) {
    if (dig[j] < RS_BINS) {
      uint32_t dst = base[dig[j]] + wc[warp][dig[j]] + rank[j];
      keys_out[dst] = k[j];
      vals_out[dst] = v[j];
    }
  }
}

// Digit histogram of all 8 byte positions, to skip passes in which every key has the same digit.
static __global__ void rs_global_hist_kernel(uint64_t const * __restrict__ keys, int64_t n, uint32_t * __restrict__ hist) {
  __shared__ uint32_t h[8][RS_BINS];
  for (int t = threadIdx.x; t < 8 * RS_BINS; t += blockDim.x) (&h[0][0])[t] = 0;
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    uint64_t key = keys[i];
#pragma unroll
    for (int p = 0; p < 8; ++p) atomicAdd(&h[p][(uint32_t)(key >> (8 * p)) & 0xffu], 1u);
  }
  __syncthreads();
  for (int t = threadIdx.x; t < 8 * RS_BINS; t += blockDim.x)
    if ((&h[0][0])[t]) atomicAdd(&hist[t], (&h[0][0])[t]);
}

// Sorts (keys, vals) by key, stably, considering bits [0, key_bits). Results end in keys/vals. n < 2^32.
// probe_passes: read a digit histogram back to the host first and skip passes in which every key has the same digit
// (synchronizes the stream); without it every pass runs and the call stays asynchronous.
inline void radix_sort_pairs(uint64_t * keys, uint32_t * vals, int64_t n, int key_bits, cudaStream_t stream,
                             bool probe_passes = true) {
  if (n <= 1) return;
  THEA_REQUIRE(n < (int64_t(1) << 32), "radix sort: too many elements");
  int passes = (key_bits + 7) / 8;
  uint32_t h_hist[8 * RS_BINS];
  memset(h_hist, 0, sizeof(h_hist));
  if (probe_passes) {
    Scratch ghist(8 * RS_BINS * sizeof(uint32_t), stream);
    THEA_CUDA_CHECK(cudaMemsetAsync(ghist.ptr, 0, ghist.bytes, stream));
    int hb = (int)std::min<int64_t>(ceil_div(n, 256), 1024);
    THEA_LAUNCH(rs_global_hist_kernel, hb, 256, 0, stream, keys, n, ghist.as<uint32_t>());
    THEA_CUDA_CHECK(cudaMemcpyAsync(h_hist, ghist.ptr, sizeof(h_hist), cudaMemcpyDeviceToHost, stream));
    THEA_CUDA_CHECK(cudaStreamSynchronize(stream));
  }

  int64_t num_tiles = ceil_div(n, RS_TILE);
  Scratch keys_alt((size_t)n * sizeof(uint64_t), stream);
  Scratch vals_alt((size_t)n * sizeof(uint32_t), stream);
  Scratch counts((size_t)num_tiles * RS_BINS * sizeof(uint32_t), stream);
  uint64_t * kin = keys;
  uint32_t * vin = vals;
  uint64_t * kout = keys_alt.as<uint64_t>();
  uint32_t * vout = vals_alt.as<uint32_t>();
  for (int p = 0; p < passes; ++p) {
    bool trivial = false;
    for (int d = 0; d < RS_BINS; ++d)
      if ((int64_t)h_hist[p * RS_BINS + d] == n) trivial = true;
    if (trivial) continue;
    THEA_LAUNCH(rs_upsweep_kernel, (unsigned)num_tiles, RS_THREADS, 0, stream, kin, n, 8 * p, counts.as<uint32_t>(),
                num_tiles);
    exclusive_scan<uint32_t>(counts.as<uint32_t>(), counts.as<uint32_t>(), num_tiles * RS_BINS, stream);
    THEA_LAUNCH(rs_downsweep_kernel, (unsigned)num_tiles, RS_THREADS, 0, stream, kin, vin, kout, vout, n, 8 * p,
                counts.as<uint32_t>(), num_tiles);
    std::swap(kin, kout);
    std::swap(vin, vout);
  }
  if (kin != keys) {
    THEA_CUDA_CHECK(cudaMemcpyAsync(keys, kin, (size_t)n * sizeof(uint64_t), cudaMemcpyDeviceToDevice, stream));
    THEA_CUDA_CHECK(cudaMemcpyAsync(vals, vin, (size_t)n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, stream));
  }
}

}  // namespace thea
