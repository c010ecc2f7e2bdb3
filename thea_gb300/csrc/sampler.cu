// Area-weighted mesh sampling: MeshSampler::sampleEvenlyByArea in EXACT count mode
// (Code/Source/Algorithms/MeshSampler.hpp:100-204) with TriangleN<3>::randomPoint (Code/Source/Triangle3.hpp:179-195).
//
// Bit-identical to the reference when drawing from the reference's Random(seed) stream: the per-triangle FP32 areas, the
// FP64 cumulative-area table built by a sequential sum in index order (so its rounding matches the reference's loop),
// one lower_bound per sample, and the FP32 parallelogram point with reflection. Sample i consumes words 3i, 3i+1, 3i+2
// of the stream (triangle choice, then s, then t).
//
// The Thea Mersenne-Twister stream (Code/Source/Random.cpp:49-132) is produced by one CTA: each 624-word twist runs as
// three dependent phases of at most 227 independent updates (the second loop of Thea's generate() starts at N - M + 1,
// so word N - M keeps its value), then all 624 words are tempered and written out. The counter mode draws the three
// words of sample i from Philox-4x32-10 (Salmon et al., SC'11) keyed by the seed, which is fully parallel.
#include "device_util.cuh"
#include "bvh.hpp"
#include "query.hpp"

#include <climits>
#include <mutex>
#include <string>

namespace thea {
namespace {

constexpr int MT_N = 624, MT_M = 397;
constexpr uint32_t MT_A = 0x9908B0DFu, MT_B = 0x9D2C5680u, MT_C = 0xEFC60000u;
constexpr uint32_t MT_UPPER = 0x80000000u, MT_LOWER = 0x7fffffffu;
constexpr int MT_THREADS = 256;

__device__ __forceinline__ uint32_t mt_mix(uint32_t a, uint32_t b, uint32_t far) {
  uint32_t x = (a & MT_UPPER) | (b & MT_LOWER);
  return far ^ (x >> 1) ^ ((x & 1u) ? MT_A : 0u);
}

__device__ __forceinline__ uint32_t mt_temper(uint32_t r) {
  r ^= r >> 11;
  r ^= (r << 7) & MT_B;
  r ^= (r << 15) & MT_C;
  r ^= r >> 18;
  return r;
}

// One twist of Thea's generate() (Random.cpp:99-132) by a block of MT_THREADS threads, from X into Y (shared memory).
// The twisted state goes to the other half of a ping-pong buffer, so each phase needs one barrier (its inputs are the
// old state and the new words of the phase before), not two. One word per thread and phase: the twist is a chain of
// three dependent phases, and their latency is the cost (a single warp with eight words per lane and phase measured
// 4.6x slower).
__device__ __forceinline__ void mt_twist_block(uint32_t const * X, uint32_t * Y) {
  int t = threadIdx.x;
  // phase A: i in [0, N - M) from old words i, i + 1, i + M; word N - M is left as it is by Thea's twist
  if (t < MT_N - MT_M) Y[t] = mt_mix(X[t], X[t + 1], X[t + MT_M]);
  if (t == 0) Y[MT_N - MT_M] = X[MT_N - MT_M];
  __syncthreads();
  // phase B: i in [N - M + 1, 2 (N - M)) from old words i, i + 1 and new word i - (N - M)
  int i = MT_N - MT_M + 1 + t;
  if (i < 2 * (MT_N - MT_M)) Y[i] = mt_mix(X[i], X[i + 1], Y[i - (MT_N - MT_M)]);
  __syncthreads();
  // phase C: i in [2 (N - M), N - 1), and i = N - 1 (old word N - 1 with new words 0 and M - 1)
  i = 2 * (MT_N - MT_M) + t;
  if (i < MT_N - 1) Y[i] = mt_mix(X[i], X[i + 1], Y[i - (MT_N - MT_M)]);
  else if (i == MT_N - 1) Y[i] = mt_mix(X[MT_N - 1], Y[0], Y[MT_M - 1]);
  __syncthreads();
}

__device__ __forceinline__ void mt_seed_state(uint32_t seed, uint32_t * st) {
  st[0] = seed;
  for (int i = 1; i < MT_N; ++i) st[i] = 1812433253u * (st[i - 1] ^ (st[i - 1] >> 30)) + (uint32_t)i;
}

// Writes `count` tempered words of Random(seed): Random::Random(seed) then bits() repeatedly.
__global__ void __launch_bounds__(MT_THREADS) thea_mt_stream_kernel(uint32_t seed, int64_t count, uint32_t * __restrict__ out) {
  __shared__ uint32_t buf[2][MT_N];
  int t = threadIdx.x;
  if (t == 0) mt_seed_state(seed, buf[0]);
  __syncthreads();
  int64_t twists = ceil_div(count, MT_N);
  int cur = 0;
  for (int64_t k = 0; k < twists; ++k) {
    mt_twist_block(buf[cur], buf[cur ^ 1]);
    uint32_t const * Y = buf[cur ^ 1];
    int64_t base = k * MT_N;
    for (int j = t; j < MT_N; j += MT_THREADS)
      if (base + j < count) out[base + j] = mt_temper(Y[j]);
    // the next twist reads Y and writes the other buffer, whose last readers finished before the barrier above
    cur ^= 1;
  }
}

// Jump-ahead (the twist is linear over GF(2) in the 19,968 state bits, MT_A entering only through the low bit of each
// mixed word): P = T^L as a bit matrix, column j the state reached from the unit state e_j after L twists. Then the
// state before twist cL is P^c applied to the seeded state; chunks of L twists run in parallel from those states.
constexpr int MT_JUMP_TWISTS = 512;  // L
constexpr int MT_STATE_BITS = MT_N * 32;
constexpr int MT_VEC_THREADS = 640;  // one output word per thread (>= MT_N)

__global__ void __launch_bounds__(MT_THREADS) mt_jump_columns_kernel(uint32_t * __restrict__ P) {
  __shared__ uint32_t buf[2][MT_N];
  int j = blockIdx.x, t = threadIdx.x;
  for (int w = t; w < MT_N; w += MT_THREADS) buf[0][w] = w == (j >> 5) ? (1u << (j & 31)) : 0u;
  __syncthreads();
  int cur = 0;
  for (int k = 0; k < MT_JUMP_TWISTS; ++k) {
    mt_twist_block(buf[cur], buf[cur ^ 1]);
    cur ^= 1;
  }
  for (int w = t; w < MT_N; w += MT_THREADS) P[(int64_t)j * MT_N + w] = buf[cur][w];
}

// out ^= P v over the columns [blockIdx.x * per, ...) of P (out zeroed beforehand; partial sums combined by atomicXor)
__global__ void __launch_bounds__(MT_VEC_THREADS) mt_jump_apply_kernel(uint32_t const * __restrict__ P,
                                                                       uint32_t const * __restrict__ v, int per,
                                                                       uint32_t * __restrict__ out) {
  int w = threadIdx.x;
  int j0 = blockIdx.x * per, j1 = min(j0 + per, MT_STATE_BITS);
  uint32_t acc = 0;
  for (int j = j0; j < j1; ++j)
    if ((__ldg(v + (j >> 5)) >> (j & 31)) & 1u)
      if (w < MT_N) acc ^= __ldg(P + (int64_t)j * MT_N + w);
  if (w < MT_N && acc) atomicXor(out + w, acc);
}

__global__ void mt_seed_kernel(uint32_t seed, uint32_t * __restrict__ st) {
  if (threadIdx.x == 0 && blockIdx.x == 0) mt_seed_state(seed, st);
}

// Chunk c: L twists (fewer for the last) from its start state, tempered words written at their stream positions
__global__ void __launch_bounds__(MT_THREADS) mt_chunk_kernel(uint32_t const * __restrict__ starts, int64_t count,
                                                              uint32_t * __restrict__ out) {
  __shared__ uint32_t buf[2][MT_N];
  int t = threadIdx.x;
  int64_t c = blockIdx.x;
  for (int w = t; w < MT_N; w += MT_THREADS) buf[0][w] = starts[c * MT_N + w];
  __syncthreads();
  int64_t twists = ceil_div(count, MT_N);
  int64_t k0 = c * MT_JUMP_TWISTS, k1 = k0 + MT_JUMP_TWISTS < twists ? k0 + MT_JUMP_TWISTS : twists;
  int cur = 0;
  for (int64_t k = k0; k < k1; ++k) {
    mt_twist_block(buf[cur], buf[cur ^ 1]);
    uint32_t const * Y = buf[cur ^ 1];
    int64_t base = k * MT_N;
    for (int j = t; j < MT_N; j += MT_THREADS)
      if (base + j < count) out[base + j] = mt_temper(Y[j]);
    cur ^= 1;
  }
}

__global__ void tri_area_kernel(float const * __restrict__ V, int32_t const * __restrict__ F, int64_t nf,
                                float * __restrict__ area) {
  int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  V3 v0 = load_v3(V + 3 * (int64_t)F[3 * f]);
  V3 v1 = load_v3(V + 3 * (int64_t)F[3 * f + 1]);
  V3 v2 = load_v3(V + 3 * (int64_t)F[3 * f + 2]);
  area[f] = tri_plane(v0, v1, v2).area;
}

// cum[i] = cum[i - 1] + area[i] in FP64, strictly in index order (MeshSampler.hpp:147-149, 166-169). One thread: the
// sequence of roundings is what makes the triangle choice bit-identical. Areas are staged through shared memory by the
// whole block so the serial chain only waits on shared-memory loads.
__global__ void serial_cdf_kernel(float const * __restrict__ area, int64_t nf, double * __restrict__ cum) {
  constexpr int CH = 2048;
  __shared__ float a[CH];
  __shared__ double c[CH];
  double run = 0.0;
  for (int64_t base = 0; base < nf; base += CH) {
    int m = (nf - base) < CH ? (int)(nf - base) : CH;
    for (int j = threadIdx.x; j < m; j += blockDim.x) a[j] = area[base + j];
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int j = 0; j < m; ++j) {
        run = (base + j == 0) ? (double)a[0] : run + (double)a[j];
        c[j] = run;
      }
    }
    __syncthreads();
    for (int j = threadIdx.x; j < m; j += blockDim.x) cum[base + j] = c[j];
    __syncthreads();
  }
}

// Parallel form of the same cumulative sum. A sum of FP32 values in an FP64 accumulator does not round as long as every
// running total fits in 53 significant bits, which holds for any mesh whose triangle areas are within a factor 2^29 of
// each other up to its size (each area has 24 significant bits, and the running total stays below 2^29 times the
// smallest of them). Then cum[i] is the exact prefix sum, which a parallel scan of the areas as 128-bit fixed-point
// integers (units of the smallest area's last bit) computes exactly. Every prefix is checked for exact representability
// in FP64; if one is not (areas spanning too many binades), the caller runs serial_cdf_kernel instead, so the result
// is always the sequential one bit for bit.
struct U128 {
  uint64_t lo, hi;
  U128() = default;
  __host__ __device__ constexpr U128(int v) : lo((uint64_t)(int64_t)v), hi(v < 0 ? ~0ull : 0ull) {}
};
__device__ __forceinline__ U128 operator+(U128 a, U128 b) {
  U128 r;
  r.lo = a.lo + b.lo;
  r.hi = a.hi + b.hi + (r.lo < a.lo ? 1ull : 0ull);
  return r;
}
__device__ __forceinline__ U128 operator-(U128 a, U128 b) {
  U128 r;
  r.lo = a.lo - b.lo;
  r.hi = a.hi - b.hi - (a.lo < b.lo ? 1ull : 0ull);
  return r;
}
__device__ __forceinline__ U128 & operator+=(U128 & a, U128 b) { return a = a + b; }
__device__ __forceinline__ U128 __shfl_up_sync(unsigned mask, U128 v, unsigned d) {
  v.lo = ::__shfl_up_sync(mask, v.lo, d);
  v.hi = ::__shfl_up_sync(mask, v.hi, d);
  return v;
}

// a = m * 2^e exactly (a >= 0 finite)
__device__ __forceinline__ void float_parts(float a, uint32_t & m, int & e) {
  uint32_t b = __float_as_uint(a);
  uint32_t ex = (b >> 23) & 0xffu, mt = b & 0x7fffffu;
  if (ex == 0) {
    m = mt;
    e = -149;
  } else {
    m = mt | 0x800000u;
    e = (int)ex - 150;
  }
}

// st[0] = smallest exponent of a nonzero area, st[1] = largest, st[2] = 1 if an area is negative, infinite or NaN
__global__ void cdf_init_kernel(int * st) {
  st[0] = INT_MAX;
  st[1] = INT_MIN;
  st[2] = 0;
}

__global__ void cdf_range_kernel(float const * __restrict__ area, int64_t nf, int * st) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int lo = INT_MAX, hi = INT_MIN, bad = 0;
  if (i < nf) {
    float a = area[i];
    if (!(a >= 0.f) || isinf(a)) {
      bad = 1;
    } else if (a > 0.f) {
      uint32_t m;
      int e;
      float_parts(a, m, e);
      lo = hi = e;
    }
  }
  for (int o = 16; o; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    bad |= __shfl_xor_sync(0xffffffffu, bad, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (lo != INT_MAX) atomicMin(st, lo);
    if (hi != INT_MIN) atomicMax(st + 1, hi);
    if (bad) atomicOr(st + 2, 1);
  }
}

// Largest spread of exponents for which 2^24-bit areas and up to 2^31 of them sum within 127 bits
constexpr int CDF_MAX_SPREAD = 127 - 24 - 31;

__global__ void cdf_fixed_kernel(float const * __restrict__ area, int64_t nf, int const * __restrict__ st,
                                 U128 * __restrict__ v) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nf) return;
  U128 r(0);
  int emin = st[0];
  if (!st[2] && st[1] - emin <= CDF_MAX_SPREAD) {
    float a = area[i];
    if (a > 0.f) {
      uint32_t m;
      int e;
      float_parts(a, m, e);
      int sh = e - emin;  // 0..CDF_MAX_SPREAD
      if (sh < 64) {
        r.lo = (uint64_t)m << sh;
        r.hi = sh == 0 ? 0ull : (uint64_t)m >> (64 - sh);
      } else {
        r.lo = 0;
        r.hi = (uint64_t)m << (sh - 64);
      }
    }
  }
  v[i] = r;
}

// cum[i] = (excl[i] + v[i]) * 2^emin, exactly; st[2] set if some total has more than 53 significant bits
__global__ void cdf_convert_kernel(U128 const * __restrict__ excl, U128 const * __restrict__ v, int64_t nf, int * st,
                                   double * __restrict__ cum) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nf) return;
  if (st[2] || st[1] - st[0] > CDF_MAX_SPREAD) {
    if (i == 0) st[2] = 1;
    return;
  }
  U128 x = excl[i] + v[i];
  if (x.lo == 0 && x.hi == 0) {
    cum[i] = 0.0;
    return;
  }
  int tz = x.lo ? __ffsll((long long)x.lo) - 1 : 64 + __ffsll((long long)x.hi) - 1;
  int bl = x.hi ? 128 - __clzll((long long)x.hi) : 64 - __clzll((long long)x.lo);
  if (bl - tz > 53) {
    atomicOr(st + 2, 1);
    return;
  }
  uint64_t mant;
  if (tz >= 64) mant = x.hi >> (tz - 64);
  else if (tz == 0) mant = x.lo;
  else mant = (x.lo >> tz) | (x.hi << (64 - tz));
  cum[i] = ldexp((double)mant, tz + st[0]);
}

// Philox-4x32-10 (Salmon, Moraes, Dror, Shaw: "Parallel random numbers: as easy as 1, 2, 3", SC'11)
__device__ __forceinline__ uint4 philox4x32_10(uint4 ctr, uint2 key) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0 = __umulhi(0xD2511F53u, ctr.x), lo0 = 0xD2511F53u * ctr.x;
    uint32_t hi1 = __umulhi(0xCD9E8D57u, ctr.z), lo1 = 0xCD9E8D57u * ctr.z;
    ctr = make_uint4(hi1 ^ ctr.y ^ key.x, lo1, hi0 ^ ctr.w ^ key.y, lo0);
    key.x += 0x9E3779B9u;
    key.y += 0xBB67AE85u;
  }
  return ctr;
}

__global__ void sample_kernel(float const * __restrict__ V, int32_t const * __restrict__ F, int64_t nf,
                              double const * __restrict__ cum, uint32_t const * __restrict__ words, uint32_t seed,
                              int64_t n, float * __restrict__ pos, float * __restrict__ nrm, int32_t * __restrict__ face) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t w0, w1, w2;
  if (words) {
    w0 = words[3 * i];
    w1 = words[3 * i + 1];
    w2 = words[3 * i + 2];
  } else {
    uint4 r = philox4x32_10(make_uint4((uint32_t)i, (uint32_t)(i >> 32), 0u, 0u), make_uint2(seed, 0x5EEDu));
    w0 = r.x; w1 = r.y; w2 = r.z;
  }
  // Random::uniform01(): (float)bits() * (1.0f / (float)0xFFFFFFFF), the factor being 2^-32
  float const NORM = 2.3283064365386963e-10f;
  double total = cum[nf - 1];
  double t = (double)(__uint2float_rn(w0) * NORM) * total;
  // std::lower_bound: first position whose value is not less than t, clamped to the last triangle
  int64_t lo = 0, len = nf;
  while (len > 0) {
    int64_t half = len >> 1;
    if (cum[lo + half] < t) { lo = lo + half + 1; len = len - half - 1; }
    else len = half;
  }
  int64_t tri = lo < nf - 1 ? lo : nf - 1;
  V3 v0 = load_v3(V + 3 * (int64_t)F[3 * tri]);
  V3 v1 = load_v3(V + 3 * (int64_t)F[3 * tri + 1]);
  V3 v2 = load_v3(V + 3 * (int64_t)F[3 * tri + 2]);
  V3 e01 = v1 - v0, e02 = v2 - v0;
  float s = __uint2float_rn(w1) * NORM;
  float u = __uint2float_rn(w2) * NORM;
  if (s + u > 1.f) {
    u = 1.f - u;
    s = 1.f - s;
  }
  V3 p = (s * e01 + u * e02) + v0;
  pos[3 * i] = p.x;
  pos[3 * i + 1] = p.y;
  pos[3 * i + 2] = p.z;
  if (nrm) {
    V3 nn = normalized(cross(e01, e02));
    nrm[3 * i] = nn.x;
    nrm[3 * i + 1] = nn.y;
    nrm[3 * i + 2] = nn.z;
  }
  if (face) face[i] = (int32_t)tri;
}

//============================================================================================================================
// Allocation-free sampling. Its scratch lives in one file-scope device array instead of the stream-ordered pool:
//   cum[]      FP64 cumulative areas, at most NOALLOC_MAX_FACES triangles (8 MiB)
//   mt_state[] the Mersenne-Twister state carried from one chunk of samples to the next (2.4 KiB)
//   words[]    the stream words of one chunk of NOALLOC_CHUNK samples (768 KiB)
// Chunks hold 65,520 samples = 196,560 words = 315 whole twists, so each chunk ends on a twist boundary and the next
// chunk resumes from the saved state with exactly the words the one-shot path would draw.
//============================================================================================================================

constexpr int64_t NOALLOC_CHUNK = 208 * 315;
static_assert((3 * NOALLOC_CHUNK) % MT_N == 0, "a chunk must consume whole twists");

struct NoAllocLayout {
  double cum[THEA_NOALLOC_MAX_FACES];
  uint32_t mt_state[MT_N];
  uint32_t words[3 * NOALLOC_CHUNK];
  int32_t bad_face;  // written by every noalloc_cdf_kernel launch: 1 if a face index lies outside [0, nv)
};

// Per-face areas computed in place (the same tri_plane arithmetic as tri_area_kernel) and summed in index order by one
// thread, exactly as serial_cdf_kernel does; no separate area array is needed. A face with an index outside [0, nv) is
// not loaded: it sets *bad_face (the caller then refuses the call) and counts as zero area.
__global__ void noalloc_cdf_kernel(float const * __restrict__ V, int64_t nv, int32_t const * __restrict__ F,
                                   int64_t nf, double * __restrict__ cum, int32_t * __restrict__ bad_face) {
  constexpr int CH = 2048;
  __shared__ float a[CH];
  __shared__ double c[CH];
  __shared__ int bad;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  double run = 0.0;
  for (int64_t base = 0; base < nf; base += CH) {
    int m = (nf - base) < CH ? (int)(nf - base) : CH;
    for (int j = threadIdx.x; j < m; j += blockDim.x) {
      int64_t f = base + j;
      int32_t i0 = F[3 * f], i1 = F[3 * f + 1], i2 = F[3 * f + 2];
      if (i0 < 0 || i1 < 0 || i2 < 0 || (int64_t)i0 >= nv || (int64_t)i1 >= nv || (int64_t)i2 >= nv) {
        bad = 1;
        a[j] = 0.f;
        continue;
      }
      V3 v0 = load_v3(V + 3 * (int64_t)i0);
      V3 v1 = load_v3(V + 3 * (int64_t)i1);
      V3 v2 = load_v3(V + 3 * (int64_t)i2);
      a[j] = tri_plane(v0, v1, v2).area;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int j = 0; j < m; ++j) {
        run = (base + j == 0) ? (double)a[0] : run + (double)a[j];
        c[j] = run;
      }
    }
    __syncthreads();
    for (int j = threadIdx.x; j < m; j += blockDim.x) cum[base + j] = c[j];
    __syncthreads();
  }
  if (threadIdx.x == 0) *bad_face = bad;
}

// Resumable form of thea_mt_stream_kernel: seeds the state when `first` is set, otherwise continues from `state`, and
// stores the state back after the last twist.
__global__ void __launch_bounds__(MT_THREADS) noalloc_mt_kernel(uint32_t seed, int first, uint32_t * __restrict__ state,
                                                                int64_t count, uint32_t * __restrict__ out) {
  __shared__ uint32_t s[MT_N];
  int t = threadIdx.x;
  if (first) {
    if (t == 0) {
      s[0] = seed;
      for (int i = 1; i < MT_N; ++i) s[i] = 1812433253u * (s[i - 1] ^ (s[i - 1] >> 30)) + (uint32_t)i;
    }
  } else {
    for (int j = t; j < MT_N; j += MT_THREADS) s[j] = state[j];
  }
  __syncthreads();
  int64_t twists = ceil_div(count, MT_N);
  for (int64_t k = 0; k < twists; ++k) {
    uint32_t v;
    if (t < MT_N - MT_M) v = mt_mix(s[t], s[t + 1], s[t + MT_M]);
    __syncthreads();
    if (t < MT_N - MT_M) s[t] = v;
    __syncthreads();
    int i = MT_N - MT_M + 1 + t;
    if (i < 2 * (MT_N - MT_M)) v = mt_mix(s[i], s[i + 1], s[i - (MT_N - MT_M)]);
    __syncthreads();
    if (i < 2 * (MT_N - MT_M)) s[i] = v;
    __syncthreads();
    i = 2 * (MT_N - MT_M) + t;
    if (i < MT_N - 1) v = mt_mix(s[i], s[i + 1], s[i - (MT_N - MT_M)]);
    else if (i == MT_N - 1) v = mt_mix(s[MT_N - 1], s[0], s[MT_M - 1]);
    __syncthreads();
    if (i < MT_N) s[i] = v;
    __syncthreads();
    int64_t base = k * MT_N;
    for (int j = t; j < MT_N; j += MT_THREADS)
      if (base + j < count) out[base + j] = mt_temper(s[j]);
  }
  __syncthreads();
  for (int j = t; j < MT_N; j += MT_THREADS) state[j] = s[j];
}

}  // namespace

// The scratch of every allocation-free call on a device. In host code the name is only a stand-in: its device address
// comes from cudaGetSymbolAddress (noalloc_scratch below).
static __device__ __align__(256) unsigned char g_sample_scratch[sizeof(NoAllocLayout)];

// Device address of g_sample_scratch on the current device, looked up once per device (with that device current) and
// cached; the lookup loads the library's module on the device if needed.
static NoAllocLayout * noalloc_scratch() {
  static std::mutex m;
  static NoAllocLayout * addr[256] = {};
  int dev = 0;
  THEA_CUDA_CHECK(cudaGetDevice(&dev));
  THEA_REQUIRE(dev >= 0 && dev < 256, "sample_by_area_noalloc: device ordinal out of range");
  std::lock_guard<std::mutex> lk(m);
  if (!addr[dev]) {
    void * p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_sample_scratch);
    if (e != cudaSuccess || !p)
      throw Error(THEA_ERR_CUDA, std::string("sample_by_area_noalloc: cudaGetSymbolAddress failed: ") +
                                     cudaGetErrorString(e));
    addr[dev] = static_cast<NoAllocLayout *>(p);
  }
  return addr[dev];
}

int64_t run_sample_by_area_noalloc(float const * V, int64_t nv, int32_t const * F, int64_t nf, int64_t n,
                                   uint32_t seed, int rng, float * pos, float * nrm, int32_t * face, cudaStream_t s) {
  THEA_REQUIRE(nf <= THEA_NOALLOC_MAX_FACES,
               "sample_by_area_noalloc: at most " + std::to_string((long long)THEA_NOALLOC_MAX_FACES) +
                   " triangles (got " + std::to_string((long long)nf) + ")");
  NoAllocLayout * scratch = noalloc_scratch();
  if (n <= 0 || nf <= 0) return 0;
  THEA_LAUNCH(noalloc_cdf_kernel, 1, 256, 0, s, V, nv, F, nf, scratch->cum, &scratch->bad_face);
  double total = 0.0;
  int32_t bad = 0;
  THEA_CUDA_CHECK(cudaMemcpyAsync(&total, scratch->cum + nf - 1, sizeof(double), cudaMemcpyDeviceToHost, s));
  THEA_CUDA_CHECK(cudaMemcpyAsync(&bad, &scratch->bad_face, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  THEA_CUDA_CHECK(cudaStreamSynchronize(s));
  THEA_REQUIRE(!bad, "sample_by_area_noalloc: a face index lies outside [0, num_vertices)");
  if (!(total > 0.0)) return 0;
  if (rng == THEA_RNG_COUNTER) {
    THEA_LAUNCH(sample_kernel, (unsigned)ceil_div(n, 256), 256, 0, s, V, F, nf, (double const *)scratch->cum,
                (uint32_t const *)nullptr, seed, n, pos, nrm, face);
    return n;
  }
  for (int64_t begin = 0; begin < n; begin += NOALLOC_CHUNK) {
    int64_t cnt = n - begin < NOALLOC_CHUNK ? n - begin : NOALLOC_CHUNK;
    THEA_LAUNCH(noalloc_mt_kernel, 1, MT_THREADS, 0, s, seed, begin == 0 ? 1 : 0, scratch->mt_state, 3 * cnt,
                scratch->words);
    THEA_LAUNCH(sample_kernel, (unsigned)ceil_div(cnt, 256), 256, 0, s, V, F, nf, (double const *)scratch->cum,
                (uint32_t const *)scratch->words, seed, cnt, pos + 3 * begin, nrm ? nrm + 3 * begin : nullptr,
                face ? face + begin : nullptr);
  }
  return n;
}

namespace {

// Streams of at least this many twists run as parallel chunks (below it one block is faster than the jump chain)
constexpr int64_t MT_PARALLEL_MIN_TWISTS = 2 * MT_JUMP_TWISTS;
constexpr int MT_APPLY_BLOCKS = 156;  // column slices of one jump (128 columns each)

// P = T^L per device, computed on the first long stream of the device (about 50 MB; kept for the process)
std::mutex g_jump_mu;
uint32_t * g_jump[64] = {nullptr};

uint32_t const * jump_matrix(cudaStream_t s) {
  int dev = 0;
  THEA_CUDA_CHECK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lk(g_jump_mu);
  if (g_jump[dev]) return g_jump[dev];
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  THEA_CUDA_CHECK(cudaStreamIsCapturing(s, &cap));
  if (cap != cudaStreamCaptureStatusNone) return nullptr;  // no allocation inside a capture: one block instead
  uint32_t * P = nullptr;
  THEA_CUDA_CHECK(thea_malloc((void **)&P, (size_t)MT_STATE_BITS * MT_N * sizeof(uint32_t)));
  THEA_LAUNCH(mt_jump_columns_kernel, MT_STATE_BITS, MT_THREADS, 0, s, P);
  THEA_CUDA_CHECK(cudaStreamSynchronize(s));
  g_jump[dev] = P;
  return P;
}

}  // namespace

void run_thea_random_words(uint32_t seed, int64_t count, uint32_t * out, cudaStream_t s) {
  if (count <= 0) return;
  int64_t twists = ceil_div(count, MT_N);
  uint32_t const * P = twists >= MT_PARALLEL_MIN_TWISTS ? jump_matrix(s) : nullptr;
  if (!P) {
    THEA_LAUNCH(thea_mt_stream_kernel, 1, MT_THREADS, 0, s, seed, count, out);
    return;
  }
  // start states of the chunks: the seeded state, then one jump (P times the previous start) per chunk
  int64_t chunks = ceil_div(twists, MT_JUMP_TWISTS);
  Scratch starts((size_t)chunks * MT_N * sizeof(uint32_t), s);
  uint32_t * st = starts.as<uint32_t>();
  THEA_CUDA_CHECK(cudaMemsetAsync(st, 0, starts.bytes, s));
  THEA_LAUNCH(mt_seed_kernel, 1, 32, 0, s, seed, st);
  int per = (int)ceil_div(MT_STATE_BITS, MT_APPLY_BLOCKS);
  for (int64_t c = 1; c < chunks; ++c)
    THEA_LAUNCH(mt_jump_apply_kernel, MT_APPLY_BLOCKS, MT_VEC_THREADS, 0, s, P, st + (c - 1) * MT_N, per,
                st + c * MT_N);
  THEA_LAUNCH(mt_chunk_kernel, (unsigned)chunks, MT_THREADS, 0, s, st, count, out);
}

int64_t run_sample_by_area(float const * V, int64_t nv, int32_t const * F, int64_t nf, int64_t n, uint32_t seed, int rng,
                           float * pos, float * nrm, int32_t * face, cudaStream_t s) {
  if (n <= 0 || nf <= 0) return 0;
  check_face_indices(F, nf, nv, "sample_by_area", s);
  Scratch area((size_t)nf * sizeof(float), s);
  Scratch cum((size_t)nf * sizeof(double), s);
  THEA_LAUNCH(tri_area_kernel, (unsigned)ceil_div(nf, 256), 256, 0, s, V, F, nf, area.as<float>());
  {
    // exact parallel cumulative areas; the serial kernel where they would not be exact
    Scratch st(4 * sizeof(int), s), fixed((size_t)nf * sizeof(U128), s), excl((size_t)nf * sizeof(U128), s);
    unsigned g = (unsigned)ceil_div(nf, 256);
    THEA_LAUNCH(cdf_init_kernel, 1, 1, 0, s, st.as<int>());
    THEA_LAUNCH(cdf_range_kernel, g, 256, 0, s, area.as<float>(), nf, st.as<int>());
    THEA_LAUNCH(cdf_fixed_kernel, g, 256, 0, s, area.as<float>(), nf, st.as<int>(), fixed.as<U128>());
    exclusive_scan<U128>(fixed.as<U128>(), excl.as<U128>(), nf, s);
    THEA_LAUNCH(cdf_convert_kernel, g, 256, 0, s, excl.as<U128>(), fixed.as<U128>(), nf, st.as<int>(),
                cum.as<double>());
    int flag = 0;
    THEA_CUDA_CHECK(cudaMemcpyAsync(&flag, st.as<int>() + 2, sizeof(int), cudaMemcpyDeviceToHost, s));
    THEA_CUDA_CHECK(cudaStreamSynchronize(s));
    if (flag) THEA_LAUNCH(serial_cdf_kernel, 1, 256, 0, s, area.as<float>(), nf, cum.as<double>());
  }
  double total = 0.0;
  THEA_CUDA_CHECK(cudaMemcpyAsync(&total, cum.as<double>() + nf - 1, sizeof(double), cudaMemcpyDeviceToHost, s));
  THEA_CUDA_CHECK(cudaStreamSynchronize(s));
  if (!(total > 0.0)) return 0;  // MeshSampler returns no samples for a zero-area mesh
  Scratch words;
  if (rng == THEA_RNG_THEA_MT) {
    words = Scratch((size_t)n * 3 * sizeof(uint32_t), s);
    run_thea_random_words(seed, 3 * n, words.as<uint32_t>(), s);
  }
  THEA_LAUNCH(sample_kernel, (unsigned)ceil_div(n, 256), 256, 0, s, V, F, nf, cum.as<double>(), words.as<uint32_t>(),
              seed, n, pos, nrm, face);
  return n;
}

}  // namespace thea
