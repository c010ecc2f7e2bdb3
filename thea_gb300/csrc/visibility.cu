// Any-hit ray queries and the Visibility surface feature.
//
// rayIntersects (BvhN.hpp:1266-1269) is rayIntersectionTime >= 0: whether any element has a hit time in [0, max_time].
// The first-hit kernel answers it too, but an occlusion query can stop at the first accepted element: the any-hit
// kernel here is the persistent-lane loop of the first-hit kernel with a fixed bound (max_time, or +inf) and an exit on
// the first hit. Nearest-first child order is kept (hits tend to lie in near boxes).
//
// Visibility::compute (SurfaceFeatures/Local/Visibility.hpp:104-126) casts, from a point on the surface, rays along
// num_rays directions of Random::common().sphere() from origins pushed out by 0.001 * scale along the direction, and
// returns the fraction of rays with no hit. Random::common() is a process-wide generator; here Random(seed) takes its
// place so that the result is reproducible: point i uses directions [i * num_rays, (i + 1) * num_rays) of the stream.
// Random::sphere (Random.cpp:225-250, Knop's method) draws x = 2 u - 1, y = 2 u - 1 until 1e-10 <= x² + y² <= 1, each
// attempt consuming two uniforms, so the accepted directions are the accepted attempts of the pairwise-grouped uniform
// stream in order: attempts are evaluated in parallel and compacted with a scan.
#include "visibility.hpp"

#include "device_util.cuh"
#include "query.hpp"
#include "transform.hpp"
#include "traverse_ops.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace thea {
namespace {

constexpr int ANY_THREADS = 128;
constexpr int ANY_WARP_BLOCK = 64;
constexpr int SPHERE_THREADS = 256;

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

// Visibility rays: ray r starts at point r / num_rays pushed out along direction r (world space, then mapped)
struct VisibilityRays {
  float const * pos;
  float const * dirs;
  int num_rays;
  float off;  // 0.001f * scale
  Inverse inv;
  __device__ __forceinline__ void get(int64_t r, V3 & ro, V3 & rd) const {
    int64_t i = r / num_rays;
    V3 u = load_v3(dirs + 3 * r);
    V3 p = load_v3(pos + 3 * i);
    // Vector3 offset = 0.001f * scale * u; Ray3(position + offset, u)
    ro = p + off * u;
    rd = u;
    if (inv.on) {
      ro = affine_point(inv.m, ro);
      rd = affine_vector(inv.m, rd);
    }
  }
};

struct EscapeCounts {
  unsigned * count;
  int num_rays;
  __device__ __forceinline__ void put(int64_t r, bool hit) const {
    if (!hit) atomicAdd(count + r / num_rays, 1u);
  }
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

// Attempt a of Random::sphere: uniforms 2a and 2a + 1 of the stream
__device__ __forceinline__ bool sphere_attempt(uint32_t const * __restrict__ words, int64_t a, float & x, float & y,
                                               float & m2) {
  float const NORM = 2.3283064365386963e-10f;  // Random::uniform01: (float)bits() * (1.0f / (float)0xFFFFFFFF)
  x = 2.f * (__uint2float_rn(words[2 * a]) * NORM) - 1.f;
  y = 2.f * (__uint2float_rn(words[2 * a + 1]) * NORM) - 1.f;
  m2 = x * x + y * y;
  return !(m2 > 1.f || (double)m2 < 1e-10);  // the reference compares with the double literal 1e-10
}

__global__ void sphere_accept_kernel(uint32_t const * __restrict__ words, int64_t attempts, uint32_t * __restrict__ flag) {
  int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= attempts) return;
  float x, y, m2;
  flag[a] = sphere_attempt(words, a, x, y, m2) ? 1u : 0u;
}

__global__ void sphere_emit_kernel(uint32_t const * __restrict__ words, int64_t attempts,
                                   uint32_t const * __restrict__ slot, int64_t count, float * __restrict__ dirs) {
  int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= attempts) return;
  float x, y, m2;
  if (!sphere_attempt(words, a, x, y, m2)) return;
  int64_t j = slot[a];
  if (j >= count) return;
  float z = 2.f * m2 - 1.f;
  float sc = 2.f * sqrtf(1.f - m2);
  dirs[3 * j] = x * sc;
  dirs[3 * j + 1] = y * sc;
  dirs[3 * j + 2] = z;
}

__global__ void fraction_kernel(unsigned const * __restrict__ escaped, int64_t n, int num_rays,
                                double * __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (double)escaped[i] / (double)num_rays;
}

}  // namespace

void run_ray_intersects(thea_bvh const * b, float const * o, float const * d, int64_t n, float max_time, uint8_t * hit,
                        cudaStream_t s) {
  if (n <= 0) return;
  dispatch_any(b, RayArrays{o, d, inverse_of(b)}, HitFlags{hit}, n, max_time, s);
}

void run_random_sphere(uint32_t seed, int64_t count, float * dirs, cudaStream_t s) {
  if (count <= 0) return;
  // accepted with probability pi/4 per attempt; draw enough attempts for `count` with a wide margin, and more if short
  int64_t attempts = count + count / 3 + 64 + 16 * (int64_t)std::sqrt((double)count);
  THEA_REQUIRE(attempts < ((int64_t)1 << 32), "random_sphere: too many directions for one call");
  while (true) {
    Scratch words((size_t)attempts * 8, s), slot((size_t)attempts * 4, s);
    run_thea_random_words(seed, 2 * attempts, words.as<uint32_t>(), s);
    unsigned grid = (unsigned)ceil_div(attempts, SPHERE_THREADS);
    THEA_LAUNCH(sphere_accept_kernel, grid, SPHERE_THREADS, 0, s, words.as<uint32_t>(), attempts, slot.as<uint32_t>());
    uint32_t last_flag = 0, last_slot = 0;
    THEA_CUDA_CHECK(cudaMemcpyAsync(&last_flag, slot.as<uint32_t>() + attempts - 1, 4, cudaMemcpyDeviceToHost, s));
    exclusive_scan<uint32_t>(slot.as<uint32_t>(), slot.as<uint32_t>(), attempts, s);
    THEA_CUDA_CHECK(cudaMemcpyAsync(&last_slot, slot.as<uint32_t>() + attempts - 1, 4, cudaMemcpyDeviceToHost, s));
    THEA_CUDA_CHECK(cudaStreamSynchronize(s));
    if ((int64_t)last_slot + last_flag >= count) {
      THEA_LAUNCH(sphere_emit_kernel, grid, SPHERE_THREADS, 0, s, words.as<uint32_t>(), attempts, slot.as<uint32_t>(),
                  count, dirs);
      return;
    }
    attempts *= 2;
    THEA_REQUIRE(attempts < ((int64_t)1 << 32), "random_sphere: too many directions for one call");
  }
}

float visibility_scale(thea_bvh const * b) {
  // AxisAlignedBoxN::scaleCentered(1.05): c = 0.5 (hi + lo); lo' = 1.05 (lo - c) + c; hi' likewise
  float const F = 1.05f;
  float lo[3], hi[3];
  for (int a = 0; a < 3; ++a) {
    float c = 0.5f * (b->hi[a] + b->lo[a]);
    lo[a] = F * (b->lo[a] - c) + c;
    hi[a] = F * (b->hi[a] - c) + c;
  }
  if (b->has_transform) {
    // getBounds() of a transformed BVH: the box of the eight mapped corners (AxisAlignedBoxN::transformAndBound)
    float wl[3] = {INFINITY, INFINITY, INFINITY}, wh[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int c = 0; c < 8; ++c) {
      V3 w = affine_point(b->xf, V3{(c & 1) ? hi[0] : lo[0], (c & 2) ? hi[1] : lo[1], (c & 4) ? hi[2] : lo[2]});
      float wc[3] = {w.x, w.y, w.z};
      for (int a = 0; a < 3; ++a) wl[a] = std::min(wl[a], wc[a]), wh[a] = std::max(wh[a], wc[a]);
    }
    for (int a = 0; a < 3; ++a) lo[a] = wl[a], hi[a] = wh[a];
  }
  // getExtent().norm()
  float e[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
  return std::sqrt(e[0] * e[0] + (e[1] * e[1] + e[2] * e[2]));
}

void run_visibility(thea_bvh const * b, float const * positions, int64_t n, int num_rays, uint32_t seed,
                    double * fraction, cudaStream_t s) {
  if (n <= 0) return;
  int64_t total = n * (int64_t)num_rays;
  Scratch dirs((size_t)total * 12, s), escaped((size_t)n * 4, s);
  run_random_sphere(seed, total, dirs.as<float>(), s);
  THEA_CUDA_CHECK(cudaMemsetAsync(escaped.ptr, 0, (size_t)n * 4, s));
  float off = 0.001f * visibility_scale(b);
  dispatch_any(b, VisibilityRays{positions, dirs.as<float>(), num_rays, off, inverse_of(b)},
               EscapeCounts{escaped.as<unsigned>(), num_rays}, total, -1.f, s);
  THEA_LAUNCH(fraction_kernel, (unsigned)ceil_div(n, 256), 256, 0, s, escaped.as<unsigned>(), n, num_rays, fraction);
  THEA_CUDA_CHECK(cudaStreamSynchronize(s));
}

}  // namespace thea
