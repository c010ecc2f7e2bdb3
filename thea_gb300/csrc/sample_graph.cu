// Sample proximity graph: PointSet3::updateGraph (Algorithms/PointSet3.hpp:324-391) without oversampling, with
// findSampleNeighbors and NeighborFunctor (PointSet3.hpp:586-681) and updateAverageSeparation (:688-702).
//
// The reference estimates the mean sample separation from 100 samples drawn with Random::common().integer(0, n - 1);
// Random(seed) takes its place here so that the graph is reproducible. Every other step is deterministic: each sample
// keeps the max_degree smallest (separation, index) pairs among its valid candidates (SamplePoint3's bounded sorted
// neighbour set orders by separation, then by sample address, i.e. array index), which does not depend on the order
// in which the range query visits them.
//
// GPU form, per radius round (at most three, doubling the radius for samples with fewer than min_degree neighbours):
// a radius query of the active samples gives candidate pairs (CSR); one thread per pair applies the angle test and
// computes the separation (Math::fastSqrt: the one-step inverse-square-root approximation); the reachability rays of
// all pairs go through the any-hit kernel; one thread per sample then selects its neighbours.
#include "sample_graph.hpp"

#include "any_hit.cuh"
#include "device_util.cuh"
#include "query.hpp"
#include "running_sum.cuh"
#include "traverse_ops.cuh"

#include <cmath>
#include <vector>

namespace thea {
namespace {

constexpr int GRAPH_THREADS = 256;
constexpr int MAX_GRAPH_DEGREE = 64;

// Math::fastRsq (Math.hpp:193-208): one Newton step from the 0x5f3759df estimate; Math::fastSqrt = 1 / fastRsq
__device__ __forceinline__ float fast_sqrt(float x) {
  float x2 = x * 0.5f;
  int i = 0x5f3759df - (__float_as_int(x) >> 1);
  float y = __int_as_float(i);
  y = y * (1.5f - ((x2 * y) * y));
  return 1.0f / y;
}

__global__ void gather_kernel(float const * __restrict__ p, int32_t const * __restrict__ ids, int64_t n,
                              float * __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int64_t j = ids[i];
  out[3 * i] = p[3 * j];
  out[3 * i + 1] = p[3 * j + 1];
  out[3 * i + 2] = p[3 * j + 2];
}

__global__ void owner_kernel(int64_t const * __restrict__ off, int64_t n, int32_t * __restrict__ owner) {
  int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n) return;
  for (int64_t p = off[a]; p < off[a + 1]; ++p) owner[p] = (int32_t)a;
}

// NeighborFunctor::isValidNeighbor up to the reachability test: identity (excluded by the range query), angle,
// separation
__global__ void pair_kernel(float const * __restrict__ pos, float const * __restrict__ nrm,
                            int32_t const * __restrict__ active, int32_t const * __restrict__ owner,
                            int32_t const * __restrict__ cand, int64_t total, float * __restrict__ sep,
                            uint8_t * __restrict__ ok) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= total) return;
  int64_t s = active[owner[p]], j = cand[p];
  bool valid = true;
  if (nrm) valid = !(dot(load_v3(nrm + 3 * s), load_v3(nrm + 3 * j)) < -0.5f);  // MIN_DOT
  V3 diff = load_v3(pos + 3 * j) - load_v3(pos + 3 * s);
  sep[p] = fast_sqrt(squared_norm(diff));
  ok[p] = valid ? 1 : 0;
}

// Reachability rays: from the sample lifted by 5 * separation along the normalised normal sum, along the difference,
// bounded by time 1 (the segment between the lifted points)
struct ReachRays {
  float const * pos;
  float const * nrm;
  int32_t const * active;
  int32_t const * owner;
  int32_t const * cand;
  float const * sep;
  Inverse inv;
  __device__ __forceinline__ void get(int64_t p, V3 & o, V3 & d) const {
    int64_t s = active[owner[p]], j = cand[p];
    V3 ps = load_v3(pos + 3 * s);
    V3 lift = normalized(load_v3(nrm + 3 * s) + load_v3(nrm + 3 * j));
    o = ps + (5.0f * sep[p]) * lift;  // LIFT_FACTOR * sep * lift_dir
    d = load_v3(pos + 3 * j) - ps;
    if (inv.on) {
      o = affine_point(inv.m, o);
      d = affine_vector(inv.m, d);
    }
  }
};

struct BlockedFlags {
  uint8_t * ok;
  __device__ __forceinline__ void put(int64_t p, bool hit) const {
    if (hit) ok[p] = 0;
  }
};

// Per active sample: the max_degree smallest (separation, index) among valid candidates; final if at least min_degree
// (or in the last round), else the sample goes to the next round
__global__ void select_kernel(int32_t const * __restrict__ active, int64_t n_active, int64_t const * __restrict__ off,
                              int32_t const * __restrict__ cand, float const * __restrict__ sep,
                              uint8_t const * __restrict__ ok, int max_degree, int min_degree, int last,
                              int32_t * __restrict__ out_nbr, float * __restrict__ out_sep,
                              int32_t * __restrict__ out_deg, uint8_t * __restrict__ again) {
  int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n_active) return;
  float bs[MAX_GRAPH_DEGREE];
  int bi[MAX_GRAPH_DEGREE];
  int cnt = 0;
  for (int64_t p = off[a]; p < off[a + 1]; ++p) {
    if (!ok[p]) continue;
    float v = sep[p];
    int j = cand[p];
    if (cnt == max_degree && !(v < bs[cnt - 1] || (v == bs[cnt - 1] && j < bi[cnt - 1]))) continue;
    int k = cnt < max_degree ? cnt++ : cnt - 1;
    while (k > 0 && (v < bs[k - 1] || (v == bs[k - 1] && j < bi[k - 1]))) {
      bs[k] = bs[k - 1];
      bi[k] = bi[k - 1];
      --k;
    }
    bs[k] = v;
    bi[k] = j;
  }
  bool fin = cnt >= min_degree || last;
  again[a] = fin ? 0 : 1;
  if (!fin) return;
  int64_t s = active[a];
  for (int k = 0; k < max_degree; ++k) {
    out_nbr[s * max_degree + k] = k < cnt ? bi[k] : -1;
    if (out_sep) out_sep[s * max_degree + k] = k < cnt ? bs[k] : 0.f;
  }
  if (out_deg) out_deg[s] = cnt;
}

// extractOriginalAdjacencies (PointSet3.cpp:157-176, DijkstraCallback :131-148): for each original sample, Dijkstra
// over the graph of all samples (originals first, then the oversampling), edge lengths the separations held in double,
// until max_degree original samples other than itself are settled; their path lengths, rounded to Real, are the new
// separations. One warp per original sample: the settled and tentative vertices live in a shared-memory hash table
// (EXTRACT_SLOTS per warp); each step the warp finds the smallest tentative (distance, index), settles it and relaxes its
// edges, one lane per edge. Ties settle the lowest index first (the reference's Fibonacci heap breaks them by its own
// internal order). A search that would outgrow the table raises `flag` and stops.
constexpr int EXTRACT_WARPS = 2;
constexpr int EXTRACT_SLOTS = 1024;  // power of two
constexpr int EXTRACT_FILL = EXTRACT_SLOTS - 2 * MAX_GRAPH_DEGREE;

__device__ __forceinline__ int extract_slot(int v) { return (int)(((uint32_t)v * 2654435761u) >> 22); }

__global__ void __launch_bounds__(EXTRACT_WARPS * 32)
extract_kernel(int32_t const * __restrict__ nbr, float const * __restrict__ sep, int32_t const * __restrict__ deg,
               int m, int64_t n_orig, int32_t * __restrict__ out_nbr, float * __restrict__ out_sep,
               int32_t * __restrict__ out_deg, unsigned * __restrict__ flag) {
  __shared__ int s_vert[EXTRACT_WARPS][EXTRACT_SLOTS];
  __shared__ double s_dist[EXTRACT_WARPS][EXTRACT_SLOTS];
  __shared__ unsigned char s_done[EXTRACT_WARPS][EXTRACT_SLOTS];
  __shared__ int s_idx[EXTRACT_WARPS][MAX_GRAPH_DEGREE];
  __shared__ float s_sep[EXTRACT_WARPS][MAX_GRAPH_DEGREE];
  int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int64_t src = (int64_t)blockIdx.x * EXTRACT_WARPS + w;
  if (src >= n_orig) return;  // the whole warp
  int * vert = s_vert[w];
  double * dist = s_dist[w];
  unsigned char * done = s_done[w];
  for (int k = lane; k < EXTRACT_SLOTS; k += 32) {
    vert[k] = -1;
    done[k] = 0;
  }
  __syncwarp();
  if (lane == 0) {
    int h = extract_slot((int)src);
    vert[h] = (int)src;
    dist[h] = 0.0;
  }
  __syncwarp();
  int found = 0, used = 1;
  bool full = false;
  while (true) {
    double bd = INFINITY;
    int bv = INT_MAX, bs = -1;
    for (int k = lane; k < EXTRACT_SLOTS; k += 32) {
      int v = vert[k];
      if (v < 0 || done[k]) continue;
      double d = dist[k];
      if (d < bd || (d == bd && v < bv)) bd = d, bv = v, bs = k;
    }
    for (int o = 16; o; o >>= 1) {
      double od = __shfl_xor_sync(0xffffffffu, bd, o);
      int ov = __shfl_xor_sync(0xffffffffu, bv, o), os = __shfl_xor_sync(0xffffffffu, bs, o);
      if (os >= 0 && (bs < 0 || od < bd || (od == bd && ov < bv))) bd = od, bv = ov, bs = os;
    }
    if (bs < 0) break;  // the component is exhausted
    if (lane == 0) done[bs] = 1;
    if (bv != (int)src && bv < n_orig) {
      if (lane == 0) {
        s_idx[w][found] = bv;
        s_sep[w][found] = (float)bd;
      }
      if (++found >= m) break;
    }
    int dv = deg[bv];
    if (used + dv > EXTRACT_FILL) {
      full = true;
      break;
    }
    bool inserted = false;
    if (lane < dv) {  // dv <= max_degree <= 64: at most two edges per lane
      for (int k = lane; k < dv; k += 32) {
        int u = nbr[(int64_t)bv * m + k];
        double nd = bd + (double)sep[(int64_t)bv * m + k];
        int h = extract_slot(u);
        for (int probe = 0; probe < EXTRACT_SLOTS; ++probe) {
          int prev = atomicCAS(&vert[h], -1, u);
          if (prev == -1) {
            dist[h] = nd;
            inserted = true;
            break;
          }
          if (prev == u) {
            if (!done[h] && nd < dist[h]) dist[h] = nd;
            break;
          }
          h = (h + 1) & (EXTRACT_SLOTS - 1);
        }
      }
    }
    // each lane inserts at most two vertices: count them all
    used += __popc(__ballot_sync(0xffffffffu, inserted)) * (dv > 32 ? 2 : 1);
    __syncwarp();
  }
  __syncwarp();
  if (lane == 0) {
    // the neighbour set's order: (separation, index)
    for (int a = 1; a < found; ++a) {
      int ia = s_idx[w][a];
      float sa = s_sep[w][a];
      int b = a - 1;
      while (b >= 0 && (s_sep[w][b] > sa || (s_sep[w][b] == sa && s_idx[w][b] > ia))) {
        s_idx[w][b + 1] = s_idx[w][b];
        s_sep[w][b + 1] = s_sep[w][b];
        --b;
      }
      s_idx[w][b + 1] = ia;
      s_sep[w][b + 1] = sa;
    }
    for (int k = 0; k < m; ++k) {
      out_nbr[src * m + k] = k < found ? s_idx[w][k] : -1;
      if (out_sep) out_sep[src * m + k] = k < found ? s_sep[w][k] : 0.f;
    }
    if (out_deg) out_deg[src] = found;
    if (full) atomicOr(flag, 1u);
  }
}

// Candidate rows (CAND_ROW per sample, the first off[a + 1] - off[a] used) -> CSR
constexpr int CAND_ROW = 64;

__global__ void rows_to_csr_kernel(int32_t const * __restrict__ rows, int64_t const * __restrict__ off, int64_t n,
                                   int32_t * __restrict__ cand) {
  int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n) return;
  int64_t o = off[a], c = off[a + 1] - o;
  for (int64_t k = 0; k < c; ++k) cand[o + k] = rows[a * CAND_ROW + k];
}

// Round 0's active list: every sample
__global__ void iota_kernel(int32_t * __restrict__ out, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (int32_t)i;
}

__global__ void flags_to_int_kernel(uint8_t const * __restrict__ f, int64_t n, int32_t * __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = f[i] ? 1 : 0;
}

// The samples to retry, in their order, and their count
__global__ void compact_active_kernel(int32_t const * __restrict__ act, uint8_t const * __restrict__ again,
                                      int32_t const * __restrict__ pos, int64_t n, int32_t * __restrict__ next,
                                      int64_t * __restrict__ count) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (again[i]) next[pos[i]] = act[i];
  if (i == n - 1) *count = (int64_t)pos[i] + (again[i] ? 1 : 0);
}

}  // namespace

void run_sample_graph(float const * positions, float const * normals, int64_t n, int max_degree, uint32_t seed,
                      thea_bvh const * surface, SampleGraphOut & out, cudaStream_t s) {
  THEA_REQUIRE(n >= 2, "sample_graph: at least two samples are needed");
  THEA_REQUIRE(n < ((int64_t)1 << 31), "sample_graph: too many samples");
  THEA_REQUIRE(max_degree >= 1 && max_degree <= MAX_GRAPH_DEGREE, "sample_graph: max_degree must be in 1..64");
  thea_build_config cfg{};
  cfg.width = 4;
  thea_bvh * pts = build_bvh(false, positions, n, nullptr, 0, cfg, s);
  try {
    // mean separation estimate (RMS nearest-neighbour distance of num_trials samples drawn by Random::integer)
    int64_t trials = std::min<int64_t>(100, n);
    std::vector<uint32_t> words((size_t)trials);
    {
      Scratch w((size_t)trials * 4, s);
      run_thea_random_words(seed, trials, w.as<uint32_t>(), s);
      THEA_CUDA_CHECK(cudaMemcpyAsync(words.data(), w.ptr, (size_t)trials * 4, cudaMemcpyDeviceToHost, s));
      THEA_CUDA_CHECK(cudaStreamSynchronize(s));
    }
    std::vector<int32_t> tid((size_t)trials);
    int32_t hi = (int32_t)n - 1;
    for (int64_t t = 0; t < trials; ++t) {
      // Random::integer(low, high) (Random.cpp:147-157)
      int32_t r = (int32_t)std::floor(0 + (hi - 0 + 1) * (double)words[(size_t)t] / 0xFFFFFFFFUL);
      tid[(size_t)t] = r > hi ? hi : r;
    }
    std::vector<float> nd2((size_t)trials);
    {
      Scratch ids((size_t)trials * 4, s), q((size_t)trials * 12, s), ki((size_t)trials * 4, s), kd((size_t)trials * 4, s);
      THEA_CUDA_CHECK(cudaMemcpyAsync(ids.ptr, tid.data(), (size_t)trials * 4, cudaMemcpyHostToDevice, s));
      THEA_LAUNCH(gather_kernel, (unsigned)ceil_div(trials, GRAPH_THREADS), GRAPH_THREADS, 0, s, positions,
                  ids.as<int32_t>(), trials, q.as<float>());
      run_knn(pts, q.as<float>(), trials, 1, INFINITY, ids.as<int32_t>(), ki.as<int32_t>(), kd.as<float>(), pts->err,
              s);
      THEA_CUDA_CHECK(cudaMemcpyAsync(nd2.data(), kd.ptr, (size_t)trials * 4, cudaMemcpyDeviceToHost, s));
      THEA_CUDA_CHECK(cudaStreamSynchronize(s));
    }
    float avg = 0.f;
    for (int64_t t = 0; t < trials; ++t) avg += nd2[(size_t)t];
    avg = std::sqrt(avg / (float)trials);
    out.avg_separation_estimate = avg;

    float radius = std::sqrt((float)max_degree) * avg;
    int d4 = (int)(0.25 * max_degree);
    int min_degree = d4 < 4 ? 4 : (d4 > max_degree ? max_degree : d4);  // Math::clamp(x, 4, max_degree)
    bool reach = surface && normals;
    // round 0: every sample; later rounds: the samples that found fewer than min_degree neighbours, compacted on the
    // device in order (only their count comes back to the host)
    Scratch act_a((size_t)n * 4, s), act_b((size_t)n * 4, s), pos((size_t)n * 4, s), cnt(8, s);
    int32_t * act = act_a.as<int32_t>();
    int32_t * nxt = act_b.as<int32_t>();
    THEA_LAUNCH(iota_kernel, (unsigned)ceil_div(n, GRAPH_THREADS), GRAPH_THREADS, 0, s, act, n);
    int64_t na = n;
    for (int round = 0; round < 3 && na > 0; ++round, radius *= 2.0f) {
      bool last = round == 2;
      Scratch q((size_t)na * 12, s), off((size_t)(na + 1) * 8, s), again((size_t)na, s);
      int32_t const * ids = act;
      THEA_LAUNCH(gather_kernel, (unsigned)ceil_div(na, GRAPH_THREADS), GRAPH_THREADS, 0, s, positions,
                  ids, na, q.as<float>());
      // candidates: Ball3(position, radius), the sample itself excluded (the identity test); one traversal counts them
      // and keeps up to CAND_ROW per sample, a second one runs only if a sample has more
      Scratch rows((size_t)na * CAND_ROW * 4, s), over(sizeof(unsigned), s);
      THEA_CUDA_CHECK(cudaMemsetAsync(over.ptr, 0, sizeof(unsigned), s));
      run_range_rows(pts, q.as<float>(), na, radius, ids, off.as<int64_t>(), rows.as<int32_t>(), CAND_ROW,
                     over.as<unsigned>(), pts->err, s);
      struct {
        int64_t total;
        unsigned over;
      } h{0, 0};
      THEA_CUDA_CHECK(cudaMemcpyAsync(&h.total, off.as<int64_t>() + na, 8, cudaMemcpyDeviceToHost, s));
      THEA_CUDA_CHECK(cudaMemcpyAsync(&h.over, over.ptr, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
      THEA_CUDA_CHECK(cudaStreamSynchronize(s));
      int64_t total = h.total;
      Scratch cand((size_t)std::max<int64_t>(total, 1) * 4, s), owner((size_t)std::max<int64_t>(total, 1) * 4, s);
      Scratch sep((size_t)std::max<int64_t>(total, 1) * 4, s), ok((size_t)std::max<int64_t>(total, 1), s);
      if (total > 0) {
        // the selection keeps the smallest (separation, index) pairs whatever the order of a sample's candidates
        if (h.over)
          run_range(pts, q.as<float>(), na, radius, ids, off.as<int64_t>(), cand.as<int32_t>(), nullptr,
                    pts->err, s, false);
        else
          THEA_LAUNCH(rows_to_csr_kernel, (unsigned)ceil_div(na, GRAPH_THREADS), GRAPH_THREADS, 0, s,
                      rows.as<int32_t>(), off.as<int64_t>(), na, cand.as<int32_t>());
        THEA_LAUNCH(owner_kernel, (unsigned)ceil_div(na, GRAPH_THREADS), GRAPH_THREADS, 0, s, off.as<int64_t>(), na,
                    owner.as<int32_t>());
        THEA_LAUNCH(pair_kernel, (unsigned)ceil_div(total, GRAPH_THREADS), GRAPH_THREADS, 0, s, positions, normals,
                    ids, owner.as<int32_t>(), cand.as<int32_t>(), total, sep.as<float>(),
                    ok.as<uint8_t>());
        if (reach)
          dispatch_any(surface,
                       ReachRays{positions, normals, ids, owner.as<int32_t>(), cand.as<int32_t>(),
                                 sep.as<float>(), inverse_of(surface)},
                       BlockedFlags{ok.as<uint8_t>()}, total, 1.0f, s);
      }
      THEA_LAUNCH(select_kernel, (unsigned)ceil_div(na, GRAPH_THREADS), GRAPH_THREADS, 0, s, ids, na,
                  off.as<int64_t>(), cand.as<int32_t>(), sep.as<float>(), ok.as<uint8_t>(), max_degree, min_degree,
                  last ? 1 : 0, out.neighbors, out.separations, out.degree, again.as<uint8_t>());
      if (last) break;
      unsigned g = (unsigned)ceil_div(na, GRAPH_THREADS);
      THEA_LAUNCH(flags_to_int_kernel, g, GRAPH_THREADS, 0, s, again.as<uint8_t>(), na, pos.as<int32_t>());
      exclusive_scan<int32_t>(pos.as<int32_t>(), pos.as<int32_t>(), na, s);
      THEA_LAUNCH(compact_active_kernel, g, GRAPH_THREADS, 0, s, act, again.as<uint8_t>(), pos.as<int32_t>(), na, nxt,
                  cnt.as<int64_t>());
      int64_t next_count = 0;
      THEA_CUDA_CHECK(cudaMemcpyAsync(&next_count, cnt.ptr, 8, cudaMemcpyDeviceToHost, s));
      THEA_CUDA_CHECK(cudaStreamSynchronize(s));
      std::swap(act, nxt);
      na = next_count;
    }
  } catch (...) {
    cudaStreamSynchronize(s);
    destroy_bvh(pts);
    throw;
  }
  THEA_CUDA_CHECK(cudaStreamSynchronize(s));
  destroy_bvh(pts);
}

}  // namespace thea

namespace thea {

void run_sample_graph_oversampled(float const * positions, float const * normals, int64_t n, float const * dense,
                                  float const * dense_normals, int64_t n_dense, int max_degree, uint32_t seed,
                                  thea_bvh const * surface, SampleGraphOut & out, cudaStream_t s) {
  THEA_REQUIRE(n >= 1 && n_dense >= 1, "sample_graph: oversampling needs samples and dense samples");
  THEA_REQUIRE(n + n_dense < ((int64_t)1 << 31), "sample_graph: too many samples");
  THEA_REQUIRE(max_degree >= 1 && max_degree <= MAX_GRAPH_DEGREE, "sample_graph: max_degree must be in 1..64");
  int64_t na = n + n_dense;
  size_t m = (size_t)max_degree;
  // the aggregate: originals first, then the oversampling (updateGraph's sample_ptrs order)
  Scratch agg((size_t)na * 12, s), aggn(normals ? (size_t)na * 12 : 0, s);
  THEA_CUDA_CHECK(cudaMemcpyAsync(agg.ptr, positions, (size_t)n * 12, cudaMemcpyDeviceToDevice, s));
  THEA_CUDA_CHECK(cudaMemcpyAsync(agg.as<float>() + 3 * n, dense, (size_t)n_dense * 12, cudaMemcpyDeviceToDevice, s));
  if (normals) {
    THEA_CUDA_CHECK(cudaMemcpyAsync(aggn.ptr, normals, (size_t)n * 12, cudaMemcpyDeviceToDevice, s));
    THEA_CUDA_CHECK(cudaMemcpyAsync(aggn.as<float>() + 3 * n, dense_normals, (size_t)n_dense * 12,
                                    cudaMemcpyDeviceToDevice, s));
  }
  Scratch gn((size_t)na * m * 4, s), gs((size_t)na * m * 4, s), gd((size_t)na * 4, s);
  SampleGraphOut g;
  g.neighbors = gn.as<int32_t>();
  g.separations = gs.as<float>();
  g.degree = gd.as<int32_t>();
  run_sample_graph(agg.as<float>(), normals ? aggn.as<float>() : nullptr, na, max_degree, seed, surface, g, s);
  out.avg_separation_estimate = g.avg_separation_estimate;
  Scratch flag(sizeof(unsigned), s);
  THEA_CUDA_CHECK(cudaMemsetAsync(flag.ptr, 0, sizeof(unsigned), s));
  THEA_LAUNCH(extract_kernel, (unsigned)ceil_div(n, EXTRACT_WARPS), EXTRACT_WARPS * 32, 0, s, g.neighbors,
              g.separations, g.degree, max_degree, n, out.neighbors, out.separations, out.degree, flag.as<unsigned>());
  unsigned h = 0;
  THEA_CUDA_CHECK(cudaMemcpyAsync(&h, flag.ptr, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  THEA_CUDA_CHECK(cudaStreamSynchronize(s));
  if (h)
    throw Error(THEA_ERR_NOT_SUPPORTED, "sample_graph: a sample's geodesic search outgrew its " +
                                            std::to_string(EXTRACT_FILL) + "-vertex working set (oversampling too "
                                            "dense for max_degree; use fewer dense samples)");
}

}  // namespace thea

namespace thea {
namespace {

constexpr int RSUM_THREADS = 1024;
constexpr int RSUM_ITEMS = 16;  // consecutive terms per thread; the cursor moves in multiples of it
constexpr int64_t RSUM_WINDOW = (int64_t)RSUM_THREADS * RSUM_ITEMS;

// Units of a thread's 16 terms in binade e; false if one of them has to be taken on its own
__device__ __forceinline__ bool rsum_group_units(float4 const (&v)[RSUM_ITEMS / 4], int e, long long & units) {
  bool ok = true;
  units = 0;
#pragma unroll
  for (int i = 0; i < RSUM_ITEMS / 4; ++i) {
    long long d0 = 0, d1 = 0, d2 = 0, d3 = 0;
    ok = ok && running_sum_step_units(e, v[i].x, d0) && running_sum_step_units(e, v[i].y, d1) &&
         running_sum_step_units(e, v[i].z, d2) && running_sum_step_units(e, v[i].w, d3);
    units += d0 + d1 + d2 + d3;
  }
  return ok;
}

// One block walks the terms in windows of RSUM_THREADS x RSUM_ITEMS. Each thread sums the units of its 16 terms in the
// binade of the sum at the window's start; a block scan over the threads finds the first group that cannot be added in
// bulk (a term to be taken alone, or a total past RUNNING_SUM_MAX_UNITS). Every group before it is added as one integer
// sum, that group's 16 terms one fl(s + x) at a time, and the next window starts after it. Each thread loads its
// group of the following window while the current one is scanned, and keeps it when the window was taken whole.
__global__ void __launch_bounds__(RSUM_THREADS)
running_sum_kernel(float const * __restrict__ x, int64_t const * __restrict__ count, int64_t n_host, float s0,
                   float * __restrict__ out) {
  __shared__ float s_sum;
  __shared__ int64_t s_cursor;
  __shared__ int s_first;
  int64_t n = count ? *count : n_host;
  int t = threadIdx.x;
  if (t == 0) {
    s_sum = s0;
    s_cursor = 0;
  }
  __syncthreads();
  float4 v[RSUM_ITEMS / 4], nv[RSUM_ITEMS / 4];
  int64_t have = -1;  // window start whose group is in v
  while (true) {
    int64_t cur = s_cursor;
    float s = s_sum;
    if (cur >= n) break;
    int e = 0;
    bool bulk = running_sum_binade(s, e);
    int64_t g0 = cur + (int64_t)t * RSUM_ITEMS;
    bool full = g0 + RSUM_ITEMS <= n;
    if (full && have != cur) {
      float4 const * p = reinterpret_cast<float4 const *>(x + g0);
#pragma unroll
      for (int i = 0; i < RSUM_ITEMS / 4; ++i) v[i] = p[i];
    }
    int64_t g1 = g0 + RSUM_WINDOW;
    bool next_full = g1 + RSUM_ITEMS <= n;
    if (next_full) {
      float4 const * p = reinterpret_cast<float4 const *>(x + g1);
#pragma unroll
      for (int i = 0; i < RSUM_ITEMS / 4; ++i) nv[i] = p[i];
    }
    long long units = 0;
    bool ok = bulk;
    if (bulk && g0 < n) {
      if (full) {
        ok = rsum_group_units(v, e, units);
      } else {
        for (int64_t j = g0; j < n; ++j) {
          long long d = 0;
          ok = ok && running_sum_step_units(e, x[j], d);
          units += d;
        }
      }
    }
    long long total = 0;
    long long before = block_exclusive_scan<long long>(units, total);
    long long base = bulk ? running_sum_units_of(s, e) : 0;
    bool fits = ok && base + before + units <= RUNNING_SUM_MAX_UNITS;
    if (t == 0) s_first = RSUM_THREADS;
    __syncthreads();
    if (!fits && g0 < n) atomicMin(&s_first, t);
    __syncthreads();
    int g = s_first;
    if (t == (g < RSUM_THREADS ? g : RSUM_THREADS - 1)) {
      if (g < RSUM_THREADS) {
        if (bulk && before > 0) s = running_sum_from_units(base + before, e);
        int64_t end = g0 + RSUM_ITEMS < n ? g0 + RSUM_ITEMS : n;
        for (int64_t j = g0; j < end; ++j) s = __fadd_rn(s, x[j]);
        s_cursor = end;
      } else {
        s = running_sum_from_units(base + before + units, e);
        s_cursor = cur + RSUM_WINDOW;
      }
      s_sum = s;
    }
    if (g == RSUM_THREADS && next_full) {
#pragma unroll
      for (int i = 0; i < RSUM_ITEMS / 4; ++i) v[i] = nv[i];
      have = cur + RSUM_WINDOW;
    } else {
      have = -1;
    }
    __syncthreads();
  }
  if (t == 0) *out = s_sum;
}

// Offsets of each sample's separations in the compact sequence (exclusive scan of the degrees, done before) -> the
// separations themselves, in order; the last thread writes the number of terms
__global__ void compact_separations_kernel(float const * __restrict__ sep, int32_t const * __restrict__ deg,
                                           int32_t const * __restrict__ off, int64_t n, int m,
                                           float * __restrict__ out, int64_t * __restrict__ count) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int d = deg[i];
  int64_t o = off[i];
  for (int k = 0; k < d; ++k) out[o + k] = sep[i * m + k];
  if (i == n - 1) *count = o + d;
}

// avg = sum / (float)edges (updateAverageSeparation's `avg_separation /= num_edges`), the sum when there are no edges
__global__ void mean_of_sum_kernel(float * __restrict__ sum, int64_t const * __restrict__ count) {
  int64_t c = *count;
  if (c > 0) *sum = *sum / (float)c;
}

}  // namespace

void run_running_sum(float const * x, int64_t const * count, int64_t n, float s0, float * out, cudaStream_t s) {
  THEA_REQUIRE(((uintptr_t)x & 15) == 0, "running_sum: terms must be 16-byte aligned");
  THEA_LAUNCH(running_sum_kernel, 1, RSUM_THREADS, 0, s, x, count, n, s0, out);
}

void run_mean_separation(float const * separations, int32_t const * degree, int64_t n, int max_degree, float * out,
                         cudaStream_t s) {
  THEA_REQUIRE(n >= 1 && n * (int64_t)max_degree < ((int64_t)1 << 31), "mean_separation: too many separations");
  Scratch off((size_t)n * 4, s), vals((size_t)n * max_degree * 4, s), count(8, s);
  exclusive_scan<int32_t>(degree, off.as<int32_t>(), n, s);
  THEA_LAUNCH(compact_separations_kernel, (unsigned)ceil_div(n, GRAPH_THREADS), GRAPH_THREADS, 0, s, separations,
              degree, off.as<int32_t>(), n, max_degree, vals.as<float>(), count.as<int64_t>());
  run_running_sum(vals.as<float>(), count.as<int64_t>(), 0, 0.f, out, s);
  THEA_LAUNCH(mean_of_sum_kernel, 1, 1, 0, s, out, count.as<int64_t>());
}

}  // namespace thea
