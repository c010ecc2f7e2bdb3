// Closest pairs between two BVHs (BvhN::closestPair, BvhN.hpp:1082-1114, and kClosestPairs, :1139-1146, with a BVH as
// the query; the reference descends both trees together, BvhN.hpp:1916-2033).
//
// A pair's distance is the distance between one element of each structure, so the closest pair is the smallest, over
// the elements of one side, of that element's nearest neighbour on the other side: the batched nearest-neighbour kernels
// answer it with one query per element, and a 64-bit atomic minimum of (squared distance bits, query index) picks the
// pair (non-negative floats order like their bit patterns). Point-point pairs query the target's points from the
// query's; point-mesh pairs query the mesh from the points, whichever side the mesh is on. The k closest pairs of two
// point sets are among the k nearest target points of each query point within the k-th smallest of the rows' nearest
// distances: those candidates are compacted in slot order and sorted by (squared distance, query index) with a stable
// radix sort that keeps each row's target order.
#include "pairs.hpp"

#include "device_util.cuh"
#include "query.hpp"
#include "transform.hpp"

#include <algorithm>
#include <cstring>

namespace thea {
namespace {

constexpr int PAIR_THREADS = 256;

// coordinates of a point BVH's elements in element order
__global__ void element_points_kernel(float4 const * __restrict__ rec, int32_t const * __restrict__ leaf_to_elem,
                                      int64_t n, float * __restrict__ out) {
  int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= n) return;
  float4 r = rec[p];
  int64_t e = leaf_to_elem[p];
  out[3 * e] = r.x;
  out[3 * e + 1] = r.y;
  out[3 * e + 2] = r.z;
}

__device__ __forceinline__ float row_d2(int64_t r, float const * d2, float const * pts, float const * cp) {
  if (d2) return d2[r];
  V3 a = load_v3(cp + 3 * r), b = load_v3(pts + 3 * r);
  return squared_norm(a - b);  // as the closest-point kernel evaluates it: |closest point - query|^2
}

// per row (one element of the searching side): key = (d2 bits, query index), minimum over rows
__global__ void pair_min_kernel(int32_t const * __restrict__ idx, float const * __restrict__ d2,
                                float const * __restrict__ pts, float const * __restrict__ cp, int64_t n,
                                int rows_are_query, unsigned long long * __restrict__ best) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n || idx[r] < 0) return;
  uint32_t q = rows_are_query ? (uint32_t)r : (uint32_t)idx[r];
  unsigned long long key = ((unsigned long long)__float_as_uint(row_d2(r, d2, pts, cp)) << 32) | q;
  atomicMin(best, key);
}

// among rows holding the best key: the lowest target index
__global__ void pair_tie_kernel(int32_t const * __restrict__ idx, float const * __restrict__ d2,
                                float const * __restrict__ pts, float const * __restrict__ cp, int64_t n,
                                int rows_are_query, unsigned long long const * __restrict__ best,
                                unsigned * __restrict__ best_target) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n || idx[r] < 0) return;
  uint32_t q = rows_are_query ? (uint32_t)r : (uint32_t)idx[r];
  unsigned long long key = ((unsigned long long)__float_as_uint(row_d2(r, d2, pts, cp)) << 32) | q;
  if (key == *best) atomicMin(best_target, rows_are_query ? (unsigned)idx[r] : (unsigned)r);
}

// key of each row's nearest distance for the k-th-smallest selection (all ones for a row without a neighbour)
__global__ void row_min_keys_kernel(int32_t const * __restrict__ idx, float const * __restrict__ d2, int64_t n,
                                    unsigned long long * __restrict__ keys, uint32_t * __restrict__ vals) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  keys[r] = idx[r] < 0 ? 0xffffffffull : (unsigned long long)__float_as_uint(d2[r]);
  vals[r] = (uint32_t)r;
}

__global__ void slot_flag_kernel(int32_t const * __restrict__ idx, int64_t slots, uint32_t * __restrict__ flag) {
  int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c < slots) flag[c] = idx[c] >= 0 ? 1u : 0u;
}

__global__ void slot_total_kernel(uint32_t const * __restrict__ flag, uint32_t const * __restrict__ pos, int64_t slots,
                                  uint32_t * __restrict__ total) {
  *total = pos[slots - 1] + flag[slots - 1];
}

// filled slot c = row * k + j of the k-NN rows, written at its compacted position: key (d2 bits, row), value c
__global__ void pair_candidates_kernel(int32_t const * __restrict__ idx, float const * __restrict__ d2,
                                       uint32_t const * __restrict__ pos, int64_t slots, int k,
                                       unsigned long long * __restrict__ keys, uint32_t * __restrict__ vals) {
  int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= slots || idx[c] < 0) return;
  uint32_t p = pos[c];
  keys[p] = ((unsigned long long)__float_as_uint(d2[c]) << 32) | (uint64_t)(c / k);
  vals[p] = (uint32_t)c;
}

__global__ void pair_take_kernel(unsigned long long const * __restrict__ keys, uint32_t const * __restrict__ vals,
                                 int32_t const * __restrict__ idx, float const * __restrict__ d2, int64_t m, int k,
                                 int32_t * __restrict__ qi, int32_t * __restrict__ ti, float * __restrict__ od2,
                                 unsigned * __restrict__ count) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= k) return;
  bool ok = j < m && keys[j] != ~0ull;
  qi[j] = ok ? (int32_t)(keys[j] & 0xffffffffu) : -1;
  ti[j] = ok ? idx[vals[j]] : -1;
  od2[j] = ok ? d2[vals[j]] : -1.f;
  if (ok) atomicAdd(count, 1u);
}

Scratch element_points(thea_bvh const * b, cudaStream_t s) {
  thea_bvh const * w = query_target(b);  // world-space records when a transform is set
  Scratch out((size_t)w->n * 12, s);
  THEA_LAUNCH(element_points_kernel, (unsigned)ceil_div(w->n, PAIR_THREADS), PAIR_THREADS, 0, s, w->pt_rec,
              w->leaf_to_elem, w->n, out.as<float>());
  return out;
}

void check_single(thea_bvh const * b, char const * what) {
  THEA_REQUIRE(b, std::string(what) + ": null BVH");
  THEA_REQUIRE(b->num_segments == 1, std::string(what) + ": forests are not supported");
  if (b->is_mesh) THEA_REQUIRE(query_target(b)->cp_rec, std::string(what) + ": the mesh BVH needs THEA_LAYOUT_CLOSEST");
}

}  // namespace

bool run_closest_pair(thea_bvh const * target, thea_bvh const * query, float thresh, PairResult & out,
                      cudaStream_t s) {
  check_single(target, "closest_pair");
  check_single(query, "closest_pair");
  if (target->is_mesh && query->is_mesh)
    throw Error(THEA_ERR_NOT_SUPPORTED, "closest_pair: mesh-mesh pairs are not supported (one side must hold points)");
  out = PairResult();
  // rows: the elements of the point side that searches the other side
  bool rows_are_query = !query->is_mesh;
  thea_bvh const * rows_bvh = rows_are_query ? query : target;
  thea_bvh const * searched = query_target(rows_are_query ? target : query);
  int64_t n = rows_bvh->n;
  if (n == 0 || searched->n == 0) return false;
  Scratch pts = element_points(rows_bvh, s);
  Scratch idx((size_t)n * 4, s), d2, cp, best(8, s), best_t(4, s);
  if (searched->is_mesh) {
    cp = Scratch((size_t)n * 12, s);
    ClosestParams c;
    c.thresh = thresh;
    c.scene_scale = scene_scale_of(searched);
    run_closest(searched, pts.as<float>(), n, c, idx.as<int32_t>(), nullptr, cp.as<float>(), nullptr, searched->err,
                s);
  } else {
    d2 = Scratch((size_t)n * 4, s);
    run_knn(searched, pts.as<float>(), n, 1, thresh, nullptr, idx.as<int32_t>(), d2.as<float>(), searched->err, s);
  }
  THEA_CUDA_CHECK(cudaMemsetAsync(best.ptr, 0xff, 8, s));
  THEA_CUDA_CHECK(cudaMemsetAsync(best_t.ptr, 0xff, 4, s));
  unsigned blocks = (unsigned)ceil_div(n, PAIR_THREADS);
  THEA_LAUNCH(pair_min_kernel, blocks, PAIR_THREADS, 0, s, idx.as<int32_t>(), d2.as<float>(), pts.as<float>(),
              cp.as<float>(), n, rows_are_query ? 1 : 0, best.as<unsigned long long>());
  THEA_LAUNCH(pair_tie_kernel, blocks, PAIR_THREADS, 0, s, idx.as<int32_t>(), d2.as<float>(), pts.as<float>(),
              cp.as<float>(), n, rows_are_query ? 1 : 0, best.as<unsigned long long>(), best_t.as<unsigned>());
  unsigned long long hb = 0;
  unsigned ht = 0;
  THEA_CUDA_CHECK(cudaMemcpyAsync(&hb, best.ptr, 8, cudaMemcpyDeviceToHost, s));
  THEA_CUDA_CHECK(cudaMemcpyAsync(&ht, best_t.ptr, 4, cudaMemcpyDeviceToHost, s));
  THEA_CUDA_CHECK(cudaStreamSynchronize(s));
  if (hb == ~0ull) return false;
  out.query_index = (int32_t)(hb & 0xffffffffu);
  out.target_index = (int32_t)ht;
  uint32_t bits = (uint32_t)(hb >> 32);
  std::memcpy(&out.d2, &bits, 4);
  // the closest points: each point element itself, and on the mesh side the closest point of the row
  int64_t row = rows_are_query ? out.query_index : out.target_index;
  float row_pt[3], other_pt[3];
  THEA_CUDA_CHECK(cudaMemcpyAsync(row_pt, pts.as<float>() + 3 * row, 12, cudaMemcpyDeviceToHost, s));
  Scratch other;
  if (searched->is_mesh) {
    THEA_CUDA_CHECK(cudaMemcpyAsync(other_pt, cp.as<float>() + 3 * row, 12, cudaMemcpyDeviceToHost, s));
  } else {  // point-point: the target point itself
    other = element_points(target, s);
    THEA_CUDA_CHECK(cudaMemcpyAsync(other_pt, other.as<float>() + 3 * (int64_t)out.target_index, 12,
                                    cudaMemcpyDeviceToHost, s));
  }
  THEA_CUDA_CHECK(cudaStreamSynchronize(s));
  std::memcpy(rows_are_query ? out.query_point : out.target_point, row_pt, 12);
  std::memcpy(rows_are_query ? out.target_point : out.query_point, other_pt, 12);
  return true;
}

int64_t run_k_closest_pairs(thea_bvh const * target, thea_bvh const * query, int k, float thresh, int32_t * qi,
                            int32_t * ti, float * d2, cudaStream_t s) {
  check_single(target, "k_closest_pairs");
  check_single(query, "k_closest_pairs");
  THEA_REQUIRE(!target->is_mesh && !query->is_mesh, "k_closest_pairs: two point BVHs are required");
  THEA_REQUIRE(k >= 1 && k <= 32, "k_closest_pairs: k must be in 1..32");
  int64_t n = query->n;
  Scratch count(4, s);
  THEA_CUDA_CHECK(cudaMemsetAsync(count.ptr, 0, 4, s));
  Scratch keys(8, s), vals(4, s), idx(4, s), dd(4, s);
  int64_t m = 0;
  if (n > 0 && target->n > 0) {
    Scratch pts = element_points(query, s);
    thea_bvh const * searched = query_target(target);
    unsigned blocks = (unsigned)ceil_div(n, PAIR_THREADS);
    // 1. every row's nearest target point; the k-th smallest of those distances bounds the k-th closest pair (the k
    //    rows with the smallest minima already give k distinct pairs within it)
    if (n >= k) {
      Scratch idx1((size_t)n * 4, s), d21((size_t)n * 4, s), rk((size_t)n * 8, s), rv((size_t)n * 4, s);
      run_knn(searched, pts.as<float>(), n, 1, thresh, nullptr, idx1.as<int32_t>(), d21.as<float>(), searched->err, s);
      THEA_LAUNCH(row_min_keys_kernel, blocks, PAIR_THREADS, 0, s, idx1.as<int32_t>(), d21.as<float>(), n,
                  rk.as<unsigned long long>(), rv.as<uint32_t>());
      radix_sort_pairs(rk.as<uint64_t>(), rv.as<uint32_t>(), n, 32, s);
      unsigned long long kth = 0;
      THEA_CUDA_CHECK(cudaMemcpyAsync(&kth, rk.as<unsigned long long>() + (k - 1), 8, cudaMemcpyDeviceToHost, s));
      THEA_CUDA_CHECK(cudaStreamSynchronize(s));
      if (kth != 0xffffffffull) {
        float tau;
        uint32_t bits = (uint32_t)kth;
        std::memcpy(&tau, &bits, 4);
        thresh = std::min(thresh, tau);  // both accept squared distances <= the threshold
      }
    }
    // 2. each row's k nearest within the bound; the global k closest pairs are among them
    int64_t slots = n * k;
    idx = Scratch((size_t)slots * 4, s);
    dd = Scratch((size_t)slots * 4, s);
    run_knn(searched, pts.as<float>(), n, k, thresh, nullptr, idx.as<int32_t>(), dd.as<float>(), searched->err, s);
    // 3. compact the filled slots in slot order, then sort them by (squared distance, row), stably
    Scratch flag((size_t)slots * 4, s), pos((size_t)slots * 4, s), total(4, s);
    unsigned sblocks = (unsigned)ceil_div(slots, PAIR_THREADS);
    THEA_LAUNCH(slot_flag_kernel, sblocks, PAIR_THREADS, 0, s, idx.as<int32_t>(), slots, flag.as<uint32_t>());
    exclusive_scan(flag.as<uint32_t>(), pos.as<uint32_t>(), slots, s);
    THEA_LAUNCH(slot_total_kernel, 1, 1, 0, s, flag.as<uint32_t>(), pos.as<uint32_t>(), slots, total.as<uint32_t>());
    uint32_t hm = 0;
    THEA_CUDA_CHECK(cudaMemcpyAsync(&hm, total.ptr, 4, cudaMemcpyDeviceToHost, s));
    THEA_CUDA_CHECK(cudaStreamSynchronize(s));
    m = hm;
    if (m > 0) {
      keys = Scratch((size_t)m * 8, s);
      vals = Scratch((size_t)m * 4, s);
      THEA_LAUNCH(pair_candidates_kernel, sblocks, PAIR_THREADS, 0, s, idx.as<int32_t>(), dd.as<float>(),
                  pos.as<uint32_t>(), slots, k, keys.as<unsigned long long>(), vals.as<uint32_t>());
      radix_sort_pairs(keys.as<uint64_t>(), vals.as<uint32_t>(), m, 64, s);
    }
  }
  THEA_LAUNCH(pair_take_kernel, 1, 32, 0, s, keys.as<unsigned long long>(), vals.as<uint32_t>(), idx.as<int32_t>(),
              dd.as<float>(), m, k, qi, ti, d2, count.as<unsigned>());
  unsigned hc = 0;
  THEA_CUDA_CHECK(cudaMemcpyAsync(&hc, count.ptr, 4, cudaMemcpyDeviceToHost, s));
  THEA_CUDA_CHECK(cudaStreamSynchronize(s));
  return (int64_t)hc;
}

}  // namespace thea
