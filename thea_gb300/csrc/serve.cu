// Serving loop (thea_server_*): meshes resident in device memory, admission by a memory budget, and continuous
// batching of mixed closest-point / ray / k-NN requests.
//
// Requests are cut into pieces; a dispatcher thread packs pending pieces into batches (one "task" per piece) and runs
// each batch on one of a few streams ("slots"): staging copies in, one persistent launch per query kind over the
// batch's task table, copies out, then a host callback that marks the slot finished. While a batch runs, requests that
// arrive are packed into the next free slot, so their copies and kernels overlap with the batches already on the
// device. The query kernels are the ones of the single-BVH calls (traverse_ops.cuh), reached through a per-task BVH
// pointer, so a request's results are the same alone and in any mix.
#include "serve.hpp"

#include "device_util.cuh"
#include "query.hpp"
#include "traverse_ops.cuh"
#include "warp_traverse.cuh"

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

namespace thea {
namespace {

constexpr int SERVE_THREADS = 128;
constexpr int MAX_TASKS = 4096;  // pieces per batch and query kind

// One piece of one request, as the kernels see it
struct ServeTask {
  void const * nodes;
  float4 const * rec;  // closest: CP records; ray: ray records; k-NN: point records
  float4 const * slabs;  // closest: oriented slabs of the mesh BVH's child slots
  float const * in0;   // query points / ray origins of the piece
  float const * in1;   // ray directions
  int32_t * out_index;
  float * out_value;
  float * out_point;
  unsigned * err;
  int64_t n;
  double bound2;       // closest, FP64 re-check: dist_bound^2 (negative: none)
  float thresh;        // closest and k-NN: FP32 threshold on squared distances; ray: max_time (negative: none)
  float scene_scale;
  int32_t k;
  int32_t pad;
  BoundCut cut;        // closest: the reference's distance-bound cut of the mesh (queries it removes get no element)
};

__device__ __forceinline__ int task_of(int64_t const * __restrict__ off, int T, int64_t q) {
  int lo = 0, hi = T - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (__ldg(off + mid) <= q) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Warp-wide fetch of the next 32 queries
__device__ __forceinline__ bool next_round(unsigned long long * counter, int64_t nq, int64_t & base) {
  unsigned long long b = 0;
  if ((threadIdx.x & 31) == 0) b = atomicAdd(counter, 32ull);
  b = __shfl_sync(0xffffffffu, b, 0);
  base = (int64_t)b;
  return base < nq;
}

// Closest-element queries that ran out of their stack-pop budget in the first kernel, finished one warp per query by
// the second (a deep query inside a large mesh would otherwise hold its whole batch for milliseconds).
struct ServeHardQueue {
  int64_t * q;
  float * bound;  // FP32 squared distance of the best element found so far (+inf if none)
  int32_t * idx;
  int64_t * slot;
  unsigned long long * count;
};

template <int W, int STACK, int PREC>
__global__ void __launch_bounds__(SERVE_THREADS)
serve_closest_kernel(ServeTask const * __restrict__ tasks, int64_t const * __restrict__ off, int T, int64_t nq,
                     unsigned long long * counter, int budget, ServeHardQueue hq) {
  F64WarpBuf * buf = nullptr;
  if constexpr (PREC == THEA_PRECISION_FP64_RECHECK) {
    __shared__ F64WarpBuf s_buf[SERVE_THREADS / 32];
    buf = &s_buf[threadIdx.x >> 5];
  }
  int lane = threadIdx.x & 31;
  int64_t base;
  while (next_round(counter, nq, base)) {
    int64_t q = base + lane;
    bool active = q < nq;
    ServeTask const * t = nullptr;
    int64_t i = 0;
    V3 p = V3{0.f, 0.f, 0.f};
    if (active) {
      int ti = task_of(off, T, q);
      t = tasks + ti;
      i = q - __ldg(off + ti);
      p = load_v3(t->in0 + 3 * i);
    }
    WideNode<W> const * nodes = active ? (WideNode<W> const *)t->nodes : nullptr;
    float4 const * rec = active ? t->rec : nullptr;
    ClosestOut r;
    r.idx = INT_MAX;
    r.d2 = 0.f;
    r.d2_64 = 0.0;
    r.slot = -1;
    r.best32 = INFINITY;
    r.done = true;
    float dist = 0.f;
    if constexpr (PREC == THEA_PRECISION_FP64_RECHECK) {
      float scale = active ? fmaxf(t->scene_scale, fmaxf(fabsf(p.x), fmaxf(fabsf(p.y), fabsf(p.z)))) : 0.f;
      F64Search s;
      if (active) closest_search_f64<W, STACK>(nodes, rec, 0, 0, p, t->bound2, scale, t->err, s, budget, t->slabs);
      else f64_search_init(s);
      f64_resolve_warp(s, active && s.done, rec, 0, p, active ? t->bound2 : -1.0, *buf);
      r = f64_result(s);
      dist = (float)sqrt(r.d2_64);
    } else {
      if (active) r = closest_query<W, STACK>(nodes, rec, 0, 0, p, t->thresh, t->err, budget, t->slabs);
      dist = sqrtf(r.d2);
    }
    if (active && !r.done) {
      unsigned long long pos = atomicAdd(hq.count, 1ull);
      hq.q[pos] = q;
      hq.bound[pos] = r.best32;
      hq.idx[pos] = PREC == THEA_PRECISION_FP64_RECHECK ? INT_MAX : r.idx;
      hq.slot[pos] = r.slot;
      active = false;
    }
    if (active) {
      bool found = r.idx != INT_MAX && !bound_cut_out(t->cut, p);
      t->out_index[i] = found ? r.idx : -1;
      if (t->out_value) t->out_value[i] = found ? dist : -1.f;
      if (t->out_point) {
        t->out_point[3 * i] = found ? r.cp.x : 0.f;
        t->out_point[3 * i + 1] = found ? r.cp.y : 0.f;
        t->out_point[3 * i + 2] = found ? r.cp.z : 0.f;
      }
    }
  }
}

template <int W, int PREC>
__global__ void __launch_bounds__(SERVE_THREADS)
serve_closest_phase2_kernel(ServeTask const * __restrict__ tasks, int64_t const * __restrict__ off, int T,
                            ServeHardQueue hq, unsigned long long * counter) {
  constexpr int WARPS = SERVE_THREADS / 32;
  __shared__ int s_code[WARPS][WARP_STACK];
  __shared__ float s_lb[WARPS][WARP_STACK];
  __shared__ float s_cd[WARPS][PREC == THEA_PRECISION_FP64_RECHECK ? WARP_CAND : 1];
  __shared__ int64_t s_ck[WARPS][PREC == THEA_PRECISION_FP64_RECHECK ? WARP_CAND : 1];
  int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned long long total = *hq.count;
  while (true) {
    unsigned long long j = 0;
    if (lane == 0) j = atomicAdd(counter, 1ull);
    j = __shfl_sync(0xffffffffu, j, 0);
    if (j >= total) break;
    int64_t q = hq.q[j];
    int ti = task_of(off, T, q);
    ServeTask const * t = tasks + ti;
    int64_t i = q - __ldg(off + ti);
    V3 p = load_v3(t->in0 + 3 * i);
    WideNode<W> const * nodes = (WideNode<W> const *)t->nodes;
    bool found;
    float dist;
    V3 cp = V3{0.f, 0.f, 0.f};
    int idx;
    if (PREC == THEA_PRECISION_FP64_RECHECK) {
      float scale = fmaxf(t->scene_scale, fmaxf(fabsf(p.x), fmaxf(fabsf(p.y), fabsf(p.z))));
      WarpBest64 b = closest_warp_query_f64<W>(nodes, t->rec, 0, 0, p, t->bound2, scale, hq.bound[j], s_code[warp],
                                               s_lb[warp], s_cd[warp], s_ck[warp], t->err);
      found = b.idx != INT_MAX;
      idx = b.idx;
      dist = (float)sqrt(b.d2);
      if (found && lane == 0 && t->out_point) {
        D3 cp64;
        double d64;
        cp_record_f64(t->rec, b.slot, p, cp64, d64);
        cp = V3{(float)cp64.x, (float)cp64.y, (float)cp64.z};
      }
    } else {
      WarpBest init;
      init.idx = hq.idx[j];
      init.d2 = init.idx != INT_MAX ? hq.bound[j] : t->thresh;
      init.slot = hq.slot[j];
      WarpBest b = closest_warp_query<W>(nodes, t->rec, 0, 0, p, init, s_code[warp], s_lb[warp], t->err, t->slabs);
      found = b.idx != INT_MAX;
      idx = b.idx;
      dist = sqrtf(b.d2);
      if (found && lane == 0 && t->out_point) cp_record_test(t->rec, b.slot, p, cp);
    }
    if (lane == 0) {
      found = found && !bound_cut_out(t->cut, p);
      t->out_index[i] = found ? idx : -1;
      if (t->out_value) t->out_value[i] = found ? dist : -1.f;
      if (t->out_point) {
        t->out_point[3 * i] = found ? cp.x : 0.f;
        t->out_point[3 * i + 1] = found ? cp.y : 0.f;
        t->out_point[3 * i + 2] = found ? cp.z : 0.f;
      }
    }
    __syncwarp();
  }
}

template <int W, int STACK>
__global__ void __launch_bounds__(SERVE_THREADS)
serve_ray_kernel(ServeTask const * __restrict__ tasks, int64_t const * __restrict__ off, int T, int64_t nq,
                 unsigned long long * counter) {
  int lane = threadIdx.x & 31;
  int64_t base;
  while (next_round(counter, nq, base)) {
    int64_t q = base + lane;
    if (q >= nq) continue;
    int ti = task_of(off, T, q);
    ServeTask const * t = tasks + ti;
    int64_t i = q - __ldg(off + ti);
    RayOut r = ray_query<W, STACK, false>((WideNode<W> const *)t->nodes, t->rec, 0, 0, load_v3(t->in0 + 3 * i),
                                          load_v3(t->in1 + 3 * i), t->thresh, t->err);
    bool found = r.idx != INT_MAX;
    t->out_index[i] = found ? r.idx : -1;
    if (t->out_value) t->out_value[i] = found ? r.t : -1.f;
  }
}

template <int W, int K, int STACK>
__global__ void __launch_bounds__(SERVE_THREADS)
serve_knn_kernel(ServeTask const * __restrict__ tasks, int64_t const * __restrict__ off, int T, int64_t nq,
                 unsigned long long * counter) {
  int lane = threadIdx.x & 31;
  int64_t base;
  while (next_round(counter, nq, base)) {
    int64_t q = base + lane;
    if (q >= nq) continue;
    int ti = task_of(off, T, q);
    ServeTask const * t = tasks + ti;
    int64_t i = q - __ldg(off + ti);
    float bd[K];
    int bi[K];
#pragma unroll
    for (int j = 0; j < K; ++j) {
      bd[j] = t->thresh;
      bi[j] = INT_MAX;
    }
    knn_query<W, K, STACK>((WideNode<W> const *)t->nodes, t->rec, 0, 0, load_v3(t->in0 + 3 * i), -1, bd, bi, t->err);
    int k = t->k;
    for (int j = 0; j < k; ++j) {
      bool v = bi[j] != INT_MAX;
      t->out_index[i * k + j] = v ? bi[j] : -1;
      if (t->out_value) t->out_value[i * k + j] = v ? bd[j] : -1.f;
    }
  }
}

template <class K> int grid_for(K kernel, int64_t nq) {
  int sms = sm_count();
  int per_sm = 0;
  THEA_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, SERVE_THREADS, 0));
  int64_t need = ceil_div(nq, SERVE_THREADS);
  return (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)std::max(1, per_sm) * sms, need));
}

float threshold_of(float bound) {
  if (!(bound >= 0.f)) return INFINITY;
  double b2 = (double)bound * (double)bound;
  float f = (float)b2;
  if ((double)f >= b2) f = std::nextafter(f, -INFINITY);
  return f;
}

bool host_memory(void const * p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return true;
  }
  return !(a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged);
}

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

double percentile(std::vector<double> v, double f) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  size_t i = (size_t)std::min<double>((double)(v.size() - 1), std::ceil(f * (double)v.size()) - 1.0);
  return v[i];
}

}  // namespace
}  // namespace thea

using thea::Clock;

struct ServeMesh {
  thea_bvh * mesh = nullptr;  // closest + ray layouts
  thea_bvh * pts = nullptr;   // the mesh's vertices, for k-NN
  int64_t bytes = 0;
  int refs = 0;               // requests submitted and not finished
  bool removing = false;
  float scene_scale = 0.f;
};

struct ServeRequest {
  uint64_t ticket = 0;
  thea_request r{};
  int64_t scheduled = 0;  // queries already packed into batches
  int pieces = 0;         // pieces packed
  int pieces_done = 0;
  bool stage_in = false, stage_out = false;  // some input / output array is host memory
  int64_t bytes_per_query = 0;               // device staging bytes per query
  thea_status status = THEA_OK;
  bool cancelled = false;
  bool done = false;
  Clock::time_point submitted, finished;
};

struct ServePiece {
  ServeRequest * req;
  int64_t first, n;
  int64_t bytes;
  void * staging = nullptr;
};

struct ServeSlot {
  thea_server * owner = nullptr;
  cudaStream_t stream = nullptr;   // batches with a large request
  cudaStream_t express = nullptr;  // batches of small requests only: the device's highest stream priority
  cudaStream_t active = nullptr;   // the stream the slot's current batch was enqueued on
  thea::ServeTask * d_tasks = nullptr;  // [3][MAX_TASKS]
  thea::ServeTask * h_tasks = nullptr;  // pinned mirror
  int64_t * d_off = nullptr;            // [3][MAX_TASKS + 1]
  int64_t * h_off = nullptr;
  unsigned long long * d_counters = nullptr;  // [5]: per query kind, then the hard queue's count and its cursor
  std::vector<ServePiece> pieces;
  bool busy = false;
  bool complete = false;  // set by the stream callback (or the test executor's clock)
  Clock::time_point test_deadline;
  thea_status launch_status = THEA_OK;
};

struct thea_server {
  thea_server_config cfg{};
  int device = 0;
  std::mutex mu;
  std::condition_variable cv;       // dispatcher: new work, a finished slot, stop
  std::condition_variable cv_done;  // waiters
  std::map<int32_t, ServeMesh> meshes;
  // BVHs of removed meshes whose last request has ended, destroyed once the lock is released: destroy_bvh synchronizes
  // the device, which waits for the slots' completion callbacks, and those take the lock
  std::vector<thea_bvh *> retired;
  int32_t next_mesh = 0;
  std::map<uint64_t, std::unique_ptr<ServeRequest>> requests;
  std::vector<ServeRequest *> pending;
  uint64_t next_ticket = 1;
  std::vector<std::unique_ptr<ServeSlot>> slots;
  int64_t resident_bytes = 0, inflight_bytes = 0;
  bool stopping = false;
  std::thread dispatcher;
  // statistics
  int64_t submitted = 0, completed = 0, failed = 0, cancelled = 0, refused = 0, queries_completed = 0, batches = 0;
  std::vector<double> lat, lat_small;
  bool have_first = false;
  Clock::time_point first_submit, last_finish;
};

namespace thea {
namespace {

void CUDART_CB slot_finished_cb(void * p) {
  ServeSlot * s = (ServeSlot *)p;
  {
    std::lock_guard<std::mutex> lk(s->owner->mu);
    s->complete = true;
  }
  s->owner->cv.notify_all();
}

void release_mesh_locked(thea_server * sv, int32_t id) {
  auto it = sv->meshes.find(id);
  if (it == sv->meshes.end()) return;
  ServeMesh & m = it->second;
  if (--m.refs == 0 && m.removing) {
    sv->resident_bytes -= m.bytes;
    if (!sv->cfg.test_executor) {
      sv->retired.push_back(m.mesh);
      sv->retired.push_back(m.pts);
    }
    sv->meshes.erase(it);
  }
}

// Destroys the retired BVHs; the caller must not hold the lock
void destroy_retired(thea_server * sv) {
  std::vector<thea_bvh *> r;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    r.swap(sv->retired);
  }
  for (thea_bvh * b : r) destroy_bvh(b);
}

void end_request_locked(thea_server * sv, ServeRequest * q, thea_status st) {
  if (q->done) return;
  q->done = true;
  q->status = q->cancelled && st == THEA_OK ? THEA_ERR_CANCELLED : st;
  q->finished = Clock::now();
  if (q->status == THEA_OK) {
    ++sv->completed;
    sv->queries_completed += q->r.num_queries;
    double l = ms_between(q->submitted, q->finished);
    sv->lat.push_back(l);
    if (q->r.num_queries <= sv->cfg.small_request_queries) sv->lat_small.push_back(l);
    sv->last_finish = q->finished;
  } else if (q->status == THEA_ERR_CANCELLED) {
    ++sv->cancelled;
  } else {
    ++sv->failed;
  }
  release_mesh_locked(sv, q->r.mesh);
  sv->cv_done.notify_all();
}

void finish_slot_locked(thea_server * sv, ServeSlot & s) {
  for (ServePiece & p : s.pieces) {
    ServeRequest * q = p.req;
    sv->inflight_bytes -= p.bytes;
    ++q->pieces_done;
    if (s.launch_status != THEA_OK && q->status == THEA_OK) q->status = s.launch_status;
    if (q->scheduled == q->r.num_queries && q->pieces_done == q->pieces) end_request_locked(sv, q, q->status);
  }
  s.pieces.clear();
  s.busy = false;
  s.complete = false;
  s.launch_status = THEA_OK;
}

// Packs pending pieces into slot s: the longest-waiting requests first once they pass max_wait_ms, then the smallest
// remaining ones. Returns false if nothing could be admitted.
bool form_batch_locked(thea_server * sv, ServeSlot & s) {
  Clock::time_point now = Clock::now();
  double max_wait = (double)sv->cfg.max_wait_ms;
  std::vector<ServeRequest *> order(sv->pending.begin(), sv->pending.end());
  std::stable_sort(order.begin(), order.end(), [&](ServeRequest * a, ServeRequest * b) {
    bool la = ms_between(a->submitted, now) > max_wait, lb = ms_between(b->submitted, now) > max_wait;
    if (la != lb) return la;
    if (la) return a->submitted < b->submitted;
    return a->r.num_queries - a->scheduled < b->r.num_queries - b->scheduled;
  });
  int64_t room = sv->cfg.memory_budget_bytes - sv->resident_bytes - sv->inflight_bytes;
  int64_t batch_q = 0;
  int tasks[3] = {0, 0, 0};
  for (ServeRequest * q : order) {
    while (q->scheduled < q->r.num_queries && batch_q < sv->cfg.max_batch_queries && tasks[q->r.type] < MAX_TASKS) {
      int64_t n = std::min<int64_t>({q->r.num_queries - q->scheduled, (int64_t)sv->cfg.max_piece_queries,
                                     (int64_t)sv->cfg.max_batch_queries - batch_q});
      int64_t bytes = n * q->bytes_per_query;
      if (bytes > room) break;
      s.pieces.push_back(ServePiece{q, q->scheduled, n, bytes, nullptr});
      room -= bytes;
      sv->inflight_bytes += bytes;
      batch_q += n;
      q->scheduled += n;
      ++q->pieces;
      ++tasks[q->r.type];
    }
  }
  sv->pending.erase(std::remove_if(sv->pending.begin(), sv->pending.end(),
                                   [](ServeRequest * q) { return q->scheduled == q->r.num_queries; }),
                    sv->pending.end());
  return !s.pieces.empty();
}

// Enqueues the slot's batch on its stream (called without the lock; only the dispatcher touches slots and the meshes of
// admitted requests stay alive until those requests end).
void launch_slot(thea_server * sv, ServeSlot & s, std::vector<ServeMesh const *> const & piece_mesh) {
  // A batch of small requests only goes to the high-priority stream: its blocks are scheduled ahead of the waiting
  // blocks of batches already launched on other slots, instead of queueing behind a large request's launch
  bool small_only = true;
  for (ServePiece const & p : s.pieces) small_only = small_only && p.req->r.num_queries <= sv->cfg.small_request_queries;
  cudaStream_t st = small_only ? s.express : s.stream;
  s.active = st;
  int T[3] = {0, 0, 0};
  int64_t nq[3] = {0, 0, 0};
  int maxk = 1;
  for (size_t pi = 0; pi < s.pieces.size(); ++pi) {
    ServePiece & p = s.pieces[pi];
    ServeRequest * q = p.req;
    thea_request const & r = q->r;
    ServeMesh const * m = piece_mesh[pi];
    int type = r.type;
    ServeTask t{};
    t.n = p.n;
    t.k = r.k;
    char * stg = nullptr;
    if (p.bytes) {
      THEA_CUDA_CHECK(thea_malloc_from_pool_async(&p.staging, (size_t)p.bytes, scratch_pool(), st));
      stg = (char *)p.staging;
    }
    // staging layout per piece: inputs (12 B, ray 24 B per query), then outputs
    auto in_arr = [&](float const * user, int64_t per, size_t & used) -> float const * {
      if (!q->stage_in) return user + per * p.first;
      float * d = (float *)(stg + used);
      used += (size_t)p.n * per * 4;
      THEA_CUDA_CHECK(cudaMemcpyAsync(d, user + per * p.first, (size_t)p.n * per * 4, cudaMemcpyHostToDevice, st));
      return d;
    };
    size_t used = 0;
    t.in0 = in_arr(r.queries, 3, used);
    if (type == THEA_REQUEST_RAY) t.in1 = in_arr(r.directions, 3, used);
    int64_t per_out = type == THEA_REQUEST_KNN ? r.k : 1;
    auto out_arr = [&](void * user, int64_t per, size_t elem) -> void * {
      if (!user) return nullptr;
      if (!q->stage_out) return (char *)user + (size_t)(per * p.first) * elem;
      void * d = stg + used;
      used += (size_t)(p.n * per) * elem;
      return d;
    };
    t.out_index = (int32_t *)out_arr(r.out_index, per_out, 4);
    t.out_value = (float *)out_arr(r.out_value, per_out, 4);
    t.out_point = type == THEA_REQUEST_CLOSEST ? (float *)out_arr(r.out_point, 3, 4) : nullptr;
    thea_bvh const * b = type == THEA_REQUEST_KNN ? m->pts : m->mesh;
    t.nodes = b->nodes;
    t.rec = type == THEA_REQUEST_CLOSEST ? b->cp_rec : type == THEA_REQUEST_RAY ? b->ray_rec : b->pt_rec;
    t.slabs = type == THEA_REQUEST_CLOSEST ? b->slabs : nullptr;
    t.err = b->err;
    t.scene_scale = m->scene_scale;
    if (type == THEA_REQUEST_RAY) {
      t.thresh = r.bound >= 0.f ? r.bound : -1.f;
    } else if (type == THEA_REQUEST_CLOSEST) {
      t.cut = closest_bound_cut(m->mesh, r.bound);
      t.thresh = t.cut.thresh;
      t.bound2 = t.cut.bound2;
    } else {
      t.thresh = threshold_of(r.bound);
      t.bound2 = r.bound >= 0.f ? (double)r.bound * (double)r.bound : -1.0;
    }
    if (type == THEA_REQUEST_KNN) maxk = std::max(maxk, r.k);
    int j = T[type]++;
    s.h_tasks[type * MAX_TASKS + j] = t;
    s.h_off[type * (MAX_TASKS + 1) + j] = nq[type];
    nq[type] += p.n;
  }
  for (int type = 0; type < 3; ++type) {
    if (!T[type]) continue;
    s.h_off[type * (MAX_TASKS + 1) + T[type]] = nq[type];
    THEA_CUDA_CHECK(cudaMemcpyAsync(s.d_tasks + type * MAX_TASKS, s.h_tasks + type * MAX_TASKS,
                                    sizeof(ServeTask) * T[type], cudaMemcpyHostToDevice, st));
    THEA_CUDA_CHECK(cudaMemcpyAsync(s.d_off + type * (MAX_TASKS + 1), s.h_off + type * (MAX_TASKS + 1),
                                    sizeof(int64_t) * (T[type] + 1), cudaMemcpyHostToDevice, st));
  }
  THEA_CUDA_CHECK(cudaMemsetAsync(s.d_counters, 0, 5 * sizeof(unsigned long long), st));
  int W = sv->cfg.width;
  for (int type = 0; type < 3; ++type) {
    if (!T[type]) continue;
    ServeTask const * tk = s.d_tasks + type * MAX_TASKS;
    int64_t const * of = s.d_off + type * (MAX_TASKS + 1);
    unsigned long long * c = s.d_counters + type;
    int64_t n = nq[type];
    int Tn = T[type];
    if (type == THEA_REQUEST_CLOSEST) {
      bool f64 = sv->cfg.precision == THEA_PRECISION_FP64_RECHECK;
      int budget = sv->cfg.hard_query_budget;
      size_t hn = budget > 0 ? (size_t)n : 0;
      Scratch hq_q(hn * sizeof(int64_t), st), hq_b(hn * sizeof(float), st), hq_i(hn * sizeof(int32_t), st),
          hq_s(hn * sizeof(int64_t), st);
      ServeHardQueue hq{hq_q.as<int64_t>(), hq_b.as<float>(), hq_i.as<int32_t>(), hq_s.as<int64_t>(),
                        s.d_counters + 3};
#define THEA_SERVE_CP(WW, SS, PP)                                                                                  \
  do {                                                                                                            \
    auto k = serve_closest_kernel<WW, SS, PP>;                                                                    \
    THEA_LAUNCH_NAMED("serve_closest_kernel", k, grid_for(k, n), SERVE_THREADS, 0, st, tk, of, Tn, n, c,         \
                      budget > 0 ? budget : 0, hq);                                                               \
    if (budget > 0) {                                                                                             \
      auto k2 = serve_closest_phase2_kernel<WW, PP>;                                                              \
      THEA_LAUNCH_NAMED("serve_closest_phase2_kernel", k2, grid_for(k2, n), SERVE_THREADS, 0, st, tk, of, Tn, hq, \
                        s.d_counters + 4);                                                                        \
    }                                                                                                             \
  } while (0)
      if (W == 4) {
        if (f64) THEA_SERVE_CP(4, 256, 1);
        else THEA_SERVE_CP(4, 256, 0);
      } else {
        if (f64) THEA_SERVE_CP(8, 512, 1);
        else THEA_SERVE_CP(8, 512, 0);
      }
#undef THEA_SERVE_CP
    } else if (type == THEA_REQUEST_RAY) {
      if (W == 4) {
        auto k = serve_ray_kernel<4, 256>;
        THEA_LAUNCH_NAMED("serve_ray_kernel", k, grid_for(k, n), SERVE_THREADS, 0, st, tk, of, Tn, n, c);
      } else {
        auto k = serve_ray_kernel<8, 512>;
        THEA_LAUNCH_NAMED("serve_ray_kernel", k, grid_for(k, n), SERVE_THREADS, 0, st, tk, of, Tn, n, c);
      }
    } else {
#define THEA_SERVE_KNN(WW, KK, SS)                                                                                 \
  do {                                                                                                            \
    auto k = serve_knn_kernel<WW, KK, SS>;                                                                        \
    THEA_LAUNCH_NAMED("serve_knn_kernel", k, grid_for(k, n), SERVE_THREADS, 0, st, tk, of, Tn, n, c);            \
  } while (0)
      if (W == 4) {
        if (maxk <= 8) THEA_SERVE_KNN(4, 8, 256);
        else if (maxk <= 16) THEA_SERVE_KNN(4, 16, 256);
        else THEA_SERVE_KNN(4, 32, 256);
      } else {
        if (maxk <= 8) THEA_SERVE_KNN(8, 8, 512);
        else if (maxk <= 16) THEA_SERVE_KNN(8, 16, 512);
        else THEA_SERVE_KNN(8, 32, 512);
      }
#undef THEA_SERVE_KNN
    }
  }
  // outputs back to host arrays, then release the staging
  for (ServePiece & p : s.pieces) {
    ServeRequest * q = p.req;
    thea_request const & r = q->r;
    if (q->stage_out) {
      char * stg = (char *)p.staging;
      size_t used = (size_t)p.n * (r.type == THEA_REQUEST_RAY ? 24 : 12) * (q->stage_in ? 1 : 0);
      int64_t per = r.type == THEA_REQUEST_KNN ? r.k : 1;
      auto back = [&](void * user, int64_t per_q, size_t elem) {
        if (!user) return;
        size_t bytes = (size_t)(p.n * per_q) * elem;
        THEA_CUDA_CHECK(cudaMemcpyAsync((char *)user + (size_t)(per_q * p.first) * elem, stg + used, bytes,
                                        cudaMemcpyDeviceToHost, st));
        used += bytes;
      };
      back(r.out_index, per, 4);
      back(r.out_value, per, 4);
      if (r.type == THEA_REQUEST_CLOSEST) back(r.out_point, 3, 4);
    }
    if (p.staging) THEA_CUDA_CHECK(cudaFreeAsync(p.staging, st));
    p.staging = nullptr;
  }
  THEA_CUDA_CHECK(cudaLaunchHostFunc(st, slot_finished_cb, &s));
}

void dispatcher_main(thea_server * sv) {
  if (!sv->cfg.test_executor) cudaSetDevice(sv->device);
  std::unique_lock<std::mutex> lk(sv->mu);
  while (true) {
    Clock::time_point now = Clock::now();
    bool any_busy = false;
    for (auto & sp : sv->slots) {
      ServeSlot & s = *sp;
      if (s.busy && sv->cfg.test_executor && now >= s.test_deadline) s.complete = true;
      if (s.busy && s.complete) finish_slot_locked(sv, s);
      any_busy = any_busy || s.busy;
    }
    if (!sv->retired.empty()) {
      lk.unlock();
      destroy_retired(sv);
      lk.lock();
    }
    if (sv->stopping && !any_busy) break;
    bool launched = false;
    if (!sv->stopping) {
      for (auto & sp : sv->slots) {
        ServeSlot & s = *sp;
        if (s.busy || sv->pending.empty()) continue;
        if (!form_batch_locked(sv, s)) break;
        s.busy = true;
        ++sv->batches;
        launched = true;
        if (sv->cfg.test_executor) {
          int64_t q = 0;
          for (ServePiece const & p : s.pieces) q += p.n;
          s.test_deadline = Clock::now() + std::chrono::nanoseconds((int64_t)sv->cfg.test_ns_per_query * q);
          continue;
        }
        std::vector<ServeMesh const *> pm;
        pm.reserve(s.pieces.size());
        for (ServePiece const & p : s.pieces) pm.push_back(&sv->meshes.at(p.req->r.mesh));
        lk.unlock();
        thea_status st = THEA_OK;
        try {
          launch_slot(sv, s, pm);
        } catch (Error const & e) {
          st = e.status;
        } catch (...) {
          st = THEA_ERR_INTERNAL;
        }
        if (st != THEA_OK) {
          // drain what was enqueued (the callback may or may not have been queued), then fail the batch
          cudaStreamSynchronize(s.active);
          cudaGetLastError();
          for (ServePiece & p : s.pieces)
            if (p.staging) cudaFree(p.staging);
        }
        lk.lock();
        if (st != THEA_OK) {
          s.launch_status = st;
          s.complete = true;
        }
      }
    }
    if (launched) continue;
    // sleep until a submit, a finished slot or stop (the test executor also wakes at its next deadline)
    Clock::time_point until = Clock::now() + std::chrono::milliseconds(50);
    if (sv->cfg.test_executor)
      for (auto & sp : sv->slots)
        if (sp->busy) until = std::min(until, sp->test_deadline);
    sv->cv.wait_until(lk, until);
  }
}

}  // namespace

thea_server * server_create(thea_server_config const & c) {
  for (int r : c.reserved) THEA_REQUIRE(r == 0, "server_create: reserved fields must be zero");
  THEA_REQUIRE(c.memory_budget_bytes >= 0 && c.slots >= 0 && c.max_batch_queries >= 0 && c.max_piece_queries >= 0 &&
                   c.small_request_queries >= 0 && c.max_wait_ms >= 0 && c.test_ns_per_query >= 0,
               "server_create: negative option");
  THEA_REQUIRE(c.width == 0 || c.width == 4 || c.width == 8, "server_create: width must be 4 or 8");
  THEA_REQUIRE(c.precision == THEA_PRECISION_FP32_REFERENCE || c.precision == THEA_PRECISION_FP64_RECHECK,
               "server_create: unknown precision");
  THEA_REQUIRE(c.max_leaf_size >= 0 && c.max_leaf_size <= 16, "server_create: max_leaf_size must be 0..16");
  std::unique_ptr<thea_server> sv(new thea_server);
  thea_server_config & cfg = sv->cfg;
  cfg = c;
  if (!cfg.memory_budget_bytes) cfg.memory_budget_bytes = int64_t(8) << 30;
  if (!cfg.slots) cfg.slots = 6;
  if (!cfg.max_batch_queries) cfg.max_batch_queries = 65536;
  if (!cfg.max_piece_queries) cfg.max_piece_queries = 65536;
  cfg.max_piece_queries = std::min(cfg.max_piece_queries, cfg.max_batch_queries);
  if (!cfg.width) cfg.width = 4;
  if (!cfg.small_request_queries) cfg.small_request_queries = 65536;
  if (!cfg.max_wait_ms) cfg.max_wait_ms = 20;
  THEA_REQUIRE(cfg.slots <= 16, "server_create: at most 16 slots");
  if (!cfg.test_executor) THEA_CUDA_CHECK(cudaGetDevice(&sv->device));
  for (int i = 0; i < cfg.slots; ++i) {
    std::unique_ptr<ServeSlot> s(new ServeSlot);
    s->owner = sv.get();
    if (!cfg.test_executor) {
      int least = 0, greatest = 0;
      THEA_CUDA_CHECK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
      THEA_CUDA_CHECK(cudaStreamCreateWithPriority(&s->stream, cudaStreamNonBlocking, least));
      THEA_CUDA_CHECK(cudaStreamCreateWithPriority(&s->express, cudaStreamNonBlocking, greatest));
      s->active = s->stream;
      THEA_CUDA_CHECK(thea_malloc(&s->d_tasks, sizeof(ServeTask) * 3 * MAX_TASKS));
      THEA_CUDA_CHECK(thea_malloc_host(&s->h_tasks, sizeof(ServeTask) * 3 * MAX_TASKS));
      THEA_CUDA_CHECK(thea_malloc(&s->d_off, sizeof(int64_t) * 3 * (MAX_TASKS + 1)));
      THEA_CUDA_CHECK(thea_malloc_host(&s->h_off, sizeof(int64_t) * 3 * (MAX_TASKS + 1)));
      THEA_CUDA_CHECK(thea_malloc(&s->d_counters, 5 * sizeof(unsigned long long)));
    }
    sv->slots.push_back(std::move(s));
  }
  thea_server * raw = sv.release();
  raw->dispatcher = std::thread(dispatcher_main, raw);
  return raw;
}

void server_destroy(thea_server * sv) {
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    for (ServeRequest * q : sv->pending) {
      q->cancelled = true;
      q->scheduled = q->r.num_queries;  // nothing more will be packed
      if (q->pieces_done == q->pieces) end_request_locked(sv, q, THEA_ERR_CANCELLED);
    }
    sv->pending.clear();
    sv->stopping = true;
  }
  sv->cv.notify_all();
  sv->dispatcher.join();
  if (!sv->cfg.test_executor)
    for (auto & sp : sv->slots) {
      ServeSlot & s = *sp;
      for (cudaStream_t t : {s.stream, s.express}) {
        if (!t) continue;
        cudaStreamSynchronize(t);
        cudaStreamDestroy(t);
      }
      cudaFree(s.d_tasks);
      cudaFreeHost(s.h_tasks);
      cudaFree(s.d_off);
      cudaFreeHost(s.h_off);
      cudaFree(s.d_counters);
    }
  if (!sv->cfg.test_executor) {
    destroy_retired(sv);
    for (auto & kv : sv->meshes) {
      destroy_bvh(kv.second.mesh);
      destroy_bvh(kv.second.pts);
    }
  }
  delete sv;
}

int32_t server_add_mesh(thea_server * sv, float const * V, int64_t nv, int32_t const * F, int64_t nf) {
  THEA_REQUIRE(V && F && nv > 0 && nf > 0, "server_add_mesh: empty or null mesh");
  // size estimate before building: records (CP + ray) and nodes of the mesh BVH, point records and nodes of the vertex BVH
  int64_t est = nf * (int64_t)(CP_REC_F4 + RAY_REC_F4) * 16 + nf * 48 + nv * 16 + nv * 48;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    if (sv->resident_bytes + sv->inflight_bytes + est > sv->cfg.memory_budget_bytes)
      throw Error(THEA_ERR_ADMISSION_REFUSED, "server_add_mesh: the mesh does not fit the memory budget");
  }
  ServeMesh m;
  if (sv->cfg.test_executor) {
    m.bytes = est;
  } else {
    cudaStream_t st = nullptr;
    THEA_CUDA_CHECK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    // vertices and faces may be host arrays: the builders stage them
    thea_build_config mc{};
    mc.width = sv->cfg.width;
    mc.max_leaf_size = sv->cfg.max_leaf_size;
    mc.layouts = THEA_LAYOUT_CLOSEST | THEA_LAYOUT_RAY;
    thea_build_config pc{};
    pc.width = sv->cfg.width;
    float const * dV = V;
    int32_t const * dF = F;
    void * tv = nullptr, * tf = nullptr;
    try {
      if (host_memory(V)) {
        THEA_CUDA_CHECK(thea_malloc(&tv, (size_t)nv * 12));
        THEA_CUDA_CHECK(cudaMemcpyAsync(tv, V, (size_t)nv * 12, cudaMemcpyHostToDevice, st));
        dV = (float const *)tv;
      }
      if (host_memory(F)) {
        THEA_CUDA_CHECK(thea_malloc(&tf, (size_t)nf * 12));
        THEA_CUDA_CHECK(cudaMemcpyAsync(tf, F, (size_t)nf * 12, cudaMemcpyHostToDevice, st));
        dF = (int32_t const *)tf;
      }
      m.mesh = build_bvh(true, dV, nv, dF, nf, mc, st);
      m.pts = build_bvh(false, dV, nv, nullptr, 0, pc, st);
      THEA_CUDA_CHECK(cudaStreamSynchronize(st));
    } catch (...) {
      cudaStreamSynchronize(st);
      cudaFree(tv);
      cudaFree(tf);
      cudaStreamDestroy(st);
      if (m.mesh) destroy_bvh(m.mesh);
      if (m.pts) destroy_bvh(m.pts);
      throw;
    }
    cudaFree(tv);
    cudaFree(tf);
    cudaStreamDestroy(st);
    m.bytes = m.mesh->device_bytes + m.pts->device_bytes;
    m.scene_scale = scene_scale_of(m.mesh);
  }
  std::lock_guard<std::mutex> lk(sv->mu);
  if (sv->resident_bytes + sv->inflight_bytes + m.bytes > sv->cfg.memory_budget_bytes) {
    if (!sv->cfg.test_executor) {
      destroy_bvh(m.mesh);
      destroy_bvh(m.pts);
    }
    throw Error(THEA_ERR_ADMISSION_REFUSED, "server_add_mesh: the mesh does not fit the memory budget");
  }
  int32_t id = sv->next_mesh++;
  m.refs = 1;  // held by the server until removed
  sv->resident_bytes += m.bytes;
  sv->meshes[id] = m;
  return id;
}

void server_remove_mesh(thea_server * sv, int32_t id) {
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    auto it = sv->meshes.find(id);
    THEA_REQUIRE(it != sv->meshes.end() && !it->second.removing, "server_remove_mesh: no such mesh");
    it->second.removing = true;
    release_mesh_locked(sv, id);
  }
  destroy_retired(sv);
}

uint64_t server_submit(thea_server * sv, thea_request const & r) {
  THEA_REQUIRE(r.type == THEA_REQUEST_CLOSEST || r.type == THEA_REQUEST_RAY || r.type == THEA_REQUEST_KNN,
               "server_submit: unknown request type");
  THEA_REQUIRE(r.num_queries >= 1, "server_submit: a request needs at least one query");
  THEA_REQUIRE(r.queries && r.out_index, "server_submit: null queries or out_index");
  THEA_REQUIRE(r.type != THEA_REQUEST_RAY || r.directions, "server_submit: a ray request needs directions");
  THEA_REQUIRE(r.type != THEA_REQUEST_KNN || (r.k >= 1 && r.k <= 32), "server_submit: k must be in 1..32");
  std::unique_ptr<ServeRequest> q(new ServeRequest);
  q->r = r;
  if (r.type != THEA_REQUEST_KNN) q->r.k = 1;
  if (r.type != THEA_REQUEST_CLOSEST) q->r.out_point = nullptr;
  if (r.type != THEA_REQUEST_RAY) q->r.directions = nullptr;
  if (!sv->cfg.test_executor) {
    bool hin = host_memory(q->r.queries), hdir = host_memory(q->r.directions);
    bool hout = host_memory(q->r.out_index), hval = host_memory(q->r.out_value), hpt = host_memory(q->r.out_point);
    THEA_REQUIRE(!q->r.directions || hin == hdir, "server_submit: origins and directions must both be host or device");
    THEA_REQUIRE((!q->r.out_value || hval == hout) && (!q->r.out_point || hpt == hout),
                 "server_submit: outputs must all be host or all device memory");
    q->stage_in = hin;
    q->stage_out = hout;
  } else {
    q->stage_in = q->stage_out = true;
  }
  int64_t per_out = q->r.type == THEA_REQUEST_KNN ? q->r.k : 1;
  int64_t in_b = q->r.type == THEA_REQUEST_RAY ? 24 : 12;
  int64_t out_b = per_out * 4 * (1 + (q->r.out_value ? 1 : 0)) + (q->r.out_point ? 12 : 0);
  q->bytes_per_query = (q->stage_in ? in_b : 0) + (q->stage_out ? out_b : 0);
  std::unique_lock<std::mutex> lk(sv->mu);
  THEA_REQUIRE(!sv->stopping, "server_submit: the server is shutting down");
  auto it = sv->meshes.find(r.mesh);
  THEA_REQUIRE(it != sv->meshes.end() && !it->second.removing, "server_submit: no such mesh");
  int64_t smallest = std::min<int64_t>(r.num_queries, sv->cfg.max_piece_queries) * q->bytes_per_query;
  ++sv->submitted;
  if (smallest > sv->cfg.memory_budget_bytes - sv->resident_bytes) {
    ++sv->refused;
    throw Error(THEA_ERR_ADMISSION_REFUSED, "server_submit: the request's smallest piece exceeds the memory budget");
  }
  ++it->second.refs;
  q->ticket = sv->next_ticket++;
  q->submitted = Clock::now();
  if (!sv->have_first) {
    sv->have_first = true;
    sv->first_submit = q->submitted;
  }
  uint64_t t = q->ticket;
  sv->pending.push_back(q.get());
  sv->requests[t] = std::move(q);
  lk.unlock();
  sv->cv.notify_all();
  return t;
}

thea_status server_wait(thea_server * sv, uint64_t ticket, int64_t timeout_us, thea_status * request_status,
                        double * latency_ms) {
  std::unique_lock<std::mutex> lk(sv->mu);
  auto it = sv->requests.find(ticket);
  THEA_REQUIRE(it != sv->requests.end(), "server_wait: unknown or retired ticket");
  ServeRequest * q = it->second.get();
  auto ready = [&] { return q->done; };
  if (timeout_us < 0) sv->cv_done.wait(lk, ready);
  else if (!sv->cv_done.wait_for(lk, std::chrono::microseconds(timeout_us), ready)) return THEA_ERR_WAIT_TIMEOUT;
  if (request_status) *request_status = q->status;
  if (latency_ms) *latency_ms = ms_between(q->submitted, q->finished);
  sv->requests.erase(it);
  return THEA_OK;
}

void server_cancel(thea_server * sv, uint64_t ticket) {
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    auto it = sv->requests.find(ticket);
    THEA_REQUIRE(it != sv->requests.end(), "server_cancel: unknown or retired ticket");
    ServeRequest * q = it->second.get();
    if (q->done) return;
    q->cancelled = true;
    auto pit = std::find(sv->pending.begin(), sv->pending.end(), q);
    if (pit != sv->pending.end()) sv->pending.erase(pit);
    q->scheduled = q->r.num_queries;  // no further pieces
    if (q->pieces_done == q->pieces) end_request_locked(sv, q, THEA_ERR_CANCELLED);
  }
  destroy_retired(sv);
}

void server_stats(thea_server * sv, thea_server_stats * o) {
  std::lock_guard<std::mutex> lk(sv->mu);
  std::memset(o, 0, sizeof(*o));
  o->submitted = sv->submitted;
  o->completed = sv->completed;
  o->failed = sv->failed;
  o->cancelled = sv->cancelled;
  o->refused = sv->refused;
  o->queries_completed = sv->queries_completed;
  o->batches = sv->batches;
  o->resident_meshes = 0;
  for (auto const & kv : sv->meshes)
    if (!kv.second.removing) ++o->resident_meshes;
  o->resident_bytes = sv->resident_bytes;
  o->inflight_bytes = sv->inflight_bytes;
  o->pending_requests = (int64_t)sv->pending.size();
  o->p50_ms = percentile(sv->lat, 0.50);
  o->p99_ms = percentile(sv->lat, 0.99);
  o->max_ms = sv->lat.empty() ? 0.0 : *std::max_element(sv->lat.begin(), sv->lat.end());
  o->small_p50_ms = percentile(sv->lat_small, 0.50);
  o->small_p99_ms = percentile(sv->lat_small, 0.99);
  if (sv->have_first && sv->completed) {
    o->busy_seconds = std::max(0.0, ms_between(sv->first_submit, sv->last_finish) / 1e3);
    o->queries_per_second = o->busy_seconds > 0 ? (double)sv->queries_completed / o->busy_seconds : 0.0;
  }
}

void server_reset_stats(thea_server * sv) {
  std::lock_guard<std::mutex> lk(sv->mu);
  sv->submitted = sv->completed = sv->failed = sv->cancelled = sv->refused = sv->queries_completed = sv->batches = 0;
  sv->lat.clear();
  sv->lat_small.clear();
  sv->have_first = false;
}

}  // namespace thea
