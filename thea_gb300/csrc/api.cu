// The C ABI (include/thea_gpu.h): argument checks, status codes, host-pointer staging, launch accounting and event
// timing. Nothing throws across the boundary.
#include "bvh.hpp"
#include "device_util.cuh"
#include "query.hpp"
#include "batch.hpp"
#include "serve.hpp"
#include "gram.hpp"
#include "serialize.hpp"
#include "transform.hpp"
#include "visibility.hpp"
#include "sample_graph.hpp"
#include "mesh_io.hpp"
#include "shape_diameter.hpp"
#include "bounding_sphere.hpp"
#include "pairs.hpp"
#include "traverse.cuh"

#include <initializer_list>
#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <vector>

namespace thea {

//============================================================================================================================
// Launch accounting and optional per-kernel event timing
//============================================================================================================================

static std::atomic<int64_t> g_launches{0};
static std::atomic<int64_t> g_allocations{0};

void note_allocation() { g_allocations.fetch_add(1, std::memory_order_relaxed); }
static std::atomic<bool> g_profiling{false};

struct TimedLaunch {
  std::string name;
  cudaEvent_t begin, end;
};
static std::mutex g_prof_mutex;
static std::vector<TimedLaunch> g_prof;

void note_launch(char const * kernel_name, cudaStream_t stream, cudaEvent_t * begin_event) {
  (void)kernel_name;
  g_launches.fetch_add(1, std::memory_order_relaxed);
  *begin_event = nullptr;
  if (g_profiling.load(std::memory_order_relaxed)) {
    if (cudaEventCreate(begin_event) == cudaSuccess) cudaEventRecord(*begin_event, stream);
    else *begin_event = nullptr;
  }
}

void note_launch_end(char const * kernel_name, cudaStream_t stream, cudaEvent_t begin_event) {
  if (!begin_event) return;
  cudaEvent_t end = nullptr;
  if (cudaEventCreate(&end) != cudaSuccess) {
    cudaEventDestroy(begin_event);
    return;
  }
  cudaEventRecord(end, stream);
  std::lock_guard<std::mutex> lk(g_prof_mutex);
  g_prof.push_back(TimedLaunch{kernel_name, begin_event, end});
}

//============================================================================================================================
// Scratch memory pool
//============================================================================================================================

cudaMemPool_t scratch_pool() {
  static std::mutex m;
  static std::map<int, cudaMemPool_t> pools;
  int dev = 0;
  THEA_CUDA_CHECK(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(m);
  auto it = pools.find(dev);
  if (it != pools.end()) return it->second;
  cudaMemPoolProps props = {};
  props.allocType = cudaMemAllocationTypePinned;
  props.handleTypes = cudaMemHandleTypeNone;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = dev;
  cudaMemPool_t pool;
  THEA_CUDA_CHECK(cudaMemPoolCreate(&pool, &props));
  uint64_t keep = ~uint64_t(0);
  THEA_CUDA_CHECK(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
  pools[dev] = pool;
  return pool;
}

//============================================================================================================================
// Status plumbing
//============================================================================================================================

static thread_local std::string g_error;

template <class F> static thea_status guarded(F && f) {
  try {
    f();
    return THEA_OK;
  } catch (Error const & e) {
    g_error = e.what();
    return e.status;
  } catch (std::bad_alloc const &) {
    g_error = "host allocation failed";
    return THEA_ERR_OUT_OF_MEMORY;
  } catch (std::exception const & e) {
    g_error = e.what();
    return THEA_ERR_INTERNAL;
  } catch (...) {
    g_error = "unknown error";
    return THEA_ERR_INTERNAL;
  }
}

//============================================================================================================================
// Device error bits -> status
//
// Query kernels raise bits in their handle's device error word (a traversal stack that would overflow, a tensor-core
// wait that gave up). Every query call ends by copying the word into the handle's pinned host mirror on its stream. A
// call that synchronizes (host arrays) then reads the mirror before it returns; every call first reads what earlier,
// asynchronous calls left there. Bits are reported once: the call that reports them clears the word and the mirror.
//============================================================================================================================

static thread_local bool t_synced = false;  // set by a query call that synchronized its stream

static void sync_stream(cudaStream_t s) {
  THEA_CUDA_CHECK(cudaStreamSynchronize(s));
  t_synced = true;
}

// Takes the bits the mirror holds (clearing the mirror and, on the stream, the device word).
static unsigned take_device_errors(thea_bvh const * b, cudaStream_t s) {
  if (!b || !b->err_host) return 0;
  unsigned bits = *(volatile unsigned *)b->err_host;
  if (!bits) return 0;
  *(volatile unsigned *)b->err_host = 0;
  THEA_CUDA_CHECK(cudaMemsetAsync(b->err, 0, sizeof(unsigned), s));
  return bits;
}

static void raise_device_errors(unsigned bits) {
  if (!bits) return;
  if (bits & ERR_STACK_OVERFLOW)
    throw Error(THEA_ERR_INTERNAL, "a traversal stack overflowed on this BVH: results of the calls since the last "
                                   "report may miss elements");
  throw Error(THEA_ERR_DEVICE_TIMEOUT, "a tensor-core wait gave up on this BVH; the affected queries were answered by "
                                       "the plain search (results are exact)");
}

// Runs a query call on handle b and reports device error bits: those earlier asynchronous calls left in the mirror, and
// those of this call when it synchronized. The call's own work runs (and writes its results) either way.
template <class F> static thea_status guarded_query(thea_bvh const * b, void * stream, F && f) {
  return guarded([&] {
    cudaStream_t s = (cudaStream_t)stream;
    unsigned bits = take_device_errors(b, s);
    t_synced = false;
    f();
    if (b && b->err_host) {
      THEA_CUDA_CHECK(cudaMemcpyAsync(b->err_host, b->err, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
      if (t_synced) {
        THEA_CUDA_CHECK(cudaStreamSynchronize(s));
        bits |= take_device_errors(b, s);
      }
    }
    raise_device_errors(bits);
  });
}

//============================================================================================================================
// Host-pointer staging
//============================================================================================================================

static bool is_host_pointer(void const * p) {
  if (!p) return false;
  cudaPointerAttributes a;
  cudaError_t e = cudaPointerGetAttributes(&a, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return true;
  }
  return !(a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged);
}

// True for device memory of the current device and for managed memory; false for host memory and for device memory
// of another GPU (a kernel on this device would fault on it unless peer access happens to be enabled).
static bool is_device_memory_here(void const * p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type == cudaMemoryTypeManaged) return true;
  if (a.type != cudaMemoryTypeDevice) return false;
  int dev = -1;
  THEA_CUDA_CHECK(cudaGetDevice(&dev));
  return a.device == dev;
}

// Device-usable addresses of caller arrays that are all pinned host memory (null entries are skipped); false if any
// array is device or pageable memory.
static bool pinned_host_views(std::initializer_list<void const *> ptrs, std::vector<void *> & out) {
  out.clear();
  for (void const * p : ptrs) {
    if (!p) {
      out.push_back(nullptr);
      continue;
    }
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    if (at.type != cudaMemoryTypeHost || !at.devicePointer) return false;
    out.push_back(at.devicePointer);
  }
  return true;
}

// Two non-blocking copy/compute streams per device, created once, used to overlap chunk transfers with kernels.
static std::array<cudaStream_t, 2> staging_streams() {
  static std::mutex m;
  static std::map<int, std::array<cudaStream_t, 2>> streams;
  int dev = 0;
  THEA_CUDA_CHECK(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(m);
  auto it = streams.find(dev);
  if (it != streams.end()) return it->second;
  std::array<cudaStream_t, 2> s;
  for (auto & x : s) THEA_CUDA_CHECK(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
  streams[dev] = s;
  return s;
}

struct IoArray {
  void * ptr;         // caller pointer (may be null for optional outputs)
  size_t elem_bytes;  // bytes per query
  bool output;
  bool host;
};

// Runs fn(begin, count, device_pointers, stream) over [0, n). Device-resident calls run once, asynchronously, on the
// caller's stream. If any array is host memory, the range is processed in chunks alternating between two staging
// streams (copy in, kernel, copy out), ordered after prior work on `stream`; the call returns once the results are in
// host memory.
template <class Fn> static void run_staged(std::vector<IoArray> arrays, int64_t n, cudaStream_t stream, Fn && fn) {
  bool any_host = false;
  size_t host_bytes = 0;
  for (auto & a : arrays) {
    a.host = a.ptr && is_host_pointer(a.ptr);
    if (a.host) {
      any_host = true;
      host_bytes += a.elem_bytes;
    }
  }
  if (!any_host) {
    std::vector<void *> ptrs;
    for (auto & a : arrays) ptrs.push_back(a.ptr);
    fn((int64_t)0, n, ptrs, stream);
    return;
  }
  if (n <= 0) return;
  t_synced = true;
  int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(n, (int64_t)((64u << 20) / host_bytes)));
  // four chunks: enough to overlap copies with kernels, few enough that kernel tails stay small (measured on the
  // 4.2 M-ray heightfield: 2 / 4 / 8 / 16 chunks gave 2,549 / 2,634 / 2,254 / 1,688 M rays/s end to end)
  chunk = std::min<int64_t>(chunk, std::max<int64_t>(1 << 16, ceil_div(n, 4)));
  auto ss = staging_streams();
  Scratch buf0((size_t)chunk * host_bytes, stream), buf1((size_t)chunk * host_bytes, stream);
  cudaEvent_t ready, done0, done1;
  THEA_CUDA_CHECK(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
  THEA_CUDA_CHECK(cudaEventCreateWithFlags(&done0, cudaEventDisableTiming));
  THEA_CUDA_CHECK(cudaEventCreateWithFlags(&done1, cudaEventDisableTiming));
  THEA_CUDA_CHECK(cudaEventRecord(ready, stream));
  THEA_CUDA_CHECK(cudaStreamWaitEvent(ss[0], ready, 0));
  THEA_CUDA_CHECK(cudaStreamWaitEvent(ss[1], ready, 0));
  std::exception_ptr failure;
  try {
    for (int64_t c = 0; c * chunk < n; ++c) {
      int64_t begin = c * chunk, cnt = std::min(chunk, n - begin);
      cudaStream_t s = ss[c & 1];
      char * base = (c & 1) ? buf1.as<char>() : buf0.as<char>();
      std::vector<void *> ptrs;
      size_t off = 0;
      for (auto & a : arrays) {
        if (!a.ptr) { ptrs.push_back(nullptr); continue; }
        if (a.host) {
          void * dev = base + off;
          off += (size_t)chunk * a.elem_bytes;
          if (!a.output)
            THEA_CUDA_CHECK(cudaMemcpyAsync(dev, (char const *)a.ptr + begin * a.elem_bytes, cnt * a.elem_bytes,
                                            cudaMemcpyHostToDevice, s));
          ptrs.push_back(dev);
        } else {
          ptrs.push_back((char *)a.ptr + begin * a.elem_bytes);
        }
      }
      fn(begin, cnt, ptrs, s);
      for (size_t i = 0; i < arrays.size(); ++i) {
        auto & a = arrays[i];
        if (a.ptr && a.host && a.output)
          THEA_CUDA_CHECK(cudaMemcpyAsync((char *)a.ptr + begin * a.elem_bytes, ptrs[i], cnt * a.elem_bytes,
                                          cudaMemcpyDeviceToHost, s));
      }
    }
  } catch (...) {
    failure = std::current_exception();
  }
  cudaEventRecord(done0, ss[0]);
  cudaEventRecord(done1, ss[1]);
  cudaStreamWaitEvent(stream, done0, 0);
  cudaStreamWaitEvent(stream, done1, 0);
  buf0.release();
  buf1.release();
  cudaError_t se = cudaStreamSynchronize(stream);
  cudaEventDestroy(ready);
  cudaEventDestroy(done0);
  cudaEventDestroy(done1);
  if (failure) std::rethrow_exception(failure);
  THEA_CUDA_CHECK(se);
}

// Copies a whole host array to a new device buffer (or passes device memory through).
struct DeviceView {
  Scratch owned;
  void const * ptr = nullptr;
  DeviceView(void const * p, size_t bytes, cudaStream_t s) {
    if (p && is_host_pointer(p)) {
      owned = Scratch(bytes, s);
      THEA_CUDA_CHECK(cudaMemcpyAsync(owned.ptr, p, bytes, cudaMemcpyHostToDevice, s));
      ptr = owned.ptr;
    } else {
      ptr = p;
    }
  }
};

// Largest float f with (double)f < bound^2: an element is accepted iff its FP32 squared distance d2 <= f, which is the
// reference's test (double)d2 < dist_bound * dist_bound (BvhN.hpp:1094, 451-466, 490-494). +inf when unbounded.
static float bound_threshold(float dist_bound) {
  if (!(dist_bound >= 0.f)) return INFINITY;
  double b2 = (double)dist_bound * (double)dist_bound;
  float f = (float)b2;
  if ((double)f >= b2) f = std::nextafter(f, -INFINITY);
  return f;
}

static unsigned * handle_error_word(thea_bvh const * b) { return b->err; }

}  // namespace thea

using namespace thea;

//============================================================================================================================
// C entry points
//============================================================================================================================

extern "C" {

THEA_API int thea_abi_version(void) { return THEA_GPU_ABI_VERSION; }

THEA_API const char * thea_status_string(thea_status s) {
  switch (s) {
    case THEA_OK: return "ok";
    case THEA_ERR_INVALID_ARGUMENT: return "invalid argument";
    case THEA_ERR_OUT_OF_MEMORY: return "out of device memory";
    case THEA_ERR_ADMISSION_REFUSED: return "admission refused";
    case THEA_ERR_DEVICE_TIMEOUT: return "device-side wait timed out";
    case THEA_ERR_CUDA: return "CUDA error";
    case THEA_ERR_INTERNAL: return "internal error";
    case THEA_ERR_NOT_SUPPORTED: return "not supported";
    case THEA_ERR_CANCELLED: return "cancelled";
    case THEA_ERR_WAIT_TIMEOUT: return "wait timed out";
  }
  return "unknown status";
}

THEA_API const char * thea_last_error_message(void) { return g_error.c_str(); }

THEA_API int64_t thea_launch_count(void) { return g_launches.load(); }

THEA_API int64_t thea_allocation_count(void) { return g_allocations.load(); }

THEA_API thea_status thea_profiling_enable(int enable) {
  g_profiling.store(enable != 0);
  return THEA_OK;
}

THEA_API thea_status thea_profiling_reset(void) {
  return guarded([&] {
    std::lock_guard<std::mutex> lk(g_prof_mutex);
    for (auto & t : g_prof) {
      cudaEventSynchronize(t.end);
      cudaEventDestroy(t.begin);
      cudaEventDestroy(t.end);
    }
    g_prof.clear();
  });
}

THEA_API thea_status thea_profiling_read(const char * kernel_substring, double * total_ms, int64_t * launches) {
  return guarded([&] {
    THEA_REQUIRE(total_ms && launches, "profiling_read: null output");
    std::lock_guard<std::mutex> lk(g_prof_mutex);
    double sum = 0;
    int64_t cnt = 0;
    for (auto & t : g_prof) {
      if (kernel_substring && !strstr(t.name.c_str(), kernel_substring)) continue;
      THEA_CUDA_CHECK(cudaEventSynchronize(t.end));
      float ms = 0;
      THEA_CUDA_CHECK(cudaEventElapsedTime(&ms, t.begin, t.end));
      sum += ms;
      ++cnt;
    }
    *total_ms = sum;
    *launches = cnt;
  });
}

static void check_config(thea_build_config const * cfg) {
  if (!cfg) return;
  for (int i = 0; i < 4; ++i) THEA_REQUIRE(cfg->reserved[i] == 0, "build config: reserved fields must be zero");
  THEA_REQUIRE(cfg->query_order == 0 || cfg->query_order == 1, "build config: query_order must be 0 or 1");
}

THEA_API thea_status thea_mesh_bvh_build(const float * vertices, int64_t num_vertices, const int32_t * faces,
                                         int64_t num_faces, const thea_build_config * config, void * stream,
                                         thea_bvh ** out_bvh) {
  return guarded([&] {
    THEA_REQUIRE(out_bvh, "mesh_bvh_build: out_bvh is null");
    *out_bvh = nullptr;
    THEA_REQUIRE(vertices && faces, "mesh_bvh_build: null vertices or faces");
    THEA_REQUIRE(num_vertices > 0 && num_faces > 0, "mesh_bvh_build: empty mesh");
    check_config(config);
    thea_build_config cfg{};
    if (config) cfg = *config;
    cudaStream_t s = (cudaStream_t)stream;
    DeviceView V(vertices, (size_t)num_vertices * 3 * sizeof(float), s);
    DeviceView F(faces, (size_t)num_faces * 3 * sizeof(int32_t), s);
    *out_bvh = build_bvh(true, (float const *)V.ptr, num_vertices, (int32_t const *)F.ptr, num_faces, cfg, s);
    sync_stream(s);
  });
}

THEA_API thea_status thea_point_bvh_build(const float * points, int64_t num_points, const thea_build_config * config,
                                          void * stream, thea_bvh ** out_bvh) {
  return guarded([&] {
    THEA_REQUIRE(out_bvh, "point_bvh_build: out_bvh is null");
    *out_bvh = nullptr;
    THEA_REQUIRE(points, "point_bvh_build: null points");
    THEA_REQUIRE(num_points > 0, "point_bvh_build: empty point set");
    check_config(config);
    thea_build_config cfg{};
    if (config) cfg = *config;
    THEA_REQUIRE(cfg.layouts == 0, "point_bvh_build: layouts apply to meshes only");
    cudaStream_t s = (cudaStream_t)stream;
    DeviceView P(points, (size_t)num_points * 3 * sizeof(float), s);
    *out_bvh = build_bvh(false, (float const *)P.ptr, num_points, nullptr, 0, cfg, s);
    sync_stream(s);
  });
}

THEA_API thea_status thea_bvh_destroy(thea_bvh * bvh) {
  return guarded([&] {
    if (!bvh) return;
    destroy_bvh(bvh);
  });
}

THEA_API thea_status thea_bvh_serialize(const thea_bvh * bvh, void * out_image, int64_t capacity, int64_t * out_bytes,
                                        void * stream) {
  return guarded([&] {
    THEA_REQUIRE(bvh && out_bytes, "bvh_serialize: null argument");
    THEA_REQUIRE(!out_image || is_host_pointer(out_image), "bvh_serialize: the image buffer must be host memory");
    *out_bytes = serialize_bvh(bvh, out_image, capacity, (cudaStream_t)stream);
  });
}

THEA_API thea_status thea_bvh_deserialize(const void * image, int64_t bytes, void * stream, thea_bvh ** out_bvh) {
  return guarded([&] {
    THEA_REQUIRE(out_bvh, "bvh_deserialize: null output");
    *out_bvh = nullptr;
    *out_bvh = deserialize_bvh(image, bytes, (cudaStream_t)stream);
  });
}

THEA_API thea_status thea_bvh_set_transform(thea_bvh * bvh, const float * affine_3x4, void * stream) {
  return guarded([&] { set_transform(bvh, affine_3x4, (cudaStream_t)stream); });
}

THEA_API thea_status thea_bvh_clear_transform(thea_bvh * bvh) {
  return guarded([&] {
    THEA_REQUIRE(bvh, "bvh_clear_transform: null handle");
    clear_transform(bvh);
  });
}

THEA_API thea_status thea_bvh_get_transform(const thea_bvh * bvh, int32_t * has_transform, float * affine_3x4,
                                            float * inverse_3x4) {
  return guarded([&] {
    THEA_REQUIRE(bvh && has_transform, "bvh_get_transform: null argument");
    *has_transform = bvh->has_transform;
    float const id[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
    if (affine_3x4) std::memcpy(affine_3x4, bvh->has_transform ? bvh->xf : id, sizeof(id));
    if (inverse_3x4) std::memcpy(inverse_3x4, bvh->has_transform ? bvh->xf_inv : id, sizeof(id));
  });
}

THEA_API thea_status thea_bvh_get_info(const thea_bvh * bvh, thea_bvh_info * info) {
  return guarded([&] {
    THEA_REQUIRE(bvh && info, "bvh_get_info: null argument");
    memset(info, 0, sizeof(*info));
    info->num_elements = bvh->n;
    info->num_nodes = bvh->num_nodes;
    info->width = bvh->width;
    info->max_leaf_size = bvh->leaf_size;
    info->is_mesh = bvh->is_mesh;
    info->depth = bvh->depth;
    info->num_segments = bvh->num_segments;
    info->device_bytes = bvh->device_bytes;
    for (int i = 0; i < 3; ++i) {
      info->bounds_lo[i] = bvh->lo[i];
      info->bounds_hi[i] = bvh->hi[i];
    }
    if (bvh->world) {
      for (int i = 0; i < 3; ++i) {
        info->bounds_lo[i] = bvh->world->lo[i];
        info->bounds_hi[i] = bvh->world->hi[i];
      }
    } else if (bvh->has_transform) {
      // world-space box of the transformed corners (AxisAlignedBoxN::transformAndBound)
      for (int i = 0; i < 3; ++i) info->bounds_lo[i] = INFINITY, info->bounds_hi[i] = -INFINITY;
      for (int c = 0; c < 8; ++c) {
        V3 w = affine_point(bvh->xf, V3{(c & 1) ? bvh->hi[0] : bvh->lo[0], (c & 2) ? bvh->hi[1] : bvh->lo[1],
                                        (c & 4) ? bvh->hi[2] : bvh->lo[2]});
        float wc[3] = {w.x, w.y, w.z};
        for (int i = 0; i < 3; ++i) {
          info->bounds_lo[i] = std::min(info->bounds_lo[i], wc[i]);
          info->bounds_hi[i] = std::max(info->bounds_hi[i], wc[i]);
        }
      }
    }
    unsigned * w = handle_error_word(bvh);
    unsigned bits = 0;
    THEA_CUDA_CHECK(cudaMemcpy(&bits, w, sizeof(bits), cudaMemcpyDeviceToHost));
    info->device_error_bits = bits;
  });
}

static void closest_impl(const thea_bvh * mesh_bvh, const float * queries, int64_t num_queries, float dist_bound,
                         int32_t precision, int32_t * out_index, float * out_distance, float * out_closest_point,
                         float * out_error, void * stream) {
  THEA_REQUIRE(mesh_bvh && mesh_bvh->is_mesh, "closest_element: a mesh BVH is required");
  THEA_REQUIRE(mesh_bvh->cp_rec, "closest_element: the BVH was built without THEA_LAYOUT_CLOSEST");
  THEA_REQUIRE(precision == THEA_PRECISION_FP32_REFERENCE || precision == THEA_PRECISION_FP64_RECHECK,
               "closest_element: unknown precision mode");
  THEA_REQUIRE(num_queries >= 0, "closest_element: negative query count");
  if (num_queries == 0) return;
  THEA_REQUIRE(queries && out_index, "closest_element: null queries or out_index");
  // the reference's handling of dist_bound (root-box cut, loosened bound), from the handle's own (object-space) box
  BoundCut cut = closest_bound_cut(mesh_bvh, dist_bound);
  mesh_bvh = query_target(mesh_bvh);
  ClosestParams cp;
  cp.thresh = cut.thresh;
  cp.bound2 = cut.bound2;
  cp.precision = precision;
  cp.scene_scale = scene_scale_of(mesh_bvh);
  unsigned * err = handle_error_word(mesh_bvh);
  // queries and results all in pinned host memory (FP32, large batch): read and written in place by the kernels
  std::vector<void *> dp;
  if (precision == THEA_PRECISION_FP32_REFERENCE && !out_error && !mesh_bvh->query_order &&
      mesh_bvh->num_segments == 1 && num_queries >= (1 << 16) &&
      pinned_host_views({queries, out_index, out_distance, out_closest_point}, dp)) {
    ClosestParams c2 = cp;
    c2.budget = 256;  // the step budget of the device-resident two-phase path
    run_closest_stream(mesh_bvh, (float const *)dp[0], num_queries, c2, (int32_t *)dp[1], (float *)dp[2],
                       (float *)dp[3], (cudaStream_t)stream);
    run_closest_cut((float const *)dp[0], num_queries, cut, nullptr, 1, nullptr, (int32_t *)dp[1], (float *)dp[2],
                    (float *)dp[3], nullptr, (cudaStream_t)stream);
    sync_stream((cudaStream_t)stream);
    return;
  }
  run_staged({{(void *)queries, 12, false, false}, {out_index, 4, true, false}, {out_distance, 4, true, false},
              {out_closest_point, 12, true, false}, {out_error, 4, true, false}},
             num_queries, (cudaStream_t)stream,
             [&](int64_t, int64_t cnt, std::vector<void *> const & p, cudaStream_t s) {
               run_closest(mesh_bvh, (float const *)p[0], cnt, cp, (int32_t *)p[1], (float *)p[2], (float *)p[3],
                           (float *)p[4], err, s);
               run_closest_cut((float const *)p[0], cnt, cut, nullptr, 1, nullptr, (int32_t *)p[1], (float *)p[2],
                               (float *)p[3], (float *)p[4], s);
             });
}

static void ray_impl(const thea_bvh * mesh_bvh, const float * origins, const float * directions, int64_t num_rays,
                     float max_time, int32_t precision, float * out_time, int32_t * out_index, float * out_normal,
                     float * out_time64, int32_t * out_index64, int32_t * out_flags, void * stream) {
  THEA_REQUIRE(mesh_bvh && mesh_bvh->is_mesh, "ray_intersection: a mesh BVH is required");
  THEA_REQUIRE(mesh_bvh->ray_rec, "ray_intersection: the BVH was built without THEA_LAYOUT_RAY");
  THEA_REQUIRE(precision == THEA_PRECISION_FP32_REFERENCE || precision == THEA_PRECISION_FP64_RECHECK,
               "ray_intersection: unknown precision mode");
  THEA_REQUIRE(num_rays >= 0, "ray_intersection: negative ray count");
  if (num_rays == 0) return;
  THEA_REQUIRE(origins && directions && out_time, "ray_intersection: null origins, directions or out_time");
  unsigned * err = handle_error_word(mesh_bvh);
  RayParams rp;
  rp.max_time = max_time >= 0.f ? max_time : -1.f;
  rp.recheck = precision == THEA_PRECISION_FP64_RECHECK;
  if (!rp.recheck) out_time64 = nullptr, out_index64 = nullptr, out_flags = nullptr;
  // rays and results all in pinned host memory: one launch reads and writes them in place
  std::vector<void *> dp;
  if (!rp.recheck && !out_normal && !mesh_bvh->has_transform && num_rays >= (1 << 16) &&
      pinned_host_views({origins, directions, out_time, out_index}, dp)) {
    run_ray_stream(mesh_bvh, (float const *)dp[0], (float const *)dp[1], num_rays, rp.max_time, (float *)dp[2],
                   (int32_t *)dp[3], err, (cudaStream_t)stream);
    sync_stream((cudaStream_t)stream);
    return;
  }
  run_staged({{(void *)origins, 12, false, false}, {(void *)directions, 12, false, false}, {out_time, 4, true, false},
              {out_index, 4, true, false}, {out_normal, 12, true, false}, {out_time64, 4, true, false},
              {out_index64, 4, true, false}, {out_flags, 4, true, false}},
             num_rays, (cudaStream_t)stream,
             [&](int64_t, int64_t cnt, std::vector<void *> const & p, cudaStream_t s) {
               float const * o = (float const *)p[0];
               float const * d = (float const *)p[1];
               Scratch o_obj, d_obj;
               if (mesh_bvh->has_transform) {
                 o_obj = Scratch((size_t)cnt * 12, s);
                 d_obj = Scratch((size_t)cnt * 12, s);
                 rays_to_object(mesh_bvh, o, d, cnt, o_obj.as<float>(), d_obj.as<float>(), s);
                 o = o_obj.as<float>();
                 d = d_obj.as<float>();
               }
               run_ray(mesh_bvh, o, d, cnt, rp, (float *)p[2], (int32_t *)p[3], (float *)p[4], (float *)p[5],
                       (int32_t *)p[6], (int32_t *)p[7], err, s);
               if (mesh_bvh->has_transform) normals_to_world(mesh_bvh, (float *)p[4], cnt, s);
             });
}

THEA_API thea_status thea_closest_element(const thea_bvh * mesh_bvh, const float * queries, int64_t num_queries,
                                          float dist_bound, int32_t * out_index, float * out_distance,
                                          float * out_closest_point, void * stream) {
  return guarded_query(mesh_bvh, stream, [&] {
    closest_impl(mesh_bvh, queries, num_queries, dist_bound, THEA_PRECISION_FP32_REFERENCE, out_index, out_distance,
                 out_closest_point, nullptr, stream);
  });
}

THEA_API thea_status thea_closest_element_ex(const thea_bvh * mesh_bvh, const float * queries, int64_t num_queries,
                                             float dist_bound, int32_t precision, int32_t * out_index,
                                             float * out_distance, float * out_closest_point, float * out_error,
                                             void * stream) {
  return guarded_query(mesh_bvh, stream, [&] {
    closest_impl(mesh_bvh, queries, num_queries, dist_bound, precision, out_index, out_distance, out_closest_point,
                 out_error, stream);
  });
}

THEA_API thea_status thea_ray_intersection(const thea_bvh * mesh_bvh, const float * origins, const float * directions,
                                           int64_t num_rays, float max_time, float * out_time, int32_t * out_index,
                                           float * out_normal, void * stream) {
  return guarded_query(mesh_bvh, stream, [&] {
    ray_impl(mesh_bvh, origins, directions, num_rays, max_time, THEA_PRECISION_FP32_REFERENCE, out_time, out_index,
             out_normal, nullptr, nullptr, nullptr, stream);
  });
}

THEA_API thea_status thea_ray_intersection_ex(const thea_bvh * mesh_bvh, const float * origins,
                                              const float * directions, int64_t num_rays, float max_time,
                                              int32_t precision, float * out_time, int32_t * out_index,
                                              float * out_normal, float * out_time_fp64, int32_t * out_index_fp64,
                                              int32_t * out_flags, void * stream) {
  return guarded_query(mesh_bvh, stream, [&] {
    ray_impl(mesh_bvh, origins, directions, num_rays, max_time, precision, out_time, out_index, out_normal,
             out_time_fp64, out_index_fp64, out_flags, stream);
  });
}

THEA_API thea_status thea_ray_intersects(const thea_bvh * mesh_bvh, const float * origins, const float * directions,
                                         int64_t num_rays, float max_time, uint8_t * out_hit, void * stream) {
  return guarded_query(mesh_bvh, stream, [&] {
    THEA_REQUIRE(mesh_bvh && mesh_bvh->is_mesh, "ray_intersects: a mesh BVH is required");
    THEA_REQUIRE(mesh_bvh->ray_rec, "ray_intersects: the BVH was built without THEA_LAYOUT_RAY");
    THEA_REQUIRE(num_rays >= 0, "ray_intersects: negative ray count");
    if (num_rays == 0) return;
    THEA_REQUIRE(origins && directions && out_hit, "ray_intersects: null origins, directions or out_hit");
    float mt = max_time >= 0.f ? max_time : -1.f;
    run_staged({{(void *)origins, 12, false, false}, {(void *)directions, 12, false, false}, {out_hit, 1, true, false}},
               num_rays, (cudaStream_t)stream,
               [&](int64_t, int64_t cnt, std::vector<void *> const & p, cudaStream_t s) {
                 run_ray_intersects(mesh_bvh, (float const *)p[0], (float const *)p[1], cnt, mt, (uint8_t *)p[2], s);
               });
  });
}

THEA_API thea_status thea_random_sphere(uint32_t seed, int64_t count, float * out_directions, void * stream) {
  return guarded([&] {
    THEA_REQUIRE(count >= 0, "random_sphere: negative count");
    if (count == 0) return;
    THEA_REQUIRE(out_directions, "random_sphere: null output");
    cudaStream_t s = (cudaStream_t)stream;
    if (is_host_pointer(out_directions)) {
      Scratch d((size_t)count * 12, s);
      run_random_sphere(seed, count, d.as<float>(), s);
      THEA_CUDA_CHECK(cudaMemcpyAsync(out_directions, d.ptr, (size_t)count * 12, cudaMemcpyDeviceToHost, s));
      sync_stream(s);
    } else {
      run_random_sphere(seed, count, out_directions, s);
    }
  });
}

THEA_API thea_status thea_visibility(const thea_bvh * mesh_bvh, const float * positions, int64_t num_points,
                                     int32_t num_rays, uint32_t seed, double * out_fraction, void * stream) {
  return guarded_query(mesh_bvh, stream, [&] {
    THEA_REQUIRE(mesh_bvh && mesh_bvh->is_mesh, "visibility: a mesh BVH is required");
    THEA_REQUIRE(mesh_bvh->ray_rec, "visibility: the BVH was built without THEA_LAYOUT_RAY");
    THEA_REQUIRE(num_points >= 0, "visibility: negative point count");
    if (num_points == 0) return;
    THEA_REQUIRE(positions && out_fraction, "visibility: null positions or out_fraction");
    if (num_rays <= 0) num_rays = 100;  // Visibility::compute: DEFAULT_NUM_RAYS for a non-positive count
    THEA_REQUIRE((int64_t)num_points * num_rays < ((int64_t)1 << 31), "visibility: too many rays for one call");
    cudaStream_t s = (cudaStream_t)stream;
    Scratch pin, pout;
    float const * pos = positions;
    double * out = out_fraction;
    if (is_host_pointer(positions)) {
      pin = Scratch((size_t)num_points * 12, s);
      THEA_CUDA_CHECK(cudaMemcpyAsync(pin.ptr, positions, (size_t)num_points * 12, cudaMemcpyHostToDevice, s));
      pos = pin.as<float>();
    }
    bool host_out = is_host_pointer(out_fraction);
    if (host_out) {
      pout = Scratch((size_t)num_points * 8, s);
      out = pout.as<double>();
    }
    run_visibility(mesh_bvh, pos, num_points, num_rays, seed, out, s);
    if (host_out) {
      THEA_CUDA_CHECK(cudaMemcpyAsync(out_fraction, out, (size_t)num_points * 8, cudaMemcpyDeviceToHost, s));
      sync_stream(s);
    }
  });
}

// thea_sample_graph with or without an oversampling
static thea_status sample_graph_call(const float * positions, const float * normals, int64_t num_samples,
                                     bool oversampled, const float * dense, const float * dense_normals,
                                     int64_t num_dense,
                                     int32_t max_degree, uint32_t seed, const thea_bvh * surface,
                                     int32_t * out_neighbors, float * out_separations, int32_t * out_degree,
                                     float * out_avg_separation, void * stream) {
  return guarded([&] {
    THEA_REQUIRE(positions && out_neighbors, "sample_graph: null positions or out_neighbors");
    THEA_REQUIRE(!surface || (surface->is_mesh && surface->ray_rec),
                 "sample_graph: the surface must be a mesh BVH with THEA_LAYOUT_RAY");
    THEA_REQUIRE(max_degree >= 1 && max_degree <= 64, "sample_graph: max_degree must be in 1..64");
    if (oversampled) {
      THEA_REQUIRE(dense && num_dense >= 1, "sample_graph_oversampled: the oversampling is empty");
      THEA_REQUIRE(num_samples >= 1, "sample_graph_oversampled: no samples");
      THEA_REQUIRE(!normals || dense_normals, "sample_graph: samples with normals need dense normals");
    } else {
      THEA_REQUIRE(num_samples >= 2, "sample_graph: at least two samples are needed");
    }
    cudaStream_t s = (cudaStream_t)stream;
    size_t n = (size_t)num_samples, m = (size_t)max_degree;
    DeviceView pos(positions, n * 12, s), nrm(normals, n * 12, s);
    DeviceView dpos(dense, (size_t)num_dense * 12, s), dnrm(normals ? dense_normals : nullptr, (size_t)num_dense * 12, s);
    // outputs: device buffers, copied out when the caller's arrays are host memory; separations and degrees are
    // always produced when the final mean separation is asked for
    bool need_sep = out_separations || out_avg_separation, need_deg = out_degree || out_avg_separation;
    bool hn = is_host_pointer(out_neighbors);
    bool hs = out_separations && is_host_pointer(out_separations), hd = out_degree && is_host_pointer(out_degree);
    Scratch bn, bs, bd;
    SampleGraphOut o;
    o.neighbors = out_neighbors;
    o.separations = out_separations;
    o.degree = out_degree;
    if (hn) { bn = Scratch(n * m * 4, s); o.neighbors = bn.as<int32_t>(); }
    if (need_sep && (!out_separations || hs)) { bs = Scratch(n * m * 4, s); o.separations = bs.as<float>(); }
    if (need_deg && (!out_degree || hd)) { bd = Scratch(n * 4, s); o.degree = bd.as<int32_t>(); }
    if (oversampled)
      run_sample_graph_oversampled((float const *)pos.ptr, (float const *)nrm.ptr, num_samples,
                                   (float const *)dpos.ptr, (float const *)dnrm.ptr, num_dense, max_degree, seed,
                                   surface, o, s);
    else
      run_sample_graph((float const *)pos.ptr, (float const *)nrm.ptr, num_samples, max_degree, seed, surface, o, s);
    if (hn) THEA_CUDA_CHECK(cudaMemcpyAsync(out_neighbors, o.neighbors, n * m * 4, cudaMemcpyDeviceToHost, s));
    if (hs) THEA_CUDA_CHECK(cudaMemcpyAsync(out_separations, o.separations, n * m * 4, cudaMemcpyDeviceToHost, s));
    if (hd) THEA_CUDA_CHECK(cudaMemcpyAsync(out_degree, o.degree, n * 4, cudaMemcpyDeviceToHost, s));
    float avg = 0.f;
    Scratch bavg;
    if (out_avg_separation) {
      // updateAverageSeparation (PointSet3.hpp:688-702): FP32 sum over samples and their sorted neighbours, in order
      bavg = Scratch(sizeof(float), s);
      run_mean_separation(o.separations, o.degree, num_samples, max_degree, bavg.as<float>(), s);
      THEA_CUDA_CHECK(cudaMemcpyAsync(&avg, bavg.ptr, sizeof(float), cudaMemcpyDeviceToHost, s));
    }
    sync_stream(s);
    if (out_avg_separation) {
      out_avg_separation[0] = o.avg_separation_estimate;
      out_avg_separation[1] = avg;
    }
  });
}

THEA_API thea_status thea_sample_graph(const float * positions, const float * normals, int64_t num_samples,
                                       int32_t max_degree, uint32_t seed, const thea_bvh * surface,
                                       int32_t * out_neighbors, float * out_separations, int32_t * out_degree,
                                       float * out_avg_separation, void * stream) {
  return sample_graph_call(positions, normals, num_samples, false, nullptr, nullptr, 0, max_degree, seed, surface,
                           out_neighbors, out_separations, out_degree, out_avg_separation, stream);
}

THEA_API thea_status thea_sample_graph_oversampled(const float * positions, const float * normals,
                                                   int64_t num_samples, const float * dense_positions,
                                                   const float * dense_normals, int64_t num_dense,
                                                   int32_t max_degree, uint32_t seed, const thea_bvh * surface,
                                                   int32_t * out_neighbors, float * out_separations,
                                                   int32_t * out_degree, float * out_avg_separation, void * stream) {
  return sample_graph_call(positions, normals, num_samples, true, dense_positions, dense_normals, num_dense, max_degree,
                           seed, surface, out_neighbors, out_separations, out_degree, out_avg_separation, stream);
}

THEA_API thea_status thea_k_closest(const thea_bvh * point_bvh, const float * queries, int64_t num_queries, int32_t k,
                                    float dist_bound, const int32_t * exclude_index, int32_t * out_index,
                                    float * out_sq_distance, void * stream) {
  return guarded_query(point_bvh, stream, [&] {
    THEA_REQUIRE(point_bvh, "k_closest: null BVH");
    THEA_REQUIRE(point_bvh->num_segments == 1, "k_closest: forests take thea_batch_k_closest");
    THEA_REQUIRE(!point_bvh->is_mesh || query_target(point_bvh)->cp_rec,
                 "k_closest: the mesh BVH was built without THEA_LAYOUT_CLOSEST");
    THEA_REQUIRE(k >= 1 && k <= 32, "k_closest: k must be in 1..32");
    THEA_REQUIRE(num_queries >= 0, "k_closest: negative query count");
    if (num_queries == 0) return;
    THEA_REQUIRE(queries && out_index && out_sq_distance, "k_closest: null queries or outputs");
    point_bvh = query_target(point_bvh);
    float thresh = bound_threshold(dist_bound);
    unsigned * err = handle_error_word(point_bvh);
    run_staged({{(void *)queries, 12, false, false}, {(void *)exclude_index, 4, false, false},
                {out_index, (size_t)k * 4, true, false}, {out_sq_distance, (size_t)k * 4, true, false}},
               num_queries, (cudaStream_t)stream,
               [&](int64_t, int64_t cnt, std::vector<void *> const & p, cudaStream_t s) {
                 run_knn(point_bvh, (float const *)p[0], cnt, k, thresh, (int32_t const *)p[1], (int32_t *)p[2],
                         (float *)p[3], err, s);
               });
  });
}

static void knn_self_impl(const thea_bvh * point_bvh, int32_t k, int32_t candidates, int32_t * out_index,
                          float * out_sq_distance, void * stream) {
  THEA_REQUIRE(point_bvh && !point_bvh->is_mesh, "k_closest_self: a point BVH is required");
  THEA_REQUIRE(k >= 1 && k <= 32, "k_closest_self: k must be in 1..32");
  THEA_REQUIRE(candidates == THEA_KNN_CANDIDATES_TRAVERSAL || candidates == THEA_KNN_CANDIDATES_GRAM,
               "k_closest_self: unknown candidate mode");
  THEA_REQUIRE(out_index && out_sq_distance, "k_closest_self: null outputs");
  point_bvh = query_target(point_bvh);
  cudaStream_t s = (cudaStream_t)stream;
  unsigned * err = handle_error_word(point_bvh);
  int64_t n = point_bvh->n;
  // rows are written in element order, so host outputs are staged whole (written in place, the rows' scattered 4-byte
  // stores cross NVLink-C2C as partial sectors: 14.3 ms against 7.1 ms staged for 1 M points, k = 16)
  bool hi = is_host_pointer(out_index), hd = is_host_pointer(out_sq_distance);
  Scratch di, dd, bound;
  int32_t * pi = out_index;
  float * pd = out_sq_distance;
  if (hi) { di = Scratch((size_t)n * k * 4, s); pi = di.as<int32_t>(); }
  if (hd) { dd = Scratch((size_t)n * k * 4, s); pd = dd.as<float>(); }
  float const * ib = nullptr;
  if (candidates == THEA_KNN_CANDIDATES_GRAM && gram_supported(n)) {
    bound = Scratch((size_t)n * 4, s);
    run_gram_bounds(point_bvh, k, bound.as<float>(), s);
    ib = bound.as<float>();
  }
  run_knn(point_bvh, nullptr, n, k, INFINITY, nullptr, pi, pd, err, s, ib);
  if (hi) THEA_CUDA_CHECK(cudaMemcpyAsync(out_index, pi, (size_t)n * k * 4, cudaMemcpyDeviceToHost, s));
  if (hd) THEA_CUDA_CHECK(cudaMemcpyAsync(out_sq_distance, pd, (size_t)n * k * 4, cudaMemcpyDeviceToHost, s));
  if (hi || hd) sync_stream(s);
}

THEA_API thea_status thea_radius_neighbors(const thea_bvh * point_bvh, const float * queries, int64_t num_queries,
                                           float radius, const int32_t * exclude_index, int64_t * out_offsets,
                                           int32_t * out_index, float * out_sq_distance, void * stream) {
  return guarded_query(point_bvh, stream, [&] {
    THEA_REQUIRE(point_bvh && !point_bvh->is_mesh, "radius_neighbors: a point BVH is required");
    THEA_REQUIRE(num_queries >= 0, "radius_neighbors: negative query count");
    THEA_REQUIRE(radius >= 0.f, "radius_neighbors: negative or NaN radius");
    if (num_queries == 0) return;
    THEA_REQUIRE(queries && out_offsets, "radius_neighbors: null queries or out_offsets");
    void const * arrays[5] = {queries, exclude_index, out_offsets, out_index, out_sq_distance};
    for (void const * p : arrays)
      THEA_REQUIRE(!p || !is_host_pointer(p), "radius_neighbors: every array must be device memory");
    THEA_REQUIRE(out_index || !out_sq_distance, "radius_neighbors: out_sq_distance needs out_index");
    run_range(query_target(point_bvh), queries, num_queries, radius, exclude_index, out_offsets, out_index,
              out_sq_distance, handle_error_word(point_bvh), (cudaStream_t)stream);
  });
}

THEA_API thea_status thea_selftest_bounded_wait(int32_t spin_limit, void * stream) {
  thea_status r = THEA_OK;
  thea_status g = guarded([&] {
    THEA_REQUIRE(spin_limit >= 1 && spin_limit <= (1 << 20), "selftest_bounded_wait: spin_limit must be 1..2^20");
    if (run_wait_probe(spin_limit, (cudaStream_t)stream)) {
      g_error = "selftest_bounded_wait: the device wait gave up as designed";
      r = THEA_ERR_DEVICE_TIMEOUT;
    }
  });
  return g != THEA_OK ? g : r;
}

THEA_API thea_status thea_selftest_set_error_bits(thea_bvh * bvh, uint32_t bits, void * stream) {
  return guarded([&] {
    THEA_REQUIRE(bvh, "selftest_set_error_bits: null handle");
    cudaStream_t s = (cudaStream_t)stream;
    unsigned cur = 0;
    THEA_CUDA_CHECK(cudaMemcpyAsync(&cur, bvh->err, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    THEA_CUDA_CHECK(cudaStreamSynchronize(s));
    cur |= bits;
    THEA_CUDA_CHECK(cudaMemcpyAsync(bvh->err, &cur, sizeof(unsigned), cudaMemcpyHostToDevice, s));
    THEA_CUDA_CHECK(cudaStreamSynchronize(s));
  });
}

THEA_API thea_status thea_selftest_running_sum(const float * terms, int64_t num_terms, float start, float * out_sum,
                                               void * stream) {
  return guarded([&] {
    THEA_REQUIRE(out_sum && (terms || num_terms == 0) && num_terms >= 0, "selftest_running_sum: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    Scratch x((size_t)std::max<int64_t>(num_terms, 1) * sizeof(float), s), r(sizeof(float), s);
    if (num_terms > 0)
      THEA_CUDA_CHECK(cudaMemcpyAsync(x.ptr, terms, (size_t)num_terms * sizeof(float), cudaMemcpyDefault, s));
    run_running_sum(x.as<float>(), nullptr, num_terms, start, r.as<float>(), s);
    float h = 0.f;
    THEA_CUDA_CHECK(cudaMemcpyAsync(&h, r.ptr, sizeof(float), cudaMemcpyDeviceToHost, s));
    sync_stream(s);
    *out_sum = h;
  });
}

THEA_API thea_status thea_k_closest_self(const thea_bvh * point_bvh, int32_t k, int32_t * out_index,
                                         float * out_sq_distance, void * stream) {
  return guarded_query(point_bvh, stream, [&] {
    knn_self_impl(point_bvh, k, THEA_KNN_CANDIDATES_TRAVERSAL, out_index, out_sq_distance, stream);
  });
}

THEA_API thea_status thea_k_closest_self_ex(const thea_bvh * point_bvh, int32_t k, int32_t candidates,
                                            int32_t * out_index, float * out_sq_distance, void * stream) {
  return guarded_query(point_bvh, stream, [&] { knn_self_impl(point_bvh, k, candidates, out_index, out_sq_distance, stream); });
}

THEA_API thea_status thea_point_gram_tile(const float * a, int32_t num_a, const float * b, int32_t num_b,
                                          float * out_keys, void * stream) {
  return guarded([&] {
    THEA_REQUIRE(a && b && out_keys, "point_gram_tile: null argument");
    THEA_REQUIRE(num_a >= 1 && num_a <= gram_tile_rows() && num_b >= 1 && num_b <= gram_tile_cols(),
                 "point_gram_tile: at most 128 rows and 512 columns");
    THEA_REQUIRE(!is_host_pointer(a) && !is_host_pointer(b) && !is_host_pointer(out_keys),
                 "point_gram_tile: arrays must be device memory");
    run_gram_tile(a, num_a, b, num_b, out_keys, nullptr, (cudaStream_t)stream);
  });
}

THEA_API thea_status thea_sample_by_area(const float * vertices, int64_t num_vertices, const int32_t * faces,
                                         int64_t num_faces, int64_t num_samples, uint32_t seed, int32_t rng,
                                         float * out_positions, float * out_normals, int32_t * out_faces,
                                         int64_t * out_num_written, void * stream) {
  return guarded([&] {
    if (out_num_written) *out_num_written = 0;
    THEA_REQUIRE(rng == THEA_RNG_THEA_MT || rng == THEA_RNG_COUNTER, "sample_by_area: unknown rng");
    THEA_REQUIRE(num_samples >= 0, "sample_by_area: negative sample count");
    if (num_samples == 0) return;
    THEA_REQUIRE(vertices && faces && num_vertices > 0 && num_faces > 0, "sample_by_area: empty mesh");
    THEA_REQUIRE(out_positions, "sample_by_area: out_positions is null");
    cudaStream_t s = (cudaStream_t)stream;
    DeviceView V(vertices, (size_t)num_vertices * 3 * sizeof(float), s);
    DeviceView F(faces, (size_t)num_faces * 3 * sizeof(int32_t), s);
    struct Out {
      void * user;
      size_t bytes;
      Scratch dev;
      void * ptr;
    };
    Out o[3] = {{out_positions, (size_t)num_samples * 12, {}, nullptr},
                {out_normals, (size_t)num_samples * 12, {}, nullptr},
                {out_faces, (size_t)num_samples * 4, {}, nullptr}};
    for (auto & x : o) {
      x.ptr = x.user;
      if (x.user && is_host_pointer(x.user)) {
        x.dev = Scratch(x.bytes, s);
        x.ptr = x.dev.ptr;
      }
    }
    int64_t got = run_sample_by_area((float const *)V.ptr, num_vertices, (int32_t const *)F.ptr, num_faces, num_samples,
                                     seed, rng, (float *)o[0].ptr, (float *)o[1].ptr, (int32_t *)o[2].ptr, s);
    for (auto & x : o)
      if (x.dev.ptr && got > 0) THEA_CUDA_CHECK(cudaMemcpyAsync(x.user, x.ptr, x.bytes, cudaMemcpyDeviceToHost, s));
    sync_stream(s);
    if (out_num_written) *out_num_written = got;
  });
}

//---------------------------------------------------------------------------------------------------------------------------
// Forests, batched queries, graphs, autotuning
//---------------------------------------------------------------------------------------------------------------------------

THEA_API thea_status thea_mesh_forest_build(const float * vertices, int64_t num_vertices, const int32_t * faces,
                                            const int64_t * mesh_face_offsets, int32_t num_meshes,
                                            const thea_build_config * config, void * stream, thea_bvh ** out_forest) {
  return guarded([&] {
    THEA_REQUIRE(out_forest, "mesh_forest_build: out_forest is null");
    *out_forest = nullptr;
    THEA_REQUIRE(vertices && faces && mesh_face_offsets, "mesh_forest_build: null argument");
    THEA_REQUIRE(num_meshes >= 1 && num_vertices > 0, "mesh_forest_build: empty input");
    check_config(config);
    thea_build_config cfg{};
    if (config) cfg = *config;
    int64_t nf = mesh_face_offsets[num_meshes];
    THEA_REQUIRE(nf > 0, "mesh_forest_build: no faces");
    cudaStream_t s = (cudaStream_t)stream;
    DeviceView V(vertices, (size_t)num_vertices * 3 * sizeof(float), s);
    DeviceView F(faces, (size_t)nf * 3 * sizeof(int32_t), s);
    *out_forest = build_forest(true, (float const *)V.ptr, num_vertices, (int32_t const *)F.ptr, nf, mesh_face_offsets,
                               num_meshes, cfg, s);
    sync_stream(s);
  });
}

THEA_API thea_status thea_point_forest_build(const float * points, const int64_t * set_offsets, int32_t num_sets,
                                             const thea_build_config * config, void * stream,
                                             thea_bvh ** out_forest) {
  return guarded([&] {
    THEA_REQUIRE(out_forest, "point_forest_build: out_forest is null");
    *out_forest = nullptr;
    THEA_REQUIRE(points && set_offsets && num_sets >= 1, "point_forest_build: null or empty argument");
    check_config(config);
    thea_build_config cfg{};
    if (config) cfg = *config;
    THEA_REQUIRE(cfg.layouts == 0, "point_forest_build: layouts apply to meshes only");
    int64_t n = set_offsets[num_sets];
    THEA_REQUIRE(n > 0, "point_forest_build: no points");
    cudaStream_t s = (cudaStream_t)stream;
    DeviceView P(points, (size_t)n * 3 * sizeof(float), s);
    *out_forest = build_forest(false, (float const *)P.ptr, n, nullptr, n, set_offsets, num_sets, cfg, s);
    sync_stream(s);
  });
}

static int check_batch_common(const thea_bvh * f, const int64_t * qoff, int64_t nq, int32_t qpw,
                              std::initializer_list<void const *> arrays, char const * what) {
  THEA_REQUIRE(f, std::string(what) + ": null forest");
  THEA_REQUIRE(qoff, std::string(what) + ": null query offsets");
  THEA_REQUIRE(nq >= 0, std::string(what) + ": negative query count");
  int chunk = qpw == 0 ? 64 : qpw;
  THEA_REQUIRE(chunk >= 32 && chunk % 32 == 0 && chunk <= 4096,
               std::string(what) + ": queries_per_warp must be a multiple of 32 in 32..4096");
  THEA_REQUIRE(!is_host_pointer(qoff), std::string(what) + ": query offsets must be device memory");
  for (void const * p : arrays)
    THEA_REQUIRE(!p || !is_host_pointer(p), std::string(what) + ": every array must be device memory");
  return chunk;
}

THEA_API thea_status thea_batch_closest_element(const thea_bvh * mesh_forest, const float * queries,
                                                const int64_t * query_offsets, int64_t num_queries, float dist_bound,
                                                int32_t precision, int32_t queries_per_warp, int32_t hard_query_budget,
                                                int32_t * out_index, float * out_distance, float * out_closest_point,
                                                float * out_error, void * stream) {
  return guarded_query(mesh_forest, stream, [&] {
    int chunk = check_batch_common(mesh_forest, query_offsets, num_queries, queries_per_warp,
                                   {queries, out_index, out_distance, out_closest_point, out_error},
                                   "batch_closest_element");
    THEA_REQUIRE(mesh_forest->is_mesh && mesh_forest->cp_rec,
                 "batch_closest_element: a mesh forest with THEA_LAYOUT_CLOSEST is required");
    THEA_REQUIRE(precision == THEA_PRECISION_FP32_REFERENCE || precision == THEA_PRECISION_FP64_RECHECK,
                 "batch_closest_element: unknown precision mode");
    if (num_queries == 0) return;
    THEA_REQUIRE(queries && out_index, "batch_closest_element: null queries or out_index");
    ClosestParams cp;
    cp.precision = precision;
    cp.scene_scale = scene_scale_of(mesh_forest);
    cp.budget = hard_query_budget == 0 ? 32 : (hard_query_budget < 0 ? 0 : hard_query_budget);
    // each mesh applies the bound as closestElement on that mesh alone would (BoundCut): per-mesh cuts on the device
    cudaStream_t s = (cudaStream_t)stream;
    Scratch cuts;
    if (dist_bound >= 0.f) {
      cuts = Scratch((size_t)mesh_forest->num_segments * sizeof(BoundCut), s);
      run_segment_cuts(mesh_forest, dist_bound, cuts.as<BoundCut>(), s);
      cp.seg_cut = cuts.as<BoundCut>();
    }
    run_batch_closest(mesh_forest, queries, query_offsets, num_queries, cp, chunk, out_index, out_distance,
                      out_closest_point, out_error, s);
    if (dist_bound >= 0.f)
      run_closest_cut(queries, num_queries, BoundCut(), query_offsets, mesh_forest->num_segments, cuts.as<BoundCut>(),
                      out_index, out_distance, out_closest_point, out_error, s);
  });
}

THEA_API thea_status thea_batch_ray_intersection(const thea_bvh * mesh_forest, const float * origins,
                                                 const float * directions, const int64_t * query_offsets,
                                                 int64_t num_rays, float max_time, int32_t queries_per_warp,
                                                 float * out_time, int32_t * out_index, void * stream) {
  return guarded_query(mesh_forest, stream, [&] {
    int chunk = check_batch_common(mesh_forest, query_offsets, num_rays, queries_per_warp,
                                   {origins, directions, out_time, out_index}, "batch_ray_intersection");
    THEA_REQUIRE(mesh_forest->is_mesh && mesh_forest->ray_rec,
                 "batch_ray_intersection: a mesh forest with THEA_LAYOUT_RAY is required");
    if (num_rays == 0) return;
    THEA_REQUIRE(origins && directions && out_time, "batch_ray_intersection: null argument");
    run_batch_ray(mesh_forest, origins, directions, query_offsets, num_rays, max_time >= 0.f ? max_time : -1.f, chunk,
                  out_time, out_index, (cudaStream_t)stream);
  });
}

THEA_API thea_status thea_batch_k_closest(const thea_bvh * point_forest, const float * queries,
                                          const int64_t * query_offsets, int64_t num_queries, int32_t k,
                                          float dist_bound, int32_t queries_per_warp, int32_t * out_index,
                                          float * out_sq_distance, void * stream) {
  return guarded_query(point_forest, stream, [&] {
    int chunk = check_batch_common(point_forest, query_offsets, num_queries, queries_per_warp,
                                   {queries, out_index, out_sq_distance}, "batch_k_closest");
    THEA_REQUIRE(!point_forest->is_mesh, "batch_k_closest: a point forest is required");
    THEA_REQUIRE(k >= 1 && k <= 32, "batch_k_closest: k must be in 1..32");
    if (num_queries == 0) return;
    THEA_REQUIRE(queries && out_index && out_sq_distance, "batch_k_closest: null argument");
    run_batch_knn(point_forest, queries, query_offsets, num_queries, k, bound_threshold(dist_bound), chunk, out_index,
                  out_sq_distance, (cudaStream_t)stream);
  });
}

}  // extern "C"

struct thea_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

extern "C" {

THEA_API thea_status thea_graph_capture_begin(void * stream) {
  return guarded([&] {
    THEA_REQUIRE(stream, "graph_capture_begin: the legacy default stream cannot be captured");
    THEA_CUDA_CHECK(cudaStreamBeginCapture((cudaStream_t)stream, cudaStreamCaptureModeThreadLocal));
  });
}

THEA_API thea_status thea_graph_capture_end(void * stream, thea_graph ** out_graph) {
  return guarded([&] {
    THEA_REQUIRE(stream && out_graph, "graph_capture_end: null argument");
    *out_graph = nullptr;
    cudaGraph_t g = nullptr;
    THEA_CUDA_CHECK(cudaStreamEndCapture((cudaStream_t)stream, &g));
    thea_graph * tg = new thea_graph;
    tg->graph = g;
    cudaError_t e = cudaGraphInstantiate(&tg->exec, g, 0);
    if (e != cudaSuccess) {
      cudaGraphDestroy(g);
      delete tg;
      THEA_CUDA_CHECK(e);
    }
    *out_graph = tg;
  });
}

THEA_API thea_status thea_graph_launch(thea_graph * graph, void * stream) {
  return guarded([&] {
    THEA_REQUIRE(graph && graph->exec, "graph_launch: null graph");
    g_launches.fetch_add(1, std::memory_order_relaxed);
    THEA_CUDA_CHECK(cudaGraphLaunch(graph->exec, (cudaStream_t)stream));
  });
}

THEA_API thea_status thea_graph_destroy(thea_graph * graph) {
  return guarded([&] {
    if (!graph) return;
    if (graph->exec) cudaGraphExecDestroy(graph->exec);
    if (graph->graph) cudaGraphDestroy(graph->graph);
    delete graph;
  });
}

THEA_API thea_status thea_autotune_batch_closest(const float * vertices, int64_t num_vertices, const int32_t * faces,
                                                 const int64_t * mesh_face_offsets, int32_t num_meshes,
                                                 const float * queries, const int64_t * query_offsets,
                                                 int64_t num_queries, int32_t precision, void * stream,
                                                 thea_tuning * out_tuning) {
  return guarded([&] {
    THEA_REQUIRE(out_tuning, "autotune_batch_closest: null output");
    THEA_REQUIRE(vertices && faces && mesh_face_offsets && queries && query_offsets && num_meshes >= 1 &&
                     num_queries > 0,
                 "autotune_batch_closest: null or empty argument");
    THEA_REQUIRE(!is_host_pointer(queries) && !is_host_pointer(query_offsets),
                 "autotune_batch_closest: queries and offsets must be device memory");
    cudaStream_t s = (cudaStream_t)stream;
    int64_t nf = mesh_face_offsets[num_meshes];
    DeviceView V(vertices, (size_t)num_vertices * 3 * sizeof(float), s);
    DeviceView F(faces, (size_t)nf * 3 * sizeof(int32_t), s);
    Scratch idx((size_t)num_queries * 4, s), dist((size_t)num_queries * 4, s);
    cudaEvent_t e0, e1;
    THEA_CUDA_CHECK(cudaEventCreate(&e0));
    THEA_CUDA_CHECK(cudaEventCreate(&e1));
    thea_tuning best{};
    best.milliseconds = INFINITY;
    int tried = 0;
    int const widths[2] = {4, 8}, leaves[3] = {1, 2, 4}, chunks[3] = {32, 64, 128}, budgets[3] = {12, 32, 128};
    for (int w : widths)
      for (int l : leaves) {
        thea_build_config cfg{};
        cfg.width = w;
        cfg.max_leaf_size = l;
        cfg.layouts = THEA_LAYOUT_CLOSEST;
        thea_bvh * f = build_forest(true, (float const *)V.ptr, num_vertices, (int32_t const *)F.ptr, nf,
                                    mesh_face_offsets, num_meshes, cfg, s);
        ClosestParams cp;
        cp.precision = precision;
        cp.scene_scale = scene_scale_of(f);
        auto time_it = [&](int chunk, int budget) {
          cp.budget = budget;
          float times[3];
          run_batch_closest(f, queries, query_offsets, num_queries, cp, chunk, idx.as<int32_t>(), dist.as<float>(),
                            nullptr, nullptr, s);
          for (float & t : times) {
            THEA_CUDA_CHECK(cudaEventRecord(e0, s));
            run_batch_closest(f, queries, query_offsets, num_queries, cp, chunk, idx.as<int32_t>(), dist.as<float>(),
                              nullptr, nullptr, s);
            THEA_CUDA_CHECK(cudaEventRecord(e1, s));
            THEA_CUDA_CHECK(cudaEventSynchronize(e1));
            THEA_CUDA_CHECK(cudaEventElapsedTime(&t, e0, e1));
          }
          std::sort(times, times + 3);
          ++tried;
          if (times[1] < best.milliseconds) {
            best.width = w;
            best.max_leaf_size = l;
            best.queries_per_warp = chunk;
            best.hard_query_budget = budget > 0 ? budget : -1;
            best.milliseconds = times[1];
          }
          return times[1];
        };
        // queries per warp with one thread per query throughout, then the two-phase budgets at the best one
        int best_chunk = chunks[0];
        float best_t = INFINITY;
        for (int c : chunks) {
          float t = time_it(c, 0);
          if (t < best_t) { best_t = t; best_chunk = c; }
        }
        for (int bud : budgets) time_it(best_chunk, bud);
        destroy_bvh(f);
      }
    best.candidates = tried;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *out_tuning = best;
  });
}

THEA_API thea_status thea_sample_by_area_noalloc(const float * vertices, int64_t num_vertices, const int32_t * faces,
                                                 int64_t num_faces, int64_t num_samples, uint32_t seed, int32_t rng,
                                                 float * out_positions, float * out_normals, int32_t * out_faces,
                                                 int64_t * out_num_written, void * stream) {
  return guarded([&] {
    if (out_num_written) *out_num_written = 0;
    THEA_REQUIRE(rng == THEA_RNG_THEA_MT || rng == THEA_RNG_COUNTER, "sample_by_area_noalloc: unknown rng");
    THEA_REQUIRE(num_samples >= 0, "sample_by_area_noalloc: negative sample count");
    THEA_REQUIRE(num_faces <= THEA_NOALLOC_MAX_FACES,
                 "sample_by_area_noalloc: the mesh has more than THEA_NOALLOC_MAX_FACES triangles");
    if (num_samples == 0) return;
    THEA_REQUIRE(vertices && faces && num_vertices > 0 && num_faces > 0, "sample_by_area_noalloc: empty mesh");
    THEA_REQUIRE(out_positions, "sample_by_area_noalloc: out_positions is null");
    void const * arrays[5] = {vertices, faces, out_positions, out_normals, out_faces};
    for (void const * p : arrays)
      THEA_REQUIRE(!p || is_device_memory_here(p),
                   "sample_by_area_noalloc: every array must be device memory of the current device");
    int64_t got = run_sample_by_area_noalloc(vertices, num_vertices, faces, num_faces, num_samples, seed, rng,
                                             out_positions, out_normals, out_faces, (cudaStream_t)stream);
    if (out_num_written) *out_num_written = got;
  });
}

//============================================================================================================================
// Serving loop
//============================================================================================================================

THEA_API thea_status thea_server_create(const thea_server_config * config, thea_server ** out_server) {
  return guarded([&] {
    THEA_REQUIRE(config && out_server, "server_create: null argument");
    *out_server = nullptr;
    *out_server = server_create(*config);
  });
}

THEA_API thea_status thea_server_destroy(thea_server * server) {
  return guarded([&] {
    if (server) server_destroy(server);
  });
}

THEA_API thea_status thea_server_add_mesh(thea_server * server, const float * vertices, int64_t num_vertices,
                                          const int32_t * faces, int64_t num_faces, int32_t * out_mesh) {
  return guarded([&] {
    THEA_REQUIRE(server && out_mesh, "server_add_mesh: null argument");
    *out_mesh = -1;
    *out_mesh = server_add_mesh(server, vertices, num_vertices, faces, num_faces);
  });
}

THEA_API thea_status thea_server_remove_mesh(thea_server * server, int32_t mesh) {
  return guarded([&] {
    THEA_REQUIRE(server, "server_remove_mesh: null server");
    server_remove_mesh(server, mesh);
  });
}

THEA_API thea_status thea_server_submit(thea_server * server, const thea_request * request, uint64_t * out_ticket) {
  return guarded([&] {
    THEA_REQUIRE(server && request && out_ticket, "server_submit: null argument");
    *out_ticket = 0;
    *out_ticket = server_submit(server, *request);
  });
}

THEA_API thea_status thea_server_wait(thea_server * server, uint64_t ticket, int64_t timeout_us,
                                      thea_status * out_request_status, double * out_latency_ms) {
  thea_status w = THEA_OK;
  thea_status g = guarded([&] {
    THEA_REQUIRE(server, "server_wait: null server");
    w = server_wait(server, ticket, timeout_us, out_request_status, out_latency_ms);
  });
  if (g != THEA_OK) return g;
  if (w == THEA_ERR_WAIT_TIMEOUT) g_error = "server_wait: the request has not finished";
  return w;
}

THEA_API thea_status thea_server_cancel(thea_server * server, uint64_t ticket) {
  return guarded([&] {
    THEA_REQUIRE(server, "server_cancel: null server");
    server_cancel(server, ticket);
  });
}

THEA_API thea_status thea_server_get_stats(thea_server * server, thea_server_stats * out_stats) {
  return guarded([&] {
    THEA_REQUIRE(server && out_stats, "server_get_stats: null argument");
    server_stats(server, out_stats);
  });
}

THEA_API thea_status thea_server_reset_stats(thea_server * server) {
  return guarded([&] {
    THEA_REQUIRE(server, "server_reset_stats: null server");
    server_reset_stats(server);
  });
}

THEA_API thea_status thea_shape_diameter(const thea_bvh * mesh_bvh, const float * positions, const float * normals,
                                         int64_t num_points, float scale, int32_t only_interior, double * out_sdf,
                                         void * stream) {
  return guarded_query(mesh_bvh, stream, [&] {
    THEA_REQUIRE(mesh_bvh && mesh_bvh->is_mesh && mesh_bvh->num_segments == 1,
                 "shape_diameter: a mesh BVH (not a forest) is required");
    THEA_REQUIRE(mesh_bvh->ray_rec, "shape_diameter: the BVH was built without THEA_LAYOUT_RAY");
    THEA_REQUIRE(normals || query_target(mesh_bvh)->cp_rec,
                 "shape_diameter: without normals the BVH needs THEA_LAYOUT_CLOSEST");
    THEA_REQUIRE(num_points >= 0, "shape_diameter: negative point count");
    if (num_points == 0) return;
    THEA_REQUIRE(positions && out_sdf, "shape_diameter: null positions or out_sdf");
    THEA_REQUIRE(num_points * 30 < ((int64_t)1 << 31), "shape_diameter: too many points for one call");
    cudaStream_t s = (cudaStream_t)stream;
    Scratch pin, nin, pout;
    float const * pos = positions;
    float const * nrm = normals;
    if (is_host_pointer(positions)) {
      pin = Scratch((size_t)num_points * 12, s);
      THEA_CUDA_CHECK(cudaMemcpyAsync(pin.ptr, positions, (size_t)num_points * 12, cudaMemcpyHostToDevice, s));
      pos = pin.as<float>();
    }
    if (normals && is_host_pointer(normals)) {
      nin = Scratch((size_t)num_points * 12, s);
      THEA_CUDA_CHECK(cudaMemcpyAsync(nin.ptr, normals, (size_t)num_points * 12, cudaMemcpyHostToDevice, s));
      nrm = nin.as<float>();
    }
    double * out = out_sdf;
    bool host_out = is_host_pointer(out_sdf);
    if (host_out) {
      pout = Scratch((size_t)num_points * 8, s);
      out = pout.as<double>();
    }
    run_shape_diameter(mesh_bvh, pos, nrm, num_points, scale, only_interior != 0, out, s);
    if (host_out) {
      THEA_CUDA_CHECK(cudaMemcpyAsync(out_sdf, out, (size_t)num_points * 8, cudaMemcpyDeviceToHost, s));
      sync_stream(s);
    }
  });
}

THEA_API thea_status thea_best_fit_sphere(const float * points, int64_t num_points, double * out_center,
                                          double * out_radius, void * stream) {
  return guarded([&] {
    THEA_REQUIRE(num_points >= 0, "best_fit_sphere: negative point count");
    THEA_REQUIRE(out_center && out_radius, "best_fit_sphere: null output");
    THEA_REQUIRE(num_points == 0 || points, "best_fit_sphere: null points");
    cudaStream_t s = (cudaStream_t)stream;
    Scratch pin;
    float const * pts = points;
    if (num_points > 0 && is_host_pointer(points)) {
      pin = Scratch((size_t)num_points * 12, s);
      THEA_CUDA_CHECK(cudaMemcpyAsync(pin.ptr, points, (size_t)num_points * 12, cudaMemcpyHostToDevice, s));
      pts = pin.as<float>();
    }
    run_bounding_sphere(pts, num_points, out_center, out_radius, s);
  });
}

THEA_API thea_status thea_bvh_closest_pair(const thea_bvh * target, const thea_bvh * query, float dist_bound,
                                           int32_t * out_query_index, int32_t * out_target_index,
                                           float * out_sq_distance, float * out_query_point, float * out_target_point,
                                           void * stream) {
  return guarded_query(target, stream, [&] {
    THEA_REQUIRE(out_query_index && out_target_index, "closest_pair: null output");
    *out_query_index = *out_target_index = -1;
    if (out_sq_distance) *out_sq_distance = -1.f;
    PairResult r;
    if (!run_closest_pair(target, query, bound_threshold(dist_bound), r, (cudaStream_t)stream)) return;
    *out_query_index = r.query_index;
    *out_target_index = r.target_index;
    if (out_sq_distance) *out_sq_distance = r.d2;
    if (out_query_point) std::memcpy(out_query_point, r.query_point, 12);
    if (out_target_point) std::memcpy(out_target_point, r.target_point, 12);
    sync_stream((cudaStream_t)stream);
  });
}

THEA_API thea_status thea_bvh_k_closest_pairs(const thea_bvh * target, const thea_bvh * query, int32_t k,
                                              float dist_bound, int32_t * out_query_index, int32_t * out_target_index,
                                              float * out_sq_distance, int32_t * out_count, void * stream) {
  return guarded_query(target, stream, [&] {
    THEA_REQUIRE(out_query_index && out_target_index && out_sq_distance, "k_closest_pairs: null output");
    THEA_REQUIRE(k >= 1 && k <= 32, "k_closest_pairs: k must be in 1..32");
    cudaStream_t s = (cudaStream_t)stream;
    Scratch dev((size_t)k * 12, s);
    int32_t * qi = (int32_t *)dev.ptr;
    int32_t * ti = qi + k;
    float * d2 = (float *)(ti + k);
    int64_t c = run_k_closest_pairs(target, query, k, bound_threshold(dist_bound), qi, ti, d2, s);
    THEA_CUDA_CHECK(cudaMemcpyAsync(out_query_index, qi, (size_t)k * 4, cudaMemcpyDefault, s));
    THEA_CUDA_CHECK(cudaMemcpyAsync(out_target_index, ti, (size_t)k * 4, cudaMemcpyDefault, s));
    THEA_CUDA_CHECK(cudaMemcpyAsync(out_sq_distance, d2, (size_t)k * 4, cudaMemcpyDefault, s));
    sync_stream(s);
    if (out_count) *out_count = (int32_t)c;
  });
}

THEA_API thea_status thea_mesh_read(const char * path, thea_mesh ** out_mesh) {
  return guarded([&] {
    THEA_REQUIRE(out_mesh, "mesh_read: null output");
    *out_mesh = nullptr;
    THEA_REQUIRE(path, "mesh_read: null path");
    thea::MeshData data = thea::read_mesh_file(path);
    *out_mesh = reinterpret_cast<thea_mesh *>(new thea::MeshData(std::move(data)));
  });
}

THEA_API thea_status thea_mesh_read_buffer(const void * data, int64_t bytes, const char * codec, thea_mesh ** out_mesh) {
  return guarded([&] {
    THEA_REQUIRE(out_mesh, "mesh_read_buffer: null output");
    *out_mesh = nullptr;
    THEA_REQUIRE(codec && bytes >= 0 && (data || bytes == 0), "mesh_read_buffer: null or negative argument");
    thea::MeshData m = thea::read_mesh_buffer(data, bytes, codec);
    *out_mesh = reinterpret_cast<thea_mesh *>(new thea::MeshData(std::move(m)));
  });
}

THEA_API thea_status thea_mesh_get_info(const thea_mesh * mesh, thea_mesh_info * info) {
  return guarded([&] {
    THEA_REQUIRE(mesh && info, "mesh_get_info: null argument");
    auto const & m = *reinterpret_cast<thea::MeshData const *>(mesh);
    info->num_vertices = (int64_t)m.vertex_source.size();
    info->num_triangles = (int64_t)m.triangle_face.size();
    info->num_faces = m.num_faces;
    info->num_submeshes = (int64_t)m.submesh_triangle_offsets.size() - 1;
  });
}

THEA_API thea_status thea_mesh_copy(const thea_mesh * mesh, float * vertices, int32_t * vertex_source,
                                    int32_t * triangles, int32_t * triangle_face, int64_t * submesh_vertex_offsets,
                                    int64_t * submesh_triangle_offsets) {
  return guarded([&] {
    THEA_REQUIRE(mesh, "mesh_copy: null mesh");
    auto const & m = *reinterpret_cast<thea::MeshData const *>(mesh);
    auto put = [](void * dst, auto const & v) {
      if (dst && !v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(v[0]));
    };
    put(vertices, m.vertices);
    put(vertex_source, m.vertex_source);
    put(triangles, m.triangles);
    put(triangle_face, m.triangle_face);
    put(submesh_vertex_offsets, m.submesh_vertex_offsets);
    put(submesh_triangle_offsets, m.submesh_triangle_offsets);
  });
}

THEA_API thea_status thea_mesh_destroy(thea_mesh * mesh) {
  return guarded([&] { delete reinterpret_cast<thea::MeshData *>(mesh); });
}

THEA_API thea_status thea_triangulate_face(const float * positions, int32_t num_vertices, int32_t * out_triangles,
                                           int32_t * out_count) {
  return guarded([&] {
    THEA_REQUIRE(out_count, "triangulate_face: null count");
    *out_count = 0;
    THEA_REQUIRE(num_vertices >= 0, "triangulate_face: negative vertex count");
    if (num_vertices < 3) return;
    THEA_REQUIRE(positions && out_triangles, "triangulate_face: null argument");
    std::vector<int32_t> tris;
    int nt = thea::triangulate_face(positions, num_vertices, tris);
    std::copy(tris.begin(), tris.end(), out_triangles);
    *out_count = nt;
  });
}

}  // extern "C"
