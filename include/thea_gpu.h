/*
 * thea_gpu.h -- C ABI of the GB300-native spatial-query path (closest point on a mesh, first ray hit, k nearest
 * neighbours, the BVH build and area-weighted mesh sampling that feed them).
 *
 * Every entry point is a plain C function over pointers and sizes. Nothing throws across this boundary: each call returns
 * a thea_status, and thea_last_error_message() gives a human-readable detail for the calling thread.
 *
 * Pointers. Array arguments may point to device memory or to host memory (pinned or pageable); the library detects which
 * with cudaPointerGetAttributes. Device-resident arrays are used in place. When any array of a query call is host
 * memory, the call stages the work through device buffers in chunks on the given stream and returns after the results
 * have been written back (the call then synchronizes the stream). Device-only calls are asynchronous on the stream.
 *
 * Streams. `stream` is a cudaStream_t passed as void*; NULL means the legacy default stream.
 *
 * Result conventions follow the reference (sidch/Thea, Code/Source/Algorithms/BvhN.hpp): "not found" is element
 * index -1, hit time -1, distance -1. Ties between elements at bit-identical distances or hit times are broken by the
 * lowest element index (the reference keeps whichever it meets first in its own traversal order).
 *
 * Arithmetic. Per-element distances and hit times are computed in FP32 with the reference's operation order and no
 * fused multiply-add, so that indices, distances, closest points and hit times are bit-identical to the reference's FP32
 * CPU path under the lowest-index tie rule.
 */
#ifndef THEA_GPU_H
#define THEA_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define THEA_API __declspec(dllexport)
#else
#define THEA_API __attribute__((visibility("default")))
#endif

#define THEA_GPU_ABI_VERSION 1

typedef enum thea_status {
  THEA_OK = 0,
  THEA_ERR_INVALID_ARGUMENT = 1,   /* bad pointer, size or option */
  THEA_ERR_OUT_OF_MEMORY = 2,      /* a device allocation failed */
  THEA_ERR_ADMISSION_REFUSED = 3,  /* serving: request does not fit the memory budget or queue */
  THEA_ERR_DEVICE_TIMEOUT = 4,     /* a bounded device-side wait gave up; the context stays usable */
  THEA_ERR_CUDA = 5,               /* a CUDA runtime call failed */
  THEA_ERR_INTERNAL = 6,
  THEA_ERR_NOT_SUPPORTED = 7,
  THEA_ERR_CANCELLED = 8           /* serving: request was cancelled before it ran */
} thea_status;

typedef struct thea_bvh thea_bvh; /* opaque, immutable after build; owns device copies of the elements and nodes */

/* Primitive layouts a mesh BVH keeps (bit mask). Closest-point queries need CLOSEST, ray queries need RAY. */
#define THEA_LAYOUT_CLOSEST 1u
#define THEA_LAYOUT_RAY 2u

typedef struct thea_build_config {
  int32_t width;          /* children per node: 4 or 8 (0 = default 4) */
  int32_t max_leaf_size;  /* elements per leaf, 1..16 (0 = default: 4 for meshes, 8 for points) */
  uint32_t layouts;       /* THEA_LAYOUT_* mask for meshes (0 = both) */
  int32_t reserved[5];    /* must be zero */
} thea_build_config;

typedef struct thea_bvh_info {
  int64_t num_elements;
  int64_t num_nodes;
  int32_t width;
  int32_t max_leaf_size;
  int32_t is_mesh;
  int32_t depth;             /* levels of wide nodes */
  int64_t device_bytes;      /* nodes + element records held by the handle */
  float bounds_lo[3];        /* bounds of all elements */
  float bounds_hi[3];
  uint32_t device_error_bits; /* nonzero if a query kernel hit an internal limit (reading it synchronizes) */
  int32_t reserved;
} thea_bvh_info;

/* ---- library ------------------------------------------------------------------------------------------------------- */

THEA_API int thea_abi_version(void);
THEA_API const char * thea_status_string(thea_status s);
THEA_API const char * thea_last_error_message(void);

/* Number of kernels this library has launched in the process (all devices). */
THEA_API int64_t thea_launch_count(void);

/* Per-kernel device timing with CUDA events recorded on the launching stream (off by default). thea_profiling_read
 * synchronizes the recorded events and returns the summed milliseconds and launch count for kernels whose name contains
 * `kernel_substring` since the last reset. */
THEA_API thea_status thea_profiling_enable(int enable);
THEA_API thea_status thea_profiling_reset(void);
THEA_API thea_status thea_profiling_read(const char * kernel_substring, double * total_ms, int64_t * launches);

/* ---- build --------------------------------------------------------------------------------------------------------- */

/* BVH over mesh triangles. Element index = face index f (faces[3f..3f+2] index `vertices`, 3 floats each).
 * Replaces MeshBvh::add + MeshBvh::init (Code/Source/Algorithms/MeshBvh.hpp:55,104-111) and BvhN::init (BvhN.hpp:705). */
THEA_API thea_status thea_mesh_bvh_build(const float * vertices, int64_t num_vertices, const int32_t * faces,
                                         int64_t num_faces, const thea_build_config * config, void * stream,
                                         thea_bvh ** out_bvh);

/* BVH over points (3 floats each). Element index = point index. Replaces BvhN<Vector3, 3>::init (BvhN.hpp:705). */
THEA_API thea_status thea_point_bvh_build(const float * points, int64_t num_points, const thea_build_config * config,
                                          void * stream, thea_bvh ** out_bvh);

/* Releases the handle after all work on `stream`-ordered queries using it has completed (synchronizes the device). */
THEA_API thea_status thea_bvh_destroy(thea_bvh * bvh);

THEA_API thea_status thea_bvh_get_info(const thea_bvh * bvh, thea_bvh_info * info);

/* ---- queries ------------------------------------------------------------------------------------------------------- */

/* Closest element of a mesh BVH to each query point.
 * Replaces BvhN::closestElement<MetricL2>(query, dist_bound, compat, &dist, &closest_point) (BvhN.hpp:1050-1063) and
 * closestPair (BvhN.hpp:1082-1114). dist_bound < 0: unbounded; otherwise only elements with squared distance strictly
 * below dist_bound^2 are accepted. Outputs per query: index (-1 if none), distance (sqrt of the squared distance, -1 if
 * none) and, if non-NULL, the closest point on the element (3 floats; unchanged slots are written as 0 when none). */
THEA_API thea_status thea_closest_element(const thea_bvh * mesh_bvh, const float * queries, int64_t num_queries,
                                          float dist_bound, int32_t * out_index, float * out_distance,
                                          float * out_closest_point, void * stream);

/* First hit of each ray (origin, direction; 3 floats each, direction not necessarily unit) with a mesh BVH.
 * Replaces BvhN::rayStructureIntersection<RayIntersectionTester>(ray, max_time) (BvhN.hpp:1292-1316) and
 * rayIntersectionTime (BvhN.hpp:1271-1289). max_time < 0: unbounded; otherwise hits need time <= max_time.
 * Outputs per ray: hit time (-1 on a miss), element index (-1 on a miss), and if non-NULL the unit face normal. */
THEA_API thea_status thea_ray_intersection(const thea_bvh * mesh_bvh, const float * origins, const float * directions,
                                           int64_t num_rays, float max_time, float * out_time, int32_t * out_index,
                                           float * out_normal, void * stream);

/* k nearest points of a point BVH to each query, 1 <= k <= 32, sorted by increasing squared distance (ties: lower
 * index first). exclude_index (nullable) gives per query an element index to skip (the reference's FilterSelf,
 * Code/Source/Algorithms/PointSet3.hpp:576-583). dist_bound < 0: unbounded; else only squared distances strictly below
 * dist_bound^2. Unused slots: index -1, squared distance -1.
 * Replaces BvhN::kClosestPairs<MetricL2>(query, BoundedSortedArrayN<k, NeighborPair>&, dist_bound) (BvhN.hpp:1139-1146). */
THEA_API thea_status thea_k_closest(const thea_bvh * point_bvh, const float * queries, int64_t num_queries, int32_t k,
                                    float dist_bound, const int32_t * exclude_index, int32_t * out_index,
                                    float * out_sq_distance, void * stream);

/* k-nearest-neighbour graph of the BVH's own points: query i is point i, excluding itself. Rows in point order. */
THEA_API thea_status thea_k_closest_self(const thea_bvh * point_bvh, int32_t k, int32_t * out_index,
                                         float * out_sq_distance, void * stream);

/* ---- sampling ------------------------------------------------------------------------------------------------------ */

#define THEA_RNG_THEA_MT 0   /* the reference's Random(seed) stream: bit-identical samples */
#define THEA_RNG_COUNTER 1   /* counter-based (Philox-4x32-10) stream: same distribution, fully parallel */

/* Area-weighted sampling of a triangle mesh, with replacement, `num_samples` points.
 * Replaces MeshSampler(mesh).sampleEvenlyByArea(n, positions, face_normals, triangles, CountMode::EXACT)
 * (Code/Source/Algorithms/MeshSampler.hpp:100-204) drawing from Random(seed) (Code/Source/Random.cpp:49-132).
 * Outputs: positions (3 floats each), optional face normals (3 floats) and face indices; *out_num_written (nullable)
 * receives the number of samples written: num_samples, or 0 when the mesh has zero total area (as the reference
 * returns). The call synchronizes the stream (it reads the total area back). */
THEA_API thea_status thea_sample_by_area(const float * vertices, int64_t num_vertices, const int32_t * faces,
                                         int64_t num_faces, int64_t num_samples, uint32_t seed, int32_t rng,
                                         float * out_positions, float * out_normals, int32_t * out_faces,
                                         int64_t * out_num_written, void * stream);

/* ---- allocation-free sampling -------------------------------------------------------------------------------------- */

/* Largest mesh (in triangles) that thea_sample_by_area_noalloc accepts. */
#define THEA_NOALLOC_MAX_FACES 1048576

/* Same results as thea_sample_by_area (bit-identical for both rng modes), for callers that cannot allocate device
 * memory: a host application that hands this library a fixed device budget through its own pool allocator, a plugin that
 * must not allocate behind its host's back, or a latency-critical loop that cannot afford cudaMalloc's implicit
 * synchronization. This entry point has no counterpart in the reference (whose sampler runs on the CPU).
 *
 * It calls no cudaMalloc, cudaFree or other allocating routine. Its scratch (the cumulative-area table of up to
 * THEA_NOALLOC_MAX_FACES triangles, the generator state and one chunk of random words: about 9 MiB) is a fixed device
 * array inside the library, resident on every GPU that loads the library until the process exits. The caller passes
 * device-resident inputs and outputs; host pointers and meshes with more than THEA_NOALLOC_MAX_FACES triangles are
 * rejected with THEA_ERR_INVALID_ARGUMENT. The first call on each device looks up the array's device address (with that
 * device current); make that first call before any stream capture. All calls on a device share the one array, and every
 * call rewrites the parts it reads before reading them; calls whose work overlaps on the GPU (different streams or
 * threads at the same time) race on it and must be serialized by the caller. The call synchronizes `stream` once, to
 * read back the total area. */
THEA_API thea_status thea_sample_by_area_noalloc(const float * vertices, int64_t num_vertices, const int32_t * faces,
                                                 int64_t num_faces, int64_t num_samples, uint32_t seed, int32_t rng,
                                                 float * out_positions, float * out_normals, int32_t * out_faces,
                                                 int64_t * out_num_written, void * stream);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* THEA_GPU_H */
