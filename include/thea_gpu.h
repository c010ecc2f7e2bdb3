/*
 * thea_gpu.h -- C ABI of the GB300-native spatial-query path (closest point on a mesh, first ray hit, k nearest
 * neighbours, the BVH build and area-weighted mesh sampling that feed them).
 *
 * Every entry point is a plain C function over pointers and sizes. Nothing throws across this boundary: each call returns
 * a thea_status, and thea_last_error_message() gives a human-readable detail for the calling thread.
 *
 * Pointers. Array arguments may point to device memory or to host memory (pinned or pageable); the library detects which
 * with cudaPointerGetAttributes. Device-resident arrays are used in place. When every array of a large FP32 first-hit
 * call (no normals) or closest-point call (no error output) is pinned host memory, the kernels read and write those
 * arrays in place over NVLink-C2C (one launch, block-sized coalesced accesses). Otherwise, when any array of a query
 * call is host memory, the call stages the work through device buffers in chunks on the given stream. Calls with host
 * arrays return after the results are in host memory (they synchronize the stream); device-only calls are
 * asynchronous on the stream.
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
  THEA_ERR_CANCELLED = 8,          /* serving: request was cancelled before it ran */
  THEA_ERR_WAIT_TIMEOUT = 9        /* serving: a host-side wait ended before the request finished */
} thea_status;

typedef struct thea_bvh thea_bvh; /* opaque, immutable after build; owns device copies of the elements and nodes */

/* Primitive layouts a mesh BVH keeps (bit mask). Closest-point queries need CLOSEST, ray queries need RAY. */
#define THEA_LAYOUT_CLOSEST 1u
#define THEA_LAYOUT_RAY 2u

typedef struct thea_build_config {
  int32_t width;          /* children per node: 4 or 8 (0 = default 4) */
  int32_t max_leaf_size;  /* elements per leaf, 1..16 (0 = default: 4 for meshes, 8 for points) */
  uint32_t layouts;       /* THEA_LAYOUT_* mask for meshes (0 = both) */
  int32_t query_order;    /* 1: traverse large query batches in Morton order of the query point; 0: caller order */
  int32_t reserved[4];    /* must be zero */
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
                              /* (1: a traversal stack would have overflowed; 2: a tensor-core wait gave up) */
  int32_t num_segments;      /* BVHs in the handle: 1, or the meshes / point sets of a forest */
} thea_bvh_info;

/* ---- library ------------------------------------------------------------------------------------------------------- */

THEA_API int thea_abi_version(void);
THEA_API const char * thea_status_string(thea_status s);
THEA_API const char * thea_last_error_message(void);

/* Number of kernels this library has launched in the process (all devices). */
THEA_API int64_t thea_launch_count(void);

/* Number of device and pinned-host allocations this library has made in the process (all devices; driver allocations
 * and allocations from its stream-ordered pool). A diagnostic: a call that leaves it unchanged allocated nothing. No
 * counterpart in the reference. */
THEA_API int64_t thea_allocation_count(void);

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

/* Affine transform of a built BVH (BvhN::setTransform / clearTransform / getTransformInv, BvhN.hpp:903-929), for
 * queries against the transformed elements without rebuilding from the caller's arrays. affine_3x4: row-major [L | t],
 * p -> L p + t; L must be invertible. As in the reference, rays are moved into object space with the FP32 inverse
 * (t' = L^-1 (-t)) and hit normals are returned in world space (normalised inverse-transpose); closest-point, k-NN and
 * radius queries are answered on the elements transformed into world space (the handle builds a world-space copy of
 * its records on the device: about twice the handle's memory while a transform is set). Single BVHs only (forests:
 * THEA_ERR_INVALID_ARGUMENT). Synchronizes the stream; must not run while queries on the handle are in flight. */
THEA_API thea_status thea_bvh_set_transform(thea_bvh * bvh, const float * affine_3x4, void * stream);
THEA_API thea_status thea_bvh_clear_transform(thea_bvh * bvh);
/* *has_transform = 0 or 1; affine_3x4 / inverse_3x4 (nullable) receive the map and its FP32 inverse (identity if none) */
THEA_API thea_status thea_bvh_get_transform(const thea_bvh * bvh, int32_t * has_transform, float * affine_3x4,
                                            float * inverse_3x4);

/* Byte image of a built BVH (any kind: mesh, points, forest), for warm starts without a rebuild: a versioned header
 * (magic "THEABVH", version 1), the handle's parameters, then its arrays. out_image == NULL: *out_bytes = the image
 * size. Otherwise the image is written to host memory out_image (capacity bytes). Synchronizes the stream. The
 * reference has no counterpart (its BvhN is not Serializable). */
THEA_API thea_status thea_bvh_serialize(const thea_bvh * bvh, void * out_image, int64_t capacity, int64_t * out_bytes,
                                        void * stream);
/* A new handle on the current device from an image made by thea_bvh_serialize (host memory). The header and section
 * sizes are checked before anything is allocated (THEA_ERR_INVALID_ARGUMENT for a foreign, truncated or newer image).
 * Queries on the new handle return what they return on the original. Synchronizes the stream. */
THEA_API thea_status thea_bvh_deserialize(const void * image, int64_t bytes, void * stream, thea_bvh ** out_bvh);

THEA_API thea_status thea_bvh_get_info(const thea_bvh * bvh, thea_bvh_info * info);

/* ---- queries ------------------------------------------------------------------------------------------------------- */

/* Closest element of a mesh BVH to each query point.
 * Replaces BvhN::closestElement<MetricL2>(query, dist_bound, compat, &dist, &closest_point) (BvhN.hpp:1050-1063) and
 * closestPair (BvhN.hpp:1082-1114). dist_bound < 0: unbounded; otherwise the bound is applied as closestPair applies it:
 * a query whose squared distance to the root box (the element bounds grown by 1.05 about their centre, mapped by the
 * transform if one is set) exceeds dist_bound^2 gets no element, and otherwise elements are accepted with squared
 * distance strictly below (dist_bound + max(0.001 |root box extent|, 100 FLT_EPSILON))^2 (the loosening closestPair
 * adds to a given bound). Outputs per query: index (-1 if none), distance (sqrt of the squared distance, -1 if
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

/* ---- precision modes ------------------------------------------------------------------------------------------------ */

/* FP32_REFERENCE: the reference's FP32 arithmetic, bit for bit (the plain calls above use it).
 * FP64_RECHECK: mixed precision. Closest element: FP32 traversal and element tests, and every element whose FP32
 * distance lies within a band of the best (relative 2^-14 plus 2^-18 of the coordinate scale) is re-evaluated in FP64;
 * the result is the FP64 nearest element (ties: lowest index) with its FP64 distance and closest point, rounded to FP32.
 * Ray: the reference's FP32 verdict stays the primary result and, beside it, the watertight FP64 test (Woop, Benthin,
 * Wald 2013) of every element the FP32 test accepted or rejected by a narrow margin gives an FP64 verdict. */
#define THEA_PRECISION_FP32_REFERENCE 0
#define THEA_PRECISION_FP64_RECHECK 1

#define THEA_RAY_FLAG_HIT_DIFFERS 1     /* the FP32 and FP64 verdicts disagree on hit vs miss */
#define THEA_RAY_FLAG_ELEMENT_DIFFERS 2 /* both hit, different elements */

/* thea_closest_element with a precision mode and, if out_error is non-NULL, per query the absolute difference between
 * the returned distance and the FP64 distance of the returned element (-1 when none). No reference counterpart beyond
 * BvhN::closestElement (BvhN.hpp:1050-1063), whose arithmetic is FP32. */
THEA_API thea_status thea_closest_element_ex(const thea_bvh * mesh_bvh, const float * queries, int64_t num_queries,
                                             float dist_bound, int32_t precision, int32_t * out_index,
                                             float * out_distance, float * out_closest_point, float * out_error,
                                             void * stream);

/* thea_ray_intersection with a precision mode. In FP64_RECHECK mode the optional outputs receive the watertight FP64
 * verdict (time -1 / index -1 on a miss) and THEA_RAY_FLAG_* bits where it differs from the FP32 verdict. */
THEA_API thea_status thea_ray_intersection_ex(const thea_bvh * mesh_bvh, const float * origins,
                                              const float * directions, int64_t num_rays, float max_time,
                                              int32_t precision, float * out_time, int32_t * out_index,
                                              float * out_normal, float * out_time_fp64, int32_t * out_index_fp64,
                                              int32_t * out_flags, void * stream);

/* BvhN::rayIntersects (BvhN.hpp:1266-1269): out_hit[i] = 1 iff rayIntersectionTime(ray i, max_time) >= 0, i.e. some
 * element is hit at a time in [0, max_time] (any time if max_time < 0). An any-hit search that stops at the first
 * accepted element. Host or device arrays. */
THEA_API thea_status thea_ray_intersects(const thea_bvh * mesh_bvh, const float * origins, const float * directions,
                                         int64_t num_rays, float max_time, uint8_t * out_hit, void * stream);
/* `count` unit directions of Random(seed).sphere() (Random.cpp:225-250), in stream order: xyz triples, host or device */
THEA_API thea_status thea_random_sphere(uint32_t seed, int64_t count, float * out_directions, void * stream);
/* Visibility::compute (Algorithms/SurfaceFeatures/Local/Visibility.hpp:104-126) for many points: the fraction of
 * num_rays rays from each point (origin pushed out by 0.001 |extent of the padded root box| along the direction) with no
 * hit. Random(seed) replaces the reference's process-wide Random::common(): point i uses directions
 * [i * num_rays, (i + 1) * num_rays) of the thea_random_sphere stream, so the result equals the reference run with that
 * generator. num_rays <= 0: 100, as in the reference. Host or device arrays; synchronizes the stream. */
THEA_API thea_status thea_visibility(const thea_bvh * mesh_bvh, const float * positions, int64_t num_points,
                                     int32_t num_rays, uint32_t seed, double * out_fraction, void * stream);

/* ShapeDiameter::compute (Algorithms/SurfaceFeatures/Local/ShapeDiameter.hpp:143-217) for many points, as the
 * ShapeDiameter(ExternalBvh const *, scale) constructor sets it up (ShapeDiameter.hpp:94-101): per point, 30 rays along
 * the reference's fixed cone about the inward normal, from the point pushed 0.001 x scale inwards; first hits whose
 * element normal faces along the ray are kept (all hits when only_interior == 0); the median is selected with
 * libstdc++'s std::nth_element permutation, values beyond one standard deviation from it are rejected and the rest
 * averaged with cosine weights, divided by scale and clamped to [0, 1] (FP64). out_sdf[i] = -1 when no ray is kept.
 * normals (nullable, unnormalised is fine): the outward normals; NULL takes each point's closest element's own normal
 * (ShapeDiameter::compute(position); lowest element index among equidistant elements). scale <= 0: the |extent| of
 * the BVH's bounds, the constructor's default. Host or device arrays; synchronizes the stream. */
THEA_API thea_status thea_shape_diameter(const thea_bvh * mesh_bvh, const float * positions, const float * normals,
                                         int64_t num_points, float scale, int32_t only_interior, double * out_sdf,
                                         void * stream);

/* BestFitSphereN<3> (Algorithms/BestFitSphereN.hpp:62-91): the smallest ball enclosing the points, which the reference
 * computes with its miniball on the points cast to double. out_center: 3 doubles; out_radius: 1 double. No points: the
 * zero ball at the origin; non-finite points are skipped. ShapeDiameter(mesh) (SurfaceFeatures/Local/ShapeDiameter.hpp:
 * 60-70) takes twice this radius over the mesh's vertices, rounded to float, as its default scale; pass it as `scale`
 * to thea_shape_diameter to reproduce that constructor. Host or device points; synchronizes the stream. */
THEA_API thea_status thea_best_fit_sphere(const float * points, int64_t num_points, double * out_center,
                                          double * out_radius, void * stream);

/* Sample proximity graph: PointSet3::updateGraph (Algorithms/PointSet3.hpp:324-391, no oversampling) with options
 * max_degree (1..64). Random(seed) replaces the reference's Random::common() in the mean-separation estimate (100
 * samples' nearest-neighbour distances); everything else is the reference's: radius sqrt(max_degree) x estimate,
 * doubled up to twice for samples with fewer than clamp(max_degree / 4, 4, max_degree) neighbours; a candidate is kept
 * unless its normal makes a dot product below -0.5 with the sample's (when normals are given) or, with normals and a
 * surface (mesh BVH with the ray layout), the segment between the two samples lifted by 5 x separation along the mean
 * normal hits the surface. Separations are Math::fastSqrt of the squared distance. Row i of out_neighbors
 * (num_samples x max_degree) lists sample i's neighbours by ascending (separation, index), -1 past its degree;
 * out_separations (nullable) the separations, 0 past the degree; out_degree (nullable) the degrees;
 * out_avg_separation (nullable, 2 floats): the estimate and the final mean edge length (updateAverageSeparation).
 * Host or device arrays; synchronizes the stream. */
THEA_API thea_status thea_sample_graph(const float * positions, const float * normals, int64_t num_samples,
                                       int32_t max_degree, uint32_t seed, const thea_bvh * surface,
                                       int32_t * out_neighbors, float * out_separations, int32_t * out_degree,
                                       float * out_avg_separation, void * stream);

/* The sample graph with a dense oversampling of the surface: PointSet3::addOversampling + updateGraph
 * (Algorithms/PointSet3.hpp:231-290, 324-391) and extractOriginalAdjacencies (PointSet3.cpp:157-176). The graph of
 * thea_sample_graph is built over the samples followed by the num_dense dense samples (dense_normals are required, and
 * used, when normals are given); then each sample's neighbours are the first max_degree other samples that Dijkstra's
 * algorithm settles from it over that graph (edge lengths: the separations, summed in double), and their separations
 * the path lengths rounded to float. Ties in path length settle the lowest index first. Outputs as thea_sample_graph,
 * for the num_samples samples only; out_avg_separation[0] is the estimate over all samples and dense samples.
 * THEA_ERR_NOT_SUPPORTED if one search needs more than 896 vertices (too dense an oversampling for max_degree). Host
 * or device arrays; synchronizes the stream. */
THEA_API thea_status thea_sample_graph_oversampled(const float * positions, const float * normals,
                                                   int64_t num_samples, const float * dense_positions,
                                                   const float * dense_normals, int64_t num_dense,
                                                   int32_t max_degree, uint32_t seed, const thea_bvh * surface,
                                                   int32_t * out_neighbors, float * out_separations,
                                                   int32_t * out_degree, float * out_avg_separation, void * stream);

/* ---- pairs between two BVHs ---------------------------------------------------------------------------------------- */

/* BvhN::closestPair<MetricL2> with another BVH as the query (BvhN.hpp:1082-1114; the reference descends both trees,
 * :1916-2033): the (query element, target element) pair at the smallest distance, points or meshes on either side;
 * single BVHs, transforms applied. Between two meshes the distance is TriangleN<3>::squaredDistance
 * (Triangle3.hpp:314-400) evaluated with the target triangle as "this" (the reference evaluates a pair with either
 * triangle as "this", depending on which tree its descent is in, which can change the last bits); both meshes need
 * THEA_LAYOUT_CLOSEST. Ties: lowest query index, then lowest target index. dist_bound >= 0: only pairs strictly closer. Outputs are host scalars: indices (-1 when no pair), the squared
 * distance (the reference's monotone approximate distance; -1 when none) and, nullable, the closest points on the two
 * elements (3 floats each). Synchronizes the stream. */
THEA_API thea_status thea_bvh_closest_pair(const thea_bvh * target, const thea_bvh * query, float dist_bound,
                                           int32_t * out_query_index, int32_t * out_target_index,
                                           float * out_sq_distance, float * out_query_point, float * out_target_point,
                                           void * stream);
/* BvhN::kClosestPairs<MetricL2> between two point BVHs (BvhN.hpp:1139-1146 with a BVH query): the k (1..32) pairs with
 * the smallest squared distances, ascending (ties: lowest query index, then lowest target index), strictly closer than
 * dist_bound when it is >= 0. k entries per output (host or device arrays), -1 past *out_count (nullable). */
THEA_API thea_status thea_bvh_k_closest_pairs(const thea_bvh * target, const thea_bvh * query, int32_t k,
                                              float dist_bound, int32_t * out_query_index, int32_t * out_target_index,
                                              float * out_sq_distance, int32_t * out_count, void * stream);

/* ---- mesh files --------------------------------------------------------------------------------------------------- */

/* A mesh file read into host arrays in the reference's element order, ready for thea_mesh_bvh_build. */
typedef struct thea_mesh thea_mesh;

typedef struct thea_mesh_info {
  int64_t num_vertices;  /* vertices of all submeshes */
  int64_t num_triangles;
  int64_t num_faces;     /* faces that produced at least one triangle */
  int64_t num_submeshes;
} thea_mesh_info;

/* MeshGroup<DisplayMesh>::load(path) (Graphics/MeshGroup.hpp:471-497) with the default codec options, for the OFF
 * (.off, .off.bin; ASCII and binary, Graphics/MeshCodecOff.hpp), OBJ (Graphics/MeshCodecObj.hpp) and PLY (ASCII and
 * binary, Graphics/MeshCodecPly.hpp) codecs, chosen by the file extension. Submeshes come in file order (OBJ: one per g/o group that has faces; each submesh's vertices are the
 * distinct vertex/texcoord/normal references of its faces in ascending order). Faces are triangulated as
 * DisplayMesh::addFace does (Graphics/DisplayMesh.cpp:249-320); faces the non-strict readers skip (bad, out-of-range or,
 * in OFF and PLY, repeated indices) are skipped. Binary PLY properties beyond a vertex's coordinates and a face's index
 * list, and elements of other kinds, are skipped as the header describes them (the reference's binary reader cannot
 * read such files). 3DS (.3ds, Graphics/MeshCodec3ds.hpp over lib3ds 1.x): one submesh per triangle mesh of the file
 * in lib3ds's order (sorted by object name, file order among equal names), node transforms not applied, meshes without
 * vertices skipped; faces with an out-of-range or repeated index are skipped but numbered, and vertex and face numbers
 * run over the whole file. */
THEA_API thea_status thea_mesh_read(const char * path, thea_mesh ** out_mesh);
/* The same readers on a file's bytes in host memory, with the codec named ("3ds", "obj", "off" or "ply"): MeshGroup::read
 * from a BinaryInputStream with an explicit codec (Graphics/MeshGroup.hpp:324-352). */
THEA_API thea_status thea_mesh_read_buffer(const void * data, int64_t bytes, const char * codec, thea_mesh ** out_mesh);
THEA_API thea_status thea_mesh_get_info(const thea_mesh * mesh, thea_mesh_info * info);
/* Copies the arrays to host buffers (each nullable): vertices (3 x num_vertices floats), vertex_source (file vertex index
 * of each vertex, 0-based), triangles (3 x num_triangles indices into vertices), triangle_face (source face index of each
 * triangle: the OFF face number, the OBJ reader's running face count, the PLY reader's count of faces handed to
 * the mesh, or the 3DS reader's face number over the file), submesh_vertex_offsets and
 * submesh_triangle_offsets (num_submeshes + 1 entries each). */
THEA_API thea_status thea_mesh_copy(const thea_mesh * mesh, float * vertices, int32_t * vertex_source,
                                    int32_t * triangles, int32_t * triangle_face, int64_t * submesh_vertex_offsets,
                                    int64_t * submesh_triangle_offsets);
THEA_API thea_status thea_mesh_destroy(thea_mesh * mesh);

/* Triangles of one polygon of num_vertices host positions (xyz) as DisplayMesh::addFace makes them: a triangle as is,
 * a quad by Polygon3::triangulateQuad (Polygon3.hpp:245-285), more vertices by Polygon3::triangulate
 * (Polygon3.cpp:179-270). Writes local vertex indices, three per triangle, to out_triangles (room for
 * 3 x (num_vertices - 2)) and the triangle count (0: a degenerate face, which the mesh skips) to out_count. */
THEA_API thea_status thea_triangulate_face(const float * positions, int32_t num_vertices, int32_t * out_triangles,
                                           int32_t * out_count);

/* k nearest elements of a BVH to each query, 1 <= k <= 32, sorted by increasing squared distance (ties: lower
 * index first): points of a point BVH, or triangles of a mesh BVH (built with THEA_LAYOUT_CLOSEST; the squared
 * distance to the triangle's closest point, as closestElement computes it). exclude_index (nullable) gives per query an element index to skip (the reference's FilterSelf,
 * Code/Source/Algorithms/PointSet3.hpp:576-583). dist_bound < 0: unbounded; else only squared distances strictly below
 * dist_bound^2. Unused slots: index -1, squared distance -1.
 * Replaces BvhN::kClosestPairs<MetricL2>(query, BoundedSortedArrayN<k, NeighborPair>&, dist_bound) (BvhN.hpp:1139-1146). */
THEA_API thea_status thea_k_closest(const thea_bvh * point_bvh, const float * queries, int64_t num_queries, int32_t k,
                                    float dist_bound, const int32_t * exclude_index, int32_t * out_index,
                                    float * out_sq_distance, void * stream);

/* k-nearest-neighbour graph of the BVH's own points: query i is point i, excluding itself. Rows in point order. */
THEA_API thea_status thea_k_closest_self(const thea_bvh * point_bvh, int32_t k, int32_t * out_index,
                                         float * out_sq_distance, void * stream);

/* ---- forests and batched queries ------------------------------------------------------------------------------------ */

/* A forest holds one BVH per mesh (or point set), built together in one pass. Mesh m owns faces
 * [mesh_face_offsets[m], mesh_face_offsets[m+1]) of `faces` (host array of num_meshes + 1 entries, each mesh non-empty);
 * faces index the shared `vertices` array. Results report element indices within their own mesh. A forest is a
 * thea_bvh: thea_bvh_destroy releases it. No reference counterpart: the reference builds one BvhN per mesh
 * (BvhN.hpp:705); this replaces a loop of MeshBvh::init calls. */
THEA_API thea_status thea_mesh_forest_build(const float * vertices, int64_t num_vertices, const int32_t * faces,
                                            const int64_t * mesh_face_offsets, int32_t num_meshes,
                                            const thea_build_config * config, void * stream, thea_bvh ** out_forest);

/* One point BVH per point set: set m owns points [set_offsets[m], set_offsets[m+1]) (host array, sets non-empty). */
THEA_API thea_status thea_point_forest_build(const float * points, const int64_t * set_offsets, int32_t num_sets,
                                             const thea_build_config * config, void * stream,
                                             thea_bvh ** out_forest);

/* Batched queries in one persistent launch. Queries are grouped by mesh: queries of mesh m are
 * [query_offsets[m], query_offsets[m+1]) (num_meshes + 1 entries). Every array must be device memory; the calls are
 * asynchronous on `stream`, allocate only from the library's stream-ordered pool and never synchronize, so a sequence of
 * them can be captured with thea_graph_capture_begin/end. queries_per_warp: queries a warp takes per work fetch
 * (multiple of 32; 0 = 64). Per-query results as the single-BVH calls; the loop of closestElement calls over many meshes
 * that this replaces is the reference's only form.
 * hard_query_budget (closest element only): each query first runs on one thread for at most this many traversal steps;
 * queries that need more (points deep inside a closed mesh, where thousands of nodes lie within the bound) are then
 * finished by a whole warp each, 32 lanes expanding nodes together. 0 = default (32), negative = one thread per query
 * throughout. Results do not depend on it. */
THEA_API thea_status thea_batch_closest_element(const thea_bvh * mesh_forest, const float * queries,
                                                const int64_t * query_offsets, int64_t num_queries, float dist_bound,
                                                int32_t precision, int32_t queries_per_warp, int32_t hard_query_budget,
                                                int32_t * out_index, float * out_distance, float * out_closest_point,
                                                float * out_error, void * stream);
THEA_API thea_status thea_batch_ray_intersection(const thea_bvh * mesh_forest, const float * origins,
                                                 const float * directions, const int64_t * query_offsets,
                                                 int64_t num_rays, float max_time, int32_t queries_per_warp,
                                                 float * out_time, int32_t * out_index, void * stream);
THEA_API thea_status thea_batch_k_closest(const thea_bvh * point_forest, const float * queries,
                                          const int64_t * query_offsets, int64_t num_queries, int32_t k,
                                          float dist_bound, int32_t queries_per_warp, int32_t * out_index,
                                          float * out_sq_distance, void * stream);

/* ---- CUDA graphs ------------------------------------------------------------------------------------------------------ */

typedef struct thea_graph thea_graph;

/* Captures the asynchronous calls issued on `stream` between begin and end (thread-local capture mode) into a CUDA
 * graph, instantiated for replay with thea_graph_launch. Calls that synchronize (host arrays, builds, sampling) cannot
 * be captured. */
THEA_API thea_status thea_graph_capture_begin(void * stream);
THEA_API thea_status thea_graph_capture_end(void * stream, thea_graph ** out_graph);
THEA_API thea_status thea_graph_launch(thea_graph * graph, void * stream);
THEA_API thea_status thea_graph_destroy(thea_graph * graph);

/* ---- autotuning ------------------------------------------------------------------------------------------------------- */

typedef struct thea_tuning {
  int32_t width;              /* chosen BVH width */
  int32_t max_leaf_size;      /* chosen leaf size */
  int32_t queries_per_warp;   /* chosen work-fetch size */
  float milliseconds;         /* time of the chosen configuration on the sample */
  int32_t candidates;         /* configurations timed */
  int32_t hard_query_budget;  /* chosen per-thread step budget (-1: one thread per query throughout) */
  int32_t reserved[2];
} thea_tuning;

/* Times batched closest-point queries on a sample workload (a mesh forest's inputs plus device queries grouped by
 * mesh) for every BVH width (4, 8) and leaf size (1, 2, 4): queries-per-warp (32, 64, 128) with one thread per query
 * throughout, then step budgets (12, 32, 128) at the best queries-per-warp; returns the fastest (36 candidates).
 * Synchronizes the stream. */
THEA_API thea_status thea_autotune_batch_closest(const float * vertices, int64_t num_vertices, const int32_t * faces,
                                                 const int64_t * mesh_face_offsets, int32_t num_meshes,
                                                 const float * queries, const int64_t * query_offsets,
                                                 int64_t num_queries, int32_t precision, void * stream,
                                                 thea_tuning * out_tuning);

/* All points within `radius` of each query, inclusive (squared FP32 distance <= radius * radius, as BallN::contains):
 * replaces BvhN::rangeQueryIndices / processRange with a Ball3 range (BvhN.hpp:1208-1219, 2118-2171), the query behind
 * PointSet3's proximity graph. Output is a CSR list in two calls. Call 1, with out_index == NULL: writes out_offsets
 * (num_queries + 1 entries; out_offsets[num_queries] = total). Call 2, with the same queries, radius and exclusions and
 * the offsets of call 1: writes out_index (total entries; query q's neighbours in [out_offsets[q], out_offsets[q + 1]),
 * in ascending element index) and, if not NULL, out_sq_distance. exclude_index (nullable): per-query element to skip.
 * All arrays are device memory. Call 2 synchronizes the stream (it reads the total). */
THEA_API thea_status thea_radius_neighbors(const thea_bvh * point_bvh, const float * queries, int64_t num_queries,
                                           float radius, const int32_t * exclude_index, int64_t * out_offsets,
                                           int32_t * out_index, float * out_sq_distance, void * stream);

/* ---- tensor-core k-NN candidates ----------------------------------------------------------------------------------- */

#define THEA_KNN_CANDIDATES_TRAVERSAL 0  /* best-first BVH traversal from an unbounded start (thea_k_closest_self) */
#define THEA_KNN_CANDIDATES_GRAM 1       /* tensor-core Gram tiles seed the traversal with an exact bound */

/* thea_k_closest_self with a choice of candidate generation; results are identical for both modes. GRAM: the points,
 * in the BVH's leaf (Morton) order, are scored in tiles of 128 queries x 512 neighbouring candidates by tcgen05 MMAs
 * (FP16 operands, FP32 accumulation in tensor memory) on keys |b|^2 - 2 a.b; each query's best-scoring candidates are
 * re-ranked with the reference's FP32 squared distance, and the k-th of those (an upper bound on the k-th neighbour
 * distance, from actual points) seeds the exact BVH search. Sets with fewer than 512 points use the traversal alone. */
THEA_API thea_status thea_k_closest_self_ex(const thea_bvh * point_bvh, int32_t k, int32_t candidates,
                                            int32_t * out_index, float * out_sq_distance, void * stream);

/* The Gram tile alone (device arrays; a: num_a <= 128 points, b: num_b <= 512 points, 3 floats each; out_keys: 128 x 512
 * floats): out_keys[r * 512 + j] = |b_j|^2 - 2 a_r . b_j with coordinates relative to a[0], divided by the largest
 * coordinate magnitude of the tile, rounded to FP16, accumulated in FP32 by the tensor cores. Rows r >= num_a and
 * columns j >= num_b are padding. */
THEA_API thea_status thea_point_gram_tile(const float * a, int32_t num_a, const float * b, int32_t num_b,
                                          float * out_keys, void * stream);

/* Diagnostic of the failure path of the library's bounded device-side waits (the tensor-core kernels wait on an mbarrier
 * for their MMAs; every such wait gives up after a fixed number of rounds and reports instead of hanging). One warp
 * waits on a barrier phase that nothing completes, with the given round limit (1..2^20). Returns
 * THEA_ERR_DEVICE_TIMEOUT when the wait gave up (the expected outcome; the context stays usable), THEA_OK if the phase
 * completed. No counterpart in the reference. Synchronizes the stream. */
THEA_API thea_status thea_selftest_bounded_wait(int32_t spin_limit, void * stream);

/* Device errors and query status. Query kernels raise bits in their handle's device error word (see
 * thea_bvh_info.device_error_bits). Every query call on a handle (closest element, rays, k-NN, radius, batched, pairs,
 * Visibility, ShapeDiameter) copies the word to a host mirror on its stream as its last step. A call that synchronizes
 * (host arrays) returns THEA_ERR_INTERNAL for bit 1 (results may miss elements) or THEA_ERR_DEVICE_TIMEOUT for bit 2
 * (results are exact: the affected queries ran without the tensor-core bound); an asynchronous call (device arrays)
 * leaves the report to the next call on the handle once its stream has passed the copy. A report clears the bits; the
 * call that reports them still runs and writes its results.
 *
 * This hook ORs `bits` into the handle's device word with a host-to-device copy on `stream` (no kernel), so that tests
 * can follow a device error to the status of the next query call. No counterpart in the reference. */
THEA_API thea_status thea_selftest_set_error_bits(thea_bvh * bvh, uint32_t bits, void * stream);

/* The FP32 running sum fl(... fl(fl(start + t[0]) + t[1]) ...) over num_terms terms (host or device memory), computed
 * as the library computes updateAverageSeparation's sum (PointSet3.hpp:688-702) for thea_sample_graph: on the device,
 * runs of terms added as exact integer multiples of the sum's ulp, bit for bit the sequential loop. Writes the sum to
 * the host float out_sum. No counterpart in the reference (it exposes the summation for tests). Synchronizes the
 * stream. */
THEA_API thea_status thea_selftest_running_sum(const float * terms, int64_t num_terms, float start, float * out_sum,
                                               void * stream);

/* ---- sampling ------------------------------------------------------------------------------------------------------ */

/* Streams of the reference's Random(seed) (THEA_RNG_THEA_MT sampling, thea_random_sphere, thea_visibility) of 1,024
 * twists (638,976 words) or more are generated in parallel chunks of 512 twists from jump-ahead start states: the first
 * such stream on a device computes the 512-twist jump as a 19,968 x 19,968 bit matrix (about 50 MB of device memory,
 * kept until the process exits; a few milliseconds); during a stream capture without that table, or for shorter
 * streams, one block generates the words in order. The words are the same either way. */
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
 * device current); make that first call before any stream capture. The address is cached per device ordinal for the
 * life of the process: after a call that tears the device's context down (cudaDeviceReset), the cached address is
 * stale and later calls on that device must not be made. All calls on a device share the one array, and every call
 * rewrites the parts it reads before reading them; calls whose work overlaps on the GPU (different streams or threads
 * at the same time) race on it and must be serialized by the caller. Face indices outside [0, num_vertices) are
 * detected on the device without being dereferenced and rejected with THEA_ERR_INVALID_ARGUMENT. The call synchronizes
 * `stream` once, to read back the total area. The cumulative areas are summed by one thread in index order (the
 * reference's sequence of FP64 roundings): measured on a GB300 with 100,000 samples, 7.5 ms a call for 81,920
 * triangles, growing linearly to 91 ms at 1,048,352, where thea_sample_by_area (an exact parallel scan) takes 0.35 and
 * 0.41 ms. */
THEA_API thea_status thea_sample_by_area_noalloc(const float * vertices, int64_t num_vertices, const int32_t * faces,
                                                 int64_t num_faces, int64_t num_samples, uint32_t seed, int32_t rng,
                                                 float * out_positions, float * out_normals, int32_t * out_faces,
                                                 int64_t * out_num_written, void * stream);

/* ---- serving ------------------------------------------------------------------------------------------------------- */

/* A request loop over meshes kept resident in device memory. The reference has no serving layer (its queries are
 * synchronous C++ calls on a BvhN); these entry points are new. Each request is one of the three query kinds against one
 * resident mesh, with the same per-query results as the single-BVH calls (thea_closest_element, thea_ray_intersection,
 * thea_k_closest over the mesh's vertices): bit-identical, whatever else is in flight.
 *
 * Continuous batching: a dispatcher thread cuts requests into pieces of at most max_piece_queries queries and packs
 * pending pieces (smallest remaining request first; a request pending longer than max_wait_ms goes first) into batches
 * of at most max_batch_queries queries, one persistent launch per query kind. Up to `slots` batches are in flight at
 * once, each on its own stream, so requests that arrive while others run are admitted as soon as a slot and memory
 * free up, and their copies and kernels overlap with the batches already on the device. A batch made only of requests
 * of at most small_request_queries queries runs on a stream of the device's highest priority.
 *
 * Admission: resident BVHs (mesh BVH with both layouts plus a point BVH over the mesh's vertices) and the device staging
 * buffers of in-flight pieces count against memory_budget_bytes. A mesh that does not fit is refused at
 * thea_server_add_mesh, a request whose smallest piece can never fit is refused at submit (both
 * THEA_ERR_ADMISSION_REFUSED), and other requests wait until earlier pieces finish. Request arrays may be host memory
 * (staged through device buffers; pinned memory makes the copies asynchronous) or device memory (used in place, no
 * staging bytes). They must stay valid, and outputs untouched, until thea_server_wait has returned the request. */

typedef struct thea_server thea_server;

typedef struct thea_server_config {
  int64_t memory_budget_bytes;   /* resident BVHs + staging of in-flight pieces (0: 8 GiB) */
  int32_t slots;                 /* batches in flight at once, one stream pair each (0: 6) */
  int32_t max_batch_queries;     /* queries per batch (0: 65536) */
  int32_t max_piece_queries;     /* largest piece of one request (0: 65536) */
  int32_t precision;             /* closest-element requests: THEA_PRECISION_* */
  int32_t width;                 /* BVH width of resident meshes, 4 or 8 (0: 4) */
  int32_t max_leaf_size;         /* leaf size of resident mesh BVHs (0: default) */
  int32_t small_request_queries; /* requests of at most this many queries get their own latency figures (0: 65536) */
  int32_t max_wait_ms;           /* pending longer than this: served before smaller requests (0: 20) */
  int32_t test_executor;         /* 1: test executor for the host-side scheduling logic. No CUDA call at all: meshes are
                                    not built (their size is estimated), no results are written, and a batch finishes
                                    test_ns_per_query x its queries after it starts. 0: the GPU. */
  int32_t test_ns_per_query;
  int32_t hard_query_budget;     /* > 0: closest-element stack pops on one thread before a query is finished by a warp
                                    of its own in a second launch; <= 0: one thread per query throughout (default:
                                    measured lower p99 latency on the config-4 mix) */
  int32_t reserved[5];           /* must be zero */
} thea_server_config;

#define THEA_REQUEST_CLOSEST 0  /* closest element: thea_closest_element */
#define THEA_REQUEST_RAY 1      /* first ray hit: thea_ray_intersection */
#define THEA_REQUEST_KNN 2      /* k nearest mesh vertices: thea_k_closest */

typedef struct thea_request {
  int32_t type;              /* THEA_REQUEST_* */
  int32_t mesh;              /* id from thea_server_add_mesh */
  int64_t num_queries;       /* >= 1 */
  const float * queries;     /* closest and k-NN: query points; ray: origins (3 floats each) */
  const float * directions;  /* ray only (3 floats each) */
  float bound;               /* closest: dist_bound; ray: max_time; k-NN: dist_bound (negative: none) */
  int32_t k;                 /* k-NN: 1..32 */
  int32_t * out_index;       /* closest and ray: num_queries; k-NN: num_queries x k (-1: none) */
  float * out_value;         /* closest: distance; ray: hit time; k-NN: squared distance (-1: none); may be NULL */
  float * out_point;         /* closest only: closest points (3 floats each); may be NULL */
} thea_request;

typedef struct thea_server_stats {
  int64_t submitted;
  int64_t completed;
  int64_t failed;
  int64_t cancelled;
  int64_t refused;           /* requests refused at submit */
  int64_t queries_completed;
  int64_t batches;
  int64_t resident_meshes;
  int64_t resident_bytes;
  int64_t inflight_bytes;    /* staging bytes of pieces admitted and not finished */
  int64_t pending_requests;
  double p50_ms;             /* latency from submit to results written, completed requests */
  double p99_ms;
  double max_ms;
  double small_p50_ms;       /* the same over requests of at most small_request_queries queries */
  double small_p99_ms;
  double busy_seconds;       /* first submit to last completion since the last reset */
  double queries_per_second; /* queries_completed / busy_seconds */
} thea_server_stats;

/* Starts the dispatcher thread on the current device. */
THEA_API thea_status thea_server_create(const thea_server_config * config, thea_server ** out_server);
/* Pending requests end THEA_ERR_CANCELLED; batches on the device are waited for; all memory is released. */
THEA_API thea_status thea_server_destroy(thea_server * server);
/* Builds and keeps resident the BVHs of one mesh (vertices and faces as for thea_mesh_bvh_build, host or device).
 * Synchronous. THEA_ERR_ADMISSION_REFUSED if it does not fit the budget. */
THEA_API thea_status thea_server_add_mesh(thea_server * server, const float * vertices, int64_t num_vertices,
                                          const int32_t * faces, int64_t num_faces, int32_t * out_mesh);
/* The mesh takes no new requests; its memory is released when the requests already submitted for it have finished. */
THEA_API thea_status thea_server_remove_mesh(thea_server * server, int32_t mesh);
/* Queues a request and returns at once with its ticket. */
THEA_API thea_status thea_server_submit(thea_server * server, const thea_request * request, uint64_t * out_ticket);
/* Waits up to timeout_us microseconds (negative: no limit) for a request. THEA_OK: the request ended and its ticket is
 * retired; *out_request_status is its outcome (THEA_OK, THEA_ERR_CANCELLED, THEA_ERR_CUDA, ...) and *out_latency_ms the
 * time from submit to results written. THEA_ERR_WAIT_TIMEOUT: not finished yet (wait again). Either output may be NULL. */
THEA_API thea_status thea_server_wait(thea_server * server, uint64_t ticket, int64_t timeout_us,
                                      thea_status * out_request_status, double * out_latency_ms);
/* Cancels the pieces of a request that have not started; a request with pieces on the device finishes those and ends
 * THEA_ERR_CANCELLED with its outputs partly written. */
THEA_API thea_status thea_server_cancel(thea_server * server, uint64_t ticket);
THEA_API thea_status thea_server_get_stats(thea_server * server, thea_server_stats * out_stats);
/* Clears the latency records and counters (not the resident meshes). */
THEA_API thea_status thea_server_reset_stats(thea_server * server);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* THEA_GPU_H */
