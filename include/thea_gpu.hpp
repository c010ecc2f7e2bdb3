// thea_gpu.hpp -- header-only C++ wrapper over the C ABI in thea_gpu.h, with the method names of the reference's
// spatial-query classes (sidch/Thea: Code/Source/Algorithms/BvhN.hpp, MeshBvh.hpp, MeshSampler.hpp) in batched form.
//
// Arrays may live in host or device memory (see thea_gpu.h). Errors surface as thea_gpu::Exception carrying the status.
#ifndef THEA_GPU_HPP
#define THEA_GPU_HPP

#include "thea_gpu.h"

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace thea_gpu {

class Exception : public std::runtime_error {
 public:
  Exception(thea_status s, std::string const & msg) : std::runtime_error(msg), status_(s) {}
  thea_status status() const { return status_; }

 private:
  thea_status status_;
};

inline void check(thea_status s) {
  if (s != THEA_OK) {
    char const * m = thea_last_error_message();
    throw Exception(s, std::string(thea_status_string(s)) + ": " + (m ? m : ""));
  }
}

struct BuildOptions {
  int32_t width = 4;          // 4 or 8 children per node
  int32_t max_leaf_size = 0;  // 0: library default
  uint32_t layouts = 0;       // THEA_LAYOUT_* mask for meshes, 0 = both
  int32_t query_order = 0;    // 1: traverse large batches in Morton order of the query point
  thea_build_config config() const {
    thea_build_config c{};
    c.width = width;
    c.max_leaf_size = max_leaf_size;
    c.layouts = layouts;
    c.query_order = query_order;
    return c;
  }
};

class BvhHandle {
 public:
  BvhHandle() = default;
  BvhHandle(BvhHandle const &) = delete;
  BvhHandle & operator=(BvhHandle const &) = delete;
  BvhHandle(BvhHandle && o) noexcept : h_(o.h_) { o.h_ = nullptr; }
  BvhHandle & operator=(BvhHandle && o) noexcept {
    std::swap(h_, o.h_);
    return *this;
  }
  ~BvhHandle() {
    if (h_) thea_bvh_destroy(h_);
  }
  thea_bvh * get() const { return h_; }
  thea_bvh_info info() const {
    thea_bvh_info i;
    check(thea_bvh_get_info(h_, &i));
    return i;
  }
  // BvhN::setTransform / clearTransform: affine_3x4 row-major [L | t]
  void setTransform(float const * affine_3x4, void * stream = nullptr) {
    check(thea_bvh_set_transform(h_, affine_3x4, stream));
  }
  void clearTransform() { check(thea_bvh_clear_transform(h_)); }
  bool hasTransform() const {
    int32_t has = 0;
    check(thea_bvh_get_transform(h_, &has, nullptr, nullptr));
    return has != 0;
  }
  // BvhN::closestPair with another BVH as the query (one side must hold points): false when no pair qualifies.
  // query_point / target_point (nullable): the closest points on the two elements.
  bool closestPair(BvhHandle const & query, int32_t * query_index, int32_t * target_index, float * sq_distance,
                   double dist_bound = -1, float * query_point = nullptr, float * target_point = nullptr,
                   void * stream = nullptr) const {
    check(thea_bvh_closest_pair(h_, query.h_, (float)dist_bound, query_index, target_index, sq_distance, query_point,
                                target_point, stream));
    return *query_index >= 0;
  }
  // BvhN::kClosestPairs between two point BVHs: the k closest pairs, ascending; returns how many were found.
  int32_t kClosestPairs(BvhHandle const & query, int32_t k, int32_t * query_indices, int32_t * target_indices,
                        float * sq_distances, double dist_bound = -1, void * stream = nullptr) const {
    int32_t count = 0;
    check(thea_bvh_k_closest_pairs(h_, query.h_, k, (float)dist_bound, query_indices, target_indices, sq_distances,
                                   &count, stream));
    return count;
  }

  // Byte image of the built BVH (thea_bvh_serialize); the class's fromImage reloads it without a rebuild.
  std::vector<unsigned char> serialize(void * stream = nullptr) const {
    int64_t n = 0;
    check(thea_bvh_serialize(h_, nullptr, 0, &n, stream));
    std::vector<unsigned char> out((size_t)n);
    check(thea_bvh_serialize(h_, out.data(), n, &n, stream));
    return out;
  }

 protected:
  template <class T>
  static T loadImage(void const * image, int64_t bytes, bool mesh, void * stream) {
    T t;
    check(thea_bvh_deserialize(image, bytes, stream, &static_cast<BvhHandle &>(t).h_));
    if ((t.info().is_mesh != 0) != mesh)
      throw Exception(THEA_ERR_INVALID_ARGUMENT, "bvh image holds the other kind of BVH");
    return t;
  }

  thea_bvh * h_ = nullptr;
};

// MeshBvh: a BVH over the triangles of a mesh; element index = face index (MeshBvh::add + MeshBvh::init).
class MeshBvh : public BvhHandle {
  friend class BvhHandle;
  MeshBvh() = default;

 public:
  // A handle on the current device from a byte image made by serialize() of a MeshBvh
  static MeshBvh fromImage(void const * image, int64_t bytes, void * stream = nullptr) {
    return loadImage<MeshBvh>(image, bytes, true, stream);
  }
  MeshBvh(float const * vertices, int64_t num_vertices, int32_t const * faces, int64_t num_faces,
          BuildOptions const & opt = BuildOptions(), void * stream = nullptr) {
    thea_build_config c = opt.config();
    check(thea_mesh_bvh_build(vertices, num_vertices, faces, num_faces, &c, stream, &h_));
  }

  // BvhN::closestElement<MetricL2>(query, dist_bound, compat, &dist, &closest_point), batched over n queries.
  void closestElement(float const * queries, int64_t n, int32_t * indices, float * distances = nullptr,
                      float * closest_points = nullptr, double dist_bound = -1, void * stream = nullptr) const {
    check(thea_closest_element(h_, queries, n, (float)dist_bound, indices, distances, closest_points, stream));
  }

  // Single host query, as the reference's per-call form: returns the element index or -1.
  int64_t closestElement(float const query[3], double dist_bound = -1, double * dist = nullptr,
                         float * closest_point = nullptr) const {
    int32_t idx = -1;
    float d = -1, cp[3] = {0, 0, 0};
    check(thea_closest_element(h_, query, 1, (float)dist_bound, &idx, &d, cp, nullptr));
    if (idx >= 0) {
      if (dist) *dist = d;
      if (closest_point) { closest_point[0] = cp[0]; closest_point[1] = cp[1]; closest_point[2] = cp[2]; }
    }
    return idx;
  }

  // BvhN::rayStructureIntersection<RayIntersectionTester>(ray, max_time), batched: time (-1 = miss), element, normal.
  void rayStructureIntersection(float const * origins, float const * directions, int64_t n, float * times,
                                int32_t * indices, float * normals = nullptr, float max_time = -1,
                                void * stream = nullptr) const {
    check(thea_ray_intersection(h_, origins, directions, n, max_time, times, indices, normals, stream));
  }

  // BvhN::rayIntersectionTime<RayIntersectionTester>(ray, max_time), batched.
  // closestElement with a precision mode (THEA_PRECISION_*) and the per-query |distance - FP64 distance| (nullable)
  void closestElementEx(float const * queries, int64_t n, int32_t precision, int32_t * indices,
                        float * distances = nullptr, float * closest_points = nullptr, float * errors = nullptr,
                        double dist_bound = -1, void * stream = nullptr) const {
    check(thea_closest_element_ex(h_, queries, n, (float)dist_bound, precision, indices, distances, closest_points,
                                  errors, stream));
  }

  // rayStructureIntersection with the FP64 watertight verdict beside the reference's FP32 one (flags: THEA_RAY_FLAG_*)
  void rayStructureIntersectionEx(float const * origins, float const * directions, int64_t n, float * times,
                                  int32_t * indices, float * times_fp64, int32_t * indices_fp64, int32_t * flags,
                                  float max_time = -1, void * stream = nullptr) const {
    check(thea_ray_intersection_ex(h_, origins, directions, n, max_time, THEA_PRECISION_FP64_RECHECK, times, indices,
                                   nullptr, times_fp64, indices_fp64, flags, stream));
  }

  void rayIntersectionTime(float const * origins, float const * directions, int64_t n, float * times,
                           float max_time = -1, void * stream = nullptr) const {
    check(thea_ray_intersection(h_, origins, directions, n, max_time, times, nullptr, nullptr, stream));
  }

  // BvhN::rayIntersects, batched: hit[i] = 1 if ray i meets an element within max_time (any-hit search).
  void rayIntersects(float const * origins, float const * directions, int64_t n, uint8_t * hit, float max_time = -1,
                     void * stream = nullptr) const {
    check(thea_ray_intersects(h_, origins, directions, n, max_time, hit, stream));
  }

  // BvhN::kClosestPairs with point queries on a mesh: the k nearest triangles of each query, n x k, sorted.
  void kClosestPairs(float const * queries, int64_t n, int32_t k, int32_t * indices, float * sq_distances,
                     double dist_bound = -1, void * stream = nullptr) const {
    check(thea_k_closest(h_, queries, n, k, (float)dist_bound, nullptr, indices, sq_distances, stream));
  }
  using BvhHandle::kClosestPairs;

  // Visibility::compute for n points (Random(seed) in place of Random::common()): escaped fraction per point.
  void visibility(float const * positions, int64_t n, double * fractions, int32_t num_rays = 100, uint32_t seed = 0,
                  void * stream = nullptr) const {
    check(thea_visibility(h_, positions, n, num_rays, seed, fractions, stream));
  }

  // ShapeDiameter(bvh, scale)::compute for n points; normals nullable (closest element's normal), scale <= 0: the
  // BVH bounds' diagonal. -1 where no ray counts.
  void shapeDiameter(float const * positions, float const * normals, int64_t n, double * sdf, double scale = -1,
                     bool only_interior = true, void * stream = nullptr) const {
    check(thea_shape_diameter(h_, positions, normals, n, (float)scale, only_interior ? 1 : 0, sdf, stream));
  }
};

// BvhN<Vector3, 3>: a BVH over points; element index = point index.
class PointBvh : public BvhHandle {
  friend class BvhHandle;
  PointBvh() = default;

 public:
  // A handle on the current device from a byte image made by serialize() of a PointBvh
  static PointBvh fromImage(void const * image, int64_t bytes, void * stream = nullptr) {
    return loadImage<PointBvh>(image, bytes, false, stream);
  }
  PointBvh(float const * points, int64_t num_points, BuildOptions const & opt = BuildOptions(),
           void * stream = nullptr) {
    thea_build_config c = opt.config();
    c.layouts = 0;
    check(thea_point_bvh_build(points, num_points, &c, stream, &h_));
  }

  // BvhN::kClosestPairs<MetricL2>(query, BoundedSortedArrayN<k, NeighborPair>&, dist_bound), batched: n x k indices
  // and squared distances, sorted, unused slots -1. exclude (nullable): per-query element to skip.
  void kClosestPairs(float const * queries, int64_t n, int32_t k, int32_t * indices, float * sq_distances,
                     double dist_bound = -1, int32_t const * exclude = nullptr, void * stream = nullptr) const {
    check(thea_k_closest(h_, queries, n, k, (float)dist_bound, exclude, indices, sq_distances, stream));
  }
  using BvhHandle::kClosestPairs;

  // BvhN::rangeQueryIndices with a Ball3: points within `radius` (inclusive) of each query as CSR, in two calls
  // (thea_radius_neighbors; device arrays): indices == nullptr writes offsets (n + 1); then the same call with those
  // offsets fills indices and squared distances (nullable), ascending per query.
  void rangeQuery(float const * queries, int64_t n, float radius, int64_t * offsets, int32_t * indices = nullptr,
                  float * sq_distances = nullptr, int32_t const * exclude = nullptr, void * stream = nullptr) const {
    check(thea_radius_neighbors(h_, queries, n, radius, exclude, offsets, indices, sq_distances, stream));
  }

  // k-nearest-neighbour graph of the indexed points (each point excluding itself), rows in point order.
  void kClosestSelf(int32_t k, int32_t * indices, float * sq_distances, void * stream = nullptr) const {
    check(thea_k_closest_self(h_, k, indices, sq_distances, stream));
  }

  // The same graph with a choice of candidate generation (THEA_KNN_CANDIDATES_*); results are identical.
  void kClosestSelf(int32_t k, int32_t candidates, int32_t * indices, float * sq_distances,
                    void * stream = nullptr) const {
    check(thea_k_closest_self_ex(h_, k, candidates, indices, sq_distances, stream));
  }
};

// Many meshes (or point sets) in one structure, queried in one persistent launch. Faces index the shared vertex array;
// mesh m owns faces [mesh_face_offsets[m], mesh_face_offsets[m + 1]) (host array, num_meshes + 1 entries). Queries
// are grouped by mesh through device-resident query_offsets.
class MeshForest : public BvhHandle {
  friend class BvhHandle;
  MeshForest() = default;

 public:
  // A handle on the current device from a byte image made by serialize() of a MeshForest
  static MeshForest fromImage(void const * image, int64_t bytes, void * stream = nullptr) {
    return loadImage<MeshForest>(image, bytes, true, stream);
  }
  MeshForest(float const * vertices, int64_t num_vertices, int32_t const * faces, int64_t const * mesh_face_offsets,
             int32_t num_meshes, BuildOptions const & opt = BuildOptions(), void * stream = nullptr) {
    thea_build_config c = opt.config();
    check(thea_mesh_forest_build(vertices, num_vertices, faces, mesh_face_offsets, num_meshes, &c, stream, &h_));
  }

  // hard_query_budget: 0 = default two-phase search, negative = one thread per query throughout
  void batchClosestElement(float const * queries, int64_t const * query_offsets, int64_t n, int32_t * indices,
                           float * distances = nullptr, float * closest_points = nullptr, float * errors = nullptr,
                           int32_t precision = THEA_PRECISION_FP32_REFERENCE, double dist_bound = -1,
                           int32_t queries_per_warp = 0, int32_t hard_query_budget = 0,
                           void * stream = nullptr) const {
    check(thea_batch_closest_element(h_, queries, query_offsets, n, (float)dist_bound, precision, queries_per_warp,
                                     hard_query_budget, indices, distances, closest_points, errors, stream));
  }

  void batchRayIntersection(float const * origins, float const * directions, int64_t const * query_offsets, int64_t n,
                            float * times, int32_t * indices = nullptr, float max_time = -1,
                            int32_t queries_per_warp = 0, void * stream = nullptr) const {
    check(thea_batch_ray_intersection(h_, origins, directions, query_offsets, n, max_time, queries_per_warp, times,
                                      indices, stream));
  }
};

class PointForest : public BvhHandle {
  friend class BvhHandle;
  PointForest() = default;

 public:
  // A handle on the current device from a byte image made by serialize() of a PointForest
  static PointForest fromImage(void const * image, int64_t bytes, void * stream = nullptr) {
    return loadImage<PointForest>(image, bytes, false, stream);
  }
  PointForest(float const * points, int64_t const * set_offsets, int32_t num_sets,
              BuildOptions const & opt = BuildOptions(), void * stream = nullptr) {
    thea_build_config c = opt.config();
    check(thea_point_forest_build(points, set_offsets, num_sets, &c, stream, &h_));
  }

  void batchKClosest(float const * queries, int64_t const * query_offsets, int64_t n, int32_t k, int32_t * indices,
                     float * sq_distances, double dist_bound = -1, int32_t queries_per_warp = 0,
                     void * stream = nullptr) const {
    check(thea_batch_k_closest(h_, queries, query_offsets, n, k, (float)dist_bound, queries_per_warp, indices,
                               sq_distances, stream));
  }
};

// CUDA-graph capture of asynchronous (device-array) calls on one stream, replayed with launch().
class Graph {
 public:
  explicit Graph(void * stream) : stream_(stream) { check(thea_graph_capture_begin(stream)); }
  Graph(Graph const &) = delete;
  Graph & operator=(Graph const &) = delete;
  void end() { check(thea_graph_capture_end(stream_, &g_)); }
  void launch(void * stream) const { check(thea_graph_launch(g_, stream)); }
  ~Graph() {
    if (g_) thea_graph_destroy(g_);
  }

 private:
  void * stream_;
  thea_graph * g_ = nullptr;
};

// The serving loop (thea_server_*): resident meshes, memory-budget admission, continuous batching.
class Server {
 public:
  explicit Server(thea_server_config const & config) { check(thea_server_create(&config, &s_)); }
  Server(Server const &) = delete;
  Server & operator=(Server const &) = delete;
  ~Server() {
    if (s_) thea_server_destroy(s_);
  }

  int32_t addMesh(float const * vertices, int64_t num_vertices, int32_t const * faces, int64_t num_faces) {
    int32_t id = -1;
    check(thea_server_add_mesh(s_, vertices, num_vertices, faces, num_faces, &id));
    return id;
  }
  void removeMesh(int32_t mesh) { check(thea_server_remove_mesh(s_, mesh)); }
  uint64_t submit(thea_request const & request) {
    uint64_t t = 0;
    check(thea_server_submit(s_, &request, &t));
    return t;
  }
  // true when the request ended (its outcome in *request_status); false if timeout_us passed first
  bool wait(uint64_t ticket, thea_status * request_status = nullptr, double * latency_ms = nullptr,
            int64_t timeout_us = -1) {
    thea_status r = thea_server_wait(s_, ticket, timeout_us, request_status, latency_ms);
    if (r == THEA_ERR_WAIT_TIMEOUT) return false;
    check(r);
    return true;
  }
  void cancel(uint64_t ticket) { check(thea_server_cancel(s_, ticket)); }
  thea_server_stats stats() const {
    thea_server_stats st{};
    check(thea_server_get_stats(s_, &st));
    return st;
  }

 private:
  thea_server * s_ = nullptr;
};

// MeshSampler::sampleEvenlyByArea (EXACT count mode), drawing from Random(seed).
class MeshSampler {
 public:
  MeshSampler(float const * vertices, int64_t num_vertices, int32_t const * faces, int64_t num_faces)
      : v_(vertices), nv_(num_vertices), f_(faces), nf_(num_faces) {}

  int64_t sampleEvenlyByArea(int64_t num_samples, float * positions, float * face_normals = nullptr,
                             int32_t * face_indices = nullptr, uint32_t seed = 0, int32_t rng = THEA_RNG_THEA_MT,
                             void * stream = nullptr) const {
    int64_t got = 0;
    check(thea_sample_by_area(v_, nv_, f_, nf_, num_samples, seed, rng, positions, face_normals, face_indices, &got,
                              stream));
    return got;
  }

 private:
  float const * v_;
  int64_t nv_;
  int32_t const * f_;
  int64_t nf_;
};

// BestFitSphereN<3> (Algorithms/BestFitSphereN.hpp): points collected on the host, the smallest enclosing ball computed
// on the GPU when first asked for. getDiameter() over a mesh's vertices is ShapeDiameter(mesh)'s default scale.
class BestFitSphere3 {
 public:
  void addPoint(float x, float y, float z) {
    pts_.push_back(x);
    pts_.push_back(y);
    pts_.push_back(z);
    updated_ = false;
  }
  void addPoints(float const * xyz, int64_t n) {
    pts_.insert(pts_.end(), xyz, xyz + 3 * n);
    updated_ = false;
  }
  void clear() {
    pts_.clear();
    updated_ = false;
  }
  // centre and radius as the reference returns them (Real = float)
  void getCenter(float * c) const {
    update();
    c[0] = (float)c_[0], c[1] = (float)c_[1], c[2] = (float)c_[2];
  }
  float getRadius() const { update(); return (float)r_; }
  float getDiameter() const { return 2.0f * getRadius(); }

 private:
  void update() const {
    if (updated_) return;
    check(thea_best_fit_sphere(pts_.data(), (int64_t)(pts_.size() / 3), c_, &r_, nullptr));
    updated_ = true;
  }
  std::vector<float> pts_;
  mutable double c_[3] = {0, 0, 0};
  mutable double r_ = 0;
  mutable bool updated_ = true;
};

// PointSet3's sample graph (Algorithms/PointSet3.hpp): samples (and optional normals) set once, an optional dense
// oversampling, then updateGraph() with Random(seed) in place of Random::common(). Host arrays.
class PointSet3 {
 public:
  explicit PointSet3(int32_t max_degree = 8, uint32_t seed = 0) : max_degree_(max_degree), seed_(seed) {}

  void setSamples(float const * positions, float const * normals, int64_t n) {
    pos_.assign(positions, positions + 3 * n);
    if (normals) nrm_.assign(normals, normals + 3 * n);
    else nrm_.clear();
    valid_ = false;
  }
  void addOversampling(float const * positions, float const * normals, int64_t n) {
    dpos_.insert(dpos_.end(), positions, positions + 3 * n);
    if (normals) dnrm_.insert(dnrm_.end(), normals, normals + 3 * n);
    valid_ = false;
  }
  int64_t numSamples() const { return (int64_t)(pos_.size() / 3); }

  // surface: a mesh BVH with the ray layout for the reachability test (used with normals), or nullptr
  void updateGraph(MeshBvh const * surface = nullptr) const {
    if (valid_) return;
    int64_t n = numSamples();
    nbr_.assign((size_t)(n * max_degree_), -1);
    sep_.assign((size_t)(n * max_degree_), 0.f);
    deg_.assign((size_t)n, 0);
    float const * nrm = nrm_.empty() ? nullptr : nrm_.data();
    thea_bvh const * surf = surface ? surface->get() : nullptr;
    if (dpos_.empty())
      check(thea_sample_graph(pos_.data(), nrm, n, max_degree_, seed_, surf, nbr_.data(), sep_.data(), deg_.data(),
                              avg_, nullptr));
    else
      check(thea_sample_graph_oversampled(pos_.data(), nrm, n, dpos_.data(), nrm ? dnrm_.data() : nullptr,
                                          (int64_t)(dpos_.size() / 3), max_degree_, seed_, surf, nbr_.data(),
                                          sep_.data(), deg_.data(), avg_, nullptr));
    valid_ = true;
  }
  // sample i's neighbours (ascending separation, then index) and their separations; numNeighbors(i) of them
  int32_t numNeighbors(int64_t i) const { updateGraph(); return deg_[(size_t)i]; }
  int32_t const * neighbors(int64_t i) const { updateGraph(); return nbr_.data() + i * max_degree_; }
  float const * separations(int64_t i) const { updateGraph(); return sep_.data() + i * max_degree_; }
  float getAverageSeparation() const { updateGraph(); return avg_[1]; }

 private:
  int32_t max_degree_;
  uint32_t seed_;
  std::vector<float> pos_, nrm_, dpos_, dnrm_;
  mutable std::vector<int32_t> nbr_, deg_;
  mutable std::vector<float> sep_;
  mutable float avg_[2] = {0, 0};
  mutable bool valid_ = false;
};

// MeshGroup<DisplayMesh>::load for 3DS, OFF, OBJ and PLY files, flattened into host arrays in the reference's element order;
// MeshBvh(file.vertices.data(), file.numVertices(), file.triangles.data(), file.numTriangles()) indexes its triangles.
class MeshFile {
 public:
  explicit MeshFile(std::string const & path) {
    thea_mesh * m = nullptr;
    check(thea_mesh_read(path.c_str(), &m));
    thea_mesh_info info{};
    thea_status s = thea_mesh_get_info(m, &info);
    if (s == THEA_OK) {
      vertices.resize((size_t)(3 * info.num_vertices));
      vertex_source.resize((size_t)info.num_vertices);
      triangles.resize((size_t)(3 * info.num_triangles));
      triangle_face.resize((size_t)info.num_triangles);
      submesh_vertex_offsets.resize((size_t)(info.num_submeshes + 1));
      submesh_triangle_offsets.resize((size_t)(info.num_submeshes + 1));
      s = thea_mesh_copy(m, vertices.data(), vertex_source.data(), triangles.data(), triangle_face.data(),
                         submesh_vertex_offsets.data(), submesh_triangle_offsets.data());
      num_faces = info.num_faces;
    }
    thea_mesh_destroy(m);
    check(s);
  }

  int64_t numVertices() const { return (int64_t)vertex_source.size(); }
  int64_t numTriangles() const { return (int64_t)triangle_face.size(); }

  std::vector<float> vertices;
  std::vector<int32_t> vertex_source, triangles, triangle_face;
  std::vector<int64_t> submesh_vertex_offsets, submesh_triangle_offsets;
  int64_t num_faces = 0;
};

}  // namespace thea_gpu

#endif  // THEA_GPU_HPP
