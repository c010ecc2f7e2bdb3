// TEST INFRASTRUCTURE ONLY -- C entry points over the REFERENCE's own spatial-query code, compiled in this build from the
// reference's sources (Code/Source/Algorithms/BvhN.hpp, BestFitSphereN.hpp with its vendored miniball, Triangle3.hpp,
// AxisAlignedBoxN.hpp, Random.cpp, ...) against eigen_subset.hpp in place of Eigen (which is absent here). Built into
// oracle/_ref/ by the oracle's Makefile when the reference sources are present; used only to pin the oracle
// (tests/golden/make_ref_golden.py writes its outputs as fixtures, and the CPU tests compare the oracle with it). Nothing here is restated: every query below is a
// call into the reference's classes.

#include "Algorithms/BestFitSphereN.hpp"
#include "Algorithms/BvhN.hpp"
#include "Algorithms/MetricL2.hpp"
#include "Algorithms/RayIntersectionTester.hpp"
#include "BoundedSortedArrayN.hpp"
#include "Random.hpp"
#include "Triangle3.hpp"

#include <cstdint>
#include <vector>

using namespace Thea;
using namespace Thea::Algorithms;

namespace {

typedef BvhN<Triangle3, 3> TriBvh;  // kd-tree (Method::AUTO with two children per node), default leaf size and depth
typedef BvhN<Vector3 const *, 3> PointBvh;  // PointSet3 keeps pointers to its samples as BVH elements

struct MeshRef {
  std::vector<Triangle3> tris;
  TriBvh * bvh = nullptr;
};

struct PointsRef {
  std::vector<Vector3> pts;
  std::vector<Vector3 const *> ptrs;
  PointBvh * bvh = nullptr;
};

Vector3 v3(float const * p, int64_t i) { return Vector3(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }

// PointSet3::FilterSelf (Algorithms/PointSet3.hpp:576-583): every element but one
struct FilterSelf : public Filter<Vector3 const *> {
  Vector3 const * self = nullptr;
  bool allows(Vector3 const * const & s) const { return s != self; }
};

template <size_t K>
int64_t knn_one(PointsRef const & r, Vector3 const & q, int64_t self, double bound, int32_t * idx, double * mad) {
  BoundedSortedArrayN<K, PointBvh::NeighborPair> set;
  FilterSelf filt;
  if (self >= 0) {
    filt.self = r.ptrs[(size_t)self];
    r.bvh->pushFilter(&filt);
  }
  r.bvh->kClosestPairs<MetricL2>(q, set, bound);
  if (self >= 0) r.bvh->popFilter();
  for (size_t j = 0; j < K; ++j) {
    idx[j] = j < set.size() ? (int32_t)set[j].getTargetIndex() : -1;
    mad[j] = j < set.size() ? set[j].getMonotoneApproxDistance() : -1.0;
  }
  return (int64_t)set.size();
}

template <size_t K> struct KnnDispatch {
  static void run(int k, PointsRef const & r, Vector3 const & q, int64_t self, double bound, int32_t * idx,
                  double * mad) {
    if (k == (int)K) knn_one<K>(r, q, self, bound, idx, mad);
    else KnnDispatch<K - 1>::run(k, r, q, self, bound, idx, mad);
  }
};
template <> struct KnnDispatch<0> {
  static void run(int, PointsRef const &, Vector3 const &, int64_t, double, int32_t *, double *) {}
};

}  // namespace

extern "C" {

int ref_version() { return 1; }

// MeshBvh over the triangles F of V: element i is triangle i (MeshBvh::add + init, Algorithms/MeshBvh.hpp:55-111)
void * ref_mesh_create(float const * V, int64_t nv, int32_t const * F, int64_t nf) {
  (void)nv;
  MeshRef * m = new MeshRef;
  m->tris.reserve((size_t)nf);
  for (int64_t f = 0; f < nf; ++f) m->tris.emplace_back(v3(V, F[3 * f]), v3(V, F[3 * f + 1]), v3(V, F[3 * f + 2]));
  m->bvh = new TriBvh(m->tris.begin(), m->tris.end());
  return m;
}

void ref_mesh_destroy(void * h) {
  MeshRef * m = static_cast<MeshRef *>(h);
  delete m->bvh;
  delete m;
}

// BvhN::closestElement<MetricL2>(q, dist_bound, {}, &dist, &closest_point) (Algorithms/BvhN.hpp:1050-1063)
void ref_closest(void * h, float const * q, int64_t n, double dist_bound, int32_t * idx, double * dist, float * cp) {
  MeshRef * m = static_cast<MeshRef *>(h);
  for (int64_t i = 0; i < n; ++i) {
    double d = -1;
    Vector3 c(0, 0, 0);
    intx e = m->bvh->closestElement<MetricL2>(v3(q, i), dist_bound, UniversalCompatibility(), &d, &c);
    idx[i] = (int32_t)e;
    dist[i] = e >= 0 ? d : -1.0;
    cp[3 * i] = c[0]; cp[3 * i + 1] = c[1]; cp[3 * i + 2] = c[2];
  }
}

// BvhN::rayStructureIntersection<RayIntersectionTester>(ray, max_time) (Algorithms/BvhN.hpp:1292-1316)
void ref_ray(void * h, float const * o, float const * d, int64_t n, float max_time, float * t, int32_t * idx,
             float * normal) {
  MeshRef * m = static_cast<MeshRef *>(h);
  for (int64_t i = 0; i < n; ++i) {
    RayN<3, Real> ray(v3(o, i), v3(d, i));
    RayStructureIntersectionN<3, Real> r = m->bvh->rayStructureIntersection<RayIntersectionTester>(ray, max_time);
    t[i] = r.getTime();
    idx[i] = (int32_t)r.getElementIndex();
    Vector3 nn = r.hasNormal() ? r.getNormal() : Vector3(0, 0, 0);
    normal[3 * i] = nn[0]; normal[3 * i + 1] = nn[1]; normal[3 * i + 2] = nn[2];
  }
}

// BvhN::closestPair<MetricL2> with another mesh BVH as the query (Algorithms/BvhN.hpp:1082-1114, 1916-2089)
int32_t ref_mesh_pair(void * target, void * query, double dist_bound, int32_t * qi, int32_t * ti, double * mad,
                      float * qpt, float * tpt) {
  MeshRef * t = static_cast<MeshRef *>(target);
  MeshRef * q = static_cast<MeshRef *>(query);
  TriBvh::NeighborPair p = t->bvh->closestPair<MetricL2>(*q->bvh, dist_bound, UniversalCompatibility(), true);
  *qi = (int32_t)p.getQueryIndex();
  *ti = (int32_t)p.getTargetIndex();
  *mad = p.getMonotoneApproxDistance();
  for (int k = 0; k < 3; ++k) {
    qpt[k] = p.getQueryPoint()[k];
    tpt[k] = p.getTargetPoint()[k];
  }
  return p.isValid() ? 1 : 0;
}

void * ref_points_create(float const * P, int64_t n) {
  PointsRef * r = new PointsRef;
  r->pts.reserve((size_t)n);
  for (int64_t i = 0; i < n; ++i) r->pts.push_back(v3(P, i));
  for (auto const & p : r->pts) r->ptrs.push_back(&p);
  r->bvh = new PointBvh(r->ptrs.begin(), r->ptrs.end());
  return r;
}

void ref_points_destroy(void * h) {
  PointsRef * r = static_cast<PointsRef *>(h);
  delete r->bvh;
  delete r;
}

// BvhN::kClosestPairs<MetricL2>(q, BoundedSortedArrayN<k, NeighborPair>, dist_bound) with PointSet3's self filter when
// exclude[i] >= 0 (Algorithms/BvhN.hpp:1139-1146; PointSet3.hpp:576-583). k in 1..32; mad = squared distances.
void ref_knn(void * h, float const * q, int64_t n, int k, double dist_bound, int32_t const * exclude, int32_t * idx,
             double * mad) {
  PointsRef * r = static_cast<PointsRef *>(h);
  for (int64_t i = 0; i < n; ++i)
    KnnDispatch<32>::run(k, *r, v3(q, i), exclude ? exclude[i] : -1, dist_bound, idx + i * k, mad + i * k);
}

// TriangleN<3>::closestPoint (Triangle3.hpp:294-304), one triangle (9 floats) and one point per row
void ref_triangle_closest_points(float const * tris, float const * p, int64_t n, float * cp) {
  for (int64_t i = 0; i < n; ++i) {
    Triangle3 t(v3(tris, 3 * i), v3(tris, 3 * i + 1), v3(tris, 3 * i + 2));
    Vector3 c = t.closestPoint(v3(p, i));
    cp[3 * i] = c[0]; cp[3 * i + 1] = c[1]; cp[3 * i + 2] = c[2];
  }
}

// TriangleN<3>::squaredDistance(triangle, this_pt, other_pt) (Triangle3.hpp:314-400), a_i as "this"
void ref_triangle_pair_distances(float const * a, float const * b, int64_t n, float * d2, float * pa, float * pb) {
  for (int64_t i = 0; i < n; ++i) {
    Triangle3 ta(v3(a, 3 * i), v3(a, 3 * i + 1), v3(a, 3 * i + 2));
    Triangle3 tb(v3(b, 3 * i), v3(b, 3 * i + 1), v3(b, 3 * i + 2));
    Vector3 x, y;
    d2[i] = ta.squaredDistance(tb, &x, &y);
    for (int k = 0; k < 3; ++k) {
      pa[3 * i + k] = x[k];
      pb[3 * i + k] = y[k];
    }
  }
}

// TriangleN<3>::rayIntersectionTime (Triangle3.hpp:536-552), one triangle and one ray per row
void ref_triangle_ray_times(float const * tris, float const * o, float const * d, int64_t n, float max_time,
                            float * t) {
  for (int64_t i = 0; i < n; ++i) {
    Triangle3 tri(v3(tris, 3 * i), v3(tris, 3 * i + 1), v3(tris, 3 * i + 2));
    t[i] = tri.rayIntersectionTime(RayN<3, Real>(v3(o, i), v3(d, i)), max_time);
  }
}

// Random(seed).bits() repeated (Random.cpp:49-97)
void ref_random_bits(uint32_t seed, int64_t n, uint32_t * out) {
  Random r(seed, false);
  for (int64_t i = 0; i < n; ++i) out[i] = r.bits();
}

// Math::treeDepth (Math.cpp:23-36)
int64_t ref_tree_depth(int64_t n, int max_leaf) { return Math::treeDepth(n, max_leaf, 0.5f); }

// BestFitSphereN<3> (the reference's miniball) over n points: centre and radius as the reference returns them (Real)
void ref_best_fit_sphere(float const * P, int64_t n, float * center, float * radius) {
  BestFitSphereN<3> s;
  for (int64_t i = 0; i < n; ++i) s.addPoint(v3(P, i));
  Vector3 const & c = s.getCenter();
  center[0] = c[0];
  center[1] = c[1];
  center[2] = c[2];
  *radius = s.getRadius();
}

}  // extern "C"
