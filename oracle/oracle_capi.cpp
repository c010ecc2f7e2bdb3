// TEST INFRASTRUCTURE ONLY -- C entry points of the CPU oracle, loaded by the tests (ctypes) and by the CPU-baseline legs
// of bench.py. Never linked into the product library. Parity status: pinned to the reference (see thea_oracle.hpp).

#include "thea_oracle.hpp"

#include <random>

using namespace oracle;

namespace {

struct MeshHandle {
  int fp64 = 0;
  MeshIndex<float> f;
  MeshIndex<double> d;
};

struct PointHandle {
  int fp64 = 0;
  PointIndex<float> f;
  PointIndex<double> d;
};

template <class S> V3<S> q3(float const * p, int64_t i) { return load3<S>(p + 3 * i); }

}  // namespace

extern "C" {

int oracle_version() { return 1; }

//---------------------------------------------------------------------------------------------------------------------------
// Mesh index (kd-tree over triangles, MeshBvh::init -> BvhN::init, MeshBvh.hpp:104-111)
//---------------------------------------------------------------------------------------------------------------------------

void * oracle_mesh_create(float const * V, int64_t nv, int32_t const * F, int64_t nf, int64_t max_leaf, int fp64) {
  MeshHandle * h = new MeshHandle;
  h->fp64 = fp64;
  if (fp64) h->d.init(V, nv, F, nf, max_leaf);
  else h->f.init(V, nv, F, nf, max_leaf);
  return h;
}

void oracle_mesh_destroy(void * h) { delete static_cast<MeshHandle *>(h); }

int64_t oracle_mesh_num_nodes(void * hv) {
  MeshHandle * h = static_cast<MeshHandle *>(hv);
  return h->fp64 ? (int64_t)h->d.tree.nodes.size() : (int64_t)h->f.tree.nodes.size();
}

int64_t oracle_mesh_max_depth(void * hv) {
  MeshHandle * h = static_cast<MeshHandle *>(hv);
  return h->fp64 ? h->d.tree.max_depth : h->f.tree.max_depth;
}

// Reference-mode closest element (FP32 handle only). dist is sqrt(mad) in double, as BvhN::closestElement returns it.
void oracle_closest_ref(void * hv, float const * q, int64_t n, double dist_bound, int32_t * idx, double * dist,
                        float * cp, int nthreads) {
  MeshHandle * h = static_cast<MeshHandle *>(hv);
  parallelFor(n, nthreads, [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) {
      double mad = -1;
      V3<float> c;
      int64_t r = h->f.closestRef(q3<float>(q, i), dist_bound, mad, c);
      idx[i] = (int32_t)r;
      if (dist) dist[i] = r >= 0 ? std::sqrt(mad) : -1.0;
      if (cp) {
        cp[3 * i] = r >= 0 ? c.x : 0.f; cp[3 * i + 1] = r >= 0 ? c.y : 0.f; cp[3 * i + 2] = r >= 0 ? c.z : 0.f;
      }
    }
  });
}

extern "C++" {
template <class S>
static void closestContractImpl(MeshIndex<S> const & m, float const * q, int64_t n, double dist_bound, int32_t * idx,
                                double * d2, double * cp, int nthreads) {
  parallelFor(n, nthreads, [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) {
      S bd2 = 0;
      V3<S> c;
      int64_t r = m.closestContract(q3<S>(q, i), dist_bound, bd2, c);
      idx[i] = (int32_t)r;
      if (d2) d2[i] = r >= 0 ? (double)bd2 : -1.0;
      if (cp) { cp[3 * i] = (double)c.x; cp[3 * i + 1] = (double)c.y; cp[3 * i + 2] = (double)c.z; }
    }
  });
}
}  // extern "C++"

// Contract-mode closest element: lowest index among equal squared distances.
void oracle_closest_contract(void * hv, float const * q, int64_t n, double dist_bound, int32_t * idx, double * d2,
                             double * cp, int nthreads) {
  MeshHandle * h = static_cast<MeshHandle *>(hv);
  if (h->fp64) closestContractImpl(h->d, q, n, dist_bound, idx, d2, cp, nthreads);
  else closestContractImpl(h->f, q, n, dist_bound, idx, d2, cp, nthreads);
}

extern "C++" {
template <class S>
static void closestBruteImpl(float const * V, int64_t nv, int32_t const * F, int64_t nf, float const * q, int64_t n,
                             double dist_bound, int32_t * idx, double * d2, double * cp, int nthreads) {
  (void)nv;
  std::vector<Tri<S>> tris((size_t)nf);
  for (int64_t f = 0; f < nf; ++f)
    tris[(size_t)f] = Tri<S>(q3<S>(V, F[3 * f]), q3<S>(V, F[3 * f + 1]), q3<S>(V, F[3 * f + 2]));
  // the bound as a BVH over these triangles applies it (MeshIndex::closestBound): its root box is the element bounds
  // grown by 1.05 about their centre
  MeshIndex<S> root_only;
  root_only.tree.nodes.resize(1);
  for (auto const & t : tris) root_only.tree.nodes[0].bounds.merge(t.bounds());
  root_only.tree.nodes[0].bounds.scaleCentered(S(1.05f));
  parallelFor(n, nthreads, [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) {
      V3<S> p = q3<S>(q, i);
      int64_t best = -1;
      S bd = 0;
      V3<S> bc;
      Box<S> qb;
      qb.merge(p);
      double mb = nf > 0 ? root_only.closestBound(qb, dist_bound) : -1;
      for (int64_t f = 0; f < nf && mb != -2; ++f) {
        V3<S> c;
        S dd = triangleClosestPoints(tris[(size_t)f], p, c);
        if (!(dd == dd)) continue;  // a NaN distance (coincident vertices) is never selected
        if (mb >= 0 && !((double)dd < mb)) continue;
        if (best < 0 || dd < bd) { best = f; bd = dd; bc = c; }
      }
      idx[i] = (int32_t)best;
      if (d2) d2[i] = best >= 0 ? (double)bd : -1.0;
      if (cp) { cp[3 * i] = (double)bc.x; cp[3 * i + 1] = (double)bc.y; cp[3 * i + 2] = (double)bc.z; }
    }
  });
}
}  // extern "C++"

// Brute-force closest element over all triangles (contract mode by construction: scans in index order, strict less).
void oracle_closest_brute(float const * V, int64_t nv, int32_t const * F, int64_t nf, float const * q, int64_t n,
                          double dist_bound, int32_t * idx, double * d2, double * cp, int fp64, int nthreads) {
  if (fp64) closestBruteImpl<double>(V, nv, F, nf, q, n, dist_bound, idx, d2, cp, nthreads);
  else closestBruteImpl<float>(V, nv, F, nf, q, n, dist_bound, idx, d2, cp, nthreads);
}

// Reference-mode ray first hit (FP32 handle only): time (-1 = miss), element index, unit face normal.
void oracle_ray_ref(void * hv, float const * o, float const * d, int64_t n, float max_time, float * t, int32_t * idx,
                    float * normal, int nthreads) {
  MeshHandle * h = static_cast<MeshHandle *>(hv);
  parallelFor(n, nthreads, [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) {
      auto hit = h->f.rayRef(q3<float>(o, i), q3<float>(d, i), max_time);
      t[i] = hit.idx >= 0 ? hit.t : -1.f;
      idx[i] = (int32_t)hit.idx;
      if (normal) {
        V3<float> nn = hit.idx >= 0 ? h->f.tris[(size_t)hit.idx].normal : V3<float>(0, 0, 0);
        normal[3 * i] = nn.x; normal[3 * i + 1] = nn.y; normal[3 * i + 2] = nn.z;
      }
    }
  });
}

extern "C++" {
template <class S>
static void rayContractImpl(MeshIndex<S> const & m, float const * o, float const * d, int64_t n, double max_time,
                            double * t, int32_t * idx, int nthreads) {
  parallelFor(n, nthreads, [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) {
      auto hit = rayContract(m, q3<S>(o, i), q3<S>(d, i), (S)max_time);
      t[i] = hit.idx >= 0 ? (double)hit.t : -1.0;
      idx[i] = (int32_t)hit.idx;
    }
  });
}
}  // extern "C++"

void oracle_ray_contract(void * hv, float const * o, float const * d, int64_t n, double max_time, double * t,
                         int32_t * idx, int nthreads) {
  MeshHandle * h = static_cast<MeshHandle *>(hv);
  if (h->fp64) rayContractImpl(h->d, o, d, n, max_time, t, idx, nthreads);
  else rayContractImpl(h->f, o, d, n, max_time, t, idx, nthreads);
}

//---------------------------------------------------------------------------------------------------------------------------
// Closest pair between two meshes (BvhN::closestPair with a mesh BVH as the query, BvhN.hpp:1082-1114, 1916-2089; the
// pair distance is TriangleN::squaredDistance with the target triangle as "this", Triangle3.hpp:314-400). Contract
// mode: smallest squared distance, ties to the lowest query index, then the lowest target index. Outputs: query index,
// target index (-1 when no pair), squared distance, closest points on the query and target triangles (3 each).
//---------------------------------------------------------------------------------------------------------------------------

extern "C++" {
template <class S>
static std::vector<Tri<S>> makeTris(float const * V, int32_t const * F, int64_t nf) {
  std::vector<Tri<S>> t((size_t)nf);
  for (int64_t f = 0; f < nf; ++f) t[(size_t)f] = Tri<S>(q3<S>(V, F[3 * f]), q3<S>(V, F[3 * f + 1]), q3<S>(V, F[3 * f + 2]));
  return t;
}

// rows: per query triangle its best (d2, target); returns the winning (query, target) after the tie rule
template <class S>
static void pairReduce(std::vector<S> const & rd2, std::vector<int64_t> const & rt, std::vector<Tri<S>> const & qt,
                       std::vector<Tri<S>> const & tt, int32_t * qi, int32_t * ti, double * d2, double * qpt,
                       double * tpt) {
  int64_t bq = -1;
  for (size_t i = 0; i < rt.size(); ++i) {
    if (rt[i] < 0) continue;
    if (bq < 0 || rd2[i] < rd2[(size_t)bq]) bq = (int64_t)i;  // ascending scan: ties keep the lowest query, and each
  }                                                             // row already holds its lowest target among ties
  *qi = (int32_t)bq;
  *ti = bq >= 0 ? (int32_t)rt[(size_t)bq] : -1;
  *d2 = bq >= 0 ? (double)rd2[(size_t)bq] : -1.0;
  if (bq >= 0) {
    V3<S> pa, pb;
    triangleTriangleSquaredDistance(tt[(size_t)*ti], qt[(size_t)bq], pa, pb);
    for (int k = 0; k < 3; ++k) { qpt[k] = (double)pb[k]; tpt[k] = (double)pa[k]; }
  }
}

template <class S>
static void meshPairContractImpl(MeshIndex<S> const & m, float const * Vq, int32_t const * Fq, int64_t nfq,
                                 double dist_bound, int32_t * qi, int32_t * ti, double * d2, double * qpt, double * tpt,
                                 int nthreads) {
  std::vector<Tri<S>> qt = makeTris<S>(Vq, Fq, nfq);
  std::vector<S> rd2((size_t)nfq);
  std::vector<int64_t> rt((size_t)nfq);
  parallelFor(nfq, nthreads, [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) rt[(size_t)i] = m.closestTriangleContract(qt[(size_t)i], dist_bound, rd2[(size_t)i]);
  });
  pairReduce(rd2, rt, qt, m.tris, qi, ti, d2, qpt, tpt);
}

template <class S>
static void meshPairBruteImpl(float const * Vt, int32_t const * Ft, int64_t nft, float const * Vq, int32_t const * Fq,
                              int64_t nfq, double dist_bound, int32_t * qi, int32_t * ti, double * d2, double * qpt,
                              double * tpt, int nthreads) {
  std::vector<Tri<S>> tt = makeTris<S>(Vt, Ft, nft), qt = makeTris<S>(Vq, Fq, nfq);
  double mb = dist_bound >= 0 ? dist_bound * dist_bound : -1;
  std::vector<S> rd2((size_t)nfq);
  std::vector<int64_t> rt((size_t)nfq, -1);
  parallelFor(nfq, nthreads, [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) {
      for (int64_t j = 0; j < nft; ++j) {
        V3<S> pa, pb;
        S d = triangleTriangleSquaredDistance(tt[(size_t)j], qt[(size_t)i], pa, pb);
        if (!(d == d)) continue;
        if (mb >= 0 && !((double)d < mb)) continue;
        if (rt[(size_t)i] < 0 || d < rd2[(size_t)i]) { rd2[(size_t)i] = d; rt[(size_t)i] = j; }
      }
    }
  });
  pairReduce(rd2, rt, qt, tt, qi, ti, d2, qpt, tpt);
}
}  // extern "C++"

void oracle_mesh_pair_contract(void * target, float const * Vq, int32_t const * Fq, int64_t nfq, double dist_bound,
                               int32_t * qi, int32_t * ti, double * d2, double * qpt, double * tpt, int nthreads) {
  MeshHandle * h = static_cast<MeshHandle *>(target);
  if (h->fp64) meshPairContractImpl(h->d, Vq, Fq, nfq, dist_bound, qi, ti, d2, qpt, tpt, nthreads);
  else meshPairContractImpl(h->f, Vq, Fq, nfq, dist_bound, qi, ti, d2, qpt, tpt, nthreads);
}

void oracle_mesh_pair_brute(float const * Vt, int32_t const * Ft, int64_t nft, float const * Vq, int32_t const * Fq,
                            int64_t nfq, double dist_bound, int32_t * qi, int32_t * ti, double * d2, double * qpt,
                            double * tpt, int fp64, int nthreads) {
  if (fp64) meshPairBruteImpl<double>(Vt, Ft, nft, Vq, Fq, nfq, dist_bound, qi, ti, d2, qpt, tpt, nthreads);
  else meshPairBruteImpl<float>(Vt, Ft, nft, Vq, Fq, nfq, dist_bound, qi, ti, d2, qpt, tpt, nthreads);
}

// Squared distance and closest points of triangle pairs (a_i as "this", b_i as "other"), FP32: one per row of 9 floats.
void oracle_triangle_pair_distances(float const * a, float const * b, int64_t n, float * d2, float * pa, float * pb) {
  for (int64_t i = 0; i < n; ++i) {
    Tri<float> ta(q3<float>(a, 3 * i), q3<float>(a, 3 * i + 1), q3<float>(a, 3 * i + 2));
    Tri<float> tb(q3<float>(b, 3 * i), q3<float>(b, 3 * i + 1), q3<float>(b, 3 * i + 2));
    V3<float> x, y;
    d2[i] = triangleTriangleSquaredDistance(ta, tb, x, y);
    pa[3 * i] = x.x; pa[3 * i + 1] = x.y; pa[3 * i + 2] = x.z;
    pb[3 * i] = y.x; pb[3 * i + 1] = y.y; pb[3 * i + 2] = y.z;
  }
}

extern "C++" {
template <class S>
static void rayBruteImpl(float const * V, int64_t nv, int32_t const * F, int64_t nf, float const * o, float const * d,
                         int64_t n, double max_time, double * t, int32_t * idx, int nthreads) {
  (void)nv;
  std::vector<Tri<S>> tris((size_t)nf);
  for (int64_t f = 0; f < nf; ++f)
    tris[(size_t)f] = Tri<S>(q3<S>(V, F[3 * f]), q3<S>(V, F[3 * f + 1]), q3<S>(V, F[3 * f + 2]));
  parallelFor(n, nthreads, [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) {
      V3<S> oo = q3<S>(o, i), dd = q3<S>(d, i);
      int64_t best = -1;
      S bt = 0;
      for (int64_t f = 0; f < nf; ++f) {
        S tt = triangleRayTime(tris[(size_t)f], oo, dd, (S)max_time);
        if (tt < S(0)) continue;
        if (best < 0 || tt < bt) { best = f; bt = tt; }
      }
      t[i] = best >= 0 ? (double)bt : -1.0;
      idx[i] = (int32_t)best;
    }
  });
}
}  // extern "C++"

void oracle_ray_brute(float const * V, int64_t nv, int32_t const * F, int64_t nf, float const * o, float const * d,
                      int64_t n, double max_time, double * t, int32_t * idx, int fp64, int nthreads) {
  if (fp64) rayBruteImpl<double>(V, nv, F, nf, o, d, n, max_time, t, idx, nthreads);
  else rayBruteImpl<float>(V, nv, F, nf, o, d, n, max_time, t, idx, nthreads);
}

//---------------------------------------------------------------------------------------------------------------------------
// Point index and k nearest neighbours
//---------------------------------------------------------------------------------------------------------------------------

void * oracle_points_create(float const * P, int64_t n, int64_t max_leaf, int fp64) {
  PointHandle * h = new PointHandle;
  h->fp64 = fp64;
  if (fp64) h->d.init(P, n, max_leaf);
  else h->f.init(P, n, max_leaf);
  return h;
}

void oracle_points_destroy(void * h) { delete static_cast<PointHandle *>(h); }

// Reference-mode k nearest neighbours (FP32 handle only). Unused slots: index -1, d2 -1.
void oracle_knn_ref(void * hv, float const * q, int64_t n, int k, double dist_bound, int32_t const * exclude,
                    int32_t * idx, double * d2, int nthreads) {
  PointHandle * h = static_cast<PointHandle *>(hv);
  parallelFor(n, nthreads, [&](int64_t b, int64_t e) {
    std::vector<Neighbor> out;
    for (int64_t i = b; i < e; ++i) {
      h->f.knnRef(q3<float>(q, i), k, dist_bound, exclude ? (int64_t)exclude[i] : -1, out);
      for (int j = 0; j < k; ++j) {
        bool v = j < (int)out.size();
        idx[i * k + j] = v ? (int32_t)out[(size_t)j].idx : -1;
        d2[i * k + j] = v ? out[(size_t)j].mad : -1.0;
      }
    }
  });
}

extern "C++" {
template <class S>
static void knnContractImpl(PointIndex<S> const & m, float const * q, int64_t n, int k, double dist_bound,
                            int32_t const * exclude, int32_t * idx, double * d2, int nthreads) {
  parallelFor(n, nthreads, [&](int64_t b, int64_t e) {
    std::vector<std::pair<S, int64_t>> out;
    for (int64_t i = b; i < e; ++i) {
      m.knnContract(q3<S>(q, i), k, dist_bound, exclude ? (int64_t)exclude[i] : -1, out);
      for (int j = 0; j < k; ++j) {
        bool v = j < (int)out.size();
        idx[i * k + j] = v ? (int32_t)out[(size_t)j].second : -1;
        d2[i * k + j] = v ? (double)out[(size_t)j].first : -1.0;
      }
    }
  });
}
}  // extern "C++"

void oracle_knn_contract(void * hv, float const * q, int64_t n, int k, double dist_bound, int32_t const * exclude,
                         int32_t * idx, double * d2, int nthreads) {
  PointHandle * h = static_cast<PointHandle *>(hv);
  if (h->fp64) knnContractImpl(h->d, q, n, k, dist_bound, exclude, idx, d2, nthreads);
  else knnContractImpl(h->f, q, n, k, dist_bound, exclude, idx, d2, nthreads);
}

extern "C++" {
template <class S>
static void knnBruteImpl(float const * P, int64_t np, float const * q, int64_t n, int k, double dist_bound,
                         int32_t const * exclude, int32_t * idx, double * d2, int nthreads) {
  double mb = dist_bound >= 0 ? dist_bound * dist_bound : -1;
  parallelFor(n, nthreads, [&](int64_t b, int64_t e) {
    std::vector<std::pair<S, int64_t>> all;
    for (int64_t i = b; i < e; ++i) {
      V3<S> p = q3<S>(q, i);
      all.clear();
      for (int64_t j = 0; j < np; ++j) {
        if (exclude && exclude[i] == j) continue;
        S dd = squaredNorm(q3<S>(P, j) - p);
        if (mb >= 0 && !((double)dd < mb)) continue;
        all.emplace_back(dd, j);
      }
      size_t kk = std::min((size_t)k, all.size());
      std::partial_sort(all.begin(), all.begin() + (long)kk, all.end());
      for (int j = 0; j < k; ++j) {
        bool v = j < (int)kk;
        idx[i * k + j] = v ? (int32_t)all[(size_t)j].second : -1;
        d2[i * k + j] = v ? (double)all[(size_t)j].first : -1.0;
      }
    }
  });
}
}  // extern "C++"

// Points within a ball (BallN::contains, BallN.hpp:83: (p - center).squaredNorm() <= radius * radius in FP32), as
// used by BvhN::rangeQueryIndices (BvhN.hpp:1208-1219). Pass 1 (idx == nullptr): counts[i]. Pass 2: fills query i's
// neighbours in ascending index at offsets[i].
void oracle_range_brute(float const * P, int64_t np, float const * q, int64_t n, float radius, int32_t const * exclude,
                        int64_t * counts, int64_t const * offsets, int32_t * idx, float * d2, int nthreads) {
  float r2 = radius * radius;
  parallelFor(n, nthreads, [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) {
      V3<float> c = q3<float>(q, i);
      int64_t w = idx ? offsets[i] : 0, cnt = 0;
      for (int64_t j = 0; j < np; ++j) {
        if (exclude && exclude[i] == j) continue;
        float dd = squaredNorm(q3<float>(P, j) - c);
        if (dd <= r2) {
          if (idx) {
            idx[w + cnt] = (int32_t)j;
            d2[w + cnt] = dd;
          }
          ++cnt;
        }
      }
      if (!idx) counts[i] = cnt;
    }
  });
}

void oracle_knn_brute(float const * P, int64_t np, float const * q, int64_t n, int k, double dist_bound,
                      int32_t const * exclude, int32_t * idx, double * d2, int fp64, int nthreads) {
  if (fp64) knnBruteImpl<double>(P, np, q, n, k, dist_bound, exclude, idx, d2, nthreads);
  else knnBruteImpl<float>(P, np, q, n, k, dist_bound, exclude, idx, d2, nthreads);
}

//---------------------------------------------------------------------------------------------------------------------------
// Sampler and random numbers
//---------------------------------------------------------------------------------------------------------------------------

int64_t oracle_sample_by_area(float const * V, int64_t nv, int32_t const * F, int64_t nf, int64_t n, uint32_t seed,
                              float * pos, float * nrm, int32_t * face) {
  return sampleEvenlyByArea(V, nv, F, nf, n, seed, pos, nrm, face);
}

void oracle_thea_random_bits(uint32_t seed, int64_t n, uint32_t * out) {
  TheaRandom r(seed);
  for (int64_t i = 0; i < n; ++i) out[i] = r.bits();
}

// Independent known-answer source: the C++ standard library's MT19937 (same seeding and tempering as Thea's variant).
void oracle_std_mt19937_bits(uint32_t seed, int64_t n, uint32_t * out) {
  std::mt19937 g(seed);
  for (int64_t i = 0; i < n; ++i) out[i] = (uint32_t)g();
}

//---------------------------------------------------------------------------------------------------------------------------
// Single-primitive entry points (FP32), for unit parity of the device functions
//---------------------------------------------------------------------------------------------------------------------------

// tris: 9 floats per triangle; per item i: closest point, squared distance, and the 'inside' flag of the projection.
void oracle_triangle_closest_points(float const * tris, float const * p, int64_t n, float * cp, float * d2) {
  for (int64_t i = 0; i < n; ++i) {
    Tri<float> t(q3<float>(tris, 3 * i), q3<float>(tris, 3 * i + 1), q3<float>(tris, 3 * i + 2));
    V3<float> c;
    d2[i] = triangleClosestPoints(t, q3<float>(p, i), c);
    cp[3 * i] = c.x; cp[3 * i + 1] = c.y; cp[3 * i + 2] = c.z;
  }
}

void oracle_triangle_ray_times(float const * tris, float const * o, float const * d, int64_t n, float max_time,
                               float * t) {
  for (int64_t i = 0; i < n; ++i) {
    Tri<float> tr(q3<float>(tris, 3 * i), q3<float>(tris, 3 * i + 1), q3<float>(tris, 3 * i + 2));
    t[i] = triangleRayTime(tr, q3<float>(o, i), q3<float>(d, i), max_time);
  }
}

// Per triangle: unit normal (3), plane offset, primary axis, area
void oracle_triangle_props(float const * tris, int64_t n, float * normal, float * dist, int32_t * axis, float * area) {
  for (int64_t i = 0; i < n; ++i) {
    Tri<float> t(q3<float>(tris, 3 * i), q3<float>(tris, 3 * i + 1), q3<float>(tris, 3 * i + 2));
    normal[3 * i] = t.normal.x; normal[3 * i + 1] = t.normal.y; normal[3 * i + 2] = t.normal.z;
    dist[i] = t.dist; axis[i] = t.primary_axis; area[i] = t.area;
  }
}

float oracle_box_ray_time(float const * lo, float const * hi, float const * o, float const * d, float max_time) {
  Box<float> b;
  b.lo = q3<float>(lo, 0); b.hi = q3<float>(hi, 0); b.is_null = false;
  return boxRayIntersectionTime(b, q3<float>(o, 0), q3<float>(d, 0), max_time);
}

int64_t oracle_tree_depth(int64_t n, int max_leaf) { return treeDepth(n, max_leaf, 0.5f); }

// Random(seed).sphere() directions in stream order
void oracle_random_sphere(uint32_t seed, int64_t n, float * out) {
  TheaRandom r(seed);
  for (int64_t i = 0; i < n; ++i) {
    V3<float> u = theaSphere(r);
    out[3 * i] = u.x; out[3 * i + 1] = u.y; out[3 * i + 2] = u.z;
  }
}

// Visibility::compute for each position with Random(seed): point i draws directions [i * num_rays, (i + 1) * num_rays)
// xf (nullable): an affine transform set on the BVH (row-major 3x4)
// |extent| of getBounds(): the padded root box, or with a transform the box of its eight mapped corners
// (transformAndBound); fills inv with the transform's inverse when xf is given
static float boundsScale(MeshHandle const * h, float const * xf, float * inv) {
  Box<float> box = h->f.tree.nodes[0].bounds;
  if (xf) {
    affineInverse(xf, inv);
    Box<float> w;
    for (int c = 0; c < 8; ++c)
      w.merge(affinePoint(xf, V3<float>((c & 1) ? box.hi.x : box.lo.x, (c & 2) ? box.hi.y : box.lo.y,
                                        (c & 4) ? box.hi.z : box.lo.z)));
    box = w;
  }
  return norm(box.extent());
}

void oracle_visibility(void * hv, float const * positions, int64_t n, int64_t num_rays, uint32_t seed,
                       float const * xf, double * out, int nthreads) {
  MeshHandle * h = static_cast<MeshHandle *>(hv);
  if (num_rays <= 0) num_rays = 100;
  std::vector<V3<float>> dirs((size_t)(n * num_rays));
  TheaRandom r(seed);
  for (auto & u : dirs) u = theaSphere(r);
  float inv[12];
  float scale = boundsScale(h, xf, inv);
  parallelFor(n, nthreads, [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i)
      out[i] = visibilityFraction(h->f, q3<float>(positions, i), dirs.data() + i * num_rays, num_rays, scale,
                                  xf ? inv : nullptr);
  });
}

// Sample proximity graph with Random(seed); surface: nullable mesh handle. Outputs as thea_sample_graph.
// ShapeDiameter per point; normals == nullptr: the closest element's normal (contract mode, no transform); scale <= 0:
// |extent| of getBounds()
void oracle_shape_diameter(void * hv, float const * positions, float const * normals, int64_t n, float scale,
                           int only_interior, float const * xf, double * out, int nthreads) {
  MeshHandle * h = static_cast<MeshHandle *>(hv);
  float inv[12];
  float bs = boundsScale(h, xf, inv);
  if (!(scale > 0.f)) scale = bs;
  parallelFor(n, nthreads, [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) {
      V3<float> p = q3<float>(positions, i), nrm;
      if (normals) {
        nrm = q3<float>(normals, i);
      } else {
        float d2;
        V3<float> cp;
        int64_t k = h->f.closestContract(p, -1.0, d2, cp);
        if (k < 0) {
          out[i] = -1.0;
          continue;
        }
        nrm = h->f.tris[(size_t)k].normal;
      }
      out[i] = shapeDiameter(h->f, p, nrm, scale, only_interior != 0, xf ? inv : nullptr);
    }
  });
}

void oracle_sample_graph(float const * P, float const * N, int64_t n, int max_degree, uint32_t seed, void * surface,
                         int32_t * out_nbr, float * out_sep, int32_t * out_deg, float * out_avg, int nthreads) {
  std::vector<V3<float>> pts((size_t)n), nrm;
  for (int64_t i = 0; i < n; ++i) pts[(size_t)i] = q3<float>(P, i);
  if (N) {
    nrm.resize((size_t)n);
    for (int64_t i = 0; i < n; ++i) nrm[(size_t)i] = q3<float>(N, i);
  }
  TheaRandom r(seed);
  MeshIndex<float> const * m = surface ? &static_cast<MeshHandle *>(surface)->f : nullptr;
  SampleGraphResult g = sampleGraph(pts, N ? &nrm : nullptr, max_degree, r, m, nthreads);
  for (int64_t i = 0; i < n; ++i) {
    auto const & v = g.nbrs[(size_t)i];
    for (int k = 0; k < max_degree; ++k) {
      bool in = k < (int)v.size();
      out_nbr[i * max_degree + k] = in ? v[(size_t)k].second : -1;
      out_sep[i * max_degree + k] = in ? v[(size_t)k].first : 0.f;
    }
    out_deg[i] = (int32_t)v.size();
  }
  out_avg[0] = g.estimate;
  out_avg[1] = g.final_avg;
}

// Affine transforms (FP32): the inverse (returns 0 if singular), points through [L | t], vectors through L, normals
// through the inverse transpose (m then holds the inverse)
int oracle_affine_inverse(float const * m, float * inv) { return affineInverse(m, inv) ? 1 : 0; }
void oracle_affine_points(float const * m, float const * p, int64_t n, float * out) {
  for (int64_t i = 0; i < n; ++i) {
    V3<float> w = affinePoint(m, q3<float>(p, i));
    out[3 * i] = w.x; out[3 * i + 1] = w.y; out[3 * i + 2] = w.z;
  }
}
void oracle_affine_vectors(float const * m, float const * v, int64_t n, float * out) {
  for (int64_t i = 0; i < n; ++i) {
    V3<float> w = affineLinear(m, q3<float>(v, i));
    out[3 * i] = w.x; out[3 * i + 1] = w.y; out[3 * i + 2] = w.z;
  }
}
void oracle_normals_to_world(float const * inv, float const * nrm, int64_t n, float * out) {
  for (int64_t i = 0; i < n; ++i) {
    V3<float> w = normalToWorld(inv, q3<float>(nrm, i));
    out[3 * i] = w.x; out[3 * i + 1] = w.y; out[3 * i + 2] = w.z;
  }
}

}  // extern "C"
