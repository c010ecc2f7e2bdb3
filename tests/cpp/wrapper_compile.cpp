// Compiles the C++ wrapper against the library. With --no-device it only checks error reporting (no CUDA calls);
// otherwise it runs one closest-point, ray and k-NN query on a tetrahedron and checks the answers.
#include "thea_gpu.hpp"

#include <cmath>
#include <cstdio>
#include <cstring>

int main(int argc, char ** argv) {
  bool no_device = argc > 1 && std::strcmp(argv[1], "--no-device") == 0;
  if (thea_abi_version() != THEA_GPU_ABI_VERSION) return 1;
  try {
    thea_gpu::MeshBvh bad(nullptr, 0, nullptr, 0);
    return 2;  // must have thrown
  } catch (thea_gpu::Exception const & e) {
    if (e.status() != THEA_ERR_INVALID_ARGUMENT) return 3;
  }
  // the serving wrapper on the test executor (no CUDA call): admission, submit, wait, stats
  {
    thea_server_config cfg{};
    cfg.test_executor = 1;
    cfg.test_ns_per_query = 100;
    thea_gpu::Server server(cfg);
    float sv[] = {0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1};
    int32_t sf[] = {0, 1, 2, 0, 1, 3, 0, 2, 3, 1, 2, 3};
    int32_t mesh = server.addMesh(sv, 4, sf, 4);
    float q[30] = {0};
    int32_t idx[80];
    float val[80];
    thea_request r{};
    r.type = THEA_REQUEST_KNN;
    r.mesh = mesh;
    r.num_queries = 10;
    r.queries = q;
    r.k = 8;
    r.out_index = idx;
    r.out_value = val;
    uint64_t t = server.submit(r);
    thea_status st = THEA_ERR_INTERNAL;
    double ms = -1;
    if (!server.wait(t, &st, &ms) || st != THEA_OK || ms < 0) return 7;
    thea_server_stats s = server.stats();
    if (s.completed != 1 || s.queries_completed != 10 || s.resident_meshes != 1) return 8;
    try {
      server.submit(thea_request{});
      return 9;  // must have thrown
    } catch (thea_gpu::Exception const & e) {
      if (e.status() != THEA_ERR_INVALID_ARGUMENT) return 10;
    }
  }
  // a foreign image is refused before any CUDA call
  try {
    unsigned char junk[256] = {0};
    thea_gpu::MeshBvh::fromImage(junk, sizeof(junk));
    return 11;  // must have thrown
  } catch (thea_gpu::Exception const & e) {
    if (e.status() != THEA_ERR_INVALID_ARGUMENT) return 12;
  }
  // a quad in an OFF file becomes two triangles of face 0 (host code only)
  {
    std::string path = std::string(argv[0]) + ".off";
    FILE * f = std::fopen(path.c_str(), "w");
    if (!f) return 14;
    std::fputs("OFF\n4 1 0\n0 0 0\n1 0 0\n1 1 0\n0 1 0\n4 0 1 2 3\n", f);
    std::fclose(f);
    thea_gpu::MeshFile mf(path);
    std::remove(path.c_str());
    int32_t const want[6] = {0, 1, 2, 2, 3, 0};
    if (mf.numVertices() != 4 || mf.numTriangles() != 2 || mf.num_faces != 1) return 15;
    if (std::memcmp(mf.triangles.data(), want, sizeof(want)) != 0 || mf.triangle_face[1] != 0) return 16;
    try {
      thea_gpu::MeshFile missing(path);
      return 17;  // must have thrown
    } catch (thea_gpu::Exception const & e) {
      if (e.status() != THEA_ERR_INVALID_ARGUMENT) return 18;
    }
  }
  // an unreadable mesh file is reported before any CUDA call
  {
    try {
      thea_gpu::MeshFile mf2(std::string(argv[0]) + ".missing.ply");
      return 19;
    } catch (thea_gpu::Exception const & e) {
      if (e.status() != THEA_ERR_INVALID_ARGUMENT) return 20;
    }
  }
  if (no_device) return 0;

  float V[] = {0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1};
  int32_t F[] = {0, 1, 2, 0, 1, 3, 0, 2, 3, 1, 2, 3};
  thea_gpu::MeshBvh mesh(V, 4, F, 4);
  float q[3] = {0.25f, 0.25f, -1.0f};
  double dist = -1;
  float cp[3];
  int64_t idx = mesh.closestElement(q, -1, &dist, cp);
  if (idx != 0 || std::fabs(dist - 1.0) > 1e-6 || cp[2] != 0.0f) { std::printf("closest %lld %f\n", (long long)idx, dist); return 4; }
  float o[3] = {0.2f, 0.2f, 2.0f}, d[3] = {0, 0, -1}, t = 0;
  int32_t ti = -1;
  mesh.rayStructureIntersection(o, d, 1, &t, &ti);
  if (ti != 3) { std::printf("ray %d %f\n", ti, t); return 5; }
  // the reloaded image answers like the original
  std::vector<unsigned char> image = mesh.serialize();
  thea_gpu::MeshBvh again = thea_gpu::MeshBvh::fromImage(image.data(), (int64_t)image.size());
  double dist2 = -1;
  if (again.closestElement(q, -1, &dist2, cp) != idx || dist2 != dist) return 13;
  thea_gpu::PointBvh pts(V, 4);
  int32_t ki[2];
  float kd[2];
  pts.kClosestPairs(q, 1, 2, ki, kd);
  if (ki[0] != 0 || ki[1] != 1) { std::printf("knn %d %d\n", ki[0], ki[1]); return 6; }
  // the closest pair between the tetrahedron's vertices and its faces is at distance 0; the nearest triangles of q
  int32_t pq = -1, pt = -1;
  float pd = -1;
  if (!mesh.closestPair(pts, &pq, &pt, &pd) || pd != 0.0f) return 21;
  int32_t mi[2];
  float md[2];
  mesh.kClosestPairs(q, 1, 2, mi, md);
  if (mi[0] != 0 || md[0] != 1.0f) { std::printf("mesh knn %d %f\n", mi[0], md[0]); return 22; }
  double sdf[1];
  float inside[3] = {0.1f, 0.1f, 0.0f}, up[3] = {0, 0, -1};
  mesh.shapeDiameter(inside, up, 1, sdf);
  if (!(sdf[0] > 0.0 && sdf[0] <= 1.0)) { std::printf("sdf %f\n", sdf[0]); return 23; }
  // the tetrahedron's smallest enclosing ball is the circle of its face x + y + z = 1 (the circumsphere's centre lies
  // outside the tetrahedron): centre (1/3, 1/3, 1/3), radius sqrt(2/3); the origin lies inside
  thea_gpu::BestFitSphere3 sphere;
  sphere.addPoints(V, 4);
  float c[3];
  sphere.getCenter(c);
  if (std::fabs(sphere.getRadius() - 0.81649658f) > 1e-6f || std::fabs(c[0] - 0.33333333f) > 1e-6f) {
    std::printf("sphere %f\n", sphere.getRadius());
    return 24;
  }
  // a ring of eight samples: each one's two nearest are its ring neighbours
  float ring[24];
  for (int i = 0; i < 8; ++i) {
    ring[3 * i] = std::cos(0.785398163f * i);
    ring[3 * i + 1] = std::sin(0.785398163f * i);
    ring[3 * i + 2] = 0.f;
  }
  thea_gpu::PointSet3 ps(2, 1);
  ps.setSamples(ring, nullptr, 8);
  int32_t const * nb = ps.neighbors(0);
  if (ps.numNeighbors(0) != 2 || nb[0] + nb[1] != 8 || (nb[0] != 1 && nb[0] != 7)) return 25;
  std::printf("wrapper ok\n");
  return 0;
}
