// Smallest enclosing ball (BestFitSphereN, Algorithms/BestFitSphereN.hpp:62-91) by pivoting: keep the support set of
// the current ball (at most four points), find the point farthest from its centre on the GPU (one pass over the points,
// a tree reduction per block), and if that point lies outside, replace the ball by the smallest ball of support + point
// (a host step over at most five points). The radius grows at every step, so the loop ends; at the end every point lies
// in the ball and the ball is the smallest ball of its own support, hence of all the points. Distances are computed in
// double from the float coordinates, as the reference casts its points to double before its miniball runs.
#include "bounding_sphere.hpp"

#include "device_util.cuh"

#include <cmath>
#include <vector>

namespace thea {
namespace {

constexpr int SPHERE_THREADS = 256;
constexpr int SPHERE_MAX_STEPS = 4096;
// relative slack of the inside test: points within this of the boundary count as inside (the rounding of a centre and
// radius computed from float coordinates in double)
constexpr double SPHERE_REL_TOL = 1e-13;

struct Farthest {
  double d2;    // squared distance to the centre, -1 when the block saw no finite point
  long long i;  // its index (lowest among equal distances)
  float x, y, z, pad;
};

__device__ __forceinline__ void take(double & d, long long & i, float & x, float & y, float & z, double d2, long long j,
                                     float px, float py, float pz) {
  if (d2 > d || (d2 == d && j < i)) d = d2, i = j, x = px, y = py, z = pz;
}

__global__ void __launch_bounds__(SPHERE_THREADS)
farthest_kernel(float const * __restrict__ pts, int64_t n, double cx, double cy, double cz, Farthest * __restrict__ out) {
  double d = -1.0;
  long long i = -1;
  float x = 0.f, y = 0.f, z = 0.f;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
    float px = pts[3 * j], py = pts[3 * j + 1], pz = pts[3 * j + 2];
    if (!(isfinite(px) && isfinite(py) && isfinite(pz))) continue;
    double dx = (double)px - cx, dy = (double)py - cy, dz = (double)pz - cz;
    take(d, i, x, y, z, dx * dx + dy * dy + dz * dz, j, px, py, pz);
  }
  for (int o = 16; o; o >>= 1) {
    double od = __shfl_xor_sync(0xffffffffu, d, o);
    long long oi = __shfl_xor_sync(0xffffffffu, i, o);
    float ox = __shfl_xor_sync(0xffffffffu, x, o), oy = __shfl_xor_sync(0xffffffffu, y, o);
    float oz = __shfl_xor_sync(0xffffffffu, z, o);
    if (oi >= 0) take(d, i, x, y, z, od, oi, ox, oy, oz);
  }
  __shared__ Farthest s[SPHERE_THREADS / 32];
  int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) s[w] = Farthest{d, i, x, y, z, 0.f};
  __syncthreads();
  if (threadIdx.x == 0) {
    Farthest b = s[0];
    for (int k = 1; k < SPHERE_THREADS / 32; ++k)
      if (s[k].i >= 0) take(b.d2, b.i, b.x, b.y, b.z, s[k].d2, s[k].i, s[k].x, s[k].y, s[k].z);
    out[blockIdx.x] = b;
  }
}

double dist2(double const * a, double const * b) {
  double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
  return dx * dx + dy * dy + dz * dz;
}

// The ball through the m points of `sub` (1 <= m <= 4) whose centre lies in their affine hull; false if they are
// affinely dependent (no such ball, or not a unique one).
bool circumball(double const (*sub)[3], int m, double * c, double & r2) {
  double const * p0 = sub[0];
  if (m == 1) {
    c[0] = p0[0], c[1] = p0[1], c[2] = p0[2];
    r2 = 0.0;
    return true;
  }
  // c = p0 + sum_j lambda_j v_j with 2 v_i . (c - p0) = |v_i|^2 for every i: a (m-1) x (m-1) Gram system
  int k = m - 1;
  double v[3][3], A[3][4];
  double scale = 0.0;
  for (int j = 0; j < k; ++j)
    for (int t = 0; t < 3; ++t) v[j][t] = sub[j + 1][t] - p0[t];
  for (int a = 0; a < k; ++a) {
    for (int b = 0; b < k; ++b) {
      A[a][b] = 2.0 * (v[a][0] * v[b][0] + v[a][1] * v[b][1] + v[a][2] * v[b][2]);
      scale = std::fmax(scale, std::fabs(A[a][b]));
    }
    A[a][k] = v[a][0] * v[a][0] + v[a][1] * v[a][1] + v[a][2] * v[a][2];
  }
  if (!(scale > 0.0)) return false;
  for (int col = 0; col < k; ++col) {  // Gaussian elimination with partial pivoting
    int piv = col;
    for (int row = col + 1; row < k; ++row)
      if (std::fabs(A[row][col]) > std::fabs(A[piv][col])) piv = row;
    if (std::fabs(A[piv][col]) <= 1e-12 * scale) return false;
    if (piv != col)
      for (int t = 0; t <= k; ++t) std::swap(A[piv][t], A[col][t]);
    for (int row = 0; row < k; ++row) {
      if (row == col) continue;
      double f = A[row][col] / A[col][col];
      for (int t = col; t <= k; ++t) A[row][t] -= f * A[col][t];
    }
  }
  for (int t = 0; t < 3; ++t) {
    c[t] = p0[t];
    for (int j = 0; j < k; ++j) c[t] += (A[j][k] / A[j][j]) * v[j][t];
  }
  r2 = 0.0;
  for (int j = 0; j < m; ++j) r2 = std::fmax(r2, dist2(sub[j], c));
  return true;
}

bool inside(double const * p, double const * c, double r2) {
  return dist2(p, c) <= r2 * (1.0 + 2.0 * SPHERE_REL_TOL) + 1e-300;
}

}  // namespace

int smallest_ball_of_few(double const * pts, int k, double * center, double * radius) {
  // every subset of at most four points: the smallest of their circumballs that holds all k points
  double best_r2 = INFINITY;
  int best_m = 0;
  for (int mask = 1; mask < (1 << k); ++mask) {
    int m = __builtin_popcount((unsigned)mask);
    if (m > 4) continue;
    double sub[4][3];
    int j = 0;
    for (int t = 0; t < k; ++t)
      if (mask & (1 << t)) {
        sub[j][0] = pts[3 * t], sub[j][1] = pts[3 * t + 1], sub[j][2] = pts[3 * t + 2];
        ++j;
      }
    double c[3], r2;
    if (!circumball(sub, m, c, r2) || !(r2 < best_r2)) continue;
    bool all = true;
    for (int t = 0; t < k && all; ++t) all = inside(pts + 3 * t, c, r2);
    if (!all) continue;
    best_r2 = r2;
    best_m = mask;
    center[0] = c[0], center[1] = c[1], center[2] = c[2];
  }
  if (!best_m) return 0;
  *radius = std::sqrt(best_r2);
  return best_m;
}

void run_bounding_sphere(float const * points, int64_t n, double * center, double * radius, cudaStream_t s) {
  center[0] = center[1] = center[2] = 0.0;
  *radius = 0.0;
  if (n <= 0) return;
  int blocks = (int)std::min<int64_t>(ceil_div(n, SPHERE_THREADS), 2 * (int64_t)sm_count());
  Scratch dev((size_t)blocks * sizeof(Farthest), s);
  std::vector<Farthest> host((size_t)blocks);
  auto farthest = [&](double const * c) {
    THEA_LAUNCH(farthest_kernel, blocks, SPHERE_THREADS, 0, s, points, n, c[0], c[1], c[2], dev.as<Farthest>());
    THEA_CUDA_CHECK(cudaMemcpyAsync(host.data(), dev.ptr, (size_t)blocks * sizeof(Farthest), cudaMemcpyDeviceToHost, s));
    THEA_CUDA_CHECK(cudaStreamSynchronize(s));
    Farthest b = host[0];
    for (int k = 1; k < blocks; ++k)
      if (host[k].i >= 0 && (b.i < 0 || host[k].d2 > b.d2 || (host[k].d2 == b.d2 && host[k].i < b.i))) b = host[k];
    return b;
  };
  double c[3] = {0.0, 0.0, 0.0};
  Farthest f = farthest(c);
  if (f.i < 0) return;  // no finite point
  // support points (double copies of float coordinates), at most four
  double sup[5][3];
  int ns = 1;
  sup[0][0] = f.x, sup[0][1] = f.y, sup[0][2] = f.z;
  c[0] = f.x, c[1] = f.y, c[2] = f.z;
  double r = 0.0;
  for (int step = 0; step < SPHERE_MAX_STEPS; ++step) {
    f = farthest(c);
    double p[3] = {f.x, f.y, f.z};
    if (inside(p, c, r * r)) {
      center[0] = c[0], center[1] = c[1], center[2] = c[2];
      *radius = r;
      return;
    }
    sup[ns][0] = p[0], sup[ns][1] = p[1], sup[ns][2] = p[2];
    double flat[15], nc[3], nr = 0.0;
    for (int j = 0; j <= ns; ++j)
      for (int t = 0; t < 3; ++t) flat[3 * j + t] = sup[j][t];
    int mask = smallest_ball_of_few(flat, ns + 1, nc, &nr);
    if (!mask || !(nr > r)) {
      // rounding: the point lies outside by a few ulps of the radius and no ball of the support set plus the point is
      // larger; grow the current ball just enough to hold it
      center[0] = c[0], center[1] = c[1], center[2] = c[2];
      *radius = std::sqrt(dist2(p, c));
      return;
    }
    int m = 0;
    for (int j = 0; j <= ns; ++j)
      if (mask & (1 << j)) {
        for (int t = 0; t < 3; ++t) sup[m][t] = flat[3 * j + t];
        ++m;
      }
    ns = m;
    c[0] = nc[0], c[1] = nc[1], c[2] = nc[2];
    r = nr;
  }
  throw Error(THEA_ERR_INTERNAL, "bounding sphere: no convergence");
}

}  // namespace thea
