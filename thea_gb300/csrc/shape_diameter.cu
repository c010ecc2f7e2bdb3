// ShapeDiameter (Algorithms/SurfaceFeatures/Local/ShapeDiameter.hpp:143-217) for many points, on the first-hit kernel.
//
// Per point the reference builds an orthonormal basis about the inward normal (Math::orthonormalBasis,
// MatrixUtil.hpp:241-249), casts 30 rays along a fixed cone of directions expressed in that basis, keeps the hit times
// of rays whose hit element's normal makes a non-negative dot product with the ray, selects the median with
// std::nth_element and averages the values within one standard deviation of it with cosine weights. Here: one thread
// per ray builds the 30n rays, the first-hit kernel casts them (normals included), and one thread per point reduces
// its 30 results in the reference's FP64 arithmetic. The reference permutes the hit times with std::nth_element but not
// the weights it pairs them with afterwards, so the selection reproduces libstdc++'s permutation (select_nth.cuh).
#include "shape_diameter.hpp"

#include "device_util.cuh"
#include "query.hpp"
#include "select_nth.cuh"
#include "transform.hpp"
#include "visibility.hpp"

namespace thea {
namespace {

constexpr int SDF_RAYS = 30;
constexpr int SDF_THREADS = 256;

// The reference's cone of ray directions in the local frame whose z axis is the inward normal (ShapeDiameter.hpp:163-193)
__constant__ float SDF_CONE[SDF_RAYS][3] = {
    {0.407497f, 0.134086f, 0.903309f},     {0.128722f, -0.822715f, 0.553688f},   {0.359298f, 0.686129f, 0.632560f},
    {0.813318f, -0.153956f, 0.561081f},    {-0.707169f, 0.296987f, 0.641647f},   {-0.478783f, -0.543441f, 0.689520f},
    {0.561083f, 0.523634f, 0.641087f},     {-0.380898f, -0.655789f, 0.651811f},  {0.722588f, 0.472155f, 0.504912f},
    {-0.535205f, 0.421235f, 0.732200f},    {0.577593f, -0.477896f, 0.661817f},   {0.393652f, -0.144484f, 0.907834f},
    {0.141508f, -0.660777f, 0.737122f},    {-0.274967f, -0.141703f, 0.950954f},  {-0.304935f, 0.474085f, 0.825989f},
    {0.711150f, 0.301383f, 0.635164f},     {-0.696119f, -0.112341f, 0.709082f},  {-0.248327f, 0.381035f, 0.890588f},
    {-0.0772394f, 0.0462501f, 0.995939f},  {0.438024f, 0.656463f, 0.614159f},    {-0.483384f, -0.542477f, 0.687065f},
    {0.498569f, -0.697466f, 0.514752f},    {-0.128902f, -0.0173429f, 0.991506f}, {0.338759f, -0.318772f, 0.885227f},
    {-0.574364f, -0.463887f, 0.674474f},   {-0.459207f, 0.260125f, 0.849390f},   {-0.628057f, -0.528928f, 0.570771f},
    {0.232916f, -0.328273f, 0.915416f},    {0.231667f, -0.796882f, 0.557951f},   {-0.270612f, -0.809654f, 0.520797f},
};

// leaf position of each element: the inverse of leaf_to_elem
__global__ void elem_position_kernel(int32_t const * __restrict__ leaf_to_elem, int64_t n, int32_t * __restrict__ pos) {
  int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p < n) pos[leaf_to_elem[p]] = (int32_t)p;
}

// Normal of each point's closest element: TriangleN::getNormal, normalized((v1 - v0) x (v2 - v0)), from the
// object-space ray record (v0, e01, e02). Points without an element keep a zero normal (their result is -1).
__global__ void closest_normal_kernel(float4 const * __restrict__ ray_rec, int32_t const * __restrict__ pos,
                                      int32_t const * __restrict__ idx, int64_t n, float * __restrict__ nrm) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  V3 out{0.f, 0.f, 0.f};
  int32_t e = idx[i];
  if (e >= 0) {
    float4 const * r = ray_rec + (size_t)pos[e] * RAY_REC_F4;
    out = normalized(cross(xyz(r[1]), xyz(r[2])));
  }
  nrm[3 * i] = out.x;
  nrm[3 * i + 1] = out.y;
  nrm[3 * i + 2] = out.z;
}

// Ray j of point i (index 30 i + j): origin position + 0.001 scale * in, direction rot * cone[j], where in is the
// inward unit normal and rot = [u v w] = Math::orthonormalBasis(in) (w = in normalised again, u =
// orthogonalDirection(in), v = w x u); the product rot * c evaluates row r as u_r c0 + (v_r c1 + w_r c2)
__global__ void sdf_rays_kernel(float const * __restrict__ P, float const * __restrict__ N, int64_t n, float off,
                                float * __restrict__ o, float * __restrict__ d) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n * SDF_RAYS) return;
  int64_t i = r / SDF_RAYS;
  int j = (int)(r - i * SDF_RAYS);
  V3 nn = normalized(load_v3(N + 3 * i));
  V3 in{-nn.x, -nn.y, -nn.z};
  V3 w = normalized(in);
  V3 u = max_abs_axis(in) == 0 ? normalized(V3{in.y, -in.x, 0.f}) : normalized(V3{0.f, in.z, -in.y});
  V3 v = cross(w, u);
  float c0 = SDF_CONE[j][0], c1 = SDF_CONE[j][1], c2 = SDF_CONE[j][2];
  V3 dir{u.x * c0 + (v.x * c1 + w.x * c2), u.y * c0 + (v.y * c1 + w.y * c2), u.z * c0 + (v.z * c1 + w.z * c2)};
  V3 p = load_v3(P + 3 * i);
  V3 org = p + off * in;  // Vector3 offset = 0.001f * scale * in; Ray3(position + offset, dir)
  o[3 * r] = org.x;
  o[3 * r + 1] = org.y;
  o[3 * r + 2] = org.z;
  d[3 * r] = dir.x;
  d[3 * r + 1] = dir.y;
  d[3 * r + 2] = dir.z;
}

// One thread per point: the reference's reduction of its kept hit times (ShapeDiameter.hpp:195-217), in FP64
__global__ void sdf_reduce_kernel(float const * __restrict__ t, float const * __restrict__ hit_nrm,
                                  float const * __restrict__ dirs, int32_t const * __restrict__ elem, int64_t n,
                                  double scale, int only_interior, double * __restrict__ out) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (elem && elem[i] < 0) {  // the point could not be mapped to the mesh
    out[i] = -1.0;
    return;
  }
  double values[SDF_RAYS], weights[SDF_RAYS];
  int num = 0;
  for (int j = 0; j < SDF_RAYS; ++j) {
    int64_t r = i * SDF_RAYS + j;
    float time = t[r];
    if (!(time >= 0.f)) continue;
    if (only_interior && !(dot(load_v3(hit_nrm + 3 * r), load_v3(dirs + 3 * r)) >= 0.f)) continue;
    values[num] = (double)time;
    weights[num] = (double)SDF_CONE[j][2];  // cos(angle) is the z component
    ++num;
  }
  if (num <= 0) {
    out[i] = -1.0;
    return;
  }
  int mid = num / 2;
  select_nth(values, num, mid);
  double sum_values = 0, sum_squares = 0;
  for (int k = 0; k < num; ++k) {
    sum_values += values[k];
    sum_squares += values[k] * values[k];
  }
  double avg = sum_values / num;
  double var = sum_squares / num - avg * avg;
  sum_values = 0;
  double sum_weights = 0;
  for (int k = 0; k < num; ++k) {
    double dv = values[k] - values[mid];
    if (dv * dv <= var) {
      sum_values += weights[k] * values[k];
      sum_weights += weights[k];
    }
  }
  double r = sum_weights > 0 ? sum_values / (sum_weights * scale) : values[mid] / scale;
  out[i] = r < 0.0 ? 0.0 : (r > 1.0 ? 1.0 : r);  // Math::clamp(r, 0, 1)
}

}  // namespace

void run_shape_diameter(thea_bvh const * b, float const * positions, float const * normals, int64_t n, float scale,
                        bool only_interior, double * out, cudaStream_t s) {
  if (n <= 0) return;
  if (!(scale > 0.f)) scale = visibility_scale(b);
  int64_t total = n * SDF_RAYS;
  unsigned blocks_pts = (unsigned)ceil_div(n, SDF_THREADS);
  Scratch nrm_buf, elem_buf, pos_buf;
  if (!normals) {
    // ShapeDiameter::compute(position): the normal of the closest element
    elem_buf = Scratch((size_t)n * 4, s);
    ClosestParams cp;
    thea_bvh const * tb = query_target(b);
    cp.scene_scale = scene_scale_of(tb);
    run_closest(tb, positions, n, cp, elem_buf.as<int32_t>(), nullptr, nullptr, nullptr, b->err, s);
    pos_buf = Scratch((size_t)b->n * 4, s);
    THEA_LAUNCH(elem_position_kernel, (unsigned)ceil_div(b->n, SDF_THREADS), SDF_THREADS, 0, s, b->leaf_to_elem, b->n,
                pos_buf.as<int32_t>());
    nrm_buf = Scratch((size_t)n * 12, s);
    THEA_LAUNCH(closest_normal_kernel, blocks_pts, SDF_THREADS, 0, s, b->ray_rec, pos_buf.as<int32_t>(),
                elem_buf.as<int32_t>(), n, nrm_buf.as<float>());
    normals = nrm_buf.as<float>();
  }
  Scratch o((size_t)total * 12, s), d((size_t)total * 12, s), t((size_t)total * 4, s), idx((size_t)total * 4, s),
      hn((size_t)total * 12, s);
  THEA_LAUNCH(sdf_rays_kernel, (unsigned)ceil_div(total, SDF_THREADS), SDF_THREADS, 0, s, positions, normals, n,
              0.001f * scale, o.as<float>(), d.as<float>());
  float const * ro = o.as<float>();
  float const * rd = d.as<float>();
  Scratch o_obj, d_obj;
  if (b->has_transform) {
    o_obj = Scratch((size_t)total * 12, s);
    d_obj = Scratch((size_t)total * 12, s);
    rays_to_object(b, ro, rd, total, o_obj.as<float>(), d_obj.as<float>(), s);
    ro = o_obj.as<float>();
    rd = d_obj.as<float>();
  }
  RayParams rp;
  run_ray(b, ro, rd, total, rp, t.as<float>(), idx.as<int32_t>(), hn.as<float>(), nullptr, nullptr, nullptr, b->err, s);
  if (b->has_transform) normals_to_world(b, hn.as<float>(), total, s);
  THEA_LAUNCH(sdf_reduce_kernel, blocks_pts, SDF_THREADS, 0, s, t.as<float>(), hn.as<float>(), d.as<float>(),
              elem_buf.as<int32_t>(), n, (double)scale, only_interior ? 1 : 0, out);
  THEA_CUDA_CHECK(cudaStreamSynchronize(s));
}

}  // namespace thea
