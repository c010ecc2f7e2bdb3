// Byte image of a built BVH (thea_bvh_serialize / thea_bvh_deserialize): a versioned header, the handle's parameters,
// then its device arrays in a fixed order. Reloading an image skips the build: a serving process can warm-start its
// resident meshes. The reference has no counterpart (its BvhN is not Serializable).
#include "serialize.hpp"
#include "transform.hpp"

#include "common.cuh"

#include <cstring>
#include <string>
#include <vector>

namespace thea {
namespace {

constexpr char MAGIC[8] = {'T', 'H', 'E', 'A', 'B', 'V', 'H', '\0'};
constexpr uint32_t IMAGE_VERSION = 1;

// Fixed-layout header (all fields little-endian as written by this library; images are for the same build family)
struct ImageHeader {
  char magic[8];
  uint32_t version;
  int32_t is_mesh, width, leaf_size, depth, query_order;
  uint32_t layouts;
  int32_t num_segments;
  int64_t n, num_nodes, device_bytes;
  float lo[3], hi[3];
  int64_t node_bytes, cp_bytes, ray_bytes, pt_bytes;  // sizes of the array sections
  int32_t has_transform, reserved;
  float xf[12];  // affine transform (row-major 3x4); the world-space copy is rebuilt on load
};

int64_t node_size(int width) { return width == 4 ? (int64_t)sizeof(WideNode<4>) : (int64_t)sizeof(WideNode<8>); }

int64_t image_bytes(ImageHeader const & h) {
  int64_t M = h.num_segments;
  return (int64_t)sizeof(ImageHeader) + h.node_bytes + h.cp_bytes + h.ray_bytes + h.pt_bytes + h.n * 4 +
         (M + 1) * 8 + M * 4 + M * 24;
}

ImageHeader header_of(thea_bvh const * b) {
  ImageHeader h;
  std::memset(&h, 0, sizeof(h));
  std::memcpy(h.magic, MAGIC, sizeof(MAGIC));
  h.version = IMAGE_VERSION;
  h.is_mesh = b->is_mesh;
  h.width = b->width;
  h.leaf_size = b->leaf_size;
  h.depth = b->depth;
  h.query_order = b->query_order;
  h.layouts = b->layouts;
  h.num_segments = b->num_segments;
  h.n = b->n;
  h.num_nodes = b->num_nodes;
  h.device_bytes = b->device_bytes;
  for (int t = 0; t < 3; ++t) {
    h.lo[t] = b->lo[t];
    h.hi[t] = b->hi[t];
  }
  h.node_bytes = b->num_nodes * node_size(b->width);
  h.cp_bytes = b->cp_rec ? b->n * CP_REC_F4 * 16 : 0;
  h.ray_bytes = b->ray_rec ? b->n * RAY_REC_F4 * 16 : 0;
  h.pt_bytes = b->pt_rec ? b->n * 16 : 0;
  h.has_transform = b->has_transform;
  std::memcpy(h.xf, b->xf, sizeof(h.xf));
  return h;
}

}  // namespace

int64_t serialize_bvh(thea_bvh const * b, void * out, int64_t capacity, cudaStream_t s) {
  ImageHeader h = header_of(b);
  int64_t total = image_bytes(h);
  if (!out) return total;
  THEA_REQUIRE(capacity >= total, "bvh_serialize: buffer too small");
  char * p = (char *)out;
  std::memcpy(p, &h, sizeof(h));
  p += sizeof(h);
  auto d2h = [&](void const * src, int64_t bytes) {
    if (bytes > 0) THEA_CUDA_CHECK(cudaMemcpyAsync(p, src, (size_t)bytes, cudaMemcpyDeviceToHost, s));
    p += bytes;
  };
  int M = b->num_segments;
  d2h(b->nodes, h.node_bytes);
  d2h(b->cp_rec, h.cp_bytes);
  d2h(b->ray_rec, h.ray_bytes);
  d2h(b->pt_rec, h.pt_bytes);
  d2h(b->leaf_to_elem, h.n * 4);
  d2h(b->seg_start, (int64_t)(M + 1) * 8);
  d2h(b->seg_root, (int64_t)M * 4);
  THEA_CUDA_CHECK(cudaStreamSynchronize(s));
  std::memcpy(p, b->seg_lo.data(), (size_t)M * 12);
  p += (int64_t)M * 12;
  std::memcpy(p, b->seg_hi.data(), (size_t)M * 12);
  return total;
}

thea_bvh * deserialize_bvh(void const * in, int64_t bytes, cudaStream_t s) {
  THEA_REQUIRE(in && bytes >= (int64_t)sizeof(ImageHeader), "bvh_deserialize: buffer shorter than a header");
  ImageHeader h;
  std::memcpy(&h, in, sizeof(h));
  THEA_REQUIRE(std::memcmp(h.magic, MAGIC, sizeof(MAGIC)) == 0, "bvh_deserialize: not a BVH image");
  THEA_REQUIRE(h.version == IMAGE_VERSION, "bvh_deserialize: image version " + std::to_string(h.version) +
                                                 " is not supported (expected " + std::to_string(IMAGE_VERSION) + ")");
  THEA_REQUIRE((h.width == 4 || h.width == 8) && h.n > 0 && h.n <= bytes && h.num_nodes > 0 &&
                   h.num_nodes <= bytes && h.num_segments >= 1 &&
                   h.num_segments <= h.n && (h.is_mesh == 0 || h.is_mesh == 1),
               "bvh_deserialize: inconsistent header");
  THEA_REQUIRE(h.node_bytes == h.num_nodes * node_size(h.width) &&
                   h.cp_bytes == (h.is_mesh && (h.layouts & THEA_LAYOUT_CLOSEST) ? h.n * CP_REC_F4 * 16 : 0) &&
                   h.ray_bytes == (h.is_mesh && (h.layouts & THEA_LAYOUT_RAY) ? h.n * RAY_REC_F4 * 16 : 0) &&
                   h.pt_bytes == (h.is_mesh ? 0 : h.n * 16),
               "bvh_deserialize: inconsistent section sizes");
  THEA_REQUIRE(h.has_transform == 0 || (h.has_transform == 1 && h.num_segments == 1),
               "bvh_deserialize: inconsistent transform");
  THEA_REQUIRE(bytes >= image_bytes(h), "bvh_deserialize: buffer shorter than the image");
  thea_bvh * b = new thea_bvh;
  try {
    THEA_CUDA_CHECK(cudaGetDevice(&b->device));
    b->is_mesh = h.is_mesh;
    b->width = h.width;
    b->leaf_size = h.leaf_size;
    b->depth = h.depth;
    b->query_order = h.query_order;
    b->layouts = h.layouts;
    b->num_segments = h.num_segments;
    b->n = h.n;
    b->num_nodes = h.num_nodes;
    b->device_bytes = h.device_bytes;
    for (int t = 0; t < 3; ++t) {
      b->lo[t] = h.lo[t];
      b->hi[t] = h.hi[t];
    }
    int M = h.num_segments;
    char const * p = (char const *)in + sizeof(h);
    auto h2d = [&](void ** dst, int64_t nbytes) {
      if (nbytes > 0) {
        THEA_CUDA_CHECK(thea_malloc_async(dst, (size_t)nbytes, s));
        THEA_CUDA_CHECK(cudaMemcpyAsync(*dst, p, (size_t)nbytes, cudaMemcpyHostToDevice, s));
      }
      p += nbytes;
    };
    h2d(&b->nodes, h.node_bytes);
    h2d((void **)&b->cp_rec, h.cp_bytes);
    h2d((void **)&b->ray_rec, h.ray_bytes);
    h2d((void **)&b->pt_rec, h.pt_bytes);
    h2d((void **)&b->leaf_to_elem, h.n * 4);
    h2d((void **)&b->seg_start, (int64_t)(M + 1) * 8);
    h2d((void **)&b->seg_root, (int64_t)M * 4);
    b->seg_start_host.resize((size_t)M + 1);
    std::memcpy(b->seg_start_host.data(), (char const *)in + sizeof(h) + h.node_bytes + h.cp_bytes + h.ray_bytes +
                                              h.pt_bytes + h.n * 4,
                (size_t)(M + 1) * 8);
    b->seg_lo.resize((size_t)3 * M);
    b->seg_hi.resize((size_t)3 * M);
    std::memcpy(b->seg_lo.data(), p, (size_t)M * 12);
    p += (int64_t)M * 12;
    std::memcpy(b->seg_hi.data(), p, (size_t)M * 12);
    THEA_CUDA_CHECK(thea_malloc_async((void **)&b->err, sizeof(unsigned), s));
    THEA_CUDA_CHECK(cudaMemsetAsync(b->err, 0, sizeof(unsigned), s));
    THEA_CUDA_CHECK(thea_malloc_host(&b->err_host, sizeof(unsigned)));
    *b->err_host = 0;
    // the host image may be reused by the caller as soon as this returns
    THEA_CUDA_CHECK(cudaStreamSynchronize(s));
    init_segment_roots(b, s);
    init_slabs(b, s);
    if (h.has_transform) set_transform(b, h.xf, s);
    return b;
  } catch (...) {
    cudaStreamSynchronize(s);
    destroy_bvh(b);
    throw;
  }
}

}  // namespace thea
