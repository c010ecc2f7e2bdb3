// Byte images of built BVHs (serialize.cu).
#pragma once

#include "bvh.hpp"

namespace thea {

// Size of the image of b (out == nullptr), or writes it to host memory `out` (capacity bytes) and returns its size.
// Synchronizes the stream.
int64_t serialize_bvh(thea_bvh const * b, void * out, int64_t capacity, cudaStream_t s);
// A new handle on the current device from an image (host memory); the header is checked before anything is allocated.
thea_bvh * deserialize_bvh(void const * in, int64_t bytes, cudaStream_t s);

}  // namespace thea
