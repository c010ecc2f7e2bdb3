// The ShapeDiameter surface feature (Algorithms/SurfaceFeatures/Local/ShapeDiameter.hpp) for many points.
#pragma once

#include "bvh.hpp"

namespace thea {

// ShapeDiameter(bvh, scale)::compute for n points (ShapeDiameter.hpp:94-101,143-217): 30 rays in a cone about the inward
// normal from each point (origins pushed 0.001 * scale inwards), first hits kept if the hit element's normal faces along
// the ray (only_interior) or always, outliers beyond one standard deviation of the median rejected, the rest averaged
// with cosine weights and divided by scale, clamped to [0, 1]; -1 where no ray is kept (or no element is found).
// normals == nullptr: each point takes the normal of its closest element (the element's own, untransformed normal, as
// the reference does). scale <= 0: the |extent| of the BVH's bounds (the constructor's default for a precomputed BVH).
// Device pointers; synchronizes the stream.
void run_shape_diameter(thea_bvh const * b, float const * positions, float const * normals, int64_t n, float scale,
                        bool only_interior, double * out, cudaStream_t s);

}  // namespace thea
