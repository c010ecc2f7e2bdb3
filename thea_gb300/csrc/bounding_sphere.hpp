// Smallest enclosing ball of a point set: the sphere BestFitSphereN computes (Algorithms/BestFitSphereN.hpp:62-91, the
// miniball of its points in double precision), which ShapeDiameter(mesh) takes as its default scale
// (Algorithms/SurfaceFeatures/Local/ShapeDiameter.hpp:60-70: the diameter of the mesh vertices' sphere).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace thea {

// Centre and radius (double) of the smallest ball holding the n points (xyz float triples, device memory). n = 0 gives
// the zero ball at the origin, n = 1 the point itself. Synchronizes the stream once per pivot step.
void run_bounding_sphere(float const * points, int64_t n, double * center, double * radius, cudaStream_t s);

// The ball of up to five points (double xyz), for tests of the host step: the smallest ball containing them all.
// Returns the number of points on its boundary that define it (its support), or 0 if none was found.
int smallest_ball_of_few(double const * pts, int k, double * center, double * radius);

}  // namespace thea
