// Tensor-core (tcgen05) Gram-tile k-NN candidates with an exact FP32 re-rank (gram.cu).
#pragma once

#include "bvh.hpp"

namespace thea {

int gram_tile_rows();  // query rows of one tile (128)
int gram_tile_cols();  // candidates of one window (512)
// The candidate path needs at least one full window of points.
bool gram_supported(int64_t n);
// bound[q] (q = leaf position of a point BVH): the k-th smallest exact FP32 squared distance among the query's best
// Gram-scored window candidates, itself excluded; +inf where none.
void run_gram_bounds(thea_bvh const * b, int k, float * bound, cudaStream_t s);
// keys[r * gram_tile_cols() + j] = |b_j|^2 - 2 a_r . b_j in the tile's normalised FP16 frame (test primitive);
// a: na <= 128 points, b: nb <= 512 points, device arrays of 3 floats each.
void run_gram_tile(float const * a, int na, float const * b, int nb, float * keys, unsigned * err, cudaStream_t s);

// Runs the bounded device-side wait of these kernels on a barrier that nothing completes; true if it gave up (the
// expected outcome) within `limit` try-wait rounds. Synchronizes the stream.
bool run_wait_probe(int limit, cudaStream_t s);

}  // namespace thea
