// Serving loop: resident meshes, admission by a device-memory budget, continuous batching of mixed closest-point,
// ray and k-NN requests (include/thea_gpu.h, thea_server_*).
#pragma once

#include "bvh.hpp"

struct thea_server;

namespace thea {

thea_server * server_create(thea_server_config const & cfg);
// Cancels what is still pending, waits for the batches on the device, releases everything.
void server_destroy(thea_server * s);
int32_t server_add_mesh(thea_server * s, float const * V, int64_t nv, int32_t const * F, int64_t nf);
void server_remove_mesh(thea_server * s, int32_t mesh);
uint64_t server_submit(thea_server * s, thea_request const & r);
// THEA_ERR_WAIT_TIMEOUT if the request is not finished within timeout_us (negative: no limit). On THEA_OK the
// request's own status and latency are written and its ticket is retired.
thea_status server_wait(thea_server * s, uint64_t ticket, int64_t timeout_us, thea_status * request_status,
                        double * latency_ms);
void server_cancel(thea_server * s, uint64_t ticket);
void server_stats(thea_server * s, thea_server_stats * out);
void server_reset_stats(thea_server * s);

}  // namespace thea
