// Library-internal hooks of the context used by the event server: stepping
// without waiting, the stop-rule probe and the device-memory estimate.
#pragma once
#include <cuda_runtime.h>

#include "ccake_gpu.h"
#include "kernels.cuh"

namespace ccake_internal {

// Enqueues n RK2 steps (graph launches, list rebuilds on schedule) on the
// context's stream; no synchronisation, no error check. Errors accumulate
// in the device counters that the probe reports.
ccake_status_t step_enqueue(ccake_ctx* ctx, int n);

// Enqueues the probe (largest T, tau, error counters) into dev and its copy
// to host (pinned) on the context's stream.
ccake_status_t probe_enqueue(ccake_ctx* ctx, ccake::Probe* dev, ccake::Probe* host);

// Clears the device error counters (enqueued).
ccake_status_t clear_errors(ccake_ctx* ctx);

cudaStream_t ctx_stream(ccake_ctx* ctx);
void ctx_set_time(ccake_ctx* ctx, double t);

// Device bytes an event of n particles is expected to hold (before its
// neighbour-list capacities are known).
int64_t estimate_bytes(const ccake_config& cfg, int64_t n);

}  // namespace ccake_internal
