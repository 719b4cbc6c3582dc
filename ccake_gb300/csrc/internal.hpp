// Library-internal hooks of the context used by the event server: stepping
// without waiting, the stop-rule probe, the device-memory estimate, and the
// pieces of grouped (multi-event) stepping.
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

// --- groups of mixed-form events advanced by grouped launches (GroupArgs) ---
// The event's descriptor: its constants, EoS (FP32 table Jacobians) and arrays.
void group_desc(ccake_ctx* ctx, ccake::EventDesc* out);
// RK2 steps a candidate list stays valid (the group's quantum).
int list_period(ccake_ctx* ctx);
// Before the event's first grouped step: error counters cleared and the
// mixed smoothing record packed (on the context's stream, synchronised).
ccake_status_t group_join(ccake_ctx* ctx);
// Enqueues the event's list build on stream s and the copy of its largest
// candidate count to *host_cand_max (pinned).
void group_build(ccake_ctx* ctx, cudaStream_t s, int32_t* host_cand_max);
// After group_build completed: grows the event's lists when the count did not
// fit them and builds them again (synchronised); *changed when the event's
// arrays moved (its slot must be refreshed).
ccake_status_t group_grow(ccake_ctx* ctx, int32_t cand_max, bool* changed);
// The event left its group at tau: the host's clock, the records' form.
void group_leave(ccake_ctx* ctx, double tau);

}  // namespace ccake_internal
