// Library-internal access to an engine context (hbt_capi.cu) for the
// serving loop (hbt_server.cu), which runs the pair binning of many
// contexts in one launch.
#pragma once

#include "../../include/hbt_gpu.h"
#include "hbt_engine.cuh"

namespace hbt {

// The context's engine descriptor (grid, screen constants, histograms).
const Device &ctx_device(const hbt_ctx *c);
// Persistent-kernel grid for the context's device.
int ctx_persistent_grid(const hbt_ctx *c);
// Adds candidate pairs binned on the context's behalf to its statistics.
void ctx_add_pairs(hbt_ctx *c, u64 same, u64 mixed);
// Merges the FP32-weight partials into the FP64 bins on `st` (no-op for
// the FP64 form).
cudaError_t ctx_merge(hbt_ctx *c, cudaStream_t st);
// Device bytes hbt_create allocates for these parameters.
size_t ctx_device_bytes(const hbt_params &p);

}  // namespace hbt
