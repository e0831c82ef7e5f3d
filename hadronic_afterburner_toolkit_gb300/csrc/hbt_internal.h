// Library-internal access to an engine context (hbt_capi.cu) for the
// serving loop (hbt_server.cu), which runs the pair binning of many
// contexts in one launch.
#pragma once

#include "../../include/hbt_gpu.h"
#include "hbt_engine.cuh"

namespace hbt {

// hbt_create's parameter checks.
bool params_valid(const hbt_params &p);
// The histogram geometry and the constants the reference derives from the
// parameters (src/HBT_correlation.cpp:25-61), psi_ref = 0.
void grid_from_params(const hbt_params &p, Grid &g);
// FP32 copies of a grid's constants for the pair screen, with the bound on
// each one's rounding.
void screen_from_grid(const Grid &g, Screen &s);
// hbt_create with the context's device memory taken, stream-ordered on its
// own stream, from `pool` (nullptr: cudaMalloc), so that creating and
// destroying contexts does not synchronise the device.
hbt_status ctx_create(const hbt_params *p, int device, cudaMemPool_t pool, hbt_ctx **out);
// The context's own stream.
cudaStream_t ctx_stream(const hbt_ctx *c);

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
// True when the context's fast pairs can go to the batched persistent
// kernels (screened kernel family, no q_inv histograms).
bool ctx_batchable(const hbt_ctx *c);
// True when a needed_number_of_pairs cap could reject one of P more pairs
// (mixed = 0: numerator families, 1: denominator families).
bool ctx_caps_may_bind(const hbt_ctx *c, int mixed, u64 P);

}  // namespace hbt
