// f3d_engine_internal.hpp -- engine functions for other parts of the library
// (the serving loop), outside the C ABI.
#pragma once

#include "fft3d_gb300.h"

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

namespace f3d {

// Whether the engine runs the fused tensor-core form, whose steps can share
// launches with other such engines.
bool engine_batchable(const f3d_engine* e);
// Engines with the same key may share a launch: block size, overlap, window
// type, temporal mode, sample format and spectrum storage.
uint64_t engine_batch_key(const f3d_engine* e);
// The key an engine for this plane will have (without fp16 spectrum storage),
// before it is created.
uint64_t plane_batch_key(const f3d_internal_params& p, const f3d_plane_geom& g);

// One temporal step of n (1..16) distinct batchable engines whose stream is
// st, one launch per kernel for all of them: engine i forwards frame fns[i]
// from src[i] (skipped when fns[i] < 0 or cached), then, when nwin[i] > 0,
// filters its window win[i] into dst[i] with its own operand tiles and seam
// rows. Queued on st. On failure *err has the message.
int engines_step(f3d_engine* const* e, int n, const int* fns, const void* const* src, const size_t* src_pitch,
                 const int* const* win, const int* nwin, void* const* dst, const size_t* dst_pitch, cudaStream_t st,
                 std::string* err);

}  // namespace f3d
