// adaptive_filter.h -- launcher of the Kachelriess-Kalender adaptive raw filter.
#pragma once

#include <cuda_runtime.h>

#include "ctbb_internal.h"

namespace ctbb {

// Floats of device scratch launch_adaptive_filter needs for a window of
// n_proj_pull frames: sup, smooth, ecc, max, min, threshold ([6][P]).
size_t adaptive_filter_scratch_floats(size_t n_proj_pull);

// d_in -> d_out (distinct buffers) for the pull window described by mr.
int launch_adaptive_filter(const struct recon_metadata &mr, const float *d_in, float *d_out,
                           float *d_scratch, cudaStream_t stream);

}  // namespace ctbb
