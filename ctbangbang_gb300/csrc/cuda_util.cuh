// cuda_util.cuh -- error handling, stream and launch bookkeeping shared by the
// CUDA translation units.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cstdint>

#include "ctbb_internal.h"

namespace ctbb {

cudaStream_t current_stream();
int num_sms();
void count_launch(uint64_t n = 1);
// Returns CTBB_OK if a CUDA device is usable, else sets the error text.  Binds
// nothing: the library-wide context binds its device at its first compute call.
int require_device();
// The adaptive filter of one window on the library-wide stream with the
// caller's scratch (6 * n_proj_pull floats), under the library-wide lock and
// counted in the stage profile.
int run_adaptive_filter_with(const struct recon_metadata &mr, const float *d_in, float *d_out, float *d_scratch);

}  // namespace ctbb

// Evaluate a CUDA runtime call; on failure record the error and return CTBB_ERR_CUDA.
#define CTBB_CUDA_TRY(expr)                                                               \
    do {                                                                                  \
        cudaError_t ctbb_e_ = (expr);                                                     \
        if (ctbb_e_ != cudaSuccess) {                                                     \
            ::ctbb::set_error("%s failed: %s (%s:%d)", #expr, cudaGetErrorString(ctbb_e_), \
                              __FILE__, __LINE__);                                        \
            return CTBB_ERR_CUDA;                                                         \
        }                                                                                 \
    } while (0)

// Propagate a non-zero ctbb status.
#define CTBB_TRY(expr)              \
    do {                            \
        int ctbb_s_ = (expr);       \
        if (ctbb_s_) return ctbb_s_; \
    } while (0)
