// ramp_tc.h -- the ramp filter as an FP16 hi/lo Toeplitz contraction on the
// tensor cores (tcgen05), writing FP16 rows with a per-row power-of-two scale.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <vector>

#include "ctbb_internal.h"

namespace ctbb {

struct RampTcPlan {
    int n = 0;                    // row length
    std::vector<float> taps;      // the 2n taps T was made from
    float sum_abs_taps = 0.0f;    // bound of |y| / max|x|
    void *d_t = nullptr;          // 2^10 T^T hi and lo, FP16 [1536][n] each
    int *d_error = nullptr;       // set by a pipeline wait that ran out
};

// Row lengths the kernel takes: multiples of 64 up to 1536.
bool ramp_tc_supported(int n);
// Device scratch launch_ramp_tc needs for n_lines rows of length n.
size_t ramp_tc_work_bytes(size_t n_lines, int n);
int prepare_ramp_tc(const float *h_taps, int n, RampTcPlan *plan, cudaStream_t stream);
// d_rows [n_lines][n] float32 (not changed) -> d_out FP16 and d_scale
// [n_lines]: y = d_out * d_scale.  rows_per_view = 0: d_out [n_lines][n];
// rows_per_view > 0 (dividing 128; all rows of a view share one scale):
// footprint quads d_out [n_lines][n][4] = (y[r][c], y[r][c+1], y[r+1][c],
// y[r+1][c+1]) / scale, zero where r + 1 or c + 1 leaves the view.
// d_work: ramp_tc_work_bytes.
int launch_ramp_tc(const RampTcPlan &plan, const float *d_rows, size_t n_lines, __half *d_out, float *d_scale,
                   void *d_work, cudaStream_t stream, int rows_per_view = 0);
// Synchronises the stream and returns CTBB_ERR_CUDA if a launch since the
// plan was prepared recorded a pipeline wait that ran out.
int ramp_tc_check(const RampTcPlan &plan, cudaStream_t stream);
void release_ramp_tc(RampTcPlan *plan);

}  // namespace ctbb
