// ramp_filter.h -- plan and launcher of the FP32 FFT ramp-filter convolution.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "ctbb_internal.h"

namespace ctbb {

constexpr int kMaxRampTransform = 8192;  // rows up to 4096 samples

struct RampFilterPlan {
    int n = 0;                     // row length (n_channels_oversampled)
    int m = 0;                     // transform size
    std::vector<float> taps;       // 2n host taps the spectrum was made from
    float2 *d_spectrum = nullptr;  // H/M [m], followed by the twiddle table [m]
    float2 *d_twiddle = nullptr;  // exp(-2 pi i t / m) [m]
    float2 *d_tw16 = nullptr;     // radix-16 pass tables of the 4096-point kernel
    size_t capacity = 0;
};

int ramp_transform_size(int n);
int prepare_ramp_filter(const float *h_taps, int n, RampFilterPlan *plan, cudaStream_t stream);
int launch_ramp_filter(const RampFilterPlan &plan, float *d_lines, size_t n_lines,
                       cudaStream_t stream);

}  // namespace ctbb
