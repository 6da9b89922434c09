// peak_probe.cu -- FP32 FMA throughput of the device, measured.
//
// The backprojector is bound by the FP32 pipe; its roofline needs the FP32
// peak of this GPU under the clocks of the run (the measured peak figures
// at hand are HBM and BF16 only).  Measurement infrastructure, built
// into libctbb_synth.so, not into the reconstruction library.  Each thread runs 16
// independent FMA chains (enough to hide the FMA latency) for a fixed number
// of iterations on registers only; the result is stored so the work is kept.
#include <cuda_runtime.h>

#include <algorithm>

#include "synth.h"

namespace synth {
namespace {

constexpr int kChains = 16;
constexpr int kIters = 4096;

__global__ void __launch_bounds__(256) ffma_probe_kernel(float *out, float a, float b)
{
    float v[kChains];
#pragma unroll
    for (int k = 0; k < kChains; ++k) v[k] = (float)(threadIdx.x + k) * 1e-3f;
    for (int i = 0; i < kIters; ++i) {
#pragma unroll
        for (int k = 0; k < kChains; ++k) v[k] = fmaf(v[k], a, b);
    }
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < kChains; ++k) s += v[k];
    if (s == 1234.5f) out[0] = s;  // keeps the chains live; practically never taken
}

}  // namespace
}  // namespace synth

using namespace synth;

// Best of `repeats` launches, in TFLOP/s (2 FLOP per FMA).
extern "C" double synth_fp32_peak_tflops(int repeats, void *stream)
{
    int n_dev = 0, dev = 0, sms = 0;
    if (cudaGetDeviceCount(&n_dev) != cudaSuccess || n_dev == 0) return -1.0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1.0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1.0;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    float *d = nullptr;
    if (cudaMalloc(&d, sizeof(float)) != cudaSuccess) return -1.0;
    int blocks = sms * 8;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double best = 0.0;
    for (int r = 0; r < (repeats > 0 ? repeats : 1) + 1; ++r) {
        cudaEventRecord(e0, s);
        ffma_probe_kernel<<<blocks, 256, 0, s>>>(d, 0.999999f, 1e-7f);
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        double flop = 2.0 * kChains * (double)kIters * blocks * 256.0;
        if (r > 0 && ms > 0) best = std::max(best, flop / (ms * 1e-3) / 1e12);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    return best;
}
