// adaptive_filter.cu -- Kachelriess-Kalender adaptive raw-data filter.
//
// Reference: adaptive_filter_kk (src/preprocessing.cu:31-156) and its kernels
// (include/preprocessing.cuh:32-285), the reference's only implementation (it
// has no CPU twin; src/main.cu:222 runs it on every block).  Per pull window of
// P frames:
//   1. sup[p]      = max(0, max of frame p)                        (extract_sup)
//   2. smooth[p]   = mean of sup over an 18 deg window, clamped     (smooth_sup)
//   3. ecc[p]      = clamp(((1 - min/max) - 0.3) / 0.2, 0, 1) over a
//                    180 deg window of smooth; min/max kept         (eccentricity)
//   4. T[p]        = <= 20-step bisection between min and max so that the
//                    fraction of the 180 deg window of smooth above T matches
//                    F_MAX * strength * ecc within 1 %                (find_thresholds)
//   5. out         = 5x5x5 normalised triangle smoothing of samples > T[p],
//                    other samples copied                          (filter_projections)
// With strength 0 the stopping test divides by zero and T climbs toward the
// window maximum; samples above it are still smoothed.  That behaviour is kept.
//
// Every float operation is written as a separate rounding (__f*_rn) in the
// reference's order, so the result equals the reference kernels evaluated
// without fused multiply-adds.  GB300 mapping: step 1 is a CTA reduction per
// frame, steps 2-3 one thread per frame, step 4 one warp per frame (the window
// counts are integers, so splitting them across lanes is exact), step 5 a
// per-frame float4 copy that lists the samples above the threshold in shared
// memory and smooths them after the copy (rows of a multiple of 4 channels;
// otherwise a shared-memory tiled stencil).  Every step takes a frame range,
// so a window whose frames arrive in order can be filtered as they come
// (AfStream).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>

#include "adaptive_filter.h"
#include "ctbb_internal.h"
#include "cuda_util.cuh"

namespace ctbb {

namespace {

constexpr float kFMax = 0.03f;  // F_MAX, include/preprocessing.cuh:23
constexpr float kPiAf = kPiBackproject;

// triangle_3d(5, i, j, k) = (3-|i-3|) + (3-|j-3|) + (3-|k-3|) + 1
// (include/preprocessing.cuh:64-67); its peak is at index 3 of 0..4.
__host__ __device__ constexpr int tri1(int i) { return 3 - (i > 3 ? i - 3 : 3 - i); }

struct AfParams {
    const float *raw;
    float *out;
    float *sup, *smooth, *ecc, *pmax, *pmin, *thr;
    int P, R, N;
    int n_proj_ffs;
    int n_avg, avg_offset;
    int n_range, range_offset;
    float strength;
    int f0, f1;  // frames this launch writes: [f0, f1) of the window [0, P)
};

__global__ void af_sup_kernel(AfParams p)
{
    int proj = p.f0 + blockIdx.x;
    size_t frame = (size_t)p.R * p.N;
    const float *src = p.raw + (size_t)proj * frame;
    float m = 0.0f;
    if ((frame & 3) == 0) {  // frames start 16-byte aligned: float4 loads
        const float4 *s4 = reinterpret_cast<const float4 *>(src);
        for (size_t i = threadIdx.x; i < frame / 4; i += blockDim.x) {
            float4 v = __ldg(s4 + i);
            m = fmaxf(fmaxf(m, fmaxf(v.x, v.y)), fmaxf(v.z, v.w));
        }
    } else {
        for (size_t i = threadIdx.x; i < frame; i += blockDim.x) m = fmaxf(m, src[i]);
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ float red[32];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0f;
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (threadIdx.x == 0) p.sup[proj] = m;
    }
}

__global__ void af_smooth_kernel(AfParams p)
{
    int proj = p.f0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (proj >= p.f1) return;
    float w = __fdiv_rn(1.0f, (float)p.n_avg);
    float acc = 0.0f;
    int max_idx = p.P - 1;
    for (int i = 0; i < p.n_avg; i++) {
        int idx = proj - p.avg_offset + i;
        idx = idx < 0 ? 0 : (idx > max_idx ? max_idx : idx);
        acc = __fadd_rn(acc, __fmul_rn(w, p.sup[idx]));
    }
    p.smooth[proj] = acc;
}

__global__ void af_ecc_kernel(AfParams p)
{
    int proj = p.f0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (proj >= p.f1) return;
    int max_idx = p.P - 1;
    float vmax = 0.0f, vmin = 10000.0f;
    for (int i = 0; i < p.n_range; i++) {
        int idx = proj - p.range_offset + i;
        idx = idx < 0 ? 0 : (idx > max_idx ? max_idx : idx);
        float v = p.smooth[idx];
        if (v > vmax) vmax = v;
        if (v < vmin) vmin = v;
    }
    p.pmax[proj] = vmax;
    p.pmin[proj] = vmin;
    float e = __fsub_rn(1.0f, __fdiv_rn(vmin, vmax));
    e = __fdiv_rn(__fsub_rn(e, 0.3f), __fsub_rn(0.5f, 0.3f));
    float out;
    if (e > 1) out = 1.0f;
    else if (e < 0) out = 0.0f;
    else out = e;
    p.ecc[proj] = out;
}

// rhs() of include/preprocessing.cuh:32-62, the window count split over a warp.
__device__ float window_fraction(const AfParams &p, int start_idx, float T, int lane)
{
    int numel = p.n_range;
    int max_idx = p.P - 1;
    int diff = start_idx + (numel - 1);
    if (diff < (numel - 1)) {
        numel += start_idx;
        start_idx = 0;
    }
    if (diff > max_idx) numel -= (diff - max_idx);
    int count = 0;
    for (int i = lane; i < numel; i += 32) count += (p.smooth[start_idx + i] > T) ? 1 : 0;
    for (int o = 16; o > 0; o >>= 1) count += __shfl_xor_sync(0xffffffffu, count, o);
    const float inv_pi = 1.0f / kPiAf;
    return __fmul_rn(__fmul_rn(inv_pi, (float)count), __fdiv_rn(1.0f, (float)p.n_proj_ffs));
}

__global__ void af_threshold_kernel(AfParams p)
{
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    int proj = p.f0 + warp;
    if (proj >= p.f1) return;
    float lower = p.pmin[proj];
    float upper = p.pmax[proj];
    float T = __fdiv_rn(__fadd_rn(p.pmax[proj], p.pmin[proj]), 2.0f);
    float lhs = __fmul_rn(__fmul_rn(kFMax, p.strength), p.ecc[proj]);
    int start = proj - p.range_offset;
    float rhs = window_fraction(p, start, T, lane);
    int iter = 0;
    // (|lhs - rhs| / lhs) > 0.01 with the float quotient promoted to double
    while ((double)__fdiv_rn(fabsf(__fsub_rn(lhs, rhs)), lhs) > 0.01) {
        if (iter >= 20) break;
        iter += 1;
        if (rhs > lhs) lower = T;
        else if (rhs < lhs) upper = T;
        else break;
        T = __fdiv_rn(__fadd_rn(lower, upper), 2.0f);
        rhs = window_fraction(p, start, T, lane);
    }
    if (lane == 0) p.thr[proj] = T;
}

// Stencil tile: TP frames x TR rows x TC channels of output per CTA.
constexpr int TP = 4, TR = 8, TC = 32;
constexpr int SP = TP + 4, SR = TR + 4, SC = TC + 4;

__global__ void __launch_bounds__(256) af_filter_kernel(AfParams p)
{
    __shared__ float tile[SP][SR][SC];
    int c0 = blockIdx.x * TC, r0 = blockIdx.y * TR, p0 = p.f0 + blockIdx.z * TP;
    size_t frame = (size_t)p.R * p.N;
    for (int t = threadIdx.x; t < SP * SR * SC; t += blockDim.x) {
        int sc = t % SC, sr = (t / SC) % SR, sp = t / (SC * SR);
        int gc = c0 + sc - 2, gr = r0 + sr - 2, gp = p0 + sp - 2;
        float v = 0.0f;
        if (gc >= 0 && gc < p.N && gr >= 0 && gr < p.R && gp >= 0 && gp < p.P)
            v = __ldg(p.raw + (size_t)gp * frame + (size_t)gr * p.N + gc);
        tile[sp][sr][sc] = v;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < TP * TR * TC; t += blockDim.x) {
        int lc = t % TC, lr = (t / TC) % TR, lp = t / (TC * TR);
        int gc = c0 + lc, gr = r0 + lr, gp = p0 + lp;
        if (gc >= p.N || gr >= p.R || gp >= p.f1) continue;
        float x = tile[lp + 2][lr + 2][lc + 2];
        float T = p.thr[gp];
        float y = x;
        if (x > T) {
            // norm = sum of in-bounds weights: an exact integer, independent of order
            int ni = 0, nj = 0, nk = 0, si = 0, sj = 0, sk = 0;
            for (int d = 0; d < 5; ++d) {
                if (gc + d - 2 >= 0 && gc + d - 2 < p.N) { ni++; si += tri1(d); }
                if (gr + d - 2 >= 0 && gr + d - 2 < p.R) { nj++; sj += tri1(d); }
                if (gp + d - 2 >= 0 && gp + d - 2 < p.P) { nk++; sk += tri1(d); }
            }
            float norm = (float)(nj * nk * si + ni * nk * sj + ni * nj * sk + ni * nj * nk);
            // taps in the reference's order (channel, row, frame); the weights
            // are compile-time constants of the fully unrolled loops
            float val = 0.0f;
#pragma unroll
            for (int ii = 0; ii < 5; ii++)
#pragma unroll
                for (int jj = 0; jj < 5; jj++)
#pragma unroll
                    for (int kk = 0; kk < 5; kk++)
                        val = __fadd_rn(val, __fmul_rn(tile[lp + kk][lr + jj][lc + ii],
                                                       (float)(tri1(ii) + tri1(jj) + tri1(kk) + 1)));
            y = __fmul_rn(__fdiv_rn(1.0f, norm), val);
        }
        p.out[(size_t)gp * frame + (size_t)gr * p.N + gc] = y;
    }
}

// 5x5x5 triangle smoothing of one sample, taps in the reference's order
// (channel, row, frame) with out-of-range taps skipped; norm is the exact
// integer sum of the in-range weights.
__device__ __noinline__ float smooth_sample(const AfParams &p, int gp, int gr, int gc)
{
    size_t frame = (size_t)p.R * p.N;
    int ni = 0, nj = 0, nk = 0, si = 0, sj = 0, sk = 0;
#pragma unroll
    for (int d = 0; d < 5; ++d) {
        if (gc + d - 2 >= 0 && gc + d - 2 < p.N) { ni++; si += tri1(d); }
        if (gr + d - 2 >= 0 && gr + d - 2 < p.R) { nj++; sj += tri1(d); }
        if (gp + d - 2 >= 0 && gp + d - 2 < p.P) { nk++; sk += tri1(d); }
    }
    float norm = (float)(nj * nk * si + ni * nk * sj + ni * nj * sk + ni * nj * nk);
    float val = 0.0f;
#pragma unroll 1
    for (int ii = 0; ii < 5; ii++) {
        int c = gc + ii - 2;
#pragma unroll 1
        for (int jj = 0; jj < 5; jj++) {
            int r = gr + jj - 2;
#pragma unroll
            for (int kk = 0; kk < 5; kk++) {
                int f = gp + kk - 2;
                if (c < 0 || c >= p.N || r < 0 || r >= p.R || f < 0 || f >= p.P) continue;
                float x = __ldg(p.raw + (size_t)f * frame + (size_t)r * p.N + c);
                val = __fadd_rn(val, __fmul_rn(x, (float)(tri1(ii) + tri1(jj) + tri1(kk) + 1)));
            }
        }
    }
    return __fmul_rn(__fdiv_rn(1.0f, norm), val);
}

// Streaming form for rows of a multiple of 4 channels: one CTA per frame
// copies the frame with float4 loads/stores and notes the samples above the
// frame's threshold -- about 1e-4 of them on clinical-size scans -- in a
// shared-memory list; after the copy the CTA smooths the listed samples (or,
// when the list overflowed, every sample above the threshold again).  The
// copy loop holds no call, so it runs at copy speed.  Same arithmetic, same
// result as the tiled form.
constexpr int kSmoothListMax = 1024;

__global__ void __launch_bounds__(256) af_filter_stream_kernel(AfParams p)
{
    __shared__ int list[kSmoothListMax];
    __shared__ int n_list;
    int gp = p.f0 + blockIdx.x;
    size_t frame = (size_t)p.R * p.N;
    const float4 *src = reinterpret_cast<const float4 *>(p.raw + (size_t)gp * frame);
    float4 *dst = reinterpret_cast<float4 *>(p.out + (size_t)gp * frame);
    float *dst1 = p.out + (size_t)gp * frame;
    const float T = __ldg(p.thr + gp);
    const int n4 = (int)(frame / 4);
    if (threadIdx.x == 0) n_list = 0;
    __syncthreads();
    // kUnroll independent 16-byte loads in flight per thread
    constexpr int kUnroll = 4;
    for (int i0 = threadIdx.x; i0 < n4; i0 += kUnroll * blockDim.x) {
        float4 v[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
            int i = i0 + u * blockDim.x;
            if (i < n4) v[u] = __ldg(src + i);
        }
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
            int i = i0 + u * blockDim.x;
            if (i >= n4) break;
            dst[i] = v[u];
            if (v[u].x > T || v[u].y > T || v[u].z > T || v[u].w > T) {
                float c[4] = {v[u].x, v[u].y, v[u].z, v[u].w};
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (c[e] > T) {
                        int slot = atomicAdd(&n_list, 1);
                        if (slot < kSmoothListMax) list[slot] = 4 * i + e;
                    }
            }
        }
    }
    __syncthreads();
    const int n = n_list;
    if (n <= kSmoothListMax) {
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
            int e = list[j];
            int gr = e / p.N, gc = e - gr * p.N;
            dst1[e] = smooth_sample(p, gp, gr, gc);
        }
    } else {
        const float *src1 = p.raw + (size_t)gp * frame;
        for (int e = threadIdx.x; e < (int)frame; e += blockDim.x) {
            if (__ldg(src1 + e) > T) {
                int gr = e / p.N, gc = e - gr * p.N;
                dst1[e] = smooth_sample(p, gp, gr, gc);
            }
        }
    }
}

// One thread per frame of the window: can this window's filtered frame
// differ from the larger window's?  Not when no sample exceeds either
// threshold (every sample is at most the frame's maximum sup), and not when
// the thresholds agree and the smoothing stencil does not reach past this
// window's ends where the larger window goes on.  NaN thresholds count as
// differing.
__global__ void af_dirty_kernel(const float *sup, const float *thr_union, const float *thr, int P, int fa, int fb,
                                int lo_edge, int hi_edge, unsigned char *dirty)
{
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= P) return;
    unsigned char d = 0;
    if (f < fa || f >= fb) {
        const float s = sup[f], tb = thr[f], tu = thr_union[f];
        const bool end = (lo_edge && f < 2) || (hi_edge && f >= P - 2);
        const bool same = (s <= tb && s <= tu) || (tb == tu && !end);
        d = same ? 0 : 1;
    }
    dirty[f] = d;
}

}  // namespace

size_t adaptive_filter_scratch_floats(size_t n_proj_pull) { return 6 * n_proj_pull; }

namespace {

int af_params(const struct recon_metadata &mr, const float *d_in, float *d_out, float *d_scratch, AfParams *pp)
{
    AfParams &p = *pp;
    p.raw = d_in;
    p.out = d_out;
    p.P = (int)mr.ri.n_proj_pull;
    p.R = (int)mr.cg.n_rows_raw;
    p.N = (int)mr.cg.n_channels;
    p.n_proj_ffs = (int)mr.cg.n_proj_ffs;
    p.sup = d_scratch;
    p.smooth = d_scratch + p.P;
    p.ecc = d_scratch + 2 * (size_t)p.P;
    p.pmax = d_scratch + 3 * (size_t)p.P;
    p.pmin = d_scratch + 4 * (size_t)p.P;
    p.thr = d_scratch + 5 * (size_t)p.P;
    // window sizes, include/preprocessing.cuh:92-96 and :119-122
    int n_avg = (int)ceilf((18.0f / 360.0f) * (float)p.n_proj_ffs);
    n_avg = n_avg + (1 - n_avg % 2);
    p.n_avg = n_avg;
    p.avg_offset = (int)floorf((float)(n_avg / 2));
    int n_range = (int)ceilf((180.0f / 360.0f) * (float)p.n_proj_ffs);
    n_range = n_range + (1 - n_range % 2);
    p.n_range = n_range;
    p.range_offset = (int)floorf((float)(n_range / 2));
    p.strength = mr.rp.adaptive_filtration_s;
    p.f0 = 0;
    p.f1 = p.P;
    if (p.P <= 0 || p.R <= 0 || p.N <= 0) {
        set_error("adaptive filter: empty pull window");
        return CTBB_ERR_ARGUMENT;
    }
    return CTBB_OK;
}

// The five steps over frame ranges: maxima of [sup0, sup1), moving means of
// [smooth0, smooth1), eccentricity, threshold and smoothing of [out0, out1)
// (eccentricity and threshold only with `thresholds`, smoothing only with
// `output`).  Each range may be empty; a step reads the earlier steps'
// results of the frames its windows cover, which the caller has launched
// before.
int af_launch(AfParams p, int sup0, int sup1, int smooth0, int smooth1, int out0, int out1, cudaStream_t stream,
              bool thresholds = true, bool output = true)
{
    int launches = 0;
    if (sup1 > sup0) {
        p.f0 = sup0;
        p.f1 = sup1;
        af_sup_kernel<<<sup1 - sup0, 256, 0, stream>>>(p);
        ++launches;
    }
    if (smooth1 > smooth0) {
        p.f0 = smooth0;
        p.f1 = smooth1;
        af_smooth_kernel<<<(smooth1 - smooth0 + 127) / 128, 128, 0, stream>>>(p);
        ++launches;
    }
    if (out1 > out0 && thresholds) {
        int n = out1 - out0;
        p.f0 = out0;
        p.f1 = out1;
        af_ecc_kernel<<<(n + 127) / 128, 128, 0, stream>>>(p);
        af_threshold_kernel<<<(n * 32 + 255) / 256, 256, 0, stream>>>(p);
        launches += 2;
    }
    if (out1 > out0 && output) {
        int n = out1 - out0;
        p.f0 = out0;
        p.f1 = out1;
        if (p.N % 4 == 0) {
            af_filter_stream_kernel<<<n, 256, 0, stream>>>(p);
        } else {
            dim3 grid((p.N + TC - 1) / TC, (p.R + TR - 1) / TR, (n + TP - 1) / TP);
            if (grid.z > 65535) {
                set_error("adaptive filter: %d frames exceed the launch grid", n);
                return CTBB_ERR_ARGUMENT;
            }
            af_filter_kernel<<<grid, 256, 0, stream>>>(p);
        }
        launches += 1;
    }
    count_launch(launches);
    CTBB_CUDA_TRY(cudaGetLastError());
    return CTBB_OK;
}

}  // namespace

int launch_adaptive_filter(const struct recon_metadata &mr, const float *d_in, float *d_out,
                           float *d_scratch, cudaStream_t stream)
{
    AfParams p;
    CTBB_TRY(af_params(mr, d_in, d_out, d_scratch, &p));
    return af_launch(p, 0, p.P, 0, p.P, 0, p.P, stream);
}

int adaptive_filter_edge_reach(const struct recon_metadata &mr)
{
    AfParams p;
    float dummy = 0.0f;
    if (af_params(mr, &dummy, &dummy, &dummy, &p) != CTBB_OK) return 0;
    return p.range_offset + p.avg_offset;
}

int launch_adaptive_filter_ends_thresholds(const struct recon_metadata &mr, const float *d_in, const float *d_sup,
                                           float *d_scratch, int fa, int fb, cudaStream_t stream)
{
    AfParams p;
    CTBB_TRY(af_params(mr, d_in, nullptr, d_scratch, &p));
    p.sup = const_cast<float *>(d_sup);  // read only: no maxima are launched
    fa = std::min(std::max(fa, 0), p.P);
    fb = std::min(std::max(fb, fa), p.P);
    CTBB_TRY(af_launch(p, 0, 0, 0, p.P, 0, fa, stream, true, false));
    return af_launch(p, 0, 0, 0, 0, fb, p.P, stream, true, false);
}

int launch_adaptive_filter_dirty(const struct recon_metadata &mr, const float *d_sup, const float *d_thr_union,
                                 const float *d_scratch, int fa, int fb, int lo_edge, int hi_edge,
                                 unsigned char *d_dirty, cudaStream_t stream)
{
    AfParams p;
    float dummy = 0.0f;
    CTBB_TRY(af_params(mr, &dummy, &dummy, const_cast<float *>(d_scratch), &p));
    fa = std::min(std::max(fa, 0), p.P);
    fb = std::min(std::max(fb, fa), p.P);
    af_dirty_kernel<<<(p.P + 255) / 256, 256, 0, stream>>>(d_sup, d_thr_union, p.thr, p.P, fa, fb, lo_edge,
                                                              hi_edge, d_dirty);
    count_launch(1);
    CTBB_CUDA_TRY(cudaGetLastError());
    return CTBB_OK;
}

int launch_adaptive_filter_output(const struct recon_metadata &mr, const float *d_in, float *d_out,
                                  const float *d_sup, float *d_scratch, int f0, int f1, cudaStream_t stream)
{
    AfParams p;
    CTBB_TRY(af_params(mr, d_in, d_out, d_scratch, &p));
    p.sup = const_cast<float *>(d_sup);
    f0 = std::min(std::max(f0, 0), p.P);
    f1 = std::min(std::max(f1, f0), p.P);
    return af_launch(p, 0, 0, 0, 0, f0, f1, stream, false, true);
}

AfStream::AfStream(const struct recon_metadata &mr) : P((int)mr.ri.n_proj_pull)
{
    int n_proj_ffs = (int)mr.cg.n_proj_ffs;
    int n_avg = (int)ceilf((18.0f / 360.0f) * (float)n_proj_ffs);
    n_avg = n_avg + (1 - n_avg % 2);
    int n_range = (int)ceilf((180.0f / 360.0f) * (float)n_proj_ffs);
    n_range = n_range + (1 - n_range % 2);
    avg_reach = n_avg / 2;
    range_reach = n_range / 2;
}

int AfStream::advance(const struct recon_metadata &mr, const float *d_in, float *d_out, float *d_scratch,
                      int arrived, cudaStream_t stream)
{
    AfParams p;
    CTBB_TRY(af_params(mr, d_in, d_out, d_scratch, &p));
    arrived = std::min(arrived, P);
    bool all = arrived == P;
    // a moving mean needs the maxima up to avg_reach frames ahead, the
    // eccentricity and threshold the means up to range_reach ahead, the
    // smoothing the thresholds and raw frames of +-2 frames
    int smoothed = all ? P : std::max(0, arrived - avg_reach);
    int finished = all ? P : std::max(0, std::min(smoothed - range_reach, arrived - 2));
    smoothed = std::max(smoothed, n_smoothed);
    finished = std::max(finished, n_filtered);
    CTBB_TRY(af_launch(p, n_sup, arrived, n_smoothed, smoothed, n_filtered, finished, stream));
    n_sup = std::max(n_sup, arrived);
    n_smoothed = smoothed;
    n_filtered = finished;
    return CTBB_OK;
}

}  // namespace ctbb

// --------------------------------------------------------------------------
// Adaptive filter without any allocation
// --------------------------------------------------------------------------
//
// For callers that must not allocate device memory while a scan is being
// processed -- a scanner-side service that reserves all device memory at
// start-up and keeps cudaMalloc (which can synchronise the whole device and
// has unbounded latency) out of its per-scan path, or a host process whose
// device memory belongs to another allocator (a framework's caching pool, a
// fixed MPS/MIG quota) -- this variant takes its per-frame statistics from a
// fixed array in the library's static device memory instead of the library's
// allocated workspace.  The caller still passes the input and output buffers.

namespace ctbb {

// Largest pull window (frames) the static scratch holds; config-3 blocks pull
// 8448 frames and config-2 blocks 11264.
constexpr size_t kNoAllocMaxFrames = 65536;

// 6 statistics per frame (sup, smooth, ecc, max, min, threshold): 1.5 MiB.
// Every GPU that loads the library holds this array until the process exits.
static __device__ __align__(256) float g_af_noalloc_scratch[6 * kNoAllocMaxFrames];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
float *g_noalloc_ptr[kMaxDevices] = {nullptr};

// Device address of the static scratch on the current device.  In host code
// the array's name is only a host-side stand-in, so the address is looked up
// once per device (with that device current) and cached.
int noalloc_scratch(float **out)
{
    int dev = 0;
    CTBB_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("adaptive filter (no allocation): device %d beyond %d", dev, kMaxDevices);
        return CTBB_ERR_ARGUMENT;
    }
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        CTBB_CUDA_TRY(cudaGetSymbolAddress(&p, g_af_noalloc_scratch));
        g_noalloc_ptr[dev] = static_cast<float *>(p);
    }
    *out = g_noalloc_ptr[dev];
    return CTBB_OK;
}

}  // namespace
}  // namespace ctbb

extern "C" int ctbb_adaptive_filter_device_noalloc(const struct recon_metadata *mr, const float *d_in,
                                                   float *d_out)
{
    using namespace ctbb;
    clear_error();
    if (!mr || !d_in || !d_out) {
        set_error("ctbb_adaptive_filter_device_noalloc: null argument");
        return CTBB_ERR_ARGUMENT;
    }
    if (mr->ri.n_proj_pull == 0 || mr->cg.n_channels == 0 || mr->cg.n_rows_raw == 0) {
        set_error("ctbb_adaptive_filter_device_noalloc: recon_metadata is not planned");
        return CTBB_ERR_STATE;
    }
    if (mr->ri.n_proj_pull > kNoAllocMaxFrames) {
        set_error("ctbb_adaptive_filter_device_noalloc: pull window of %zu frames exceeds the "
                  "fixed scratch of %zu frames; use ctbb_adaptive_filter_device",
                  mr->ri.n_proj_pull, kNoAllocMaxFrames);
        return CTBB_ERR_ARGUMENT;
    }
    CTBB_TRY(require_device());
    float *scratch = nullptr;
    CTBB_TRY(noalloc_scratch(&scratch));
    // Every statistic is written for all frames before it is read, so the
    // previous call's contents need no clearing.
    return run_adaptive_filter_with(*mr, d_in, d_out, scratch);
}
