// ramp_filter.cu -- reconstruction-kernel convolution of rebinned rows.
//
// Computes, for every row x of length N (= n_channels_oversampled), the linear
// convolution y[l] = sum_{k<N} f[N + l - k] x[k] with the 2N-tap kernel f
// (centre tap at index N), which is what the reference's filter_cpu
// (src/rebin_filter_cpu.cu:647-709) evaluates through a zero-padded double FFT of
// size M = 2 * 2^ceil(log2 N), and what its GPU filter kernel
// (include/rebin_filter.cuh:369-409) evaluates as a direct sum.
//
// GB300 design: FP32 FFT convolution in shared memory.  Two real rows are
// packed into one complex row (x_a + i x_b); because the kernel is real the
// real and imaginary parts of the inverse transform are the two filtered rows.
// CTAs are persistent and loop over row pairs.  For M = 4096 (row lengths
// 1025..2048, every built-in scanner) ramp_fft4096_kernel runs 16 x 16 x 16
// radix-16 passes: thread j owns butterfly j of every pass, the first forward
// pass reads the rows from HBM (inputs >= M/2 are the zero padding), the last
// forward pass, the spectrum multiply and the first inverse pass stay in
// registers, and the last inverse pass writes HBM -- four shared-memory round
// trips per pair, indices padded by one element per 16 (conflict-free), pass
// twiddles from [r][k] tables, 16-point DFTs as 4 x 4 with the complex adds as
// packed FP32.  Other M take ramp_fft_kernel (radix 16 Stockham passes, one
// radix-2/4/8 pass first when log2 M is not a multiple of 4).  HBM traffic is
// one read and one write of the rows.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <utility>
#include <vector>

#include "ctbb_internal.h"
#include "cuda_util.cuh"
#include "ramp_filter.h"

namespace ctbb {

namespace {

constexpr int kFftThreads = 256;

// Host double-precision radix-2 DFT (bit reversal + butterflies), used once per
// kernel to compute its spectrum.  data: n interleaved complex values.
void ctbb_fft_radix2_double(double *data, int n, int sign)
{
    for (int i = 1, j = 0; i < n; ++i) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) {
            std::swap(data[2 * i], data[2 * j]);
            std::swap(data[2 * i + 1], data[2 * j + 1]);
        }
    }
    const double two_pi = 6.283185307179586476925286766559;
    for (int len = 2; len <= n; len <<= 1) {
        int half = len >> 1;
        for (int k = 0; k < half; ++k) {
            double ang = sign * two_pi * (double)k / (double)len;
            double wr = std::cos(ang), wi = std::sin(ang);
            for (int s = 0; s < n; s += len) {
                int a = s + k, b = a + half;
                double br = data[2 * b] * wr - data[2 * b + 1] * wi;
                double bi = data[2 * b] * wi + data[2 * b + 1] * wr;
                data[2 * b] = data[2 * a] - br;
                data[2 * b + 1] = data[2 * a + 1] - bi;
                data[2 * a] += br;
                data[2 * a + 1] += bi;
            }
        }
    }
}

struct FftParams {
    float *lines;        // [n_lines][n]
    size_t n_lines;
    int n;               // row length
    int m;               // transform size (power of two)
    int log2m;
    const float2 *spectrum;  // H[k] / M, [m]
};

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// Shared-memory index with one float2 of padding per 16.  64-bit accesses are
// served per half-warp; with this padding the 16 lanes of every load and
// store of every Stockham pass (radix 2..16, any power-of-two size up to the
// maximum) fall on 16 distinct bank pairs.
__device__ __forceinline__ int pad(int e) { return e + (e >> 4); }

// R-point DFT in registers, V[m] = sum_r v[r] exp(sign 2 pi i r m / R), R a
// power of two <= 16: radix-2 decimation in time over bit-reversed inputs with
// compile-time twiddles.
template <int R>
__device__ __forceinline__ void dft_registers(float2 (&v)[R], int sign)
{
    // bit-reversal permutation
#pragma unroll
    for (int i = 0; i < R; ++i) {
        int j = 0;
#pragma unroll
        for (int b = 1, t = i; b < R; b <<= 1, t >>= 1) j = (j << 1) | (t & 1);
        if (j > i) {
            float2 tmp = v[i];
            v[i] = v[j];
            v[j] = tmp;
        }
    }
    // exp(-2 pi i k / 16), k = 0..7
    const float c16[8] = {1.0f, 0.92387953251128674f, 0.70710678118654752f, 0.38268343236508977f,
                          0.0f, -0.38268343236508977f, -0.70710678118654752f, -0.92387953251128674f};
    const float s16[8] = {0.0f, -0.38268343236508977f, -0.70710678118654752f, -0.92387953251128674f,
                          -1.0f, -0.92387953251128674f, -0.70710678118654752f, -0.38268343236508977f};
#pragma unroll
    for (int half = 1; half < R; half <<= 1) {
#pragma unroll
        for (int k = 0; k < half; ++k) {
            int idx = k * (16 / (2 * half));  // exponent in units of 2 pi / 16
            float wr = c16[idx], wi = sign < 0 ? s16[idx] : -s16[idx];
#pragma unroll
            for (int j = k; j < R; j += 2 * half) {
                float2 a = v[j];
                float2 b = v[j + half];
                if (idx != 0) b = make_float2(b.x * wr - b.y * wi, b.x * wi + b.y * wr);
                v[j] = make_float2(a.x + b.x, a.y + b.y);
                v[j + half] = make_float2(a.x - b.x, a.y - b.y);
            }
        }
    }
}

// One Stockham pass of radix R over m points, src -> dst (padded indices).
// tw[t] = exp(-2 pi i t / m); the inverse uses the conjugate.  pre_mul (the
// kernel spectrum) multiplies the inputs of the first inverse pass.
template <int R>
struct Log2;
template <> struct Log2<2> { static constexpr int v = 1; };
template <> struct Log2<4> { static constexpr int v = 2; };
template <> struct Log2<8> { static constexpr int v = 3; };
template <> struct Log2<16> { static constexpr int v = 4; };

// One Stockham pass of radix R over m = 2^log2m points, src -> dst (padded
// indices); ns = 2^log2ns is the size of the sub-transforms already done.
// All index arithmetic is shifts and masks.  tw[t] = exp(-2 pi i t / m); the
// inverse uses the conjugate.  pre_mul (the kernel spectrum) multiplies the
// inputs of the first inverse pass.
template <int R>
__device__ __forceinline__ void stockham_pass(const float2 *__restrict__ src, float2 *__restrict__ dst,
                                              const float2 *__restrict__ tw, int log2m, int log2ns, int sign,
                                              const float2 *__restrict__ pre_mul)
{
    constexpr int lr = Log2<R>::v;
    const int nb = 1 << (log2m - lr);
    const int log2t = log2m - log2ns - lr;  // twiddle stride m / (ns R)
    const int ns_mask = (1 << log2ns) - 1;
    for (int j = threadIdx.x; j < nb; j += blockDim.x) {
        int k = j & ns_mask;
        float2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            v[r] = src[pad(j + r * nb)];
            if (pre_mul) v[r] = cmul(v[r], __ldg(pre_mul + j + r * nb));
        }
        if (k != 0) {
            // twiddles w^r, w = exp(sign 2 pi i k tstride / m): w, w^2, w^4, w^8 are
            // read from the table, the others formed by at most two products
            float2 wp[R];
            wp[0] = make_float2(1.0f, 0.0f);
#pragma unroll
            for (int b = 1; b < R; b <<= 1) {
                float2 w = __ldg(tw + ((b * k) << log2t));
                if (sign > 0) w.y = -w.y;
                wp[b] = w;
            }
#pragma unroll
            for (int r = 3; r < R; ++r) {
                if ((r & (r - 1)) == 0) continue;
                int hi = 1;
                while ((hi << 1) <= r) hi <<= 1;
                wp[r] = cmul(wp[hi], wp[r - hi]);
            }
#pragma unroll
            for (int r = 1; r < R; ++r) v[r] = cmul(v[r], wp[r]);
        }
        dft_registers<R>(v, sign);
        int base = ((j >> log2ns) << (log2ns + lr)) + k;
#pragma unroll
        for (int r = 0; r < R; ++r) dst[pad(base + (r << log2ns))] = v[r];
    }
}

// Full transform (radix 16 passes, one radix 2/4/8 pass first when log2 m is
// not a multiple of 4); returns the buffer holding the result.
__device__ float2 *fft_smem(float2 *a, float2 *b, const float2 *tw, int m, int log2m, int sign,
                            const float2 *pre_mul)
{
    int log2ns = 0;
    int rem = log2m & 3;
    if (rem) {
        if (rem == 1) stockham_pass<2>(a, b, tw, log2m, log2ns, sign, pre_mul);
        else if (rem == 2) stockham_pass<4>(a, b, tw, log2m, log2ns, sign, pre_mul);
        else stockham_pass<8>(a, b, tw, log2m, log2ns, sign, pre_mul);
        __syncthreads();
        float2 *t = a; a = b; b = t;
        log2ns += rem;
        pre_mul = nullptr;
    }
    while (log2ns < log2m) {
        stockham_pass<16>(a, b, tw, log2m, log2ns, sign, pre_mul);
        __syncthreads();
        float2 *t = a; a = b; b = t;
        log2ns += 4;
        pre_mul = nullptr;
    }
    (void)m;
    return a;
}

// ---- 4096-point transforms (16 x 16 x 16): the size every row length in
// 1025..2048 uses.  Thread j of 256 owns butterfly j of each pass; the three
// forward passes read inputs j + 256 r (r = 0..15), so the last forward pass
// leaves X[j + 256 r] in thread j's registers -- exactly the inputs of the first
// inverse pass.  Spectrum multiply and that pass run in registers; the first
// forward pass reads the rows from global memory (inputs r >= 8 are the zero
// padding, since N <= M / 2) and the last inverse pass writes them back.
constexpr int kM4096 = 4096;
constexpr int kTw16Entries = 15 * 16 + 15 * 256;  // pass-2 and pass-3 twiddles

// z * w for sign < 0, z * conj(w) for sign > 0
template <int SIGN>
__device__ __forceinline__ float2 twiddle(float2 z, float2 w)
{
    if (SIGN < 0) return make_float2(fmaf(z.x, w.x, -z.y * w.y), fmaf(z.x, w.y, z.y * w.x));
    return make_float2(fmaf(z.x, w.x, z.y * w.y), fmaf(z.y, w.x, -z.x * w.y));
}

// omega4 * z with omega4 = exp(SIGN 2 pi i / 4) = SIGN i
template <int SIGN>
__device__ __forceinline__ float2 mul_omega4(float2 z)
{
    return SIGN < 0 ? make_float2(z.y, -z.x) : make_float2(-z.y, z.x);
}

// Complex add / subtract as packed FP32 pairs (sm_100 family: one
// instruction for the real and imaginary parts).
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }

// In-place 4-point DFT of (a, b, c, d), outputs in natural order.
template <int SIGN>
__device__ __forceinline__ void dft4(float2 &a, float2 &b, float2 &c, float2 &d)
{
    float2 s0 = cadd(a, c), d0 = csub(a, c);
    float2 s1 = cadd(b, d), d1 = mul_omega4<SIGN>(csub(b, d));
    a = cadd(s0, s1);
    c = csub(s0, s1);
    b = cadd(d0, d1);
    d = csub(d0, d1);
}

// z * exp(SIGN 2 pi i e / 16) for the internal twiddles of the 4 x 4 split
template <int SIGN, int E>
__device__ __forceinline__ float2 w16(float2 z)
{
    constexpr float c1 = 0.92387953251128674f, s1 = 0.38268343236508977f, h = 0.70710678118654752f;
    constexpr float sg = SIGN < 0 ? -1.0f : 1.0f;
    if (E == 0) return z;
    if (E == 4) return mul_omega4<SIGN>(z);
    if (E == 2) return make_float2(h * (z.x - sg * z.y), h * (z.y + sg * z.x));
    if (E == 6) return make_float2(-h * (z.x + sg * z.y), h * (sg * z.x - z.y));
    // general: cos(2 pi E / 16), sin
    constexpr float c = E == 1 ? c1 : E == 3 ? s1 : E == 9 ? -c1 : 0.0f;
    constexpr float sn = sg * (E == 1 ? s1 : E == 3 ? c1 : E == 9 ? -s1 : 0.0f);
    return make_float2(fmaf(z.x, c, -z.y * sn), fmaf(z.x, sn, z.y * c));
}

// 16-point DFT in registers, V[k] = sum_n v[n] exp(SIGN 2 pi i n k / 16), as
// 4 x 4: n = 4 n1 + n2, k = k1 + 4 k2.  HALF: inputs 8..15 are zero.
template <int SIGN, bool HALF>
__device__ __forceinline__ void dft16(float2 (&v)[16])
{
    // DFT4 over n1 for each n2: elements n2, n2 + 4, n2 + 8, n2 + 12 -> k1
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) {
        if (HALF) {
            float2 a = v[n2], b = v[n2 + 4];
            float2 wb = mul_omega4<SIGN>(b);
            v[n2] = cadd(a, b);
            v[n2 + 4] = cadd(a, wb);
            v[n2 + 8] = csub(a, b);
            v[n2 + 12] = csub(a, wb);
        } else {
            dft4<SIGN>(v[n2], v[n2 + 4], v[n2 + 8], v[n2 + 12]);
        }
    }
    // twiddles exp(SIGN 2 pi i n2 k1 / 16); element (n2, k1) sits at n2 + 4 k1
    v[1 + 4 * 1] = w16<SIGN, 1>(v[1 + 4 * 1]);
    v[1 + 4 * 2] = w16<SIGN, 2>(v[1 + 4 * 2]);
    v[1 + 4 * 3] = w16<SIGN, 3>(v[1 + 4 * 3]);
    v[2 + 4 * 1] = w16<SIGN, 2>(v[2 + 4 * 1]);
    v[2 + 4 * 2] = w16<SIGN, 4>(v[2 + 4 * 2]);
    v[2 + 4 * 3] = w16<SIGN, 6>(v[2 + 4 * 3]);
    v[3 + 4 * 1] = w16<SIGN, 3>(v[3 + 4 * 1]);
    v[3 + 4 * 2] = w16<SIGN, 6>(v[3 + 4 * 2]);
    v[3 + 4 * 3] = w16<SIGN, 9>(v[3 + 4 * 3]);
    // DFT4 over n2 for each k1: elements 4 k1 .. 4 k1 + 3 -> k2
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) dft4<SIGN>(v[4 * k1], v[4 * k1 + 1], v[4 * k1 + 2], v[4 * k1 + 3]);
    // element (k1, k2) now sits at 4 k1 + k2; output k = k1 + 4 k2
    float2 t[16];
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
        for (int k2 = 0; k2 < 4; ++k2) t[k1 + 4 * k2] = v[4 * k1 + k2];
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = t[k];
}

// Twiddles of a pass: v[r] *= w^(r k) (conjugated for the inverse) from a
// table laid out [r - 1][k] so that a warp reads consecutive k.
template <int SIGN, int NK>
__device__ __forceinline__ void apply_twiddles(float2 (&v)[16], const float2 *__restrict__ tab, int k)
{
#pragma unroll
    for (int r = 1; r < 16; ++r) v[r] = twiddle<SIGN>(v[r], __ldg(tab + (r - 1) * NK + k));
}

template <int MIN_BLOCKS>
__global__ void __launch_bounds__(kFftThreads, MIN_BLOCKS)
    ramp_fft4096_kernel(FftParams p, const float2 *__restrict__ tw2, const float2 *__restrict__ tw3)
{
    extern __shared__ float2 smem[];
    float2 *buf_a = smem;
    float2 *buf_b = smem + pad(kM4096 - 1) + 1;
    const int j = threadIdx.x;
    const int k2 = j & 15;                         // pass-2 sub-transform index
    const int out2 = ((j >> 4) << 8) + k2;         // pass-2 output base
    // padded shared-memory offsets as base + compile-time stride:
    // pad(j + 256 r) = rd + 272 r, pad(16 j + r) = wr1 + r, pad(out2 + 16 r) = wr2 + 17 r
    const int rd = j + (j >> 4);
    const int wr1 = 17 * j;
    const int wr2 = out2 + (out2 >> 4);
    size_t n_pairs = (p.n_lines + 1) / 2;
    for (size_t pair = blockIdx.x; pair < n_pairs; pair += gridDim.x) {
        size_t la = 2 * pair, lb = la + 1;
        bool has_b = lb < p.n_lines;
        const float *ra = p.lines + la * (size_t)p.n;
        const float *rb = p.lines + lb * (size_t)p.n;
        float2 v[16];
        // forward pass 1 (sub-transforms of size 1: no twiddles), from global
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            int idx = j + 256 * r;
            float xa = 0.0f, xb = 0.0f;
            if (idx < p.n) {
                xa = __ldg(ra + idx);
                if (has_b) xb = __ldg(rb + idx);
            }
            v[r] = make_float2(xa, xb);
        }
#pragma unroll
        for (int r = 8; r < 16; ++r) v[r] = make_float2(0.0f, 0.0f);
        dft16<-1, true>(v);
#pragma unroll
        for (int r = 0; r < 16; ++r) buf_a[wr1 + r] = v[r];
        __syncthreads();
        // forward pass 2 (size-16 sub-transforms)
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = buf_a[rd + 272 * r];
        apply_twiddles<-1, 16>(v, tw2, k2);
        dft16<-1, false>(v);
#pragma unroll
        for (int r = 0; r < 16; ++r) buf_b[wr2 + 17 * r] = v[r];
        __syncthreads();
        // forward pass 3 (size-256 sub-transforms): X[j + 256 r]
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = buf_b[rd + 272 * r];
        apply_twiddles<-1, 256>(v, tw3, j);
        dft16<-1, false>(v);
        // kernel spectrum H / M, then inverse pass 1, all in registers
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = cmul(v[r], __ldg(p.spectrum + j + 256 * r));
        dft16<1, false>(v);
#pragma unroll
        for (int r = 0; r < 16; ++r) buf_a[wr1 + r] = v[r];
        __syncthreads();
        // inverse pass 2
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = buf_a[rd + 272 * r];
        apply_twiddles<1, 16>(v, tw2, k2);
        dft16<1, false>(v);
#pragma unroll
        for (int r = 0; r < 16; ++r) buf_b[wr2 + 17 * r] = v[r];
        __syncthreads();
        // inverse pass 3: y[j + 256 r], only the first N are kept (r < 8)
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = buf_b[rd + 272 * r];
        apply_twiddles<1, 256>(v, tw3, j);
        dft16<1, false>(v);
        float *wa = p.lines + la * (size_t)p.n;
        float *wb = p.lines + lb * (size_t)p.n;
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            int idx = j + 256 * r;
            if (idx < p.n) {
                wa[idx] = v[r].x;
                if (has_b) wb[idx] = v[r].y;
            }
        }
        // buf_a is rewritten next by pass 1 of the next pair: its last reads
        // (inverse pass 2) precede the barrier after inverse pass 2; buf_b is
        // rewritten after the barrier that follows that pass 1.
    }
}

__global__ void __launch_bounds__(kFftThreads, 3) ramp_fft_kernel(FftParams p, const float2 *__restrict__ tw)
{
    // twiddles come from the read-only cache (one table for every CTA), which
    // leaves shared memory to the two transform buffers
    extern __shared__ float2 smem[];
    const int padded = pad(p.m - 1) + 1;
    float2 *buf_a = smem;
    float2 *buf_b = buf_a + padded;
    size_t n_pairs = (p.n_lines + 1) / 2;
    for (size_t pair = blockIdx.x; pair < n_pairs; pair += gridDim.x) {
        size_t la = 2 * pair, lb = la + 1;
        bool has_b = lb < p.n_lines;
        const float *ra = p.lines + la * (size_t)p.n;
        const float *rb = p.lines + lb * (size_t)p.n;
        __syncthreads();  // previous pair's stores done before buf_a is rewritten
        for (int i = threadIdx.x; i < p.m; i += blockDim.x) {
            float xa = 0.f, xb = 0.f;
            if (i < p.n) {
                xa = ra[i];
                if (has_b) xb = rb[i];
            }
            buf_a[pad(i)] = make_float2(xa, xb);
        }
        __syncthreads();
        float2 *res = fft_smem(buf_a, buf_b, tw, p.m, p.log2m, -1, nullptr);
        float2 *other = (res == buf_a) ? buf_b : buf_a;
        res = fft_smem(res, other, tw, p.m, p.log2m, +1, p.spectrum);
        float *wa = p.lines + la * (size_t)p.n;
        float *wb = p.lines + lb * (size_t)p.n;
        for (int i = threadIdx.x; i < p.n; i += blockDim.x) {
            float2 v = res[pad(i)];
            wa[i] = v.x;
            if (has_b) wb[i] = v.y;
        }
    }
}

// 4096-point kernel: 2 or 3 CTAs per SM (0: the generic kernel)
int fft4096_mode()
{
    static int v = [] {
        const char *e = getenv("CTBB_FFT4096");
        return e ? atoi(e) : 2;
    }();
    return v;
}

}  // namespace

int ramp_transform_size(int n)
{
    int m = 1;
    while (m < n) m <<= 1;
    return 2 * m;
}

int prepare_ramp_filter(const float *h_taps, int n, RampFilterPlan *plan, cudaStream_t stream)
{
    int m = ramp_transform_size(n);
    if (m > kMaxRampTransform) {
        set_error("ramp filter: row length %d needs a %d-point transform (max %d)", n, m,
                  kMaxRampTransform);
        return CTBB_ERR_ARGUMENT;
    }
    bool same = plan->n == n && plan->taps.size() == (size_t)(2 * n) &&
                memcmp(plan->taps.data(), h_taps, sizeof(float) * 2 * (size_t)n) == 0;
    if (same && plan->d_spectrum) return CTBB_OK;
    plan->n = n;
    plan->m = m;
    plan->taps.assign(h_taps, h_taps + 2 * (size_t)n);
    // Zero-padded kernel as filter_cpu lays it out: F[i] = f[N + i] (i < N),
    // F[M - N + 1 + t] = f[t + 1] (t < N - 1); H = DFT(F) / M in double.
    std::vector<double> F(2 * (size_t)m, 0.0);
    int centre = (int)std::floor((2.0f * n - 1.0f) / 2.0f) + 1;
    for (int i = 0; i < n; ++i) F[2 * (size_t)i] = h_taps[centre + i];
    for (int i = m - n + 1; i < m; ++i) F[2 * (size_t)i] = h_taps[i - (m - n + 1) + 1];
    ctbb_fft_radix2_double(F.data(), m, -1);
    std::vector<float2> H(m), tw(m);
    for (int k = 0; k < m; ++k) H[k] = make_float2((float)(F[2 * (size_t)k] / m), (float)(F[2 * (size_t)k + 1] / m));
    const double two_pi = 6.283185307179586476925286766559;
    for (int t = 0; t < m; ++t) {
        double a = -two_pi * (double)t / (double)m;
        tw[t] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    // radix-16 tables of the 4096-point kernel, [r - 1][k]: pass 2
    // exp(-2 pi i r k / 256) (k < 16), pass 3 exp(-2 pi i r k / 4096) (k < 256)
    std::vector<float2> tw16(kTw16Entries);
    for (int r = 1; r < 16; ++r) {
        for (int k = 0; k < 16; ++k) {
            double a = -two_pi * (double)(r * k) / 256.0;
            tw16[(r - 1) * 16 + k] = make_float2((float)std::cos(a), (float)std::sin(a));
        }
        for (int k = 0; k < 256; ++k) {
            double a = -two_pi * (double)(r * k) / 4096.0;
            tw16[15 * 16 + (r - 1) * 256 + k] = make_float2((float)std::cos(a), (float)std::sin(a));
        }
    }
    size_t need = 2 * (size_t)m + kTw16Entries;
    if (!plan->d_spectrum || plan->capacity < need) {
        if (plan->d_spectrum) cudaFree(plan->d_spectrum);
        plan->d_spectrum = nullptr;
        CTBB_CUDA_TRY(cudaMalloc(&plan->d_spectrum, sizeof(float2) * need));
        plan->capacity = need;
    }
    plan->d_twiddle = plan->d_spectrum + m;
    plan->d_tw16 = plan->d_twiddle + m;
    CTBB_CUDA_TRY(cudaMemcpyAsync(plan->d_spectrum, H.data(), sizeof(float2) * m, cudaMemcpyHostToDevice, stream));
    CTBB_CUDA_TRY(cudaMemcpyAsync(plan->d_twiddle, tw.data(), sizeof(float2) * m, cudaMemcpyHostToDevice, stream));
    CTBB_CUDA_TRY(cudaMemcpyAsync(plan->d_tw16, tw16.data(), sizeof(float2) * kTw16Entries,
                                  cudaMemcpyHostToDevice, stream));
    // the host vectors die at return: make the copies complete first
    CTBB_CUDA_TRY(cudaStreamSynchronize(stream));
    return CTBB_OK;
}

int launch_ramp_filter(const RampFilterPlan &plan, float *d_lines, size_t n_lines, cudaStream_t stream)
{
    if (n_lines == 0) return CTBB_OK;
    FftParams p;
    p.lines = d_lines;
    p.n_lines = n_lines;
    p.n = plan.n;
    p.m = plan.m;
    p.log2m = 0;
    while ((1 << p.log2m) < p.m) p.log2m++;
    p.spectrum = plan.d_spectrum;
    auto padded = [](size_t m) { return m + ((m - 1) >> 4) + 1; };
    size_t smem = sizeof(float2) * 2 * padded((size_t)p.m);
    // the shared-memory limits are a per-device setting of each kernel
    static std::atomic<uint64_t> attr_devices{0};
    int dev = 0;
    CTBB_CUDA_TRY(cudaGetDevice(&dev));
    const uint64_t bit = dev < 64 ? (uint64_t)1 << dev : 0;
    if (!bit || !(attr_devices.load() & bit)) {
        size_t max_smem = sizeof(float2) * 2 * padded(kMaxRampTransform);
        CTBB_CUDA_TRY(cudaFuncSetAttribute(ramp_fft_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)max_smem));
        CTBB_CUDA_TRY(cudaFuncSetAttribute(ramp_fft4096_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)(sizeof(float2) * 2 * padded(kM4096))));
        CTBB_CUDA_TRY(cudaFuncSetAttribute(ramp_fft4096_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)(sizeof(float2) * 2 * padded(kM4096))));
        attr_devices.fetch_or(bit);
    }
    int per_sm = (int)std::max<size_t>(1, (size_t)(220 * 1024) / smem);
    if (per_sm > 4) per_sm = 4;
    size_t n_pairs = (n_lines + 1) / 2;
    int grid = (int)std::min<size_t>(n_pairs, (size_t)num_sms() * per_sm);
    int mode = fft4096_mode();
    if (p.m == kM4096 && mode == 3) {
        ramp_fft4096_kernel<3><<<grid, kFftThreads, smem, stream>>>(p, plan.d_tw16, plan.d_tw16 + 15 * 16);
    } else if (p.m == kM4096 && mode == 2) {
        grid = (int)std::min<size_t>(n_pairs, (size_t)num_sms() * std::min(per_sm, 2));
        ramp_fft4096_kernel<2><<<grid, kFftThreads, smem, stream>>>(p, plan.d_tw16, plan.d_tw16 + 15 * 16);
    } else
        ramp_fft_kernel<<<grid, kFftThreads, smem, stream>>>(p, plan.d_twiddle);
    count_launch();
    CTBB_CUDA_TRY(cudaGetLastError());
    return CTBB_OK;
}

}  // namespace ctbb
