// ramp_tc.cu -- ramp filter as a Toeplitz contraction on the tensor cores,
// with FP16 output rows and a per-row scale (the reduced-storage path).
//
// The reference filters every rebinned row of n = n_channels_oversampled
// samples by the linear convolution y[l] = sum_k f[n + l - k] x[k] with the
// 2n taps f (GPU: `filter`, include/rebin_filter.cuh:369-409, taps in
// constant memory at :33; CPU: filter_cpu, src/rebin_filter_cpu.cu:647-709,
// the same sum through a zero-padded double FFT).  That sum is a product of
// the rows X [rows][n] with the Toeplitz matrix T[k][l] = f[n + l - k]:
// Y = X T.  Here it runs as one GEMM per launch on the 5th-generation tensor
// cores:
//
//   * precision: X and T are split into 16-bit hi + lo pairs, x = x_hi + x_lo
//     with x_hi = h(x), x_lo = h(x - x_hi), and Y = X_hi T_hi + X_hi T_lo +
//     X_lo T_hi, accumulated in FP32 in tensor memory.  The halves are FP16
//     (11 significant bits each, 22 together), not BF16 (8 + 8): the ramp
//     filter's output is a near-cancellation of terms as large as f[n] x, and
//     with BF16 halves the residual of x times that centre tap alone left 3e-4
//     of the row maximum (CPU emulation with exact accumulation: 4.9e-5
//     absolute on 0.15-maximum rows, against 8e-7 with FP16 halves at the
//     same tensor-core rate).  FP16's exponent range is narrower (5 bits
//     against 8), so X is scaled per row (per view) by a power of two to a
//     maximum of 2^13-2^14 and T by 2^10 (its far taps stay normal); both
//     scales are exact and undone in the epilogue;
//   * tiles: a CTA owns 128 rows x 256 output samples (TMEM 128 lanes x 256
//     FP32 columns); the K loop runs over 64-sample slices of the row (23 for
//     n = 1472), each one stage of a 2-stage shared-memory ring holding
//     X_hi, X_lo (128 x 64) and T_hi, T_lo (256 x 64), all FP16, loaded by
//     TMA (cp.async.bulk.tensor) with the 128-byte swizzle the MMA
//     descriptors name; one thread issues 3 x 4 tcgen05.mma (M128 N256 K16)
//     per stage and tcgen05.commit frees the stage;
//   * epilogue: the four warps read their 32 TMEM lanes (tcgen05.ld), undo
//     the input scales, scale each row by 2^-e_row and store FP16.  The
//     exponent comes from the row's input: |y| <= max|x| sum|f|, and 2^e_row is
//     the smallest power of two putting that bound below 2^14, so no row
//     overflows FP16 and the scale is exact; the backprojector multiplies by
//     2^e_row again.
//
// The split of X and the row exponents are one pass before the GEMM
// (ramp_tc_split_kernel).  T (both halves, padded to 1536 output samples) is
// made on the host once per tap set.  Every mbarrier wait is bounded: a wait
// that runs out records an error code in device memory, the CTA stops
// issuing work, frees its tensor memory and returns; the host reads the code.
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "ctbb_internal.h"
#include "cuda_util.cuh"
#include "ramp_tc.h"

namespace ctbb {

namespace {

constexpr int BM = 128;            // rows per CTA (TMEM lanes)
constexpr int BN = 256;            // output samples per CTA (TMEM columns)
constexpr int BK = 64;             // samples of the row per stage (128 bytes of FP16)
constexpr int kStages = 2;
constexpr int kTileA = BM * BK * 2;  // bytes of one A tile (16 KiB)
constexpr int kTileB = BN * BK * 2;  // bytes of one B tile (32 KiB)
constexpr int kStageBytes = 2 * kTileA + 2 * kTileB;
constexpr int kSmemBytes = kStages * kStageBytes + 1024 /* alignment */ + 256 /* barriers */;
constexpr int kNPad = 1536;          // T padded to a whole number of 256-sample tiles
constexpr uint32_t kWaitLimit = 1u << 30;
constexpr uint64_t kWaitNs = 2000000000ull;  // 2 s

// ---- PTX wrappers --------------------------------------------------------

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait for the phase with the given parity: false once kWaitNs of
// wall time (or kWaitLimit polls) have passed without it, or as soon as
// another CTA has recorded a wait that ran out (*error non-zero), so that one
// failure ends the launch in one wait's time, not one per CTA.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, const int *error)
{
    uint32_t addr = smem_u32(bar);
    uint64_t t0 = 0;
    for (uint32_t it = 0; it < kWaitLimit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(addr), "r"(parity)
            : "memory");
        if (done) return true;
        if ((it & 255) == 0) {
            if (*reinterpret_cast<const volatile int *>(error)) return false;
            const uint64_t t = global_ns();
            if (it == 0) t0 = t;
            else if (t - t0 > kWaitNs) return false;
        }
    }
    return false;
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// Shared-memory matrix descriptor of a K-major 16-bit tile whose rows are 128
// bytes with the 128-byte swizzle (what TMA writes with SWIZZLE_128B): start
// address, stride of 8-row groups 1024 bytes, descriptor version 1, layout 2.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFF) >> 4);          // start address
    d |= (uint64_t)(16 >> 4) << 16;                   // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;                 // stride byte offset: 8 rows x 128 B
    d |= (uint64_t)1 << 46;                           // descriptor version
    d |= (uint64_t)2 << 61;                           // 128-byte swizzle
    return d;
}

// Instruction descriptor of kind::f16: D FP32, A and B FP16, both K-major,
// N = 256, M = 128.
constexpr uint32_t kIdesc = (1u << 4) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
constexpr int kTapExp = 10;  // T is stored times 2^10

__device__ __forceinline__ void umma(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
        "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate));
}

__device__ __forceinline__ void umma_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32])
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// ---- the split of X: FP16 hi / lo planes and the row exponents -------------

// Exponents of a row (or view) of largest |x| m: the input's, e_in with
// m 2^-e_in in [2^13, 2^14), and the stored output's, e_out, the smallest
// with m sum|f| 2^-e_out <= 2^14 (FP16 holds up to 65504).
__device__ __forceinline__ void row_exponents(float m, float sum_abs_taps, int *e_in, int *e_out)
{
    *e_in = 0;
    *e_out = 0;
    if (m > 0.0f && isfinite(m)) {
        int ex;
        frexpf(m, &ex);          // m = f 2^ex, f in [0.5, 1)
        *e_in = ex - 14;         // m 2^-e_in in [2^13, 2^14)
        float bound = m * sum_abs_taps;
        if (bound > 0.0f && isfinite(bound)) {
            frexpf(bound / 16384.0f, &ex);
            *e_out = ex;
        }
    }
    *e_in = max(-120, min(120, *e_in));
    *e_out = max(-120, min(120, *e_out));
}

// Scales of a row: scale = 2^e_out (what the backprojector multiplies by) and
// the epilogue's factor 2^(e_in - 10 - e_out) from the accumulator to the
// stored value.
__device__ __forceinline__ void write_row(const float *__restrict__ xr, int n, int lane, int e_in, int e_out,
                                          __half *__restrict__ hr, __half *__restrict__ lr, float *scale,
                                          float *mult)
{
    if (lane == 0) {
        *scale = ldexpf(1.0f, e_out);
        *mult = ldexpf(1.0f, e_in - kTapExp - e_out);
    }
    const float s = ldexpf(1.0f, -e_in);
    for (int i = lane; i < n; i += 32) {
        float v = xr[i] * s;  // exact: a power of two
        __half h = __float2half_rn(v);
        hr[i] = h;
        lr[i] = __float2half_rn(v - __half2float(h));
    }
}

// One warp per row: max |x|, its exponents, then x_hi, x_lo.
__global__ void __launch_bounds__(256) ramp_tc_split_kernel(const float *__restrict__ x, size_t n_lines, int n,
                                                            float sum_abs_taps, __half *__restrict__ hi,
                                                            __half *__restrict__ lo, float *__restrict__ scale,
                                                            float *__restrict__ mult)
{
    const int lane = threadIdx.x & 31;
    size_t warp = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5;
    const size_t warps = ((size_t)gridDim.x * blockDim.x) >> 5;
    for (size_t row = warp; row < n_lines; row += warps) {
        const float *xr = x + row * (size_t)n;
        float m = 0.0f;
        for (int i = lane; i < n; i += 32) m = fmaxf(m, fabsf(xr[i]));
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        int e_in, e_out;
        row_exponents(m, sum_abs_taps, &e_in, &e_out);
        write_row(xr, n, lane, e_in, e_out, hi + row * (size_t)n, lo + row * (size_t)n, scale + row, mult + row);
    }
}

// The same split with one exponent per view: a CTA per view of rpv rows (8
// warps), the exponent from the largest |x| of all its rows.
__global__ void __launch_bounds__(256) ramp_tc_split_view_kernel(const float *__restrict__ x, size_t n_lines, int n,
                                                                 int rpv, float sum_abs_taps, __half *__restrict__ hi,
                                                                 __half *__restrict__ lo, float *__restrict__ scale,
                                                                 float *__restrict__ mult)
{
    __shared__ float red[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (size_t g0 = (size_t)blockIdx.x * rpv; g0 < n_lines; g0 += (size_t)gridDim.x * rpv) {
        const size_t g1 = g0 + rpv < n_lines ? g0 + rpv : n_lines;
        float m = 0.0f;
        for (size_t row = g0 + warp; row < g1; row += 8) {
            const float *xr = x + row * (size_t)n;
            for (int i = lane; i < n; i += 32) m = fmaxf(m, fabsf(xr[i]));
        }
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0) red[warp] = m;
        __syncthreads();
        m = red[0];
        for (int w = 1; w < 8; ++w) m = fmaxf(m, red[w]);
        __syncthreads();
        int e_in, e_out;
        row_exponents(m, sum_abs_taps, &e_in, &e_out);
        for (size_t row = g0 + warp; row < g1; row += 8)
            write_row(x + row * (size_t)n, n, lane, e_in, e_out, hi + row * (size_t)n, lo + row * (size_t)n,
                      scale + row, mult + row);
    }
}

// ---- the GEMM ----------------------------------------------------------------

struct TcParams {
    size_t n_lines;               // rows of X (M)
    int n;                        // row length (K and the valid output samples)
    const float *mult;            // [n_lines]: accumulator -> stored value
    __half *out;                  // [n_lines][n] (plain) or [n_lines][n][4] (footprint quads)
    int *error;                   // non-zero: a bounded wait ran out
    int rows_per_view;            // footprint quads: detector rows of a view (divides BM)
};

// Output samples a CTA stores: plain rows all BN it computes; footprint quads
// (sample c with c + 1 and the next row) one less, the last column serving as
// c + 1 of the one before it.
template <bool QUAD>
__host__ __device__ constexpr int tile_step() { return QUAD ? BN - 1 : BN; }

template <bool QUAD>
__global__ void __launch_bounds__(128, 1) ramp_tc_gemm_kernel(const __grid_constant__ CUtensorMap map_xh,
                                                              const __grid_constant__ CUtensorMap map_xl,
                                                              const __grid_constant__ CUtensorMap map_th,
                                                              const __grid_constant__ CUtensorMap map_tl,
                                                              TcParams p)
{
    extern __shared__ uint8_t smem_raw[];
    // 1024-byte aligned stages (the 128-byte swizzle repeats every 8 rows)
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + kStages * kStageBytes);
    uint64_t *empty = full + kStages;
    uint64_t *done = empty + kStages;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);

    // a wait of another CTA ran out: this launch's result is void already
    // (read once, so that the whole CTA leaves together)
    __shared__ int s_void;
    if (threadIdx.x == 0) s_void = *reinterpret_cast<const volatile int *>(p.error);
    __syncthreads();
    if (s_void) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n_tile = blockIdx.x;               // 256-sample slice of the output
    const size_t m0 = (size_t)blockIdx.y * BM;   // first row
    const int k_tiles = p.n / BK;
    // K order: the slices of the row farthest from this tile's outputs first.
    // Near the diagonal the taps are large (the centre tap and its odd
    // neighbours, which cancel it to a small output); far ones sum to about
    // 1 % of them.  With the large products last, the FP32 accumulator stays
    // small for most of its additions, where the tensor cores' accumulation
    // rounds relative to its magnitude.
    __shared__ uint8_t k_order[kNPad / BK];
    if (threadIdx.x == 0) {
        const int centre2 = 2 * (n_tile * tile_step<QUAD>() + BN / 2);  // twice the centre, in samples
        for (int i = 0; i < k_tiles; ++i) k_order[i] = (uint8_t)i;
        for (int i = 0; i < k_tiles; ++i)  // selection sort by distance, descending (k_tiles <= 24)
            for (int j = i + 1; j < k_tiles; ++j) {
                const int di = abs(2 * (k_order[i] * BK + BK / 2) - centre2);
                const int dj = abs(2 * (k_order[j] * BK + BK / 2) - centre2);
                if (dj > di) {
                    uint8_t t = k_order[i];
                    k_order[i] = k_order[j];
                    k_order[j] = t;
                }
            }
    }

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 2) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(BN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 0 && lane == 0) {
        // TMA producer
        for (int kt = 0; kt < k_tiles; ++kt) {
            const int s = kt % kStages;
            if (kt >= kStages && !mbar_wait(&empty[s], ((kt / kStages) - 1) & 1, p.error)) {
                atomicExch(p.error, 1);
                *abort_flag = 1;
                break;
            }
            if (*abort_flag) break;
            uint8_t *st = smem + s * kStageBytes;
            const int kx = k_order[kt] * BK;
            mbar_expect_tx(&full[s], kStageBytes);
            tma_load_2d(st, &map_xh, kx, (int)m0, &full[s]);
            tma_load_2d(st + kTileA, &map_xl, kx, (int)m0, &full[s]);
            tma_load_2d(st + 2 * kTileA, &map_th, kx, n_tile * tile_step<QUAD>(), &full[s]);
            tma_load_2d(st + 2 * kTileA + kTileB, &map_tl, kx, n_tile * tile_step<QUAD>(), &full[s]);
        }
    } else if (warp == 1 && lane == 0) {
        // MMA issuer
        bool ok = true;
        for (int kt = 0; kt < k_tiles; ++kt) {
            const int s = kt % kStages;
            if (!mbar_wait(&full[s], (kt / kStages) & 1, p.error)) {
                atomicExch(p.error, 2);
                *abort_flag = 1;
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t st = smem_u32(smem + s * kStageBytes);
            const uint32_t a_hi = st, a_lo = st + kTileA, b_hi = st + 2 * kTileA, b_lo = st + 2 * kTileA + kTileB;
#pragma unroll
            for (int kk = 0; kk < BK / 16; ++kk) {
                const uint32_t off = kk * 32;  // 16 FP16 along K
                const uint32_t acc0 = (kt > 0 || kk > 0) ? 1u : 0u;
                umma(tmem, sw128_desc(a_hi + off), sw128_desc(b_hi + off), acc0);
                umma(tmem, sw128_desc(a_hi + off), sw128_desc(b_lo + off), 1u);
                umma(tmem, sw128_desc(a_lo + off), sw128_desc(b_hi + off), 1u);
            }
            umma_commit(&empty[s]);  // the stage is free once these MMAs have read it
        }
        if (ok) umma_commit(done);
        else asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(done)) : "memory");
    }
    __syncwarp();

    // epilogue: every warp its 32 TMEM lanes (rows)
    const bool got = mbar_wait(done, 0, p.error);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!got && lane == 0) atomicExch(p.error, 3);
    const size_t row = m0 + (size_t)warp * 32 + lane;
    const bool row_ok = got && !*abort_flag && row < p.n_lines;
    const float inv = row_ok ? __ldg(p.mult + row) : 0.0f;
    if (QUAD) {
        // Footprint quads: the scaled FP16 tile is staged in the (now idle)
        // stage ring, then sample (r, c) is stored with (r, c + 1), (r + 1, c)
        // and (r + 1, c + 1) as one 8-byte word.  The tile's rows are whole
        // views (the rows per view divide 128), so row r + 1 of the tile's
        // last row -- the last detector row of a view, whose footprint the
        // backprojector never reads -- is stored as zeros, as is row r + 1 of
        // the last row of every view in the tile.
        constexpr int kLd = BN + 8;  // staged row stride (halves)
        __half *stage = reinterpret_cast<__half *>(smem);
        const bool ok_all = got && !*abort_flag;
        if (ok_all) {
            for (int c = 0; c < BN / 32; ++c) {
                float v[32];
                tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c * 32), v);
                __half *dst = stage + (warp * 32 + lane) * kLd + c * 32;
#pragma unroll
                for (int j = 0; j < 32; j += 2)
                    *reinterpret_cast<__half2 *>(dst + j) = __floats2half2_rn(v[j] * inv, v[j + 1] * inv);
            }
        }
        __syncthreads();
        if (ok_all) {
            const int c_base = n_tile * tile_step<true>();
            for (int r = warp; r < BM; r += 4) {
                const size_t grow = m0 + r;
                if (grow >= p.n_lines) break;
                const __half *s0 = stage + r * kLd;
                const __half *s1 = s0 + kLd;
                uint2 *dst = reinterpret_cast<uint2 *>(p.out) + grow * (size_t)p.n;
                for (int c = lane; c < tile_step<true>(); c += 32) {
                    const int col = c_base + c;
                    if (col >= p.n) break;
                    __half2 top = __halves2half2(s0[c], s0[c + 1]);
                    __half2 bot = (r + 1) % p.rows_per_view != 0 ? __halves2half2(s1[c], s1[c + 1])
                                                                  : __float2half2_rn(0.0f);
                    dst[col] = make_uint2(*reinterpret_cast<uint32_t *>(&top), *reinterpret_cast<uint32_t *>(&bot));
                }
            }
        }
    } else if (got && !*abort_flag) {
        for (int c = 0; c < BN / 32; ++c) {
            const int col0 = n_tile * BN + c * 32;
            if (col0 >= p.n) break;  // warp-uniform
            float v[32];
            tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c * 32), v);
            if (row_ok) {
                uint32_t packed[16];
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    __half2 h = __floats2half2_rn(v[2 * j] * inv, v[2 * j + 1] * inv);
                    packed[j] = *reinterpret_cast<uint32_t *>(&h);
                }
                uint4 *dst = reinterpret_cast<uint4 *>(p.out + row * (size_t)p.n + col0);
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    dst[j] = make_uint4(packed[4 * j], packed[4 * j + 1], packed[4 * j + 2], packed[4 * j + 3]);
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 2) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN));
}

// ---- host ---------------------------------------------------------------------

// IEEE binary16 of a finite float, round to nearest even (normal, subnormal
// and zero results; magnitudes at or above 65520 become infinity).
uint16_t half_bits(float f)
{
    uint32_t u;
    std::memcpy(&u, &f, 4);
    const uint32_t sign = (u >> 16) & 0x8000u;
    const float a = std::fabs(f);
    if (a >= 65520.0f) return (uint16_t)(sign | 0x7C00u);
    if (a < 6.103515625e-05f) {  // subnormal range: multiples of 2^-24
        const float q = std::nearbyint(a * 16777216.0f);  // round to nearest even (default mode)
        return (uint16_t)(sign | (uint32_t)q);
    }
    uint32_t m = u & 0x7FFFFFFFu;
    uint32_t e = (m >> 23) - 127 + 15;
    uint32_t mant = m & 0x7FFFFFu;
    uint32_t h = (e << 10) | (mant >> 13);
    const uint32_t rest = mant & 0x1FFFu;
    if (rest > 0x1000u || (rest == 0x1000u && (h & 1u))) ++h;  // carries into the exponent as it should
    return (uint16_t)(sign | h);
}

float half_value(uint16_t h)
{
    const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    const uint32_t e = (h >> 10) & 0x1Fu, mant = h & 0x3FFu;
    float v;
    if (e == 0) v = std::ldexp((float)mant, -24);
    else v = std::ldexp((float)(mant | 0x400u), (int)e - 25);
    uint32_t u;
    std::memcpy(&u, &v, 4);
    u |= sign;
    std::memcpy(&v, &u, 4);
    return v;
}

using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

int encode_fn(EncodeTiled *out)
{
    static EncodeTiled fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        CTBB_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
        if (q != cudaDriverEntryPointSuccess || !p) {
            set_error("ramp filter (tensor cores): cuTensorMapEncodeTiled not available");
            return CTBB_ERR_CUDA;
        }
        fn = reinterpret_cast<EncodeTiled>(p);
    }
    *out = fn;
    return CTBB_OK;
}

// 2-D FP16 tensor map of a row-major [rows][cols] matrix, box box_rows x 64.
int make_map(CUtensorMap *map, const void *base, size_t rows, int cols, int box_rows)
{
    EncodeTiled enc;
    CTBB_TRY(encode_fn(&enc));
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
    cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
    cuuint32_t elem[2] = {1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void *>(base), dims, strides, box, elem,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("ramp filter (tensor cores): cuTensorMapEncodeTiled failed (%d)", (int)r);
        return CTBB_ERR_CUDA;
    }
    return CTBB_OK;
}

}  // namespace

bool ramp_tc_supported(int n) { return n > 0 && n % BK == 0 && n <= kNPad; }

size_t ramp_tc_work_bytes(size_t n_lines, int n)
{
    return n_lines * (size_t)n * 2 * sizeof(uint16_t) + n_lines * 2 * sizeof(float) + 256;
}

int prepare_ramp_tc(const float *h_taps, int n, RampTcPlan *plan, cudaStream_t stream)
{
    if (!ramp_tc_supported(n)) {
        set_error("ramp filter (tensor cores): row length %d is not a multiple of %d up to %d", n, BK, kNPad);
        return CTBB_ERR_ARGUMENT;
    }
    if (plan->n == n && plan->d_t && std::memcmp(plan->taps.data(), h_taps, 2 * n * sizeof(float)) == 0)
        return CTBB_OK;
    // T^T[l][k] = 2^10 f[n + l - k] for l < n (zero rows up to 1536), split
    // into FP16 halves
    std::vector<uint16_t> th((size_t)kNPad * n, 0), tl((size_t)kNPad * n, 0);
    double sum_abs = 0.0;
    float max_abs = 0.0f;
    for (int j = 0; j < 2 * n; ++j) {
        sum_abs += std::fabs((double)h_taps[j]);
        max_abs = std::max(max_abs, std::fabs(h_taps[j]));
    }
    if (!(max_abs * 1024.0f < 60000.0f)) {
        set_error("ramp filter (tensor cores): taps up to %g do not fit FP16 after the 2^10 scale", (double)max_abs);
        return CTBB_ERR_ARGUMENT;
    }
    for (int l = 0; l < n; ++l)
        for (int k = 0; k < n; ++k) {
            float f = std::ldexp(h_taps[n + l - k], kTapExp);
            uint16_t h = half_bits(f);
            th[(size_t)l * n + k] = h;
            tl[(size_t)l * n + k] = half_bits(f - half_value(h));
        }
    if (!plan->d_t) {
        CTBB_CUDA_TRY(cudaMalloc(&plan->d_t, (size_t)2 * kNPad * kNPad * sizeof(uint16_t)));
        CTBB_CUDA_TRY(cudaMalloc(&plan->d_error, sizeof(int)));
    }
    CTBB_CUDA_TRY(cudaMemcpyAsync(plan->d_t, th.data(), th.size() * 2, cudaMemcpyHostToDevice, stream));
    CTBB_CUDA_TRY(cudaMemcpyAsync(static_cast<uint16_t *>(plan->d_t) + (size_t)kNPad * n, tl.data(), tl.size() * 2,
                                  cudaMemcpyHostToDevice, stream));
    CTBB_CUDA_TRY(cudaMemsetAsync(plan->d_error, 0, sizeof(int), stream));
    CTBB_CUDA_TRY(cudaStreamSynchronize(stream));  // the host vectors go out of scope
    plan->n = n;
    plan->taps.assign(h_taps, h_taps + 2 * n);
    plan->sum_abs_taps = (float)sum_abs;
    return CTBB_OK;
}

int launch_ramp_tc(const RampTcPlan &plan, const float *d_rows, size_t n_lines, __half *d_out, float *d_scale,
                   void *d_work, cudaStream_t stream, int rows_per_view)
{
    if (n_lines == 0) return CTBB_OK;
    const int n = plan.n;
    if (!plan.d_t || n <= 0) {
        set_error("ramp filter (tensor cores): not prepared");
        return CTBB_ERR_STATE;
    }
    if (n_lines >= ((size_t)1 << 31)) {
        set_error("ramp filter (tensor cores): %zu rows exceed the tensor map", n_lines);
        return CTBB_ERR_ARGUMENT;
    }
    __half *xh = static_cast<__half *>(d_work);
    __half *xl = xh + n_lines * (size_t)n;
    float *mult = reinterpret_cast<float *>(xl + n_lines * (size_t)n);
    if (rows_per_view > 0 && BM % rows_per_view != 0) {
        set_error("ramp filter (tensor cores): %d rows per view do not divide %d", rows_per_view, BM);
        return CTBB_ERR_ARGUMENT;
    }
    if (rows_per_view > 0) {
        int blocks = (int)std::min<size_t>((n_lines + rows_per_view - 1) / rows_per_view, (size_t)num_sms() * 8);
        ramp_tc_split_view_kernel<<<blocks, 256, 0, stream>>>(d_rows, n_lines, n, rows_per_view, plan.sum_abs_taps,
                                                              xh, xl, d_scale, mult);
    } else {
        int blocks = (int)std::min<size_t>((n_lines + 7) / 8, (size_t)num_sms() * 16);
        ramp_tc_split_kernel<<<blocks, 256, 0, stream>>>(d_rows, n_lines, n, plan.sum_abs_taps, xh, xl, d_scale,
                                                         mult);
    }
    count_launch();
    CTBB_CUDA_TRY(cudaGetLastError());
    CUtensorMap mxh, mxl, mth, mtl;
    CTBB_TRY(make_map(&mxh, xh, n_lines, n, BM));
    CTBB_TRY(make_map(&mxl, xl, n_lines, n, BM));
    const uint16_t *t = static_cast<const uint16_t *>(plan.d_t);
    CTBB_TRY(make_map(&mth, t, kNPad, n, BN));
    CTBB_TRY(make_map(&mtl, t + (size_t)kNPad * n, kNPad, n, BN));
    static bool attr = false;
    if (!attr) {
        CTBB_CUDA_TRY(cudaFuncSetAttribute(ramp_tc_gemm_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           kSmemBytes));
        CTBB_CUDA_TRY(cudaFuncSetAttribute(ramp_tc_gemm_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           kSmemBytes));
        attr = true;
    }
    const bool quad = rows_per_view > 0;
    TcParams p;
    p.n_lines = n_lines;
    p.n = n;
    p.mult = mult;
    p.out = d_out;
    p.error = plan.d_error;
    p.rows_per_view = rows_per_view > 0 ? rows_per_view : BM;
    const int step = quad ? tile_step<true>() : tile_step<false>();
    dim3 grid((n + step - 1) / step, (unsigned)((n_lines + BM - 1) / BM));
    if ((grid.x - 1) * step + BN > kNPad) {
        set_error("ramp filter (tensor cores): row length %d beyond the padded kernel", n);
        return CTBB_ERR_ARGUMENT;
    }
    if (quad) ramp_tc_gemm_kernel<true><<<grid, 128, kSmemBytes, stream>>>(mxh, mxl, mth, mtl, p);
    else ramp_tc_gemm_kernel<false><<<grid, 128, kSmemBytes, stream>>>(mxh, mxl, mth, mtl, p);
    count_launch();
    CTBB_CUDA_TRY(cudaGetLastError());
    return CTBB_OK;
}

int ramp_tc_check(const RampTcPlan &plan, cudaStream_t stream)
{
    int err = 0;
    CTBB_CUDA_TRY(cudaMemcpyAsync(&err, plan.d_error, sizeof(int), cudaMemcpyDeviceToHost, stream));
    CTBB_CUDA_TRY(cudaStreamSynchronize(stream));
    if (err) {
        set_error("ramp filter (tensor cores): a pipeline wait ran out (stage %d)", err);
        return CTBB_ERR_CUDA;
    }
    return CTBB_OK;
}

void release_ramp_tc(RampTcPlan *plan)
{
    if (plan->d_t) cudaFree(plan->d_t);
    if (plan->d_error) cudaFree(plan->d_error);
    *plan = RampTcPlan{};
}

}  // namespace ctbb
