// backproject.cu -- weighted-FBP cone-beam backprojection of one 32-slice block.
//
// Algorithm of the reference CPU backprojector (src/backproject_cpu.cu:49-154),
// the path this library must match:
//
//   for each half-turn angle i < n_proj_turn/2 and voxel (x, y, z):
//     s = sum_k interp2(view(i + k n/2); p_idx, q_idx) * W(q),  h = sum_k W(q)
//     image += (s / h) * 2 pi' / n_proj_turn   (if h != 0)
//   theta = tube_start + 2 pi' i / n_proj_turn + k pi',  p = x sin - y cos,
//   p_idx = p / (r_f fai / 2) + 2 cc,  ray = z_rot (theta - asin(p / r_f)) / (2 pi'),
//   l = sqrt(r_f^2 - p^2) - x cos - y sin,  q = (z - ray) / (l tan(theta_cone / 2)),
//   q_idx = (q + 1)/2 (R - 1) + k R,  W(q) = 1 (|q| < 0.6), cos^2 taper to |q| = 1.
//
// interp2 (src/interp.cu:29-64) returns 0 when p_idx or q_idx leaves
// [0, dim - 2]; the weight W is still added to h in that case, and this kernel
// keeps that rule.  Both borders are jumps in the result, so the quantities
// that decide them (voxel centre, p, p_idx, and near the border q_idx) are
// evaluated with the reference's float operations; the smooth parts (weights,
// interpolation) use FMA and reciprocals.  The reference's pi' = 3.1415368979f
// is used where it uses it.
//
// GB300 mapping.  Two forms share the arithmetic below.  The column form (the
// default, backproject_column_tile) gives a thread the (x, y) column over up to
// 32 slices: per angle it computes the geometry of each half turn once and
// parks it in shared memory, then runs the slices in sub-chunks of 8, each
// fetching all of a visit's footprints before it uses any (one wait on the
// gathers per visit); 128-thread CTAs of 16 x 8 columns, 8 per SM.  The slice-chunk form
// (backproject_tile; windows of more than 8 half turns) gives a thread ZPT (8)
// consecutive slices of a column, 128-thread CTAs of 32 x 4 columns.  In both
// each warp is an 8 x 4 tile of columns so that its gathers fall on few
// detector channels.  Per angle i the asin and root
// of the k = 0 view are carried to every half turn to first order in |p|
// (the reference's half turns are pi', not pi, apart), and a warp-uniform
// window limits k to the half turns whose rays can reach the chunk.  Per visited (i, k) the geometry is computed once for the chunk,
// which a warp vote classes as flat (W = 1), inner (all |q| < 1) or other
// (window edge, clamps, last-turn border); slices run in pairs with packed
// FP32 (FFMA2 / FADD2 / FMUL2); the per-angle sums s, h stay in registers and
// the image sums in shared memory.  The per-view table (theta, sin, cos and
// the ray term) is built on the host with the reference's float expressions.
// Samples are gathered through the read-only cache.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <vector>

#include "backproject.h"
#include "ctbb_internal.h"
#include "cuda_util.cuh"

namespace ctbb {

namespace {


constexpr float kQ = 0.6f;
// slices per sub-chunk: the unit of the flat / inner / other decision
constexpr int kSub = 8;

// interp2 drops a sample when q_idx > R*nht - 2, which only the last half
// turn can reach.  Its weight still counts, so the decision is a jump in the
// image; near it the reference's own float q_idx decides.  This recomputes that
// q_idx with the reference's operations and rounding (asin through double,
// i.e. correctly rounded); it runs only when the fast coordinate is within
// kBorderBand rows of the border.
__device__ __forceinline__ bool last_turn_sample_valid(const BpParams &p, float x, float y, float theta,
                                                    float s, float c, float phat, float z, int k)
{
    float asn = (float)asin((double)__fdiv_rn(phat, p.rf));
    float ray = __fdiv_rn(__fmul_rn(p.z_rot, __fsub_rn(theta, asn)), p.two_pi);
    float lhat = __fsub_rn(__fsub_rn(__fsqrt_rn(__fsub_rn(p.rf2, __fmul_rn(phat, phat))), __fmul_rn(x, c)),
                           __fmul_rn(y, s));
    float qhat = __fdiv_rn(__fsub_rn(z, ray), __fmul_rn(lhat, p.tan_cone));
    float q_idx = __fadd_rn(__fmul_rn(__fdiv_rn(__fadd_rn(qhat, 1.0f), 2.0f), (float)p.n_rows - 1.0f),
                            (float)(k * p.n_rows));
    return !(q_idx > (float)(p.n_rows * p.nht - 2)) && !(q_idx < 0.0f);
}

constexpr float kBorderBand = 1e-3f;
// inner chunks: |q| <= kInnerMax keeps every row below R-1 after rounding;
// rows kRowMargin below the last-turn border are far from its band
constexpr float kInnerMax = 0.999f;
constexpr float kRowMargin = 0.01f;
// half-turn window margin (angle rounding is ~1e-6 half turns)
constexpr float kWindowMargin = 0.01f;

// p_idx = p / (r_f fai / 2) + 2 cc as the reference rounds it (division, then
// add), used where the interp2 border decision is close.
__device__ __forceinline__ float p_index_exact(const BpParams &p, float phat)
{
    return __fadd_rn(__fdiv_rn(phat, p.ds_half), p.two_cc);
}

// asin(a) for |a| <= 0.5 as a + a^3 P(a^2), P of degree 4 fitted here by
// weighted least squares on Chebyshev nodes (max error 0.67 ulp in float);
// larger |a| (only the corners of very wide fields) fall back to asinf.
__device__ __forceinline__ float asin_fast(float a)
{
    if (fabsf(a) > 0.5f) return asinf(a);
    float t = a * a;
    float p = fmaf(t, 0.042095037962576944f, 0.024220510033133892f);
    p = fmaf(t, p, 0.04546249911296045f);
    p = fmaf(t, p, 0.07495353339646753f);
    p = fmaf(t, p, 0.16666751488866943f);
    return fmaf(a * t, p, a);
}

// Row floors through the float unit: for |ql| < 2^22, ql + 1.5 2^23 rounded
// down is exactly 1.5 2^23 + floor(ql) (the binade [2^23, 2^24) has unit
// spacing), so one packed add gives both the floor as a float (t - 1.5 2^23,
// exact) and as an integer (the bits of t are kFloorMagicBits + floor(ql)).
// The row address is then view + bits(t) * row stride with the view's base
// moved back by kFloorMagicBits rows (64-bit modular arithmetic, folded into
// BpParams::rebin_rows on the host): one multiply-add, no conversion.
constexpr float kFloorMagic = 12582912.0f;       // 1.5 * 2^23
constexpr uint32_t kFloorMagicBits = 0x4B400000u;  // its bits
__device__ __forceinline__ float2 row_floor(float2 ql)
{
    return __fadd2_rd(ql, make_float2(kFloorMagic, kFloorMagic));
}

// The 2x2 footprint {(p, row), (p+1, row), (p, row+1), (p+1, row+1)} of a
// view, row in [0, R-2] given as t = kFloorMagic + row (row_floor);
// `view_rows` is the view's (p, 0) address moved back by kFloorMagicBits rows.
template <bool QUAD>
__device__ __forceinline__ void fetch_footprint(uint64_t view_rows, int nos, float t, float &v00, float &v01,
                                                float &v10, float &v11)
{
    if constexpr (QUAD) {
        // footprint quads: the four FP16 samples in one 8-byte word
        const uint2 *q = reinterpret_cast<const uint2 *>(
            view_rows + (uint64_t)__float_as_uint(t) * (uint64_t)((unsigned)nos * sizeof(uint2)));
        const uint2 w = __ldg(q);
        const float2 top = __half22float2(*reinterpret_cast<const __half2 *>(&w.x));
        const float2 bot = __half22float2(*reinterpret_cast<const __half2 *>(&w.y));
        v00 = top.x;
        v01 = top.y;
        v10 = bot.x;
        v11 = bot.y;
    } else {
        const float *r0 = reinterpret_cast<const float *>(
            view_rows + (uint64_t)__float_as_uint(t) * (uint64_t)((unsigned)nos * sizeof(float)));
        v00 = __ldg(r0);
        v01 = __ldg(r0 + 1);
        v10 = __ldg(r0 + nos);
        v11 = __ldg(r0 + nos + 1);
    }
}

// Packed FP32 pairs (sm_100 family): one instruction for two lanes.
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// NOS > 0: the row length as a compile-time constant (the second row of a
// footprint is then an immediate offset); 0: taken from p.nos.
// One CTA tile (bx, by, bz) of a block's backprojection with the parameters
// p (kernel parameters, or a block's entry of a batch copied to shared
// memory).
template <int ZPT, int NOS, int THREADS, bool QUAD, class Params>
__device__ __forceinline__ void backproject_tile(const Params &p, int bx, int by, int bz)
{
    constexpr unsigned kElem = QUAD ? sizeof(uint2) : sizeof(float);
    constexpr int SUB = ZPT < kSub ? ZPT : kSub;  // slices per sub-chunk
    const int nos = NOS > 0 ? NOS : p.nos;
    // A CTA covers cta_w x (256 / cta_w) voxel columns; each warp a warp_w x
    // (32 / warp_w) sub-tile, which bounds how far apart its lanes' detector
    // samples lie (a row of 32 columns spreads over up to ~110 channels).
    const int lane = threadIdx.x, warp = threadIdx.y;
    const int tiles_x = p.cta_w / p.warp_w;
    int xi = bx * p.cta_w + (warp % tiles_x) * p.warp_w + lane % p.warp_w;
    int yi = by * (THREADS / p.cta_w) + (warp / tiles_x) * (32 / p.warp_w) + lane / p.warp_w;
    int z0 = bz * ZPT;
    if (xi >= p.nx || yi >= p.ny) return;
    // voxel centre with the reference's float operations (no contraction)
    float x = __fadd_rn(__fmul_rn(p.pix_x, __fsub_rn((float)xi, p.x_c)), p.x0);
    float y = __fadd_rn(__fmul_rn(p.pix_y, __fsub_rn((float)yi, p.y_c)), p.y0);

    // the image sums live in shared memory (touched once per angle), which
    // leaves the registers to the per-angle sums and the gathers in flight
    __shared__ float2 img_sh[ZPT / 2][THREADS];  // slice pairs, one 8-byte word per thread
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    float2 *img = &img_sh[0][tid];
#pragma unroll
    for (int m = 0; m < ZPT / 2; ++m) img[m * THREADS] = make_float2(0.0f, 0.0f);
    // Slice z of the block sits at zbase + z * coll, zbase the block's slice 0,
    // and q of slice z is q0 + z dq with q0 that of slice 0: the same
    // arithmetic whatever the launch shape, so that the |q| < 1 decisions (a
    // jump in the result) do not depend on it.  The exact per-slice z is only
    // needed by the border recheck and is read from zpos there.
    const float zbase = __ldg(p.zpos);
    const float z0f = (float)z0;
    const float zchunk = fmaf(z0f, p.coll, zbase);
    const unsigned view_stride = (unsigned)(p.n_rows * nos);  // < 2^20
    const float p_max = (float)(nos - 2);
    const float p_mid = 0.5f * p_max;
    const float q_max_last = (float)(p.n_rows - 2);
    const float z_end = fmaf((float)(ZPT - 1), p.coll, zchunk);
    const float z_lo = fminf(zchunk, z_end), z_hi = fmaxf(zchunk, z_end);
    const unsigned warp_lanes = __activemask();

    for (int i = 0; i < p.n_half; ++i) {
        float2 s2[ZPT / 2], h2[ZPT / 2];  // per-angle sums of slice pairs
        int n_flat[ZPT / SUB];  // flat visits of each sub-chunk: W = 1 for every slice
#pragma unroll
        for (int sc = 0; sc < ZPT / SUB; ++sc) n_flat[sc] = 0;
#pragma unroll
        for (int m = 0; m < ZPT / 2; ++m) {
            s2[m] = make_float2(0.0f, 0.0f);
            h2[m] = make_float2(0.0f, 0.0f);
        }
        // The views i + k n_half are nearly half turns apart: p nearly flips
        // its sign from one to the next.  Not exactly: the reference steps
        // half turns by pi' = 3.1415368979, so view k is turned a further
        // k (pi - pi') = k 5.6e-5 rad and |p_k| differs from |p_0| by up to
        // k r 5.6e-5 (0.04 mm at the corner of a 500 mm field, 1e-3 detector
        // rows in q at config-3 geometry).  asin(|p| / r_f) and
        // sqrt(r_f^2 - p^2) are taken once per angle at |p_0| and carried to
        // each |p_k| to first order: d = |p_k| - |p_0|, asin += d / root,
        // root -= (|p_0| / root) d (second-order terms below 1e-8 rad), with
        // the constants folded: asin_k = |p_k| / root + A, root_k = B - s |p_k|.
        const float4 *vt = p.views + (size_t)i * p.nht;
        float a_abs, root, inv_root, slope, a_off, root_off;
        int k_lo = 0, k_hi = p.nht - 1;
        {
            float4 t0 = __ldg(vt);
            float phat0 = __fsub_rn(__fmul_rn(x, t0.y), __fmul_rn(y, t0.z));
            a_abs = fabsf(asin_fast(phat0 * p.inv_rf));
            float l2 = fmaf(-phat0, phat0, p.rf2);
            inv_root = rsqrtf(l2);
            root = l2 * inv_root;
            const float p0_abs = fabsf(phat0);
            slope = p0_abs * inv_root;
            a_off = fmaf(-p0_abs, inv_root, a_abs);
            root_off = fmaf(slope, p0_abs, root);
            if (p.k_window) {
                // Half turns whose rays can reach the chunk: ray_k lies within
                // |asin zr| of (theta_0 + k pi') zr, and |q| < 1 needs
                // |z - ray_k| < lhat_k tan_cone <= (root + |x cos + y sin|) tan_cone.
                // A margin of kWindowMargin half turns absorbs the rounding of the
                // angles and of this bound; the exact test below still decides
                // every visited half turn.
                float reach = fmaf(root + fabsf(fmaf(x, t0.z, y * t0.y)), p.tan_cone, a_abs * p.abs_zr);
                float base = t0.w;
                float lo = (z_lo - reach - base) * p.inv_half_feed;
                float hi = (z_hi + reach - base) * p.inv_half_feed;
                k_lo = max(k_lo, (int)ceilf(fminf(lo, hi) - kWindowMargin));
                k_hi = min(k_hi, (int)floorf(fmaxf(lo, hi) + kWindowMargin));
            }
        }
        k_lo = __reduce_min_sync(warp_lanes, k_lo);
        k_hi = __reduce_max_sync(warp_lanes, k_hi);
        for (int k = k_lo; k <= k_hi; ++k) {
            float4 t = __ldg(vt + k);
            // q of the chunk's slices: q(z) = q0 + z dq (dq > 0)
            float phat = __fsub_rn(__fmul_rn(x, t.y), __fmul_rn(y, t.z));
            // this view's asin(|p| / r_f) and sqrt(r_f^2 - p^2) from the angle's
            const float a_k = fmaf(fabsf(phat), inv_root, a_off);
            const float root_k = fmaf(-slope, fabsf(phat), root_off);
            // zbase - ray with ray = (theta - asin(p / r_f)) z_rot / 2 pi'
            float zb_ray = fmaf(copysignf(a_k, phat), p.zrot_over_2pi, zbase - t.w);
            float lhat = root_k - x * t.z - y * t.y;
            float inv_den = __fdividef(1.0f, lhat * p.tan_cone);
            float q0 = zb_ray * inv_den;
            float dq = p.coll * inv_den;
            const float q_first = fmaf(z0f, dq, q0);
            const float q_end = fmaf(z0f + (float)(ZPT - 1), dq, q0);
            // no slice of the chunk inside |q| < 1: nothing to add, not even weight
            if (q_first >= 1.0f || q_end <= -1.0f) continue;
            // p and its border decision exactly as the reference rounds them
            float p_idx = fmaf(phat, p.inv_ds_half, p.two_cc);
            // within the band of either border (|p_idx - p_mid| > p_mid - band; the
            // fast p_idx is within 2e-4 of the exact one, the band is 1e-3):
            // the exact p_idx decides, with the reference's own comparisons
            if (fabsf(p_idx - p_mid) > p_mid - kBorderBand) p_idx = p_index_exact(p, phat);
            bool p_ok = (p_idx >= 0.0f) && (p_idx <= p_max);
            bool last = (k == p.nht - 1);
            int ip = p_ok ? (int)p_idx : (p_idx < 0.0f ? 0 : nos - 2);
            float wp = p_idx - (float)ip;
            const uint64_t view_rows =
                p.rebin_rows + ((uint64_t)__float_as_uint(t.x) * view_stride + (unsigned)ip) * kElem;
            // quads: the view's scale, folded into the weights of its samples
            float2 vs2 = make_float2(1.0f, 1.0f);
            if constexpr (QUAD) {
                const float vs = __ldg(p.vscale + (size_t)__float_as_uint(t.x) * p.n_rows);
                vs2 = make_float2(vs, vs);
            }
            // Slices are processed in pairs (z, z + 1) with packed FP32
            // arithmetic (one FFMA2 / FADD2 / FMUL2 per two slices); floors,
            // conversions and loads stay per slice.
            const float2 wp2 = make_float2(wp, wp);
            const float2 omwp2 = make_float2(1.0f - wp, 1.0f - wp);
            const float2 dq2 = make_float2(dq, dq), q02 = make_float2(q0, q0);
            const float2 hr2 = make_float2(p.half_rows, p.half_rows);
            // bilinear value of a pair from its rows t = kFloorMagic + row
            // (clamped or not by the caller)
            auto pair_value = [&](float2 ql, float2 tr) -> float2 {
                float2 wq = sub2(ql, sub2(tr, make_float2(kFloorMagic, kFloorMagic)));
                float a00, a01, a10, a11, b00, b01, b10, b11;
                fetch_footprint<QUAD>(view_rows, nos, tr.x, a00, a01, a10, a11);
                fetch_footprint<QUAD>(view_rows, nos, tr.y, b00, b01, b10, b11);
                float2 c0 = fma2(wp2, make_float2(a01, b01), mul2(omwp2, make_float2(a00, b00)));
                float2 c1 = fma2(wp2, make_float2(a11, b11), mul2(omwp2, make_float2(a10, b10)));
                return fma2(wq, sub2(c1, c0), c0);
            };
            // cos^2 taper weight of a pair: W = 1 below Q (cos(0) = 1), then
            // cos^2(pi/2 (|q| - Q) / (1 - Q))
            auto pair_weight = [&](float2 q) -> float2 {
                float2 t = make_float2(fmaxf(fabsf(q.x) - kQ, 0.0f), fmaxf(fabsf(q.y) - kQ, 0.0f));
                float2 arg = mul2(t, make_float2(p.taper_scale, p.taper_scale));
                float2 c = make_float2(__cosf(arg.x), __cosf(arg.y));
                return mul2(c, c);
            };
            // Sub-chunks of SUB slices share the geometry above.  Each is
            // skipped when no lane has a slice inside |q| < 1, else classed per
            // warp so that no two paths both run
            // (q is monotone in z, so |q| is largest at an end of the chunk):
            //  flat:  every |q| <= Q, so W = 1; with R >= 8 every row lies in
            //         [0, R-2] and below the last-turn border;
            //  inner: every |q| < 1, so every row lies in [0, R-2]; in the last
            //         half turn also every row well below its border;
            //  other: per-slice validity, clamped rows, last-turn border.
            unsigned lanes = __activemask();
#pragma unroll
            for (int sc = 0; sc < ZPT / SUB; ++sc) {
                const float q0c = fmaf(z0f + (float)(sc * SUB), dq, q0);
                const float q_endc = fmaf(z0f + (float)(sc * SUB + SUB - 1), dq, q0);
                if (ZPT > SUB && __all_sync(lanes, q0c >= 1.0f || q_endc <= -1.0f)) continue;
                float a_max = fmaxf(fabsf(q0c), fabsf(q_endc));
                if (__all_sync(lanes, p.flat_path && a_max <= kQ)) {
                    if (p_ok) {
                        float ql0 = fmaf(q0, p.half_rows, p.half_rows);
                        float dql = dq * p.half_rows;
                        const float2 ql02 = make_float2(ql0, ql0), dql2 = make_float2(dql, dql);
#pragma unroll
                        for (int mm = 0; mm < SUB / 2; ++mm) {
                            const int m = sc * (SUB / 2) + mm;
                            float2 ql = fma2(make_float2(z0f + (float)(2 * m), z0f + (float)(2 * m + 1)), dql2, ql02);
                            if constexpr (QUAD) s2[m] = fma2(pair_value(ql, row_floor(ql)), vs2, s2[m]);
                            else s2[m] = add2(s2[m], pair_value(ql, row_floor(ql)));
                        }
                    }
                    ++n_flat[sc];
                    continue;
                }
                bool inner = a_max < kInnerMax && (!last || fmaf(a_max, p.half_rows, p.half_rows) < q_max_last - kRowMargin);
                if (__all_sync(lanes, inner)) {
                    if (p_ok) {
#pragma unroll
                        for (int mm = 0; mm < SUB / 2; ++mm) {
                            const int m = sc * (SUB / 2) + mm;
                            float2 q = fma2(make_float2(z0f + (float)(2 * m), z0f + (float)(2 * m + 1)), dq2, q02);
                            float2 w = pair_weight(q);
                            h2[m] = add2(h2[m], w);
                            float2 ql = fma2(q, hr2, hr2);
                            if constexpr (QUAD) w = mul2(w, vs2);
                            s2[m] = fma2(w, pair_value(ql, row_floor(ql)), s2[m]);
                        }
                    } else {
#pragma unroll
                        for (int mm = 0; mm < SUB / 2; ++mm) {
                            const int m = sc * (SUB / 2) + mm;
                            float2 q = fma2(make_float2(z0f + (float)(2 * m), z0f + (float)(2 * m + 1)), dq2, q02);
                            h2[m] = add2(h2[m], pair_weight(q));
                        }
                    }
                    continue;
                }
                // Other chunks.  Branch-free gathers: every slice loads its 2x2
                // footprint from inside the view (row clamped to [0, R-2], channel 0
                // when p is off the detector) and validity only scales the weight, so
                // the loads of all slices can be issued together.  Only a warp with
                // a row near the last-turn border takes the per-slice border test.
                const float t_max = kFloorMagic + (float)(p.n_rows - 2);  // row R-2
                bool border = last && fmaf(q_endc, p.half_rows, p.half_rows) > q_max_last - kBorderBand;
                if (__any_sync(lanes, border)) {
#pragma unroll
                    for (int mm = 0; mm < SUB / 2; ++mm) {
                        const int m = sc * (SUB / 2) + mm;
                        float2 q = fma2(make_float2(z0f + (float)(2 * m), z0f + (float)(2 * m + 1)), dq2, q02);
                        bool in_x = fabsf(q.x) < 1.0f, in_y = fabsf(q.y) < 1.0f;
                        float2 w = pair_weight(q);
                        w = make_float2(in_x ? w.x : 0.0f, in_y ? w.y : 0.0f);
                        h2[m] = add2(h2[m], w);
                        float2 ql = fma2(q, hr2, hr2);
                        float2 tr = row_floor(ql);
                        tr = make_float2(fminf(fmaxf(tr.x, kFloorMagic), t_max), fminf(fmaxf(tr.y, kFloorMagic), t_max));
                        float2 v = pair_value(ql, tr);
                        bool ok_x = p_ok && in_x, ok_y = p_ok && in_y;
                        if (ok_x) {
                            float d = ql.x - q_max_last;
                            if (d > kBorderBand) ok_x = false;
                            else if (d > -kBorderBand)
                                ok_x = last_turn_sample_valid(p, x, y, __ldg(p.theta + (size_t)i * p.nht + k), t.y,
                                                              t.z, phat, __ldg(p.zpos + z0 + 2 * m), k);
                        }
                        if (ok_y) {
                            float d = ql.y - q_max_last;
                            if (d > kBorderBand) ok_y = false;
                            else if (d > -kBorderBand)
                                ok_y = last_turn_sample_valid(p, x, y, __ldg(p.theta + (size_t)i * p.nht + k), t.y,
                                                              t.z, phat, __ldg(p.zpos + z0 + 2 * m + 1), k);
                        }
                        float2 wv = make_float2(ok_x ? w.x : 0.0f, ok_y ? w.y : 0.0f);
                        if constexpr (QUAD) wv = mul2(wv, vs2);
                        s2[m] = fma2(wv, v, s2[m]);
                    }
                    continue;
                }
#pragma unroll
                for (int mm = 0; mm < SUB / 2; ++mm) {
                    const int m = sc * (SUB / 2) + mm;
                    float2 q = fma2(make_float2(z0f + (float)(2 * m), z0f + (float)(2 * m + 1)), dq2, q02);
                    bool in_x = fabsf(q.x) < 1.0f, in_y = fabsf(q.y) < 1.0f;
                    // a pair outside |q| < 1 in every lane adds nothing
                    if (!__any_sync(lanes, in_x || in_y)) continue;
                    float2 w = pair_weight(q);
                    w = make_float2(in_x ? w.x : 0.0f, in_y ? w.y : 0.0f);
                    h2[m] = add2(h2[m], w);
                    float2 ql = fma2(q, hr2, hr2);
                    float2 tr = row_floor(ql);
                    tr = make_float2(fminf(fmaxf(tr.x, kFloorMagic), t_max), fminf(fmaxf(tr.y, kFloorMagic), t_max));
                    float2 v = pair_value(ql, tr);
                    float2 wv = p_ok ? w : make_float2(0.0f, 0.0f);
                    if constexpr (QUAD) wv = mul2(wv, vs2);
                    s2[m] = fma2(wv, v, s2[m]);
                }
            }
        }
#pragma unroll
        for (int m = 0; m < ZPT / 2; ++m) {
            const float nf = (float)n_flat[m / (SUB / 2)];
            float2 hz = add2(h2[m], make_float2(nf, nf));
            // s is 0 wherever h is (every weight that adds to s adds to h), and
            // the smallest nonzero h is far above 1e-30: s / max(h, 1e-30) is
            // the reference's "if (h != 0) img += s / h"
            float2 rh = make_float2(__fdividef(1.0f, fmaxf(hz.x, 1e-30f)), __fdividef(1.0f, fmaxf(hz.y, 1e-30f)));
            img[m * THREADS] = fma2(s2[m], rh, img[m * THREADS]);
        }
    }
    size_t plane = (size_t)p.nx * p.ny;
#pragma unroll
    for (int z = 0; z < ZPT; ++z)
        if (z0 + z < p.n_slices) {
            float2 v = img[(z / 2) * THREADS];
            p.out[(size_t)(z0 + z) * plane + (size_t)yi * p.nx + xi] = ((z & 1) ? v.y : v.x) * p.out_scale;
        }
}

template <int ZPT, int MIN_BLOCKS, int NOS, int THREADS = 256, bool QUAD = false>
__global__ void __launch_bounds__(THREADS, MIN_BLOCKS) backproject_kernel(BpParams p)
{
    backproject_tile<ZPT, NOS, THREADS, QUAD>(p, blockIdx.x, blockIdx.y, blockIdx.z);
}

// ---- column form --------------------------------------------------------
enum { kOutScaled = 0, kOutPartial = 1, kOutFirst = 2, kOutMiddle = 3, kOutLast = 4 };

// A thread owns the voxel column (x, y) over up to ZMAX slices (zpt of them,
// in sub-chunks of SUB = 8).  Per angle, the geometry of every half turn in
// the column's window -- q of the block's slice 0, its step per slice, the
// channel weights and the footprint row address -- is computed once for all of the
// column's slices and parked in shared memory (each thread its own entries,
// no barrier).  Each sub-chunk then sums its visits with the per-angle sums of
// its slices in registers and folds s / h into the image sums.  Against the
// slice-chunk form above (geometry once per 8 slices) this divides the
// per-visit geometry, the angle set-up and the window search by the number of
// sub-chunks, for one shared-memory load per visit.
//
// Whether p_idx lies on the detector, and (FP16 footprint words) the view's
// scale, are folded into the two channel weights: a sample whose p_idx is off
// the detector then reads the nearest edge channel of its view and adds
// exactly zero to s while its weight still adds to h (interp2's rule); a visit
// with p off the detector in every lane fetches nothing.
//
// Geometry entry of half turn k (window slot kk) for thread tid:
//   geo_w[kk][tid] = {q0, dq, (1 - wp) c, wp c}   c = [p on the detector] * scale
//   geo_a[kk][tid] = address of the view's (ip, row 0) moved back as in row_floor
//
// Angle chunk ac of n_ac runs half-turn angles [ac n_half / n_ac, (ac + 1)
// n_half / n_ac); out_mode says where its image sums go:
//   kOutScaled   out = sums * out_scale (one chunk)
//   kOutPartial  partial[ac] = sums (a combine kernel adds the chunks)
//   kOutFirst    out = sums               (the first of chunks run one after
//   kOutMiddle   out = out + sums          another: the same additions, in the
//   kOutLast     out = (out + sums) * out_scale   same order, as the combine)
template <int ZMAX, int SUB, int NOS, int THREADS, bool QUAD, class Params>
__device__ __forceinline__ void backproject_column_tile(const Params &p, int bx, int by, int bz, int ac, int n_ac,
                                                        int out_mode, float4 *geo_w, uint2 *geo_a)
{
    static_assert(SUB % 2 == 0 && ZMAX % SUB == 0, "sub-chunks of whole slice pairs");
    constexpr unsigned kElem = QUAD ? sizeof(uint2) : sizeof(float);
    const int nos = NOS > 0 ? NOS : p.nos;
    const int lane = threadIdx.x, warp = threadIdx.y;
    const int tiles_x = p.cta_w / p.warp_w;
    const int xi = bx * p.cta_w + (warp % tiles_x) * p.warp_w + lane % p.warp_w;
    const int yi = by * (THREADS / p.cta_w) + (warp / tiles_x) * (32 / p.warp_w) + lane / p.warp_w;
    const int zpt = p.col_zpt;
    const int z0 = bz * zpt;
    const int i_begin = (int)(((long long)ac * p.n_half) / n_ac);
    const int i_end = (int)(((long long)(ac + 1) * p.n_half) / n_ac);
    if (xi >= p.nx || yi >= p.ny) return;
    const int nsub = (min(zpt, p.n_slices - z0) + SUB - 1) / SUB;
    const float x = __fadd_rn(__fmul_rn(p.pix_x, __fsub_rn((float)xi, p.x_c)), p.x0);
    const float y = __fadd_rn(__fmul_rn(p.pix_y, __fsub_rn((float)yi, p.y_c)), p.y0);

    __shared__ float2 img_sh[ZMAX / 2][THREADS];
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    float2 *img = &img_sh[0][tid];
#pragma unroll
    for (int m = 0; m < ZMAX / 2; ++m) img[m * THREADS] = make_float2(0.0f, 0.0f);
    float4 *gw = geo_w + tid;
    uint2 *ga = geo_a + tid;

    // slice z of the block at zbase + z coll and its q at q0 + z dq, zbase and
    // q0 those of the block's slice 0, z the slice's index in the block (the
    // same arithmetic for every launch shape, see backproject_tile)
    const float zbase = __ldg(p.zpos);
    const float zchunk = fmaf((float)z0, p.coll, zbase);
    const unsigned view_stride = (unsigned)(p.n_rows * nos);
    const float p_max = (float)(nos - 2);
    const float p_mid = 0.5f * p_max;
    const float q_max_last = (float)(p.n_rows - 2);
    const float hr = p.half_rows;
    const float z_end = fmaf((float)(nsub * SUB - 1), p.coll, zchunk);
    const float z_lo = fminf(zchunk, z_end), z_hi = fmaxf(zchunk, z_end);
    const unsigned lanes = __activemask();

    for (int i = i_begin; i < i_end; ++i) {
        const float4 *vt = p.views + (size_t)i * p.nht;
        float inv_root, slope, a_off, root_off;
        int k_lo = 0, k_hi = p.nht - 1;
        {
            // the angle's k = 0 view: asin and root carried to each half turn
            // to first order (see backproject_tile)
            const float4 t0 = __ldg(vt);
            const float phat0 = __fsub_rn(__fmul_rn(x, t0.y), __fmul_rn(y, t0.z));
            const float a_abs = fabsf(asin_fast(phat0 * p.inv_rf));
            const float l2 = fmaf(-phat0, phat0, p.rf2);
            inv_root = rsqrtf(l2);
            const float root = l2 * inv_root;
            const float p0_abs = fabsf(phat0);
            slope = p0_abs * inv_root;
            a_off = fmaf(-p0_abs, inv_root, a_abs);
            root_off = fmaf(slope, p0_abs, root);
            if (p.k_window) {
                const float reach = fmaf(root + fabsf(fmaf(x, t0.z, y * t0.y)), p.tan_cone, a_abs * p.abs_zr);
                const float lo = (z_lo - reach - t0.w) * p.inv_half_feed;
                const float hi = (z_hi + reach - t0.w) * p.inv_half_feed;
                k_lo = max(k_lo, (int)ceilf(fminf(lo, hi) - kWindowMargin));
                k_hi = min(k_hi, (int)floorf(fmaxf(lo, hi) + kWindowMargin));
            }
        }
        k_lo = __reduce_min_sync(lanes, k_lo);
        k_hi = __reduce_max_sync(lanes, k_hi);
        // the window's geometry, once for every slice of the column
        for (int k = k_lo; k <= k_hi; ++k) {
            const float4 t = __ldg(vt + k);
            const float phat = __fsub_rn(__fmul_rn(x, t.y), __fmul_rn(y, t.z));
            const float a_k = fmaf(fabsf(phat), inv_root, a_off);
            const float root_k = fmaf(-slope, fabsf(phat), root_off);
            const float zb_ray = fmaf(copysignf(a_k, phat), p.zrot_over_2pi, zbase - t.w);
            const float lhat = root_k - x * t.z - y * t.y;
            const float inv_den = __fdividef(1.0f, lhat * p.tan_cone);
            float p_idx = fmaf(phat, p.inv_ds_half, p.two_cc);
            if (fabsf(p_idx - p_mid) > p_mid - kBorderBand) p_idx = p_index_exact(p, phat);
            const bool p_ok = (p_idx >= 0.0f) && (p_idx <= p_max);
            // off the detector: the nearest edge channel (its weight is zero;
            // the address stays near the warp's other lanes' lines)
            const int ip = p_ok ? (int)p_idx : (p_idx < 0.0f ? 0 : nos - 2);
            const float wp = p_idx - (float)ip;
            const unsigned row = __float_as_uint(t.x);
            float c = p_ok ? 1.0f : 0.0f;
            if constexpr (QUAD) c *= __ldg(p.vscale + (size_t)row * p.n_rows);
            const uint64_t view_rows = p.rebin_rows + ((uint64_t)row * view_stride + (unsigned)ip) * kElem;
            const int kk = k - k_lo;
            const float q0 = zb_ray * inv_den, dq = p.coll * inv_den;
            gw[kk * THREADS] = make_float4(q0, dq, (1.0f - wp) * c, wp * c);
            ga[kk * THREADS] = make_uint2((unsigned)view_rows, (unsigned)(view_rows >> 32));
        }
        for (int sc = 0; sc < nsub; ++sc) {
            float2 s2[SUB / 2], h2[SUB / 2];
#pragma unroll
            for (int m = 0; m < SUB / 2; ++m) {
                s2[m] = make_float2(0.0f, 0.0f);
                h2[m] = make_float2(0.0f, 0.0f);
            }
            int n_flat = 0;
            const float zc = (float)(z0 + sc * SUB);  // the sub-chunk's first slice
            for (int k = k_lo; k <= k_hi; ++k) {
                const int kk = k - k_lo;
                const float4 g = gw[kk * THREADS];
                const float dq = g.y;
                // q of the sub-chunk's slices: q0 + (zc + m) dq, m = 0 .. SUB - 1
                const float q0c = fmaf(zc, dq, g.x);
                const float q_endc = fmaf(zc + (float)(SUB - 1), dq, g.x);
                // no slice of the sub-chunk inside |q| < 1 in any lane: nothing to add
                if (__all_sync(lanes, q0c >= 1.0f || q_endc <= -1.0f)) continue;
                const uint2 av = ga[kk * THREADS];
                const uint64_t view_rows = ((uint64_t)av.y << 32) | av.x;
                const bool last = (k == p.nht - 1);
                const float2 wp2 = make_float2(g.w, g.w);
                const float2 omwp2 = make_float2(g.z, g.z);
                const float2 dq2 = make_float2(dq, dq), q02 = make_float2(g.x, g.x);
                const float2 hr2 = make_float2(hr, hr);
                // cos^2 taper weight of a pair: W = 1 below Q (cos(0) = 1), then
                // cos^2(pi/2 (|q| - Q) / (1 - Q))
                auto pair_weight = [&](float2 q) -> float2 {
                    float2 t = make_float2(fmaxf(fabsf(q.x) - kQ, 0.0f), fmaxf(fabsf(q.y) - kQ, 0.0f));
                    float2 arg = mul2(t, make_float2(p.taper_scale, p.taper_scale));
                    float2 cc = make_float2(__cosf(arg.x), __cosf(arg.y));
                    return mul2(cc, cc);
                };
                // p off the detector in every lane: interp2 gives 0, so only the
                // weights count (h), nothing is fetched
                if (!__any_sync(lanes, (g.z != 0.0f) || (g.w != 0.0f))) {
                    const float a_max0 = fmaxf(fabsf(q0c), fabsf(q_endc));
                    if (__all_sync(lanes, a_max0 <= kQ)) {
                        ++n_flat;
                        continue;
                    }
#pragma unroll
                    for (int m = 0; m < SUB / 2; ++m) {
                        const float2 q = fma2(make_float2(zc + (float)(2 * m), zc + (float)(2 * m + 1)), dq2, q02);
                        const float2 w = pair_weight(q);
                        h2[m] = add2(h2[m], make_float2(fabsf(q.x) < 1.0f ? w.x : 0.0f, fabsf(q.y) < 1.0f ? w.y : 0.0f));
                    }
                    continue;
                }
                auto pair_value = [&](float2 ql, float2 tr) -> float2 {
                    float2 wq = sub2(ql, sub2(tr, make_float2(kFloorMagic, kFloorMagic)));
                    float a00, a01, a10, a11, b00, b01, b10, b11;
                    fetch_footprint<QUAD>(view_rows, nos, tr.x, a00, a01, a10, a11);
                    fetch_footprint<QUAD>(view_rows, nos, tr.y, b00, b01, b10, b11);
                    float2 c0 = fma2(wp2, make_float2(a01, b01), mul2(omwp2, make_float2(a00, b00)));
                    float2 c1 = fma2(wp2, make_float2(a11, b11), mul2(omwp2, make_float2(a10, b10)));
                    return fma2(wq, sub2(c1, c0), c0);
                };
                // every footprint of the sub-chunk is fetched before any is used,
                // so that a visit waits for its gathers once
                float fp[SUB][4];
                float2 wq2[SUB / 2];
                auto fetch_all = [&](const float2 *ql) {
#pragma unroll
                    for (int m = 0; m < SUB / 2; ++m) {
                        const float2 tr = row_floor(ql[m]);
                        wq2[m] = sub2(ql[m], sub2(tr, make_float2(kFloorMagic, kFloorMagic)));
                        fetch_footprint<QUAD>(view_rows, nos, tr.x, fp[2 * m][0], fp[2 * m][1], fp[2 * m][2],
                                              fp[2 * m][3]);
                        fetch_footprint<QUAD>(view_rows, nos, tr.y, fp[2 * m + 1][0], fp[2 * m + 1][1],
                                              fp[2 * m + 1][2], fp[2 * m + 1][3]);
                    }
                };
                auto fetched_value = [&](int m) -> float2 {
                    float2 c0 = fma2(wp2, make_float2(fp[2 * m][1], fp[2 * m + 1][1]),
                                     mul2(omwp2, make_float2(fp[2 * m][0], fp[2 * m + 1][0])));
                    float2 c1 = fma2(wp2, make_float2(fp[2 * m][3], fp[2 * m + 1][3]),
                                     mul2(omwp2, make_float2(fp[2 * m][2], fp[2 * m + 1][2])));
                    return fma2(wq2[m], sub2(c1, c0), c0);
                };
                const float a_max = fmaxf(fabsf(q0c), fabsf(q_endc));
                if (__all_sync(lanes, p.flat_path && a_max <= kQ)) {
                    const float ql0 = fmaf(g.x, hr, hr);
                    const float dql = dq * hr;
                    const float2 ql02 = make_float2(ql0, ql0), dql2 = make_float2(dql, dql);
                    float2 ql[SUB / 2];
#pragma unroll
                    for (int m = 0; m < SUB / 2; ++m)
                        ql[m] = fma2(make_float2(zc + (float)(2 * m), zc + (float)(2 * m + 1)), dql2, ql02);
                    fetch_all(ql);
#pragma unroll
                    for (int m = 0; m < SUB / 2; ++m) s2[m] = add2(s2[m], fetched_value(m));
                    ++n_flat;
                    continue;
                }
                const bool inner =
                    a_max < kInnerMax && (!last || fmaf(a_max, hr, hr) < q_max_last - kRowMargin);
                if (__all_sync(lanes, inner)) {
                    float2 ql[SUB / 2], q[SUB / 2];
#pragma unroll
                    for (int m = 0; m < SUB / 2; ++m) {
                        q[m] = fma2(make_float2(zc + (float)(2 * m), zc + (float)(2 * m + 1)), dq2, q02);
                        ql[m] = fma2(q[m], hr2, hr2);
                    }
                    fetch_all(ql);
#pragma unroll
                    for (int m = 0; m < SUB / 2; ++m) {
                        float2 w = pair_weight(q[m]);
                        h2[m] = add2(h2[m], w);
                        s2[m] = fma2(w, fetched_value(m), s2[m]);
                    }
                    continue;
                }
                const float t_max = kFloorMagic + (float)(p.n_rows - 2);  // row R-2
                const bool border = last && fmaf(q_endc, hr, hr) > q_max_last - kBorderBand;
                if (__any_sync(lanes, border)) {
                    // rare: rows near the last half turn's border, decided by the
                    // reference's own q_idx (p_idx off the detector adds nothing)
                    const bool p_ok = (g.z != 0.0f) || (g.w != 0.0f);
                    const float4 t = __ldg(vt + k);
                    const float phat = __fsub_rn(__fmul_rn(x, t.y), __fmul_rn(y, t.z));
                    const float theta = __ldg(p.theta + (size_t)i * p.nht + k);
#pragma unroll
                    for (int m = 0; m < SUB / 2; ++m) {
                        float2 q = fma2(make_float2(zc + (float)(2 * m), zc + (float)(2 * m + 1)), dq2, q02);
                        bool in_x = fabsf(q.x) < 1.0f, in_y = fabsf(q.y) < 1.0f;
                        float2 w = pair_weight(q);
                        w = make_float2(in_x ? w.x : 0.0f, in_y ? w.y : 0.0f);
                        h2[m] = add2(h2[m], w);
                        float2 ql = fma2(q, hr2, hr2);
                        float2 tr = row_floor(ql);
                        tr = make_float2(fminf(fmaxf(tr.x, kFloorMagic), t_max), fminf(fmaxf(tr.y, kFloorMagic), t_max));
                        float2 v = pair_value(ql, tr);
                        bool ok_x = p_ok && in_x, ok_y = p_ok && in_y;
                        const int zs = z0 + sc * SUB + 2 * m;
                        if (ok_x) {
                            float d = ql.x - q_max_last;
                            if (d > kBorderBand) ok_x = false;
                            else if (d > -kBorderBand)
                                ok_x = last_turn_sample_valid(p, x, y, theta, t.y, t.z, phat,
                                                              __ldg(p.zpos + min(zs, p.n_slices - 1)), k);
                        }
                        if (ok_y) {
                            float d = ql.y - q_max_last;
                            if (d > kBorderBand) ok_y = false;
                            else if (d > -kBorderBand)
                                ok_y = last_turn_sample_valid(p, x, y, theta, t.y, t.z, phat,
                                                              __ldg(p.zpos + min(zs + 1, p.n_slices - 1)), k);
                        }
                        s2[m] = fma2(make_float2(ok_x ? w.x : 0.0f, ok_y ? w.y : 0.0f), v, s2[m]);
                    }
                    continue;
                }
#pragma unroll
                for (int m = 0; m < SUB / 2; ++m) {
                    float2 q = fma2(make_float2(zc + (float)(2 * m), zc + (float)(2 * m + 1)), dq2, q02);
                    bool in_x = fabsf(q.x) < 1.0f, in_y = fabsf(q.y) < 1.0f;
                    if (!__any_sync(lanes, in_x || in_y)) continue;
                    float2 w = pair_weight(q);
                    w = make_float2(in_x ? w.x : 0.0f, in_y ? w.y : 0.0f);
                    h2[m] = add2(h2[m], w);
                    float2 ql = fma2(q, hr2, hr2);
                    float2 tr = row_floor(ql);
                    tr = make_float2(fminf(fmaxf(tr.x, kFloorMagic), t_max), fminf(fmaxf(tr.y, kFloorMagic), t_max));
                    s2[m] = fma2(w, pair_value(ql, tr), s2[m]);
                }
                        }
            const float nf = (float)n_flat;
            float2 *im = img + sc * (SUB / 2) * THREADS;
#pragma unroll
            for (int m = 0; m < SUB / 2; ++m) {
                float2 hz = add2(h2[m], make_float2(nf, nf));
                float2 rh = make_float2(__fdividef(1.0f, fmaxf(hz.x, 1e-30f)), __fdividef(1.0f, fmaxf(hz.y, 1e-30f)));
                im[m * THREADS] = fma2(s2[m], rh, im[m * THREADS]);
            }
        }
    }
    const size_t plane = (size_t)p.nx * p.ny;
    const size_t pix = (size_t)yi * p.nx + xi;
    float *dst = out_mode == kOutPartial ? p.partial + (size_t)ac * p.n_slices * plane : p.out;
    for (int z = 0; z < nsub * SUB; ++z)
        if (z0 + z < p.n_slices) {
            const float2 v2 = img[(z / 2) * THREADS];
            const float v = (z & 1) ? v2.y : v2.x;
            float *o = dst + (size_t)(z0 + z) * plane + pix;
            switch (out_mode) {
            case kOutScaled: *o = v * p.out_scale; break;
            case kOutMiddle: *o = *o + v; break;
            case kOutLast: *o = (*o + v) * p.out_scale; break;
            default: *o = v;  // kOutPartial, kOutFirst
            }
        }
}

// The angle chunks' partial sums of n voxels added in chunk order and scaled.
__global__ void backproject_combine_kernel(const float *__restrict__ partial, float *__restrict__ out, size_t n,
                                           int chunks, float scale)
{
    for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (size_t)gridDim.x * blockDim.x) {
        float s = partial[v];
        for (int c = 1; c < chunks; ++c) s += partial[(size_t)c * n + v];
        out[v] = s * scale;
    }
}

// Dynamic shared memory of the column form: a geometry entry (24 bytes) per
// thread and half turn of the window (at most nht).
__host__ __device__ constexpr size_t column_geo_bytes(int nht, int threads)
{
    return (size_t)nht * threads * (sizeof(float4) + sizeof(uint2));
}

// grid z: slice chunks x angle chunks (p.n_achunks; more than one writes the
// chunks' partial sums to p.partial)
template <int ZMAX, int SUB, int MIN_BLOCKS, int NOS, int THREADS, bool QUAD>
__global__ void __launch_bounds__(THREADS, MIN_BLOCKS) backproject_column_kernel(BpParams p)
{
    extern __shared__ float4 col_dyn[];
    float4 *geo_w = col_dyn;
    uint2 *geo_a = reinterpret_cast<uint2 *>(col_dyn + (size_t)p.nht * THREADS);
    const int n_zc = (p.n_slices + p.col_zpt - 1) / p.col_zpt;
    const int ac = blockIdx.z / n_zc;
    backproject_column_tile<ZMAX, SUB, NOS, THREADS, QUAD>(p, blockIdx.x, blockIdx.y, blockIdx.z - ac * n_zc, ac,
                                                           p.n_achunks, p.partial ? kOutPartial : kOutScaled,
                                                           geo_w, geo_a);
}

// The blocks of a batch -- blocks of any number of scans -- in one launch:
// grid.x runs over the CTA tiles of every block in turn (tile_start[b] is the
// first tile of block b, tile_start[n_blocks] the total); a CTA finds its
// block, copies the block's parameters to shared memory and runs its tile.
template <int ZPT, int MIN_BLOCKS, int NOS, int THREADS, bool QUAD>
__global__ void __launch_bounds__(THREADS, MIN_BLOCKS)
    backproject_batch_kernel(const BpParams *__restrict__ params, const unsigned *__restrict__ tile_start,
                             int n_blocks)
{
    __shared__ BpParams sp;
    __shared__ int s_block;
    const unsigned tile = blockIdx.x;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    if (tid == 0) {
        int lo = 0, hi = n_blocks - 1;  // the last b with tile_start[b] <= tile
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(tile_start + mid) <= tile) lo = mid;
            else hi = mid - 1;
        }
        s_block = lo;
    }
    __syncthreads();
    const int b = s_block;
    {
        const uint32_t *src = reinterpret_cast<const uint32_t *>(params + b);
        uint32_t *dst = reinterpret_cast<uint32_t *>(&sp);
        for (int w = tid; w < (int)(sizeof(BpParams) / 4); w += THREADS) dst[w] = __ldg(src + w);
    }
    __syncthreads();
    const unsigned local = tile - __ldg(tile_start + b);
    const int cta_h = THREADS / sp.cta_w;
    const unsigned gx = (unsigned)((sp.nx + sp.cta_w - 1) / sp.cta_w);
    const unsigned gy = (unsigned)((sp.ny + cta_h - 1) / cta_h);
    backproject_tile<ZPT, NOS, THREADS, QUAD>(sp, (int)(local % gx), (int)((local / gx) % gy), (int)(local / (gx * gy)));
}

// The column form over a batch's blocks (see backproject_batch_kernel); the
// geometry entries are sized for the batch's largest window (max_nht).
template <int ZMAX, int SUB, int MIN_BLOCKS, int NOS, int THREADS, bool QUAD>
__global__ void __launch_bounds__(THREADS, MIN_BLOCKS)
    backproject_column_batch_kernel(const BpParams *__restrict__ params, const unsigned *__restrict__ tile_start,
                                    int n_blocks, int max_nht, int ac, int n_ac)
{
    __shared__ BpParams sp;
    __shared__ int s_block;
    extern __shared__ float4 col_dyn[];
    const unsigned tile = blockIdx.x;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    if (tid == 0) {
        int lo = 0, hi = n_blocks - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(tile_start + mid) <= tile) lo = mid;
            else hi = mid - 1;
        }
        s_block = lo;
    }
    __syncthreads();
    const int b = s_block;
    {
        const uint32_t *src = reinterpret_cast<const uint32_t *>(params + b);
        uint32_t *dst = reinterpret_cast<uint32_t *>(&sp);
        for (int w = tid; w < (int)(sizeof(BpParams) / 4); w += THREADS) dst[w] = __ldg(src + w);
    }
    __syncthreads();
    const unsigned local = tile - __ldg(tile_start + b);
    const int cta_h = THREADS / sp.cta_w;
    const unsigned gx = (unsigned)((sp.nx + sp.cta_w - 1) / sp.cta_w);
    const unsigned gy = (unsigned)((sp.ny + cta_h - 1) / cta_h);
    float4 *geo_w = col_dyn;
    uint2 *geo_a = reinterpret_cast<uint2 *>(col_dyn + (size_t)max_nht * THREADS);
    const int mode = n_ac == 1 ? kOutScaled : ac == 0 ? kOutFirst : ac == n_ac - 1 ? kOutLast : kOutMiddle;
    backproject_column_tile<ZMAX, SUB, NOS, THREADS, QUAD>(sp, (int)(local % gx), (int)((local / gx) % gy),
                                                           (int)(local / (gx * gy)), ac, n_ac, mode, geo_w, geo_a);
}

// Threads (voxel columns) per CTA of the backprojector: 256 or 128.
int bp_cta_threads()
{
    static int v = [] {
        const char *e = getenv("CTBB_BP_THREADS");
        int t = e ? atoi(e) : 128;
        return t == 256 ? 256 : 128;
    }();
    return v;
}

// Voxel columns along x per CTA of the backprojector (256 columns per CTA).
// Measured on config 2 (ms per 32-slice block): warps of 32 x 1 columns 21.9,
// 16 x 2 20.4, 8 x 4 19.4-19.8, 4 x 8 19.5-19.7; CTAs of 64 x 4 best by 1 %.
int bp_cta_width()
{
    static int v = [] {
        const char *e = getenv("CTBB_BP_CTA_W");
        int w = e ? atoi(e) : 64;
        return (w == 8 || w == 16 || w == 32 || w == 64 || w == 128) ? w : 32;
    }();
    return v;
}

// Voxel columns along x per warp of the backprojector's CTA tile.
int bp_warp_width()
{
    static int v = [] {
        const char *e = getenv("CTBB_BP_WARP_W");
        int w = e ? atoi(e) : 8;
        return (w == 4 || w == 8 || w == 16 || w == 32) ? w : 32;
    }();
    return v;
}

// CTAs per SM the backprojector is compiled for: 128-thread CTAs 7 (72
// registers, default) or 8 (64); 256-thread CTAs 4 (64) or 3 (80).
int bp_min_blocks()
{
    static int v = [] {
        const char *e = getenv("CTBB_BP_MINB");
        return e ? atoi(e) : 7;
    }();
    return v;
}

}  // namespace

int build_backproject_tables(const struct recon_metadata &mr, BackprojectTables *t)
{
    const struct ct_geom &cg = mr.cg;
    const struct recon_params &rp = mr.rp;
    const float pi = kPiBackproject;
    BlockDims d = block_dims(mr);
    if (d.n_half_turns <= 0) {
        set_error("backproject: pull window holds no complete half turn");
        return CTBB_ERR_STATE;
    }
    t->tube_start = bp_tube_start(mr);
    t->nht = d.n_half_turns;
    t->n_half = (int)(cg.n_proj_turn / 2);
    t->n_slices = (int)mr.ri.n_slices_block;
    t->views.resize((size_t)t->n_half * t->nht * 4);
    t->theta.resize((size_t)t->n_half * t->nht);
    for (int i = 0; i < t->n_half; ++i)
        for (int k = 0; k < t->nht; ++k) {
            // src/backproject_cpu.cu:102-103
            float theta = t->tube_start + (2.0f * pi / (float)cg.n_proj_turn) * (float)i + (float)k * pi;
            float *v = &t->views[((size_t)i * t->nht + k) * 4];
            t->set_view_row(i, k, (unsigned)(i + k * t->n_half));
            t->theta[(size_t)i * t->nht + k] = theta;
            v[1] = std::sin(theta);
            v[2] = std::cos(theta);
            v[3] = theta * (cg.z_rot / (2.0f * pi));  // theta z_rot / 2 pi': the ray's table term
        }
    t->zpos.resize(t->n_slices);
    for (int zi = 0; zi < t->n_slices; ++zi)  // src/backproject_cpu.cu:107
        t->zpos[zi] = (float)zi * rp.coll_slicewidth + cg.z_rot / 2.0f +
                      cg.z_rot * t->tube_start / (2.0f * pi);
    return CTBB_OK;
}

void BackprojectTables::set_view_row(int i, int k, unsigned row)
{
    uint32_t bits = row;
    std::memcpy(&views[((size_t)i * nht + k) * 4], &bits, sizeof(bits));
}

int make_backproject_params(const struct recon_metadata &mr, const BackprojectTables &t, const float4 *d_views,
                            const float *d_theta, const float *d_zpos, const float *d_rebin, float *d_block,
                            const float *d_vscale, const BpShape &shape, BpParams *pp)
{
    const bool quad = d_vscale != nullptr;
    const struct ct_geom &cg = mr.cg;
    const struct recon_params &rp = mr.rp;
    const float pi = kPiBackproject;
    BpParams &p = *pp;
    std::memset(&p, 0, sizeof(p));
    p.rebin = d_rebin;
    p.vscale = d_vscale;
    // row_floor's addressing: the base moved back by kFloorMagicBits rows,
    // modulo 2^64 (every row address comes back inside the buffer)
    p.rebin_rows = (uint64_t)(uintptr_t)d_rebin - (uint64_t)kFloorMagicBits * (uint64_t)cg.n_channels_oversampled *
                                                      (quad ? sizeof(uint2) : sizeof(float));
    p.out = d_block;
    p.views = d_views;
    p.theta = d_theta;
    p.zpos = d_zpos;
    p.nx = (int)rp.nx;
    p.ny = (int)rp.ny;
    p.n_slices = t.n_slices;
    p.nos = (int)cg.n_channels_oversampled;
    p.n_rows = (int)cg.n_rows;
    p.nht = t.nht;
    p.n_half = t.n_half;
    p.pix_x = rp.recon_fov / (float)rp.nx;
    p.pix_y = rp.recon_fov / (float)rp.ny;
    p.x_c = (float)(rp.nx - 1) / 2.0f;
    p.y_c = (float)(rp.ny - 1) / 2.0f;
    p.x0 = rp.x_origin;
    p.y0 = rp.y_origin;
    p.ds_half = cg.r_f * cg.fan_angle_increment / 2.0f;
    p.inv_ds_half = 1.0f / p.ds_half;
    p.coll = rp.coll_slicewidth;
    p.two_cc = 2.0f * cg.central_channel;
    p.rf = cg.r_f;
    p.inv_rf = 1.0f / cg.r_f;
    p.rf2 = std::pow(cg.r_f, 2.0f);
    p.z_rot = cg.z_rot;
    p.two_pi = 2.0f * pi;
    p.zrot_over_2pi = cg.z_rot / (2.0f * pi);
    p.tan_cone = std::tan(cg.theta_cone / 2.0f);
    p.half_rows = ((float)cg.n_rows - 1.0f) / 2.0f;
    // |q| <= Q maps to rows within (R-1)(1 +- Q)/2; for R >= 8 that is inside
    // [0, R-2] with a margin of more than a tenth of a row, including the
    // last-turn border at R-2
    p.flat_path = cg.n_rows >= 8 ? 1 : 0;
    p.k_window = std::fabs(cg.z_rot) > 1e-3f ? 1 : 0;
    p.abs_zr = std::fabs(p.zrot_over_2pi);
    p.inv_half_feed = p.k_window ? 2.0f / cg.z_rot : 0.0f;
    p.taper_scale = (pi / 2.0f) / (1.0f - kQ);
    p.out_scale = 2.0f * pi / (float)cg.n_proj_turn;
    if (p.n_rows < 2 || p.nos < 2) {
        set_error("backproject: detector too small");
        return CTBB_ERR_ARGUMENT;
    }
    p.col_zpt = (shape.col && t.nht <= kColumnMaxHalfTurns) ? shape.zpt : 0;
    p.n_achunks = 1;
    p.partial = nullptr;
    p.warp_w = shape.warp_w;
    p.cta_w = std::max(shape.cta_w, p.warp_w);
    if (shape.threads / p.cta_w < 32 / p.warp_w) p.cta_w = (shape.threads / 32) * p.warp_w;  // whole warp tiles in y
    return CTBB_OK;
}

namespace {

dim3 grid_of(const BpParams &p, const BpShape &s)
{
    const int cta_h = s.threads / p.cta_w;
    return dim3((p.nx + p.cta_w - 1) / p.cta_w, (p.ny + cta_h - 1) / cta_h,
                ((p.n_slices + s.zpt - 1) / s.zpt) * (s.col ? std::max(p.n_achunks, 1) : 1));
}

// Calls f(Z, MB, T, QUAD) with the compile-time instance of a launch shape;
// CTBB_ERR_ARGUMENT for a shape no kernel was compiled for.  batch: the
// instances the batch kernel is compiled for (a subset).
template <class F>
int with_shape(const BpShape &s, bool quad, bool batch, F &&f)
{
    using std::integral_constant;
    auto I = [](auto v) { return v; };
    (void)I;
    if (quad) {
        if (s.zpt == 8 && s.threads == 128 && s.min_blocks == 7)
            return f(integral_constant<int, 8>(), integral_constant<int, 7>(), integral_constant<int, 128>(),
                     std::true_type());
    } else if (s.zpt == 8 && s.threads == 128 && s.min_blocks == 7) {
        return f(integral_constant<int, 8>(), integral_constant<int, 7>(), integral_constant<int, 128>(),
                 std::false_type());
    } else if (s.zpt == 8 && s.threads == 256 && s.min_blocks == 4) {
        return f(integral_constant<int, 8>(), integral_constant<int, 4>(), integral_constant<int, 256>(),
                 std::false_type());
    } else if (s.zpt == 16 && s.threads == 256 && s.min_blocks == 3) {
        return f(integral_constant<int, 16>(), integral_constant<int, 3>(), integral_constant<int, 256>(),
                 std::false_type());
    } else if (!batch) {
        if (s.zpt == 8 && s.threads == 128 && s.min_blocks == 8)
            return f(integral_constant<int, 8>(), integral_constant<int, 8>(), integral_constant<int, 128>(),
                     std::false_type());
        if (s.zpt == 8 && s.threads == 256 && s.min_blocks == 3)
            return f(integral_constant<int, 8>(), integral_constant<int, 3>(), integral_constant<int, 256>(),
                     std::false_type());
        if (s.zpt == 16 && s.threads == 256 && s.min_blocks == 2)
            return f(integral_constant<int, 16>(), integral_constant<int, 2>(), integral_constant<int, 256>(),
                     std::false_type());
        if (s.zpt == 4 && s.threads == 256 && s.min_blocks == 3)
            return f(integral_constant<int, 4>(), integral_constant<int, 3>(), integral_constant<int, 256>(),
                     std::false_type());
    }
    set_error("backproject: no kernel for %d slices per thread, %d threads, %d CTAs per SM%s%s", s.zpt, s.threads,
              s.min_blocks, quad ? " (FP16 footprint rows)" : "", batch ? " (batch)" : "");
    return CTBB_ERR_ARGUMENT;
}

}  // namespace

// Backprojector form: the column form unless CTBB_BP_FORM=tile.
bool bp_column_form()
{
    static bool v = [] {
        const char *e = getenv("CTBB_BP_FORM");
        return !(e && strcmp(e, "tile") == 0);
    }();
    return v;
}

// Slices per thread of the column form (32; 16 or 8).
int bp_column_zpt()
{
    static int v = [] {
        const char *e = getenv("CTBB_BP_COL_ZPT");
        int z = e ? atoi(e) : 32;
        return (z == 8 || z == 16 || z == 32) ? z : 32;
    }();
    return v;
}

BpShape fit_bp_shape(const BpShape &s, int nht)
{
    if (!s.col || nht <= kColumnMaxHalfTurns) return s;
    BpShape t;  // the slice-chunk form's default
    t.cta_w = s.cta_w;
    t.warp_w = s.warp_w;
    return t;
}

BpShape window_bp_shape(int zpt, bool quad, int nht)
{
    BpShape s = default_bp_shape(zpt, quad);
    if (s.col && nht <= kColumnMaxHalfTurns && s.zpt == 32) {
        // Measured per window on 256^2 and 512^2 blocks of 16-64 detector rows
        // (FP32 rows and FP16 words alike), against 32 slices at 8 CTAs per
        // SM: 16 slices per thread 11-13 % faster at 6-7 half turns and 2-6 %
        // at 5; 7 CTAs per SM 0.5-1.7 % faster at 4; at 2-3 half turns 32
        // slices at 8 CTAs are the fastest.
        static const bool zpt_named = getenv("CTBB_BP_COL_ZPT") != nullptr;
        static const bool minb_named = getenv("CTBB_BP_MINB") != nullptr;
        if (nht >= 5 && !zpt_named) {
            s.zpt = 16;
            s.min_blocks = 8;
        } else if (nht == 4 && !minb_named && s.min_blocks == 8) {
            s.min_blocks = 7;
        }
    }
    return fit_bp_shape(s, nht);
}

BpShape default_bp_shape(int zpt, bool quad)
{
    if (bp_column_form()) {
        BpShape s;
        s.col = 1;
        s.zpt = bp_column_zpt();
        s.threads = 128;
        // 8 CTAs per SM (64 registers) unless CTBB_BP_MINB names 6 or 7
        const int mb = getenv("CTBB_BP_MINB") ? bp_min_blocks() : 8;
        s.min_blocks = mb == 6 ? 6 : (mb == 7 ? 7 : 8);
        // CTAs of 16 x 8 voxel columns unless CTBB_BP_CTA_W names the width
        s.cta_w = getenv("CTBB_BP_CTA_W") ? bp_cta_width() : 16;
        s.warp_w = bp_warp_width();
        // the half-turn angles in 16 chunks unless CTBB_BP_ACHUNKS names 1-16
        const char *a = getenv("CTBB_BP_ACHUNKS");
        const int ach = a ? atoi(a) : 16;
        s.achunks = (ach >= 1 && ach <= kMaxAngleChunks) ? ach : 16;
        return s;
    }
    if (quad) return BpShape{};
    BpShape s;
    s.zpt = (zpt == 4 || zpt == 16) ? zpt : 8;
    s.threads = s.zpt == 8 ? bp_cta_threads() : 256;
    if (s.zpt == 8) s.min_blocks = s.threads == 128 ? (bp_min_blocks() == 8 ? 8 : 7) : (bp_min_blocks() == 3 ? 3 : 4);
    else s.min_blocks = (s.zpt == 16 && bp_min_blocks() == 2) ? 2 : 3;
    s.cta_w = bp_cta_width();
    s.warp_w = bp_warp_width();
    return s;
}

// The column form's instances: 128-thread CTAs, at most 32 slices per thread
// at 8 (64 registers), 7 or 6 CTAs per SM, or at most 16 slices at 8.
// f(ZMAX, SUB, MIN_BLOCKS).
template <class F>
int with_column_shape(const BpShape &s, F &&f)
{
    using std::integral_constant;
    if (s.col && s.threads == 128 && (s.zpt == 8 || s.zpt == 16 || s.zpt == 32)) {
        if (s.min_blocks == 7)
            return f(integral_constant<int, 32>(), integral_constant<int, 8>(), integral_constant<int, 7>());
        if (s.min_blocks == 6)
            return f(integral_constant<int, 32>(), integral_constant<int, 8>(), integral_constant<int, 6>());
        if (s.min_blocks == 8 && s.zpt <= 16)
            return f(integral_constant<int, 16>(), integral_constant<int, 8>(), integral_constant<int, 8>());
        if (s.min_blocks == 8)
            return f(integral_constant<int, 32>(), integral_constant<int, 8>(), integral_constant<int, 8>());
    }
    set_error("backproject: no column-form kernel for %d slices per thread, %d threads, %d CTAs per SM", s.zpt,
              s.threads, s.min_blocks);
    return CTBB_ERR_ARGUMENT;
}

size_t backproject_partial_bytes(const BpParams &p, const BpShape &shape)
{
    if (!shape.col || shape.achunks <= 1) return 0;
    return (size_t)shape.achunks * p.n_slices * p.nx * p.ny * sizeof(float);
}

int launch_backproject_params(const BpParams &p_in, const BpShape &shape, cudaStream_t stream, void *scratch,
                              size_t scratch_bytes)
{
    BpParams p = p_in;
    p.n_achunks = 1;
    p.partial = nullptr;
    const size_t part_bytes = backproject_partial_bytes(p, shape);
    if (part_bytes && scratch && scratch_bytes >= part_bytes && shape.achunks <= p.n_half) {
        p.n_achunks = shape.achunks;
        p.partial = static_cast<float *>(scratch);
    }
    const bool quad = p.vscale != nullptr;
    const dim3 grid = grid_of(p, shape);
    const dim3 block(32, shape.threads / 32);
    if (shape.col) {
        if (p.nht > kColumnMaxHalfTurns || p.col_zpt != shape.zpt) {
            set_error("backproject: column form needs at most %d half turns (%d) and matching parameters",
                      kColumnMaxHalfTurns, p.nht);
            return CTBB_ERR_ARGUMENT;
        }
        const size_t smem = column_geo_bytes(p.nht, 128);
        CTBB_TRY(with_column_shape(shape, [&](auto zm, auto sb, auto mb) -> int {
            constexpr int ZM = decltype(zm)::value, SB = decltype(sb)::value, MB = decltype(mb)::value;
            // at most 24 KB of geometry beside the image sums (16 KB at most):
            // within the default 48 KB, no attribute needed
            if (quad) {
                if (p.nos == 1472) backproject_column_kernel<ZM, SB, MB, 1472, 128, true><<<grid, block, smem, stream>>>(p);
                else backproject_column_kernel<ZM, SB, MB, 0, 128, true><<<grid, block, smem, stream>>>(p);
            } else if (p.nos == 1472) {
                backproject_column_kernel<ZM, SB, MB, 1472, 128, false><<<grid, block, smem, stream>>>(p);
            } else if (p.nos == 1344) {
                backproject_column_kernel<ZM, SB, MB, 1344, 128, false><<<grid, block, smem, stream>>>(p);
            } else {
                backproject_column_kernel<ZM, SB, MB, 0, 128, false><<<grid, block, smem, stream>>>(p);
            }
            return CTBB_OK;
        }));
        count_launch();
        CTBB_CUDA_TRY(cudaGetLastError());
        if (p.partial) {
            const size_t n = (size_t)p.n_slices * p.nx * p.ny;
            const unsigned blocks = (unsigned)std::min<size_t>((n + 255) / 256, 152 * 16);
            backproject_combine_kernel<<<blocks, 256, 0, stream>>>(p.partial, p.out, n, p.n_achunks, p.out_scale);
            count_launch();
            CTBB_CUDA_TRY(cudaGetLastError());
        }
        return CTBB_OK;
    }
    CTBB_TRY(with_shape(shape, quad, false, [&](auto z, auto mb, auto t, auto q) -> int {
        constexpr int Z = decltype(z)::value, MB = decltype(mb)::value, T = decltype(t)::value;
        constexpr bool Q = decltype(q)::value;
        if (p.nos == 1472) backproject_kernel<Z, MB, 1472, T, Q><<<grid, block, 0, stream>>>(p);
        else if (p.nos == 1344) backproject_kernel<Z, MB, 1344, T, Q><<<grid, block, 0, stream>>>(p);
        else backproject_kernel<Z, MB, 0, T, Q><<<grid, block, 0, stream>>>(p);
        return CTBB_OK;
    }));
    count_launch();
    CTBB_CUDA_TRY(cudaGetLastError());
    return CTBB_OK;
}

int launch_backproject(const struct recon_metadata &mr, const BackprojectTables &t,
                       const float4 *d_views, const float *d_theta, const float *d_zpos, const float *d_rebin,
                       float *d_block, int zpt, cudaStream_t stream, const float *d_vscale, const BpShape *shape,
                       void *scratch, size_t scratch_bytes)
{
    const BpShape s = shape ? fit_bp_shape(*shape, t.nht) : window_bp_shape(zpt, d_vscale != nullptr, t.nht);
    BpParams p;
    CTBB_TRY(make_backproject_params(mr, t, d_views, d_theta, d_zpos, d_rebin, d_block, d_vscale, s, &p));
    return launch_backproject_params(p, s, stream, scratch, scratch_bytes);
}

size_t backproject_batch_bytes(size_t n_blocks) { return n_blocks * sizeof(BpParams) + (n_blocks + 1) * 4 + 256; }

int launch_backproject_batch(const std::vector<BpParams> &blocks, const BpShape &shape, void *d_buf, size_t buf_bytes,
                             cudaStream_t stream)
{
    if (blocks.empty()) return CTBB_OK;
    const bool quad = blocks[0].vscale != nullptr;
    for (const BpParams &p : blocks)
        if ((p.vscale != nullptr) != quad || p.nos != blocks[0].nos) {
            set_error("backproject batch: blocks of different row storage or row length");
            return CTBB_ERR_ARGUMENT;
        }
    if (backproject_batch_bytes(blocks.size()) > buf_bytes) {
        set_error("backproject batch: parameter buffer too small");
        return CTBB_ERR_ARGUMENT;
    }
    std::vector<unsigned> start(blocks.size() + 1, 0);
    for (size_t b = 0; b < blocks.size(); ++b) {
        dim3 g = grid_of(blocks[b], shape);
        unsigned long long next = (unsigned long long)start[b] + (unsigned long long)g.x * g.y * g.z;
        if (next >= (1ull << 31)) {
            set_error("backproject batch: more than 2^31 CTA tiles");
            return CTBB_ERR_ARGUMENT;
        }
        start[b + 1] = (unsigned)next;
    }
    BpParams *d_params = static_cast<BpParams *>(d_buf);
    unsigned *d_start = reinterpret_cast<unsigned *>(d_params + blocks.size());
    int max_nht = 0;
    for (const BpParams &p : blocks) {
        if (shape.col && (p.col_zpt != shape.zpt || p.nht > kColumnMaxHalfTurns)) {
            set_error("backproject batch: a block's parameters do not fit the column form");
            return CTBB_ERR_ARGUMENT;
        }
        max_nht = std::max(max_nht, p.nht);
    }
    CTBB_CUDA_TRY(cudaMemcpyAsync(d_params, blocks.data(), blocks.size() * sizeof(BpParams), cudaMemcpyHostToDevice,
                                  stream));
    CTBB_CUDA_TRY(cudaMemcpyAsync(d_start, start.data(), start.size() * sizeof(unsigned), cudaMemcpyHostToDevice,
                                  stream));
    const unsigned total = start.back();
    const dim3 block(32, shape.threads / 32);
    const int nos = blocks[0].nos, n = (int)blocks.size();
    if (shape.col) {
        // the angle chunks one launch after another, each over every block's
        // tiles, each adding to the blocks' images (the CTAs in flight then
        // share a chunk's views)
        int n_ac = std::max(1, shape.achunks);
        for (const BpParams &p : blocks) n_ac = std::min(n_ac, p.n_half);
        const size_t smem = column_geo_bytes(max_nht, 128);
        for (int ac = 0; ac < n_ac; ++ac) {
            CTBB_TRY(with_column_shape(shape, [&](auto zm, auto sb, auto mb) -> int {
                constexpr int ZM = decltype(zm)::value, SB = decltype(sb)::value, MB = decltype(mb)::value;
                if (quad) {
                    if (nos == 1472)
                        backproject_column_batch_kernel<ZM, SB, MB, 1472, 128, true><<<total, block, smem, stream>>>(
                            d_params, d_start, n, max_nht, ac, n_ac);
                    else
                        backproject_column_batch_kernel<ZM, SB, MB, 0, 128, true><<<total, block, smem, stream>>>(
                            d_params, d_start, n, max_nht, ac, n_ac);
                } else if (nos == 1472) {
                    backproject_column_batch_kernel<ZM, SB, MB, 1472, 128, false><<<total, block, smem, stream>>>(
                        d_params, d_start, n, max_nht, ac, n_ac);
                } else {
                    backproject_column_batch_kernel<ZM, SB, MB, 0, 128, false><<<total, block, smem, stream>>>(
                        d_params, d_start, n, max_nht, ac, n_ac);
                }
                return CTBB_OK;
            }));
            count_launch();
            CTBB_CUDA_TRY(cudaGetLastError());
        }
        return CTBB_OK;
    }
    CTBB_TRY(with_shape(shape, quad, true, [&](auto z, auto mb, auto t, auto q) -> int {
        constexpr int Z = decltype(z)::value, MB = decltype(mb)::value, T = decltype(t)::value;
        constexpr bool Q = decltype(q)::value;
        if (nos == 1472) backproject_batch_kernel<Z, MB, 1472, T, Q><<<total, block, 0, stream>>>(d_params, d_start, n);
        else backproject_batch_kernel<Z, MB, 0, T, Q><<<total, block, 0, stream>>>(d_params, d_start, n);
        return CTBB_OK;
    }));
    count_launch();
    CTBB_CUDA_TRY(cudaGetLastError());
    // the host vectors above are copied from pageable memory: the copies are
    // staged before cudaMemcpyAsync returns
    return CTBB_OK;
}

std::vector<BpShape> backproject_shape_candidates(bool quad)
{
    // 128-thread CTAs are 32 x 4 (cta_w 32) or 16 x 8 (cta_w 16) voxel columns
    std::vector<BpShape> c;
    c.push_back(BpShape{32, 128, 8, 16, 8, 1, 16});
    c.push_back(BpShape{32, 128, 7, 16, 8, 1, 16});
    c.push_back(BpShape{32, 128, 8, 32, 8, 1, 16});
    c.push_back(BpShape{32, 128, 7, 32, 8, 1, 16});
    c.push_back(BpShape{32, 128, 7, 16, 8, 1, 8});
    c.push_back(BpShape{16, 128, 8, 16, 8, 1, 16});
    c.push_back(BpShape{8, 128, 7, 32, 8, 0});
    return c;
}

}  // namespace ctbb
