// rebin.cu -- flying-focal-spot split + fan-to-parallel rebinning.
//
// One fused gather kernel per FFS mode replaces the reference's reshape /
// azimuthal / radial kernel chain (src/rebin_filter.cu:58-912) and the CPU twin
// it must match (src/rebin_filter_cpu.cu:95-645):
//
//   * no FFS  (rebin_nffs_cpu :95-159) and z-FFS (rebin_zffs_cpu :290-416):
//     one bilinear sample in (channel, view) per output sample;
//   * phi-FFS (rebin_pffs_cpu :161-288) and phi+z-FFS (rebin_affs_cpu :418-645):
//     the reference first rebins azimuthally into an oversampled intermediate
//     (channels 2ch / 2ch+1 from the +da / -da focal spots) and then radially
//     along that intermediate's channel axis.  Here each output sample evaluates
//     the two intermediate samples it needs on the fly, so the intermediate is
//     never stored.
//
// Geometry-only quantities (fan angles, beta_lookup search, view offsets) are
// computed on the host with the reference's float expressions; the kernels do
// clamps, floors, multiplies and adds only, written with __f*_rn intrinsics so
// that no multiply-add is fused.  The unfiltered result is therefore bit-exact
// with the reference CPU path compiled without FMA contraction.
//
// A thread covers one output channel, 8 views and 4 raw rows: the view-axis
// taps of a (channel, view) are computed once for its rows.  A launch may
// cover a range of views (the streamed whole-scan path).
//
// Output layout: rebin[view][out_row][channel_os], views = n_proj/n_ffs -
// 2*add_projections (the leading add_projections views are dropped, as the
// reference's copy loops do, e.g. src/rebin_filter_cpu.cu:119-131).
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "ctbb_internal.h"
#include "cuda_util.cuh"
#include "rebin.h"

namespace ctbb {

namespace {

// ---- host restatements of the reference's float geometry helpers ----------
// src/rebin_filter_cpu.cu:37-65.  C++ overloads as in the reference: pow(2.0f,
// int) promotes to double, so b0 is computed in double and rounded to float.

float angle_f(float x1, float x2, float y1, float y2)
{
    return std::asin((x1 * y2 - x2 * y1) / (std::sqrt(x1 * x1 + x2 * x2) * std::sqrt(y1 * y1 + y2 * y2)));
}

float beta_rk_f(float da, float dr, float channel, int os_flag, const struct ct_geom &cg)
{
    float b0 = (float)((channel - std::pow(2.0f, os_flag) * cg.central_channel) *
                       (cg.fan_angle_increment / std::pow(2.0f, os_flag)));
    return angle_f(-(cg.r_f + dr), -(da), -(cg.src_to_det * std::cos(b0) + dr),
                   -(cg.src_to_det * std::sin(b0) + da));
}

float d_alpha_r_f(float da, float dr, const struct ct_geom &cg)
{
    return angle_f(cg.r_f, 0, cg.r_f + dr, da);
}

float r_fr_f(float da, float dr, const struct ct_geom &cg)
{
    return std::sqrt((cg.r_f + dr) * (cg.r_f + dr) + da * da);
}

float get_beta_idx_f(float beta, const float *lookup, int n)
{
    int lo = 0;
    while (beta > lookup[lo] && lo < (n - 1)) lo++;
    if (lo == 0) lo++;
    return (float)lo - 1.0f + (beta - lookup[lo - 1]) / (lookup[lo] - lookup[lo - 1]);
}

// Clamp + floor + alias rule of interp3 (src/interp.cu:66-130) along one axis
// whose coordinate does not depend on the view: base tap, upper tap and
// weight, evaluated exactly as interp3 does.
void axis_taps(float idx, int dim, int *i0, int *i1, float *u, float *one_minus_u)
{
    if (idx > (float)(dim - 1)) idx = (float)dim - 1.0f;
    if (idx < 0) idx = 0.0f;
    float fl = std::floor(idx);
    *u = idx - fl;
    *one_minus_u = 1.0f - *u;
    *i0 = (int)fl;
    *i1 = (idx == (float)dim - 1.0f) ? *i0 : *i0 + 1;
}

}  // namespace

// --------------------------------------------------------------------------
// Host tables
// --------------------------------------------------------------------------

int build_rebin_tables(const struct recon_metadata &mr, RebinTables *t)
{
    const struct ct_geom &cg = mr.cg;
    const struct recon_params &rp = mr.rp;
    const int N = (int)cg.n_channels, Nos = (int)cg.n_channels_oversampled;
    const float pi = kPiRebin;
    const float two_pi = 2.0f * pi;
    t->n_ffs = (int)mr.ri.n_ffs;
    t->n_channels = N;
    t->n_os = Nos;
    t->n_rows_raw = (int)cg.n_rows_raw;
    t->n_rows = (int)cg.n_rows;
    t->n_proj = (int)(mr.ri.n_proj_pull / mr.ri.n_ffs);
    t->add_projections = (int)cg.add_projections;
    t->n_views = t->n_proj - 2 * t->add_projections;
    t->reverse_rows = cg.reverse_row_interleave ? 1 : 0;
    if (t->n_views <= 0) {
        set_error("rebin: pull window of %zu frames keeps no views", mr.ri.n_proj_pull);
        return CTBB_ERR_STATE;
    }
    t->out_taps.assign(2 * (size_t)Nos, AxisTap{});
    t->focal.assign(4 * (size_t)N, FocalTerm{});
    t->focal_offset.assign(4, 0.0f);

    auto set_tap = [&](int s, int c, float bidx, int dim) {
        AxisTap &a = t->out_taps[(size_t)s * Nos + c];
        axis_taps(bidx, dim, &a.i0, &a.i1, &a.u, &a.one_minus_u);
    };

    if (t->n_ffs == 1) {
        // rebin_nffs_cpu :107-117
        t->mode = RebinMode::kNoFfs;
        t->focal.assign((size_t)Nos, FocalTerm{});
        for (int c = 0; c < Nos; ++c) {
            const float beta = std::asin(((float)c - 2 * cg.central_channel) * (cg.fan_angle_increment / 2));
            float beta_idx = beta / cg.fan_angle_increment + cg.central_channel;
            set_tap(0, c, beta_idx, N);
            t->focal[c].t_alpha = beta * (float)cg.n_proj_turn / (2.0f * pi);
        }
    } else if (t->n_ffs == 2 && rp.z_ffs == 1) {
        // rebin_zffs_cpu :297-352
        t->mode = RebinMode::kZFfs;
        const double da = 0.0;
        const double dr = cg.src_to_det * rp.coll_slicewidth /
                          (4.0 * (cg.src_to_det - cg.r_f) * std::tan(cg.anode_angle));
        std::vector<float> lk1(N), lk2(N);
        for (int i = 0; i < N; i++) {
            lk1[i] = beta_rk_f((float)da, (float)-dr, (float)i, 0, cg);
            lk2[i] = beta_rk_f((float)da, (float)dr, (float)i, 0, cg);
        }
        t->focal.assign(2 * (size_t)Nos, FocalTerm{});
        float dal1 = d_alpha_r_f((float)da, (float)-dr, cg) * (float)cg.n_proj_ffs / (2.0f * pi);
        float dal2 = d_alpha_r_f((float)da, (float)dr, cg) * (float)cg.n_proj_ffs / (2.0f * pi);
        t->focal_offset[0] = dal1;
        t->focal_offset[1] = dal2;
        for (int c = 0; c < Nos; ++c) {
            float b1 = std::asin(((float)c - 2.0f * cg.central_channel) * (cg.fan_angle_increment / 2.0f) *
                                 cg.r_f / r_fr_f(0.0f, (float)-dr, cg));
            float b2 = std::asin(((float)c - 2.0f * cg.central_channel) * (cg.fan_angle_increment / 2.0f) *
                                 cg.r_f / r_fr_f(0.0f, (float)dr, cg));
            set_tap(0, c, get_beta_idx_f(b1, lk1.data(), N), N);
            set_tap(1, c, get_beta_idx_f(b2, lk2.data(), N), N);
            t->focal[c].t_alpha = b1 * (float)cg.n_proj_ffs / (2.0f * pi);
            t->focal[(size_t)Nos + c].t_alpha = b2 * (float)cg.n_proj_ffs / (2.0f * pi);
        }
    } else if (t->n_ffs == 2) {
        // rebin_pffs_cpu :165-246
        t->mode = RebinMode::kPhiFfs;
        const double da = cg.src_to_det * cg.r_f * cg.fan_angle_increment /
                          (4.0f * (cg.src_to_det - cg.r_f));
        std::vector<float> lookup(Nos);
        float dal_p = d_alpha_r_f((float)da, 0, cg) * (float)cg.n_proj_ffs / (2.0f * pi);
        float dal_m = d_alpha_r_f((float)-da, 0, cg) * (float)cg.n_proj_ffs / (2.0f * pi);
        t->focal_offset[0] = dal_p;
        t->focal_offset[1] = dal_m;
        for (int ch = 0; ch < N; ++ch) {
            float b1 = beta_rk_f((float)da, 0, (float)ch, 0, cg);
            float b2 = beta_rk_f((float)-da, 0, (float)ch, 0, cg);
            lookup[2 * ch] = b1;
            lookup[2 * ch + 1] = b2;
            t->focal[0 * (size_t)N + ch].t_alpha = b1 * (float)cg.n_proj_ffs / (2.0f * pi);
            t->focal[1 * (size_t)N + ch].t_alpha = b2 * (float)cg.n_proj_ffs / (2.0f * pi);
        }
        for (int c = 0; c < Nos; ++c) {
            float beta = std::asin((c - 2 * cg.central_channel) * (cg.fan_angle_increment / 2));
            set_tap(0, c, get_beta_idx_f(beta, lookup.data(), Nos), Nos);
        }
    } else if (t->n_ffs == 4) {
        // rebin_affs_cpu :424-601
        t->mode = RebinMode::kBothFfs;
        const double da = cg.src_to_det * cg.r_f * cg.fan_angle_increment /
                          (4.0f * (cg.src_to_det - cg.r_f));
        const double dr = cg.src_to_det * rp.coll_slicewidth /
                          (4.0 * (cg.src_to_det - cg.r_f) * std::tan(cg.anode_angle));
        std::vector<float> lk1(Nos), lk2(Nos);
        // focal order within a group of 4 frames: (+da,-dr) (-da,-dr) (+da,+dr) (-da,+dr)
        const float sda[4] = {(float)da, (float)-da, (float)da, (float)-da};
        const float sdr[4] = {(float)-dr, (float)-dr, (float)dr, (float)dr};
        for (int q = 0; q < 4; ++q)
            t->focal_offset[q] = d_alpha_r_f(sda[q], sdr[q], cg) * (float)cg.n_proj_ffs / (2.0f * pi);
        for (int ch = 0; ch < N; ++ch) {
            for (int q = 0; q < 4; ++q) {
                float b = beta_rk_f(sda[q], sdr[q], (float)ch, 0, cg);
                t->focal[(size_t)q * N + ch].t_alpha = b * (float)cg.n_proj_ffs / (2.0f * pi);
                if (q < 2) lk1[2 * ch + q] = b;
                else lk2[2 * ch + (q - 2)] = b;
            }
        }
        for (int c = 0; c < Nos; ++c) {
            float b1 = std::asin((c - 2 * cg.central_channel) * (cg.fan_angle_increment / 2) * cg.r_f /
                                 r_fr_f(0.0f, (float)-dr, cg));
            float b2 = std::asin((c - 2 * cg.central_channel) * (cg.fan_angle_increment / 2) * cg.r_f /
                                 r_fr_f(0.0f, (float)dr, cg));
            set_tap(0, c, get_beta_idx_f(b1, lk1.data(), Nos), Nos);
            set_tap(1, c, get_beta_idx_f(b2, lk2.data(), Nos), Nos);
        }
    } else {
        set_error("rebin: unsupported n_ffs %d", t->n_ffs);
        return CTBB_ERR_CONFIG;
    }
    (void)two_pi;
    return CTBB_OK;
}

// --------------------------------------------------------------------------
// Device helpers
// --------------------------------------------------------------------------

struct RebinParams {
    const float *raw;           // [P][R_raw][N]
    float *out;                 // [V][R][Nos]
    const AxisTap *taps;        // [2][Nos]
    const FocalTerm *focal;     // mode dependent
    float focal_offset[4];
    int n_ffs, N, Nos, R_raw, R, n_proj, add, n_views, reverse_rows;
    int split_view_coord;
    int v_begin, v_end;  // views this launch writes
};

// View-axis coordinate of focal spot q at view proj, divided down to the index
// of that focal spot's own frame sequence (src/rebin_filter_cpu.cu:210-219, :346-356,
// :519-544): ((n_ffs*proj - t_alpha) - t_offset - q) / n_ffs.
__device__ __forceinline__ float focal_alpha(int n_ffs, int proj, float t_alpha, float t_off, int q)
{
    float a = __fsub_rn(__fsub_rn((float)(n_ffs * proj), t_alpha), t_off);
    if (q) a = __fsub_rn(a, (float)q);
    return n_ffs == 1 ? a : __fmul_rn(a, n_ffs == 2 ? 0.5f : 0.25f);
}

// interp3 taps along the view axis (clamp to [0, n-1], alias at the edge).
__device__ __forceinline__ void view_taps(float a, int n, int *i0, int *i1, float *w)
{
    if (a > (float)(n - 1)) a = (float)n - 1.0f;
    if (a < 0.0f) a = 0.0f;
    float fl = floorf(a);
    *w = __fsub_rn(a, fl);
    *i0 = (int)fl;
    *i1 = (a == (float)n - 1.0f) ? *i0 : *i0 + 1;
}

// The same taps from the coordinate ((n_ffs proj - t_alpha) - t_off - q) /
// n_ffs evaluated in split form.  In float that expression rounds at the
// magnitude of n_ffs proj: within one block's pull window (proj below ~2500)
// to 5e-4 frames, but in the whole-scan union (proj up to ~11000 at 40
// turns) to 4e-3 frames, which moves the view weights of the later blocks by
// up to 1e-3.  Here c = t_alpha + t_off + q (a few hundred frames) is split
// into floor(c) and the exact remainder c - floor(c); n_ffs proj - floor(c)
// is an exact integer J = n_ffs Q + m with 0 <= m < n_ffs, and the coordinate
// is Q + (m - (c - floor(c))) / n_ffs, whose fraction is rounded at a
// magnitude below n_ffs.  The result differs from the exact coordinate by
// about 1e-7 views, from any block's own float coordinate by at most that
// block's rounding.  Same clamp and edge alias as view_taps.
__device__ __forceinline__ void view_taps_split(int n_ffs, int proj, float t_alpha, float t_off, int q, int n,
                                                int *i0, int *i1, float *w)
{
    float c = __fadd_rn(__fadd_rn(t_alpha, t_off), (float)q);
    float cf = floorf(c);
    float c_frac = __fsub_rn(c, cf);  // exact: same binade or finer
    int J = n_ffs * proj - (int)cf;
    // floor(J / n_ffs) and its remainder, n_ffs a power of two (1, 2, 4): an
    // arithmetic shift floors for negative J as well
    const int lg = n_ffs >> 1;  // log2 n_ffs for 1, 2, 4
    int Q = J >> lg;
    int m = J - (Q << lg);
    float r = __fsub_rn((float)m, c_frac);  // in (-1, n_ffs)
    r = n_ffs == 1 ? r : __fmul_rn(r, n_ffs == 2 ? 0.5f : 0.25f);
    if (r < 0.0f) {  // floor
        Q -= 1;
        r = __fadd_rn(r, 1.0f);
        if (r >= 1.0f) {  // -r rounded to below 1 ulp of 1
            Q += 1;
            r = 0.0f;
        }
    }
    if (Q < 0) {
        *i0 = 0;
        *i1 = n > 1 ? 1 : 0;
        *w = 0.0f;
    } else if (Q > n - 1 || (Q == n - 1 && r > 0.0f)) {
        *i0 = n - 1;
        *i1 = n - 1;
        *w = 0.0f;
    } else {
        *i0 = Q;
        *i1 = (Q == n - 1) ? Q : Q + 1;
        *w = r;
    }
}

// Views per thread: the per-channel taps and focal terms are loaded once and
// reused along the view axis.
constexpr int kViewsPerThread = 8;

// --------------------------------------------------------------------------
// Kernels.  Idx is the index type of the raw and output arrays (32-bit when
// both hold fewer than 2^31 samples).
// --------------------------------------------------------------------------

// Raw rows per thread: the view-axis taps of a (channel, view) are computed
// once and used for every row of the group.  Measured on a config-2 window
// (phi+z FFS): 1 row 717 us, 2 rows 730, 4 rows 572, 8 rows 645, 16 rows
// 1003 (the L2 stops holding the rows in flight: 4.3 GB of reads for 1.1 GB).
constexpr int kRowsPerThread = 4;

// no-FFS and z-FFS: bilinear in (channel, view).  grid: x channel blocks,
// y groups of kRowsPerThread raw rows, z chunks of kViewsPerThread views.
template <class Idx>
__global__ void rebin_bilinear_kernel(RebinParams p)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    int r0 = blockIdx.y * kRowsPerThread;
    int r1 = min(r0 + kRowsPerThread, p.R_raw);
    int v0 = p.v_begin + blockIdx.z * kViewsPerThread;
    if (c >= p.Nos) return;
    const Idx frame_stride = (Idx)p.R_raw * p.N;
    const Idx nos = (Idx)p.Nos;
    for (int s = 0; s < p.n_ffs; ++s) {
        const AxisTap tap = p.taps[s * p.Nos + c];
        const float t_alpha = p.focal[s * p.Nos + c].t_alpha;
        const float t_off = p.n_ffs == 1 ? 0.0f : p.focal_offset[s];
        const float omu = tap.one_minus_u, u = tap.u;
        const float *base = p.raw + s * frame_stride;
        for (int v = v0; v < min(v0 + kViewsPerThread, p.v_end); ++v) {
            int i0, i1;
            float w;
            if (p.split_view_coord)
                view_taps_split(p.n_ffs, v + p.add, t_alpha, t_off, s, p.n_proj, &i0, &i1, &w);
            else
                view_taps(focal_alpha(p.n_ffs, v + p.add, t_alpha, t_off, s), p.n_proj, &i0, &i1, &w);
            const float *f0 = base + (Idx)(p.n_ffs * i0) * frame_stride;
            const float *f1 = base + (Idx)(p.n_ffs * i1) * frame_stride;
            float omw = __fsub_rn(1.0f, w);
            float *out_v = p.out + (Idx)v * p.R * nos + c;
#pragma unroll 4
            for (int row = r0; row < r1; ++row) {
                const Idx ro = (Idx)row * p.N;
                float a1 = __ldg(f0 + ro + tap.i0), a2 = __ldg(f0 + ro + tap.i1);
                float a5 = __ldg(f1 + ro + tap.i0), a6 = __ldg(f1 + ro + tap.i1);
                float t1 = __fmul_rn(__fmul_rn(a1, omu), omw);
                float t2 = __fmul_rn(__fmul_rn(a2, u), omw);
                float t5 = __fmul_rn(__fmul_rn(a5, omu), w);
                float t6 = __fmul_rn(__fmul_rn(a6, u), w);
                int out_row = row;
                if (p.n_ffs == 2) out_row = 2 * row + (p.reverse_rows ? 1 - s : s);
                out_v[(Idx)out_row * nos] = __fadd_rn(__fadd_rn(__fadd_rn(t1, t2), t5), t6);
            }
        }
    }
}

// phi-FFS and phi+z-FFS: radial interpolation between two samples of the
// (virtual) azimuthally rebinned intermediate, each a view-axis lerp of one
// focal spot.  For phi+z-FFS side s = 0 (-dr) uses focal spots 0/1 and s = 1
// (+dr) focal spots 2/3.
template <class Idx>
__global__ void rebin_two_stage_kernel(RebinParams p)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    int r0 = blockIdx.y * kRowsPerThread;
    int r1 = min(r0 + kRowsPerThread, p.R_raw);
    int v0 = p.v_begin + blockIdx.z * kViewsPerThread;
    if (c >= p.Nos) return;
    const Idx frame_stride = (Idx)p.R_raw * p.N;
    const Idx nos = (Idx)p.Nos;
    int sides = p.n_ffs == 4 ? 2 : 1;
    for (int s = 0; s < sides; ++s) {
        const AxisTap tap = p.taps[s * p.Nos + c];
        int qb = 2 * s;
        int q0 = qb + (tap.i0 & 1), ch0 = tap.i0 >> 1;
        int q1 = qb + (tap.i1 & 1), ch1 = tap.i1 >> 1;
        const float ta0 = p.focal[q0 * p.N + ch0].t_alpha, to0 = p.focal_offset[q0];
        const float ta1 = p.focal[q1 * p.N + ch1].t_alpha, to1 = p.focal_offset[q1];
        const float *b0 = p.raw + ch0 + q0 * frame_stride;
        const float *b1 = p.raw + ch1 + q1 * frame_stride;
        for (int v = v0; v < min(v0 + kViewsPerThread, p.v_end); ++v) {
            int proj = v + p.add;
            int i0, i1, j0, j1;
            float w0, w1;
            if (p.split_view_coord) {
                view_taps_split(p.n_ffs, proj, ta0, to0, q0, p.n_proj, &i0, &i1, &w0);
                view_taps_split(p.n_ffs, proj, ta1, to1, q1, p.n_proj, &j0, &j1, &w1);
            } else {
                view_taps(focal_alpha(p.n_ffs, proj, ta0, to0, q0), p.n_proj, &i0, &i1, &w0);
                view_taps(focal_alpha(p.n_ffs, proj, ta1, to1, q1), p.n_proj, &j0, &j1, &w1);
            }
            const float *f00 = b0 + (Idx)(p.n_ffs * i0) * frame_stride;
            const float *f01 = b0 + (Idx)(p.n_ffs * i1) * frame_stride;
            const float *f10 = b1 + (Idx)(p.n_ffs * j0) * frame_stride;
            const float *f11 = b1 + (Idx)(p.n_ffs * j1) * frame_stride;
            const float omw0 = __fsub_rn(1.0f, w0), omw1 = __fsub_rn(1.0f, w1);
            float *out_v = p.out + (Idx)v * p.R * nos + c;
#pragma unroll 4
            for (int row = r0; row < r1; ++row) {
                const Idx ro = (Idx)row * p.N;
                float T0 = __fadd_rn(__fmul_rn(__ldg(f00 + ro), omw0), __fmul_rn(__ldg(f01 + ro), w0));
                float T1 = __fadd_rn(__fmul_rn(__ldg(f10 + ro), omw1), __fmul_rn(__ldg(f11 + ro), w1));
                int out_row = row;
                if (p.n_ffs == 4) out_row = 2 * row + (p.reverse_rows ? 1 - s : s);
                out_v[(Idx)out_row * nos] = __fadd_rn(__fmul_rn(T0, tap.one_minus_u), __fmul_rn(T1, tap.u));
            }
        }
    }
}

int rebin_frames_needed(const RebinTables &t, int v)
{
    // view-axis coordinate of a focal spot's frame sequence: proj - t_alpha /
    // n_ffs - small focal terms, with |t_alpha| / n_ffs below the fan half
    // angle in views, which add_projections exceeds by 10; +1 for the upper
    // tap and one view of margin
    return t.n_ffs * (v + 2 * t.add_projections + 2);
}

int launch_rebin(const RebinTables &t, const DeviceRebinTables &dt, const float *d_raw,
                 float *d_out, cudaStream_t stream, int v_begin, int v_end)
{
    if (v_end < 0 || v_end > t.n_views) v_end = t.n_views;
    if (v_begin < 0) v_begin = 0;
    if (v_end <= v_begin) return CTBB_OK;
    RebinParams p;
    p.raw = d_raw;
    p.out = d_out;
    p.taps = dt.taps;
    p.focal = dt.focal;
    for (int i = 0; i < 4; ++i) p.focal_offset[i] = t.focal_offset[i];
    p.n_ffs = t.n_ffs;
    p.N = t.n_channels;
    p.Nos = t.n_os;
    p.R_raw = t.n_rows_raw;
    p.R = t.n_rows;
    p.n_proj = t.n_proj;
    p.add = t.add_projections;
    p.n_views = t.n_views;
    p.reverse_rows = t.reverse_rows;
    p.split_view_coord = t.split_view_coord;
    p.v_begin = v_begin;
    p.v_end = v_end;
    int chunks = (v_end - v_begin + kViewsPerThread - 1) / kViewsPerThread;
    int row_groups = (t.n_rows_raw + kRowsPerThread - 1) / kRowsPerThread;
    if (chunks > 65535 || row_groups > 65535) {
        set_error("rebin: %d views / %d rows exceed the launch grid", t.n_views, t.n_rows_raw);
        return CTBB_ERR_ARGUMENT;
    }
    size_t n_raw = (size_t)t.n_ffs * t.n_proj * t.n_rows_raw * t.n_channels;
    size_t n_out = (size_t)t.n_views * t.n_rows * t.n_os;
    bool narrow = n_raw < ((size_t)1 << 31) && n_out < ((size_t)1 << 31);
    dim3 block(128);
    dim3 grid((t.n_os + 127) / 128, row_groups, chunks);
    bool bilinear = t.mode == RebinMode::kNoFfs || t.mode == RebinMode::kZFfs;
    if (bilinear && narrow) rebin_bilinear_kernel<int><<<grid, block, 0, stream>>>(p);
    else if (bilinear) rebin_bilinear_kernel<size_t><<<grid, block, 0, stream>>>(p);
    else if (narrow) rebin_two_stage_kernel<int><<<grid, block, 0, stream>>>(p);
    else rebin_two_stage_kernel<size_t><<<grid, block, 0, stream>>>(p);
    count_launch();
    CTBB_CUDA_TRY(cudaGetLastError());
    return CTBB_OK;
}

int upload_rebin_tables(const RebinTables &t, DeviceRebinTables *dt, cudaStream_t stream)
{
    size_t nt = t.out_taps.size() * sizeof(AxisTap);
    size_t nf = t.focal.size() * sizeof(FocalTerm);
    if (dt->capacity < nt + nf) {
        if (dt->base) cudaFree(dt->base);
        dt->base = nullptr;
        dt->capacity = 0;
        CTBB_CUDA_TRY(cudaMalloc(&dt->base, nt + nf));
        dt->capacity = nt + nf;
    }
    dt->taps = reinterpret_cast<AxisTap *>(dt->base);
    dt->focal = reinterpret_cast<FocalTerm *>(reinterpret_cast<char *>(dt->base) + nt);
    CTBB_CUDA_TRY(cudaMemcpyAsync(dt->taps, t.out_taps.data(), nt, cudaMemcpyHostToDevice, stream));
    CTBB_CUDA_TRY(cudaMemcpyAsync(dt->focal, t.focal.data(), nf, cudaMemcpyHostToDevice, stream));
    return CTBB_OK;
}

}  // namespace ctbb
