/*
 * ctbb_oracle.cpp -- CPU restatement of the reference's helical wFBP path.
 *
 * TEST INFRASTRUCTURE.  This file is the oracle: only tests/, the smoke check
 * of __graft_entry__.py and bench.py's CPU-baseline / reference arm may load
 * it, and only as the checker or the timed CPU baseline.  The product
 * (ctbangbang_gb300) never links or calls it.
 *
 * Every stage is written once as a template on the real type:
 *   Real = float  reproduces the reference CPU path's float arithmetic (the
 *                 same operations, order and C++ promotions), so with
 *                 -ffp-contract=off it matches the reference compiled from
 *                 its own sources (oracle/_ref) bit for bit;
 *   Real = double is the FP64 oracle: the same algorithm and constants
 *                 (including the reference's two values of pi) in double,
 *                 the error reference for "HU RMS / max vs FP64".
 *
 * Followed reference code (file:line in the reference project):
 *   interp2 / interp3            src/interp.cu:29-130
 *   adaptive filter              include/preprocessing.cuh:32-285, src/preprocessing.cu:31-156
 *   rebin no/phi/z/both FFS      src/rebin_filter_cpu.cu:95-645 (helpers :37-65)
 *   ramp filter                  src/rebin_filter_cpu.cu:647-709 (FFT convolution, M = 2*2^ceil(log2 N))
 *   load_filter                  src/rebin_filter.cu:922-959
 *   backprojection               src/backproject_cpu.cu:34-154
 *   finalize                     src/finalize_image_stack_cpu.cu:24-117
 * Parity: pinned against oracle/_ref (the reference's own CPU sources) and
 * the golden fixtures in tests/golden/ generated from it.
 */
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../include/ctbb_gb300.h"
#include "fft_radix2.h"

namespace {

template <class R>
struct Pi;
template <>
struct Pi<float> {
    static constexpr float rebin = 3.1415926535897f;  // src/rebin_filter_cpu.cu:21
    static constexpr float bp = 3.1415368979f;        // src/backproject_cpu.cu:29, include/preprocessing.cuh:25
    // literals of the reference written as float literals there
    static constexpr float f_max = 0.03f, e_lo = 0.3f, e_hi = 0.5f, q_taper = 0.6f;
};
template <>
struct Pi<double> {
    static constexpr double rebin = 3.1415926535897;
    static constexpr double bp = 3.1415368979;
    static constexpr double f_max = 0.03, e_lo = 0.3, e_hi = 0.5, q_taper = 0.6;
};

// ------------------------------------------------------------------ interp
template <class R>
R interp2(const R *a, int d1, int d2, R i1, R i2)
{
    if (i1 > (d1 - 2) || (i1 < 0) || i2 > (d2 - 2) || (i2 < 0)) return R(0);
    R v = i1 - std::floor(i1);
    R w = i2 - std::floor(i2);
    int f1 = (int)std::floor(i1), f2 = (int)std::floor(i2);
    int a1 = f2 * d1 + f1, a2 = f2 * d1 + f1 + 1;
    int a3 = (f2 + 1) * d1 + f1, a4 = (f2 + 1) * d1 + f1 + 1;
    return a[a1] * (R(1) - v) * (R(1) - w) + a[a2] * v * (R(1) - w) + a[a3] * (R(1) - v) * w +
           a[a4] * v * w;
}

template <class R>
R interp3(const R *a, int d1, int d2, int d3, R i1, R i2, R i3)
{
    if (i1 > (d1 - 1)) i1 = d1 - R(1);
    if (i1 < 0) i1 = R(0);
    if (i2 > (d2 - 1)) i2 = d2 - R(1);
    if (i2 < 0) i2 = R(0);
    if (i3 > (d3 - 1)) i3 = d3 - R(1);
    if (i3 < 0) i3 = R(0);
    R u = i1 - std::floor(i1), v = i2 - std::floor(i2), w = i3 - std::floor(i3);
    long f1 = (long)std::floor(i1), f2 = (long)std::floor(i2), f3 = (long)std::floor(i3);
    long p1 = (long)d1 * d2;
    long a1 = f3 * p1 + f2 * d1 + f1, a2 = a1 + 1;
    long a3 = f3 * p1 + (f2 + 1) * d1 + f1, a4 = a3 + 1;
    long a5 = (f3 + 1) * p1 + f2 * d1 + f1, a6 = a5 + 1;
    long a7 = (f3 + 1) * p1 + (f2 + 1) * d1 + f1, a8 = a7 + 1;
    if (i1 == d1 - R(1)) { a2 = a1; a4 = a3; a6 = a5; a8 = a7; }
    if (i2 == d2 - R(1)) { a3 = a1; a4 = a2; a7 = a5; a8 = a6; }
    if (i3 == d3 - R(1)) { a5 = a1; a6 = a2; a7 = a3; a8 = a4; }
    return a[a1] * (1 - u) * (1 - v) * (1 - w) + a[a2] * u * (1 - v) * (1 - w) +
           a[a3] * (1 - u) * v * (1 - w) + a[a4] * u * v * (1 - w) + a[a5] * (1 - u) * (1 - v) * w +
           a[a6] * u * (1 - v) * w + a[a7] * (1 - u) * v * w + a[a8] * u * v * w;
}

// ------------------------------------------------------------------ adaptive filter
template <class R>
void adaptive_filter(const struct recon_metadata &mr, const R *raw, R *out)
{
    const R pi = Pi<R>::bp;
    const int P = (int)mr.ri.n_proj_pull, Rr = (int)mr.cg.n_rows_raw, N = (int)mr.cg.n_channels;
    const size_t frame = (size_t)Rr * N;
    const int n_proj_ffs = (int)mr.cg.n_proj_ffs;
    const int max_idx = P - 1;
    std::vector<R> sup(P), smooth(P), ecc(P), pmax(P), pmin(P), thr(P);
    for (int p = 0; p < P; ++p) {  // extract_sup
        R m = 0;
        for (int i = 0; i < N; i++)
            for (int j = 0; j < Rr; j++) m = std::max(m, raw[frame * p + (size_t)j * N + i]);
        sup[p] = m;
    }
    int n_avg = (int)std::ceil((R(18) / R(360)) * (R)n_proj_ffs);
    n_avg = n_avg + (1 - n_avg % 2);
    int off_avg = (int)std::floor((R)(n_avg / 2));
    for (int p = 0; p < P; ++p) {  // smooth_sup
        R acc = 0;
        for (int i = 0; i < n_avg; i++) {
            int idx = std::min(std::max(p - off_avg + i, 0), max_idx);
            acc += (R(1) / (R)n_avg) * sup[idx];
        }
        smooth[p] = acc;
    }
    int n_range = (int)std::ceil((R(180) / R(360)) * (R)n_proj_ffs);
    n_range = n_range + (1 - n_range % 2);
    int off = (int)std::floor((R)(n_range / 2));
    for (int p = 0; p < P; ++p) {  // eccentricity
        R vmax = 0, vmin = 10000;
        for (int i = 0; i < n_range; i++) {
            R v = smooth[std::min(std::max(p - off + i, 0), max_idx)];
            if (v > vmax) vmax = v;
            if (v < vmin) vmin = v;
        }
        pmax[p] = vmax;
        pmin[p] = vmin;
        R e = 1 - vmin / vmax;
        e = (e - Pi<R>::e_lo) / (Pi<R>::e_hi - Pi<R>::e_lo);
        ecc[p] = e > 1 ? R(1) : (e < 0 ? R(0) : e);
    }
    auto rhs = [&](int start, R T) {
        int numel = n_range;
        int diff = start + (numel - 1);
        if (diff < (numel - 1)) {
            numel += start;
            start = 0;
        }
        if (diff > max_idx) numel -= (diff - max_idx);
        int sum = 0;
        for (int i = 0; i < numel; i++)
            if (smooth[start + i] > T) sum += 1;
        return (R(1) / pi) * (R)sum * (R(1) / (R)n_proj_ffs);
    };
    const R strength = (R)mr.rp.adaptive_filtration_s;
    for (int p = 0; p < P; ++p) {  // find_thresholds
        R lower = pmin[p], upper = pmax[p];
        R T = (pmax[p] + pmin[p]) / R(2);
        R lhs = Pi<R>::f_max * strength * ecc[p];
        R r = rhs(p - off, T);
        int iter = 0;
        while ((double)(std::fabs(lhs - r) / lhs) > 0.01) {
            if (iter >= 20) break;
            iter += 1;
            if (r > lhs) lower = T;
            else if (r < lhs) upper = T;
            else break;
            T = (lower + upper) / R(2);
            r = rhs(p - off, T);
        }
        thr[p] = T;
    }
    auto tri = [](int i) { return 3 - std::abs(i - 3); };
    for (int p = 0; p < P; ++p) {  // filter_projections
        R T = thr[p];
        for (int i = 0; i < N; i++)
            for (int j = 0; j < Rr; j++) {
                size_t idx = frame * p + (size_t)j * N + i;
                if (raw[idx] > T) {
                    R norm = 0, val = 0;
                    for (int ii = 0; ii < 5; ii++)
                        for (int jj = 0; jj < 5; jj++)
                            for (int kk = 0; kk < 5; kk++) {
                                int fr = j + jj - 2, fc = i + ii - 2, fp = p + kk - 2;
                                if (fr < 0 || fc < 0 || fp < 0 || fr >= Rr || fc >= N || fp >= P) continue;
                                R w = (R)(tri(ii) + tri(jj) + tri(kk) + 1);
                                norm += w;
                                val += raw[frame * fp + (size_t)fr * N + fc] * w;
                            }
                    out[idx] = (R(1) / norm) * val;
                } else {
                    out[idx] = raw[idx];
                }
            }
    }
}

// ------------------------------------------------------------------ rebin helpers
template <class R>
R angle(R x1, R x2, R y1, R y2)
{
    return std::asin((x1 * y2 - x2 * y1) / (std::sqrt(x1 * x1 + x2 * x2) * std::sqrt(y1 * y1 + y2 * y2)));
}

template <class R>
R beta_rk(R da, R dr, R channel, int os_flag, const struct ct_geom &cg)
{
    // pow(R(2), int) promotes to double, as in the reference
    R b0 = (R)((channel - std::pow(R(2), os_flag) * (R)cg.central_channel) *
               ((R)cg.fan_angle_increment / std::pow(R(2), os_flag)));
    R D = cg.src_to_det;
    return angle<R>(-((R)cg.r_f + dr), -(da), -(D * std::cos(b0) + dr), -(D * std::sin(b0) + da));
}

template <class R>
R d_alpha_r(R da, R dr, const struct ct_geom &cg)
{
    return angle<R>(cg.r_f, 0, (R)cg.r_f + dr, da);
}

template <class R>
R r_fr(R da, R dr, const struct ct_geom &cg)
{
    return std::sqrt(((R)cg.r_f + dr) * ((R)cg.r_f + dr) + da * da);
}

template <class R>
R get_beta_idx(R beta, const R *lookup, int n)
{
    int lo = 0;
    while (beta > lookup[lo] && lo < (n - 1)) lo++;
    if (lo == 0) lo++;
    return (R)lo - R(1) + (beta - lookup[lo - 1]) / (lookup[lo] - lookup[lo - 1]);
}

// rebin of the kept views: out[view][row][Nos] (no filter)
// Views [v0, v1) of the block (v1 < 0: all); each view is independent.
template <class R>
void rebin(const struct recon_metadata &mr, const R *raw, R *out, int v0 = 0, int v1 = -1)
{
    const struct ct_geom &cg = mr.cg;
    const struct recon_params &rp = mr.rp;
    const R pi = Pi<R>::rebin;
    const int n_ffs = (int)mr.ri.n_ffs;
    const int N = (int)cg.n_channels, Nos = (int)cg.n_channels_oversampled;
    const int Rr = (int)cg.n_rows_raw, Rout = (int)cg.n_rows;
    const int n_proj = (int)(mr.ri.n_proj_pull / mr.ri.n_ffs);
    const int add = (int)cg.add_projections;
    const int V = n_proj - 2 * add;
    const R fai = cg.fan_angle_increment, cc = cg.central_channel, rf = cg.r_f;
    const size_t frame = (size_t)Rr * N;
    const R n_proj_ffs = (R)cg.n_proj_ffs;
    // focal-spot sub-sequence s of the raw frames (frames s, s + n_ffs, ...)
    std::vector<R> sub((size_t)n_proj * frame);
    auto split = [&](int s) {
        for (int i = 0; i < n_proj; i++)
            std::memcpy(&sub[(size_t)i * frame], raw + ((size_t)n_ffs * i + s) * frame, frame * sizeof(R));
    };
    auto out_at = [&](int view, int row, int c) -> R & { return out[((size_t)view * Rout + row) * Nos + c]; };

    if (n_ffs == 1) {  // rebin_nffs_cpu
        split(0);
        for (int c = 0; c < Nos; c++) {
            const R beta = std::asin(((R)c - 2 * cc) * (fai / 2));
            R beta_idx = beta / fai + cc;
            for (int v = v0; v < (v1 < 0 ? V : std::min(v1, V)); v++) {
                int proj = v + add;
                R alpha_idx = (R)proj - beta * (R)cg.n_proj_turn / (R(2) * pi);
                for (int row = 0; row < Rout; row++)
                    out_at(v, row, c) = interp3<R>(sub.data(), N, Rout, n_proj, beta_idx, (R)row, alpha_idx);
            }
        }
        return;
    }
    if (n_ffs == 2 && rp.z_ffs == 1) {  // rebin_zffs_cpu
        const double da = 0.0;
        const double dr = cg.src_to_det * rp.coll_slicewidth /
                          (4.0 * (cg.src_to_det - cg.r_f) * std::tan(cg.anode_angle));
        std::vector<R> raw2((size_t)n_proj * frame);
        split(1);
        raw2.swap(sub);
        split(0);  // sub = raw_1 (even frames), raw2 = raw_2 (odd)
        std::vector<R> lk1(N), lk2(N);
        for (int i = 0; i < N; i++) {
            lk1[i] = beta_rk<R>((R)da, (R)-dr, (R)i, 0, cg);
            lk2[i] = beta_rk<R>((R)da, (R)dr, (R)i, 0, cg);
        }
        for (int v = v0; v < (v1 < 0 ? V : std::min(v1, V)); v++) {
            int proj = v + add;
            for (int row = 0; row < Rr; row++)
                for (int c = 0; c < Nos; c++) {
                    R b1 = std::asin(((R)c - R(2) * cc) * (fai / R(2)) * rf / r_fr<R>(R(0), (R)-dr, cg));
                    R a1 = (R)(n_ffs * proj) - b1 * n_proj_ffs / (R(2) * pi) -
                           d_alpha_r<R>((R)da, (R)-dr, cg) * n_proj_ffs / (R(2) * pi);
                    R bi1 = get_beta_idx<R>(b1, lk1.data(), N);
                    R b2 = std::asin(((R)c - R(2) * cc) * (fai / R(2)) * rf / r_fr<R>(R(0), (R)dr, cg));
                    R a2 = (R)(n_ffs * proj) - b2 * n_proj_ffs / (R(2) * pi) -
                           d_alpha_r<R>((R)da, (R)dr, cg) * n_proj_ffs / (R(2) * pi);
                    R bi2 = get_beta_idx<R>(b2, lk2.data(), N);
                    a1 = a1 / R(2);
                    a2 = (a2 - R(1)) / R(2);
                    int r1 = cg.reverse_row_interleave ? 2 * row + 1 : 2 * row;
                    int r2 = cg.reverse_row_interleave ? 2 * row : 2 * row + 1;
                    out_at(v, r1, c) = interp3<R>(sub.data(), N, Rr, n_proj, bi1, (R)row, a1);
                    out_at(v, r2, c) = interp3<R>(raw2.data(), N, Rr, n_proj, bi2, (R)row, a2);
                }
        }
        return;
    }
    const double da = cg.src_to_det * cg.r_f * cg.fan_angle_increment / (4.0f * (cg.src_to_det - cg.r_f));
    if (n_ffs == 2) {  // rebin_pffs_cpu
        std::vector<R> raw2((size_t)n_proj * frame);
        split(1);
        raw2.swap(sub);
        split(0);
        std::vector<R> lookup(Nos), tmp((size_t)Rr * Nos);
        for (int ch = 0; ch < N; ch++) {
            lookup[2 * ch] = beta_rk<R>((R)da, 0, (R)ch, 0, cg);
            lookup[2 * ch + 1] = beta_rk<R>((R)-da, 0, (R)ch, 0, cg);
        }
        for (int v = v0; v < (v1 < 0 ? V : std::min(v1, V)); v++) {
            int proj = v + add;
            for (int row = 0; row < Rr; row++)
                for (int ch = 0; ch < N; ch++) {
                    R b1 = lookup[2 * ch], b2 = lookup[2 * ch + 1];
                    R a1 = (R)(n_ffs * proj) - b1 * n_proj_ffs / (R(2) * pi) -
                           d_alpha_r<R>((R)da, 0, cg) * n_proj_ffs / (R(2) * pi);
                    R a2 = (R)(n_ffs * proj) - b2 * n_proj_ffs / (R(2) * pi) -
                           d_alpha_r<R>((R)-da, 0, cg) * n_proj_ffs / (R(2) * pi);
                    a1 = a1 / R(2);
                    a2 = (a2 - R(1)) / R(2);
                    tmp[(size_t)row * Nos + 2 * ch] = interp3<R>(sub.data(), N, Rr, n_proj, (R)ch, (R)row, a1);
                    tmp[(size_t)row * Nos + 2 * ch + 1] = interp3<R>(raw2.data(), N, Rr, n_proj, (R)ch, (R)row, a2);
                }
            // radial pass on this view (interp3 with integer row and view = 1-D lerp)
            for (int row = 0; row < Rr; row++)
                for (int c = 0; c < Nos; c++) {
                    R beta = std::asin(((R)c - 2 * cc) * (fai / 2));
                    R bi = get_beta_idx<R>(beta, lookup.data(), Nos);
                    out_at(v, row, c) = interp3<R>(&tmp[(size_t)row * Nos], Nos, 1, 1, bi, R(0), R(0));
                }
        }
        return;
    }
    // rebin_affs_cpu
    const double dr = cg.src_to_det * rp.coll_slicewidth / (4.0 * (cg.src_to_det - cg.r_f) * std::tan(cg.anode_angle));
    std::vector<std::vector<R>> rq(4, std::vector<R>((size_t)n_proj * frame));
    for (int q = 0; q < 4; ++q) {
        split(q);
        rq[q].swap(sub);
    }
    const R sda[4] = {(R)da, (R)-da, (R)da, (R)-da};
    const R sdr[4] = {(R)-dr, (R)-dr, (R)dr, (R)dr};
    std::vector<R> lk1(Nos), lk2(Nos), t1((size_t)Rr * Nos), t2((size_t)Rr * Nos);
    for (int ch = 0; ch < N; ch++) {
        lk1[2 * ch] = beta_rk<R>(sda[0], sdr[0], (R)ch, 0, cg);
        lk1[2 * ch + 1] = beta_rk<R>(sda[1], sdr[1], (R)ch, 0, cg);
        lk2[2 * ch] = beta_rk<R>(sda[2], sdr[2], (R)ch, 0, cg);
        lk2[2 * ch + 1] = beta_rk<R>(sda[3], sdr[3], (R)ch, 0, cg);
    }
    const R *lkq[4] = {&lk1[0], &lk1[1], &lk2[0], &lk2[1]};
    for (int v = v0; v < (v1 < 0 ? V : std::min(v1, V)); v++) {
        int proj = v + add;
        for (int row = 0; row < Rr; row++)
            for (int ch = 0; ch < N; ch++)
                for (int q = 0; q < 4; ++q) {
                    R b = lkq[q][2 * ch];
                    R a = (R)(n_ffs * proj) - b * n_proj_ffs / (R(2) * pi) -
                          d_alpha_r<R>(sda[q], sdr[q], cg) * n_proj_ffs / (R(2) * pi);
                    a = q == 0 ? a / R(4) : (a - (R)q) / R(4);
                    R val = interp3<R>(rq[q].data(), N, Rr, n_proj, (R)ch, (R)row, a);
                    (q < 2 ? t1 : t2)[(size_t)row * Nos + 2 * ch + (q & 1)] = val;
                }
        for (int row = 0; row < Rr; row++)
            for (int c = 0; c < Nos; c++) {
                int r1 = cg.reverse_row_interleave ? 2 * row + 1 : 2 * row;
                int r2 = cg.reverse_row_interleave ? 2 * row : 2 * row + 1;
                R b1 = std::asin(((R)c - 2 * cc) * (fai / 2) * rf / r_fr<R>(R(0), (R)-dr, cg));
                R b2 = std::asin(((R)c - 2 * cc) * (fai / 2) * rf / r_fr<R>(R(0), (R)dr, cg));
                R bi1 = get_beta_idx<R>(b1, lk1.data(), Nos);
                R bi2 = get_beta_idx<R>(b2, lk2.data(), Nos);
                out_at(v, r1, c) = interp3<R>(&t1[(size_t)row * Nos], Nos, 1, 1, bi1, R(0), R(0));
                out_at(v, r2, c) = interp3<R>(&t2[(size_t)row * Nos], Nos, 1, 1, bi2, R(0), R(0));
            }
    }
}

// ------------------------------------------------------------------ ramp filter
// y[l] = sum_k f[N + l - k] x[k] through a zero-padded double FFT (filter_cpu).
template <class R>
void filter_rows(R *rows, size_t n_rows, int N, const float *taps)
{
    int M = 2 * (int)std::pow(2.0f, std::ceil(std::log2((float)N)));
    std::vector<double> F(2 * (size_t)M, 0.0), X(2 * (size_t)M);
    for (int i = 0; i < N; i++) F[2 * (size_t)i] = taps[(int)std::floor((2.0f * N - 1.0f) / 2.0f) + 1 + i];
    for (int i = (M - N + 1); i < M; i++) F[2 * (size_t)i] = taps[i - (M - N + 1) + 1];
    ctbb_oracle_fft_radix2(F.data(), M, -1);
    for (size_t r = 0; r < n_rows; ++r) {
        R *row = rows + r * (size_t)N;
        std::fill(X.begin(), X.end(), 0.0);
        for (int i = 0; i < N; i++) X[2 * (size_t)i] = (double)row[i];
        ctbb_oracle_fft_radix2(X.data(), M, -1);
        for (int k = 0; k < M; k++) {
            double xr = X[2 * (size_t)k], xi = X[2 * (size_t)k + 1];
            double fr = F[2 * (size_t)k], fi = F[2 * (size_t)k + 1];
            X[2 * (size_t)k] = xr * fr - xi * fi;
            X[2 * (size_t)k + 1] = xr * fi + xi * fr;
        }
        ctbb_oracle_fft_radix2(X.data(), M, +1);
        for (int i = 0; i < N; i++) {
            if (sizeof(R) == sizeof(float))
                row[i] = (R)((1.0f / (float)M) * (float)X[2 * (size_t)i]);
            else
                row[i] = (R)(X[2 * (size_t)i] / (double)M);
        }
    }
}

// ------------------------------------------------------------------ backprojection
template <class R>
R weight_W(R q)
{
    const R pi = Pi<R>::bp;
    const R Q = Pi<R>::q_taper;
    if (std::fabs(q) < Q) return R(1);
    if ((std::fabs(q) >= Q) && (std::fabs(q) < R(1)))
        return std::pow(std::cos((pi / R(2)) * (std::fabs(q) - Q) / (R(1) - Q)), R(2));
    return R(0);
}

template <class R>
R tube_start_of(const struct recon_metadata &mr)
{
    const struct ct_geom &cg = mr.cg;
    if (sizeof(R) == sizeof(float)) {
        float t = (float)(std::fmod((double)(mr.tube_angles[0] + ((mr.ri.idx_pull_start + cg.add_projections_ffs) *
                                                                 360.0f / cg.n_proj_ffs)),
                                    360.0) *
                          Pi<float>::bp / 180.0f);
        return (R)t;
    }
    double a = (double)mr.tube_angles[0] +
               (double)(mr.ri.idx_pull_start + cg.add_projections_ffs) * 360.0 / (double)cg.n_proj_ffs;
    return (R)(std::fmod(a, 360.0) * Pi<double>::bp / 180.0);
}

// Angles [i0, i1) of one block into out_block [n_slices_block][ny][nx]
// (added), for the pixels x in [x_lo, x_hi), y in [y_lo, y_hi) (x_hi, y_hi < 0:
// to the edge); every pixel is independent of the others.
template <class R>
void backproject(const struct recon_metadata &mr, const R *rebin, int i0, int i1, R *out_block, int x_lo = 0,
                 int x_hi = -1, int y_lo = 0, int y_hi = -1)
{
    const struct ct_geom &cg = mr.cg;
    const struct recon_params &rp = mr.rp;
    const R pi = Pi<R>::bp;
    const int nx = (int)rp.nx, ny = (int)rp.ny, nz = (int)mr.ri.n_slices_block;
    const int Nos = (int)cg.n_channels_oversampled, Rw = (int)cg.n_rows;
    const R tube_start = tube_start_of<R>(mr);
    const int nht = (int)((mr.ri.n_proj_pull / mr.ri.n_ffs - 2 * cg.add_projections) / (cg.n_proj_turn / 2));
    const size_t view = (size_t)Nos * Rw;
    std::vector<R> s_t((size_t)nx * ny * nz), h_t((size_t)nx * ny * nz), proj(view * nht);
    const R r_f = cg.r_f, fai = cg.fan_angle_increment, cc = cg.central_channel, z_rot = cg.z_rot;
    const R coll = rp.coll_slicewidth, fov = rp.recon_fov;
    for (int i = i0; i < i1; i++) {
        for (int kk = 0; kk < nht; kk++)
            std::memcpy(&proj[view * kk], &rebin[((size_t)i + (size_t)kk * cg.n_proj_turn / 2) * view], view * sizeof(R));
        std::fill(s_t.begin(), s_t.end(), R(0));
        std::fill(h_t.begin(), h_t.end(), R(0));
        for (int xi = x_lo; xi < (x_hi < 0 ? nx : x_hi); xi++) {
            R x = (fov / (R)rp.nx) * ((R)xi - (R)(rp.nx - 1) / R(2)) + (R)rp.x_origin;
            for (int yi = y_lo; yi < (y_hi < 0 ? ny : y_hi); yi++) {
                R y = (fov / (R)rp.ny) * ((R)yi - (R)(rp.ny - 1) / R(2)) + (R)rp.y_origin;
                for (int k = 0; k < nht; k++) {
                    R theta = tube_start + (R(2) * pi / (R)cg.n_proj_turn) * (R)i + (R)k * pi;
                    R phat = x * std::sin(theta) - y * std::cos(theta);
                    R p_idx = phat / (r_f * fai / R(2)) + R(2) * cc;
                    for (int zi = 0; zi < nz; zi++) {
                        R z = (R)zi * coll + z_rot / R(2) + z_rot * tube_start / (R(2) * pi);
                        R ray_pos = (z_rot * (theta - std::asin(phat / r_f)) / (R(2) * pi));
                        R lhat = std::sqrt(std::pow(r_f, R(2)) - std::pow(phat, R(2))) - x * std::cos(theta) -
                                 y * std::sin(theta);
                        R qhat = (z - ray_pos) / (lhat * std::tan((R)cg.theta_cone / R(2)));
                        R q_idx = ((qhat + R(1)) / R(2)) * ((R)cg.n_rows - R(1)) + (R)((size_t)k * cg.n_rows);
                        size_t vi = (size_t)nz * ny * xi + (size_t)nz * yi + zi;
                        s_t[vi] += interp2<R>(proj.data(), Nos, Rw * nht, p_idx, q_idx) * weight_W<R>(qhat);
                        h_t[vi] += weight_W<R>(qhat);
                    }
                }
            }
        }
        for (int xi = x_lo; xi < (x_hi < 0 ? nx : x_hi); xi++)
            for (int yi = y_lo; yi < (y_hi < 0 ? ny : y_hi); yi++)
                for (int zi = 0; zi < nz; zi++) {
                    size_t o = (size_t)zi * nx * ny + (size_t)yi * nx + xi;
                    size_t in = (size_t)nz * ny * xi + (size_t)nz * yi + zi;
                    if (h_t[in] != 0) out_block[o] += (R(1) / h_t[in]) * s_t[in] * 2 * pi / (R)cg.n_proj_turn;
                }
    }
}

int n_half_turns(const struct recon_metadata &mr)
{
    return (int)((mr.ri.n_proj_pull / mr.ri.n_ffs - 2 * mr.cg.add_projections) / (mr.cg.n_proj_turn / 2));
}

// ------------------------------------------------------------------ finalize
template <class R>
void finalize(const struct recon_metadata &mr, const R *image, R *final_out)
{
    const struct recon_params &rp = mr.rp;
    const struct recon_info &ri = mr.ri;
    const size_t plane = (size_t)rp.nx * rp.ny;
    const int nb = (int)ri.n_slices_block;
    int recon_direction = 1;
    {
        float d = rp.end_pos - rp.start_pos;
        if (d != 0.0f) {
            recon_direction = (int)(std::fabs(d) / d);
            if (recon_direction != 1 && recon_direction != -1) recon_direction = 1;
        }
    }
    double dtp = mr.table_positions[1000] - mr.table_positions[0];
    int table_direction = (int)(dtp / std::fabs(dtp));
    const int n_raw = (int)(ri.n_slices_block * ri.n_blocks);
    std::vector<R> temp(plane * ri.n_slices_recon);
    for (int s = 0; s < (int)ri.n_slices_recon; s++) {
        int src = s;
        if (recon_direction != table_direction) src = (s / nb) * nb + (nb - 1 - s % nb);
        std::memcpy(&temp[plane * s], &image[plane * src], plane * sizeof(R));
    }
    int n_final = (int)(std::floor(std::fabs(rp.end_pos - rp.start_pos) / rp.slice_thickness) + 1);
    std::vector<R> raw_loc(n_raw), w(n_raw);
    for (int i = 0; i < n_raw; i++) raw_loc[i] = (R)ri.recon_start_pos + (R)(recon_direction * i) * (R)rp.coll_slicewidth;
    for (int k = 0; k < n_final; k++) {
        R loc = (R)rp.start_pos + (R)(recon_direction * k) * (R)rp.slice_thickness;
        R sum = 0;
        for (int s = 0; s < n_raw; s++) {
            w[s] = std::max(R(0), R(1) - std::fabs(raw_loc[s] - loc) / (R)rp.slice_thickness);
            sum += w[s];
        }
        R *out = final_out + plane * k;
        for (size_t px = 0; px < plane; px++) out[px] = 0;
        for (size_t px = 0; px < plane; px++)
            for (int s = 0; s < n_raw; s++)
                if (w[s] != 0) out[px] += (w[s] / sum) * temp[plane * s + px];
    }
}

int n_final_of(const struct recon_metadata &mr)
{
    return (int)(std::floor(std::fabs(mr.rp.end_pos - mr.rp.start_pos) / mr.rp.slice_thickness) + 1);
}

size_t n_views_of(const struct recon_metadata &mr)
{
    return mr.ri.n_proj_pull / mr.ri.n_ffs - 2 * mr.cg.add_projections;
}

}  // namespace

extern "C" {

/* load_filter (src/rebin_filter.cu:922-959): returns 0, or 1 if the file is missing. */
int oracle_load_filter(const struct recon_metadata *mr, float *taps)
{
    const char *name = nullptr;
    switch (mr->rp.recon_kernel) {
    case -100: name = "ramp"; break;
    case -1: name = "exp"; break;
    case 1: name = "smooth"; break;
    case 2: name = "medium"; break;
    case 3: name = "sharp"; break;
    default: break;
    }
    char path[4096 + 128];
    if (name)
        snprintf(path, sizeof(path), "%s/resources/filters/f_%zu_%s.txt", mr->install_dir, mr->cg.n_channels, name);
    else
        snprintf(path, sizeof(path), "%s/resources/filters/f_%zu_b%i.txt", mr->install_dir, mr->cg.n_channels,
                 mr->rp.recon_kernel);
    FILE *f = fopen(path, "rb");
    if (!f) return 1;
    size_t n = 2 * mr->cg.n_channels_oversampled;
    size_t got = fread(taps, sizeof(float), n, f);
    fclose(f);
    return got == n ? 0 : 1;
}

/* ---- float: the reference CPU path's arithmetic ---- */

int oracle_adaptive_filter(struct recon_metadata *mr)
{
    size_t n = mr->ri.n_proj_pull * mr->cg.n_rows_raw * mr->cg.n_channels;
    std::vector<float> out(n);
    adaptive_filter<float>(*mr, mr->ctd.raw, out.data());
    std::memcpy(mr->ctd.raw, out.data(), n * sizeof(float));
    return 0;
}

int oracle_rebin(struct recon_metadata *mr)
{
    rebin<float>(*mr, mr->ctd.raw, mr->ctd.rebin);
    return 0;
}

int oracle_filter_rows(float *rows, size_t n_rows, int n, const float *taps)
{
    filter_rows<float>(rows, n_rows, n, taps);
    return 0;
}

int oracle_rebin_filter(struct recon_metadata *mr)
{
    std::vector<float> taps(2 * mr->cg.n_channels_oversampled);
    if (oracle_load_filter(mr, taps.data())) return 1;
    rebin<float>(*mr, mr->ctd.raw, mr->ctd.rebin);
    filter_rows<float>(mr->ctd.rebin, n_views_of(*mr) * mr->cg.n_rows, (int)mr->cg.n_channels_oversampled,
                       taps.data());
    return 0;
}

/* Angles [i0, i1) of the current block, added into out_block. */
int oracle_backproject_range(const struct recon_metadata *mr, const float *rebin_data, int i0, int i1,
                             float *out_block)
{
    backproject<float>(*mr, rebin_data, i0, i1, out_block);
    return 0;
}

int oracle_backproject(struct recon_metadata *mr)
{
    size_t block = (size_t)mr->rp.nx * mr->rp.ny * mr->ri.n_slices_block;
    std::vector<float> out(block, 0.0f);
    backproject<float>(*mr, mr->ctd.rebin, 0, (int)(mr->cg.n_proj_turn / 2), out.data());
    std::memcpy(mr->ctd.image + (size_t)(mr->ri.cb.block_idx - 1) * block, out.data(), block * sizeof(float));
    return 0;
}

int oracle_finalize(struct recon_metadata *mr)
{
    size_t plane = (size_t)mr->rp.nx * mr->rp.ny;
    int n_final = n_final_of(*mr);
    mr->ctd.final_image_stack = (float *)calloc(plane * n_final, sizeof(float));
    finalize<float>(*mr, mr->ctd.image, mr->ctd.final_image_stack);
    return 0;
}

int oracle_n_half_turns(const struct recon_metadata *mr) { return n_half_turns(*mr); }

/* ---- double: the FP64 oracle ---- */

/* One block: raw window (float, [P][R_raw][N]) -> adaptive filter -> rebin ->
   filter -> backprojection into out_block [n_slices_block][ny][nx] (double). */
int oracle64_block(const struct recon_metadata *mr, const float *raw, int adaptive, const float *taps,
                   double *out_block)
{
    size_t n = mr->ri.n_proj_pull * mr->cg.n_rows_raw * mr->cg.n_channels;
    std::vector<double> r(raw, raw + n), f(n);
    if (adaptive) {
        adaptive_filter<double>(*mr, r.data(), f.data());
        r.swap(f);
    }
    size_t nv = n_views_of(*mr);
    std::vector<double> rb(nv * mr->cg.n_rows * mr->cg.n_channels_oversampled);
    rebin<double>(*mr, r.data(), rb.data());
    filter_rows<double>(rb.data(), nv * mr->cg.n_rows, (int)mr->cg.n_channels_oversampled, taps);
    size_t block = (size_t)mr->rp.nx * mr->rp.ny * mr->ri.n_slices_block;
    std::fill(out_block, out_block + block, 0.0);
    backproject<double>(*mr, rb.data(), 0, (int)(mr->cg.n_proj_turn / 2), out_block);
    return 0;
}

/* Backprojection of angles [i0, i1) of the block from float filtered rows
   [n_views][n_rows][n_os], in double, into out_block (overwritten). */
int oracle64_backproject_range(const struct recon_metadata *mr, const float *rows, int i0, int i1,
                               double *out_block)
{
    size_t nv = n_views_of(*mr);
    std::vector<double> rb(rows, rows + nv * mr->cg.n_rows * mr->cg.n_channels_oversampled);
    size_t block = (size_t)mr->rp.nx * mr->rp.ny * mr->ri.n_slices_block;
    std::fill(out_block, out_block + block, 0.0);
    backproject<double>(*mr, rb.data(), i0, i1, out_block);
    return 0;
}

/* Rebin (no filter) of views [v0, v1) of the block from a float raw window
   [P][R_raw][N] into out [n_views][n_rows][n_os] (only those views written). */
int oracle_rebin_views(const struct recon_metadata *mr, const float *raw, int v0, int v1, float *out)
{
    rebin<float>(*mr, raw, out, v0, v1);
    return 0;
}

/* oracle_backproject_range for the pixels x in [x0, x1), y in [y0, y1) only
   (out_block written there, zeroed first there). */
int oracle_backproject_patch(const struct recon_metadata *mr, const float *rebin_data, int x0, int x1, int y0,
                             int y1, float *out_block)
{
    const size_t nx = mr->rp.nx, ny = mr->rp.ny;
    for (size_t z = 0; z < mr->ri.n_slices_block; ++z)
        for (int y = y0; y < y1; ++y)
            for (int x = x0; x < x1; ++x) out_block[(z * ny + (size_t)y) * nx + (size_t)x] = 0.0f;
    backproject<float>(*mr, rebin_data, 0, (int)(mr->cg.n_proj_turn / 2), out_block, x0, x1, y0, y1);
    return 0;
}

/* The FP64 oracle's stages one at a time, for callers that split the work
   over threads: adaptive filter of a float raw window into double; rebin of
   views [v0, v1) of a double raw window; ramp filter of n double rows;
   backprojection of the pixels x in [x0, x1), y in [y0, y1) (all angles)
   from double filtered rows into out_block (written there, zeroed first). */
int oracle64_adaptive_filter(const struct recon_metadata *mr, const float *raw, double *out)
{
    size_t n = mr->ri.n_proj_pull * mr->cg.n_rows_raw * mr->cg.n_channels;
    std::vector<double> r(raw, raw + n);
    adaptive_filter<double>(*mr, r.data(), out);
    return 0;
}

int oracle64_rebin_views(const struct recon_metadata *mr, const double *raw, int v0, int v1, double *out)
{
    rebin<double>(*mr, raw, out, v0, v1);
    return 0;
}

int oracle64_filter_rows(double *rows, size_t n_rows, int n, const float *taps)
{
    filter_rows<double>(rows, n_rows, n, taps);
    return 0;
}

int oracle64_backproject_patch(const struct recon_metadata *mr, const double *rows, int x0, int x1, int y0, int y1,
                               double *out_block)
{
    const size_t nx = mr->rp.nx, ny = mr->rp.ny;
    for (size_t z = 0; z < mr->ri.n_slices_block; ++z)
        for (int y = y0; y < y1; ++y)
            for (int x = x0; x < x1; ++x) out_block[(z * ny + (size_t)y) * nx + (size_t)x] = 0.0;
    backproject<double>(*mr, rows, 0, (int)(mr->cg.n_proj_turn / 2), out_block, x0, x1, y0, y1);
    return 0;
}

/* The FP64 finalize of one final slice k as weights: w_out[s] is the weight
   (w_s / sum, 0 where finalize skips the raw slice) of raw slice s, and
   src_out[s] the image slice raw slice s is read from after the block
   reorder -- final[k][px] = sum_s w_out[s] image[src_out[s]][px], the sum
   finalize<double> forms.  Returns the number of raw slices. */
int oracle64_finalize_weights(const struct recon_metadata *mr, int k, double *w_out, int *src_out)
{
    const struct recon_params &rp = mr->rp;
    const struct recon_info &ri = mr->ri;
    const int nb = (int)ri.n_slices_block;
    int recon_direction = 1;
    {
        float d = rp.end_pos - rp.start_pos;
        if (d != 0.0f) {
            recon_direction = (int)(std::fabs(d) / d);
            if (recon_direction != 1 && recon_direction != -1) recon_direction = 1;
        }
    }
    double dtp = mr->table_positions[1000] - mr->table_positions[0];
    int table_direction = (int)(dtp / std::fabs(dtp));
    const int n_raw = (int)(ri.n_slices_block * ri.n_blocks);
    double loc = (double)rp.start_pos + (double)(recon_direction * k) * (double)rp.slice_thickness;
    double sum = 0.0;
    for (int s = 0; s < n_raw; s++) {
        double raw_loc = (double)ri.recon_start_pos + (double)(recon_direction * s) * (double)rp.coll_slicewidth;
        w_out[s] = std::max(0.0, 1.0 - std::fabs(raw_loc - loc) / (double)rp.slice_thickness);
        sum += w_out[s];
        src_out[s] = (recon_direction != table_direction) ? (s / nb) * nb + (nb - 1 - s % nb) : s;
    }
    for (int s = 0; s < n_raw; s++) w_out[s] = w_out[s] != 0.0 ? w_out[s] / sum : 0.0;
    return n_raw;
}

/* Final slices of the plan: floor(|end - start| / slice_thickness) + 1
   (src/finalize_image_stack_cpu.cu:67). */
int oracle_n_slices_final(const struct recon_metadata *mr) { return n_final_of(*mr); }

int oracle64_finalize(const struct recon_metadata *mr, const double *image, double *final_out)
{
    finalize<double>(*mr, image, final_out);
    return 0;
}

float oracle_interp2(const float *a, int d1, int d2, float i1, float i2) { return interp2<float>(a, d1, d2, i1, i2); }
float oracle_interp3(const float *a, int d1, int d2, int d3, float i1, float i2, float i3)
{
    return interp3<float>(a, d1, d2, d3, i1, i2, i3);
}

}  // extern "C"
