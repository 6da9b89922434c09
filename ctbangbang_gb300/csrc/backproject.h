// backproject.h -- host tables and launcher of the FP32 wFBP backprojector.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "ctbb_internal.h"

namespace ctbb {

struct BackprojectTables {
    float tube_start = 0.0f;
    int nht = 0;               // half turns in the pull window
    int n_half = 0;            // n_proj_turn / 2
    int n_slices = 0;          // slices per block
    // [n_half][nht][4] {row index, sin, cos, theta z_rot / 2 pi'}: the row
    // index (its bits, an unsigned int) is the view's position in the rows
    // buffer the launch reads, i + k n_half unless remapped (set_view_row)
    std::vector<float> views;
    std::vector<float> theta;  // [n_half][nht]: theta of view (i, k)
    std::vector<float> zpos;   // [n_slices]
    void set_view_row(int i, int k, unsigned row);
};

// Kernel parameters of one block's backprojection.
struct BpParams {
    const float *rebin;    // [V][R][Nos] float32, or footprint quads [V][R][Nos][4] FP16
    const float *vscale;   // quads: scale of row r of view v at [v R + r] (one per view); else null
    uint64_t rebin_rows;   // address of rebin - kFloorMagicBits rows (mod 2^64): see row_floor
    float *out;            // [n_slices_block][ny][nx]
    const float4 *views;   // [n_half][nht] {row index bits, sin, cos, theta z_rot / 2 pi'}
    const float *theta;    // [n_half][nht] theta (the last-turn border recheck)
    const float *zpos;     // [n_slices_block]
    int nx, ny, n_slices, nos, n_rows, nht, n_half;
    float pix_x, pix_y, x_c, y_c, x0, y0;  // x = pix_x * (xi - x_c) + x0
    float ds_half;         // r_f fai / 2
    float inv_ds_half;     // 1 / ds_half
    float two_cc;          // 2 * central channel
    float coll;            // slice spacing
    float rf, inv_rf, rf2; // r_f, 1 / r_f, r_f^2
    float z_rot, two_pi;   // z_rot, 2 pi'
    float zrot_over_2pi;
    float tan_cone;
    int k_window;          // half-turn window per angle (z_rot != 0)
    int warp_w;            // voxel columns along x per warp (32, 16, 8 or 4)
    int cta_w;             // voxel columns along x per CTA (a multiple of warp_w)
    float abs_zr;          // |z_rot / (2 pi')|
    float inv_half_feed;   // 2 / z_rot: half turns per mm of ray travel
    float half_rows;       // (R - 1) / 2
    float taper_scale;     // (pi'/2) / (1 - Q)
    float out_scale;       // 2 pi' / n_proj_turn
    int flat_path;         // R >= 8: rows of |q| <= Q never reach a border
    int col_zpt;           // column form: slices per thread (a multiple of 8, at most 32)
    int n_achunks;         // column form: angle chunks (grid z = slice chunks x angle chunks)
    float *partial;        // n_achunks > 1: [n_achunks][n_slices][ny][nx] unscaled image sums
};

// A launch shape: slices per thread, threads per CTA, CTAs per SM the kernel
// is compiled for, voxel columns along x per CTA and per warp, and the form:
// col = 0 the slice-chunk form (zpt slices per thread share one visit's
// geometry), col = 1 the column form (zpt = 8, 16 or 32 slices per thread in
// sub-chunks of 8 share one angle's geometry; windows of at most
// kColumnMaxHalfTurns half turns).
// achunks (column form): the half-turn angles split into that many chunks,
// each run by CTAs of its own that write unscaled partial image sums, which a
// second kernel adds in chunk order (smaller CTA lifetimes: a shorter tail).
struct BpShape {
    int zpt = 8, threads = 128, min_blocks = 7, cta_w = 64, warp_w = 8, col = 0, achunks = 1;
    bool operator==(const BpShape &o) const
    {
        return zpt == o.zpt && threads == o.threads && min_blocks == o.min_blocks && cta_w == o.cta_w &&
               warp_w == o.warp_w && col == o.col && achunks == o.achunks;
    }
};
constexpr int kColumnMaxHalfTurns = 8;
constexpr int kMaxAngleChunks = 16;  // the most angle chunks a launch shape uses
// The shape the environment knobs (CTBB_BP_*) name: the column form (unless
// CTBB_BP_FORM=tile), else the slice-chunk form with zpt slices per thread
// (FP16 footprint words: its default shape).
BpShape default_bp_shape(int zpt, bool quad);
// s, or the slice-chunk form's default where s is the column form and the
// window of nht half turns is more than it holds.
BpShape fit_bp_shape(const BpShape &s, int nht);
// default_bp_shape fitted to a window of nht half turns: where the knobs
// leave them open, the column form's slices per thread and CTAs per SM
// chosen by the window's width (measured), then fit_bp_shape.
BpShape window_bp_shape(int zpt, bool quad, int nht);
// Shapes the autotuner times (those the batch kernel is compiled for).
std::vector<BpShape> backproject_shape_candidates(bool quad);

int build_backproject_tables(const struct recon_metadata &mr, BackprojectTables *t);
int make_backproject_params(const struct recon_metadata &mr, const BackprojectTables &t, const float4 *d_views,
                            const float *d_theta, const float *d_zpos, const float *d_rebin, float *d_block,
                            const float *d_vscale, const BpShape &shape, BpParams *p);
// scratch: device memory for the partial image sums of shape.achunks > 1
// (backproject_partial_bytes); with less, the angles run as one chunk.
int launch_backproject_params(const BpParams &p, const BpShape &shape, cudaStream_t stream, void *scratch = nullptr,
                              size_t scratch_bytes = 0);
// Bytes of partial image sums a launch of this shape needs (0: none).
size_t backproject_partial_bytes(const BpParams &p, const BpShape &shape);
// Device bytes launch_backproject_batch needs for n blocks' parameters.
size_t backproject_batch_bytes(size_t n_blocks);
// All blocks (of any scans; one row storage and row length) in one launch of
// the given shape -- the column form one launch per angle chunk, each adding
// to the blocks' images in chunk order; d_buf holds
// backproject_batch_bytes(blocks.size()).
int launch_backproject_batch(const std::vector<BpParams> &blocks, const BpShape &shape, void *d_buf,
                             size_t buf_bytes, cudaStream_t stream);
int launch_backproject(const struct recon_metadata &mr, const BackprojectTables &t,
                       const float4 *d_views, const float *d_theta, const float *d_zpos, const float *d_rebin,
                       float *d_block, int zpt, cudaStream_t stream, const float *d_vscale = nullptr,
                       const BpShape *shape = nullptr, void *scratch = nullptr, size_t scratch_bytes = 0);
// d_vscale non-null: d_rebin holds footprint quads [V][R][Nos][4] FP16 (the
// reduced-storage rows, see ramp_tc.h) with view v's scale at d_vscale[v R].

}  // namespace ctbb
