// backproject.h -- host tables and launcher of the FP32 wFBP backprojector.
#pragma once

#include <cuda_runtime.h>

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

int build_backproject_tables(const struct recon_metadata &mr, BackprojectTables *t);
int launch_backproject(const struct recon_metadata &mr, const BackprojectTables &t,
                       const float4 *d_views, const float *d_theta, const float *d_zpos, const float *d_rebin,
                       float *d_block, int zpt, cudaStream_t stream, const float *d_vscale = nullptr);
// d_vscale non-null: d_rebin holds footprint quads [V][R][Nos][4] FP16 (the
// reduced-storage rows, see ramp_tc.h) with view v's scale at d_vscale[v R].

}  // namespace ctbb
