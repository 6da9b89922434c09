// rebin.h -- host tables and launcher of the FFS / fan-to-parallel rebinning.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "ctbb_internal.h"

namespace ctbb {

enum class RebinMode { kNoFfs, kPhiFfs, kZFfs, kBothFfs };

// interp3 taps along one axis (base, aliased upper tap, weight, 1 - weight).
struct AxisTap {
    int i0, i1;
    float u, one_minus_u;
};

// View-axis term of one (focal spot, channel): beta * n_proj_ffs / (2 pi).
struct FocalTerm {
    float t_alpha;
};

struct RebinTables {
    RebinMode mode = RebinMode::kNoFfs;
    int n_ffs = 1, n_channels = 0, n_os = 0, n_rows_raw = 0, n_rows = 0;
    int n_proj = 0, add_projections = 0, n_views = 0, reverse_rows = 0;
    // View-axis coordinate in split form (integer frames + a fraction) instead
    // of the reference's float expression: for a window far longer than one
    // block's (the whole-scan union), where that float rounds at the
    // window's large frame offsets (rebin.cu, view_taps_split).
    int split_view_coord = 0;
    std::vector<AxisTap> out_taps;   // [side][n_os]
    std::vector<FocalTerm> focal;    // no/z-FFS: [side][n_os]; phi/both: [focal][n_channels]
    std::vector<float> focal_offset; // d_alpha_r * n_proj_ffs / (2 pi) per focal spot
};

struct DeviceRebinTables {
    void *base = nullptr;
    size_t capacity = 0;
    AxisTap *taps = nullptr;
    FocalTerm *focal = nullptr;
};

int build_rebin_tables(const struct recon_metadata &mr, RebinTables *t);
int upload_rebin_tables(const RebinTables &t, DeviceRebinTables *dt, cudaStream_t stream);
// Views [v_begin, v_end) of the output (v_end < 0: all views).
int launch_rebin(const RebinTables &t, const DeviceRebinTables &dt, const float *d_raw,
                 float *d_out, cudaStream_t stream, int v_begin = 0, int v_end = -1);
// Frames of the pull window view v reads (focal-spot frames of the view-axis
// taps of every channel): all lie below rebin_frames_needed(t, v).
int rebin_frames_needed(const RebinTables &t, int v);

}  // namespace ctbb
