// ctbb_internal.h -- declarations shared by the library's translation units.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>

#include "../../include/ctbb_gb300.h"

namespace ctbb {

// Thread-local last error text; every failing entry point sets it.
void set_error(const char *fmt, ...);
void clear_error();

// Constants of the reference.  Two values of pi are in use there: the rebinning
// code and the planner use 3.1415926535897f (src/rebin_filter_cpu.cu:21,
// src/setup.cu:33); the backprojector and the adaptive filter use
// 3.1415368979f (src/backproject_cpu.cu:29, include/preprocessing.cuh:25).
// Parity with the reference CPU path needs both, each where the reference uses it.
constexpr float kPiRebin = 3.1415926535897f;
constexpr float kPiBackproject = 3.1415368979f;
constexpr int kBlockSlices = 32;  // BLOCK_SLICES, src/setup.cu:34

// Host planner helpers (planner.cpp).
int array_search(float key, const double *array, int numel, int search_type);
int recon_direction_of(const struct recon_params &rp);
int array_direction_of(const double *table_positions);
void pull_window(const struct ct_geom &cg, int n_ffs, int idx_a, int idx_b,
                 int *idx_pull_start, int *idx_pull_end, int *n_proj_pull);

// Derived sizes of one block.
struct BlockDims {
    size_t n_proj_pull;   // P
    size_t n_ffs;
    size_t n_proj;        // P / n_ffs
    size_t n_views;       // n_proj - 2 * add_projections
    size_t n_channels;    // N
    size_t n_os;          // 2N
    size_t n_rows;        // R (after z-FFS)
    size_t n_rows_raw;    // R_raw
    int n_half_turns;     // (n_proj - 2 add) / (n_turn / 2)
    size_t raw_elems() const { return n_proj_pull * n_rows_raw * n_channels; }
    size_t rebin_elems() const { return n_views * n_rows * n_os; }
};
BlockDims block_dims(const struct recon_metadata &mr);

// Next block's plan (update_block_info without host re-allocation).
int plan_next_block(const struct recon_metadata &mr, struct recon_info *ri_out);

// Reference float expressions for the backprojector's start angle
// (src/backproject_cpu.cu:55): fmod(double(tube_angles[0] + (pull+add_ffs)*360/n_ffs), 360) * pi'/180.
float bp_tube_start(const struct recon_metadata &mr);

}  // namespace ctbb
