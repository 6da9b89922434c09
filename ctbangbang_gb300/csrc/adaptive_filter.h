// adaptive_filter.h -- launcher of the Kachelriess-Kalender adaptive raw filter.
#pragma once

#include <cuda_runtime.h>

#include "ctbb_internal.h"

namespace ctbb {

// Floats of device scratch launch_adaptive_filter needs for a window of
// n_proj_pull frames: sup, smooth, ecc, max, min, threshold ([6][P]).
size_t adaptive_filter_scratch_floats(size_t n_proj_pull);

// d_in -> d_out (distinct buffers) for the pull window described by mr.
int launch_adaptive_filter(const struct recon_metadata &mr, const float *d_in, float *d_out,
                           float *d_scratch, cudaStream_t stream);

// Frames from either end of a pull window within which the filter's output
// depends on where the window ends: the 180-degree statistics window of a
// frame reaches range_offset frames, and each moving mean in it a further
// avg_offset (include/preprocessing.cuh:92-96, :119-122).  Frames at least
// this far from both ends are filtered the same in any window holding them.
int adaptive_filter_edge_reach(const struct recon_metadata &mr);

// The filter of one pull window whose per-frame maxima are given (d_sup, P
// floats: the maxima of a larger window at this window's offset -- a frame's
// maximum does not depend on the window), in three steps for a caller that
// decides between them which frames it needs.  d_scratch holds 6 * P floats
// (its sup slot is not used).
//  * thresholds: moving means of every frame, then the eccentricity and
//    threshold of frames [0, fa) and [fb, P);
//  * dirty: for those frames, whether the output can differ from the larger
//    window's, given that window's thresholds at this window's offset
//    (d_thr_union): some sample of the frame lies above one threshold and not
//    the other, or -- with lo_edge / hi_edge, this window's first / last frame
//    not being the larger window's -- the frame lies within the 5-frame
//    smoothing stencil's reach of that end and has a sample above its
//    threshold.  d_dirty gets one byte per frame of [0, P) (1 = can differ;
//    frames [fa, fb) are 0);
//  * output: the filtered frames [f0, f1) from the thresholds of the first
//    step (every frame of [f0, f1) must lie in [0, fa) or [fb, P)).
int launch_adaptive_filter_ends_thresholds(const struct recon_metadata &mr, const float *d_in, const float *d_sup,
                                           float *d_scratch, int fa, int fb, cudaStream_t stream);
int launch_adaptive_filter_dirty(const struct recon_metadata &mr, const float *d_sup, const float *d_thr_union,
                                 const float *d_scratch, int fa, int fb, int lo_edge, int hi_edge,
                                 unsigned char *d_dirty, cudaStream_t stream);
int launch_adaptive_filter_output(const struct recon_metadata &mr, const float *d_in, float *d_out,
                                  const float *d_sup, float *d_scratch, int f0, int f1, cudaStream_t stream);

// The same filter over a window whose frames arrive in order: advance() is
// told how many leading frames of d_in are present and launches every step
// for the frames whose windows those cover (maxima as frames arrive; moving
// means avg_reach frames behind; eccentricity, threshold and smoothing a
// further range_reach behind).  Once all P frames have arrived the result
// equals launch_adaptive_filter's.  filtered() frames of d_out are final.
struct AfStream {
    explicit AfStream(const struct recon_metadata &mr);
    int advance(const struct recon_metadata &mr, const float *d_in, float *d_out, float *d_scratch, int arrived,
                cudaStream_t stream);
    int filtered() const { return n_filtered; }
    int P = 0, avg_reach = 0, range_reach = 0;
    int n_sup = 0, n_smoothed = 0, n_filtered = 0;
};

}  // namespace ctbb
