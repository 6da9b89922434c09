/*
 * synth.h -- synthetic helical scans and the FP32 peak probe (test and
 * benchmark infrastructure; not part of the reconstruction library).
 *
 * The reference ships no raw data, so every workload of the tests and the
 * benchmark is a seeded phantom projected here.  The functions take the
 * reference's struct recon_metadata (include/ctbb_gb300.h) for the scan
 * geometry and the per-frame tube angles and table positions.
 */
#ifndef CTBB_SYNTH_H
#define CTBB_SYNTH_H

#include <stddef.h>
#include <stdint.h>

#include "../../include/ctbb_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* One phantom object: an ellipsoid (kind 1) or an infinite z-cylinder (kind 0)
   with attenuation mu (added to what lies beneath) [1/mm]. */
struct ctbb_phantom_object {
    int kind;
    float mu;
    float center[3];
    float semi_axes[3];
    float rotation[9];          /* row-major world->body rotation */
};

/* Text of the last failure of this library on this thread ("" if none). */
const char *synth_last_error(void);

/* Forward-project n_objects into frames [frame0, frame0+n_frames) of a helical
   FFS scan described by mr->cg / mr->rp and the tables mr->tube_angles,
   mr->table_positions (length rp.n_readings).  i0 > 0 adds Poisson noise with
   that unattenuated count (seeded; counter-based so host and device agree
   up to libm rounding).  out: [n_frames][n_rows_raw][n_channels] line integrals.
   The host variant runs on the CPU (no CUDA call); the device variant takes
   device pointers for out and the two tables and runs on `stream` (a
   cudaStream_t; NULL = legacy default stream).  0 on success. */
int synth_project_host(const struct recon_metadata *mr, const struct ctbb_phantom_object *objects,
                       int n_objects, size_t frame0, size_t n_frames, float i0, uint64_t seed, float *out);
int synth_project_device(const struct recon_metadata *mr, const struct ctbb_phantom_object *objects,
                         int n_objects, const float *d_tube_angles, const double *d_table_positions,
                         size_t frame0, size_t n_frames, float i0, uint64_t seed, float *d_out,
                         void *stream);

/* Measured FP32 FMA throughput of the current device (best of `repeats`
   launches of a register-only FMA loop on `stream`), TFLOP/s; -1 without a
   device. */
double synth_fp32_peak_tflops(int repeats, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* CTBB_SYNTH_H */
