/*
 * ref_adaptive_host.cpp -- runs the reference's adaptive-filter kernel bodies
 * (include/preprocessing.cuh:32-285) as host loops.
 *
 * TEST INFRASTRUCTURE (oracle/_ref only).  The reference has no CPU adaptive
 * filter: src/main.cu:222 calls the GPU function even under --no-gpu.  Its
 * kernels are plain per-projection loops, so this translation unit defines the
 * CUDA qualifiers away, provides threadIdx/blockIdx/blockDim as globals and
 * launches every "thread" in turn, in the same kernel order as
 * src/preprocessing.cu:54-138 (128 threads per block, n_proj_pull/128 blocks).
 */
#include <algorithm>
#include <math.h>
#include <stdlib.h>
#include <string.h>

using std::max;

struct ctbb_host_dim3 {
    unsigned int x, y, z;
};
static ctbb_host_dim3 threadIdx, blockIdx, blockDim;

#define __global__
#define __device__
#define __constant__ static

#include <preprocessing.cuh>

#define CTBB_FOR_EACH_THREAD(n_threads_total, body)                                   \
    do {                                                                              \
        blockDim.x = 128;                                                             \
        for (unsigned int b_ = 0; b_ < (unsigned int)((n_threads_total) / 128); ++b_) \
            for (unsigned int t_ = 0; t_ < 128; ++t_) {                               \
                blockIdx.x = b_;                                                      \
                threadIdx.x = t_;                                                     \
                body;                                                                 \
            }                                                                         \
    } while (0)

int ref_adaptive_filter_host(struct recon_metadata *mr)
{
    struct ct_geom cg = mr->cg;
    struct recon_info ri = mr->ri;
    d_cg = cg;
    d_ri = ri;

    size_t P = ri.n_proj_pull;
    size_t n = cg.n_channels * cg.n_rows_raw * P;
    float *sup = (float *)calloc(P, sizeof(float));
    float *sup_smooth = (float *)calloc(P, sizeof(float));
    float *ecc = (float *)calloc(P, sizeof(float));
    float *pmax = (float *)calloc(P, sizeof(float));
    float *pmin = (float *)calloc(P, sizeof(float));
    float *thr = (float *)calloc(P, sizeof(float));
    float *filtered = (float *)calloc(n, sizeof(float));
    float *raw = mr->ctd.raw;

    CTBB_FOR_EACH_THREAD(P, extract_sup(raw, sup));
    CTBB_FOR_EACH_THREAD(P, smooth_sup(sup, sup_smooth));
    CTBB_FOR_EACH_THREAD(P, eccentricity(sup_smooth, ecc, pmax, pmin));
    CTBB_FOR_EACH_THREAD(P, find_thresholds(mr->rp.adaptive_filtration_s, ecc, sup_smooth,
                                            pmax, pmin, thr));
    CTBB_FOR_EACH_THREAD(P, filter_projections(raw, thr, filtered));

    memcpy(raw, filtered, n * sizeof(float));
    free(sup);
    free(sup_smooth);
    free(ecc);
    free(pmax);
    free(pmin);
    free(thr);
    free(filtered);
    return 0;
}

extern "C" int ref_adaptive_thresholds(struct recon_metadata *mr, float *thr_out)
{
    /* same sequence, stopping after find_thresholds (checkpoint for tests) */
    d_cg = mr->cg;
    d_ri = mr->ri;
    size_t P = mr->ri.n_proj_pull;
    float *sup = (float *)calloc(P, sizeof(float));
    float *sup_smooth = (float *)calloc(P, sizeof(float));
    float *ecc = (float *)calloc(P, sizeof(float));
    float *pmax = (float *)calloc(P, sizeof(float));
    float *pmin = (float *)calloc(P, sizeof(float));
    CTBB_FOR_EACH_THREAD(P, extract_sup(mr->ctd.raw, sup));
    CTBB_FOR_EACH_THREAD(P, smooth_sup(sup, sup_smooth));
    CTBB_FOR_EACH_THREAD(P, eccentricity(sup_smooth, ecc, pmax, pmin));
    CTBB_FOR_EACH_THREAD(P, find_thresholds(mr->rp.adaptive_filtration_s, ecc, sup_smooth,
                                            pmax, pmin, thr_out));
    free(sup);
    free(sup_smooth);
    free(ecc);
    free(pmax);
    free(pmin);
    return 0;
}
