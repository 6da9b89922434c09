// finalize.h -- host tables and launcher of the slice reorder / thickening.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "ctbb_internal.h"

namespace ctbb {

struct FinalizeTables {
    int n_final = 0;
    int n_raw = 0;
    std::vector<int> offsets;    // [n_final + 1] CSR row starts
    std::vector<int> slices;     // image slice of each non-zero weight
    std::vector<float> weights;  // weight / sum of weights
};

int build_finalize_tables(const struct recon_metadata &mr, FinalizeTables *t);
int launch_finalize(const struct recon_metadata &mr, const FinalizeTables &t, const int *d_offsets,
                    const int *d_slices, const float *d_weights, const float *d_image, float *d_final,
                    float mu_water, cudaStream_t stream);

}  // namespace ctbb
