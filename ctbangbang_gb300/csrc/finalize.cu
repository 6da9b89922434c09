// finalize.cu -- block reorder, triangle slice thickening and HU conversion.
//
// Reference: finalize_image_stack_cpu (src/finalize_image_stack_cpu.cu:24-117)
// and its GPU twin (src/finalize_image_stack.cu:26-120).  When the recon
// direction differs from the table direction each 32-slice block is flipped in
// z; then final slice k at start + dir k ST is the normalised triangle average
// (FWHM = ST) of the raw slices at recon_start + dir i coll.  The weights and
// their normalisation are computed on the host in float exactly as the
// reference does, and the device accumulates w_i * image_i in increasing i with
// separate multiply and add, so the thickened stack is bit-exact.  The HU
// conversion (mu - mu_w) / mu_w * 1000 is new (the reference has none) and is
// applied only when mu_water > 0.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "ctbb_internal.h"
#include "cuda_util.cuh"
#include "finalize.h"

namespace ctbb {

namespace {

__global__ void thicken_kernel(const float *__restrict__ image, float *__restrict__ out,
                               const int *__restrict__ offsets, const int *__restrict__ slices,
                               const float *__restrict__ weights, size_t plane, float mu_water)
{
    size_t px = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    int k = blockIdx.y;
    if (px >= plane) return;
    float acc = 0.0f;
    for (int e = offsets[k]; e < offsets[k + 1]; ++e)
        acc = __fadd_rn(acc, __fmul_rn(weights[e], __ldg(image + (size_t)slices[e] * plane + px)));
    if (mu_water > 0.0f) acc = 1000.0f * (acc - mu_water) / mu_water;
    out[(size_t)k * plane + px] = acc;
}

}  // namespace

int build_finalize_tables(const struct recon_metadata &mr, FinalizeTables *t)
{
    const struct recon_params &rp = mr.rp;
    const struct recon_info &ri = mr.ri;
    if (!mr.table_positions || rp.n_readings <= 1000) {
        set_error("finalize: frame tables missing (or fewer than 1001 frames)");
        return CTBB_ERR_STATE;
    }
    int recon_direction = recon_direction_of(rp);
    double dtp = mr.table_positions[1000] - mr.table_positions[0];
    // the reference divides dtp by |dtp| (src/finalize_image_stack_cpu.cu:35);
    // a table that does not move (axial scan) has no direction to flip by
    if (!std::isfinite(dtp) || dtp == 0.0) {
        set_error("finalize: table positions 0 and 1000 are equal or not finite (the table does not move), "
                  "so the slice order is undefined");
        return CTBB_ERR_CONFIG;
    }
    int table_direction = (int)(dtp / std::fabs(dtp));
    int n_raw = (int)(ri.n_slices_block * ri.n_blocks);
    int n_block = (int)ri.n_slices_block;
    int n_final = ctbb_n_slices_final(&mr);
    t->n_final = n_final;
    t->n_raw = n_raw;
    t->offsets.assign(1, 0);
    t->slices.clear();
    t->weights.clear();

    // raw slice i is image slice map(i) after the optional per-block flip
    auto image_slice = [&](int i) {
        if (recon_direction != table_direction) {
            int b = i / n_block, z = i % n_block;
            return b * n_block + (n_block - 1 - z);
        }
        return i;
    };
    std::vector<float> raw_loc(n_raw), w(n_raw);
    for (int i = 0; i < n_raw; i++)
        raw_loc[i] = ri.recon_start_pos + (float)(recon_direction * i) * rp.coll_slicewidth;
    for (int k = 0; k < n_final; k++) {
        float slice_location = rp.start_pos + (float)(recon_direction * k) * rp.slice_thickness;
        float sum_weights = 0;
        for (int s = 0; s < n_raw; s++) {
            w[s] = std::fmax(0.0f, 1.0f - std::fabs(raw_loc[s] - slice_location) / rp.slice_thickness);
            sum_weights += w[s];
        }
        for (int s = 0; s < n_raw; s++) {
            if (w[s] != 0) {
                t->slices.push_back(image_slice(s));
                t->weights.push_back(w[s] / sum_weights);
            }
        }
        t->offsets.push_back((int)t->slices.size());
    }
    return CTBB_OK;
}

int launch_finalize(const struct recon_metadata &mr, const FinalizeTables &t, const int *d_offsets,
                    const int *d_slices, const float *d_weights, const float *d_image, float *d_final,
                    float mu_water, cudaStream_t stream)
{
    size_t plane = (size_t)mr.rp.nx * mr.rp.ny;
    if (t.n_final <= 0) return CTBB_OK;
    if (t.n_final > 65535) {
        set_error("finalize: %d final slices exceed the launch grid", t.n_final);
        return CTBB_ERR_ARGUMENT;
    }
    dim3 block(256);
    dim3 grid((unsigned)((plane + 255) / 256), (unsigned)t.n_final);
    thicken_kernel<<<grid, block, 0, stream>>>(d_image, d_final, d_offsets, d_slices, d_weights,
                                               plane, mu_water);
    count_launch();
    CTBB_CUDA_TRY(cudaGetLastError());
    return CTBB_OK;
}

}  // namespace ctbb
