/*
 * ref_harness.cpp -- shims and an extern "C" driver around the reference's
 * own CPU path, compiled from the reference sources where they lie.
 *
 * TEST INFRASTRUCTURE.  Built only by oracle/ref/Makefile into
 * oracle/_ref/libctbb_ref.so, in the container that has the reference mounted.
 * Used to pin this project's oracle restatement (oracle/ctbb_oracle.cpp) and to
 * generate the golden fixtures under tests/golden/.  Never shipped, never used
 * by the product.
 *
 * The reference translation units linked beside this file (unmodified):
 *   src/setup.cu, src/parse_config.cu, src/interp.cu, src/rebin_filter_cpu.cu,
 *   src/backproject_cpu.cu, src/finalize_image_stack_cpu.cu
 * plus include/preprocessing.cuh through ref_adaptive_host.cpp.
 */
#include <complex.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <fftw3.h>
#include <ctbb/ctbb_read.h>

#include <recon_structs.h>
#include <setup.h>
#include <interp.h>
#include <rebin_filter_cpu.h>
#include <backproject_cpu.h>
#include <finalize_image_stack_cpu.h>

#include "../fft_radix2.h"

/* ---------------- FFTW3 API shim ---------------- */

struct ctbb_shim_fftw_plan_s {
    int n;
    int sign;
    fftw_complex *in;
    fftw_complex *out;
};

void *fftw_malloc(size_t n) { return malloc(n); }
void fftw_free(void *p) { free(p); }

fftw_plan fftw_plan_dft_1d(int n, fftw_complex *in, fftw_complex *out, int sign, unsigned)
{
    fftw_plan p = (fftw_plan)malloc(sizeof(*p));
    p->n = n;
    p->sign = sign;
    p->in = in;
    p->out = out;
    return p;
}

void fftw_execute(const fftw_plan p)
{
    if (p->out != p->in) memcpy(p->out, p->in, sizeof(fftw_complex) * (size_t)p->n);
    ctbb_oracle_fft_radix2((double *)p->out, p->n, p->sign);
}

void fftw_destroy_plan(fftw_plan p) { free(p); }

/* ---------------- libctbb_read shim (FileType 0 only) ---------------- */

void ReadBinaryFrame(FILE *fp, int frame_idx, int n_channels, int n_rows, float *frame,
                     int offset)
{
    size_t n = (size_t)n_channels * (size_t)n_rows;
    memset(frame, 0, n * sizeof(float));
    long pos = (long)offset + (long)frame_idx * (long)(n * sizeof(float));
    if (fseek(fp, pos, SEEK_SET) != 0) return;
    size_t got = fread(frame, sizeof(float), n, fp);
    (void)got; /* a short read leaves the zero fill past EOF */
}

#define CTBB_SHIM_UNSUPPORTED(name)                                                      \
    fprintf(stderr, "ctbb_read shim: %s is a vendor format reader (not available)\n", name)

float ReadPTRTubeAngle(FILE *, int, int, int) { CTBB_SHIM_UNSUPPORTED("ReadPTRTubeAngle"); return 0.f; }
float ReadPTRTablePosition(FILE *, int, int, int) { CTBB_SHIM_UNSUPPORTED("ReadPTRTablePosition"); return 0.f; }
void ReadPTRFrame(FILE *, int, int, int, float *) { CTBB_SHIM_UNSUPPORTED("ReadPTRFrame"); }
float ReadCTDv1794TubeAngle(FILE *, int, int, int) { CTBB_SHIM_UNSUPPORTED("ReadCTDv1794TubeAngle"); return 0.f; }
float ReadCTDv1794TablePosition(FILE *, int, int, int) { CTBB_SHIM_UNSUPPORTED("ReadCTDv1794TablePosition"); return 0.f; }
void ReadCTDv1794Frame(FILE *, int, int, int, float *) { CTBB_SHIM_UNSUPPORTED("ReadCTDv1794Frame"); }
float ReadCTDv2007TubeAngle(FILE *, int, int, int) { CTBB_SHIM_UNSUPPORTED("ReadCTDv2007TubeAngle"); return 0.f; }
float ReadCTDv2007TablePosition(FILE *, int, int, int) { CTBB_SHIM_UNSUPPORTED("ReadCTDv2007TablePosition"); return 0.f; }
void ReadCTDv2007Frame(FILE *, int, int, int, float *) { CTBB_SHIM_UNSUPPORTED("ReadCTDv2007Frame"); }
float ReadIMATubeAngle(FILE *, int, int, int, int, int) { CTBB_SHIM_UNSUPPORTED("ReadIMATubeAngle"); return 0.f; }
float ReadIMATablePosition(FILE *, int, int, int, int, int) { CTBB_SHIM_UNSUPPORTED("ReadIMATablePosition"); return 0.f; }
void ReadIMAFrame(FILE *, int, int, int, float *, int, int) { CTBB_SHIM_UNSUPPORTED("ReadIMAFrame"); }
float ReadForceTubeAngle(FILE *, int, int, int) { CTBB_SHIM_UNSUPPORTED("ReadForceTubeAngle"); return 0.f; }
float ReadForceTablePosition(FILE *, int, int, int) { CTBB_SHIM_UNSUPPORTED("ReadForceTablePosition"); return 0.f; }
void ReadForceFrame(FILE *, int, int, int, float *) { CTBB_SHIM_UNSUPPORTED("ReadForceFrame"); }
float ReadDICOMTubeAngle(FILE *, int, int, int) { CTBB_SHIM_UNSUPPORTED("ReadDICOMTubeAngle"); return 0.f; }
float ReadDICOMTablePosition(FILE *, int, int, int) { CTBB_SHIM_UNSUPPORTED("ReadDICOMTablePosition"); return 0.f; }
void ReadDICOMFrame(FILE *, int, int, int, float *) { CTBB_SHIM_UNSUPPORTED("ReadDICOMFrame"); }

/* ---------------- load_filter (lives in the GPU file src/rebin_filter.cu) -------- */

/* Restated from src/rebin_filter.cu:922-959: the file name is chosen by
   ReconKernel and 2*n_channels_oversampled float32 taps are read.  The
   reference exit(1)s on a missing file; the harness aborts likewise. */
void load_filter(float *f_array, struct recon_metadata *mr)
{
    struct ct_geom cg = mr->cg;
    struct recon_params rp = mr->rp;
    char path[4096 + 255] = {0};
    const char *name = NULL;
    switch (rp.recon_kernel) {
    case -100: name = "ramp"; break;
    case -1: name = "exp"; break;
    case 1: name = "smooth"; break;
    case 2: name = "medium"; break;
    case 3: name = "sharp"; break;
    default: break;
    }
    if (name)
        snprintf(path, sizeof(path), "%s/resources/filters/f_%lu_%s.txt", mr->install_dir,
                 (unsigned long)cg.n_channels, name);
    else
        snprintf(path, sizeof(path), "%s/resources/filters/f_%lu_b%i.txt", mr->install_dir,
                 (unsigned long)cg.n_channels, rp.recon_kernel);
    FILE *f = fopen(path, "rb");
    if (!f) {
        fprintf(stderr, "ref harness: filter file %s not found\n", path);
        abort();
    }
    size_t got = fread(f_array, sizeof(float), 2 * cg.n_channels_oversampled, f);
    (void)got;
    fclose(f);
}

/* ---------------- adaptive filter (ref_adaptive_host.cpp) ---------------- */
int ref_adaptive_filter_host(struct recon_metadata *mr);

/* ---------------- extern "C" driver ---------------- */

extern "C" {

size_t ref_sizeof_recon_metadata(void) { return sizeof(struct recon_metadata); }
size_t ref_offsetof(int which)
{
    switch (which) {
    case 0: return offsetof(struct recon_metadata, flags);
    case 1: return offsetof(struct recon_metadata, rp);
    case 2: return offsetof(struct recon_metadata, ri);
    case 3: return offsetof(struct recon_metadata, cg);
    case 4: return offsetof(struct recon_metadata, ctd);
    case 5: return offsetof(struct recon_metadata, tube_angles);
    case 6: return offsetof(struct recon_metadata, table_positions);
    case 7: return offsetof(struct recon_params, nx);
    case 8: return offsetof(struct recon_params, table_dir);
    case 9: return offsetof(struct recon_info, cb);
    case 10: return offsetof(struct ct_geom, table_direction);
    default: return (size_t)-1;
    }
}

int ref_configure_recon_params(const char *prm, struct recon_params *out)
{
    *out = configure_recon_params((char *)prm);
    return 0;
}

/* main.cu:196-202 minus configure_paths (which derives install_dir from
   /proc/self/exe); the caller fills mr->rp and mr->install_dir first. */
int ref_configure(struct recon_metadata *mr)
{
    mr->cg = configure_ct_geom(mr);
    configure_reconstruction(mr);
    return 0;
}

int ref_configure_ct_geom(struct recon_metadata *mr)
{
    mr->cg = configure_ct_geom(mr);
    return 0;
}

int ref_configure_reconstruction(struct recon_metadata *mr)
{
    configure_reconstruction(mr);
    return 0;
}

int ref_update_block_info(struct recon_metadata *mr) { update_block_info(mr); return 0; }
int ref_extract_projections(struct recon_metadata *mr) { extract_projections(mr); return 0; }
int ref_adaptive_filter_kk(struct recon_metadata *mr) { return ref_adaptive_filter_host(mr); }
int ref_rebin_filter_cpu(struct recon_metadata *mr) { return rebin_filter_cpu(mr); }
int ref_backproject_cpu(struct recon_metadata *mr) { return backproject_cpu(mr); }
int ref_finalize_image_stack_cpu(struct recon_metadata *mr) { return finalize_image_stack_cpu(mr); }
int ref_load_filter(struct recon_metadata *mr, float *out) { load_filter(out, mr); return 0; }

/* free what setup/finalize allocated, without writing the output file */
int ref_free(struct recon_metadata *mr)
{
    free(mr->ctd.rebin);
    free(mr->ctd.image);
    free(mr->ctd.raw);
    free(mr->ctd.final_image_stack);
    free(mr->tube_angles);
    free(mr->table_positions);
    mr->ctd.rebin = mr->ctd.image = mr->ctd.raw = mr->ctd.final_image_stack = NULL;
    mr->tube_angles = NULL;
    mr->table_positions = NULL;
    return 0;
}

float ref_interp2(float *array, int d1, int d2, float i1, float i2)
{
    struct array_dims d;
    d.idx1 = d1;
    d.idx2 = d2;
    d.idx3 = 0;
    return interp2(array, d, i1, i2);
}

float ref_interp3(float *array, int d1, int d2, int d3, float i1, float i2, float i3)
{
    struct array_dims d;
    d.idx1 = d1;
    d.idx2 = d2;
    d.idx3 = d3;
    return interp3(array, d, i1, i2, i3);
}

} /* extern "C" */
