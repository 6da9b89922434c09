/*
 * fftw3.h (shim) -- the five FFTW3 public-API calls the reference's
 * src/rebin_filter_cpu.cu:654-707 makes, backed by this project's radix-2 FFT
 * (oracle/fft_radix2.h).  libfftw3 is not installed in this image; its
 * arithmetic (a 1-D complex DFT) is restated, not linked.
 *
 * TEST INFRASTRUCTURE: only used to build the reference CPU path in oracle/_ref.
 */
#ifndef CTBB_SHIM_FFTW3_H
#define CTBB_SHIM_FFTW3_H

#include <stddef.h>

/* complex.h is included before this header by the reference, so FFTW's
   public API makes fftw_complex the native double complex type. */
typedef double _Complex fftw_complex;
typedef struct ctbb_shim_fftw_plan_s *fftw_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_ESTIMATE (1U << 6)

void *fftw_malloc(size_t n);
void fftw_free(void *p);
fftw_plan fftw_plan_dft_1d(int n, fftw_complex *in, fftw_complex *out, int sign,
                           unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);

#endif
