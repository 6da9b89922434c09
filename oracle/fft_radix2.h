/*
 * fft_radix2.h -- double-precision iterative radix-2 Cooley-Tukey DFT.
 *
 * TEST INFRASTRUCTURE (oracle).  Used by the oracle's ramp filter and by the
 * FFTW-API shim that lets the reference's rebin_filter_cpu.cu build without
 * libfftw3.  Textbook decimation-in-time: bit-reversal permutation followed by
 * log2(n) butterfly stages; twiddles from sin/cos of 2*pi*k/len.
 *
 * Convention (same as FFTW's public API): X[k] = sum_j x[j] exp(sign*2*pi*i*j*k/n),
 * sign = -1 forward, +1 backward, no normalisation.  n must be a power of two.
 */
#ifndef CTBB_ORACLE_FFT_RADIX2_H
#define CTBB_ORACLE_FFT_RADIX2_H

#include <math.h>
#include <stddef.h>

/* data: n complex values stored as interleaved (re, im) doubles, in place. */
static inline void ctbb_oracle_fft_radix2(double *data, int n, int sign)
{
    /* bit reversal */
    for (int i = 1, j = 0; i < n; ++i) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) {
            double tr = data[2 * i], ti = data[2 * i + 1];
            data[2 * i] = data[2 * j];
            data[2 * i + 1] = data[2 * j + 1];
            data[2 * j] = tr;
            data[2 * j + 1] = ti;
        }
    }
    const double two_pi = 6.283185307179586476925286766559;
    for (int len = 2; len <= n; len <<= 1) {
        int half = len >> 1;
        for (int k = 0; k < half; ++k) {
            double ang = sign * two_pi * (double)k / (double)len;
            double wr = cos(ang), wi = sin(ang);
            for (int s = 0; s < n; s += len) {
                int a = s + k, b = s + k + half;
                double br = data[2 * b] * wr - data[2 * b + 1] * wi;
                double bi = data[2 * b] * wi + data[2 * b + 1] * wr;
                data[2 * b] = data[2 * a] - br;
                data[2 * b + 1] = data[2 * a + 1] - bi;
                data[2 * a] += br;
                data[2 * a + 1] += bi;
            }
        }
    }
}

#endif
