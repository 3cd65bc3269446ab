/* Oracle FFT (TEST INFRASTRUCTURE ONLY - the GPU library never links it).
 *
 * The reference solves its constant-coefficient Poisson preconditioner with
 * Sandia's parallel fft_3d (Plimpton) on FFTW 2.1.5 (poisson.cpp:87,431,453,
 * makefile:4-14).  Neither library is vendored in the reference, so this file
 * restates the published algorithm they implement: an unscaled complex
 * discrete Fourier transform,
 *     X[k] = sum_n x[n] exp(sign * 2*pi*i*n*k/N),
 * computed here by a mixed-radix (4, 2, 3, 5) Stockham auto-sort FFT in double
 * precision with twiddles taken directly from libm cos/sin (no recurrences).
 * Roundoff is O(eps log N), the same class as FFTW.  Pinned against numpy.fft
 * by the known-answer tests in tests/test_oracle_fft.py.
 */
#ifndef TPM_ORACLE_OFFT_H
#define TPM_ORACLE_OFFT_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct offt_plan offt_plan;

/* n must factor into 2, 3 and 5; returns NULL otherwise. */
offt_plan *offt_plan_create(int n);
void offt_plan_destroy(offt_plan *p);

/* In-place transform of `count` interleaved (re,im) sequences of length n.
 * Element t of sequence s sits at data[2*(s*seq_stride + t*elem_stride)].
 * sign = -1: forward (exp(-i...)), sign = +1: backward.  Unscaled. */
void offt_many(offt_plan *p, double *data, long count, long seq_stride, long elem_stride,
               int sign);

/* Unscaled 3-D complex transform of an x-fastest [nz][ny][nx] interleaved array. */
void offt_3d(double *data, int nx, int ny, int nz, int sign);

#ifdef __cplusplus
}
#endif
#endif
