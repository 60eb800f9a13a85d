/* Stand-in for the part of FFTW's single-precision interface that src/prototypes/singlepulse.cpp
 * uses; written for this oracle build (FFTW is not installed).  TEST INFRASTRUCTURE ONLY.
 * Conventions follow FFTW's documentation: transforms are unnormalised, a real-to-complex
 * transform of length n writes n/2 + 1 bins, a complex-to-real transform reads n/2 + 1 bins
 * (the imaginary parts of bin 0 and bin n/2 are ignored).  The arithmetic is a radix-2 FFT in
 * double, rounded to float on output; n must be a power of two.
 * Buffers from fftwf_malloc are zero-filled and carry 64 spare bytes: the prototype allocates
 * n/2 complex values for spectra that hold n/2 + 1 (singlepulse.cpp:169,201-203), so the last
 * bin lands in the spare bytes, and convolve() never writes that bin of its product
 * (singlepulse.cpp:74), which therefore reads as zero. */
#ifndef MDSM_FFTW_SHIM_H
#define MDSM_FFTW_SHIM_H
#include <stddef.h>
#include <stdio.h> /* FFTW's own header includes it (for its FILE-based wisdom calls) */
#ifdef __cplusplus
extern "C" {
#endif
typedef float fftwf_complex[2];
typedef struct mdsm_fftwf_plan_s *fftwf_plan;
#define FFTW_ESTIMATE (1U << 6)
fftwf_plan fftwf_plan_dft_r2c_1d(int n, float *in, fftwf_complex *out, unsigned flags);
fftwf_plan fftwf_plan_dft_c2r_1d(int n, fftwf_complex *in, float *out, unsigned flags);
void fftwf_execute(const fftwf_plan p);
void fftwf_destroy_plan(fftwf_plan p);
void *fftwf_malloc(size_t n);
void fftwf_free(void *p);
#ifdef __cplusplus
}
#endif
#endif
