/* Radix-2 FFT behind the FFTW stand-in (fftw3.h); written for this oracle build.  TEST
 * INFRASTRUCTURE ONLY.  Iterative Cooley-Tukey (bit-reversal permutation, then log2(n) butterfly
 * passes) in double with twiddles from cos/sin. */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "fftw3.h"

struct mdsm_fftwf_plan_s {
    int n, kind;  /* kind 0: real -> complex, 1: complex -> real */
    float *r;
    fftwf_complex *c;
};

void *fftwf_malloc(size_t n) { return calloc(1, n + 64); }
void fftwf_free(void *p) { free(p); }

static fftwf_plan mk(int n, int kind, float *r, fftwf_complex *c)
{
    if (n < 2 || (n & (n - 1))) return NULL;
    fftwf_plan p = (fftwf_plan)malloc(sizeof *p);
    p->n = n;
    p->kind = kind;
    p->r = r;
    p->c = c;
    return p;
}

fftwf_plan fftwf_plan_dft_r2c_1d(int n, float *in, fftwf_complex *out, unsigned flags)
{
    (void)flags;
    return mk(n, 0, in, out);
}

fftwf_plan fftwf_plan_dft_c2r_1d(int n, fftwf_complex *in, float *out, unsigned flags)
{
    (void)flags;
    return mk(n, 1, out, in);
}

void fftwf_destroy_plan(fftwf_plan p) { free(p); }

/* In-place complex FFT of (re, im), sign -1 forward, +1 inverse, unnormalised. */
static void fft(double *re, double *im, int n, int sign)
{
    for (int i = 1, j = 0; i < n; i++) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) {
            double t = re[i]; re[i] = re[j]; re[j] = t;
            t = im[i]; im[i] = im[j]; im[j] = t;
        }
    }
    for (int len = 2; len <= n; len <<= 1) {
        const double ang = sign * 2.0 * M_PI / len;
        for (int k = 0; k < len / 2; k++) {
            const double wr = cos(ang * k), wi = sin(ang * k);
            for (int i = k; i < n; i += len) {
                const int j = i + len / 2;
                const double xr = re[j] * wr - im[j] * wi, xi = re[j] * wi + im[j] * wr;
                re[j] = re[i] - xr;
                im[j] = im[i] - xi;
                re[i] += xr;
                im[i] += xi;
            }
        }
    }
}

void fftwf_execute(const fftwf_plan p)
{
    const int n = p->n;
    double *re = (double *)malloc(sizeof(double) * (size_t)n);
    double *im = (double *)malloc(sizeof(double) * (size_t)n);
    if (p->kind == 0) {
        for (int i = 0; i < n; i++) { re[i] = p->r[i]; im[i] = 0.0; }
        fft(re, im, n, -1);
        for (int k = 0; k <= n / 2; k++) {
            p->c[k][0] = (float)re[k];
            p->c[k][1] = (float)im[k];
        }
    } else {
        /* Hermitian extension of bins 0..n/2; bins 0 and n/2 are taken as real */
        re[0] = p->c[0][0];
        im[0] = 0.0;
        re[n / 2] = p->c[n / 2][0];
        im[n / 2] = 0.0;
        for (int k = 1; k < n / 2; k++) {
            re[k] = p->c[k][0];
            im[k] = p->c[k][1];
            re[n - k] = p->c[k][0];
            im[n - k] = -p->c[k][1];
        }
        fft(re, im, n, +1);
        for (int i = 0; i < n; i++) p->r[i] = (float)re[i];
    }
    free(re);
    free(im);
}
