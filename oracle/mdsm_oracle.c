/*
 * mdsm_oracle.c -- CPU oracle for MDSM's incoherent dedispersion search path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path, and the CPU baseline that
 * bench.py reports beside it.  Nothing in the product library calls into this file.
 *
 * Build with -ffp-contract=off: every float/double expression below is meant to be
 * evaluated exactly as written (one rounding per operation), because the reference was
 * compiled for x86-64 without FMA on the host side, and its device-side contractions are
 * restated explicitly with fmaf().
 *
 * Citations are file:line inside the MDSM source tree (src/...).
 */
#include "mdsm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------------------ */
/* delays and shift tables                                                              */
/* ------------------------------------------------------------------------------------ */

/* src/mdsm/dedispersion_manager.cpp:262-265 */
float orc_dmdelay(float f1, float f2)
{
    double a = 1.0 / (double)f1 / (double)f1;
    double b = 1.0 / (double)f2 / (double)f2;
    return (float)(4148.741601 * (a - b));
}

/* src/mdsm/dedispersion_manager.cpp:286-289: f_c = fch1 + foff*c evaluated in float. */
void orc_dmshifts(int nchans, float fch1, float foff, float *out)
{
    for (int c = 0; c < nchans; c++) {
        float fc = fch1 + foff * (float)c;
        out[c] = orc_dmdelay(fc, fch1);
    }
}

/* src/mdsm/dedispersion_manager.cpp:291-297 (brute-force branch). */
unsigned orc_ref_maxshift(const float *dmshifts, int nchans, float lowdm, float dmstep, int tdms,
                          float tsamp)
{
    float hiDM = lowdm + dmstep * (float)(unsigned)(tdms - 1);
    float v = dmshifts[nchans - 1] * hiDM;
    v = v / tsamp;
    return (unsigned)v;
}

/* One DM trial's shift for channel delay `dms` under each mode.  `idx` is the trial's index in
 * its segment, which is what the reference kernels see as blockIdx.y*blockDim.y+threadIdx.y
 * (L1 kernel) or blockIdx.y (opt kernel). */
static int32_t shift_one(float dms, double delay64, float lowdm, float dmstep, int idx, float tsamp,
                         int mode)
{
    switch (mode) {
    case ORC_SHIFT_L1_FMA:
    case ORC_SHIFT_L1_MULADD: {
        /* host side, dedispersion_thread.cu:76,85-86: startdm/tsamp and dmstep/tsamp in float */
        float mstartdm = lowdm / tsamp;
        float mdmstep = dmstep / tsamp;
        /* device side, dedispersion_kernel.cu:27 */
        float st = (mode == ORC_SHIFT_L1_FMA) ? fmaf((float)(unsigned)idx, mdmstep, mstartdm)
                                              : mstartdm + (float)(unsigned)idx * mdmstep;
        /* dedispersion_kernel.cu:36: __float2int_rz(dm_shifts[c] * shift_temp) */
        float p = dms * st;
        return (int32_t)truncf(p);
    }
    case ORC_SHIFT_OPT_FMA:
    case ORC_SHIFT_OPT_MULADD: {
        /* dedispersion_kernel.cu:54: (startdm + blockIdx.y*dmstep)/tsamp */
        float num = (mode == ORC_SHIFT_OPT_FMA) ? fmaf((float)(unsigned)idx, dmstep, lowdm)
                                                : lowdm + (float)(unsigned)idx * dmstep;
        float st = num / tsamp;
        /* dedispersion_kernel.cu:70: floor(dm_shifts[c*chanfactor]*shift_temp) */
        float p = dms * st;
        return (int32_t)floorf(p);
    }
    case ORC_SHIFT_FP64_TRUNC:
    case ORC_SHIFT_FP64_ROUND: {
        double dm = (double)lowdm + (double)idx * (double)dmstep;
        double v = delay64 * dm / (double)tsamp;
        return (mode == ORC_SHIFT_FP64_TRUNC) ? (int32_t)trunc(v) : (int32_t)floor(v + 0.5);
    }
    }
    return 0;
}

void orc_shift_table(const float *dmshifts, int nchans, double fch1, double foff, double K,
                     const orc_segment *segs, int nsegs, float tsamp, int mode, int32_t *out)
{
    double *d64 = (double *)malloc(sizeof(double) * (size_t)(nchans > 0 ? nchans : 1));
    for (int c = 0; c < nchans; c++) {
        double fc = fch1 + foff * (double)c;
        d64[c] = K * (1.0 / (fc * fc) - 1.0 / (fch1 * fch1));
    }
    long row = 0;
    for (int s = 0; s < nsegs; s++) {
        for (int i = 0; i < segs[s].ndms; i++, row++) {
            int32_t *o = out + row * (long)nchans;
            for (int c = 0; c < nchans; c++)
                o[c] = shift_one(dmshifts[c], d64[c], segs[s].lowdm, segs[s].dmstep, i, tsamp, mode);
        }
    }
    free(d64);
}

/* ------------------------------------------------------------------------------------ */
/* brute-force dedispersion                                                             */
/* ------------------------------------------------------------------------------------ */

/* src/mdsm/dedispersion_kernel.cu:24-41 (and :66-72): per output, channels summed in order
 * from 0.0f.  Loop order here is d, c, t, which keeps that per-output order. */
void orc_dedisperse_f32(const float *x, int nchans, long stride, int nsamp, const int32_t *S,
                        int ndms, float *y)
{
#pragma omp parallel for schedule(dynamic, 1)
    for (int d = 0; d < ndms; d++) {
        float *yr = y + (long)d * nsamp;
        for (int t = 0; t < nsamp; t++) yr[t] = 0.0f;
        for (int c = 0; c < nchans; c++) {
            const float *xr = x + (long)c * stride + S[(long)d * nchans + c];
            for (int t = 0; t < nsamp; t++) yr[t] += xr[t];
        }
    }
}

#define ORC_DEDISP_INT(NAME, T)                                                              \
    void NAME(const T *x, int nchans, long stride, int nsamp, const int32_t *S, int ndms,     \
              int32_t *y)                                                                    \
    {                                                                                        \
        _Pragma("omp parallel for schedule(dynamic, 1)")                                     \
        for (int d = 0; d < ndms; d++) {                                                     \
            int32_t *yr = y + (long)d * nsamp;                                               \
            for (int t = 0; t < nsamp; t++) yr[t] = 0;                                       \
            for (int c = 0; c < nchans; c++) {                                               \
                const T *xr = x + (long)c * stride + S[(long)d * nchans + c];                \
                for (int t = 0; t < nsamp; t++) yr[t] += (int32_t)xr[t];                     \
            }                                                                                \
        }                                                                                    \
    }
ORC_DEDISP_INT(orc_dedisperse_u8_i32, uint8_t)
ORC_DEDISP_INT(orc_dedisperse_u16_i32, uint16_t)
ORC_DEDISP_INT(orc_dedisperse_i16_i32, int16_t)

void orc_dedisperse_f64(const float *x, int nchans, long stride, int nsamp, const int32_t *S,
                        int ndms, double *y)
{
#pragma omp parallel for schedule(dynamic, 1)
    for (int d = 0; d < ndms; d++) {
        double *yr = y + (long)d * nsamp;
        for (int t = 0; t < nsamp; t++) yr[t] = 0.0;
        for (int c = 0; c < nchans; c++) {
            const float *xr = x + (long)c * stride + S[(long)d * nchans + c];
            for (int t = 0; t < nsamp; t++) yr[t] += (double)xr[t];
        }
    }
}

/* ------------------------------------------------------------------------------------ */
/* two-stage subband dedispersion                                                       */
/* ------------------------------------------------------------------------------------ */

/* src/mdsm/dedispersion_thread.cu:151-153 */
int orc_subband_tempval(const float *dmshifts, int nchans, int nsubs, float highdm, float tsamp)
{
    float v = dmshifts[(nsubs - 1) * (nchans / nsubs)] * highdm;
    v = v / tsamp;
    return (int)v;
}

void orc_subband_shifts(const float *dms, int nchans, int nsubs, float lowdm, float sub_dmstep,
                        int ncalls, float dmstep, int calldms, float tsamp, int use_fma,
                        int32_t *S1, int32_t *S2)
{
    int cps = nchans / nsubs;
    /* stage 1: dedispersion_kernel.cu:148,163,167 with startdm = lowdm (one device,
     * dedispersion_thread.cu:161) and dmstep = sub_dmstep */
    for (int j = 0; j < ncalls; j++) {
        float num = use_fma ? fmaf((float)(unsigned)j, sub_dmstep, lowdm)
                            : lowdm + (float)(unsigned)j * sub_dmstep;
        float st = num / tsamp;
        for (int b = 0; b < nsubs; b++) {
            int tv = (int)(dms[b * cps] * st);                       /* :163 */
            for (int c = b * cps; c < (b + 1) * cps; c++) {
                float v = use_fma ? fmaf(dms[c], st, -(float)tv)     /* :167 */
                                  : dms[c] * st - (float)tv;
                S1[(long)j * nchans + c] = (int32_t)v;
            }
        }
    }
    /* stage 2: dedispersion_thread.cu:197-205 then dedispersion_kernel.cu:54,70 with
     * chanfactor = nchans/nsubs */
    for (int j = 0; j < ncalls; j++) {
        float half = ((float)calldms * dmstep) / 2.0f;
        float a = lowdm + sub_dmstep * (float)j;
        float dm0 = a - half;
        if (!(dm0 > 0.0f)) dm0 = 0.0f;
        for (int k = 0; k < calldms; k++) {
            float num = use_fma ? fmaf((float)(unsigned)k, dmstep, dm0)
                                : dm0 + (float)(unsigned)k * dmstep;
            float st = num / tsamp;
            for (int b = 0; b < nsubs; b++)
                S2[((long)j * calldms + k) * nsubs + b] = (int32_t)floorf(dms[b * cps] * st);
        }
    }
}

/* dedispersion_kernel.cu:152-174: z[j][b][t], band rows of nsamp1 samples. */
void orc_subband_stage1_f32(const float *x, int nchans, long stride, int nsubs, int nsamp1,
                            const int32_t *S1, int ncalls, float *z)
{
    int cps = nchans / nsubs;
#pragma omp parallel for collapse(2) schedule(dynamic, 1)
    for (int j = 0; j < ncalls; j++)
        for (int b = 0; b < nsubs; b++) {
            float *zr = z + ((long)j * nsubs + b) * nsamp1;
            for (int t = 0; t < nsamp1; t++) zr[t] = 0.0f;
            for (int c = b * cps; c < (b + 1) * cps; c++) {
                const float *xr = x + (long)c * stride + S1[(long)j * nchans + c];
                for (int t = 0; t < nsamp1; t++) zr[t] += xr[t];
            }
        }
}

/* dedispersion_kernel.cu:60-76 over subband rows (nchans = nsubs), one call per sub-DM. */
void orc_subband_stage2_f32(const float *z, int nsubs, int nsamp1, int nsamp, const int32_t *S2,
                            int ncalls, int calldms, float *y)
{
#pragma omp parallel for collapse(2) schedule(dynamic, 1)
    for (int j = 0; j < ncalls; j++)
        for (int k = 0; k < calldms; k++) {
            long d = (long)j * calldms + k;
            float *yr = y + d * nsamp;
            const float *zb = z + (long)j * nsubs * nsamp1;
            for (int t = 0; t < nsamp; t++) yr[t] = 0.0f;
            for (int b = 0; b < nsubs; b++) {
                const float *zr = zb + (long)b * nsamp1 + S2[d * nsubs + b];
                for (int t = 0; t < nsamp; t++) yr[t] += zr[t];
            }
        }
}

/* ------------------------------------------------------------------------------------ */
/* reference detector                                                                   */
/* ------------------------------------------------------------------------------------ */

/* src/mdsm/dedispersion_output.cpp:14-53, the same comparison network. */
float orc_median_of_five(float n1, float n2, float n3, float n4, float n5)
{
    float *a = &n1, *b = &n2, *c = &n3, *d = &n4, *e = &n5, *tmp;
    if (*b < *a) { tmp = a; a = b; b = tmp; }
    if (*d < *c) { tmp = c; c = d; d = tmp; }
    if (*c < *a) { tmp = b; b = d; d = tmp; c = a; }
    a = e;
    if (*b < *a) { tmp = a; a = b; b = tmp; }
    if (*a < *c) { tmp = b; b = d; d = tmp; a = c; }
    if (*d < *a) return *d;
    return *a;
}

/* src/mdsm/dedispersion_output.cpp:144-169: 32K-value chunks, each summed in double; the
 * running mean is a float; the last chunk is skipped by the loop's exit test (:164). */
void orc_ref_stats(const float *buf, unsigned vals, float *mean_out, float *rms_out)
{
    unsigned mod = vals < 32u * 1024u ? vals : 32u * 1024u;
    unsigned iters = 0, j = 0;
    double mean2 = 0.0;
    float localmean = 0.0f;
    for (;;) {
        double total = 0.0, total2 = 0.0;
        for (j = 0; j < mod; j++) {
            double v = (double)buf[(size_t)iters * mod + j];
            total += v;
            total2 += v * v;
        }
        localmean = (float)((double)localmean + total / (double)j);
        mean2 += total2 / (double)j;
        iters++;
        if ((unsigned)(iters * mod + j) >= vals) break;
    }
    localmean = localmean / (float)iters;
    float sq = localmean * localmean;
    float localrms = (float)sqrt(mean2 / (double)iters - (double)sq);
    *mean_out = localmean;
    *rms_out = localrms;
}

/* src/mdsm/dedispersion_output.cpp:176-210 with num_threads = 1 and mean == NULL. */
long orc_ref_detect(const float *buf, int tdms, int nsamp, float lowdm, float dmstep,
                    float threshold, float mean, float rms, int32_t *dm_idx, int32_t *samp,
                    float *snr, long cap)
{
    long n = 0;
    float lim = rms * threshold;
    for (int k = 0; k < tdms; k++) {
        float thisdm = (lowdm + 0.0f) + (float)(unsigned)k * dmstep;
        if (!((double)thisdm > 1.0)) continue;
        const float *r = buf + (long)k * nsamp;
        for (unsigned l = 0; l < (unsigned)nsamp - 4u; l++) {
            float m = orc_median_of_five(r[l], r[l + 1], r[l + 2], r[l + 3], r[l + 4]);
            if (m - mean >= lim) {
                if (n < cap) {
                    dm_idx[n] = k;
                    samp[n] = (int32_t)l;
                    snr[n] = m / rms;
                }
                n++;
            }
        }
    }
    return n;
}

long orc_ref_detect_chunked(const float *buf, int tdms, int nsamp, float lowdm, float dmstep,
                            float threshold, const float *mean, const float *rms, int spc,
                            int32_t *dm_idx, int32_t *samp, float *snr, long cap)
{
    long n = 0;
    for (int k = 0; k < tdms; k++) {
        float thisdm = (lowdm + 0.0f) + (float)(unsigned)k * dmstep;
        if (!((double)thisdm > 1.0)) continue;
        const float *r = buf + (long)k * nsamp;
        for (unsigned l = 0; l < (unsigned)nsamp - 4u; l++) {
            float m = orc_median_of_five(r[l], r[l + 1], r[l + 2], r[l + 3], r[l + 4]);
            float cm = mean[l / (unsigned)spc], cr = rms[l / (unsigned)spc];
            float lim = cr * threshold;
            if (m - cm >= lim) {
                if (n < cap) {
                    dm_idx[n] = k;
                    samp[n] = (int32_t)l;
                    snr[n] = (m - cm) / cr;
                }
                n++;
            }
        }
    }
    return n;
}

long orc_ref_detect_subband(const float *buf, long stride, int nrows, int nvalid,
                            const float *dmv, float threshold, const float *mean,
                            const float *rms, int spc, int32_t *dm_idx, int32_t *samp,
                            float *snr, long cap)
{
    long n = 0;
    for (int k = 0; k < nrows; k++) {
        const float *r = buf + (long)k * stride;
        float lm = 0.0f, lr = 0.0f;
        if (!mean) {
            double total = 0.0, total2 = 0.0;
            for (int t = 0; t < nvalid; t++) {
                total += (double)r[t];
                total2 += (double)r[t] * (double)r[t];  /* pow(x, 2): exact for a float x */
            }
            lm = (float)(total / nvalid);
            lr = (float)sqrt(total2 / nvalid - (double)lm * (double)lm);
        }
        if (!((double)dmv[k] > 1.0)) continue;
        for (unsigned t = 0; t < (unsigned)nvalid - 4u; t++) {
            float m = orc_median_of_five(r[t], r[t + 1], r[t + 2], r[t + 3], r[t + 4]);
            float cm = mean ? mean[t / (unsigned)spc] : lm;
            float cr = mean ? rms[t / (unsigned)spc] : lr;
            float lim = cr * threshold;
            if (m - cm >= lim) {
                if (n < cap) {
                    dm_idx[n] = k;
                    samp[n] = (int32_t)t;
                    snr[n] = m / cr;
                }
                n++;
            }
        }
    }
    return n;
}

/* ------------------------------------------------------------------------------------ */
/* RFI clipping                                                                         */
/* ------------------------------------------------------------------------------------ */

/* Reads element i of a row of the given kind as double. */
static double rd(const void *x, int kind, long i)
{
    switch (kind) {
    case 0: return (double)((const uint8_t *)x)[i];
    case 1: return (double)((const uint16_t *)x)[i];
    case 2: return (double)((const int16_t *)x)[i];
    default: return (double)((const float *)x)[i];
    }
}

static void wr(void *x, int kind, long i, double v)
{
    switch (kind) {
    case 0: { double r = nearbyint(v); r = r < 0 ? 0 : (r > 255 ? 255 : r);
              ((uint8_t *)x)[i] = (uint8_t)r; break; }
    case 1: { double r = nearbyint(v); r = r < 0 ? 0 : (r > 65535 ? 65535 : r);
              ((uint16_t *)x)[i] = (uint16_t)r; break; }
    case 2: { double r = nearbyint(v); r = r < -32768 ? -32768 : (r > 32767 ? 32767 : r);
              ((int16_t *)x)[i] = (int16_t)r; break; }
    default: ((float *)x)[i] = (float)v; break;
    }
}

/* Mean and sigma over n elements at x + i*step.  Integer kinds: exact int64 sums.
 * Float kind: runs of 1024 elements, each summed left to right in double, partials summed
 * left to right. */
static void clip_stats(const void *x, int kind, long base, long step, long n, double *mu,
                       double *sig)
{
    double m, var;
    if (kind != 3) {
        long long s1 = 0, s2 = 0;
        for (long i = 0; i < n; i++) {
            long long v = (long long)rd(x, kind, base + i * step);
            s1 += v;
            s2 += v * v;
        }
        m = (double)s1 / (double)n;
        var = (double)s2 / (double)n - m * m;
    } else {
        double s1 = 0.0, s2 = 0.0;
        for (long c0 = 0; c0 < n; c0 += 1024) {
            double p1 = 0.0, p2 = 0.0;
            long c1 = c0 + 1024 < n ? c0 + 1024 : n;
            for (long i = c0; i < c1; i++) {
                double v = rd(x, kind, base + i * step);
                p1 += v;
                p2 += v * v;
            }
            s1 += p1;
            s2 += p2;
        }
        m = s1 / (double)n;
        var = s2 / (double)n - m * m;
    }
    *mu = m;
    *sig = var > 0.0 ? sqrt(var) : 0.0;
}

/* src/prototypes/rfi_clipper.cu:8-67 per row: mean and sigma, then |x - mean| >= k*sigma is
 * replaced by the mean.  Deviations: the accumulators start at zero (:33 leaves them
 * uninitialised) and the |x - mean| <= sigma/4 branch (:61) is not applied. */
void orc_rfi_clip(void *x, int kind, int nchans, long stride, long len, double k_chan,
                  double k_spec)
{
    if (k_chan > 0.0) {
#pragma omp parallel for schedule(dynamic, 1)
        for (int c = 0; c < nchans; c++) {
            double mu, sig;
            clip_stats(x, kind, (long)c * stride, 1, len, &mu, &sig);
            double lim = k_chan * sig;
            for (long i = 0; i < len; i++) {
                long at = (long)c * stride + i;
                if (fabs(rd(x, kind, at) - mu) >= lim) wr(x, kind, at, mu);
            }
        }
    }
    if (k_spec > 0.0) {
#pragma omp parallel for schedule(dynamic, 256)
        for (long t = 0; t < len; t++) {
            double mu, sig;
            clip_stats(x, kind, t, stride, nchans, &mu, &sig);
            double lim = k_spec * sig;
            for (int c = 0; c < nchans; c++) {
                long at = (long)c * stride + t;
                if (fabs(rd(x, kind, at) - mu) >= lim) wr(x, kind, at, mu);
            }
        }
    }
}

/* ------------------------------------------------------------------------------------ */
/* boxcar single-pulse detector                                                         */
/* ------------------------------------------------------------------------------------ */

void orc_series_stats(const double *y, long n, double *mean, double *sigma)
{
    double s1 = 0.0, s2 = 0.0;
    for (long c0 = 0; c0 < n; c0 += 1024) {
        double p1 = 0.0, p2 = 0.0;
        long c1 = c0 + 1024 < n ? c0 + 1024 : n;
        for (long i = c0; i < c1; i++) {
            p1 += y[i];
            p2 += y[i] * y[i];
        }
        s1 += p1;
        s2 += p2;
    }
    double m = s1 / (double)n;
    double var = s2 / (double)n - m * m;
    *mean = m;
    *sigma = var > 0.0 ? sqrt(var) : 0.0;
}

/* src/prototypes/singlepulse.cpp restated: boxcars normalised by 1/sqrt(w) (:41-67), a
 * threshold (:240-245), and pruning of neighbours around the strongest response (:90-146),
 * here as a per-sample best width followed by non-maximum suppression. */
/* Exact statistics of an integer series: sum in int64, sum of squares in 128 bits, then
 * mean = S1/n and sigma = sqrt(S2/n - mean^2) in double, with S2 converted as
 * hi*2^64 + lo (two roundings). */
void orc_series_stats_int(const double *y, long n, double *mean, double *sigma)
{
    long long s1 = 0;
    unsigned __int128 s2 = 0;
    for (long i = 0; i < n; i++) {
        long long v = (long long)y[i];
        s1 += v;
        s2 += (unsigned __int128)((unsigned long long)(v * v));
    }
    unsigned long long hi = (unsigned long long)(s2 >> 64), lo = (unsigned long long)s2;
    double e2 = ((double)hi * 18446744073709551616.0 + (double)lo) / (double)n;
    double m = (double)s1 / (double)n;
    double var = e2 - m * m;
    *mean = m;
    *sigma = var > 0.0 ? sqrt(var) : 0.0;
}

/* One DM row of orc_boxcar_detect; returns the candidates found, appended to *out (grown). */
typedef struct { int32_t samp, width; float snr; } BoxCand;

static long boxcar_row(const double *yr, long n, int nw, float thr, int is_int, float *B,
                       float *best, int *bw, BoxCand **out, long *capo)
{
    double mu, sig;
    if (is_int)
        orc_series_stats_int(yr, n, &mu, &sig);
    else
        orc_series_stats(yr, n, &mu, &sig);
    if (!(sig > 0.0)) return 0;
    const float mu_f = (float)mu;
    for (long t = 0; t < n; t++) B[t] = (float)yr[t];
    for (long t = 0; t < n; t++) { best[t] = -INFINITY; bw[t] = 0; }
    for (int l = 0; l < nw; l++) {
        long w = 1L << l;
        if (l > 0) {
            long h = w / 2;
            for (long t = 0; t + w <= n; t++) B[t] = B[t] + B[t + h];
        }
        const float wm = (float)w * mu_f;
        const float inv = (float)(1.0 / (sig * sqrt((double)w)));
        for (long t = 0; t + w <= n; t++) {
            const float s = (B[t] - wm) * inv;
            if (s > best[t]) { best[t] = s; bw[t] = (int)w; }
        }
    }
    long cnt = 0;
    for (long t = 0; t < n; t++) {
        if (!(best[t] >= thr)) continue;
        long h = bw[t] / 2 > 1 ? bw[t] / 2 : 1;
        int keep = 1;
        long lo = t - h < 0 ? 0 : t - h, hi = t + h > n - 1 ? n - 1 : t + h;
        for (long u = lo; u < t && keep; u++) if (!(best[u] < best[t])) keep = 0;
        for (long u = t + 1; u <= hi && keep; u++) if (!(best[u] <= best[t])) keep = 0;
        if (!keep) continue;
        if (cnt == *capo) {
            *capo = *capo ? 2 * *capo : 64;
            *out = (BoxCand *)realloc(*out, sizeof(BoxCand) * (size_t)*capo);
        }
        (*out)[cnt].samp = (int32_t)t;
        (*out)[cnt].width = bw[t];
        (*out)[cnt].snr = best[t];
        cnt++;
    }
    return cnt;
}

long orc_boxcar_detect(const double *y, int ndms, long n, int nw, double threshold,
                       int32_t *dm_idx, int32_t *samp, int32_t *width, float *snr, long cap,
                       int is_int)
{
    const float thr = (float)threshold;
    BoxCand **rows = (BoxCand **)calloc((size_t)(ndms > 0 ? ndms : 1), sizeof(BoxCand *));
    long *cnt = (long *)calloc((size_t)(ndms > 0 ? ndms : 1), sizeof(long));
    /* rows are independent: one per thread at a time, each with its own work arrays */
#pragma omp parallel
    {
        float *B = (float *)malloc(sizeof(float) * (size_t)n);
        float *best = (float *)malloc(sizeof(float) * (size_t)n);
        int *bw = (int *)malloc(sizeof(int) * (size_t)n);
#pragma omp for schedule(dynamic, 1)
        for (int d = 0; d < ndms; d++) {
            long capo = 0;
            cnt[d] = boxcar_row(y + (long)d * n, n, nw, thr, is_int, B, best, bw, &rows[d], &capo);
        }
        free(B);
        free(best);
        free(bw);
    }
    long total = 0;
    for (int d = 0; d < ndms; d++) {
        for (long i = 0; i < cnt[d]; i++) {
            if (total < cap) {
                dm_idx[total] = d;
                samp[total] = rows[d][i].samp;
                width[total] = rows[d][i].width;
                snr[total] = rows[d][i].snr;
            }
            total++;
        }
        free(rows[d]);
    }
    free(rows);
    free(cnt);
    return total;
}

/* ------------------------------------------------------------------------------------ */
/* sigproc unpack and detrend                                                           */
/* ------------------------------------------------------------------------------------ */

/* src/mdsm/file_handler.cpp:193-290 (and char2ints/char4ints at :11-24). */
long orc_unpack(const uint8_t *raw, long nbytes, int nbits, float *out)
{
    long k = 0;
    switch (nbits) {
    case 1:
        for (long i = 0; i < nbytes; i++)
            for (int j = 0; j < 8; j++) out[k++] = (float)((raw[i] >> j) & 1);
        return k;
    case 2:
        for (long i = 0; i < nbytes; i++)
            for (int j = 0; j < 4; j++) out[k++] = (float)((raw[i] >> (2 * j)) & 3);
        return k;
    case 4:
        for (long i = 0; i < nbytes; i++) {
            out[k++] = (float)(raw[i] & 15);
            out[k++] = (float)((raw[i] & 240) >> 4);
        }
        return k;
    case 8:
        for (long i = 0; i < nbytes; i++) out[k++] = (float)raw[i];
        return k;
    case 16:
        for (long i = 0; i + 1 < nbytes; i += 2) {
            uint16_t v = (uint16_t)(raw[i] | ((uint16_t)raw[i + 1] << 8));
            out[k++] = (float)v;
        }
        return k;
    case 32:
        memcpy(out, raw, (size_t)(nbytes / 4) * 4);
        return nbytes / 4;
    }
    return -1;
}

/* src/prototypes/detrend.cu:12-100: per block, least-squares line on x = -len/2 + 0.5 + i,
 * subtract it, divide by the residual rms.  Evaluated in double. */
void orc_detrend_normalise(float *y, long n, int len)
{
#pragma omp parallel for schedule(static)
    for (long b0 = 0; b0 < n - len + 1; b0 += len) {
        double sy = 0, sxy = 0, sxx = 0;
        for (int i = 0; i < len; i++) {
            double xi = -len / 2.0 + 0.5 + i;
            sy += y[b0 + i];
            sxy += xi * y[b0 + i];
            sxx += xi * xi;
        }
        double a = sy / len, bb = sxy / sxx, ss = 0;
        for (int i = 0; i < len; i++) {
            double xi = -len / 2.0 + 0.5 + i;
            double v = y[b0 + i] - (a + bb * xi);
            y[b0 + i] = (float)v;
            ss += v * v;
        }
        double sd = sqrt(ss / len);
        for (int i = 0; i < len; i++) y[b0 + i] = (float)(y[b0 + i] / sd);
    }
}

/* ------------------------------------------------------------------------------------ */
/* single-pulse search in the prototype's template form                                */
/* ------------------------------------------------------------------------------------ */

/* src/prototypes/singlepulse.cpp:20 -- the downfactor ladder; :161-164 keeps the factors up to
 * maxDownfact.  widths[0] = 1 (the unsmoothed series, :240-245), then the kept factors. */
static const int kSpDownfactors[12] = {2, 3, 4, 6, 9, 14, 20, 30, 45, 70, 100, 150};

int orc_sp_widths(int max_downfact, int *widths)
{
    int nw = 0;
    widths[nw++] = 1;
    for (int i = 0; i < 12 && kSpDownfactors[i] <= max_downfact; i++) widths[nw++] = kSpDownfactors[i];
    return nw;
}

/* src/prototypes/singlepulse.cpp:90-120 and the store test at :279, as written.  For each
 * candidate x not yet masked, every later candidate y within factor/2 bins that is not masked
 * either gets mask 1 if x.value > y.value, else mask = (char)(x's list index): the prototype
 * writes `mask[j] = i` where `mask[i] = 1` was presumably meant, so y is still masked unless
 * x's index is a multiple of 256 (then y survives).  keep[i] = mask[i] == 0 and the value is
 * not 0 (masked entries are zeroed and the caller stores only non-zero values). */
void orc_sp_prune_related(const int32_t *bins, const float *values, long num, int factor,
                          unsigned char *keep)
{
    char *mask = (char *)calloc((size_t)(num > 0 ? num : 1), 1);
    for (long i = 0; i + 1 < num; i++) {
        if (mask[i]) continue;
        for (long j = i + 1; j < num; j++) {
            if ((unsigned)(bins[j] - bins[i]) > (unsigned)factor / 2u) break;
            if (mask[j]) continue;
            if (values[i] > values[j]) mask[j] = 1;
            else mask[j] = (char)(i & 0xff);
        }
    }
    for (long i = 0; i < num; i++) keep[i] = (unsigned char)(!mask[i] && values[i] != 0.0f);
    free(mask);
}

/* src/prototypes/singlepulse.cpp:122-146, as written, with the mask starting at zero: for each
 * unmasked x and each later y (list order) until |y.bin - x.bin| > maxdf/2, an unmasked y
 * within max(x.df/2, y.df/2, 1) bins masks the weaker of the two (x when the values tie). */
void orc_sp_prune_downfactors(const int64_t *bins, const float *values, const int32_t *df,
                              long n, int maxdf, unsigned char *mask)
{
    memset(mask, 0, (size_t)n);
    for (long i = 0; i < n; i++) {
        if (mask[i]) continue;
        for (long j = i + 1; j < n; j++) {
            const long long d = llabs((long long)(bins[j] - bins[i]));
            if (d > (long long)((unsigned)maxdf / 2u)) break;
            if (mask[j]) continue;
            unsigned prox = (unsigned)df[i] / 2u > (unsigned)df[j] / 2u ? (unsigned)df[i] / 2u
                                                                        : (unsigned)df[j] / 2u;
            prox = prox > 1u ? prox : 1u;
            if (d <= (long long)prox) {
                if (values[i] > values[j]) mask[j] = 1;
                else mask[i] = 1;
            }
        }
    }
}

/* Template response of width w at sample t: the series in float (0 outside [0, n)), summed
 * left to right over [t - w/2, t - w/2 + w) in FP32, then (sum - w*mu) * inv.  The prototype
 * convolves with the same centred template (:41-67; the odd widths centred on t, the even ones
 * one sample longer on the left) by FFT; this direct sum is its exact value. */
static float sp_value(const float *x, long n, long t, int w, float mu_f, float inv)
{
    const long s = t - w / 2;
    float acc = (s >= 0 && s < n) ? x[s] : 0.0f;
    for (int k = 1; k < w; k++) {
        const long u = s + k;
        acc = acc + ((u >= 0 && u < n) ? x[u] : 0.0f);
    }
    return (acc - (float)w * mu_f) * inv;
}

void orc_sp_values(const double *y, long n, int w, int normalise, int is_int, float *out)
{
    float *x = (float *)malloc(sizeof(float) * (size_t)n);
    for (long t = 0; t < n; t++) x[t] = (float)y[t];
    double mu = 0.0, sig = 1.0;
    if (normalise) {
        if (is_int) orc_series_stats_int(y, n, &mu, &sig);
        else orc_series_stats(y, n, &mu, &sig);
    }
    const float mu_f = (float)mu, inv = (float)(1.0 / (sig * sqrt((double)w)));
    for (long t = 0; t < n; t++) out[t] = sp_value(x, n, t, w, mu_f, inv);
    free(x);
}

/* The prototype's search (singlepulse.cpp:148-300) per DM row, in chunks of chunk_len samples:
 * for each chunk and each width (1 first, then the ladder) the samples whose response is >=
 * threshold form a list in sample order; lists of widths > 1 are pruned with pruneRelated; the
 * survivors of all chunks and widths, in that order, are pruned with pruneRelatedDownfactors
 * and the unmasked ones are the candidates (dm, sample, width, response).
 * Deviations, each a defect of the prototype's main loop: the first chunk reads its own DM row
 * (:229 reads row 0), every sample of a chunk is searched (:240,261 stop `overlap` samples
 * short), a trailing partial chunk is searched too (:186 drops it), a candidate carries its own
 * sample and value (:243 adds the overlap to the sample, :281 takes the value of entry j and
 * the list index as the sample), the list loop does not reuse the DM loop's counter (:295),
 * the downfactor mask starts at zero and the unmasked candidates are kept (:291-297 keeps the
 * masked ones of an uninitialised mask), and the response is the exact template sum (the
 * prototype's spectra hold n/2 bins where the real transform has n/2 + 1).
 * normalise = 0 takes the series as already normalised (mean 0, sigma 1), as the prototype
 * does; 1 uses the row's mean and sigma (orc_series_stats_int for integer series). */
long orc_singlepulse_detect(const double *y, int ndms, long n, int max_downfact, long chunk_len,
                            int normalise, int is_int, double threshold, int32_t *dm_idx,
                            int32_t *samp, int32_t *width, float *snr, long cap)
{
    int widths[13];
    const int nw = orc_sp_widths(max_downfact, widths);
    const int maxdf = widths[nw - 1];
    const float thr = (float)threshold;
    long total = 0;
    float *x = (float *)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1));
    int32_t *lb = (int32_t *)malloc(sizeof(int32_t) * (size_t)(chunk_len + 1));
    float *lv = (float *)malloc(sizeof(float) * (size_t)(chunk_len + 1));
    unsigned char *keep = (unsigned char *)malloc((size_t)(chunk_len + 1));
    for (int d = 0; d < ndms; d++) {
        const double *yr = y + (long)d * n;
        for (long t = 0; t < n; t++) x[t] = (float)yr[t];
        double mu = 0.0, sig = 1.0;
        if (normalise) {
            if (is_int) orc_series_stats_int(yr, n, &mu, &sig);
            else orc_series_stats(yr, n, &mu, &sig);
            if (!(sig > 0.0)) continue;
        }
        const float mu_f = (float)mu;
        float inv[13];
        for (int k = 0; k < nw; k++) inv[k] = (float)(1.0 / (sig * sqrt((double)widths[k])));
        long cnt = 0, capc = 1024;
        int64_t *cb = (int64_t *)malloc(sizeof(int64_t) * (size_t)capc);
        float *cv = (float *)malloc(sizeof(float) * (size_t)capc);
        int32_t *cw = (int32_t *)malloc(sizeof(int32_t) * (size_t)capc);
        for (long c0 = 0; c0 < n; c0 += chunk_len) {
            const long c1 = c0 + chunk_len < n ? c0 + chunk_len : n;
            for (int k = 0; k < nw; k++) {
                long num = 0;
                for (long t = c0; t < c1; t++) {
                    const float v = sp_value(x, n, t, widths[k], mu_f, inv[k]);
                    if (v >= thr) {
                        lb[num] = (int32_t)(t - c0);
                        lv[num] = v;
                        num++;
                    }
                }
                if (num == 0) continue;
                if (k > 0) orc_sp_prune_related(lb, lv, num, widths[k], keep);
                else for (long i = 0; i < num; i++) keep[i] = 1;
                for (long i = 0; i < num; i++) {
                    if (!keep[i]) continue;
                    if (cnt == capc) {
                        capc *= 2;
                        cb = (int64_t *)realloc(cb, sizeof(int64_t) * (size_t)capc);
                        cv = (float *)realloc(cv, sizeof(float) * (size_t)capc);
                        cw = (int32_t *)realloc(cw, sizeof(int32_t) * (size_t)capc);
                    }
                    cb[cnt] = c0 + lb[i];
                    cv[cnt] = lv[i];
                    cw[cnt] = widths[k];
                    cnt++;
                }
            }
        }
        unsigned char *mask = (unsigned char *)malloc((size_t)(cnt > 0 ? cnt : 1));
        orc_sp_prune_downfactors(cb, cv, cw, cnt, maxdf, mask);
        for (long i = 0; i < cnt; i++) {
            if (mask[i]) continue;
            if (total < cap) {
                dm_idx[total] = d;
                samp[total] = (int32_t)cb[i];
                width[total] = cw[i];
                snr[total] = cv[i];
            }
            total++;
        }
        free(mask);
        free(cb);
        free(cv);
        free(cw);
    }
    free(x);
    free(lb);
    free(lv);
    free(keep);
    return total;
}

/* ------------------------------------------------------------------------------------ */
/* the prototype kernels' own float arithmetic (to pin the oracle to their GPU output)  */
/* ------------------------------------------------------------------------------------ */

/* src/prototypes/detrend.cu:12-100 in its own float arithmetic and order, for a block of 256
 * threads: per-thread strided sums, a shared-memory tree (:41-51), the line fit in thread 0
 * (:55-56), the residuals (:67-75), a second tree (:83-85) and the division by the rms
 * (:90,97-99).  The second tree has no barrier between its steps in the prototype; this
 * restatement takes the synchronised order.  contract bit 1: the products summed into sxy, sxx
 * and the rms are fused multiply-adds; bit 2: the fitted line a + b*x is one. */
void orc_detrend_ref_f32(float *y, int ndms, int nsamp, int len, int contract)
{
    enum { NT = 256 };
    const int nblk = nsamp / len;
#pragma omp parallel for schedule(static)
    for (long blk = 0; blk < (long)ndms * nblk; blk++) {
        float *in = y + blk * len;
        float sx[NT], sy[NT], sz[NT];
        for (int tid = 0; tid < NT; tid++) {
            float a = 0, b = 0, c = 0;
            for (int i = tid; i < len; i += NT) {
                const float x = (float)(-len / 2.0 + 0.5 + i);
                const float v = in[i];
                a = a + v;
                if (contract & 1) {
                    b = fmaf(x, v, b);
                    c = fmaf(x, x, c);
                } else {
                    b = b + x * v;
                    c = c + x * x;
                }
            }
            sx[tid] = a;
            sy[tid] = b;
            sz[tid] = c;
        }
        for (int h = NT / 2; h >= 1; h /= 2)
            for (int tid = 0; tid < h; tid++) {
                sx[tid] = sx[tid] + sx[tid + h];
                sy[tid] = sy[tid] + sy[tid + h];
                sz[tid] = sz[tid] + sz[tid + h];
            }
        const float bb = sy[0] / sz[0];
        const float aa = sx[0] / (float)len;
        for (int tid = 0; tid < NT; tid++) {
            float s = 0;
            for (int i = tid; i < len; i += NT) {
                const float x = (float)(-len / 2.0 + 0.5 + i);
                const float line = (contract & 2) ? fmaf(bb, x, aa) : aa + bb * x;
                const float val = in[i] - line;
                in[i] = val;
                s = (contract & 1) ? fmaf(val, val, s) : s + val * val;
            }
            sz[tid] = s;
        }
        for (int h = NT / 2; h >= 1; h /= 2)
            for (int tid = 0; tid < h; tid++) sz[tid] = sz[tid] + sz[tid + h];
        const float sd = sqrtf(sz[0] / (float)len);
        for (int i = 0; i < len; i++) in[i] = in[i] / sd;
    }
}

/* src/prototypes/rfi_clipper.cu:8-67 in its own float arithmetic and order, rows [nrows][nsamp],
 * blockdim threads per row: per-thread strided sums (:17-25), thread 0's sequential sum of the
 * partials (:34-37) starting from zero (the prototype leaves val1/val2 uninitialised), mean and
 * standard deviation (:40-41), and the clip |x - mean| >= 4 sigma or <= sigma/4 to the mean
 * (:60-62).  contract bit 1: the squares summed are fused multiply-adds; bit 2: val2 -
 * (nsamp*mean)*mean is one.  means[r] receives the row mean. */
void orc_rfi_clip_ref_f32(float *x, int nrows, int nsamp, int blockdim, int contract,
                          float *means)
{
#pragma omp parallel for schedule(static)
    for (int r = 0; r < nrows; r++) {
        float *row = x + (long)r * nsamp;
        float *p1 = (float *)calloc((size_t)blockdim, sizeof(float));
        float *p2 = (float *)calloc((size_t)blockdim, sizeof(float));
        for (int tid = 0; tid < blockdim; tid++)
            for (int s = tid; s < nsamp; s += blockdim) {
                const float v = row[s];
                p1[tid] = p1[tid] + v;
                p2[tid] = (contract & 1) ? fmaf(v, v, p2[tid]) : p2[tid] + v * v;
            }
        float v1 = 0.0f, v2 = 0.0f;
        for (int i = 0; i < blockdim; i++) {
            v1 = v1 + p1[i];
            v2 = v2 + p2[i];
        }
        const float mean = v1 / (float)nsamp;
        const float nm = (float)nsamp * mean;
        const float num = (contract & 2) ? fmaf(-nm, mean, v2) : v2 - nm * mean;
        const float sd = sqrtf(num / (float)nsamp);
        means[r] = mean;
        for (int s = 0; s < nsamp; s++) {
            const float v = row[s];
            const float tv = fabsf(v - mean);
            if (tv >= sd * 4.0f || tv <= sd / 4.0f) row[s] = mean;
        }
        free(p1);
        free(p2);
    }
}
