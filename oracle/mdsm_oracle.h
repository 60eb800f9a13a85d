/*
 * mdsm_oracle.h -- CPU oracle for MDSM's incoherent dedispersion search path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA path
 * is compared against.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg (and its reference arm) may load it.  The product library
 * (mdsm_gb300/) never links, loads or calls anything in oracle/.
 *
 * Every function restates one piece of the reference algorithm and cites the
 * reference file:line it follows (paths relative to the MDSM source tree).
 */
#ifndef MDSM_ORACLE_H_
#define MDSM_ORACLE_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Shift-table modes (how an integer sample shift is derived from a DM). */
enum {
    ORC_SHIFT_L1_FMA    = 0, /* dedispersion_kernel.cu:27,36 with a + i*b contracted to fma   */
    ORC_SHIFT_L1_MULADD = 1, /* dedispersion_kernel.cu:27,36 evaluated as mul then add        */
    ORC_SHIFT_OPT_FMA   = 2, /* dedispersion_kernel.cu:54,70 (floor), start + i*step as fma    */
    ORC_SHIFT_OPT_MULADD= 3, /* dedispersion_kernel.cu:54,70 (floor), mul then add             */
    ORC_SHIFT_FP64_TRUNC= 4, /* exact double delay, truncated                                  */
    ORC_SHIFT_FP64_ROUND= 5  /* exact double delay, rounded to nearest (pulse-injection rule)  */
};

/* One uniform run of DM trials: dm_i = lowdm + i*dmstep, i < ndms. */
typedef struct {
    float lowdm;
    float dmstep;
    int   ndms;
} orc_segment;

/* dedispersion_manager.cpp:262-265 -- 4148.741601*(f1^-2 - f2^-2) in double, returned as float. */
float orc_dmdelay(float f1, float f2);

/* dedispersion_manager.cpp:286-289 -- per-channel delay (seconds per unit DM), float[nchans]. */
void orc_dmshifts(int nchans, float fch1, float foff, float *out);

/* dedispersion_manager.cpp:291-297 -- the reference's maxshift for a brute-force plan. */
unsigned orc_ref_maxshift(const float *dmshifts, int nchans, float lowdm, float dmstep, int tdms,
                          float tsamp);

/* Integer shift table S[d][c] (row-major, ndms x nchans) for a multi-segment plan.
 * K is the dispersion constant used by the FP64 modes only (the FP32 modes take the
 * delays from dmshifts[], which were built with 4148.741601). */
void orc_shift_table(const float *dmshifts, int nchans, double fch1, double foff, double K,
                     const orc_segment *segs, int nsegs, float tsamp, int mode, int32_t *out);

/* Brute-force dedispersion y[d][t] = sum_c x[c][t + S[d][c]] for t < nsamp.
 * Input rows are channel-major with `stride` elements per channel.  Channels are summed in
 * order c = 0..nchans-1 starting from 0, as dedispersion_kernel.cu:24-41 and :66-72 do, so the
 * float result is bit-identical to the reference's float accumulation. */
void orc_dedisperse_f32(const float *x, int nchans, long stride, int nsamp, const int32_t *S,
                        int ndms, float *y);
void orc_dedisperse_u8_i32(const uint8_t *x, int nchans, long stride, int nsamp,
                           const int32_t *S, int ndms, int32_t *y);
void orc_dedisperse_u16_i32(const uint16_t *x, int nchans, long stride, int nsamp,
                            const int32_t *S, int ndms, int32_t *y);
void orc_dedisperse_i16_i32(const int16_t *x, int nchans, long stride, int nsamp,
                            const int32_t *S, int ndms, int32_t *y);
/* FP64 oracle: same sum in double (exact for integer-valued input). */
void orc_dedisperse_f64(const float *x, int nchans, long stride, int nsamp, const int32_t *S,
                        int ndms, double *y);

/* ---- two-stage subband dedispersion (binsize 1) ----
 * Stage 1, dedispersion_kernel.cu:144-175 launched as dedispersion_thread.cu:146-172:
 *   z[j][b][t] = sum_{c in band b} x[c][t + (int)(dms[c]*st_j - (int)(dms[b*cps]*st_j))],
 *   st_j = (lowdm + j*sub_dmstep)/tsamp, t < nsamp1 = nsamp + tempval.
 * Stage 2, dedispersion_kernel.cu:51-77 launched as dedispersion_thread.cu:186-210:
 *   y[j*calldms + k][t] = sum_b z[j][b][t + floor(dms[b*cps] * (dm0_j + k*dmstep)/tsamp)],
 *   dm0_j = max(lowdm + j*sub_dmstep - calldms*dmstep/2, 0).
 * use_fma selects the contracted evaluation of start + i*step.
 */
void orc_subband_shifts(const float *dmshifts, int nchans, int nsubs, float lowdm,
                        float sub_dmstep, int ncalls, float dmstep, int calldms, float tsamp,
                        int use_fma, int32_t *S1 /*[ncalls][nchans]*/,
                        int32_t *S2 /*[ncalls*calldms][nsubs]*/);
int orc_subband_tempval(const float *dmshifts, int nchans, int nsubs, float highdm, float tsamp);
void orc_subband_stage1_f32(const float *x, int nchans, long stride, int nsubs, int nsamp1,
                            const int32_t *S1, int ncalls, float *z);
void orc_subband_stage2_f32(const float *z, int nsubs, int nsamp1, int nsamp, const int32_t *S2,
                            int ncalls, int calldms, float *y);

/* ---- reference detector (dedispersion_output.cpp:14-53,135-213, one GPU) ---- */
float orc_median_of_five(float a, float b, float c, float d, float e);
/* Global mean/rms exactly as process_brute computes them (:144-170). */
void orc_ref_stats(const float *buf, unsigned vals, float *mean, float *rms);
/* Candidates of process_brute (:172-211) with mean==NULL: writes (dm index, sample) pairs and
 * the printed snr; returns the number found (at most cap are stored). */
long orc_ref_detect(const float *buf, int tdms, int nsamp, float lowdm, float dmstep,
                    float threshold, float mean, float rms, int32_t *dm_idx, int32_t *samp,
                    float *snr, long cap);

/* process_brute (:172-211) with caller noise statistics (mean != NULL): the test uses
 * mean[l / spc] and rms[l / spc]; the printed snr is (median - mean) / rms. */
long orc_ref_detect_chunked(const float *buf, int tdms, int nsamp, float lowdm, float dmstep,
                            float threshold, const float *mean, const float *rms, int spc,
                            int32_t *dm_idx, int32_t *samp, float *snr, long cap);
/* process_subband (:56-132) over nrows rows of nvalid samples (row pitch stride) whose DMs are
 * dmv[row].  mean == NULL: per-row statistics (sequential double sums, :87-97) and
 * snr = median / localrms; else chunk statistics (mean[t / spc], rms[t / spc]) and
 * snr = median / rms. */
long orc_ref_detect_subband(const float *buf, long stride, int nrows, int nvalid,
                            const float *dmv, float threshold, const float *mean,
                            const float *rms, int spc, int32_t *dm_idx, int32_t *samp,
                            float *snr, long cap);

/* ---- RFI clipping (rfi_clipper.cu:8-67, with its two defects fixed) ---- */
/* Per-channel clip over [0, len) then per-spectrum clip over channels, in place.
 * kind: 0 = uint8, 1 = uint16, 2 = int16, 3 = float32.  k_chan/k_spec <= 0 skips that pass. */
void orc_rfi_clip(void *x, int kind, int nchans, long stride, long len, double k_chan,
                  double k_spec);

/* ---- boxcar single-pulse detector (singlepulse.cpp:41-146, restated) ---- */
/* Per-DM mean/sigma in double with a fixed chunked order (chunk = 1024 samples). */
void orc_series_stats(const double *y, long n, double *mean, double *sigma);
/* Exact statistics of an integer series (int64 / 128-bit sums). */
void orc_series_stats_int(const double *y, long n, double *mean, double *sigma);
/* Widths 1,2,4..2^(nw-1).  Per DM: mean and sigma in double (orc_series_stats_int for integer
 * series, orc_series_stats otherwise); the series in float; boxcar sums by pairwise doubling in
 * float; SNR = (B - w*mu) * inv in float with inv = (float)(1/(sigma*sqrt(w))); per-sample
 * best width (first of equals); non-maximum suppression with radius max(w/2,1).  y is
 * [ndms][n] (double; exact copies of int32 or float series).  Returns candidates found. */
long orc_boxcar_detect(const double *y, int ndms, long n, int nw, double threshold,
                       int32_t *dm_idx, int32_t *samp, int32_t *width, float *snr, long cap,
                       int is_int);

/* ---- sigproc sample unpack (file_handler.cpp:193-290) ---- */
long orc_unpack(const uint8_t *raw, long nbytes, int nbits, float *out);

/* ---- detrend + normalise (detrend.cu:12-100), double, per block of len samples ---- */
void orc_detrend_normalise(float *y, long n, int len);

/* Single-pulse search in the prototype's template form (src/prototypes/singlepulse.cpp).
 * orc_sp_widths: 1 then the downfactors <= max_downfact (:20,161-164); returns the count.
 * orc_sp_prune_related / orc_sp_prune_downfactors: :90-120 / :122-146 as written.
 * orc_sp_values: the width-w response at every sample.
 * orc_singlepulse_detect: the per-DM search of :148-300 (chunked thresholds, both prunes);
 * candidates in list order (dm, chunk, width, sample). */
int orc_sp_widths(int max_downfact, int *widths);
void orc_sp_prune_related(const int32_t *bins, const float *values, long num, int factor,
                          unsigned char *keep);
void orc_sp_prune_downfactors(const int64_t *bins, const float *values, const int32_t *df,
                              long n, int maxdf, unsigned char *mask);
void orc_sp_values(const double *y, long n, int w, int normalise, int is_int, float *out);
long orc_singlepulse_detect(const double *y, int ndms, long n, int max_downfact, long chunk_len,
                            int normalise, int is_int, double threshold, int32_t *dm_idx,
                            int32_t *samp, int32_t *width, float *snr, long cap);
/* The prototype kernels' own float arithmetic: src/prototypes/detrend.cu:12-100 (256 threads
 * per block) and src/prototypes/rfi_clipper.cu:8-67 (blockdim threads per row), each with the
 * device compiler's possible contractions as switches (see mdsm_oracle.c). */
void orc_detrend_ref_f32(float *y, int ndms, int nsamp, int len, int contract);
void orc_rfi_clip_ref_f32(float *x, int nrows, int nsamp, int blockdim, int contract,
                          float *means);
#ifdef __cplusplus
}
#endif
#endif
