/*
 * mdsm_gb300.h -- C ABI of the GB300 implementation of MDSM's incoherent dedispersion search
 * path.  Plain pointers and sizes only; every entry point returns an mdsm_status (0 = OK) and
 * mdsm_last_error() describes the last failure on the calling thread.
 *
 * Buffers:
 *   *_device entry points take device pointers (caller-owned) and a cudaStream_t as void*.
 *   *_host   entry points take host pointers (caller-owned; pinned buffers copy fastest) and do
 *            the host<->device copies inside the call, on library-owned device buffers.
 *   Filterbank input is channel-major: channel c's samples start at element c*stride, the
 *   layout of the reference's input buffer (src/mdsm/dedispersion_thread.cu:284-298).
 *   Dedispersed output is DM-major [ndms][nsamp] (src/mdsm/dedispersion_kernel.cu:46,75).
 *
 * Thread safety: different plans may be used from different threads concurrently; one plan is
 * used by one thread at a time.  The detector entry points may be called from several threads
 * (calls on one device take turns on its work area; the no-allocation detector is the
 * exception, see there).  The compatibility functions at the end keep the reference's single
 * global instance (src/mdsm/dedispersion_manager.cpp:14-34).
 */
#ifndef MDSM_GB300_H_
#define MDSM_GB300_H_

#include <stddef.h>
#include <stdint.h>

#include "survey.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    MDSM_OK = 0,
    MDSM_EINVAL = 1,   /* bad argument or configuration                                  */
    MDSM_ENOMEM = 2,   /* host or device allocation failed                               */
    MDSM_ECUDA = 3,    /* a CUDA call failed                                             */
    MDSM_ETIMEOUT = 4, /* a bounded device-side wait ran out; the kernel returned early  */
    MDSM_ESTATE = 5,   /* call out of protocol order                                     */
    MDSM_ERANGE = 6,   /* a buffer is smaller than the plan needs                        */
    MDSM_EBUDGET = 7,  /* HBM budget refused an admission                                */
    MDSM_EPARSE = 8,   /* observation file could not be parsed                           */
    MDSM_EIO = 9,      /* file could not be opened                                       */
    MDSM_EAGAIN = 10   /* nothing ready yet (serving poll)                               */
} mdsm_status;

/* input sample types */
enum { MDSM_U8 = 0, MDSM_U16 = 1, MDSM_I16 = 2, MDSM_F32 = 3, MDSM_I32 = 4 };
/* output (dedispersed series) types */
enum { MDSM_OUT_F32 = 0, MDSM_OUT_I32 = 1 };
/* accumulation: AUTO = exact INT32 for integer samples whose sums over all channels fit INT32,
 * else FP32 (integer samples: exact INT32 sums per 16 channels, Kahan-compensated FP32 across
 * them); I32 is refused (MDSM_ERANGE) where the sums may not fit.  The plan info reports the
 * accumulation in effect (I32 or F32). */
enum { MDSM_ACC_AUTO = 0, MDSM_ACC_I32 = 1, MDSM_ACC_F32 = 2 };

/* How a DM trial's integer sample shift is formed (all computed once, on the host, into a
 * table; the kernels index with integers only). */
enum {
    MDSM_SHIFT_L1 = 0,         /* trunc(dmshift_f32[c] * fma(i, dmstep/tsamp, lowdm/tsamp)):
                                  src/mdsm/dedispersion_kernel.cu:27,36 (the default kernel)   */
    MDSM_SHIFT_L1_MULADD = 1,  /* the same, start + i*step evaluated without contraction      */
    MDSM_SHIFT_OPT = 2,        /* floor(dmshift_f32[c] * (fma(i, dmstep, lowdm)/tsamp)):
                                  src/mdsm/dedispersion_kernel.cu:54,70                        */
    MDSM_SHIFT_OPT_MULADD = 3,
    MDSM_SHIFT_FP64_TRUNC = 4, /* trunc(K*(f^-2 - ftop^-2)*DM/tsamp) in double               */
    MDSM_SHIFT_FP64_ROUND = 5  /* the same, rounded to nearest                                */
};

/* One uniform run of DM trials, dm_i = lowdm + i*dmstep (one reference launch). */
typedef struct {
    float lowdm;
    float dmstep;
    int ndms;
} mdsm_segment;

/* Brute-force plan.  Replaces the brute-force set-up of initialiseMDSM
 * (src/mdsm/dedispersion_manager.cpp:286-318) and the shift upload of the worker
 * (src/mdsm/dedispersion_thread.cu:261-263). */
typedef struct {
    int nchans;
    float fch1;    /* MHz, frequency of channel 0                                   */
    float foff;    /* MHz per channel (negative: channel 0 is the top of the band)   */
    float tsamp;   /* seconds                                                       */
    int nsamp;     /* output samples per block                                      */
    const mdsm_segment *segs;
    int nsegs;
    int shift_mode;  /* MDSM_SHIFT_*                                                */
    double K;        /* dispersion constant for the FP64 modes; 0 -> 4148.741601    */
    int in_dtype;    /* MDSM_U8 / MDSM_U16 / MDSM_I16 / MDSM_F32                    */
    int out_dtype;   /* MDSM_OUT_F32 / MDSM_OUT_I32                                 */
    int acc;         /* MDSM_ACC_*                                                  */
    int dm_block;    /* DM trials per CTA tile; 0 = choose                          */
    int kernel;      /* 0 = choose (packed kernel where it applies), 1 = generic kernel */
} mdsm_brute_desc;

/* Two-stage subband plan, one or more passes.  Replaces the subband set-up of initialiseMDSM
 * and subband_dedispersion (src/mdsm/dedispersion_thread.cu:97-217).  Pass fields used:
 * lowdm, highdm, dmstep, sub_dmstep, ncalls, calldms, binsize.  A pass with binsize b > 1
 * dedisperses the block summed over b samples (mdsm_downsample_device, mode 0) at tsamp*b and
 * writes nsamp/b samples per output row; nsamp must be a multiple of every binsize. */
typedef struct {
    int nchans;
    float fch1, foff, tsamp;
    int nsamp;
    int nsubs;
    const SUBBAND_PASSES *passes;
    int npasses;
    int use_fma;   /* 1: start + i*step contracted (as the device code evaluates it)   */
    int in_dtype, out_dtype, acc;
} mdsm_subband_desc;

typedef struct mdsm_plan_s mdsm_plan;

typedef struct {
    int nchans, ndms, nsamp, maxshift;
    long long in_stride;  /* device row pitch (elements) the device entry points expect      */
    long long in_bytes;   /* device input bytes the device entry points may read            */
    long long out_bytes;  /* ndms * nsamp * output element size                              */
    int in_dtype, out_dtype, acc;
    int dm_block, time_tile;
    int kernel;           /* 1 generic, 2 packed 8-bit, 3 packed 16-bit                     */
    int nstages;          /* 1 brute force; subband: 2 per pass (mdsm_plan_stage_info)       */
    long long work_bytes; /* plan-owned device scratch (subband intermediate)               */
} mdsm_plan_info;

/* src/mdsm/dedispersion_manager.cpp:262-265 */
float mdsm_dmdelay(float f1, float f2);
const char *mdsm_last_error(void);
const char *mdsm_version(void);

mdsm_status mdsm_brute_plan_create(const mdsm_brute_desc *desc, mdsm_plan **out);
mdsm_status mdsm_subband_plan_create(const mdsm_subband_desc *desc, mdsm_plan **out);
void mdsm_plan_destroy(mdsm_plan *plan);
mdsm_status mdsm_plan_get_info(const mdsm_plan *plan, mdsm_plan_info *info);

/* One launch stage of a plan (brute force: stage 0; subband pass i: stages 2i and 2i+1): the
 * kernel it runs (1 generic, 2 packed 8-bit, 3 packed 16-bit), its DM block and time tile,
 * and whether it writes uint16 subband series. */
typedef struct {
    int kernel, dm_block, time_tile, out_u16;
    int nchans, ndms, ngroups, nsamp;
    long long smem_bytes;
} mdsm_stage_info;
mdsm_status mdsm_plan_stage_info(const mdsm_plan *plan, int stage, mdsm_stage_info *info);
/* Integer shifts, row-major [ndms][nchans] (brute) or stage tables (subband: stage 1
 * [ncalls][nchans] of the first pass when which = 1, stage 2 [ndms][nsubs] when which = 2). */
mdsm_status mdsm_plan_shift_table(const mdsm_plan *plan, int which, int32_t *out);
/* DM value of every output row (float). */
mdsm_status mdsm_plan_dm_values(const mdsm_plan *plan, float *out);
/* Per-channel delays, float[nchans] (src/mdsm/dedispersion_manager.cpp:286-289). */
mdsm_status mdsm_plan_dmshifts(const mdsm_plan *plan, float *out);

/* Host-only table builders (no device needed).  Same arithmetic as the plans use.
 * mdsm_dmshifts: src/mdsm/dedispersion_manager.cpp:286-289.
 * mdsm_brute_shift_table: S [ndms][nchans], dm values [ndms], *maxshift = max(S); replaces the
 *   shift formed inside src/mdsm/dedispersion_kernel.cu:27,36 / :54,70.
 * mdsm_subband_shift_tables: pass `pass`'s S1 [ncalls][nchans] and S2 [ncalls*calldms][nsubs]
 *   (src/mdsm/dedispersion_kernel.cu:148,163,167 and :54,70 as launched by
 *   src/mdsm/dedispersion_thread.cu:146-210). */
mdsm_status mdsm_dmshifts(int nchans, float fch1, float foff, float *out);
mdsm_status mdsm_brute_shift_table(const mdsm_brute_desc *desc, int32_t *S, float *dm_values,
                                   int *maxshift);
mdsm_status mdsm_subband_shift_tables(const mdsm_subband_desc *desc, int pass, int32_t *S1,
                                      int32_t *S2);

/* Dedisperse one block on the device.  d_in: channel-major with row pitch in_stride elements
 * (>= nsamp + maxshift, a multiple of 16 bytes) and in_bytes readable bytes (>= info.in_bytes).
 * d_out: [ndms] rows of out_stride elements.  Replaces call_dedisperse's kernel dispatch
 * (src/mdsm/dedispersion_wrapper.cu:7-9 -> dedispersion_thread.cu:332-341).  Asynchronous on
 * stream: a device-side wait that ran out (the kernels' waits are bounded; the block's results
 * are then invalid) is reported by the next mdsm_plan_check. */
mdsm_status mdsm_dedisperse_device(mdsm_plan *plan, const void *d_in, long long in_stride,
                                   size_t in_bytes, void *d_out, long long out_stride,
                                   void *stream);
/* The same through host buffers: h_in channel-major with pitch h_in_stride elements (the
 * reference's nsamp + maxshift), h_out [ndms][nsamp].  Copies H2D, runs, copies D2H and
 * synchronises the stream (src/mdsm/dedispersion_thread.cu:284-298,352-355).  Brute-force
 * blocks of at least 32768 samples run in up to 16 time segments whose copy-in, kernel and
 * copy-out overlap (two library-owned copy streams ordered by events); pinned host buffers
 * let the copies run at full speed.  Results do not depend on the segmentation. */
mdsm_status mdsm_dedisperse_host(mdsm_plan *plan, const void *h_in, long long h_in_stride,
                                 void *h_out, void *stream);
/* Synchronises stream and reports device-side failures of the plan's calls since the last
 * check: MDSM_ETIMEOUT when a bounded device-side wait ran out (the kernel returned early and
 * the results of those calls are invalid), else MDSM_OK.  Clears the record; the plan stays
 * usable.  (The host-buffer entry point checks by itself.) */
mdsm_status mdsm_plan_check(mdsm_plan *plan, void *stream);
/* Test hook for the failure path (no counterpart in the reference): on stream, a one-block
 * kernel whose single bounded wait -- the mbarrier wait the dedispersion kernels use, with
 * spin_limit (1..65536) try_waits instead of their 2^22 -- waits on a barrier that nothing
 * arrives at.  The wait runs out, the kernel records the timeout in the plan's device error
 * word and returns, so the next mdsm_plan_check returns MDSM_ETIMEOUT; no fault, trap or hang
 * is involved and the plan works as before afterwards. */
mdsm_status mdsm_plan_wait_selftest(mdsm_plan *plan, unsigned spin_limit, void *stream);
/* Number of kernels the last dedisperse call on this plan launched. */
int mdsm_plan_last_launches(const mdsm_plan *plan);
/* Profiling (no counterpart in the reference): with stage timing on, every
 * mdsm_dedisperse_device call records CUDA events on its stream before the first stage and
 * after each stage (mdsm_plan_stage_info numbers them; a pass's downsampling counts with its
 * first stage).  mdsm_plan_stage_times waits for the last call's final event and writes up to
 * cap stage durations in milliseconds, *n = the number of stages timed. */
mdsm_status mdsm_plan_set_stage_timing(mdsm_plan *plan, int on);
mdsm_status mdsm_plan_stage_times(mdsm_plan *plan, float *ms, int cap, int *n);

/* ---------------------------------------------------------------------------------------- */
/* RFI clipping (src/prototypes/rfi_clipper.cu:8-67): per-channel then per-spectrum.          */
/* In place on a channel-major device buffer of len samples per row.  k <= 0 skips a pass.   */
/* Integer samples are replaced by the mean rounded to nearest even.                          */
mdsm_status mdsm_rfi_clip_device(void *d_x, int dtype, int nchans, long long stride,
                                 long long len, double k_chan, double k_spec, void *stream);

/* ---------------------------------------------------------------------------------------- */
/* Reference detector (src/mdsm/dedispersion_output.cpp:135-213, mean == NULL, one device):  */
/* global mean/rms over the block, median-of-five, median - mean >= threshold*rms and DM>1.   */
typedef struct {
    int32_t dm_idx;
    int32_t sample;
    float snr;
    int32_t width;   /* boxcar width (1 for the median-of-five detector) */
} mdsm_candidate;

/* d_series: float [ndms][nsamp] on the device.  lowdm/dmstep describe a single uniform plan
 * as the reference assumes.  Candidates are written to h_cands (up to cap, sorted by dm then
 * sample); *ncand receives the total found.  mean/rms receive the statistics. */
mdsm_status mdsm_ref_detect_device(const float *d_series, int ndms, int nsamp, float lowdm,
                                   float dmstep, float threshold, mdsm_candidate *h_cands,
                                   long long cap, long long *ncand, float *mean, float *rms,
                                   void *stream);

/* The reference detector above, for callers that cannot allocate device memory: a real-time
 * stage that must not stall on the device allocator between blocks, a host that hands out all
 * device memory once at start-up, or a plugin where allocation is not permitted.  This entry
 * point has no counterpart in the reference.  It calls no cudaMalloc/cudaFree and no allocating
 * library routine: its work arrays live in one fixed device array of about 2 MiB that every GPU
 * loading the library holds until exit.  Limits: ndms*nsamp < 2^31 values (MDSM_EINVAL
 * beyond, as mdsm_ref_detect_device) and cap <= 65536 candidates (MDSM_ERANGE beyond).  Each
 * call looks up the array's address in the current context (cudaGetSymbolAddress), so a
 * context torn down and created again (cudaDeviceReset) is handled; like the allocating
 * detector it synchronises the stream, so it cannot be captured in a CUDA graph.  All calls
 * share the array and leave its contents behind (the candidate counter is cleared at each
 * call), so calls that overlap on the GPU race.  Results equal mdsm_ref_detect_device's. */
mdsm_status mdsm_ref_detect_device_noalloc(const float *d_series, int ndms, int nsamp,
                                           float lowdm, float dmstep, float threshold,
                                           mdsm_candidate *h_cands, long long cap,
                                           long long *ncand, float *mean, float *rms,
                                           void *stream);

/* process_brute with caller noise statistics (dedispersion_output.cpp:135-213, mean != NULL):
 * h_mean/h_rms hold one value per spc samples (nchunks >= (nsamp - 5) / spc + 1 values); the
 * test is median - h_mean[t / spc] >= h_rms[t / spc] * threshold with DM > 1 and the
 * candidate's snr is (median - mean) / rms (the reference's file line adds that chunk's mean
 * and rms).  Candidates sorted by (dm_idx, sample), width 1. */
mdsm_status mdsm_ref_detect_chunked_device(const float *d_series, int ndms, int nsamp,
                                           float lowdm, float dmstep, float threshold,
                                           const float *h_mean, const float *h_rms,
                                           long long nchunks, int spc, mdsm_candidate *h_cands,
                                           long long cap, long long *ncand, void *stream);
/* process_subband (dedispersion_output.cpp:56-132) on a subband plan's float output (rows of
 * out_stride elements; a pass with downsample b holds nsamp / b samples per row): with
 * h_mean == NULL, per-row mean and rms from sequential double sums (:87-97), else the caller's
 * chunk statistics as above; the test median - mean >= rms * threshold with the row's DM > 1,
 * snr = median / rms.  Candidates carry the global row, the sample within the pass and, in
 * width, the pass's downsample factor (the sample's time is t0 + sample * tsamp * width).
 * Deviations, each a defect of the reference: every pass reads its own rows (the reference
 * reads the first pass's rows for every pass), the row's DM is the plan's (the reference
 * prints lowdm + k * dmstep, without the second stage's centring), and the per-row branch
 * runs (the reference dereferences mean[0] first). */
mdsm_status mdsm_ref_detect_subband_device(const mdsm_plan *plan, const float *d_series,
                                           long long out_stride, float threshold,
                                           const float *h_mean, const float *h_rms,
                                           long long nchunks, int spc, mdsm_candidate *h_cands,
                                           long long cap, long long *ncand, void *stream);

/* Boxcar single-pulse search (src/prototypes/singlepulse.cpp:41-146, restated): widths
 * 1,2,4..2^(nwidths-1); per-DM mean/sigma in FP64; boxcar sums and SNR = (sum - w*mean) /
 * (sigma*sqrt(w)) in FP32, explicitly rounded in a fixed order; per-sample
 * best width; non-maximum suppression with radius max(w/2,1).  d_series is [ndms][nsamp] of
 * dtype MDSM_OUT_F32 or MDSM_OUT_I32.  Candidates sorted by dm then sample.  MDSM_ETIMEOUT if
 * a bounded wait for the search's staging copies ran out (no candidates are then returned; the
 * same status reaches a serving block's result and mdsm_batch_candidates). */
mdsm_status mdsm_boxcar_detect_device(const void *d_series, int series_dtype, int ndms,
                                      int nsamp, int nwidths, double threshold,
                                      mdsm_candidate *h_cands, long long cap, long long *ncand,
                                      void *stream);

/* Single-pulse search in the form of the reference's prototype (src/prototypes/singlepulse.cpp:
 * 20-23,41-146,148-300), on the device.  Widths: 1, then the prototype's downfactor ladder
 * {2,3,4,6,9,14,20,30,45,70,100,150} up to max_downfact (>= 2; the prototype uses 30).  The
 * response of width w at sample t is the template sum over [t - w/2, t - w/2 + w) (the
 * prototype's centred templates; zero outside the series) in FP32, left to right, then
 * (sum - w*mean) / (sigma*sqrt(w)): with normalise = 0 mean 0 and sigma 1 (the prototype's
 * input is already normalised, e.g. by mdsm_detrend_normalise_device), with normalise = 1 the
 * row's own statistics as the boxcar search forms them.  Per DM, in chunks of chunk_len
 * samples (the prototype: 8000): each width's samples with response >= threshold, pruned by
 * the prototype's pruneRelated (:90-120) for widths > 1; then the DM's survivors in (chunk,
 * width, sample) order pruned by its pruneRelatedDownfactors (:122-146); the rest are the
 * candidates, written in that order (width = the template width, snr = the response).  The two
 * prune functions behave as the prototype writes them; its main loop's defects are not
 * reproduced.  MDSM_ERANGE if more than max(4*cap, 2^18) crossings survive the first prune. */
mdsm_status mdsm_singlepulse_detect_device(const void *d_series, int series_dtype, int ndms,
                                           int nsamp, int max_downfact, int chunk_len,
                                           int normalise, double threshold,
                                           mdsm_candidate *h_cands, long long cap,
                                           long long *ncand, void *stream);

/* Time downsampling of a channel-major block: out[c][t] = f(sum_{k<b} in[c][t*b+k]) for
 * t < len/b, f = sum (mode 0; integer samples widen: uint8 -> uint16 or int32, 16-bit -> int32),
 * mean (mode 1) or sum/sqrt(b) (mode 2) in float32.  The reference's binning kernels
 * (src/mdsm/dedispersion_kernel.cu:203-264, src/prototypes/binner.cu:13-71) compute the
 * mean and sum/sqrt(b) but index channel-major blocks as interleaved. */
mdsm_status mdsm_downsample_device(const void *d_in, int in_dtype, int nchans,
                                   long long in_stride, long long len, int binsize, int mode,
                                   void *d_out, int out_dtype, long long out_stride, void *stream);

/* ---------------------------------------------------------------------------------------- */
/* Sigproc filterbank ingest.                                                                */
typedef struct {
    int nchans, nbits, nifs, machine_id, telescope_id, data_type, nbeams, ibeam;
    int barycentric, pulsarcentric, nbins, nsamples, nfchannels;
    double tstart, tsamp, fch1, foff, refdm, az_start, za_start, src_raj, src_dej, period;
    long long npuls;
    long long header_bytes;  /* bytes before the first sample                              */
    char source_name[81], rawdatafile[81];
} mdsm_sigproc_header;

/* src/mdsm/file_handler.cpp:33-187 (same keywords and types; an unknown keyword returns
 * MDSM_EPARSE instead of exiting). */
mdsm_status mdsm_sigproc_read_header(const char *path, mdsm_sigproc_header *h);
/* Header of a dedispersed-series file, one channel of 32-bit samples
 * (src/pelican-mdsm/modules/DedispersedDataWriter.cpp:49-63); samples are appended after. */
mdsm_status mdsm_sigproc_write_series_header(const char *path, double fch1, double foff,
                                             double tsamp, double tstart);
/* Unpack nspectra time-major spectra of nchans nbits-bit samples (1/2/4 least significant
 * field first, 16-bit unsigned, 32-bit float: file_handler.cpp:193-290) on the device and
 * write them channel-major into d_out (uint8, uint16, float32, or int16, which reads 16-bit
 * samples as two's-complement signed) at columns
 * [col0, col0 + nspectra) of rows of out_stride elements; invert reverses the channel order
 * (the corner turns of src/MDSM.cpp:100-125 and MdsmModule.cpp:135-151). */
mdsm_status mdsm_unpack_device(const void *d_raw, long long nspectra, int nchans, int nbits,
                               int invert, void *d_out, int out_dtype, long long out_stride,
                               long long col0, void *stream);

/* ---------------------------------------------------------------------------------------- */
/* Batched form: several brute-force plans (beams of uneven block length, channel count and  */
/* DM plan) in one pass, optionally with RFI clipping before dedispersion and a boxcar search */
/* after; the pass can be captured once in a CUDA graph and replayed.  Replaces the one-beam, */
/* one-launch-per-segment loop of src/mdsm/dedispersion_thread.cu:64-94,220-243.  The plans  */
/* must outlive the batch.                                                                    */
/*  * Fused form (every plan uint8 samples with int32 output; the search, if on, over widths */
/*    1..256): clip, dedispersion and search in ONE persistent launch over four work lists   */
/*    (channel clips, spectrum clips, DM-block x time-tile tiles, search runs) tied by per-   */
/*    beam completion counts with bounded device waits; the rows' statistics are folded into */
/*    the dedispersion store.  The fused launch stages every beam with one tile shape, whose */
/*    shared memory the beam with the widest DM span sizes.                                   */
/*  * Unfused: clip launches, one persistent dedispersion launch over the packed beams' tiles */
/*    (a launch per beam for the rest) or one launch per beam with each plan's own tile      */
/*    shape, then per-beam search launches.                                                   */
/* mdsm_batch_autotune times, with the search on as configured, the fused tile shapes (DM    */
/* trials per block x samples per tile x compute warps) and item orders where the beams fit  */
/* them, and the unfused passes, on the registered buffers, and keeps the fastest.            */
/* With MDSM_AUTOTUNE_CACHE set to a file path the choice is cached per beam geometry.        */
typedef struct mdsm_batch_s mdsm_batch;
mdsm_status mdsm_batch_create(mdsm_plan *const *plans, int nbeams, mdsm_batch **out);
mdsm_status mdsm_batch_set_buffers(mdsm_batch *b, const void *const *d_in,
                                   const long long *in_stride, void *const *d_out,
                                   const long long *out_stride);
/* In-place clip of every beam's input before dedispersion (as mdsm_rfi_clip_device). */
mdsm_status mdsm_batch_enable_clip(mdsm_batch *b, double k_chan, double k_spec);
mdsm_status mdsm_batch_enable_detect(mdsm_batch *b, int nwidths, double threshold,
                                     long long cap);
mdsm_status mdsm_batch_autotune(mdsm_batch *b, void *stream, int *choice);
/* use_graph: the first call runs the pass and captures it; later calls replay the graph. */
mdsm_status mdsm_batch_run(mdsm_batch *b, int use_graph, void *stream);
int mdsm_batch_last_launches(const mdsm_batch *b);
/* The candidates the last mdsm_batch_autotune timed (none when it took a cached choice):
 * *n of them, the first cap written as (choice, milliseconds per pass). */
mdsm_status mdsm_batch_autotune_times(const mdsm_batch *b, int *choices, float *ms, int cap,
                                      int *n);
/* What an autotuner choice means: fused = 1 for the fused launch with its DM trials per block,
 * samples per tile, compute warps and item order (0: a beam's DM blocks of one tile adjacent,
 * 1: a DM block's tiles adjacent); fused = 0 for the unfused shapes, order = 0 persistent
 * tile-major, 1 persistent DM-block-major, 2 one launch per beam. */
mdsm_status mdsm_batch_choice_info(int choice, int *fused, int *dm_block, int *time_tile,
                                   int *warps, int *order);
mdsm_status mdsm_batch_candidates(mdsm_batch *b, int beam, mdsm_candidate *out, long long cap,
                                  long long *ncand, void *stream);
void mdsm_batch_destroy(mdsm_batch *b);

/* ---------------------------------------------------------------------------------------- */
/* Serving form: a continuous-batching search server over many beams on one GPU.  Each beam   */
/* keeps its overlap tail resident in HBM; blocks from any beam are admitted into a bounded   */
/* set of in-flight slots (CUDA streams) as they arrive, subject to an HBM budget and a host */
/* staging budget, and overlap on the device; each block is dedispersed and boxcar-searched */
/* and only its candidates are copied back.  Replaces the one-stream block loop of           */
/* src/mdsm/dedispersion_thread.cu:246-401 and the host detector thread of                   */
/* src/mdsm/dedispersion_output.cpp:216-356.  Add every beam before the first submit.        */
typedef struct {
    long long hbm_budget_bytes;  /* device bytes beams and slots may hold                    */
    long long host_stage_bytes;  /* pinned bytes of blocks waiting for a slot                */
    int max_inflight;            /* slots (blocks on the device at once)                     */
    int detector;                /* 1 boxcar search, 0 none                                  */
    int nwidths;                 /* boxcar widths 1..2^(nwidths-1)                           */
    double threshold;            /* boxcar SNR threshold                                     */
    long long cand_cap;          /* candidates kept per block                                */
} mdsm_server_desc;

typedef struct {
    int beam;
    long long block;             /* block index within its beam                              */
    long long ticket;            /* submission order over all beams                          */
    double submit_time, done_time;  /* seconds, steady clock                                 */
    long long ncand;             /* candidates found (may exceed cand_cap)                   */
    int status;
} mdsm_block_result;

typedef struct {
    long long admitted, refused, completed, held_bytes, dm_trial_samples;
    double wall_s, p50_latency_s, p99_latency_s, max_latency_s;
} mdsm_server_stats;

typedef struct mdsm_server_s mdsm_server;

mdsm_status mdsm_server_create(const mdsm_server_desc *desc, mdsm_server **out);
mdsm_status mdsm_server_add_beam_brute(mdsm_server *sv, const mdsm_brute_desc *desc, int *beam);
mdsm_status mdsm_server_add_beam_subband(mdsm_server *sv, const mdsm_subband_desc *desc,
                                         int *beam);
mdsm_status mdsm_server_beam_info(mdsm_server *sv, int beam, mdsm_plan_info *info);
/* Block 0 of a beam holds nsamp + maxshift samples per channel, later blocks nsamp new samples
 * (row pitch h_stride elements).  The data are copied into a pinned staging buffer before
 * return.  MDSM_EBUDGET: not admitted now (staging budget full); retry after results are
 * polled. */
mdsm_status mdsm_server_submit(mdsm_server *sv, int beam, const void *h_block,
                               long long h_stride, long long *ticket);
/* Zero-copy form of submit, as the reference hands its caller the input buffer to fill
 * (initialiseMDSM / next_chunk): acquire returns a pinned staging buffer for the beam's next
 * block, [nchans][*cols] samples of the beam's type (*cols = nsamp + maxshift for block 0, else
 * nsamp); the producer writes the block there and commit queues it.  One acquired block per
 * beam at a time; one producer thread per beam.  MDSM_EBUDGET as for submit. */
mdsm_status mdsm_server_acquire(mdsm_server *sv, int beam, void **h_block, long long *cols);
mdsm_status mdsm_server_commit(mdsm_server *sv, int beam, long long *ticket);
/* One finished block (completion order), its candidates sorted by dm then sample.
 * MDSM_EAGAIN when none is ready within wait_ms. */
mdsm_status mdsm_server_poll(mdsm_server *sv, mdsm_block_result *res, mdsm_candidate *cands,
                             long long cap, int wait_ms);
mdsm_status mdsm_server_drain(mdsm_server *sv);
mdsm_status mdsm_server_get_stats(mdsm_server *sv, mdsm_server_stats *out);
void mdsm_server_destroy(mdsm_server *sv);

/* Detrend and normalise float series in place (src/prototypes/detrend.cu:12-100): per block
 * of len samples of each of ndms rows of nsamp samples, subtract the least-squares line on
 * x = -len/2 + 0.5 + i and divide by the residual rms (sums in double).  A trailing partial
 * block is left as it is. */
mdsm_status mdsm_detrend_normalise_device(float *d_series, int ndms, long long nsamp, int len,
                                          void *stream);

/* ---------------------------------------------------------------------------------------- */
/* Compatibility layer: the reference stage interface (src/mdsm/dedispersion_manager.h:7-12) */
/* with C linkage.  include/dedispersion_manager.h wraps these under the reference's C++      */
/* names and default arguments.  Same buffer ownership, one-block latency and stop protocol.  */
SURVEY *mdsm_processSurveyParameters(const char *xml_path);
/* Returns the library-owned host input buffer, float [nchans][nsamp + maxshift]
 * (dedispersion_manager.cpp's layout, as MDSM.cpp:113 and MdsmModule.cpp:143-149 fill it). */
float *mdsm_initialiseMDSM(SURVEY *survey);
float *mdsm_next_chunk(unsigned int data_read, unsigned *samples, double timestamp,
                       double blockRate, float *mean, float *rms);
int mdsm_start_processing(unsigned int data_read);
void mdsm_tearDownMDSM(void);
/* Candidates of the last block handed to start_processing (waits for its processing). */
long long mdsm_compat_candidates(mdsm_candidate *out, long long cap);
/* Blocks since initialiseMDSM whose float input was all integers 0..255 and so ran on the
 * 8-bit kernels (same output bit for bit: every partial sum is an integer below 2^24). */
long long mdsm_compat_blocks_8bit(void);
void mdsm_free_survey(SURVEY *survey);

#ifdef __cplusplus
}
#endif
#endif
