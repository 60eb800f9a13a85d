// internal.h -- shared declarations of the mdsm_gb300 library (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <mutex>
#include <string>
#include <vector>

#include "mdsm_gb300.h"

namespace mdsm {

// ----------------------------------------------------------------------------------------
// errors
// ----------------------------------------------------------------------------------------
void set_error(const std::string &msg);
mdsm_status fail(mdsm_status st, const std::string &msg);
mdsm_status cuda_fail(cudaError_t e, const char *what);

#define MDSM_CUDA_TRY(x)                                                  \
    do {                                                                  \
        cudaError_t e_ = (x);                                             \
        if (e_ != cudaSuccess) return ::mdsm::cuda_fail(e_, #x);          \
    } while (0)

#define MDSM_TRY(x)                                                       \
    do {                                                                  \
        mdsm_status s_ = (x);                                             \
        if (s_ != MDSM_OK) return s_;                                     \
    } while (0)

// device-side error word bits
enum : unsigned {
    ERR_WAIT_TIMEOUT = 1u,   // a bounded mbarrier wait ran out
    ERR_CAND_OVERFLOW = 2u,  // candidate buffer full (count still exact)
};

size_t dtype_size(int dtype);

// Set in the candidate count of the boxcar search (k_boxcar) when one of its bounded staging
// waits ran out: the count and records of that search are not valid.
constexpr unsigned long long kBoxCountLate = 1ull << 62;

// candidate record as the device kernels write it
struct DevCand {
    int32_t dm_idx, sample, width;
    float snr;
};

// arguments of one beam / stage of the shift-and-sum kernels (dedisp.cu)
struct KArgs {
    const unsigned char *in;
    long long in_stride, in_group_stride;    // elements
    unsigned char *out;
    long long out_stride, out_group_stride;  // elements
    const int32_t *rel;                      // [g][blk][c][DB]
    const int32_t *sminspan;                 // [g][blk][c][2]
    int nchans, ndms, nsamp, nblk, rowcap, nst, out_i32;
    int ps;  // packed kernels: bytes per phase copy of a staged row
    unsigned *err;
    // optional (packed kernels, int32 output): exact moments of every output row, accumulated
    // as the row is stored -- (sum, sum of squares low 64 bits, high 64 bits) per row at
    // mom + 3 * (group * mom_group_rows + row)
    unsigned long long *mom;
    long long mom_group_rows;
};

// ----------------------------------------------------------------------------------------
// one launch of the generic shift-and-sum kernel: out[g][d][t] = sum_c in[g][c][t + S[g][d][c]]
// ----------------------------------------------------------------------------------------
struct StageGeom {
    int nchans = 0;   // channels summed per group
    int ndms = 0;     // output rows per group
    int ngroups = 1;
    int nsamp = 0;    // output samples per row
    long long in_stride = 0, in_group_stride = 0;    // elements
    long long out_stride = 0, out_group_stride = 0;  // elements
    int in_dtype = MDSM_U8;
    int acc_int = 1;      // 1: int32 accumulation, 0: float
    int out_i32 = 0;      // output element type: int32 (1) or float32 (0)
    int out_u16 = 0;      // uint16 output (the uint8 packed kernel, sums that fit 16 bits)
    int Db = 32, T = 256, R = 8, DPW = 4;
    int cc = 16, nst = 3; // channels per pipeline stage, stages
    int rowcap = 0;       // elements per staged row
    int nblk = 0;         // DM blocks per group
    int max_span = 0;     // max over blocks/channels of smax - smin
    int max_shift = 0;    // max shift in the table
    // host tables
    std::vector<int32_t> rel;     // [ngroups][nblk][nchans][Db]  shift - smin
    std::vector<int32_t> sminspan;// [ngroups][nblk][nchans][2]   (smin, span)
    // device copies
    int32_t *d_rel = nullptr;
    int32_t *d_sminspan = nullptr;
    size_t smem_bytes = 0;
    int ps = 0;           // packed kernels: bytes per phase copy of a staged row
    int kernel = 0;       // requested (0 choose, 1 generic); after tiling: 1 generic, 2 packed
                          // uint8, 3 packed uint16
};

// Build the blocked tables of a stage from a full shift table S[g][d][c] (row-major).  Picks
// the tile shape: Db starts at 8*DPW (DPW as set on entry) and shrinks until the staged rows
// fit in shared memory.
mdsm_status build_stage_tables(StageGeom &g, const std::vector<int32_t> &S);
mdsm_status upload_stage(StageGeom &g);
void free_stage(StageGeom &g);
// Bytes of input (from the group base) the kernel may read for in_stride, with tile overrun.
long long stage_in_bytes(const StageGeom &g, long long in_stride, long long in_group_stride);
// Launch the stage kernel.  Returns number of kernels launched via *launches.
// nsamp_run >= 0 computes only output samples [0, nsamp_run) (a time segment of the block,
// with in/out already offset to its first sample); -1 computes all g.nsamp.
// mom (optional): exact row moments of int32 output accumulated by the packed kernels as they
// store (see KArgs); ignored by the generic kernel (stage_folds_moments tells which).
mdsm_status launch_stage(const StageGeom &g, const void *in, long long in_stride,
                         long long in_group_stride, void *out, long long out_stride,
                         long long out_group_stride, unsigned *d_err, cudaStream_t st,
                         int *launches, long long nsamp_run = -1,
                         unsigned long long *mom = nullptr, long long mom_group_rows = 0);
inline bool stage_folds_moments(const StageGeom &g)
{
    return (g.kernel == 2 || g.kernel == 3) && g.out_i32 && !g.out_u16;
}

// ----------------------------------------------------------------------------------------
// batched persistent launch (dedisp.cu)
// ----------------------------------------------------------------------------------------
struct BatchBeam {
    const StageGeom *g = nullptr;
    const void *in = nullptr;
    long long in_stride = 0;
    void *out = nullptr;
    long long out_stride = 0;
};

struct BatchState {
    std::vector<BatchBeam> beams;
    void *d_items = nullptr;    // int4 (beam, DM block, tile, group)
    void *d_kargs = nullptr;    // per-beam kernel arguments
    unsigned *d_counter = nullptr;
    unsigned *d_err = nullptr;
    int nitems = 0, rawcap = 0, ps = 0, tile_major = 1;
    size_t smem = 0;
};

// ----------------------------------------------------------------------------------------
// fused batched launch (dedisp.cu): clip, dedisperse and boxcar-search uint8 beams in one
// persistent launch; see k_batch_fused
// ----------------------------------------------------------------------------------------
struct FusedBeam {
    unsigned char *in;          // uint8 block [nchans][in_stride]
    long long in_stride;        // elements
    long long ncols;            // nsamp + maxshift: the columns the clip covers
    int nchans, ndms, nsamp;
    unsigned nspec_items;       // phase-2 items of this beam
    unsigned ndd_done;          // phase-3 completions of this beam (items x compute warps)
    const int32_t *out;         // int32 series [ndms][out_stride]
    long long out_stride;
    unsigned long long *mom;    // [ndms][3] exact row moments
    DevCand *cands;             // [cap]
    unsigned long long *count;
};

struct FusedArgs {
    const FusedBeam *fb;
    const int2 *cc_items;       // (beam, channel)
    const int2 *cs_items;       // (beam, first column)
    const int4 *bx_items;       // (beam, row, first tile, last tile + 1)
    int n_cc, n_cs, n_bx;
    unsigned *counters;         // [4], zero at the start of the launch
    unsigned *done;             // [nbeams][3], zero at the start of the launch
    double k_chan, k_spec, threshold;
    long long cap;
    unsigned *err;
};

struct FusedShapeInfo {
    int dm_block, time_tile, compute_warps;
};
int fused_num_shapes();
int fused_box_tile();  // output samples per tile of the fused launch's search items
FusedShapeInfo fused_shape_info(int shape);
mdsm_status fused_tables(int shape, StageGeom &g, const std::vector<int32_t> &S);
KArgs fused_kargs(const StageGeom &g, const void *d_rel_common, const unsigned char *in,
                  long long in_stride, int32_t *out, long long out_stride, int rawcap, int ps,
                  unsigned long long *mom, unsigned *err);
mdsm_status fused_launch(int shape, const FusedArgs &f, const KArgs *d_kargs,
                         const int4 *d_items, int n_dd, int rawcap, int ps, cudaStream_t st);
constexpr int kFusedSpecColsHost = 512;  // columns of one spectrum-clip item

mdsm_status batch_prepare(BatchState &b, const std::vector<BatchBeam> &beams);
mdsm_status batch_set_buffers(BatchState &b, const std::vector<const void *> &in,
                              const std::vector<long long> &in_stride,
                              const std::vector<void *> &out,
                              const std::vector<long long> &out_stride, unsigned *d_err,
                              int tile_major);
mdsm_status batch_launch(BatchState &b, int mode, cudaStream_t st, int *launches);
void batch_release(BatchState &b);

// ----------------------------------------------------------------------------------------
// plans
// ----------------------------------------------------------------------------------------
struct Plan {
    int kind = 0;   // 1 brute, 2 subband
    int nchans = 0, ndms = 0, nsamp = 0, maxshift = 0;
    float fch1 = 0, foff = 0, tsamp = 0;
    int in_dtype = MDSM_U8, out_dtype = MDSM_OUT_F32, acc = MDSM_ACC_AUTO;
    std::vector<float> dmshifts;     // float[nchans]
    std::vector<float> dm_values;    // float[ndms]
    std::vector<int32_t> S;          // brute: [ndms][nchans]
    std::vector<int32_t> S1, S2;     // subband first pass stage tables (reporting)
    std::vector<StageGeom> stages;   // brute: 1; subband: 2 per pass
    // subband intermediate
    long long n1 = 0;                // stage-1 output samples per row
    void *d_work = nullptr;
    size_t work_bytes = 0;
    std::vector<long long> pass_row0;   // first output row of each pass
    std::vector<int> pass_bin;          // downsample factor of each pass
    std::vector<int> pass_ds_dtype;     // sample type of its downsampled block
    std::vector<long long> pass_ds_pitch;
    void *d_ds = nullptr;               // downsampled block (passes with downsample > 1)
    size_t ds_bytes = 0;
    // host-path buffers
    void *d_in = nullptr, *d_out = nullptr;
    size_t d_in_bytes = 0, d_out_bytes = 0;
    // host path, brute force: copy-in and copy-out streams and per-segment events
    cudaStream_t s_in = nullptr, s_out = nullptr;
    std::vector<cudaEvent_t> seg_ev;
    unsigned *d_err = nullptr;
    int last_launches = 0;
    long long in_stride = 0;         // device pitch for the host path
    // optional per-stage timing of device-path calls: events before the first stage and after
    // each stage (a subband pass's downsampling belongs to its first stage)
    bool stage_timing = false;
    std::vector<cudaEvent_t> stage_ev;
    int stage_ev_used = 0;
};

mdsm_status plan_in_requirements(const Plan &p, long long in_stride, long long *in_bytes);
// mom (optional): [ndms][3] exact moments of every int32 output row (sum, sum of squares as
// two 64-bit words), zeroed and accumulated on st when every final stage folds them
// (*folded = true); otherwise left alone (*folded = false).
mdsm_status plan_run_device(Plan &p, const void *d_in, long long in_stride, size_t in_bytes,
                            void *d_out, long long out_stride, cudaStream_t st,
                            unsigned long long *mom = nullptr, bool *folded = nullptr);
mdsm_status check_err_word(unsigned *d_err, cudaStream_t st);
// one-block kernel whose bounded wait runs out after `limit` try_waits (dedisp.cu)
mdsm_status wait_selftest(unsigned *d_err, unsigned limit, cudaStream_t st);

// Float rows [nrows][in_stride] -> uint8 rows [nrows][out_stride] over columns [0, ncols):
// every value that is bit for bit an integer 0..255 is stored as that integer; any other
// value (fractions, negatives, -0, NaN, > 255) sets *flag.  Asynchronous on st.
mdsm_status pack_u8_rows(const float *in, long long in_stride, int nrows, long long ncols,
                         uint8_t *out, long long out_stride, unsigned *flag, cudaStream_t st);

// host shift formulas (the reference's arithmetic, evaluated on the host)
float dmdelay_ref(float f1, float f2);
void dmshifts_ref(int nchans, float fch1, float foff, float *out);
int32_t shift_of(float dms, double delay64, float lowdm, float dmstep, int idx, float tsamp,
                 int mode);

// ----------------------------------------------------------------------------------------
// detection / rfi launchers (detect.cu, rfi.cu, singlepulse.cu)
// ----------------------------------------------------------------------------------------
// The detectors' grow-only per-device work buffer; the lease holds it until the call returns.
mdsm_status scratch_get(size_t bytes, void **out, std::unique_lock<std::mutex> *lease);
// Per-DM (mean, sigma) in double of float32 / int32 series (the boxcar searches' statistics).
size_t series_stats_part_bytes(int ndms, long long n);
mdsm_status series_stats_launch(const void *y, int dtype, int ndms, long long n, double2 *part,
                                double2 *musig, cudaStream_t st);
mdsm_status singlepulse_detect(const void *d_series, int dtype, int ndms, int nsamp,
                               int max_downfact, int chunk_len, int normalise, double threshold,
                               mdsm_candidate *h_cands, long long cap, long long *ncand,
                               cudaStream_t st);
// ----------------------------------------------------------------------------------------
mdsm_status ref_detect(const float *d_series, int ndms, int nsamp, float lowdm, float dmstep,
                       float threshold, mdsm_candidate *h_cands, long long cap,
                       long long *ncand, float *mean, float *rms, cudaStream_t st);
mdsm_status ref_detect_noalloc(const float *d_series, int ndms, int nsamp, float lowdm,
                               float dmstep, float threshold, mdsm_candidate *h_cands,
                               long long cap, long long *ncand, float *mean, float *rms,
                               cudaStream_t st);
// process_brute over the rows of several worker threads in turn (rpt rows each, DM of row k
// of thread t lowdm + (unsigned)(tshift * t) + k dmstep), with the statistics over the first
// stat_vals values (-1: all of them).
// Worker thread `thread`'s plan, of nthr threads, for blocks of nsamp samples of the survey
// (wrapper.cpp; the reference's launchers' DM slices).
mdsm_status plan_for_thread(const SURVEY *s, int thread, int nthr, int nsamp, mdsm_plan **out);
mdsm_status ref_detect_threads(const float *d_series, int ndms, int nsamp, long long stat_vals,
                               int rpt, int tshift, float lowdm, float dmstep, float threshold,
                               mdsm_candidate *h_cands, long long cap, long long *ncand,
                               float *mean, float *rms, cudaStream_t st);
// h_dmv (optional): each row's DM in place of lowdm + k dmstep
mdsm_status ref_detect_chunked(const float *d_series, int ndms, int nsamp, float lowdm,
                               float dmstep, float threshold, const float *h_mean,
                               const float *h_rms, long long nchunks, int spc,
                               mdsm_candidate *h_cands, long long cap, long long *ncand,
                               cudaStream_t st, const float *h_dmv = nullptr);
struct Plan;
mdsm_status ref_detect_subband(const Plan &p, const float *d_series, long long out_stride,
                               float threshold, const float *h_mean, const float *h_rms,
                               long long nchunks, int spc, mdsm_candidate *h_cands, long long cap,
                               long long *ncand, cudaStream_t st);
mdsm_status boxcar_detect(const void *d_series, int dtype, int ndms, int nsamp, int nwidths,
                          double threshold, mdsm_candidate *h_cands, long long cap,
                          long long *ncand, cudaStream_t st);
size_t boxcar_work_bytes(int ndms, int nsamp, long long cap);
// mom (optional, int32 series): the rows' exact moments as plan_run_device folds them; the
// statistics then come from them instead of a pass over the series.
mdsm_status boxcar_launch(const void *d_series, int dtype, int ndms, int nsamp, int nwidths,
                          double threshold, void *d_work, size_t work_bytes, long long cap,
                          mdsm_candidate *h_cands, long long *h_count, cudaStream_t st,
                          const unsigned long long *mom = nullptr);
void devcand_to_candidate(mdsm_candidate *c, long long n);
mdsm_status downsample(const void *in, int in_dtype, int nchans, long long in_stride,
                       long long len, int b, int mode, void *out, int out_dtype,
                       long long out_stride, cudaStream_t st);
mdsm_status rfi_clip(void *d_x, int dtype, int nchans, long long stride, long long len,
                     double k_chan, double k_spec, cudaStream_t st);

}  // namespace mdsm

struct mdsm_plan_s {
    mdsm::Plan p;
};
