// detect.cu -- single-pulse detection on dedispersed series, on the device.
//
// 1. The reference detector (src/mdsm/dedispersion_output.cpp:14-53,135-213): global mean/rms
//    over the whole block exactly as process_brute forms them (32K-value chunks, double sums,
//    a float running mean, the last chunk skipped by its loop test), then a median-of-five
//    filter and the test median - mean >= threshold*rms with DM > 1.  Every operation is an
//    explicitly rounded IEEE operation so candidates are identical to the host reference's.
// 2. A boxcar search (src/prototypes/singlepulse.cpp:41-146, restated): per-DM mean/sigma,
//    boxcar sums of widths 1..2^(nw-1) built by pairwise doubling, SNR per width, the best
//    width per sample and non-maximum suppression.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "box.cuh"
#include "internal.h"
#include "ptx.cuh"

namespace mdsm {

// ---------------------------------------------------------------------------------------------
// scratch: one grow-only device buffer per device for the detectors' work arrays.  A call
// holds its device's buffer (a lock) until it returns, so detector calls from several threads
// take turns; every such call synchronises its stream before returning.
// ---------------------------------------------------------------------------------------------
namespace {
struct ScratchSlot {
    std::mutex mu;
    void *p = nullptr;
    size_t bytes = 0;
};
std::mutex g_slots_mu;
std::map<int, std::unique_ptr<ScratchSlot>> g_slots;
}  // namespace

mdsm_status scratch_get(size_t bytes, void **out, std::unique_lock<std::mutex> *lease)
{
    int dev = 0;
    MDSM_CUDA_TRY(cudaGetDevice(&dev));
    ScratchSlot *slot = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_slots_mu);
        std::unique_ptr<ScratchSlot> &u = g_slots[dev];
        if (!u) u.reset(new ScratchSlot());
        slot = u.get();
    }
    *lease = std::unique_lock<std::mutex>(slot->mu);
    if (slot->bytes < bytes) {
        if (slot->p) cudaFree(slot->p);
        slot->p = nullptr;
        slot->bytes = 0;
        MDSM_CUDA_TRY(cudaMalloc(&slot->p, bytes));
        slot->bytes = bytes;
    }
    *out = slot->p;
    return MDSM_OK;
}


__device__ __forceinline__ float median5(float n1, float n2, float n3, float n4, float n5)
{
    // dedispersion_output.cpp:14-53, the same comparison network on values
    float a = n1, b = n2, c = n3, d = n4, e = n5, t;
    if (b < a) { t = a; a = b; b = t; }
    if (d < c) { t = c; c = d; d = t; }
    if (c < a) { t = b; b = d; d = t; c = a; }
    a = e;
    if (b < a) { t = a; a = b; b = t; }
    if (a < c) { t = b; b = d; d = t; a = c; }
    return (d < a) ? d : a;
}

// One thread per 32K chunk: sequential double sums (dedispersion_output.cpp:155-160).
__global__ void k_ref_chunk_sums(const float *__restrict__ buf, unsigned mod, unsigned nchunks,
                                 double2 *__restrict__ sums)
{
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nchunks) return;
    const float *p = buf + (size_t)i * mod;
    double t1 = 0.0, t2 = 0.0;
    for (unsigned j = 0; j < mod; ++j) {
        const double v = (double)__ldg(p + j);
        t1 = __dadd_rn(t1, v);
        t2 = __fma_rn(v, v, t2);  // v*v exact: same as dmul + dadd
    }
    sums[i] = make_double2(t1, t2);
}

// One thread: dedispersion_output.cpp:161-168.
__global__ void k_ref_finish(const double2 *__restrict__ sums, unsigned mod, unsigned nchunks,
                             float *__restrict__ stats)
{
    float localmean = 0.0f;
    double mean2 = 0.0;
    for (unsigned i = 0; i < nchunks; ++i) {
        const double2 s = sums[i];
        localmean = __double2float_rn(__dadd_rn((double)localmean, __ddiv_rn(s.x, (double)mod)));
        mean2 = __dadd_rn(mean2, __ddiv_rn(s.y, (double)mod));
    }
    localmean = __fdiv_rn(localmean, (float)nchunks);
    const float sq = __fmul_rn(localmean, localmean);
    const double v = __dadd_rn(__ddiv_rn(mean2, (double)nchunks), -(double)sq);
    stats[0] = localmean;
    stats[1] = __double2float_rn(__dsqrt_rn(v));
}

// dedispersion_output.cpp:176-210 (mean == NULL).  Rows are the worker threads' rows in turn,
// rpt per thread; row k of thread t has DM lowdm + (unsigned)(tshift * t) + k dmstep in float,
// left to right (:187,194; one thread: rpt = ndms, tshift = 0).
__global__ void k_ref_detect(const float *__restrict__ buf, int ndms, int nsamp, float lowdm,
                             float dmstep, float threshold, const float *__restrict__ stats,
                             DevCand *__restrict__ cands, unsigned long long *__restrict__ count,
                             long long cap, int rpt, int tshift)
{
    const int row = blockIdx.y;
    const unsigned t = (unsigned)row / (unsigned)rpt, k = (unsigned)row % (unsigned)rpt;
    const float thisdm = __fadd_rn(__fadd_rn(lowdm, (float)((unsigned)tshift * t)),
                                   __fmul_rn((float)k, dmstep));
    if (!((double)thisdm > 1.0)) return;
    const float mean = stats[0], rms = stats[1];
    const float lim = __fmul_rn(rms, threshold);
    const float *r = buf + (size_t)row * nsamp;
    const unsigned nl = (unsigned)nsamp - 4u;
    for (unsigned l = blockIdx.x * blockDim.x + threadIdx.x; l < nl; l += gridDim.x * blockDim.x) {
        const float m = median5(__ldg(r + l), __ldg(r + l + 1), __ldg(r + l + 2), __ldg(r + l + 3),
                                __ldg(r + l + 4));
        if (__fsub_rn(m, mean) >= lim) {
            const unsigned long long at = atomicAdd(count, 1ull);
            if ((long long)at < cap) cands[at] = DevCand{row, (int32_t)l, 1, __fdiv_rn(m, rms)};
        }
    }
}

static void sort_cands(mdsm_candidate *c, long long n)
{
    std::sort(c, c + n, [](const mdsm_candidate &a, const mdsm_candidate &b) {
        return a.dm_idx != b.dm_idx ? a.dm_idx < b.dm_idx : a.sample < b.sample;
    });
}

// The candidate count and up to cap records from the device (on stream st, synchronised), in
// mdsm_candidate order, sorted by (dm, sample).  The staging vector is host memory only.
static mdsm_status fetch_cands(DevCand *d_c, unsigned long long *d_count, long long cap,
                               mdsm_candidate *h, long long *ncand, cudaStream_t st)
{
    unsigned long long n = 0;
    MDSM_CUDA_TRY(cudaMemcpyAsync(&n, d_count, sizeof(n), cudaMemcpyDeviceToHost, st));
    MDSM_CUDA_TRY(cudaStreamSynchronize(st));
    if (n & kBoxCountLate) return fail(MDSM_ETIMEOUT, "boxcar detector: a staging wait ran out");
    *ncand = (long long)n;
    const long long got = std::min<long long>((long long)n, cap);
    if (got > 0 && h) {
        std::vector<DevCand> tmp((size_t)got);
        MDSM_CUDA_TRY(cudaMemcpyAsync(tmp.data(), d_c, (size_t)got * sizeof(DevCand),
                                      cudaMemcpyDeviceToHost, st));
        MDSM_CUDA_TRY(cudaStreamSynchronize(st));
        for (long long i = 0; i < got; ++i) {
            h[i].dm_idx = tmp[i].dm_idx;
            h[i].sample = tmp[i].sample;
            h[i].width = tmp[i].width;
            h[i].snr = tmp[i].snr;
        }
        sort_cands(h, got);
    }
    return MDSM_OK;
}

mdsm_status ref_detect(const float *d_series, int ndms, int nsamp, float lowdm, float dmstep,
                       float threshold, mdsm_candidate *h_cands, long long cap,
                       long long *ncand, float *mean, float *rms, cudaStream_t st)
{
    return ref_detect_threads(d_series, ndms, nsamp, -1, ndms, 0, lowdm, dmstep, threshold,
                              h_cands, cap, ncand, mean, rms, st);
}

mdsm_status ref_detect_threads(const float *d_series, int ndms, int nsamp, long long stat_vals,
                               int rpt, int tshift, float lowdm, float dmstep, float threshold,
                               mdsm_candidate *h_cands, long long cap, long long *ncand,
                               float *mean, float *rms, cudaStream_t st)
{
    if (rpt <= 0) return fail(MDSM_EINVAL, "reference detector: rows per thread");
    const unsigned long long vals64 = stat_vals >= 0
                                          ? (unsigned long long)stat_vals
                                          : (unsigned long long)ndms * (unsigned long long)nsamp;
    if (vals64 == 0 || vals64 > (unsigned long long)ndms * (unsigned long long)nsamp)
        return fail(MDSM_EINVAL, "reference detector: statistics over the series' values");
    if (vals64 > 0xFFFFFFFFull / 2)
        return fail(MDSM_EINVAL, "reference detector counts values in 32 bits");
    const unsigned vals = (unsigned)vals64;
    const unsigned mod = vals < 32768u ? vals : 32768u;
    // iterations of dedispersion_output.cpp:154-165: stops once (iters+1)*mod >= vals
    unsigned nchunks = 1;
    while ((unsigned long long)(nchunks + 1) * mod < vals) ++nchunks;
    if (cap < 0) cap = 0;
    const size_t off_cnt = 0, off_stats = 16, off_sums = 64;
    const size_t off_c = off_sums + ((size_t)nchunks * sizeof(double2) + 255) / 256 * 256;
    const size_t bytes = off_c + (size_t)std::max<long long>(cap, 1) * sizeof(DevCand);
    void *sc = nullptr;
    std::unique_lock<std::mutex> lease;
    MDSM_TRY(scratch_get(bytes, &sc, &lease));
    char *base = static_cast<char *>(sc);
    auto *d_count = reinterpret_cast<unsigned long long *>(base + off_cnt);
    auto *d_stats = reinterpret_cast<float *>(base + off_stats);
    auto *d_sums = reinterpret_cast<double2 *>(base + off_sums);
    auto *d_c = reinterpret_cast<DevCand *>(base + off_c);
    MDSM_CUDA_TRY(cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), st));
    k_ref_chunk_sums<<<(nchunks + 127) / 128, 128, 0, st>>>(d_series, mod, nchunks, d_sums);
    k_ref_finish<<<1, 1, 0, st>>>(d_sums, mod, nchunks, d_stats);
    dim3 grid((unsigned)std::min<long long>((nsamp + 255) / 256, 64), (unsigned)ndms);
    k_ref_detect<<<grid, 256, 0, st>>>(d_series, ndms, nsamp, lowdm, dmstep, threshold, d_stats,
                                       d_c, d_count, cap, rpt, tshift);
    MDSM_CUDA_TRY(cudaGetLastError());
    float hs[2];
    MDSM_CUDA_TRY(cudaMemcpyAsync(hs, d_stats, sizeof(hs), cudaMemcpyDeviceToHost, st));
    MDSM_TRY(fetch_cands(d_c, d_count, cap, h_cands, ncand, st));
    if (mean) *mean = hs[0];
    if (rms) *rms = hs[1];
    return MDSM_OK;
}

// ---------------------------------------------------------------------------------------------
// The reference detectors' other forms: process_brute with caller noise statistics (one mean
// and rms per samplesPerChunk samples, dedispersion_output.cpp:198-209) and process_subband
// (:56-132): per-row statistics when the caller gives none, else the caller's chunk
// statistics.  One kernel applies the median-of-five test to any set of rows.
// ---------------------------------------------------------------------------------------------

// One thread per row: dedispersion_output.cpp:87-97, sequential double sums (total += x,
// total2 += pow(x, 2), exact for a float x) and the float mean / rms the reference keeps.
__global__ void k_row_stats_seq(const float *__restrict__ buf, long long stride, int nrows,
                                int nvalid, float2 *__restrict__ stats)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nrows) return;
    const float *r = buf + (size_t)k * stride;
    double t1 = 0.0, t2 = 0.0;
    for (int t = 0; t < nvalid; ++t) {
        const double v = (double)__ldg(r + t);
        t1 = __dadd_rn(t1, v);
        t2 = __fma_rn(v, v, t2);  // v*v exact: same as dmul + dadd
    }
    const float lm = __double2float_rn(__ddiv_rn(t1, (double)nvalid));
    const double var = __dadd_rn(__ddiv_rn(t2, (double)nvalid), -__dmul_rn((double)lm, (double)lm));
    stats[k] = make_float2(lm, __double2float_rn(__dsqrt_rn(var)));
}

// Median-of-five test on rows [nrows][nvalid] (row pitch stride) whose DMs are dmv[row]:
// median - mean >= rms * threshold and DM > 1, with (mean, rms) the row's (rowstats) or the
// caller's chunk values cmean/crms[t / spc].  snr_mode 0 prints median / rms (process_subband,
// and process_brute without caller statistics), 1 (median - mean) / rms (process_brute with
// them).  Candidates carry the row, the sample and `width`.
__global__ void k_median_detect(const float *__restrict__ buf, long long stride, int nrows,
                                int nvalid, const float *__restrict__ dmv, float threshold,
                                const float2 *__restrict__ rowstats,
                                const float *__restrict__ cmean, const float *__restrict__ crms,
                                int spc, int snr_mode, int width, int row0,
                                DevCand *__restrict__ cands,
                                unsigned long long *__restrict__ count, long long cap)
{
    const int k = blockIdx.y;
    if (k >= nrows || !((double)__ldg(dmv + k) > 1.0)) return;
    const float *r = buf + (size_t)k * stride;
    float2 rs = make_float2(0.0f, 0.0f);
    if (rowstats) rs = rowstats[k];
    const unsigned nl = (unsigned)nvalid - 4u;
    for (unsigned l = blockIdx.x * blockDim.x + threadIdx.x; l < nl; l += gridDim.x * blockDim.x) {
        const float m = median5(__ldg(r + l), __ldg(r + l + 1), __ldg(r + l + 2), __ldg(r + l + 3),
                                __ldg(r + l + 4));
        const float mean = rowstats ? rs.x : __ldg(cmean + l / (unsigned)spc);
        const float rms = rowstats ? rs.y : __ldg(crms + l / (unsigned)spc);
        if (__fsub_rn(m, mean) >= __fmul_rn(rms, threshold)) {
            const float snr = snr_mode ? __fdiv_rn(__fsub_rn(m, mean), rms) : __fdiv_rn(m, rms);
            const unsigned long long at = atomicAdd(count, 1ull);
            if ((long long)at < cap) cands[at] = DevCand{row0 + k, (int32_t)l, width, snr};
        }
    }
}

namespace {

// Work area of the median detectors: counter, DM values, row statistics, chunk statistics,
// candidate records.
struct MedianWork {
    unsigned long long *count;
    float *dmv;
    float2 *rowstats;
    float *cmean, *crms;
    DevCand *cands;
};

mdsm_status median_work(int nrows, long long nchunks, long long cap, MedianWork *w,
                        std::unique_lock<std::mutex> *lease)
{
    auto up = [](size_t b) { return (b + 255) / 256 * 256; };
    const size_t o_dmv = 256, o_rs = o_dmv + up((size_t)nrows * 4);
    const size_t o_cm = o_rs + up((size_t)nrows * 8), o_cr = o_cm + up((size_t)nchunks * 4);
    const size_t o_c = o_cr + up((size_t)nchunks * 4);
    void *sc = nullptr;
    MDSM_TRY(scratch_get(o_c + (size_t)std::max<long long>(cap, 1) * sizeof(DevCand), &sc,
                         lease));
    char *b = static_cast<char *>(sc);
    w->count = reinterpret_cast<unsigned long long *>(b);
    w->dmv = reinterpret_cast<float *>(b + o_dmv);
    w->rowstats = reinterpret_cast<float2 *>(b + o_rs);
    w->cmean = reinterpret_cast<float *>(b + o_cm);
    w->crms = reinterpret_cast<float *>(b + o_cr);
    w->cands = reinterpret_cast<DevCand *>(b + o_c);
    return MDSM_OK;
}

}  // namespace

mdsm_status ref_detect_chunked(const float *d_series, int ndms, int nsamp, float lowdm,
                               float dmstep, float threshold, const float *h_mean,
                               const float *h_rms, long long nchunks, int spc,
                               mdsm_candidate *h_cands, long long cap, long long *ncand,
                               cudaStream_t st, const float *h_dmv)
{
    if (spc <= 0 || nchunks < (long long)(nsamp - 5) / spc + 1)
        return fail(MDSM_ERANGE, "chunk statistics: fewer values than (nsamp - 4) / spc");
    if (cap < 0) cap = 0;
    MedianWork w;
    std::unique_lock<std::mutex> lease;
    MDSM_TRY(median_work(ndms, nchunks, cap, &w, &lease));
    // the reference's DM of row k: lowdm + k * dmstep in float (dedispersion_output.cpp:194)
    std::vector<float> dmv((size_t)ndms);
    for (int k = 0; k < ndms; ++k)
        dmv[(size_t)k] = h_dmv ? h_dmv[k] : (lowdm + 0.0f) + (float)(unsigned)k * dmstep;
    MDSM_CUDA_TRY(cudaMemsetAsync(w.count, 0, sizeof(unsigned long long), st));
    MDSM_CUDA_TRY(cudaMemcpyAsync(w.dmv, dmv.data(), dmv.size() * 4, cudaMemcpyHostToDevice, st));
    MDSM_CUDA_TRY(cudaMemcpyAsync(w.cmean, h_mean, (size_t)nchunks * 4, cudaMemcpyHostToDevice, st));
    MDSM_CUDA_TRY(cudaMemcpyAsync(w.crms, h_rms, (size_t)nchunks * 4, cudaMemcpyHostToDevice, st));
    dim3 grid((unsigned)std::min<long long>((nsamp + 255) / 256, 64), (unsigned)ndms);
    k_median_detect<<<grid, 256, 0, st>>>(d_series, nsamp, ndms, nsamp, w.dmv, threshold,
                                          nullptr, w.cmean, w.crms, spc, 1, 1, 0, w.cands,
                                          w.count, cap);
    MDSM_CUDA_TRY(cudaGetLastError());
    return fetch_cands(w.cands, w.count, cap, h_cands, ncand, st);
}

mdsm_status ref_detect_subband(const Plan &p, const float *d_series, long long out_stride,
                               float threshold, const float *h_mean, const float *h_rms,
                               long long nchunks, int spc, mdsm_candidate *h_cands, long long cap,
                               long long *ncand, cudaStream_t st)
{
    if (p.kind != 2) return fail(MDSM_EINVAL, "subband detector: not a subband plan");
    if (h_mean && (!h_rms || spc <= 0 || nchunks < (long long)(p.nsamp - 5) / spc + 1))
        return fail(MDSM_ERANGE, "chunk statistics: fewer values than (nsamp - 4) / spc");
    if (cap < 0) cap = 0;
    MedianWork w;
    std::unique_lock<std::mutex> lease;
    MDSM_TRY(median_work(p.ndms, h_mean ? nchunks : 0, cap, &w, &lease));
    MDSM_CUDA_TRY(cudaMemsetAsync(w.count, 0, sizeof(unsigned long long), st));
    MDSM_CUDA_TRY(cudaMemcpyAsync(w.dmv, p.dm_values.data(), (size_t)p.ndms * 4,
                                  cudaMemcpyHostToDevice, st));
    if (h_mean) {
        MDSM_CUDA_TRY(cudaMemcpyAsync(w.cmean, h_mean, (size_t)nchunks * 4,
                                      cudaMemcpyHostToDevice, st));
        MDSM_CUDA_TRY(cudaMemcpyAsync(w.crms, h_rms, (size_t)nchunks * 4,
                                      cudaMemcpyHostToDevice, st));
    }
    for (size_t i = 0; i < p.pass_row0.size(); ++i) {
        const int row0 = (int)p.pass_row0[i];
        const int rows = (int)((i + 1 < p.pass_row0.size() ? p.pass_row0[i + 1] : p.ndms) - row0);
        const int b = p.pass_bin[i];
        const int nvalid = p.nsamp / b;
        if (rows <= 0 || nvalid < 5) continue;
        const float *rb = d_series + (size_t)row0 * out_stride;
        float2 *rs = nullptr;
        if (!h_mean) {
            rs = w.rowstats + row0;
            k_row_stats_seq<<<(rows + 127) / 128, 128, 0, st>>>(rb, out_stride, rows, nvalid, rs);
        }
        dim3 grid((unsigned)std::min<long long>((nvalid + 255) / 256, 64), (unsigned)rows);
        k_median_detect<<<grid, 256, 0, st>>>(rb, out_stride, rows, nvalid, w.dmv + row0,
                                              threshold, rs, w.cmean, w.crms, spc, 0, b, row0,
                                              w.cands, w.count, cap);
    }
    MDSM_CUDA_TRY(cudaGetLastError());
    return fetch_cands(w.cands, w.count, cap, h_cands, ncand, st);
}

// ---------------------------------------------------------------------------------------------
// Reference detector without allocation.
//
// Some callers cannot call cudaMalloc: a real-time pipeline stage that must not stall on the
// device allocator between blocks, a host that hands all device memory out once at start-up
// (an HBM-budget admission loop does this), or a plugin running where allocation is not
// permitted.  This variant keeps its work arrays (per-chunk sums, the statistics, the candidate
// counter and the candidate records) in one fixed array in device global memory instead of
// the library's allocated scratch buffer.  The array is defined at file scope, so every GPU
// that loads the library holds it (kNoAllocBytes, about 2 MiB) until the process exits.
//
// Limits: ndms*nsamp < 2^31 values (as the allocating detector: MDSM_EINVAL beyond) and at
// most kNoAllocCands stored candidates (cap; MDSM_ERANGE beyond).
// Every call uses the same array and leaves its contents behind; the candidate counter is
// cleared at the start of each call.  Calls whose work overlaps on the GPU (different streams
// or threads without ordering between them) race on the array.
// ---------------------------------------------------------------------------------------------
constexpr unsigned kNoAllocChunks = 65536u;
// the value count is below 2^31, so 32768-value chunks number at most 2^31 / 2^15
static_assert((unsigned long long)kNoAllocChunks * 32768ull >= 0xFFFFFFFFull / 2 + 1,
              "the fixed array holds the statistics of every block the detector accepts");
constexpr long long kNoAllocCands = 65536;
constexpr size_t kNoAllocHeader = 256;  // counter at 0, statistics at 16
constexpr size_t kNoAllocBytes =
    kNoAllocHeader + (size_t)kNoAllocChunks * sizeof(double2) + (size_t)kNoAllocCands * 16;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// The device address of g_noalloc_scratch in the current context.  Host code may not use the
// symbol's name as a pointer (on the host it names a stand-in, not device memory).  The address
// is looked up on every call (a cheap query): a cached one would go stale when the context is
// torn down and created again (cudaDeviceReset).
static mdsm_status noalloc_scratch(char **out)
{
    void *ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    *out = static_cast<char *>(ptr);
    return MDSM_OK;
}

mdsm_status ref_detect_noalloc(const float *d_series, int ndms, int nsamp, float lowdm,
                               float dmstep, float threshold, mdsm_candidate *h_cands,
                               long long cap, long long *ncand, float *mean, float *rms,
                               cudaStream_t st)
{
    const unsigned long long vals64 = (unsigned long long)ndms * (unsigned long long)nsamp;
    if (vals64 > 0xFFFFFFFFull / 2)
        return fail(MDSM_EINVAL, "reference detector counts values in 32 bits");
    const unsigned vals = (unsigned)vals64;
    const unsigned mod = vals < 32768u ? vals : 32768u;
    unsigned nchunks = 1;
    while ((unsigned long long)(nchunks + 1) * mod < vals) ++nchunks;  // <= kNoAllocChunks
    if (cap < 0) cap = 0;
    if (cap > kNoAllocCands)
        return fail(MDSM_ERANGE, "no-allocation detector: cap " + std::to_string(cap) +
                                     " exceeds the fixed array's " +
                                     std::to_string(kNoAllocCands) + " candidates");
    char *base = nullptr;
    MDSM_TRY(noalloc_scratch(&base));
    auto *d_count = reinterpret_cast<unsigned long long *>(base);
    auto *d_stats = reinterpret_cast<float *>(base + 16);
    auto *d_sums = reinterpret_cast<double2 *>(base + kNoAllocHeader);
    auto *d_c = reinterpret_cast<DevCand *>(base + kNoAllocHeader +
                                            (size_t)kNoAllocChunks * sizeof(double2));
    MDSM_CUDA_TRY(cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), st));
    k_ref_chunk_sums<<<(nchunks + 127) / 128, 128, 0, st>>>(d_series, mod, nchunks, d_sums);
    k_ref_finish<<<1, 1, 0, st>>>(d_sums, mod, nchunks, d_stats);
    dim3 grid((unsigned)std::min<long long>((nsamp + 255) / 256, 64), (unsigned)ndms);
    k_ref_detect<<<grid, 256, 0, st>>>(d_series, ndms, nsamp, lowdm, dmstep, threshold, d_stats,
                                       d_c, d_count, cap, ndms, 0);
    MDSM_CUDA_TRY(cudaGetLastError());
    float hs[2];
    MDSM_CUDA_TRY(cudaMemcpyAsync(hs, d_stats, sizeof(hs), cudaMemcpyDeviceToHost, st));
    MDSM_TRY(fetch_cands(d_c, d_count, cap, h_cands, ncand, st));  // (synchronises st)
    if (mean) *mean = hs[0];
    if (rms) *rms = hs[1];
    return MDSM_OK;
}

// ---------------------------------------------------------------------------------------------
// boxcar search
// ---------------------------------------------------------------------------------------------

template <typename T>
__device__ __forceinline__ double ld_d(const T *p, long long i)
{
    return (double)__ldg(p + i);
}

// Per (DM, 1024-sample chunk) sums, left to right.
template <typename T>
__global__ void k_series_chunk_sums(const T *__restrict__ y, long long n, int nch,
                                    double2 *__restrict__ part)
{
    const int d = blockIdx.y;
    const int ch = blockIdx.x * blockDim.x + threadIdx.x;
    if (ch >= nch) return;
    const T *r = y + (size_t)d * n;
    const long long c0 = (long long)ch * 1024, c1 = min(c0 + 1024, n);
    double p1 = 0.0, p2 = 0.0;
    for (long long i = c0; i < c1; ++i) {
        const double v = ld_d(r, i);
        p1 = __dadd_rn(p1, v);
        p2 = __fma_rn(v, v, p2);  // v*v exact: same as dmul + dadd
    }
    part[(size_t)d * nch + ch] = make_double2(p1, p2);
}

__global__ void k_series_finish(const double2 *__restrict__ part, int ndms, int nch, long long n,
                                double2 *__restrict__ musig)
{
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= ndms) return;
    double s1 = 0.0, s2 = 0.0;
    for (int i = 0; i < nch; ++i) {
        const double2 p = part[(size_t)d * nch + i];
        s1 = __dadd_rn(s1, p.x);
        s2 = __dadd_rn(s2, p.y);
    }
    const double m = __ddiv_rn(s1, (double)n);
    const double var = __dadd_rn(__ddiv_rn(s2, (double)n), -__dmul_rn(m, m));
    musig[d] = make_double2(m, var > 0.0 ? __dsqrt_rn(var) : 0.0);
}

// Exact statistics of int32 series: one CTA per DM, int64 sum and 128-bit (hi, lo) sum of
// squares.  Integer sums do not depend on order, so the reduction is parallel; the conversion
// to mean and sigma is the fixed double formula the oracle uses.
__global__ void __launch_bounds__(256)
    k_series_stats_int(const int32_t *__restrict__ y, long long n, double2 *__restrict__ musig)
{
    const int d = blockIdx.x;
    const int32_t *r = y + (size_t)d * n;
    long long s1 = 0;
    unsigned long long lo = 0, hi = 0;  // sum of squares, 128 bits
    auto acc = [&](long long v) {
        s1 += v;
        const unsigned long long nl = lo + (unsigned long long)(v * v);
        hi += (nl < lo);
        lo = nl;
    };
    long long i0 = 0;
    if ((reinterpret_cast<uintptr_t>(r) & 15) == 0) {  // 16-byte loads, 4 values each
        const long long n4 = n >> 2;
        const int4 *r4 = reinterpret_cast<const int4 *>(r);
        for (long long i = threadIdx.x; i < n4; i += blockDim.x) {
            const int4 v = __ldg(r4 + i);
            acc(v.x);
            acc(v.y);
            acc(v.z);
            acc(v.w);
        }
        i0 = n4 << 2;
    }
    for (long long i = i0 + threadIdx.x; i < n; i += blockDim.x) acc(__ldg(r + i));
    // warp shuffles, then the 8 warps' partials through shared memory
    for (int o = 16; o > 0; o >>= 1) {
        const long long s1o = __shfl_down_sync(0xffffffffu, s1, o);
        const unsigned long long loo = __shfl_down_sync(0xffffffffu, lo, o);
        const unsigned long long hio = __shfl_down_sync(0xffffffffu, hi, o);
        s1 += s1o;
        const unsigned long long nl = lo + loo;
        hi += hio + (nl < lo);
        lo = nl;
    }
    __shared__ long long a1[8];
    __shared__ unsigned long long alo[8], ahi[8];
    const int warp = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        a1[warp] = s1;
        alo[warp] = lo;
        ahi[warp] = hi;
    }
    __syncthreads();
    if (threadIdx.x == 0)
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
            a1[0] += a1[w];
            const unsigned long long nl = alo[0] + alo[w];
            ahi[0] += ahi[w] + (nl < alo[0]);
            alo[0] = nl;
        }
    if (threadIdx.x == 0) {
        const double e2 = __ddiv_rn(__dadd_rn(__dmul_rn((double)ahi[0], 18446744073709551616.0),
                                              (double)alo[0]),
                                    (double)n);
        const double m = __ddiv_rn((double)a1[0], (double)n);
        const double var = __dadd_rn(e2, -__dmul_rn(m, m));
        musig[d] = make_double2(m, var > 0.0 ? __dsqrt_rn(var) : 0.0);
    }
}

// Per-DM (mean, sigma) of float32 or int32 series into musig (the statistics both searches
// use); part: series_stats_part_bytes() of work space for the float form.
size_t series_stats_part_bytes(int ndms, long long n)
{
    return (size_t)ndms * (size_t)((n + 1023) / 1024) * sizeof(double2);
}

mdsm_status series_stats_launch(const void *y, int dtype, int ndms, long long n, double2 *part,
                                double2 *musig, cudaStream_t st)
{
    if (dtype == MDSM_OUT_F32) {
        const int nch = (int)((n + 1023) / 1024);
        dim3 g1((unsigned)((nch + 127) / 128), (unsigned)ndms);
        k_series_chunk_sums<float><<<g1, 128, 0, st>>>(static_cast<const float *>(y), n, nch,
                                                       part);
        k_series_finish<<<(ndms + 127) / 128, 128, 0, st>>>(part, ndms, nch, n, musig);
    } else {
        k_series_stats_int<<<ndms, 256, 0, st>>>(static_cast<const int32_t *>(y), n, musig);
    }
    MDSM_CUDA_TRY(cudaGetLastError());
    return MDSM_OK;
}

constexpr int kBoxThreads = 256;
constexpr int kBoxK = 15;   // positions per thread (tiles of 3840 - WMAX + 1 samples, rounded)
constexpr int kBoxKE = 7;   // the exact path's positions per thread (its region 1792 samples)

// One CTA per (DM, run of `tpc` consecutive tiles): the tile loop of box.cuh.
template <typename T, int NW>
__global__ void __launch_bounds__(kBoxThreads, 4)
    k_boxcar(const T *__restrict__ y, long long n, int tpc, double threshold,
             const double2 *__restrict__ musig, DevCand *__restrict__ cands,
             unsigned long long *__restrict__ count, long long cap)
{
    extern __shared__ __align__(16) unsigned char sm[];
    const int d = blockIdx.y;
    const double mu = musig[d].x, sig = musig[d].y;
    if (!(sig > 0.0)) return;
    constexpr int TILE = BoxGeom<NW, kBoxThreads, kBoxK, kBoxKE>::TILE;
    const long long ntiles = (n + TILE - 1) / TILE;
    const long long tile_lo = (long long)blockIdx.x * tpc;
    const long long tile_hi = tile_lo + tpc < ntiles ? tile_lo + tpc : ntiles;
    box_run<T, NW, kBoxThreads, kBoxK, kBoxKE, true>(y + (size_t)d * n, n, tile_lo, tile_hi, mu,
                                                     sig, threshold, d, cands, count, cap, sm,
                                                     BoxBarCta{}, (int)threadIdx.x, true);
}

// The boxcar search of every DM row, for 1..9 widths (a template per width count).
template <typename T>
static cudaError_t launch_boxcar(const T *y, int ndms, long long n, int nw, double threshold,
                                 const double2 *musig, DevCand *cands,
                                 unsigned long long *count, long long cap, cudaStream_t st);

// Shared memory of k_boxcar: the staged samples, two sum buffers and the best SNR of NBEST
// positions.
template <int NW>
static size_t boxcar_smem()
{
    return BoxGeom<NW, kBoxThreads, kBoxK, kBoxKE>::SMEM;
}

template <typename T, int NW>
static cudaError_t launch_boxcar_nw(const T *y, int ndms, long long n, double threshold,
                                    const double2 *musig, DevCand *cands,
                                    unsigned long long *count, long long cap, cudaStream_t st)
{
    const size_t smem = boxcar_smem<NW>();
    cudaError_t e = cudaFuncSetAttribute(k_boxcar<T, NW>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    // runs of up to 8 tiles per CTA while that leaves >= 8192 CTAs (several waves of 4 per SM)
    constexpr int TILE = BoxGeom<NW, kBoxThreads, kBoxK, kBoxKE>::TILE;
    const long long ntiles = (n + TILE - 1) / TILE;
    int tpc = (int)std::min<long long>(8, std::max<long long>(1, ntiles * ndms / 8192));
    tpc = (int)std::min<long long>(tpc, ntiles);
    const long long runs = (ntiles + tpc - 1) / tpc;
    tpc = (int)((ntiles + runs - 1) / runs);  // the same number of runs, evened out
    dim3 g3((unsigned)((ntiles + tpc - 1) / tpc), (unsigned)ndms);
    k_boxcar<T, NW><<<g3, kBoxThreads, smem, st>>>(y, n, tpc, threshold, musig, cands, count, cap);
    return cudaGetLastError();
}

template <typename T>
static cudaError_t launch_boxcar(const T *y, int ndms, long long n, int nw, double threshold,
                                 const double2 *musig, DevCand *cands,
                                 unsigned long long *count, long long cap, cudaStream_t st)
{
    switch (nw) {
#define BOX(K) case K: return launch_boxcar_nw<T, K>(y, ndms, n, threshold, musig, cands, count, cap, st)
    BOX(1); BOX(2); BOX(3); BOX(4); BOX(5); BOX(6); BOX(7); BOX(8); BOX(9);
#undef BOX
    default: return cudaErrorInvalidValue;
    }
}

mdsm_status boxcar_detect(const void *d_series, int dtype, int ndms, int nsamp, int nwidths,
                          double threshold, mdsm_candidate *h_cands, long long cap,
                          long long *ncand, cudaStream_t st)
{
    if (dtype != MDSM_OUT_F32 && dtype != MDSM_OUT_I32)
        return fail(MDSM_EINVAL, "boxcar detector: series must be float32 or int32");
    if (nwidths < 1 || nwidths > 9) return fail(MDSM_EINVAL, "boxcar detector: widths up to 256");
    if (cap < 0) cap = 0;
    const int nch = (nsamp + 1023) / 1024;
    const size_t off_cnt = 0, off_part = 256;
    const size_t off_ms = off_part + ((size_t)ndms * nch * sizeof(double2) + 255) / 256 * 256;
    const size_t off_c = off_ms + ((size_t)ndms * sizeof(double2) + 255) / 256 * 256;
    const size_t bytes = off_c + (size_t)std::max<long long>(cap, 1) * sizeof(DevCand);
    void *sc = nullptr;
    std::unique_lock<std::mutex> lease;
    MDSM_TRY(scratch_get(bytes, &sc, &lease));
    char *base = static_cast<char *>(sc);
    auto *d_count = reinterpret_cast<unsigned long long *>(base + off_cnt);
    auto *d_part = reinterpret_cast<double2 *>(base + off_part);
    auto *d_ms = reinterpret_cast<double2 *>(base + off_ms);
    auto *d_c = reinterpret_cast<DevCand *>(base + off_c);
    MDSM_CUDA_TRY(cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), st));
    dim3 g1((unsigned)((nch + 127) / 128), (unsigned)ndms);
    if (dtype == MDSM_OUT_F32) {
        const float *y = static_cast<const float *>(d_series);
        k_series_chunk_sums<float><<<g1, 128, 0, st>>>(y, nsamp, nch, d_part);
        k_series_finish<<<(ndms + 127) / 128, 128, 0, st>>>(d_part, ndms, nch, nsamp, d_ms);
        MDSM_CUDA_TRY(launch_boxcar(y, ndms, nsamp, nwidths, threshold, d_ms, d_c, d_count, cap,
                                    st));
    } else {
        const int32_t *y = static_cast<const int32_t *>(d_series);
        k_series_stats_int<<<ndms, 256, 0, st>>>(y, nsamp, d_ms);
        MDSM_CUDA_TRY(launch_boxcar(y, ndms, nsamp, nwidths, threshold, d_ms, d_c, d_count, cap,
                                    st));
    }
    MDSM_CUDA_TRY(cudaGetLastError());
    return fetch_cands(d_c, d_count, cap, h_cands, ncand, st);
}

// (mean, sigma) of int32 series from their exact moments folded into the dedispersion store
// (sum, sum of squares as two 64-bit words): the same conversion as k_series_stats_int's.
__global__ void k_mom_finish(const unsigned long long *__restrict__ mom, int ndms, long long n,
                             double2 *__restrict__ musig)
{
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= ndms) return;
    const long long s1 = (long long)mom[3 * (size_t)d];
    const unsigned long long lo = mom[3 * (size_t)d + 1], hi = mom[3 * (size_t)d + 2];
    const double e2 = __ddiv_rn(__dadd_rn(__dmul_rn((double)hi, 18446744073709551616.0),
                                          (double)lo),
                                (double)n);
    const double m = __ddiv_rn((double)s1, (double)n);
    const double var = __dadd_rn(e2, -__dmul_rn(m, m));
    musig[d] = make_double2(m, var > 0.0 ? __dsqrt_rn(var) : 0.0);
}

// Bytes of device work area boxcar_launch needs.
size_t boxcar_work_bytes(int ndms, int nsamp, long long cap)
{
    const int nch = (nsamp + 1023) / 1024;
    return 256 + ((size_t)ndms * nch * sizeof(double2) + 255) / 256 * 256 +
           ((size_t)ndms * sizeof(double2) + 255) / 256 * 256 +
           (size_t)std::max<long long>(cap, 1) * sizeof(DevCand);
}

// The boxcar search launched on `st` without waiting: statistics, search, then asynchronous
// copies of the candidate count and up to `cap` records into pinned host memory (h_cands holds
// the device record layout until devcand_to_candidate() puts it in mdsm_candidate order).
mdsm_status boxcar_launch(const void *d_series, int dtype, int ndms, int nsamp, int nwidths,
                          double threshold, void *d_work, size_t work_bytes, long long cap,
                          mdsm_candidate *h_cands, long long *h_count, cudaStream_t st,
                          const unsigned long long *mom)
{
    if (dtype != MDSM_OUT_F32 && dtype != MDSM_OUT_I32)
        return fail(MDSM_EINVAL, "boxcar detector: series must be float32 or int32");
    if (nwidths < 1 || nwidths > 9) return fail(MDSM_EINVAL, "boxcar detector: widths up to 256");
    if (work_bytes < boxcar_work_bytes(ndms, nsamp, cap))
        return fail(MDSM_ERANGE, "boxcar detector: work area too small");
    if (cap < 1) cap = 1;
    const int nch = (nsamp + 1023) / 1024;
    char *base = static_cast<char *>(d_work);
    auto *d_count = reinterpret_cast<unsigned long long *>(base);
    auto *d_part = reinterpret_cast<double2 *>(base + 256);
    const size_t off_ms = 256 + ((size_t)ndms * nch * sizeof(double2) + 255) / 256 * 256;
    auto *d_ms = reinterpret_cast<double2 *>(base + off_ms);
    auto *d_c = reinterpret_cast<DevCand *>(base + off_ms +
                                            ((size_t)ndms * sizeof(double2) + 255) / 256 * 256);
    MDSM_CUDA_TRY(cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), st));
    dim3 g1((unsigned)((nch + 127) / 128), (unsigned)ndms);
    if (dtype == MDSM_OUT_F32) {
        const float *y = static_cast<const float *>(d_series);
        k_series_chunk_sums<float><<<g1, 128, 0, st>>>(y, nsamp, nch, d_part);
        k_series_finish<<<(ndms + 127) / 128, 128, 0, st>>>(d_part, ndms, nch, nsamp, d_ms);
        MDSM_CUDA_TRY(launch_boxcar(y, ndms, nsamp, nwidths, threshold, d_ms, d_c, d_count, cap,
                                    st));
    } else {
        const int32_t *y = static_cast<const int32_t *>(d_series);
        if (mom)  // moments already folded into the series' store: no pass over the series
            k_mom_finish<<<(ndms + 127) / 128, 128, 0, st>>>(mom, ndms, nsamp, d_ms);
        else
            k_series_stats_int<<<ndms, 256, 0, st>>>(y, nsamp, d_ms);
        MDSM_CUDA_TRY(launch_boxcar(y, ndms, nsamp, nwidths, threshold, d_ms, d_c, d_count, cap,
                                    st));
    }
    MDSM_CUDA_TRY(cudaGetLastError());
    MDSM_CUDA_TRY(cudaMemcpyAsync(h_count, d_count, sizeof(long long), cudaMemcpyDeviceToHost, st));
    static_assert(sizeof(DevCand) == sizeof(mdsm_candidate), "record sizes differ");
    MDSM_CUDA_TRY(cudaMemcpyAsync(h_cands, d_c, (size_t)cap * sizeof(DevCand),
                                  cudaMemcpyDeviceToHost, st));
    return MDSM_OK;
}

// Put n device-layout records (dm, sample, width, snr) into mdsm_candidate order, in place.
void devcand_to_candidate(mdsm_candidate *c, long long n)
{
    for (long long i = 0; i < n; ++i) {
        DevCand dc;
        std::memcpy(&dc, &c[i], sizeof dc);
        c[i].dm_idx = dc.dm_idx;
        c[i].sample = dc.sample;
        c[i].snr = dc.snr;
        c[i].width = dc.width;
    }
}

// ---------------------------------------------------------------------------------------------
// detrend and normalise (src/prototypes/detrend.cu:12-100): per block of len samples of each
// DM series, fit a line on x_i = -len/2 + 0.5 + i by least squares, subtract it, divide by the
// residual rms.  Sums in double (the prototype's are float tree reductions).
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ double block_sum_d(double v, double *red)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    double t = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += red[i];
    return t;
}

__global__ void __launch_bounds__(256)
    k_detrend(float *__restrict__ y, long long n, int len)
{
    __shared__ double red[8];
    float *b = y + (size_t)blockIdx.y * n + (size_t)blockIdx.x * len;
    double sy = 0, sxy = 0, sxx = 0;
    for (int i = threadIdx.x; i < len; i += blockDim.x) {
        const double x = -len / 2.0 + 0.5 + i;
        const double v = (double)b[i];
        sy += v;
        sxy += x * v;
        sxx += x * x;
    }
    sy = block_sum_d(sy, red);
    sxy = block_sum_d(sxy, red);
    sxx = block_sum_d(sxx, red);
    const double a = sy / len, bb = sxy / sxx;
    double ss = 0;
    for (int i = threadIdx.x; i < len; i += blockDim.x) {
        const double x = -len / 2.0 + 0.5 + i;
        const float v = (float)((double)b[i] - (a + bb * x));
        b[i] = v;
        ss += (double)v * (double)v;
    }
    ss = block_sum_d(ss, red);
    const double sd = sqrt(ss / len);
    for (int i = threadIdx.x; i < len; i += blockDim.x) b[i] = (float)((double)b[i] / sd);
}

mdsm_status detrend_normalise(float *d_series, int ndms, long long nsamp, int len,
                              cudaStream_t st)
{
    if (!d_series || ndms <= 0 || len <= 0 || nsamp < len)
        return fail(MDSM_EINVAL, "detrend: bad arguments");
    const long long nblk = nsamp / len;
    if (nblk > 2147483647LL || ndms > 65535) return fail(MDSM_EINVAL, "detrend: too large");
    k_detrend<<<dim3((unsigned)nblk, (unsigned)ndms), 256, 0, st>>>(d_series, nsamp, len);
    MDSM_CUDA_TRY(cudaGetLastError());
    return MDSM_OK;
}

}  // namespace mdsm

extern "C" mdsm_status mdsm_detrend_normalise_device(float *d_series, int ndms, long long nsamp,
                                                     int len, void *stream)
{
    return mdsm::detrend_normalise(d_series, ndms, nsamp, len, static_cast<cudaStream_t>(stream));
}
