// output.cpp -- process_output, the output thread of the reference's manager
// (src/mdsm/dedispersion_output.cpp:216-356), with the search on the device.  The thread keeps
// the reference's barrier, lock and file protocol: it waits at the input barrier; from cycle
// `iterations` on it searches the shared output buffer, which holds the block handed in two
// cycles earlier, with that block's values (nsamp, timestamp, blockRate, noise statistics);
// it waits at the output barrier, advances those values under the read lock and leaves when
// `stop` is set.  The search is the reference's: process_brute (:135-213) over every worker
// thread's rows in turn, with the block's own statistics or the caller's per-chunk ones, or
// process_subband (:56-132) per thread and pass, as this library's device detectors restate
// them; the lines have the reference's format.  Differences: no progress lines on stdout, and
// a device failure is reported on stderr and leaves that block without candidates instead of
// ending the process.
#include <cuda_runtime.h>
#include <pthread.h>
#include <stdio.h>
#include <string.h>
#include <time.h>

#include <algorithm>
#include <string>
#include <vector>

#include "dedispersion_output.h"
#include "internal.h"

namespace mdsm {
namespace {

constexpr long long kOutCap = 1 << 21;  // candidates of one block (more are reported)

struct OutState {
    cudaStream_t st = nullptr;
    void *d_buf = nullptr;
    size_t d_bytes = 0;
    std::vector<mdsm_plan *> plans;  // subband: per worker thread, for plan_nsamp
    int plan_nsamp = -1;
    FILE *fp = nullptr;
    long long written = 0;  // samples written to the current file
    std::vector<mdsm_candidate> cands;  // one block's candidates (kOutCap, allocated once)
};

void report(const char *what) { fprintf(stderr, "mdsm output: %s: %s\n", what, mdsm_last_error()); }

bool wait_barrier(pthread_barrier_t *b)
{
    const int r = pthread_barrier_wait(b);
    return r == 0 || r == PTHREAD_BARRIER_SERIAL_THREAD;
}

// The current file, opened as dedispersion_output.cpp:233-240 (single file, at start) and
// :254-282 (a new file whenever the last one was closed: basedir/prefix_<time>_<secs>.dat, the
// time of the block or of the host clock).
FILE *open_file(const SURVEY *s, double ts)
{
    char path[512];
    if (s->single_file_mode) {
        snprintf(path, sizeof path, "%s/%s.dat", s->basedir, s->fileprefix);
    } else {
        time_t now = s->use_pc_time ? time(nullptr) : (time_t)ts;
        struct tm tmv;
        localtime_r(&now, &tmv);
        char tb[32];
        strftime(tb, sizeof tb, "%F_%T", &tmv);
        snprintf(path, sizeof path, "%s/%s_%s_%u.dat", s->basedir, s->fileprefix, tb,
                 s->secs_per_file);
    }
    return fopen(path, "w");
}

mdsm_status ensure_buf(OutState &o, size_t bytes)
{
    if (o.d_buf && o.d_bytes >= bytes) return MDSM_OK;
    if (o.d_buf) cudaFree(o.d_buf);
    o.d_buf = nullptr;
    o.d_bytes = 0;
    MDSM_CUDA_TRY(cudaMalloc(&o.d_buf, bytes));
    o.d_bytes = bytes;
    return MDSM_OK;
}

void drop_plans(OutState &o)
{
    for (mdsm_plan *p : o.plans)
        if (p) mdsm_plan_destroy(p);
    o.plans.clear();
    o.plan_nsamp = -1;
}

// process_brute over the buffer (every worker thread's tdms / num_threads rows of nsamp
// samples, thread after thread): the statistics of its first read_nsamp * tdms values, or the
// caller's per-chunk statistics (cmean, crms, one pair per samplesPerChunk samples).
mdsm_status search_brute(OutState &o, const OUTPUT_PARAMS *p, int read_nsamp, double ts,
                         double rate, const float *cmean, const float *crms)
{
    const SURVEY *s = p->survey;
    const unsigned nt = s->num_threads ? s->num_threads : 1;
    const int nsamp = (int)s->nsamp;
    const int rpt = (int)(s->tdms / nt);
    const int ndms = rpt * (int)nt;
    if (rpt <= 0 || nsamp < 5) return MDSM_OK;
    if (p->dedispersed_size != (size_t)rpt * (size_t)nsamp || p->nthreads != (int)nt)
        return fail(MDSM_EINVAL, "output thread: the buffer must hold num_threads workers' "
                                 "rows of nsamp");
    const size_t n = (size_t)ndms * (size_t)nsamp;
    MDSM_TRY(ensure_buf(o, n * 4));
    MDSM_CUDA_TRY(cudaMemcpyAsync(o.d_buf, p->output_buffer, n * 4, cudaMemcpyHostToDevice, o.st));
    // dedispersion_output.cpp:187: the DM offset of each thread, in float, truncated to int
    const int tshift = (int)((float)s->tdms * s->dmstep / (float)nt);
    std::vector<mdsm_candidate> &c = o.cands;
    c.resize((size_t)kOutCap);
    long long nc = 0;
    const float *y = static_cast<const float *>(o.d_buf);
    const float thr = s->detection_threshold;
    std::vector<float> dmv((size_t)ndms);
    for (int row = 0; row < ndms; ++row) {
        const unsigned t = (unsigned)row / (unsigned)rpt, k = (unsigned)row % (unsigned)rpt;
        dmv[(size_t)row] = (s->lowdm + (float)((unsigned)tshift * t)) + (float)k * s->dmstep;
    }
    const int spc = s->samplesPerChunk ? (int)s->samplesPerChunk : nsamp;
    if (cmean) {
        const long long nchunks = (nsamp - 5) / spc + 1;
        MDSM_TRY(ref_detect_chunked(y, ndms, nsamp, s->lowdm, s->dmstep, thr, cmean, crms, nchunks,
                                    spc, c.data(), kOutCap, &nc, o.st, dmv.data()));
    } else {
        MDSM_TRY(ref_detect_threads(y, ndms, nsamp, (long long)read_nsamp * (long long)s->tdms,
                                    rpt, tshift, s->lowdm, s->dmstep, thr, c.data(), kOutCap, &nc,
                                    nullptr, nullptr, o.st));
    }
    if (nc > kOutCap) fprintf(stderr, "mdsm output: %lld candidates, %lld written\n", nc, kOutCap);
    const long long got = std::min(nc, kOutCap);
    for (long long i = 0; i < got; ++i) {
        const mdsm_candidate &e = c[(size_t)i];
        const double t = ts + (double)(unsigned)e.sample * rate;
        if (cmean)
            fprintf(o.fp, "%lf, %f, %f, %f, %f  \n", t, dmv[(size_t)e.dm_idx], e.snr,
                    cmean[e.sample / spc], crms[e.sample / spc]);
        else
            fprintf(o.fp, "%lf, %f, %f\n", t, dmv[(size_t)e.dm_idx], e.snr);
    }
    return MDSM_OK;
}

// process_subband per worker thread and pass: the thread's series, packed as the workers pack
// them (per pass, rows of nsamp / binsize samples), back into rows of nsamp on the device,
// searched with the thread's plan (its passes' rows and DMs).
mdsm_status search_subband(OutState &o, const OUTPUT_PARAMS *p, double ts, double rate,
                           const float *cmean, const float *crms)
{
    const SURVEY *s = p->survey;
    const int nt = s->num_threads ? (int)s->num_threads : 1;
    const int nsamp = (int)s->nsamp;
    if (p->nthreads != nt)
        return fail(MDSM_EINVAL, "output thread: the buffer must hold num_threads workers' series");
    if (o.plan_nsamp != nsamp || (int)o.plans.size() != nt) {
        drop_plans(o);
        o.plans.assign((size_t)nt, nullptr);
        for (int t = 0; t < nt; ++t) MDSM_TRY(plan_for_thread(s, t, nt, nsamp, &o.plans[(size_t)t]));
        o.plan_nsamp = nsamp;
    }
    const int spc = s->samplesPerChunk ? (int)s->samplesPerChunk : nsamp;
    const long long nchunks = (nsamp - 5) / spc + 1;
    std::vector<mdsm_candidate> &c = o.cands;
    c.resize((size_t)kOutCap);
    for (int t = 0; t < nt; ++t) {
        const Plan &pl = o.plans[(size_t)t]->p;
        MDSM_TRY(ensure_buf(o, (size_t)pl.ndms * (size_t)nsamp * 4));
        const float *src = p->output_buffer + p->dedispersed_size * (size_t)t;
        size_t done = 0;
        for (size_t i = 0; i < pl.pass_row0.size(); ++i) {
            const long long b = pl.pass_bin[i];
            const long long r0 = pl.pass_row0[i];
            const long long r1 = i + 1 < pl.pass_row0.size() ? pl.pass_row0[i + 1] : pl.ndms;
            const long long cols = nsamp / b;
            long long rows = r1 - r0;
            if (cols <= 0 || rows <= 0) continue;
            rows = std::min<long long>(rows, (long long)((p->dedispersed_size - done) / (size_t)cols));
            if (rows <= 0) break;
            MDSM_CUDA_TRY(cudaMemcpy2DAsync(static_cast<float *>(o.d_buf) + r0 * nsamp,
                                            (size_t)nsamp * 4, src + done, (size_t)cols * 4,
                                            (size_t)cols * 4, (size_t)rows, cudaMemcpyHostToDevice,
                                            o.st));
            done += (size_t)rows * (size_t)cols;
        }
        long long nc = 0;
        MDSM_TRY(ref_detect_subband(pl, static_cast<const float *>(o.d_buf), nsamp,
                                    s->detection_threshold, cmean, crms, nchunks, spc, c.data(),
                                    kOutCap, &nc, o.st));
        if (nc > kOutCap)
            fprintf(stderr, "mdsm output: %lld candidates, %lld written\n", nc, kOutCap);
        const long long got = std::min(nc, kOutCap);
        for (long long i = 0; i < got; ++i) {
            const mdsm_candidate &e = c[(size_t)i];
            const double tt = ts + (double)e.sample * rate * (double)std::max(1, e.width);
            fprintf(o.fp, "%lf, %f, %f\n", tt, pl.dm_values[(size_t)e.dm_idx], e.snr);
        }
    }
    return MDSM_OK;
}

}  // namespace
}  // namespace mdsm

using namespace mdsm;

extern "C" void *process_output(void *output_params)
{
    OUTPUT_PARAMS *p = static_cast<OUTPUT_PARAMS *>(output_params);
    SURVEY *s = p->survey;
    OutState o;
    const int dev = s->gpu_ids && s->num_gpus ? (int)s->gpu_ids[0] : 0;
    bool device_ok = cudaSetDevice(dev) == cudaSuccess &&
                     cudaStreamCreateWithFlags(&o.st, cudaStreamNonBlocking) == cudaSuccess;
    if (!device_ok) report("device");
    // the values of the block before last (pp*) and of the last block (p*), as :221-227
    int pnsamp = (int)s->nsamp, ppnsamp = (int)s->nsamp;
    double ptimestamp = 0, pptimestamp = 0, pblockRate = 0, ppblockRate = 0;
    float *pmean = nullptr, *ppmean = nullptr, *prms = nullptr, *pprms = nullptr;
    if (s->single_file_mode) o.fp = open_file(s, 0.0);
    int iters = 0;
    for (int loop = 0;; ++loop) {
        if (!wait_barrier(p->input_barrier)) report("input barrier");
        if (loop >= p->iterations) {
            if (!o.fp || (!s->single_file_mode && o.written == 0)) {
                if (!s->single_file_mode && o.fp) fclose(o.fp);
                o.fp = open_file(s, pptimestamp);
            }
            if (o.fp && device_ok) {
                const mdsm_status r =
                    s->useBruteForce
                        ? search_brute(o, p, ppnsamp, pptimestamp, ppblockRate, ppmean, pprms)
                        : search_subband(o, p, pptimestamp, ppblockRate, ppmean, pprms);
                if (r != MDSM_OK) report("search");
                fflush(o.fp);
            }
            if (!s->single_file_mode) {
                o.written += ppnsamp;
                if ((double)o.written * ppblockRate > (double)s->secs_per_file) {
                    o.written = 0;
                    if (o.fp) fclose(o.fp);
                    o.fp = nullptr;
                }
            }
        }
        if (!wait_barrier(p->output_barrier)) report("output barrier");
        pthread_rwlock_rdlock(p->rw_lock);
        ppnsamp = pnsamp;
        pnsamp = (int)s->nsamp;
        pptimestamp = ptimestamp;
        ptimestamp = s->timestamp;
        ppblockRate = pblockRate;
        pblockRate = s->blockRate;
        ppmean = pmean;
        pmean = s->noiseMean;
        pprms = prms;
        prms = s->noiseRMS;
        bool leave = false;
        if (p->stop) {
            if (iters >= p->iterations - 1)
                leave = true;
            else
                ++iters;
        }
        pthread_rwlock_unlock(p->rw_lock);
        if (leave) {
            for (int i = 0; i < p->maxiters - p->iterations; ++i) {
                wait_barrier(p->input_barrier);
                wait_barrier(p->output_barrier);
            }
            break;
        }
    }
    if (o.fp) fclose(o.fp);
    drop_plans(o);
    if (o.d_buf) cudaFree(o.d_buf);
    if (o.st) cudaStreamDestroy(o.st);
    return output_params;
}
