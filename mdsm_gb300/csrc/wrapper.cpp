// wrapper.cpp -- the reference's internal C ABI pair (src/mdsm/dedispersion_wrapper.cu:4-13):
// call_initialise_devices and call_dedisperse, the per-GPU worker thread its manager spawns
// (src/mdsm/dedispersion_manager.cpp:348-374).  The worker keeps the reference's barrier and
// lock protocol (src/mdsm/dedispersion_thread.cu:246-401) so that manager and its output thread
// run unchanged against it; inside a block it runs this library's plans instead of the
// reference kernels.  Differences, each invisible to the reference's manager and callers: the
// overlap tail stays on the device (one device-to-device copy) instead of being written back
// into the caller's input buffer, the series covers every DM trial and sample (the L1 kernel
// leaves tdms % 32 trials and nsamp % 210 samples at zero), and a failing block is reported
// on stderr with its output zeroed instead of exiting the process.
#include <cuda_runtime.h>
#include <pthread.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "dedispersion_thread.h"
#include "internal.h"

namespace mdsm {
namespace {

struct WorkerState {
    mdsm_plan *plan = nullptr;
    int plan_nsamp = -1;
    cudaStream_t st = nullptr;
    void *d_in[2] = {nullptr, nullptr};
    size_t d_in_bytes = 0;
    void *d_out = nullptr;
    size_t d_out_bytes = 0;
    int cur = 0;            // device buffer holding the current block
    long long pitch = 0;    // device row pitch (elements) of the current plan
    long long tail_col = -1;  // column of the previous block's tail in d_in[cur ^ 1]
    long long tail_pitch = 0;
};

void report(const THREAD_PARAMS *tp, const char *what)
{
    fprintf(stderr, "mdsm worker %d: %s: %s\n", (int)tp->thread_num, what, mdsm_last_error());
}

}  // namespace

// Worker thread `thread`'s plan (of nthr sharing the sub-DM calls) for blocks of nsamp
// samples: the DM slice and shift arithmetic the reference's launchers use
// (dedispersion_thread.cu:64-94, 97-217, 220-243).
mdsm_status plan_for_thread(const SURVEY *s, int thread, int nthr, int nsamp, mdsm_plan **out)
{
    if (s->useBruteForce) {
        // (the brute-force DM ranges split by the survey's thread count)
        const unsigned nb = s->num_threads ? s->num_threads : 1;
        // dedispersion_thread.cu:76,229: float arithmetic, left to right
        const float startdm = s->lowdm + s->dmstep * (float)s->tdms / (float)nb * (float)thread;
        mdsm_segment seg{startdm, s->dmstep, (int)(s->tdms / nb)};
        mdsm_brute_desc d;
        memset(&d, 0, sizeof d);
        d.nchans = (int)s->nchans;
        d.fch1 = s->fch1;
        d.foff = s->foff;
        d.tsamp = s->tsamp;
        d.nsamp = nsamp;
        d.segs = &seg;
        d.nsegs = 1;
        d.shift_mode = s->useL1Cache ? MDSM_SHIFT_L1 : MDSM_SHIFT_OPT;
        d.in_dtype = MDSM_F32;
        d.out_dtype = MDSM_OUT_F32;
        return mdsm_brute_plan_create(&d, out);
    }
    if (nthr < 1) nthr = 1;
    std::vector<SUBBAND_PASSES> passes(s->pass_parameters, s->pass_parameters + s->num_passes);
    for (SUBBAND_PASSES &p : passes) {
        // dedispersion_thread.cu:160-161: the sub-DM calls are split among the threads
        p.ncalls = p.ncalls / nthr;
        p.lowdm = p.lowdm + p.sub_dmstep * (float)p.ncalls * (float)thread;
    }
    mdsm_subband_desc d;
    memset(&d, 0, sizeof d);
    d.nchans = (int)s->nchans;
    d.fch1 = s->fch1;
    d.foff = s->foff;
    d.tsamp = s->tsamp;
    d.nsamp = nsamp;
    d.nsubs = (int)s->nsubs;
    d.passes = passes.data();
    d.npasses = (int)passes.size();
    d.use_fma = 1;
    d.in_dtype = MDSM_F32;
    d.out_dtype = MDSM_OUT_F32;
    return mdsm_subband_plan_create(&d, out);
}

namespace {

mdsm_status build_plan(const THREAD_PARAMS *tp, int nsamp, mdsm_plan **out)
{
    return plan_for_thread(tp->survey, tp->thread_num, tp->num_threads, nsamp, out);
}

// Grow-only device buffer; *fresh tells whether it was (re)allocated.
mdsm_status ensure_dev(void **p, size_t *have, size_t want, bool *fresh)
{
    *fresh = false;
    if (*p && *have >= want) return MDSM_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *have = 0;
    MDSM_CUDA_TRY(cudaMalloc(p, want));
    *have = want;
    *fresh = true;
    return MDSM_OK;
}

// Make the plan for nsamp current, with device buffers to match (new input buffers are
// zeroed; copy_in zeroes the columns past the caller's rows of every block).  A tail kept in
// the buffer that is about to be replaced moves to the new one.
mdsm_status prepare(WorkerState &w, const THREAD_PARAMS *tp, int nsamp)
{
    if (w.plan && w.plan_nsamp == nsamp) return MDSM_OK;
    mdsm_plan *np = nullptr;
    MDSM_TRY(build_plan(tp, nsamp, &np));
    mdsm_plan_info info;
    mdsm_plan_get_info(np, &info);
    // device rows hold the caller's whole rows (nsamp + the manager's maxshift, which may
    // differ from the plan's by a sample either way) and whatever the plan reads
    const long long hp4 = ((long long)nsamp + tp->maxshift + 3) / 4 * 4;
    const long long pitch = std::max<long long>(info.in_stride, hp4);
    long long need = 0;
    if (plan_in_requirements(np->p, pitch, &need) != MDSM_OK) {
        mdsm_plan_destroy(np);
        return MDSM_EINVAL;
    }
    // the caller's whole rows land in the buffer, past what the plan reads when its own
    // maximum shift is the smaller one (the subband passes' usually is)
    const long long rows_b = (long long)tp->survey->nchans * pitch * 4;
    const size_t in_b = (size_t)std::max<long long>(need, rows_b) + 256;
    // keep the tail of the previous block: it sits in d_in[cur ^ 1], which only grows
    std::vector<char> keep;
    const bool had_tail = w.tail_col >= 0;
    if (had_tail && w.d_in_bytes < in_b) {
        // buffers are about to be replaced: move the tail to the new first buffer afterwards
        const long long ms = tp->maxshift;
        keep.resize((size_t)tp->survey->nchans * ms * 4);
        MDSM_CUDA_TRY(cudaMemcpy2D(keep.data(), (size_t)ms * 4,
                                   static_cast<float *>(w.d_in[w.cur ^ 1]) + w.tail_col,
                                   (size_t)w.tail_pitch * 4, (size_t)ms * 4, tp->survey->nchans,
                                   cudaMemcpyDeviceToHost));
    }
    bool fresh = false;
    for (int k = 0; k < 2; ++k) {
        size_t have = w.d_in_bytes;
        MDSM_TRY(ensure_dev(&w.d_in[k], &have, in_b, &fresh));
        if (fresh) MDSM_CUDA_TRY(cudaMemset(w.d_in[k], 0, in_b));
    }
    w.d_in_bytes = std::max(w.d_in_bytes, in_b);
    MDSM_TRY(ensure_dev(&w.d_out, &w.d_out_bytes, (size_t)info.out_bytes + 256, &fresh));
    if (!keep.empty()) {
        MDSM_CUDA_TRY(cudaMemcpy2D(w.d_in[w.cur ^ 1], (size_t)tp->maxshift * 4, keep.data(),
                                   (size_t)tp->maxshift * 4, (size_t)tp->maxshift * 4,
                                   tp->survey->nchans, cudaMemcpyHostToDevice));
        w.tail_col = 0;
        w.tail_pitch = tp->maxshift;
    }
    if (w.plan) mdsm_plan_destroy(w.plan);
    w.plan = np;
    w.plan_nsamp = nsamp;
    w.pitch = pitch;
    return MDSM_OK;
}

// dedispersion_thread.cu:280-303: the block into the device.  The first data block copies
// every column of the caller's [nchans][nsamp + maxshift] buffer; later blocks take the
// previous block's last maxshift samples per channel from the device and the caller's new
// samples from columns [maxshift, nsamp + maxshift).
mdsm_status copy_in(WorkerState &w, const THREAD_PARAMS *tp, int nsamp, bool first)
{
    const long long ms = tp->maxshift, hp = (long long)nsamp + ms, nch = tp->survey->nchans;
    w.cur ^= 1;
    float *dst = static_cast<float *>(w.d_in[w.cur]);
    if (first || w.tail_col < 0) {
        MDSM_CUDA_TRY(cudaMemcpy2DAsync(dst, (size_t)w.pitch * 4, tp->input, (size_t)hp * 4,
                                        (size_t)hp * 4, nch, cudaMemcpyHostToDevice, w.st));
    } else {
        if (ms > 0)
            MDSM_CUDA_TRY(cudaMemcpy2DAsync(dst, (size_t)w.pitch * 4,
                                            static_cast<float *>(w.d_in[w.cur ^ 1]) + w.tail_col,
                                            (size_t)w.tail_pitch * 4, (size_t)ms * 4, nch,
                                            cudaMemcpyDeviceToDevice, w.st));
        MDSM_CUDA_TRY(cudaMemcpy2DAsync(dst + ms, (size_t)w.pitch * 4, tp->input + ms,
                                        (size_t)hp * 4, (size_t)nsamp * 4, nch,
                                        cudaMemcpyHostToDevice, w.st));
    }
    // columns past the caller's rows (the plan's true maximum shift may exceed the manager's
    // maxshift by a sample): zero, as a fresh buffer holds them
    if (w.pitch > hp)
        MDSM_CUDA_TRY(cudaMemset2DAsync(dst + hp, (size_t)w.pitch * 4, 0,
                                        (size_t)(w.pitch - hp) * 4, nch, w.st));
    w.tail_col = nsamp;
    w.tail_pitch = w.pitch;
    return MDSM_OK;
}

mdsm_status dedisperse_block(WorkerState &w, int nsamp)
{
    return mdsm_dedisperse_device(w.plan, w.d_in[w.cur], w.pitch, w.d_in_bytes, w.d_out, nsamp,
                                  w.st);
}

// dedispersion_thread.cu:352-355: the thread's series into its output buffer, in the
// reference's layout (subband: per pass, rows of nsamp/binsize samples, packed).
mdsm_status copy_out(WorkerState &w, const THREAD_PARAMS *tp, int nsamp)
{
    const Plan &p = w.plan->p;
    const size_t want = tp->dedispersed_size;
    size_t done = 0;
    if (p.kind == 1) {
        const size_t n = std::min(want, (size_t)p.ndms * (size_t)nsamp);
        MDSM_CUDA_TRY(cudaMemcpyAsync(tp->output, w.d_out, n * 4, cudaMemcpyDeviceToHost, w.st));
        done = n;
    } else {
        for (size_t i = 0; i < p.pass_row0.size() && done < want; ++i) {
            const long long b = p.pass_bin[i];
            const long long r0 = p.pass_row0[i];
            const long long r1 = i + 1 < p.pass_row0.size() ? p.pass_row0[i + 1] : p.ndms;
            const long long cols = nsamp / b;
            long long rows = r1 - r0;
            if (cols <= 0 || rows <= 0) continue;
            rows = std::min<long long>(rows, (long long)((want - done) / (size_t)cols));
            if (rows <= 0) break;
            MDSM_CUDA_TRY(cudaMemcpy2DAsync(tp->output + done, (size_t)cols * 4,
                                            static_cast<float *>(w.d_out) + r0 * nsamp,
                                            (size_t)nsamp * 4, (size_t)cols * 4, rows,
                                            cudaMemcpyDeviceToHost, w.st));
            done += (size_t)rows * cols;
        }
    }
    MDSM_CUDA_TRY(cudaStreamSynchronize(w.st));
    if (done < want) memset(tp->output + done, 0, (want - done) * 4);
    return MDSM_OK;
}

void release(WorkerState &w)
{
    if (w.plan) mdsm_plan_destroy(w.plan);
    for (void *p : w.d_in)
        if (p) cudaFree(p);
    if (w.d_out) cudaFree(w.d_out);
    if (w.st) cudaStreamDestroy(w.st);
    w = WorkerState();
}

bool barrier(pthread_barrier_t *b)
{
    const int r = pthread_barrier_wait(b);
    return r == 0 || r == PTHREAD_BARRIER_SERIAL_THREAD;
}

}  // namespace
}  // namespace mdsm

using namespace mdsm;

// src/mdsm/dedispersion_thread.cu:4-62
extern "C" DEVICES *call_initialise_devices(SURVEY *survey)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
        set_error("No CUDA-capable device found");
        fprintf(stderr, "No CUDA-capable device found\n");
        return nullptr;
    }
    DEVICES *d = static_cast<DEVICES *>(malloc(sizeof(DEVICES)));
    if (!d) return nullptr;
    d->devices = static_cast<DEVICE_INFO *>(malloc((size_t)n * sizeof(DEVICE_INFO)));
    d->num_devices = 0;
    d->minTotalGlobalMem = 1024UL * 1024 * 16;
    for (int i = 0; i < n; ++i) {
        cudaDeviceProp prop;
        if (cudaGetDeviceProperties(&prop, i) != cudaSuccess) continue;
        if (!((double)(prop.totalGlobalMem / 1024) > 1024 * 2.5 * 1024)) continue;
        bool use = true;
        if (survey && survey->gpu_ids) {
            use = false;
            for (unsigned j = 0; j < survey->num_gpus; ++j)
                if (survey->gpu_ids[j] == (unsigned)i) use = true;
        }
        if (!use) continue;
        DEVICE_INFO &di = d->devices[d->num_devices];
        int clk = 0;
        cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, i);
        di.multiprocessor_count = prop.multiProcessorCount;
        di.constant_memory = (int)prop.totalConstMem;
        di.shared_memory = (int)prop.sharedMemPerBlock;
        di.register_count = prop.regsPerBlock;
        di.thread_count = prop.maxThreadsPerBlock;
        di.clock_rate = clk;
        di.device_id = i;
        if (prop.totalGlobalMem / 1024 < d->minTotalGlobalMem)
            d->minTotalGlobalMem = prop.totalGlobalMem / 1024;
        d->num_devices++;
    }
    if (d->num_devices == 0) {
        free(d->devices);
        free(d);
        set_error("No CUDA-capable device found");
        fprintf(stderr, "No CUDA-capable device found\n");
        return nullptr;
    }
    return d;
}

// src/mdsm/dedispersion_thread.cu:246-401
extern "C" void *call_dedisperse(void *thread_params)
{
    THREAD_PARAMS *tp = static_cast<THREAD_PARAMS *>(thread_params);
    SURVEY *s = tp->survey;
    int nsamp = (int)s->nsamp;
    int loop_counter = 0, iters = 0;
    WorkerState w;
    bool ok = cudaSetDevice(tp->device_id) == cudaSuccess &&
              cudaStreamCreateWithFlags(&w.st, cudaStreamNonBlocking) == cudaSuccess;
    if (!ok) {
        set_error("cannot use device " + std::to_string(tp->device_id));
        report(tp, "start");
    }
    while (true) {
        bool data = loop_counter >= tp->iterations;
        bool good = ok && data;
        if (good && (prepare(w, tp, nsamp) != MDSM_OK ||
                     copy_in(w, tp, nsamp, loop_counter == 1) != MDSM_OK)) {
            report(tp, "copy in");
            good = false;
        }
        if (!barrier(tp->input_barrier)) fprintf(stderr, "mdsm worker: input barrier\n");
        if (good && dedisperse_block(w, nsamp) != MDSM_OK) {
            report(tp, "dedisperse");
            good = false;
        }
        if (!barrier(tp->output_barrier)) fprintf(stderr, "mdsm worker: output barrier\n");
        if (data) {
            if (!good || copy_out(w, tp, nsamp) != MDSM_OK) {
                if (good) report(tp, "copy out");
                memset(tp->output, 0, tp->dedispersed_size * 4);
            }
        }
        pthread_rwlock_rdlock(tp->rw_lock);
        nsamp = (int)tp->survey->nsamp;
        if (tp->stop) {
            if (iters >= tp->iterations - 1) {
                pthread_rwlock_unlock(tp->rw_lock);
                for (int i = 0; i < tp->maxiters - tp->iterations; ++i) {
                    barrier(tp->input_barrier);
                    barrier(tp->output_barrier);
                }
                break;
            }
            ++iters;
        }
        pthread_rwlock_unlock(tp->rw_lock);
        ++loop_counter;
    }
    release(w);
    return thread_params;
}
