// serve.cpp -- continuous-batching search server over many beams on one GPU.
//
// The reference processes one stream of blocks with one worker pthread per GPU and barriers
// (src/mdsm/dedispersion_manager.cpp:269-501, src/mdsm/dedispersion_thread.cu:246-401): block
// k+1 is copied in only after block k's output has been copied out, the overlap tail goes
// through host memory, and detection runs on one host thread.  Here many beams share the GPU:
//  * each beam keeps its last maxshift samples resident in HBM (two device block buffers used
//    in turn; the tail moves with one device-to-device copy), so only new samples cross the
//    host link;
//  * blocks from any beam are admitted as they arrive into a bounded set of slots (one CUDA
//    stream each, with the slot's output and candidate buffers), subject to an HBM budget;
//    blocks admitted while others run overlap with them on the device (copies and kernels
//    of different slots run concurrently);
//  * a block's pipeline is H2D of the new samples -> tail copy -> dedispersion -> boxcar
//    search -> D2H of the candidates only (the dedispersed block stays on the device);
//  * one dispatcher thread admits, one completion step records per-block latency (submit to
//    candidates on the host) and returns results in completion order;
//  * new samples wait in pinned staging buffers from a pool that is allocated once up to the
//    host staging budget and reused (pinning memory per block would cost more than copying
//    it); a producer either hands its block to submit (copied in by several threads) or
//    writes it in place into a buffer from acquire and queues it with commit.
// A beam's blocks are processed in order; different beams are independent, so a beam's
// results are the same whether it runs alone or mixed with others.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "internal.h"

namespace mdsm {

mdsm_status plan_create_brute(const mdsm_brute_desc &d, Plan &p);
mdsm_status plan_create_subband(const mdsm_subband_desc &d, Plan &p);

namespace {

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

struct StageBuf {
    void *h = nullptr;  // pinned
    size_t bytes = 0;
    bool used = false;
};

struct Beam {
    mdsm_plan *plan = nullptr;
    int acquired = -1;         // staging buffer handed out by acquire, not yet committed
    void *d_buf[2] = {nullptr, nullptr};
    size_t buf_bytes = 0;
    long long stride = 0;      // device row pitch (elements)
    long long next_block = 0;  // blocks submitted
    cudaEvent_t in_ready = nullptr;     // the last launched block's input (and tail) complete
    cudaEvent_t buf_free[2] = {nullptr, nullptr};  // last reader of each block buffer done
    size_t elem = 1;
};

struct Pending {
    int beam;
    long long block;
    long long ticket;
    double t_submit;
    int stage;      // staging buffer holding the new samples [nchans][cols]
    long long cols;
};

struct Slot {
    cudaStream_t st = nullptr;
    cudaEvent_t done = nullptr;
    void *d_out = nullptr;
    size_t out_bytes = 0;
    void *d_det = nullptr;  // detector work arrays + device candidates
    size_t det_bytes = 0;
    unsigned long long *d_mom = nullptr;  // the block's row moments, folded into its store
    size_t mom_bytes = 0;
    mdsm_candidate *h_cands = nullptr;  // pinned
    long long *h_count = nullptr;       // pinned
    bool busy = false;
    Pending job{};
};

}  // namespace

struct Server {
    mdsm_server_desc desc{};
    int device = 0;
    std::deque<Beam> beams;  // stable addresses while beams are added
    std::vector<Slot> slots;
    std::deque<Pending> queue;
    std::deque<std::pair<mdsm_block_result, std::vector<mdsm_candidate>>> results;
    std::mutex mu;
    std::condition_variable cv;
    std::thread worker;
    bool stop = false;
    long long tickets = 0;
    long long held_bytes = 0;     // device bytes held (beams + slots)
    std::vector<StageBuf> pool;   // pinned staging buffers
    long long pool_bytes = 0;     // pinned bytes allocated (<= host staging budget)
    std::vector<double> latencies;
    long long admitted = 0, refused = 0, completed = 0, units = 0;
    double t_first = 0, t_last = 0;
    mdsm_status fault = MDSM_OK;
    std::string fault_msg;

    void run();
    bool launch(Slot &s, Pending &p);
    void harvest(Slot &s);
    mdsm_status stage_get(size_t bytes, int *idx, bool admission = true);
    void prestage(size_t bytes, int count);
    void *stage_ptr(int idx)
    {
        std::lock_guard<std::mutex> lk(mu);
        return pool[(size_t)idx].h;
    }
};

// Pin `count` more staging buffers of `bytes` ahead of time, as far as the host staging budget
// allows without dropping any, so that blocks queued while the GPU is busy do not wait for
// page pinning (several hundred MB a block) inside the serving loop.
void Server::prestage(size_t bytes, int count)
{
    for (int i = 0; i < count; ++i) {
        {
            std::lock_guard<std::mutex> lk(mu);
            if (pool_bytes + (long long)bytes > desc.host_stage_bytes) return;
            pool_bytes += (long long)bytes;
        }
        void *h = nullptr;
        const bool ok = cudaHostAlloc(&h, bytes, 0) == cudaSuccess;
        std::lock_guard<std::mutex> lk(mu);
        if (!ok) {
            pool_bytes -= (long long)bytes;
            return;
        }
        size_t slot = pool.size();
        for (size_t k = 0; k < pool.size(); ++k)
            if (!pool[k].h) {
                slot = k;
                break;
            }
        if (slot == pool.size()) pool.emplace_back();
        pool[slot].h = h;
        pool[slot].bytes = bytes;
        pool[slot].used = false;
    }
}

// A free pinned buffer of at least `bytes` (the smallest that fits), else a new one while the
// budget allows (freeing idle buffers that are too small to make room), else MDSM_EBUDGET.
mdsm_status Server::stage_get(size_t bytes, int *idx, bool admission)
{
    std::unique_lock<std::mutex> lk(mu);
    int best = -1;
    for (size_t i = 0; i < pool.size(); ++i)
        if (!pool[i].used && pool[i].h && pool[i].bytes >= bytes &&
            (best < 0 || pool[i].bytes < pool[(size_t)best].bytes))
            best = (int)i;
    if (best >= 0) {
        pool[(size_t)best].used = true;
        *idx = best;
        return MDSM_OK;
    }
    std::vector<void *> drop;
    for (size_t i = 0; i < pool.size() && pool_bytes + (long long)bytes > desc.host_stage_bytes;
         ++i)
        if (!pool[i].used && pool[i].h) {
            drop.push_back(pool[i].h);
            pool_bytes -= (long long)pool[i].bytes;
            pool[i] = StageBuf();
        }
    if (pool_bytes + (long long)bytes > desc.host_stage_bytes) {
        if (admission) refused++;
        lk.unlock();
        for (void *h : drop) cudaFreeHost(h);
        return fail(MDSM_EBUDGET, "admission: host staging budget full, retry later");
    }
    pool_bytes += (long long)bytes;  // reserved before the (slow) pinning, outside the lock
    lk.unlock();
    for (void *h : drop) cudaFreeHost(h);
    void *h = nullptr;
    if (cudaHostAlloc(&h, bytes, 0) != cudaSuccess) {
        lk.lock();
        pool_bytes -= (long long)bytes;
        return fail(MDSM_ENOMEM, "pinned staging allocation failed");
    }
    lk.lock();
    size_t slot = pool.size();
    for (size_t i = 0; i < pool.size(); ++i)
        if (!pool[i].h) {
            slot = i;
            break;
        }
    if (slot == pool.size()) pool.emplace_back();
    pool[slot].h = h;
    pool[slot].bytes = bytes;
    pool[slot].used = true;
    *idx = (int)slot;
    return MDSM_OK;
}

void Server::harvest(Slot &s)
{
    mdsm_block_result r{};
    r.beam = s.job.beam;
    r.block = s.job.block;
    r.ticket = s.job.ticket;
    r.submit_time = s.job.t_submit;
    r.done_time = now_s();
    r.ncand = *s.h_count;
    r.status = MDSM_OK;
    if ((unsigned long long)r.ncand & kBoxCountLate) {  // the search's staging wait ran out
        r.status = MDSM_ETIMEOUT;
        r.ncand = 0;
    }
    const long long got = std::max<long long>(0, std::min<long long>(r.ncand, desc.cand_cap));
    devcand_to_candidate(s.h_cands, got);
    std::vector<mdsm_candidate> c(s.h_cands, s.h_cands + got);
    std::sort(c.begin(), c.end(), [](const mdsm_candidate &a, const mdsm_candidate &b) {
        return a.dm_idx != b.dm_idx ? a.dm_idx < b.dm_idx : a.sample < b.sample;
    });
    const Plan &p = beams[r.beam].plan->p;
    std::lock_guard<std::mutex> lk(mu);
    latencies.push_back(r.done_time - r.submit_time);
    completed++;
    units += (long long)p.ndms * p.nsamp;
    t_last = r.done_time;
    results.emplace_back(r, std::move(c));
    pool[(size_t)s.job.stage].used = false;
    s.busy = false;
    cv.notify_all();
}

bool Server::launch(Slot &s, Pending &job)
{
    Beam &b = beams[job.beam];
    Plan &p = b.plan->p;
    const int cur = (int)(job.block & 1), prv = cur ^ 1;
    const long long ms = p.maxshift, ns = p.nsamp;
    const size_t E = b.elem;
    cudaStream_t st = s.st;
    const void *h_stage = stage_ptr(job.stage);
    // A beam's blocks run one after another: the previous block's input holds this block's
    // tail, and its dedispersion must be done (the plan's intermediate buffers are per beam,
    // and the block before it read the buffer this block overwrites).  Other beams overlap.
    if (job.block > 0) cudaStreamWaitEvent(st, b.in_ready, 0);
    if (job.block > 0) cudaStreamWaitEvent(st, b.buf_free[prv], 0);
    cudaError_t e = cudaSuccess;
    if (job.block == 0) {
        e = cudaMemcpy2DAsync(b.d_buf[cur], b.stride * E, h_stage, (size_t)job.cols * E,
                              (size_t)(ns + ms) * E, p.nchans, cudaMemcpyHostToDevice, st);
    } else {
        if (ms > 0)
            e = cudaMemcpy2DAsync(b.d_buf[cur], b.stride * E,
                                  static_cast<char *>(b.d_buf[prv]) + ns * E, b.stride * E,
                                  (size_t)ms * E, p.nchans, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpy2DAsync(static_cast<char *>(b.d_buf[cur]) + ms * E, b.stride * E,
                                  h_stage, (size_t)job.cols * E, (size_t)ns * E, p.nchans,
                                  cudaMemcpyHostToDevice, st);
    }
    if (e == cudaSuccess) e = cudaEventRecord(b.in_ready, st);
    if (e != cudaSuccess) {
        fault = cuda_fail(e, "serving: input copy");
        return false;
    }
    // with the boxcar search, the dedispersion store also folds the rows' exact moments, so
    // the search's statistics need no pass of their own over the series
    bool folded = false;
    unsigned long long *mom = desc.detector == 1 && p.out_dtype == MDSM_OUT_I32 ? s.d_mom : nullptr;
    mdsm_status rc = plan_run_device(p, b.d_buf[cur], b.stride, b.buf_bytes, s.d_out, ns, st,
                                     mom, &folded);
    if (rc == MDSM_OK && cudaEventRecord(b.buf_free[cur], st) != cudaSuccess)
        rc = fail(MDSM_ECUDA, "serving: event record");
    if (rc == MDSM_OK && desc.detector == 1)
        rc = boxcar_launch(s.d_out, p.out_dtype, p.ndms, (int)ns, desc.nwidths, desc.threshold,
                           s.d_det, s.det_bytes, desc.cand_cap, s.h_cands, s.h_count, st,
                           folded ? mom : nullptr);
    if (rc == MDSM_OK && desc.detector != 1) {
        *s.h_count = 0;
    }
    if (rc == MDSM_OK && cudaEventRecord(s.done, st) != cudaSuccess)
        rc = fail(MDSM_ECUDA, "serving: event record");
    if (rc != MDSM_OK) {
        fault = rc;
        return false;
    }
    s.job = job;
    s.busy = true;
    return true;
}

void Server::run()
{
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
        // completions
        bool any_busy = false;
        for (auto &s : slots) {
            if (!s.busy) continue;
            if (cudaEventQuery(s.done) == cudaSuccess) {
                lk.unlock();
                harvest(s);
                lk.lock();
            } else {
                any_busy = true;
            }
        }
        // admissions: first queued block whose beam has no earlier block still queued
        for (auto &s : slots) {
            if (s.busy || queue.empty() || fault != MDSM_OK) continue;
            Pending job = queue.front();
            queue.pop_front();
            admitted++;
            lk.unlock();
            const bool ok = launch(s, job);
            lk.lock();
            if (!ok) {
                fault_msg = mdsm_last_error();
                cv.notify_all();
            }
        }
        if (stop && queue.empty()) {
            bool idle = true;
            for (auto &s : slots) idle &= !s.busy;
            if (idle) break;
        }
        if (any_busy || !queue.empty()) {
            lk.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(50));
            lk.lock();
        } else {
            cv.wait_for(lk, std::chrono::milliseconds(5));
        }
    }
}

}  // namespace mdsm

using namespace mdsm;

struct mdsm_server_s {
    Server s;
};

namespace {

mdsm_status add_beam(mdsm_server *sv, mdsm_plan *plan, int *beam)
{
    Server &S = sv->s;
    Plan &p = plan->p;
    Beam b;
    b.plan = plan;
    b.elem = dtype_size(p.in_dtype);
    b.stride = p.in_stride;
    long long need = 0;
    MDSM_TRY(plan_in_requirements(p, b.stride, &need));
    b.buf_bytes = (size_t)need + 256;
    const long long bytes = 2LL * (long long)b.buf_bytes + (long long)p.work_bytes;
    {
        std::lock_guard<std::mutex> lk(S.mu);
        if (S.held_bytes + bytes > S.desc.hbm_budget_bytes)
            return fail(MDSM_EBUDGET, "HBM budget: beam needs " + std::to_string(bytes) +
                                          " bytes, " +
                                          std::to_string(S.desc.hbm_budget_bytes - S.held_bytes) +
                                          " left");
        S.held_bytes += bytes;
    }
    for (int i = 0; i < 2; ++i) {
        MDSM_CUDA_TRY(cudaMalloc(&b.d_buf[i], b.buf_bytes));
        MDSM_CUDA_TRY(cudaMemset(b.d_buf[i], 0, b.buf_bytes));
    }
    MDSM_CUDA_TRY(cudaEventCreateWithFlags(&b.in_ready, cudaEventDisableTiming));
    for (int i = 0; i < 2; ++i)
        MDSM_CUDA_TRY(cudaEventCreateWithFlags(&b.buf_free[i], cudaEventDisableTiming));
    // slot buffers must hold this beam's output
    const size_t out_bytes = (size_t)p.ndms * p.nsamp * 4;
    for (auto &sl : S.slots) {
        if (sl.out_bytes < out_bytes) {
            if (sl.d_out) cudaFree(sl.d_out);
            S.held_bytes += (long long)(out_bytes - sl.out_bytes);
            MDSM_CUDA_TRY(cudaMalloc(&sl.d_out, out_bytes));
            sl.out_bytes = out_bytes;
        }
        const size_t det = boxcar_work_bytes(p.ndms, p.nsamp, S.desc.cand_cap);
        if (sl.det_bytes < det) {
            if (sl.d_det) cudaFree(sl.d_det);
            MDSM_CUDA_TRY(cudaMalloc(&sl.d_det, det));
            sl.det_bytes = det;
        }
        const size_t mb = (size_t)p.ndms * 3 * sizeof(unsigned long long);
        if (sl.mom_bytes < mb) {
            if (sl.d_mom) cudaFree(sl.d_mom);
            MDSM_CUDA_TRY(cudaMalloc(reinterpret_cast<void **>(&sl.d_mom), mb));
            sl.mom_bytes = mb;
        }
    }
    {
        std::lock_guard<std::mutex> lk(S.mu);
        S.beams.push_back(b);
        *beam = (int)S.beams.size() - 1;
    }
    // staging for the blocks in flight plus two queued, sized for a first block (with tail)
    S.prestage((size_t)(p.nsamp + p.maxshift) * p.nchans * b.elem, S.desc.max_inflight + 2);
    return MDSM_OK;
}

}  // namespace

extern "C" {

mdsm_status mdsm_server_create(const mdsm_server_desc *desc, mdsm_server **out)
{
    if (!desc || !out || desc->max_inflight <= 0 || desc->hbm_budget_bytes <= 0)
        return fail(MDSM_EINVAL, "server: bad description");
    if (desc->detector == 1 && (desc->nwidths < 1 || desc->nwidths > 9))
        return fail(MDSM_EINVAL, "server: boxcar widths must be 1..9 levels");
    mdsm_server *sv = new mdsm_server();
    Server &S = sv->s;
    S.desc = *desc;
    if (S.desc.cand_cap <= 0) S.desc.cand_cap = 4096;
    cudaGetDevice(&S.device);
    S.slots.resize(desc->max_inflight);
    for (auto &sl : S.slots) {
        if (cudaStreamCreateWithFlags(&sl.st, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess ||
            cudaHostAlloc((void **)&sl.h_cands, (size_t)S.desc.cand_cap * sizeof(mdsm_candidate),
                          0) != cudaSuccess ||
            cudaHostAlloc((void **)&sl.h_count, sizeof(long long), 0) != cudaSuccess) {
            mdsm_server_destroy(sv);
            return fail(MDSM_ECUDA, "server: stream/event/pinned allocation failed");
        }
    }
    S.worker = std::thread([&S] { S.run(); });
    *out = sv;
    return MDSM_OK;
}

mdsm_status mdsm_server_add_beam_brute(mdsm_server *sv, const mdsm_brute_desc *d, int *beam)
{
    if (!sv || !d || !beam) return fail(MDSM_EINVAL, "null argument");
    mdsm_plan *plan = nullptr;
    MDSM_TRY(mdsm_brute_plan_create(d, &plan));
    mdsm_status st = add_beam(sv, plan, beam);
    if (st != MDSM_OK) mdsm_plan_destroy(plan);
    return st;
}

mdsm_status mdsm_server_add_beam_subband(mdsm_server *sv, const mdsm_subband_desc *d, int *beam)
{
    if (!sv || !d || !beam) return fail(MDSM_EINVAL, "null argument");
    mdsm_plan *plan = nullptr;
    MDSM_TRY(mdsm_subband_plan_create(d, &plan));
    mdsm_status st = add_beam(sv, plan, beam);
    if (st != MDSM_OK) mdsm_plan_destroy(plan);
    return st;
}

mdsm_status mdsm_server_beam_info(mdsm_server *sv, int beam, mdsm_plan_info *info)
{
    if (!sv || beam < 0 || beam >= (int)sv->s.beams.size()) return fail(MDSM_EINVAL, "bad beam");
    return mdsm_plan_get_info(sv->s.beams[beam].plan, info);
}

mdsm_status mdsm_server_acquire(mdsm_server *sv, int beam, void **h_block, long long *cols)
{
    if (!sv || !h_block || !cols) return fail(MDSM_EINVAL, "null argument");
    Server &S = sv->s;
    if (beam < 0 || beam >= (int)S.beams.size()) return fail(MDSM_EINVAL, "bad beam");
    Beam &b = S.beams[beam];
    {
        std::lock_guard<std::mutex> lk(S.mu);
        if (S.fault != MDSM_OK) return fail(S.fault, "server stopped after a fault: " + S.fault_msg);
        if (b.acquired >= 0) return fail(MDSM_EINVAL, "beam already holds an acquired block");
    }
    const Plan &p = b.plan->p;
    const long long c = b.next_block == 0 ? (long long)p.nsamp + p.maxshift : p.nsamp;
    int idx = -1;
    MDSM_TRY(S.stage_get((size_t)c * p.nchans * b.elem, &idx));
    b.acquired = idx;
    *h_block = S.stage_ptr(idx);
    *cols = c;
    return MDSM_OK;
}

mdsm_status mdsm_server_commit(mdsm_server *sv, int beam, long long *ticket)
{
    if (!sv) return fail(MDSM_EINVAL, "null argument");
    Server &S = sv->s;
    if (beam < 0 || beam >= (int)S.beams.size()) return fail(MDSM_EINVAL, "bad beam");
    Beam &b = S.beams[beam];
    if (b.acquired < 0) return fail(MDSM_EINVAL, "commit without an acquired block");
    const Plan &p = b.plan->p;
    const long long cols = b.next_block == 0 ? (long long)p.nsamp + p.maxshift : p.nsamp;
    Pending job{beam, b.next_block, 0, now_s(), b.acquired, cols};
    b.acquired = -1;
    {
        std::lock_guard<std::mutex> lk(S.mu);
        job.ticket = S.tickets++;
        if (S.t_first == 0) S.t_first = job.t_submit;
        S.queue.push_back(job);
        b.next_block++;
    }
    S.cv.notify_all();
    if (ticket) *ticket = job.ticket;
    return MDSM_OK;
}

mdsm_status mdsm_server_submit(mdsm_server *sv, int beam, const void *h_block,
                               long long h_stride, long long *ticket)
{
    if (!sv || !h_block) return fail(MDSM_EINVAL, "null argument");
    Server &S = sv->s;
    if (beam < 0 || beam >= (int)S.beams.size()) return fail(MDSM_EINVAL, "bad beam");
    Beam &b = S.beams[beam];
    const Plan &p = b.plan->p;
    const long long need = b.next_block == 0 ? (long long)p.nsamp + p.maxshift : p.nsamp;
    if (h_stride < need) return fail(MDSM_ERANGE, "block row pitch smaller than its samples");
    void *stage = nullptr;
    long long cols = 0;
    MDSM_TRY(mdsm_server_acquire(sv, beam, &stage, &cols));
    // copy the new samples (row pitch cols) so the caller's buffer is free on return; large
    // blocks are copied by several threads, a band of channels each
    const size_t row = (size_t)cols * b.elem;
    const int nthr = (int)std::min<long long>(
        std::max(1u, std::min(16u, std::thread::hardware_concurrency())),
        std::max<long long>(1, (long long)row * p.nchans / (4ll << 20)));
    auto copy_rows = [&](int c0, int c1) {
        for (int c = c0; c < c1; ++c)
            std::memcpy(static_cast<char *>(stage) + (size_t)c * row,
                        static_cast<const char *>(h_block) + (size_t)c * h_stride * b.elem, row);
    };
    if (nthr <= 1) {
        copy_rows(0, p.nchans);
    } else {
        std::vector<std::thread> th;
        for (int i = 0; i < nthr; ++i)
            th.emplace_back(copy_rows, (int)((long long)p.nchans * i / nthr),
                            (int)((long long)p.nchans * (i + 1) / nthr));
        for (auto &t : th) t.join();
    }
    return mdsm_server_commit(sv, beam, ticket);
}

mdsm_status mdsm_server_poll(mdsm_server *sv, mdsm_block_result *res, mdsm_candidate *cands,
                             long long cap, int wait_ms)
{
    if (!sv || !res) return fail(MDSM_EINVAL, "null argument");
    Server &S = sv->s;
    std::unique_lock<std::mutex> lk(S.mu);
    if (S.results.empty() && wait_ms > 0)
        S.cv.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return !S.results.empty(); });
    if (S.results.empty()) {
        if (S.fault != MDSM_OK) return fail(S.fault, "server stopped after a fault: " + S.fault_msg);
        return MDSM_EAGAIN;
    }
    auto item = std::move(S.results.front());
    S.results.pop_front();
    *res = item.first;
    if (cands)
        for (long long i = 0; i < (long long)item.second.size() && i < cap; ++i)
            cands[i] = item.second[(size_t)i];
    return MDSM_OK;
}

mdsm_status mdsm_server_drain(mdsm_server *sv)
{
    if (!sv) return fail(MDSM_EINVAL, "null argument");
    Server &S = sv->s;
    std::unique_lock<std::mutex> lk(S.mu);
    for (;;) {
        bool idle = S.queue.empty();
        for (auto &sl : S.slots) idle &= !sl.busy;
        if (idle || S.fault != MDSM_OK) break;
        S.cv.wait_for(lk, std::chrono::milliseconds(2));
    }
    return S.fault == MDSM_OK ? MDSM_OK : fail(S.fault, "server fault: " + S.fault_msg);
}

mdsm_status mdsm_server_get_stats(mdsm_server *sv, mdsm_server_stats *out)
{
    if (!sv || !out) return fail(MDSM_EINVAL, "null argument");
    Server &S = sv->s;
    std::lock_guard<std::mutex> lk(S.mu);
    std::memset(out, 0, sizeof(*out));
    out->admitted = S.admitted;
    out->refused = S.refused;
    out->completed = S.completed;
    out->held_bytes = S.held_bytes;
    out->dm_trial_samples = S.units;
    out->wall_s = S.t_last > S.t_first ? S.t_last - S.t_first : 0;
    if (!S.latencies.empty()) {
        std::vector<double> v = S.latencies;
        std::sort(v.begin(), v.end());
        auto q = [&](double f) { return v[(size_t)std::min<double>(v.size() - 1, f * (v.size() - 1) + 0.5)]; };
        out->p50_latency_s = q(0.50);
        out->p99_latency_s = q(0.99);
        out->max_latency_s = v.back();
    }
    return MDSM_OK;
}

void mdsm_server_destroy(mdsm_server *sv)
{
    if (!sv) return;
    Server &S = sv->s;
    {
        std::lock_guard<std::mutex> lk(S.mu);
        S.stop = true;
    }
    S.cv.notify_all();
    if (S.worker.joinable()) S.worker.join();
    for (auto &sl : S.slots) {
        if (sl.st) cudaStreamSynchronize(sl.st);
        if (sl.st) cudaStreamDestroy(sl.st);
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.d_out) cudaFree(sl.d_out);
        if (sl.d_det) cudaFree(sl.d_det);
        if (sl.d_mom) cudaFree(sl.d_mom);
        if (sl.h_cands) cudaFreeHost(sl.h_cands);
        if (sl.h_count) cudaFreeHost(sl.h_count);
    }
    for (auto &b : S.beams) {
        for (int i = 0; i < 2; ++i)
            if (b.d_buf[i]) cudaFree(b.d_buf[i]);
        if (b.in_ready) cudaEventDestroy(b.in_ready);
        for (int i = 0; i < 2; ++i)
            if (b.buf_free[i]) cudaEventDestroy(b.buf_free[i]);
        mdsm_plan_destroy(b.plan);
    }
    for (auto &sb : S.pool)
        if (sb.h) cudaFreeHost(sb.h);
    delete sv;
}

}  // extern "C"
