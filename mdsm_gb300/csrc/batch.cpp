// batch.cpp -- the batched form: many beams of uneven block length, channel count and DM plan
// dedispersed by one persistent launch over the work list of all their tiles, optionally with
// RFI clipping before and a boxcar search after, the whole pass captured once in a CUDA graph
// and replayed.  An autotuner times the launch shapes on the caller's buffers and keeps the
// fastest; choices can be cached per beam geometry in a text file.
//
// The reference dedisperses one beam per process, one launch per DM segment, each launch
// followed by a synchronous copy (src/mdsm/dedispersion_thread.cu:69-94,220-243,332-355).
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "internal.h"

using namespace mdsm;

struct mdsm_batch_s {
    std::vector<mdsm_plan *> plans;
    BatchState st;
    unsigned *d_err = nullptr;
    bool buffers = false;
    int choice = 0;           // 0 persistent tile-major, 1 persistent DM-block-major, 2 per beam
    bool tuned = false;
    int launches = 0;
    // graph
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int graph_choice = -1;
    // fused stages
    bool clip = false;
    double k_chan = 0, k_spec = 0;
    bool detect = false;
    int nwidths = 9;
    double threshold = 6.0;
    long long cap = 4096;
    std::vector<void *> d_det;
    std::vector<mdsm_candidate *> h_cands;
    std::vector<long long *> h_count;
    std::vector<const void *> in;
    std::vector<long long> in_stride;
    std::vector<void *> out;
    std::vector<long long> out_stride;
};

namespace {

void drop_graph(mdsm_batch *b)
{
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    b->graph_choice = -1;
}

std::string geometry_key(const mdsm_batch *b)
{
    std::ostringstream k;
    for (mdsm_plan *p : b->plans) {
        const StageGeom &g = p->p.stages[0];
        k << g.nchans << "x" << g.ndms << "x" << g.nsamp << "k" << g.kernel << "s" << g.max_span
          << ";";
    }
    return k.str();
}

std::string cache_path()
{
    const char *e = std::getenv("MDSM_AUTOTUNE_CACHE");
    if (e && *e) return e;
    return std::string();
}

int cache_lookup(const std::string &key)
{
    const std::string path = cache_path();
    if (path.empty()) return -1;
    std::ifstream f(path);
    std::string line;
    while (std::getline(f, line)) {
        const size_t sp = line.rfind(' ');
        if (sp != std::string::npos && line.substr(0, sp) == key) return atoi(line.c_str() + sp + 1);
    }
    return -1;
}

void cache_store(const std::string &key, int choice)
{
    const std::string path = cache_path();
    if (path.empty()) return;
    std::ofstream f(path, std::ios::app);
    f << key << " " << choice << "\n";
}

// One pass (no graph): optional clip, dedispersion with `choice`, optional detection.
mdsm_status pass(mdsm_batch *b, int choice, cudaStream_t st)
{
    const size_t nb = b->plans.size();
    b->launches = 0;
    if (b->clip)
        for (size_t i = 0; i < nb; ++i) {
            const Plan &p = b->plans[i]->p;
            MDSM_TRY(rfi_clip(const_cast<void *>(b->in[i]), p.in_dtype, p.nchans, b->in_stride[i],
                              (long long)p.nsamp + p.maxshift, b->k_chan, b->k_spec, st));
            b->launches += (b->k_chan > 0) + (b->k_spec > 0);
        }
    if (choice != 2 && b->st.tile_major != (choice == 0 ? 1 : 0))
        MDSM_TRY(batch_set_buffers(b->st, b->in, b->in_stride, b->out, b->out_stride, b->d_err,
                                   choice == 0 ? 1 : 0));
    MDSM_TRY(batch_launch(b->st, choice == 2 ? 1 : 0, st, &b->launches));
    if (b->detect)
        for (size_t i = 0; i < nb; ++i) {
            const Plan &p = b->plans[i]->p;
            MDSM_TRY(boxcar_launch(b->out[i], p.out_dtype, p.ndms, p.nsamp, b->nwidths,
                                   b->threshold, b->d_det[i],
                                   boxcar_work_bytes(p.ndms, p.nsamp, b->cap), b->cap,
                                   b->h_cands[i], b->h_count[i], st));
            b->launches += 3;
        }
    return MDSM_OK;
}

}  // namespace

extern "C" {

mdsm_status mdsm_batch_create(mdsm_plan *const *plans, int nbeams, mdsm_batch **out)
{
    if (!plans || nbeams <= 0 || !out) return fail(MDSM_EINVAL, "batch: no plans");
    std::vector<BatchBeam> beams;
    for (int i = 0; i < nbeams; ++i) {
        if (!plans[i] || plans[i]->p.kind != 1)
            return fail(MDSM_EINVAL, "batch: plans must be brute-force plans");
        BatchBeam bb;
        bb.g = &plans[i]->p.stages[0];
        beams.push_back(bb);
    }
    mdsm_batch *b = new mdsm_batch();
    b->plans.assign(plans, plans + nbeams);
    mdsm_status st = batch_prepare(b->st, beams);
    if (st == MDSM_OK && cudaMalloc(&b->d_err, sizeof(unsigned)) != cudaSuccess)
        st = fail(MDSM_ENOMEM, "batch: error word");
    if (st == MDSM_OK) cudaMemset(b->d_err, 0, sizeof(unsigned));
    if (st != MDSM_OK) {
        mdsm_batch_destroy(b);
        return st;
    }
    *out = b;
    return MDSM_OK;
}

mdsm_status mdsm_batch_set_buffers(mdsm_batch *b, const void *const *d_in,
                                   const long long *in_stride, void *const *d_out,
                                   const long long *out_stride)
{
    if (!b || !d_in || !in_stride || !d_out || !out_stride) return fail(MDSM_EINVAL, "null argument");
    const size_t nb = b->plans.size();
    b->in.assign(d_in, d_in + nb);
    b->in_stride.assign(in_stride, in_stride + nb);
    b->out.assign(d_out, d_out + nb);
    b->out_stride.assign(out_stride, out_stride + nb);
    for (size_t i = 0; i < nb; ++i) {
        const Plan &p = b->plans[i]->p;
        if (in_stride[i] < (long long)p.nsamp + p.maxshift || out_stride[i] < p.nsamp)
            return fail(MDSM_ERANGE, "batch: beam " + std::to_string(i) + " row pitch too small");
    }
    drop_graph(b);
    b->buffers = true;
    return batch_set_buffers(b->st, b->in, b->in_stride, b->out, b->out_stride, b->d_err,
                             b->choice == 1 ? 0 : 1);
}

mdsm_status mdsm_batch_enable_clip(mdsm_batch *b, double k_chan, double k_spec)
{
    if (!b) return fail(MDSM_EINVAL, "null argument");
    b->clip = k_chan > 0 || k_spec > 0;
    b->k_chan = k_chan;
    b->k_spec = k_spec;
    drop_graph(b);
    return MDSM_OK;
}

mdsm_status mdsm_batch_enable_detect(mdsm_batch *b, int nwidths, double threshold,
                                     long long cap)
{
    if (!b || nwidths < 1 || nwidths > 9 || cap < 1) return fail(MDSM_EINVAL, "bad arguments");
    for (void *p : b->d_det) cudaFree(p);
    for (auto *p : b->h_cands) cudaFreeHost(p);
    for (auto *p : b->h_count) cudaFreeHost(p);
    b->d_det.clear();
    b->h_cands.clear();
    b->h_count.clear();
    for (mdsm_plan *pl : b->plans) {
        const Plan &p = pl->p;
        void *d = nullptr;
        mdsm_candidate *hc = nullptr;
        long long *hn = nullptr;
        MDSM_CUDA_TRY(cudaMalloc(&d, boxcar_work_bytes(p.ndms, p.nsamp, cap)));
        MDSM_CUDA_TRY(cudaHostAlloc((void **)&hc, (size_t)cap * sizeof(mdsm_candidate), 0));
        MDSM_CUDA_TRY(cudaHostAlloc((void **)&hn, sizeof(long long), 0));
        b->d_det.push_back(d);
        b->h_cands.push_back(hc);
        b->h_count.push_back(hn);
    }
    b->detect = true;
    b->nwidths = nwidths;
    b->threshold = threshold;
    b->cap = cap;
    drop_graph(b);
    return MDSM_OK;
}

// Times each launch shape twice on the registered buffers (after one warm pass) and keeps
// the fastest.  A cached choice for the same beam geometry is reused when
// MDSM_AUTOTUNE_CACHE names a file.
mdsm_status mdsm_batch_autotune(mdsm_batch *b, void *stream, int *choice)
{
    if (!b || !b->buffers) return fail(MDSM_ESTATE, "batch: set buffers first");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const std::string key = geometry_key(b);
    int best = cache_lookup(key);
    if (best < 0) {
        const bool clip = b->clip, det = b->detect;
        b->clip = b->detect = false;  // time the dedispersion launch shapes alone
        float best_ms = 1e30f;
        cudaEvent_t e0, e1;
        MDSM_CUDA_TRY(cudaEventCreate(&e0));
        MDSM_CUDA_TRY(cudaEventCreate(&e1));
        for (int c = 0; c < 3; ++c) {
            MDSM_TRY(pass(b, c, st));
            MDSM_CUDA_TRY(cudaEventRecord(e0, st));
            for (int r = 0; r < 2; ++r) MDSM_TRY(pass(b, c, st));
            MDSM_CUDA_TRY(cudaEventRecord(e1, st));
            MDSM_CUDA_TRY(cudaEventSynchronize(e1));
            float ms = 0;
            MDSM_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
            if (ms < best_ms) {
                best_ms = ms;
                best = c;
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        b->clip = clip;
        b->detect = det;
        cache_store(key, best);
    }
    b->choice = best;
    b->tuned = true;
    drop_graph(b);
    if (choice) *choice = best;
    return MDSM_OK;
}

// One pass over all beams.  use_graph: the first call runs the pass as ordinary launches and
// captures it into a CUDA graph; later calls replay the graph.
mdsm_status mdsm_batch_run(mdsm_batch *b, int use_graph, void *stream)
{
    if (!b || !b->buffers) return fail(MDSM_ESTATE, "batch: set buffers first");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (!use_graph) return pass(b, b->choice, st);
    if (!b->exec || b->graph_choice != b->choice) {
        // This call's pass runs as ordinary launches (which also sets kernel attributes); the
        // same pass is then captured, not executed, and replayed from the next call on.
        drop_graph(b);
        MDSM_TRY(pass(b, b->choice, st));
        MDSM_CUDA_TRY(cudaStreamSynchronize(st));
        cudaStream_t cs;
        MDSM_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        MDSM_CUDA_TRY(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
        const mdsm_status ps = pass(b, b->choice, cs);
        cudaGraph_t g = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(cs, &g);
        cudaStreamDestroy(cs);
        if (ps != MDSM_OK) {
            if (g) cudaGraphDestroy(g);
            return ps;
        }
        if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
        b->graph = g;
        MDSM_CUDA_TRY(cudaGraphInstantiate(&b->exec, b->graph, 0));
        b->graph_choice = b->choice;
        return MDSM_OK;
    }
    MDSM_CUDA_TRY(cudaGraphLaunch(b->exec, st));
    return MDSM_OK;
}

int mdsm_batch_last_launches(const mdsm_batch *b) { return b ? b->launches : 0; }

// Candidates of beam `beam` from the last pass (synchronises the stream first).
mdsm_status mdsm_batch_candidates(mdsm_batch *b, int beam, mdsm_candidate *out, long long cap,
                                  long long *ncand, void *stream)
{
    if (!b || !b->detect || beam < 0 || beam >= (int)b->plans.size() || !ncand)
        return fail(MDSM_EINVAL, "batch: detection not enabled or bad beam");
    MDSM_CUDA_TRY(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
    const long long n = *b->h_count[beam];
    const long long got = std::min<long long>(std::min<long long>(n, b->cap), cap);
    std::vector<mdsm_candidate> tmp(b->h_cands[beam], b->h_cands[beam] + std::min(n, b->cap));
    devcand_to_candidate(tmp.data(), (long long)tmp.size());
    std::sort(tmp.begin(), tmp.end(), [](const mdsm_candidate &x, const mdsm_candidate &y) {
        return x.dm_idx != y.dm_idx ? x.dm_idx < y.dm_idx : x.sample < y.sample;
    });
    for (long long i = 0; i < got; ++i) out[i] = tmp[(size_t)i];
    *ncand = n;
    return MDSM_OK;
}

void mdsm_batch_destroy(mdsm_batch *b)
{
    if (!b) return;
    drop_graph(b);
    batch_release(b->st);
    for (void *p : b->d_det) cudaFree(p);
    for (auto *p : b->h_cands) cudaFreeHost(p);
    for (auto *p : b->h_count) cudaFreeHost(p);
    if (b->d_err) cudaFree(b->d_err);
    delete b;
}

}  // extern "C"
