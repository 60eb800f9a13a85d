// batch.cpp -- the batched form: many beams of uneven block length, channel count and DM plan
// in one persistent launch, the whole pass captured once in a CUDA graph and replayed.
//
// Fused form (every beam a uint8 brute-force plan with int32 output, boxcar widths 1..256 if
// detection is on): RFI clip, dedispersion and boxcar search in ONE persistent launch
// (k_batch_fused) over four work lists tied by per-beam completion counts, with the rows'
// statistics folded into the dedispersion store.  The autotuner times its tile shapes (DM
// trials per block x samples per tile x compute warps) and item orders on the caller's
// buffers and keeps the fastest.
// Otherwise: clip launches, one persistent dedispersion launch over the packed beams' tiles
// (one launch per beam for the rest) and per-beam search launches, in one graph; the autotuner
// picks the dedispersion launch shape.  Choices can be cached per beam geometry in a file.
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

// The fused launch's tables, work lists and buffers for one tile shape and item order.
struct FusedRun {
    int shape = -1, order = 0;
    bool clip = false, detect = false;
    std::vector<StageGeom> geoms;      // per beam, this shape's tables (device copies owned)
    int rawcap = 0, ps = 0, n_dd = 0;
    FusedArgs f{};
    void *d_kargs = nullptr, *d_fb = nullptr, *d_dd = nullptr, *d_cc = nullptr, *d_cs = nullptr,
         *d_bx = nullptr;
    unsigned *d_sync = nullptr;        // 4 work counters, then 3 completion counts per beam
    size_t sync_bytes = 0;
    unsigned long long *d_mom = nullptr;  // all beams' row moments
    size_t mom_bytes = 0;
    DevCand *d_cands = nullptr;        // [beam][cap]
    unsigned long long *d_counts = nullptr;
    std::vector<size_t> mom_off;       // per beam, its rows' moments in d_mom
    std::vector<int> rest;             // beams whose staging does not fit this shape: their own
                                       // clip, dedispersion and search launches after the fused one
};

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
    std::vector<std::pair<int, float>> tune_ms;  // the last tuning: (choice, ms per pass)
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
    // fused form
    bool fusable = false;      // every beam a uint8 brute-force plan with int32 output
    FusedRun fz;
    bool fz_dirty = true;
};

namespace {

void fused_free(FusedRun &z)
{
    for (StageGeom &g : z.geoms) free_stage(g);
    for (void *p : {z.d_kargs, z.d_fb, z.d_dd, z.d_cc, z.d_cs, z.d_bx})
        if (p) cudaFree(p);
    if (z.d_sync) cudaFree(z.d_sync);
    if (z.d_mom) cudaFree(z.d_mom);
    if (z.d_cands) cudaFree(z.d_cands);
    if (z.d_counts) cudaFree(z.d_counts);
    z = FusedRun();
}

template <typename T>
mdsm_status upload(const std::vector<T> &v, void **d)
{
    if (*d) cudaFree(*d);
    *d = nullptr;
    MDSM_CUDA_TRY(cudaMalloc(d, std::max<size_t>(1, v.size()) * sizeof(T)));
    if (!v.empty())
        MDSM_CUDA_TRY(cudaMemcpy(*d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return MDSM_OK;
}

// Tables and work lists of the fused launch for tile shape `shape` and item order `order`
// (0: a beam's DM blocks of one time tile adjacent, 1: a DM block's time tiles adjacent), with
// the batch's buffers, clip and detection settings.
mdsm_status fused_build(mdsm_batch *b, int shape, int order, bool clip, bool detect)
{
    fused_free(b->fz);
    FusedRun &z = b->fz;
    z.shape = shape;
    z.order = order;
    z.clip = clip;
    z.detect = detect;
    const size_t nb = b->plans.size();
    z.geoms.resize(nb);
    std::vector<char> fused(nb, 0);
    for (size_t i = 0; i < nb; ++i) {
        const Plan &p = b->plans[i]->p;
        StageGeom g = p.stages[0];  // geometry; the tables are rebuilt for this shape
        g.rel.clear();
        g.sminspan.clear();
        g.d_rel = nullptr;
        g.d_sminspan = nullptr;
        z.geoms[i] = g;
        // A beam whose staging does not fit this shape (or whose last tile would read past the
        // caller's buffer, which holds what the plan's own tile shape reads: mdsm_plan_info
        // in_bytes) runs on its own launches instead.
        if (fused_tables(shape, z.geoms[i], p.S) != MDSM_OK ||
            stage_in_bytes(z.geoms[i], b->in_stride[i], 0) >
                stage_in_bytes(p.stages[0], b->in_stride[i], 0)) {
            free_stage(z.geoms[i]);
            z.rest.push_back((int)i);
            continue;
        }
        fused[i] = 1;
        z.rawcap = std::max(z.rawcap, z.geoms[i].rowcap);
        z.ps = std::max(z.ps, z.geoms[i].ps);
    }
    if (z.rest.size() == nb)
        return fail(MDSM_EINVAL, "fused batch: no beam's staging fits this tile shape");
    // (each beam keeps its own phase stride and offsets: the launch expands a beam's chunks
    // with its stride; the shared-memory buffers are sized for the widest)
    // moments and candidates
    std::vector<size_t> &mom_off = z.mom_off;
    mom_off.assign(nb, 0);
    for (size_t i = 0; i < nb; ++i) {
        mom_off[i] = z.mom_bytes / sizeof(unsigned long long);
        z.mom_bytes += (size_t)b->plans[i]->p.ndms * 3 * sizeof(unsigned long long);
    }
    MDSM_CUDA_TRY(cudaMalloc(&z.d_mom, std::max<size_t>(z.mom_bytes, 8)));
    MDSM_CUDA_TRY(cudaMalloc(&z.d_cands, nb * (size_t)b->cap * sizeof(DevCand)));
    MDSM_CUDA_TRY(cudaMalloc(&z.d_counts, nb * sizeof(unsigned long long)));
    z.sync_bytes = (4 + 3 * nb) * sizeof(unsigned);
    MDSM_CUDA_TRY(cudaMalloc(&z.d_sync, z.sync_bytes));
    // work lists; beams with more channels first
    std::vector<int> beams(nb);
    for (size_t i = 0; i < nb; ++i) beams[i] = (int)i;
    std::stable_sort(beams.begin(), beams.end(), [&](int x, int y) {
        return b->plans[x]->p.nchans > b->plans[y]->p.nchans;
    });
    std::vector<KArgs> ka(nb);
    std::vector<FusedBeam> fb(nb);
    std::vector<int4> dd, bx;
    std::vector<int2> cc, cs;
    const int kFusedBoxTile = fused_box_tile(), tpc = 16;  // search items: runs of 16 tiles
    for (int i : beams) {
        if (!fused[i]) continue;
        const Plan &p = b->plans[i]->p;
        const StageGeom &g = z.geoms[i];
        unsigned char *in = static_cast<unsigned char *>(const_cast<void *>(b->in[i]));
        int32_t *out = static_cast<int32_t *>(b->out[i]);
        unsigned long long *mom = detect ? z.d_mom + mom_off[i] : nullptr;  // (for the search)
        ka[i] = fused_kargs(g, g.d_rel, in, b->in_stride[i], out, b->out_stride[i], z.rawcap,
                            g.ps, mom, b->d_err);
        const long long ncols = (long long)p.nsamp + p.maxshift;
        const int ntiles = (p.nsamp + g.T - 1) / g.T;
        const size_t dd0 = dd.size();
        if (order == 0) {
            for (int t = 0; t < ntiles; ++t)
                for (int k = 0; k < g.nblk; ++k) dd.push_back(make_int4(i, k, t, 0));
        } else {
            for (int k = 0; k < g.nblk; ++k)
                for (int t = 0; t < ntiles; ++t) dd.push_back(make_int4(i, k, t, 0));
        }
        FusedBeam &B = fb[i];
        B.in = in;
        B.in_stride = b->in_stride[i];
        B.ncols = ncols;
        B.nchans = p.nchans;
        B.ndms = p.ndms;
        B.nsamp = p.nsamp;
        B.nspec_items =
            clip ? (unsigned)((ncols + kFusedSpecColsHost - 1) / kFusedSpecColsHost) : 0u;
        B.ndd_done = (unsigned)(dd.size() - dd0);  // one count per dedispersion item
        B.out = out;
        B.out_stride = b->out_stride[i];
        B.mom = mom;
        B.cands = z.d_cands + (size_t)i * (size_t)b->cap;
        B.count = z.d_counts + i;
        if (clip && b->k_chan > 0)
            for (int c = 0; c < p.nchans; ++c) cc.push_back(make_int2(i, c));
        if (clip)
            for (long long c0 = 0; c0 < ncols; c0 += kFusedSpecColsHost)
                cs.push_back(make_int2(i, (int)c0));
        if (detect) {
            const int nbt = (p.nsamp + kFusedBoxTile - 1) / kFusedBoxTile;
            for (int d = 0; d < p.ndms; ++d)
                for (int t0 = 0; t0 < nbt; t0 += tpc)
                    bx.push_back(make_int4(i, d, t0, std::min(nbt, t0 + tpc)));
        }
    }
    if (dd.size() > 0x7fffffffULL || bx.size() > 0x7fffffffULL || cc.size() > 0x7fffffffULL)
        return fail(MDSM_EINVAL, "fused batch: work lists too long");
    z.n_dd = (int)dd.size();
    MDSM_TRY(upload(ka, &z.d_kargs));
    MDSM_TRY(upload(fb, &z.d_fb));
    MDSM_TRY(upload(dd, &z.d_dd));
    MDSM_TRY(upload(cc, &z.d_cc));
    MDSM_TRY(upload(cs, &z.d_cs));
    MDSM_TRY(upload(bx, &z.d_bx));
    FusedArgs &f = z.f;
    f.fb = static_cast<const FusedBeam *>(z.d_fb);
    f.cc_items = static_cast<const int2 *>(z.d_cc);
    f.cs_items = static_cast<const int2 *>(z.d_cs);
    f.bx_items = static_cast<const int4 *>(z.d_bx);
    f.n_cc = (int)cc.size();
    f.n_cs = (int)cs.size();
    f.n_bx = (int)bx.size();
    f.counters = z.d_sync;
    f.done = z.d_sync + 4;
    f.k_chan = clip ? b->k_chan : 0.0;
    f.k_spec = clip ? b->k_spec : 0.0;
    f.threshold = b->threshold;
    f.cap = b->cap;
    f.err = b->d_err;
    return MDSM_OK;
}

// One fused pass: counters and moments zeroed, the launch, the candidates' copies; then each
// beam left out of the fused launch on its own launches (clip, its plan's dedispersion with
// the moments folded, search).
mdsm_status fused_pass(mdsm_batch *b, cudaStream_t st)
{
    FusedRun &z = b->fz;
    MDSM_CUDA_TRY(cudaMemsetAsync(z.d_sync, 0, z.sync_bytes, st));
    MDSM_CUDA_TRY(cudaMemsetAsync(z.d_mom, 0, z.mom_bytes, st));
    MDSM_CUDA_TRY(
        cudaMemsetAsync(z.d_counts, 0, b->plans.size() * sizeof(unsigned long long), st));
    MDSM_TRY(fused_launch(z.shape, z.f, static_cast<const KArgs *>(z.d_kargs),
                          static_cast<const int4 *>(z.d_dd), z.n_dd, z.rawcap, z.ps, st));
    b->launches = 1;
    std::vector<char> is_rest(b->plans.size(), 0);
    for (int i : z.rest) {
        is_rest[(size_t)i] = 1;
        const Plan &p = b->plans[(size_t)i]->p;
        const StageGeom &g = p.stages[0];
        if (z.clip) {
            MDSM_TRY(rfi_clip(const_cast<void *>(b->in[(size_t)i]), p.in_dtype, p.nchans,
                              b->in_stride[(size_t)i], (long long)p.nsamp + p.maxshift, b->k_chan,
                              b->k_spec, st));
            b->launches += (b->k_chan > 0) + (b->k_spec > 0);
        }
        unsigned long long *mom =
            z.detect && stage_folds_moments(g) ? z.d_mom + z.mom_off[(size_t)i] : nullptr;
        MDSM_TRY(launch_stage(g, b->in[(size_t)i], b->in_stride[(size_t)i], 0, b->out[(size_t)i],
                              b->out_stride[(size_t)i], 0, b->d_err, st, &b->launches, -1, mom,
                              p.ndms));
        if (z.detect) {
            MDSM_TRY(boxcar_launch(b->out[(size_t)i], p.out_dtype, p.ndms, p.nsamp, b->nwidths,
                                   b->threshold, b->d_det[(size_t)i],
                                   boxcar_work_bytes(p.ndms, p.nsamp, b->cap), b->cap,
                                   b->h_cands[(size_t)i], b->h_count[(size_t)i], st, mom));
            b->launches += p.out_dtype == MDSM_OUT_F32 ? 3 : 2;  // statistics (2 or 1), search
        }
    }
    if (z.detect)
        for (size_t i = 0; i < b->plans.size(); ++i) {
            if (is_rest[i]) continue;
            static_assert(sizeof(DevCand) == sizeof(mdsm_candidate), "record sizes differ");
            MDSM_CUDA_TRY(cudaMemcpyAsync(b->h_count[i], z.d_counts + i, sizeof(long long),
                                          cudaMemcpyDeviceToHost, st));
            MDSM_CUDA_TRY(cudaMemcpyAsync(b->h_cands[i], z.d_cands + i * (size_t)b->cap,
                                          (size_t)b->cap * sizeof(DevCand),
                                          cudaMemcpyDeviceToHost, st));
        }
    return MDSM_OK;
}

bool fused_wanted(const mdsm_batch *b) { return b->fusable && (!b->detect || b->nwidths == 9); }

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

// Autotuner choices: 0-2 the unfused dedispersion launch shapes (persistent tile-major,
// persistent DM-block-major, one launch per beam); 10 + 2 shape + order the fused launch.
constexpr int kFusedChoice0 = 10;

// One pass (no graph): optional clip, dedispersion with `choice`, optional detection.
mdsm_status pass(mdsm_batch *b, int choice, cudaStream_t st)
{
    const size_t nb = b->plans.size();
    b->launches = 0;
    if (choice >= kFusedChoice0) {
        const int shape = (choice - kFusedChoice0) / 2, order = (choice - kFusedChoice0) % 2;
        FusedRun &z = b->fz;
        if (b->fz_dirty || z.shape != shape || z.order != order || z.clip != b->clip ||
            z.detect != b->detect) {
            if (fused_build(b, shape, order, b->clip, b->detect) != MDSM_OK) {
                // a beam's staging does not fit the fused launch: the unfused pass from now on
                fused_free(b->fz);
                b->fusable = false;
                b->choice = choice = 0;
                goto unfused;
            }
            b->fz_dirty = false;
        }
        return fused_pass(b, st);
    }
unfused:
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
    b->fusable = true;
    for (int i = 0; i < nbeams; ++i) {
        const Plan &p = plans[i]->p;
        if (p.in_dtype != MDSM_U8 || p.out_dtype != MDSM_OUT_I32 || p.S.empty())
            b->fusable = false;
    }
    b->choice = b->fusable ? kFusedChoice0 : 0;
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
    b->fz_dirty = true;
    return batch_set_buffers(b->st, b->in, b->in_stride, b->out, b->out_stride, b->d_err,
                             b->choice == 1 ? 0 : 1);
}

mdsm_status mdsm_batch_enable_clip(mdsm_batch *b, double k_chan, double k_spec)
{
    if (!b) return fail(MDSM_EINVAL, "null argument");
    b->clip = k_chan > 0 || k_spec > 0;
    b->k_chan = k_chan;
    b->k_spec = k_spec;
    b->fz_dirty = true;
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
    b->fz_dirty = true;
    if (b->choice >= kFusedChoice0 && !fused_wanted(b)) b->choice = 0;
    drop_graph(b);
    return MDSM_OK;
}

// Times each candidate twice on the registered buffers (after one warm pass) and keeps the
// fastest: the fused launch's tile shapes and item orders where the beams allow it, and the
// unfused passes (the persistent dedispersion launch in either item order, or one launch per
// beam with each plan's own tile shape, each followed by the search launches).  Every
// candidate does the same work: the clip is left out of the timed passes (it changes the
// input in place); the search stays in.  A cached choice for the same beam geometry is
// reused when MDSM_AUTOTUNE_CACHE names a file.
mdsm_status mdsm_batch_autotune(mdsm_batch *b, void *stream, int *choice)
{
    if (!b || !b->buffers) return fail(MDSM_ESTATE, "batch: set buffers first");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const bool fused = fused_wanted(b);
    // (the beams' geometry decides whether they fit the fused launch; the search settings
    // decide whether it is wanted)
    const std::string key =
        geometry_key(b) + (b->detect ? "det" + std::to_string(b->nwidths) : "");
    int best = cache_lookup(key);
    if (best < 0) {
        const bool clip = b->clip;
        const bool det = b->detect;
        b->clip = false;
        float best_ms = 1e30f;
        cudaEvent_t e0, e1;
        MDSM_CUDA_TRY(cudaEventCreate(&e0));
        MDSM_CUDA_TRY(cudaEventCreate(&e1));
        std::vector<int> cands;
        if (fused)
            for (int c = 0; c < 2 * fused_num_shapes(); ++c) cands.push_back(kFusedChoice0 + c);
        cands.push_back(0);
        cands.push_back(1);
        cands.push_back(2);
        std::string why;
        b->tune_ms.clear();
        for (int c : cands) {
            if (c >= kFusedChoice0 && fused_build(b, (c - kFusedChoice0) / 2,
                                                  (c - kFusedChoice0) % 2, false,
                                                  b->detect) != MDSM_OK) {
                why = mdsm_last_error();  // a beam's staging does not fit this shape
                continue;
            }
            if (c >= kFusedChoice0) b->fz_dirty = false;
            MDSM_TRY(pass(b, c, st));
            MDSM_CUDA_TRY(cudaEventRecord(e0, st));
            for (int r = 0; r < 2; ++r) MDSM_TRY(pass(b, c, st));
            MDSM_CUDA_TRY(cudaEventRecord(e1, st));
            MDSM_CUDA_TRY(cudaEventSynchronize(e1));
            float ms = 0;
            MDSM_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
            b->tune_ms.emplace_back(c, ms / 2);
            if (ms < best_ms) {
                best_ms = ms;
                best = c;
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        b->clip = clip;
        b->detect = det;
        if (best < 0)
            return fail(MDSM_EINVAL, "batch: no launch shape fits these beams (" + why + ")");
        if (best < kFusedChoice0) fused_free(b->fz);
        cache_store(key, best);
    }
    b->choice = best;
    b->tuned = true;
    b->fz_dirty = true;
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

mdsm_status mdsm_batch_autotune_times(const mdsm_batch *b, int *choices, float *ms, int cap,
                                      int *n)
{
    if (!b || !n || (cap > 0 && (!choices || !ms))) return fail(MDSM_EINVAL, "null argument");
    *n = (int)b->tune_ms.size();
    for (int i = 0; i < std::min(cap, *n); ++i) {
        choices[i] = b->tune_ms[(size_t)i].first;
        ms[i] = b->tune_ms[(size_t)i].second;
    }
    return MDSM_OK;
}

mdsm_status mdsm_batch_choice_info(int choice, int *fused, int *dm_block, int *time_tile,
                                   int *warps, int *order)
{
    if (!fused || !dm_block || !time_tile || !warps || !order)
        return fail(MDSM_EINVAL, "null argument");
    if (choice >= kFusedChoice0 && choice < kFusedChoice0 + 2 * fused_num_shapes()) {
        const FusedShapeInfo si = fused_shape_info((choice - kFusedChoice0) / 2);
        *fused = 1;
        *dm_block = si.dm_block;
        *time_tile = si.time_tile;
        *warps = si.compute_warps;
        *order = (choice - kFusedChoice0) % 2;
        return MDSM_OK;
    }
    if (choice < 0 || choice > 2) return fail(MDSM_EINVAL, "no such choice");
    *fused = 0;
    *dm_block = *time_tile = *warps = 0;
    *order = choice;
    return MDSM_OK;
}

// Candidates of beam `beam` from the last pass (synchronises the stream first).
mdsm_status mdsm_batch_candidates(mdsm_batch *b, int beam, mdsm_candidate *out, long long cap,
                                  long long *ncand, void *stream)
{
    if (!b || !b->detect || beam < 0 || beam >= (int)b->plans.size() || !ncand)
        return fail(MDSM_EINVAL, "batch: detection not enabled or bad beam");
    MDSM_CUDA_TRY(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
    const long long n = *b->h_count[beam];
    if ((unsigned long long)n & kBoxCountLate)
        return fail(MDSM_ETIMEOUT, "batch: a staging wait of the search ran out");
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
    fused_free(b->fz);
    batch_release(b->st);
    for (void *p : b->d_det) cudaFree(p);
    for (auto *p : b->h_cands) cudaFreeHost(p);
    for (auto *p : b->h_count) cudaFreeHost(p);
    if (b->d_err) cudaFree(b->d_err);
    delete b;
}

}  // extern "C"
