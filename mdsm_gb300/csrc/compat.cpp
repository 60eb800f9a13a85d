// compat.cpp -- the reference's stage interface (src/mdsm/dedispersion_manager.h:7-12) over the
// GB300 library, with C linkage; include/dedispersion_manager.h gives it the reference's C++
// names and default arguments.
//
// Contract kept from the reference (src/mdsm/dedispersion_manager.cpp:269-501,
// src/mdsm/dedispersion_thread.cu:246-401, src/mdsm/dedispersion_output.cpp:216-356):
//  * one global instance; processSurveyParameters -> initialiseMDSM -> (next_chunk,
//    start_processing)* -> tearDownMDSM from one caller thread;
//  * initialiseMDSM returns the library-owned input buffer, channel-major
//    [nchans][nsamp + maxshift] float; block 0 fills every column, later blocks fill columns
//    [maxshift, maxshift + nsamp) and the library supplies the previous block's last maxshift
//    samples itself;
//  * next_chunk returns the dedispersed output of the previous block ([ndms][nsamp] float,
//    valid until the next next_chunk) or NULL on the first call; `samples` is that block's
//    sample count;
//  * start_processing returns once the input buffer may be refilled; data_read == 0 stops,
//    and the second start_processing(0) returns 0;
//  * candidates of every block are written as text "time, dm, snr" to the reference's output
//    files (dedispersion_output.cpp:194-196,233-302).
// GB300 design: one worker thread runs a block's dedispersion, detection and copy-out while
// the caller reads the next block (the reference's dedispersion and output threads), joined
// by the next call instead of barriers.  The overlap tail stays on the device and is moved
// there with one device-to-device copy (no host memcpy per channel), only the new samples
// cross the host link, the input/output buffers are pinned, and detection runs on the
// device.  Errors set mdsm_last_error() and return NULL / 0 instead of exit(0).
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "internal.h"

namespace mdsm {

namespace {

// ------------------------------------------------------------------------------------------
// a small XML reader for the observation file schema
// ------------------------------------------------------------------------------------------
struct XNode {
    std::string tag;
    std::vector<std::pair<std::string, std::string>> attrs;
    std::string text;
    std::vector<XNode> kids;
    const char *attr(const char *name) const
    {
        for (auto &a : attrs)
            if (strcasecmp(a.first.c_str(), name) == 0) return a.second.c_str();
        return nullptr;
    }
};

struct XParser {
    const std::string &s;
    size_t i = 0;
    bool ok = true;
    explicit XParser(const std::string &src) : s(src) {}
    void ws()
    {
        while (i < s.size() && isspace((unsigned char)s[i])) ++i;
    }
    void skip_misc()
    {
        for (;;) {
            ws();
            if (s.compare(i, 4, "<!--") == 0) {
                size_t e = s.find("-->", i + 4);
                i = e == std::string::npos ? s.size() : e + 3;
            } else if (s.compare(i, 2, "<?") == 0 || s.compare(i, 2, "<!") == 0) {
                size_t e = s.find('>', i);
                i = e == std::string::npos ? s.size() : e + 1;
            } else {
                return;
            }
        }
    }
    std::string name()
    {
        size_t b = i;
        while (i < s.size() && (isalnum((unsigned char)s[i]) || s[i] == '_' || s[i] == '-' ||
                                s[i] == ':' || s[i] == '.'))
            ++i;
        return s.substr(b, i - b);
    }
    bool element(XNode &n)
    {
        skip_misc();
        if (i >= s.size() || s[i] != '<') return false;
        ++i;
        n.tag = name();
        if (n.tag.empty()) return ok = false;
        for (;;) {
            ws();
            if (i >= s.size()) return ok = false;
            if (s[i] == '/') {
                if (i + 1 < s.size() && s[i + 1] == '>') {
                    i += 2;
                    return true;
                }
                return ok = false;
            }
            if (s[i] == '>') {
                ++i;
                break;
            }
            std::string an = name();
            ws();
            if (an.empty() || i >= s.size() || s[i] != '=') return ok = false;
            ++i;
            ws();
            if (i >= s.size() || (s[i] != '"' && s[i] != '\'')) return ok = false;
            char q = s[i++];
            size_t e = s.find(q, i);
            if (e == std::string::npos) return ok = false;
            n.attrs.emplace_back(an, s.substr(i, e - i));
            i = e + 1;
        }
        for (;;) {
            skip_misc();
            if (i >= s.size()) return ok = false;
            if (s.compare(i, 2, "</") == 0) {
                i += 2;
                name();
                ws();
                if (i < s.size() && s[i] == '>') ++i;
                return true;
            }
            if (s[i] == '<') {
                XNode k;
                if (!element(k)) return false;
                n.kids.push_back(std::move(k));
            } else {
                size_t e = s.find('<', i);
                if (e == std::string::npos) return ok = false;
                n.text += s.substr(i, e - i);
                i = e;
            }
        }
    }
};

float fattr(const XNode &n, const char *a, float dflt)
{
    const char *v = n.attr(a);
    return v ? (float)atof(v) : dflt;
}
unsigned uattr(const XNode &n, const char *a, unsigned dflt)
{
    const char *v = n.attr(a);
    return v ? (unsigned)strtoul(v, nullptr, 10) : dflt;
}

// ------------------------------------------------------------------------------------------
// the single instance
// ------------------------------------------------------------------------------------------
struct Instance {
    bool live = false;
    SURVEY *survey = nullptr;
    mdsm_plan *plan = nullptr;
    cudaStream_t st = nullptr;
    float *h_in = nullptr;            // pinned [nchans][nsamp+maxshift]
    float *h_out[2] = {nullptr, nullptr};
    void *d_in[2] = {nullptr, nullptr};
    size_t d_in_bytes = 0;
    void *d_out = nullptr;
    long long stride = 0;             // device row pitch (elements, 16-byte rows)
    long long hstride = 0;            // host row pitch: nsamp + maxshift, as callers index it
    long long blocks = 0;             // blocks processed
    unsigned pending_read = 0;        // data_read given to the last next_chunk
    unsigned prev_read = 0;           // samples of the last processed block
    long long returned = 0;           // blocks count when next_chunk last returned output
    bool stopping = false, stopped_once = false;
    double ts = 0, rate = 0;
    const float *cmean = nullptr, *crms = nullptr;  // caller noise statistics of the block
    std::vector<mdsm_candidate> cands;  // candidates of the last processed block
    FILE *fp = nullptr;
    long long written = 0;
    // 8-bit path: a uint8 plan of the same geometry, run when a block's floats are all
    // integers 0..255 (then every partial sum is an integer below 2^24, exact in float in any
    // order, so the packed kernels give the float kernels' output bit for bit)
    mdsm_plan *plan8 = nullptr;
    void *d_in8 = nullptr;
    size_t d_in8_bytes = 0;
    long long stride8 = 0;
    unsigned *d_flag = nullptr, *h_flag = nullptr;
    long long blocks8 = 0;
    // The block after its copies runs on a worker thread (g_worker), as the reference's
    // dedispersion and output threads do, so the caller reads the next block meanwhile;
    // next_chunk, start_processing and tearDown wait for it.
    mdsm_status wstatus = MDSM_OK;
    std::string werror;
};

// One block handed to the worker: what next_chunk gave for it, captured when it is submitted.
struct Job {
    unsigned data_read = 0;
    int cur = 0, device = 0;
    bool eight = false;
    double ts = 0, rate = 0;
    std::vector<float> mean, rms;  // caller noise statistics (empty: the detector's own)
};

Instance g;

// The worker of the block in flight; joined at exit too, if a caller never tears down.
struct Worker {
    std::thread t;
    ~Worker()
    {
        if (t.joinable()) t.join();
    }
};
Worker g_worker;

// Candidate lines as the reference's detectors print them: "time, DM, snr" (process_brute
// with its own statistics, dedispersion_output.cpp:202-204; process_subband, :114-127, whose
// time counts samples of the pass's downsample factor, held in the candidate's width), or
// with caller statistics "time, DM, snr, mean, rms" (process_brute, :205-208).
void write_candidates(const std::vector<mdsm_candidate> &c, long long nc, double ts, double rate,
                      int spc, const float *cmean, const float *crms)
{
    SURVEY *s = g.survey;
    if (!g.fp || (!s->single_file_mode && g.written == 0)) {
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
        if (g.fp) fclose(g.fp);
        g.fp = fopen(path, "w");
    }
    if (!g.fp) return;
    std::vector<float> dmv(g.plan->p.ndms);
    mdsm_plan_dm_values(g.plan, dmv.data());
    const bool with_stats = g.plan->p.kind == 1 && cmean;
    for (long long i = 0; i < nc && i < (long long)c.size(); ++i) {
        const double t = ts + (double)c[i].sample * rate * (double)std::max(1, c[i].width);
        if (with_stats)
            fprintf(g.fp, "%lf, %f, %f, %f, %f  \n", t, dmv[c[i].dm_idx], c[i].snr,
                    cmean[c[i].sample / spc], crms[c[i].sample / spc]);
        else
            fprintf(g.fp, "%lf, %f, %f\n", t, dmv[c[i].dm_idx], c[i].snr);
    }
    fflush(g.fp);
    if (!s->single_file_mode) {
        g.written += g.prev_read;
        if (g.written * rate > s->secs_per_file) {
            g.written = 0;
            fclose(g.fp);
            g.fp = nullptr;
        }
    }
}

void release()
{
    if (g_worker.t.joinable()) g_worker.t.join();
    if (g.fp) fclose(g.fp);
    if (g.plan) mdsm_plan_destroy(g.plan);
    if (g.plan8) mdsm_plan_destroy(g.plan8);
    if (g.d_in8) cudaFree(g.d_in8);
    if (g.d_flag) cudaFree(g.d_flag);
    if (g.h_flag) cudaFreeHost(g.h_flag);
    if (g.h_in) cudaFreeHost(g.h_in);
    for (int i = 0; i < 2; ++i) {
        if (g.h_out[i]) cudaFreeHost(g.h_out[i]);
        if (g.d_in[i]) cudaFree(g.d_in[i]);
    }
    if (g.d_out) cudaFree(g.d_out);
    if (g.st) cudaStreamDestroy(g.st);
    g = Instance();
}

// The 8-bit path where it gives the float plan's output exactly: float sums of integers
// 0..255 over at most 65793 channels stay below 2^24 (exact), and passes without
// downsampling (a downsampled pass averages samples into fractions).  Set-up failures leave
// the float path alone.
void setup_8bit(const SURVEY *s)
{
    const Plan &p = g.plan->p;
    if ((long long)p.nchans * 255 >= (1LL << 24)) return;
    mdsm_status st;
    if (s->useBruteForce) {
        mdsm_segment seg{s->lowdm, s->dmstep, (int)s->tdms};
        mdsm_brute_desc d;
        memset(&d, 0, sizeof d);
        d.nchans = (int)s->nchans;
        d.fch1 = s->fch1;
        d.foff = s->foff;
        d.tsamp = s->tsamp;
        d.nsamp = (int)s->nsamp;
        d.segs = &seg;
        d.nsegs = 1;
        d.shift_mode = s->useL1Cache ? MDSM_SHIFT_L1 : MDSM_SHIFT_OPT;
        d.in_dtype = MDSM_U8;
        d.out_dtype = MDSM_OUT_F32;
        st = mdsm_brute_plan_create(&d, &g.plan8);
    } else {
        for (unsigned i = 0; i < s->num_passes; ++i)
            if (s->pass_parameters[i].binsize > 1) return;
        mdsm_subband_desc d;
        memset(&d, 0, sizeof d);
        d.nchans = (int)s->nchans;
        d.fch1 = s->fch1;
        d.foff = s->foff;
        d.tsamp = s->tsamp;
        d.nsamp = (int)s->nsamp;
        d.nsubs = (int)s->nsubs;
        d.passes = s->pass_parameters;
        d.npasses = (int)s->num_passes;
        d.use_fma = 1;
        d.in_dtype = MDSM_U8;
        d.out_dtype = MDSM_OUT_F32;
        st = mdsm_subband_plan_create(&d, &g.plan8);
    }
    if (st != MDSM_OK) {
        g.plan8 = nullptr;
        return;
    }
    const Plan &q = g.plan8->p;
    long long need = 0;
    const bool same = q.nchans == p.nchans && q.ndms == p.ndms && q.nsamp == p.nsamp &&
                      q.maxshift == p.maxshift && q.S == p.S && q.S1 == p.S1 && q.S2 == p.S2;
    if (!same || plan_in_requirements(q, q.in_stride, &need) != MDSM_OK ||
        cudaMalloc(&g.d_in8, (size_t)need + 256) != cudaSuccess ||
        cudaMalloc((void **)&g.d_flag, sizeof(unsigned)) != cudaSuccess ||
        cudaHostAlloc((void **)&g.h_flag, sizeof(unsigned), 0) != cudaSuccess) {
        if (g.plan8) mdsm_plan_destroy(g.plan8);
        if (g.d_in8) cudaFree(g.d_in8);
        if (g.d_flag) cudaFree(g.d_flag);
        if (g.h_flag) cudaFreeHost(g.h_flag);
        g.plan8 = nullptr;
        g.d_in8 = nullptr;
        g.d_flag = g.h_flag = nullptr;
        return;
    }
    cudaMemset(g.d_in8, 0, (size_t)need + 256);
    g.d_in8_bytes = (size_t)need + 256;
    g.stride8 = q.in_stride;
}

// Wait for the block on the worker; its failure becomes this thread's error.
mdsm_status join_worker()
{
    if (g_worker.t.joinable()) g_worker.t.join();
    const mdsm_status st = g.wstatus;
    if (st != MDSM_OK) set_error(g.werror);
    g.wstatus = MDSM_OK;
    return st;
}

// A block's first half, on the caller's thread: tail carry and H2D of the new samples (the
// caller may refill its buffer once this returns), and the 8-bit check.
mdsm_status stage_block(Job &j)
{
    Plan &p = g.plan->p;
    const long long ms = p.maxshift, ns = p.nsamp;
    const int cur = (int)(g.blocks & 1), prv = cur ^ 1;
    j.cur = cur;
    if (g.blocks == 0) {
        MDSM_CUDA_TRY(cudaMemcpy2DAsync(g.d_in[cur], g.stride * 4, g.h_in, g.hstride * 4,
                                        (size_t)(ns + ms) * 4, p.nchans, cudaMemcpyHostToDevice,
                                        g.st));
    } else {
        if (ms > 0)
            MDSM_CUDA_TRY(cudaMemcpy2DAsync(g.d_in[cur], g.stride * 4,
                                            static_cast<float *>(g.d_in[prv]) + ns, g.stride * 4,
                                            (size_t)ms * 4, p.nchans, cudaMemcpyDeviceToDevice,
                                            g.st));
        MDSM_CUDA_TRY(cudaMemcpy2DAsync(static_cast<float *>(g.d_in[cur]) + ms, g.stride * 4,
                                        g.h_in + ms, g.hstride * 4, (size_t)ns * 4, p.nchans,
                                        cudaMemcpyHostToDevice, g.st));
    }
    if (g.plan8) {
        // all of the block's input (tail and new samples) integers 0..255?
        MDSM_CUDA_TRY(cudaMemsetAsync(g.d_flag, 0, sizeof(unsigned), g.st));
        MDSM_TRY(pack_u8_rows(static_cast<const float *>(g.d_in[cur]), g.stride, p.nchans, ns + ms,
                              static_cast<uint8_t *>(g.d_in8), g.stride8, g.d_flag, g.st));
        MDSM_CUDA_TRY(cudaMemcpyAsync(g.h_flag, g.d_flag, sizeof(unsigned),
                                      cudaMemcpyDeviceToHost, g.st));
    }
    MDSM_CUDA_TRY(cudaStreamSynchronize(g.st));
    j.eight = g.plan8 && *g.h_flag == 0;
    MDSM_CUDA_TRY(cudaGetDevice(&j.device));
    return MDSM_OK;
}

// A block's second half, on the worker: dedispersion, detection, D2H of the series and the
// candidate lines.
mdsm_status finish_block(const Job &j)
{
    MDSM_CUDA_TRY(cudaSetDevice(j.device));
    Plan &p = g.plan->p;
    const long long ns = p.nsamp;
    if (j.eight) {
        MDSM_TRY(plan_run_device(g.plan8->p, g.d_in8, g.stride8, g.d_in8_bytes, g.d_out, ns,
                                 g.st));
        MDSM_TRY(check_err_word(g.plan8->p.d_err, g.st));
        g.blocks8++;
    } else {
        MDSM_TRY(plan_run_device(p, g.d_in[j.cur], g.stride, g.d_in_bytes, g.d_out, ns, g.st));
    }
    long long nc = 0;
    std::vector<mdsm_candidate> c(1 << 16);
    // the reference's detectors (dedispersion_output.cpp:56-213): with the caller's noise
    // statistics of the block when next_chunk was given them, one value per samplesPerChunk
    const int spc = g.survey->samplesPerChunk ? (int)g.survey->samplesPerChunk : (int)ns;
    const long long nchunks = (ns - 5) / spc + 1;
    const float *cmean = j.mean.empty() ? nullptr : j.mean.data();
    const float *crms = j.rms.empty() ? nullptr : j.rms.data();
    const float *y = static_cast<const float *>(g.d_out);
    const float thr = g.survey->detection_threshold;
    if (p.kind == 1 && cmean)
        MDSM_TRY(ref_detect_chunked(y, p.ndms, (int)ns, g.survey->lowdm, g.survey->dmstep, thr,
                                    cmean, crms, nchunks, spc, c.data(), (long long)c.size(),
                                    &nc, g.st));
    else if (p.kind == 1)
        MDSM_TRY(ref_detect(y, p.ndms, (int)ns, g.survey->lowdm, g.survey->dmstep, thr, c.data(),
                            (long long)c.size(), &nc, nullptr, nullptr, g.st));
    else
        MDSM_TRY(ref_detect_subband(p, y, ns, thr, cmean, crms, nchunks, spc, c.data(),
                                    (long long)c.size(), &nc, g.st));
    MDSM_CUDA_TRY(cudaMemcpyAsync(g.h_out[j.cur], g.d_out, (size_t)p.ndms * ns * 4,
                                  cudaMemcpyDeviceToHost, g.st));
    MDSM_TRY(check_err_word(p.d_err, g.st));
    c.resize((size_t)std::min<long long>(nc, (long long)c.size()));
    g.cands = c;
    g.prev_read = j.data_read;
    write_candidates(c, nc, j.ts, j.rate, spc, cmean, crms);
    g.blocks++;
    return MDSM_OK;
}

// Hand one block in: its copies here, the rest on the worker.
mdsm_status submit_block(unsigned data_read)
{
    MDSM_TRY(join_worker());
    Job j;
    j.data_read = data_read;
    j.ts = g.ts;
    j.rate = g.rate;
    if (g.cmean) {
        // the caller's arrays hold one value per samplesPerChunk samples of this block
        const long long ns = g.plan->p.nsamp;
        const int spc = g.survey->samplesPerChunk ? (int)g.survey->samplesPerChunk : (int)ns;
        const long long nchunks = (ns - 5) / spc + 1;
        j.mean.assign(g.cmean, g.cmean + nchunks);
        j.rms.assign(g.crms, g.crms + nchunks);
    }
    MDSM_TRY(stage_block(j));
    g_worker.t = std::thread([j]() {
        g.wstatus = finish_block(j);
        if (g.wstatus != MDSM_OK) g.werror = mdsm_last_error();
    });
    return MDSM_OK;
}

}  // namespace
}  // namespace mdsm

using namespace mdsm;

extern "C" {

// src/mdsm/dedispersion_manager.cpp:40-199 (same tags, attributes and defaults).
SURVEY *mdsm_processSurveyParameters(const char *xml_path)
{
    std::ifstream f(xml_path ? xml_path : "");
    if (!f) {
        set_error(std::string("Cannot open observation file '") + (xml_path ? xml_path : "") + "'");
        return nullptr;
    }
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string src = ss.str();
    XParser px(src);
    XNode root;
    if (!px.element(root) || !px.ok) {
        set_error("observation file: parse error near byte " + std::to_string(px.i));
        return nullptr;
    }
    if (strcasecmp(root.tag.c_str(), "observation") != 0) {
        set_error("Invalid root element in observation parameter xml file, should be 'observation'");
        return nullptr;
    }
    SURVEY *s = static_cast<SURVEY *>(calloc(1, sizeof(SURVEY)));
    // defaults: dedispersion_manager.cpp:84-95
    s->useBruteForce = 0;
    s->useL1Cache = 1;
    s->detection_threshold = 5.0f;
    strcpy(s->fileprefix, "output");
    strcpy(s->basedir, ".");
    s->secs_per_file = 600;
    s->use_pc_time = 1;
    s->single_file_mode = 0;
    std::vector<SUBBAND_PASSES> passes;
    for (const XNode &e : root.kids) {
        const char *t = e.tag.c_str();
        if (!strcasecmp(t, "frequencies")) {
            s->fch1 = fattr(e, "top", 0);
            s->foff = fattr(e, "offset", 0);
        } else if (!strcasecmp(t, "dm")) {
            s->lowdm = fattr(e, "lowDM", 0);
            s->tdms = uattr(e, "numDMs", 0);
            s->dmstep = fattr(e, "dmStep", 0);
            s->useBruteForce = uattr(e, "useBruteForce", 0) != 0;
            s->useL1Cache = uattr(e, "useL1Cache", 0) != 0;
        } else if (!strcasecmp(t, "channels")) {
            s->nchans = uattr(e, "number", 0);
            s->nsubs = uattr(e, "subbands", 0);
        } else if (!strcasecmp(t, "timing")) {
            s->tsamp = fattr(e, "tsamp", 0);
        } else if (!strcasecmp(t, "samples")) {
            s->nsamp = uattr(e, "number", 0);
        } else if (!strcasecmp(t, "detection")) {
            s->detection_threshold = fattr(e, "threshold", 5.0f);
        } else if (!strcasecmp(t, "output")) {
            const char *v;
            if ((v = e.attr("filePrefix"))) snprintf(s->fileprefix, sizeof s->fileprefix, "%s", v);
            if ((v = e.attr("baseDirectory"))) snprintf(s->basedir, sizeof s->basedir, "%s", v);
            s->secs_per_file = uattr(e, "secondsPerFile", 600);
            s->use_pc_time = (char)uattr(e, "usePCTime", 1);
            s->single_file_mode = (char)uattr(e, "singleFileMode", 0);
        } else if (!strcasecmp(t, "gpus")) {
            std::vector<unsigned> ids;
            std::string v = e.attr("ids") ? e.attr("ids") : "";
            std::stringstream is(v);
            std::string tok;
            while (std::getline(is, tok, ','))
                if (!tok.empty()) ids.push_back((unsigned)strtoul(tok.c_str(), nullptr, 10));
            s->num_gpus = (unsigned)ids.size();
            s->gpu_ids = static_cast<unsigned *>(malloc(sizeof(unsigned) * (ids.size() + 1)));
            for (size_t i = 0; i < ids.size(); ++i) s->gpu_ids[i] = ids[i];
        } else if (!strcasecmp(t, "passes")) {
            for (const XNode &pn : e.kids) {
                SUBBAND_PASSES ps;
                memset(&ps, 0, sizeof ps);
                for (const XNode &q : pn.kids) {
                    const char *qt = q.tag.c_str();
                    const char *tx = q.text.c_str();
                    if (!strcasecmp(qt, "lowDm")) ps.lowdm = (float)atof(tx);
                    else if (!strcasecmp(qt, "highDm")) ps.highdm = (float)atof(tx);
                    else if (!strcasecmp(qt, "deltaDm")) ps.dmstep = (float)atof(tx);
                    else if (!strcasecmp(qt, "downsample")) ps.binsize = atoi(tx);
                    else if (!strcasecmp(qt, "subDm")) ps.sub_dmstep = (float)atof(tx);
                    else if (!strcasecmp(qt, "numDms")) ps.ndms = atoi(tx);
                    else if (!strcasecmp(qt, "dmsPerCall")) ps.calldms = atoi(tx);
                    else if (!strcasecmp(qt, "ncalls")) ps.ncalls = atoi(tx);
                }
                passes.push_back(ps);
            }
        }
    }
    s->num_passes = (unsigned)passes.size();
    if (!passes.empty()) {
        s->pass_parameters =
            static_cast<SUBBAND_PASSES *>(malloc(sizeof(SUBBAND_PASSES) * passes.size()));
        memcpy(s->pass_parameters, passes.data(), sizeof(SUBBAND_PASSES) * passes.size());
    }
    if (!s->useBruteForce) {  // :190-194
        s->tdms = 0;
        for (auto &ps : passes) s->tdms += (unsigned)ps.ndms;
    }
    return s;
}

void mdsm_free_survey(SURVEY *s)
{
    if (!s) return;
    free(s->pass_parameters);
    free(s->gpu_ids);
    free(s);
}

// src/mdsm/dedispersion_manager.cpp:269-382
float *mdsm_initialiseMDSM(SURVEY *s)
{
    if (!s) {
        set_error("initialiseMDSM: null survey");
        return nullptr;
    }
    if (g.live) release();
    g.survey = s;
    if (s->nsamp == 0) s->nsamp = 1u << 16;  // reference: fill GPU memory; here a fixed block
    mdsm_status st;
    if (s->useBruteForce) {
        mdsm_segment seg{s->lowdm, s->dmstep, (int)s->tdms};
        mdsm_brute_desc d;
        memset(&d, 0, sizeof d);
        d.nchans = (int)s->nchans;
        d.fch1 = s->fch1;
        d.foff = s->foff;
        d.tsamp = s->tsamp;
        d.nsamp = (int)s->nsamp;
        d.segs = &seg;
        d.nsegs = 1;
        d.shift_mode = s->useL1Cache ? MDSM_SHIFT_L1 : MDSM_SHIFT_OPT;
        d.in_dtype = MDSM_F32;
        d.out_dtype = MDSM_OUT_F32;
        st = mdsm_brute_plan_create(&d, &g.plan);
    } else {
        mdsm_subband_desc d;
        memset(&d, 0, sizeof d);
        d.nchans = (int)s->nchans;
        d.fch1 = s->fch1;
        d.foff = s->foff;
        d.tsamp = s->tsamp;
        d.nsamp = (int)s->nsamp;
        d.nsubs = (int)s->nsubs;
        d.passes = s->pass_parameters;
        d.npasses = (int)s->num_passes;
        d.use_fma = 1;
        d.in_dtype = MDSM_F32;
        d.out_dtype = MDSM_OUT_F32;
        st = mdsm_subband_plan_create(&d, &g.plan);
    }
    if (st != MDSM_OK) {
        g.survey = nullptr;
        return nullptr;
    }
    Plan &p = g.plan->p;
    s->maxshift = (unsigned)p.maxshift;
    s->num_threads = 1;
    if (s->samplesPerChunk == 0) s->samplesPerChunk = s->nsamp;
    // The host buffer keeps the reference's layout, rows of nsamp + maxshift samples
    // (dedispersion_manager.cpp allocates it so and the callers, MDSM.cpp:113 and
    // MdsmModule.cpp:143-149, index it so); the device copy uses the plan's padded pitch.
    g.hstride = (long long)p.nsamp + p.maxshift;
    const long long dev_stride = p.in_stride;
    long long need = 0;
    if (plan_in_requirements(p, dev_stride, &need) != MDSM_OK) return nullptr;
    g.stride = dev_stride;
    if (cudaStreamCreateWithFlags(&g.st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaHostAlloc((void **)&g.h_in, (size_t)g.hstride * p.nchans * 4, 0) != cudaSuccess ||
        cudaHostAlloc((void **)&g.h_out[0], (size_t)p.ndms * p.nsamp * 4, 0) != cudaSuccess ||
        cudaHostAlloc((void **)&g.h_out[1], (size_t)p.ndms * p.nsamp * 4, 0) != cudaSuccess ||
        cudaMalloc(&g.d_in[0], (size_t)need + 256) != cudaSuccess ||
        cudaMalloc(&g.d_in[1], (size_t)need + 256) != cudaSuccess ||
        cudaMalloc(&g.d_out, (size_t)p.ndms * p.nsamp * 4) != cudaSuccess) {
        set_error("initialiseMDSM: allocation failed");
        release();
        return nullptr;
    }
    cudaMemset(g.d_in[0], 0, (size_t)need + 256);
    cudaMemset(g.d_in[1], 0, (size_t)need + 256);
    memset(g.h_in, 0, (size_t)g.hstride * p.nchans * 4);
    g.d_in_bytes = (size_t)need + 256;
    setup_8bit(s);
    g.live = true;
    return g.h_in;
}

// src/mdsm/dedispersion_manager.cpp:416-484
float *mdsm_next_chunk(unsigned int data_read, unsigned *samples, double timestamp,
                       double blockRate, float *mean, float *rms)
{
    if (!g.live) {
        set_error("next_chunk before initialiseMDSM");
        return nullptr;
    }
    // the block handed in by the last start_processing is the one reported here
    if (join_worker() != MDSM_OK) {
        if (samples) *samples = 0;
        return nullptr;
    }
    // caller-owned noise statistics of the block being handed in (one value per
    // samplesPerChunk samples); read by the detector when the block is processed
    g.cmean = mean && rms ? mean : nullptr;
    g.crms = mean && rms ? rms : nullptr;
    g.pending_read = data_read;
    if (data_read == 0) g.stopping = true;
    g.survey->timestamp = timestamp;
    g.survey->blockRate = blockRate;
    g.ts = timestamp;
    g.rate = blockRate;
    if (g.blocks == 0) {
        if (samples) *samples = (unsigned)-1;
        return nullptr;
    }
    // A block's output is reported once; a repeated call with nothing new reports 0 samples.
    const bool fresh = g.blocks != g.returned;
    g.returned = g.blocks;
    if (samples) *samples = fresh ? g.prev_read : 0u;
    return g.h_out[(g.blocks - 1) & 1];
}

// src/mdsm/dedispersion_manager.cpp:487-501
int mdsm_start_processing(unsigned int data_read)
{
    if (!g.live) {
        set_error("start_processing before initialiseMDSM");
        return 0;
    }
    if (data_read == 0) {
        if (join_worker() != MDSM_OK) return 0;
        if (g.stopped_once) return 0;
        g.stopped_once = true;
        return (int)(g.blocks + 1);
    }
    if (submit_block(data_read) != MDSM_OK) return 0;
    return (int)(g.blocks + 1);  // the block now in flight counted
}

void mdsm_tearDownMDSM(void) { release(); }

long long mdsm_compat_candidates(mdsm_candidate *out, long long cap)
{
    if (join_worker() != MDSM_OK) return 0;
    const long long n = (long long)g.cands.size();
    for (long long i = 0; i < n && i < cap; ++i) out[i] = g.cands[i];
    return n;
}

long long mdsm_compat_blocks_8bit(void)
{
    join_worker();
    return g.blocks8;
}

}  // extern "C"
