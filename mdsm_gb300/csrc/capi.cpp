// capi.cpp -- the exported C ABI (include/mdsm_gb300.h) over the plan, kernel and detector code.
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "internal.h"

namespace mdsm {

namespace {
thread_local std::string g_last_error;
}

void set_error(const std::string &msg) { g_last_error = msg; }

mdsm_status fail(mdsm_status st, const std::string &msg)
{
    set_error(msg);
    return st;
}

mdsm_status cuda_fail(cudaError_t e, const char *what)
{
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    return MDSM_ECUDA;
}

mdsm_status plan_create_brute(const mdsm_brute_desc &d, Plan &p);
mdsm_status brute_tables(const mdsm_brute_desc &d, std::vector<float> &dmshifts,
                         std::vector<int32_t> &S, std::vector<float> &dmv);
void subband_tables(const SUBBAND_PASSES &ps, int nchans, int nsubs, float tsamp, bool use_fma,
                    const float *dms, std::vector<int32_t> &S1, std::vector<int32_t> &S2,
                    std::vector<float> &dmv);
mdsm_status plan_create_subband(const mdsm_subband_desc &d, Plan &p);

namespace {

void plan_release(Plan &p)
{
    for (auto &g : p.stages) free_stage(g);
    if (p.d_work) cudaFree(p.d_work);
    if (p.d_ds) cudaFree(p.d_ds);
    p.d_ds = nullptr;
    if (p.d_in) cudaFree(p.d_in);
    if (p.d_out) cudaFree(p.d_out);
    if (p.d_err) cudaFree(p.d_err);
    for (cudaEvent_t e : p.seg_ev) cudaEventDestroy(e);
    p.seg_ev.clear();
    for (cudaEvent_t e : p.stage_ev) cudaEventDestroy(e);
    p.stage_ev.clear();
    p.stage_ev_used = 0;
    if (p.s_in) cudaStreamDestroy(p.s_in);
    if (p.s_out) cudaStreamDestroy(p.s_out);
    p.s_in = p.s_out = nullptr;
    p.d_work = p.d_in = p.d_out = nullptr;
    p.d_err = nullptr;
}

mdsm_status ensure(void **buf, size_t *have, size_t want)
{
    if (*have >= want && *buf) return MDSM_OK;
    if (*buf) cudaFree(*buf);
    *buf = nullptr;
    *have = 0;
    MDSM_CUDA_TRY(cudaMalloc(buf, want));
    *have = want;
    return MDSM_OK;
}

}  // namespace
}  // namespace mdsm

using namespace mdsm;

namespace {

constexpr long long kHostSegMin = 16384;  // output samples per segment, at least
constexpr int kHostSegMax = 16;           // segments per block, at most
constexpr long long kHostSegEdge = 4096;  // first and last segment of a long block

// Brute force from host buffers with the block cut into time segments: segment s's new input
// columns are copied in on one stream, its output columns are computed on the caller's stream
// once they have landed, and copied out on a third stream while later segments compute, so
// the host-link copies hide behind the kernel.  Segment s computes outputs [t0, t0 + len) and
// needs input columns [t0, t0 + len + maxshift); the copy of segment s + 1 only writes columns
// past those.  Results are those of one launch over the whole block: every output sample is
// computed by the same tile code from the same inputs.
mdsm_status dedisperse_host_pipelined(Plan &p, const void *h_in, long long h_in_stride,
                                      void *h_out, cudaStream_t st)
{
    const StageGeom &g = p.stages[0];
    const long long SZ = (long long)dtype_size(p.in_dtype);
    const long long row = (long long)p.nsamp + p.maxshift;
    // Segment starts, multiples of 512 (whole tiles of either kernel, 16-byte aligned
    // offsets).  Long blocks get short first and last segments (kHostSegEdge samples): the
    // first copy-in and the last copy-out are the parts nothing overlaps.
    std::vector<long long> starts{0};
    long long m_lo = 0, m_hi = p.nsamp;  // the uniformly cut middle
    if (p.nsamp >= 2 * kHostSegEdge + 2 * kHostSegMin) {
        m_lo = kHostSegEdge;
        m_hi = (p.nsamp - kHostSegEdge) / 512 * 512;
        starts.push_back(m_lo);
    }
    const long long nmid = std::max<long long>(
        1, std::min<long long>(kHostSegMax - (long long)starts.size() - (m_hi < p.nsamp),
                               (m_hi - m_lo) / kHostSegMin));
    const long long seg = ((m_hi - m_lo + nmid - 1) / nmid + 511) / 512 * 512;
    for (long long t = m_lo + seg; t < m_hi; t += seg) starts.push_back(t);
    if (m_hi < p.nsamp) starts.push_back(m_hi);
    const long long nseg = (long long)starts.size();
    if (!p.s_in) MDSM_CUDA_TRY(cudaStreamCreateWithFlags(&p.s_in, cudaStreamNonBlocking));
    if (!p.s_out) MDSM_CUDA_TRY(cudaStreamCreateWithFlags(&p.s_out, cudaStreamNonBlocking));
    while ((long long)p.seg_ev.size() < 2 * nseg + 2) {
        cudaEvent_t e;
        MDSM_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        p.seg_ev.push_back(e);
    }
    // the previous work of the caller's stream (earlier users of d_in / d_out) comes first
    MDSM_CUDA_TRY(cudaEventRecord(p.seg_ev[2 * nseg], st));
    MDSM_CUDA_TRY(cudaStreamWaitEvent(p.s_in, p.seg_ev[2 * nseg], 0));
    MDSM_CUDA_TRY(cudaStreamWaitEvent(p.s_out, p.seg_ev[2 * nseg], 0));
    const char *hi = static_cast<const char *>(h_in);
    char *ho = static_cast<char *>(h_out);
    char *di = static_cast<char *>(p.d_in);
    char *dout = static_cast<char *>(p.d_out);
    long long done = 0;  // input columns copied so far
    p.last_launches = 0;
    for (long long s = 0; s < nseg; ++s) {
        const long long t0 = starts[(size_t)s];
        const long long len = (s + 1 < nseg ? starts[(size_t)s + 1] : (long long)p.nsamp) - t0;
        const long long hi_col = s == nseg - 1 ? row : std::min(row, t0 + len + p.maxshift);
        if (hi_col > done) {
            MDSM_CUDA_TRY(cudaMemcpy2DAsync(di + done * SZ, (size_t)(p.in_stride * SZ),
                                            hi + done * SZ, (size_t)(h_in_stride * SZ),
                                            (size_t)((hi_col - done) * SZ), (size_t)p.nchans,
                                            cudaMemcpyHostToDevice, p.s_in));
            done = hi_col;
        }
        MDSM_CUDA_TRY(cudaEventRecord(p.seg_ev[2 * s], p.s_in));
        MDSM_CUDA_TRY(cudaStreamWaitEvent(st, p.seg_ev[2 * s], 0));
        MDSM_TRY(launch_stage(g, di + t0 * SZ, p.in_stride, 0, dout + t0 * 4, p.nsamp, 0,
                              p.d_err, st, &p.last_launches, len));
        MDSM_CUDA_TRY(cudaEventRecord(p.seg_ev[2 * s + 1], st));
        MDSM_CUDA_TRY(cudaStreamWaitEvent(p.s_out, p.seg_ev[2 * s + 1], 0));
        MDSM_CUDA_TRY(cudaMemcpy2DAsync(ho + t0 * 4, (size_t)p.nsamp * 4, dout + t0 * 4,
                                        (size_t)p.nsamp * 4, (size_t)len * 4, (size_t)p.ndms,
                                        cudaMemcpyDeviceToHost, p.s_out));
    }
    MDSM_CUDA_TRY(cudaEventRecord(p.seg_ev[2 * nseg + 1], p.s_out));
    MDSM_CUDA_TRY(cudaStreamWaitEvent(st, p.seg_ev[2 * nseg + 1], 0));
    return check_err_word(p.d_err, st);
}

}  // namespace

extern "C" {

float mdsm_dmdelay(float f1, float f2) { return dmdelay_ref(f1, f2); }

const char *mdsm_last_error(void) { return g_last_error.c_str(); }

const char *mdsm_version(void) { return "mdsm_gb300 0.1 (sm_103a)"; }

mdsm_status mdsm_brute_plan_create(const mdsm_brute_desc *desc, mdsm_plan **out)
{
    if (!desc || !out) return fail(MDSM_EINVAL, "null argument");
    *out = nullptr;
    mdsm_plan *h = new (std::nothrow) mdsm_plan();
    if (!h) return fail(MDSM_ENOMEM, "out of host memory");
    mdsm_status st = plan_create_brute(*desc, h->p);
    if (st != MDSM_OK) {
        plan_release(h->p);
        delete h;
        return st;
    }
    *out = h;
    return MDSM_OK;
}

mdsm_status mdsm_subband_plan_create(const mdsm_subband_desc *desc, mdsm_plan **out)
{
    if (!desc || !out) return fail(MDSM_EINVAL, "null argument");
    *out = nullptr;
    mdsm_plan *h = new (std::nothrow) mdsm_plan();
    if (!h) return fail(MDSM_ENOMEM, "out of host memory");
    mdsm_status st = plan_create_subband(*desc, h->p);
    if (st != MDSM_OK) {
        plan_release(h->p);
        delete h;
        return st;
    }
    *out = h;
    return MDSM_OK;
}

void mdsm_plan_destroy(mdsm_plan *plan)
{
    if (!plan) return;
    plan_release(plan->p);
    delete plan;
}

mdsm_status mdsm_plan_get_info(const mdsm_plan *plan, mdsm_plan_info *info)
{
    if (!plan || !info) return fail(MDSM_EINVAL, "null argument");
    const Plan &p = plan->p;
    std::memset(info, 0, sizeof(*info));
    info->nchans = p.nchans;
    info->ndms = p.ndms;
    info->nsamp = p.nsamp;
    info->maxshift = p.maxshift;
    info->in_stride = p.in_stride;
    long long need = 0;
    plan_in_requirements(p, p.in_stride, &need);
    info->in_bytes = need;
    info->out_bytes = (long long)p.ndms * p.nsamp * 4;
    info->in_dtype = p.in_dtype;
    info->out_dtype = p.out_dtype;
    info->acc = p.acc;
    info->dm_block = p.stages.empty() ? 0 : p.stages.back().Db;
    info->time_tile = p.stages.empty() ? 0 : p.stages.back().T;
    info->kernel = p.stages.empty() ? 0 : p.stages.back().kernel;
    info->nstages = (int)p.stages.size();
    info->work_bytes = (long long)p.work_bytes;
    return MDSM_OK;
}

mdsm_status mdsm_plan_stage_info(const mdsm_plan *plan, int stage, mdsm_stage_info *info)
{
    if (!plan || !info) return fail(MDSM_EINVAL, "null argument");
    const Plan &p = plan->p;
    if (stage < 0 || stage >= (int)p.stages.size()) return fail(MDSM_EINVAL, "no such stage");
    const StageGeom &g = p.stages[(size_t)stage];
    std::memset(info, 0, sizeof(*info));
    info->kernel = g.kernel;
    info->dm_block = g.Db;
    info->time_tile = g.T;
    info->out_u16 = g.out_u16;
    info->nchans = g.nchans;
    info->ndms = g.ndms;
    info->ngroups = g.ngroups;
    info->nsamp = (int)g.nsamp;
    info->smem_bytes = (long long)g.smem_bytes;
    return MDSM_OK;
}

mdsm_status mdsm_plan_shift_table(const mdsm_plan *plan, int which, int32_t *out)
{
    if (!plan || !out) return fail(MDSM_EINVAL, "null argument");
    const Plan &p = plan->p;
    const std::vector<int32_t> *v = p.kind == 1 ? &p.S : (which == 2 ? &p.S2 : &p.S1);
    std::memcpy(out, v->data(), v->size() * sizeof(int32_t));
    return MDSM_OK;
}

mdsm_status mdsm_plan_dm_values(const mdsm_plan *plan, float *out)
{
    if (!plan || !out) return fail(MDSM_EINVAL, "null argument");
    std::memcpy(out, plan->p.dm_values.data(), plan->p.dm_values.size() * sizeof(float));
    return MDSM_OK;
}

mdsm_status mdsm_plan_dmshifts(const mdsm_plan *plan, float *out)
{
    if (!plan || !out) return fail(MDSM_EINVAL, "null argument");
    std::memcpy(out, plan->p.dmshifts.data(), plan->p.dmshifts.size() * sizeof(float));
    return MDSM_OK;
}

mdsm_status mdsm_dmshifts(int nchans, float fch1, float foff, float *out)
{
    if (nchans <= 0 || !out) return fail(MDSM_EINVAL, "bad arguments");
    dmshifts_ref(nchans, fch1, foff, out);
    return MDSM_OK;
}

mdsm_status mdsm_brute_shift_table(const mdsm_brute_desc *desc, int32_t *S, float *dm_values,
                                   int *maxshift)
{
    if (!desc) return fail(MDSM_EINVAL, "null argument");
    std::vector<float> dms, dmv;
    std::vector<int32_t> T;
    MDSM_TRY(brute_tables(*desc, dms, T, dmv));
    if (S) std::memcpy(S, T.data(), T.size() * sizeof(int32_t));
    if (dm_values) std::memcpy(dm_values, dmv.data(), dmv.size() * sizeof(float));
    if (maxshift) {
        int m = 0;
        for (int32_t v : T) m = v > m ? v : m;
        *maxshift = m;
    }
    return MDSM_OK;
}

mdsm_status mdsm_subband_shift_tables(const mdsm_subband_desc *desc, int pass, int32_t *S1,
                                      int32_t *S2)
{
    if (!desc || pass < 0 || pass >= desc->npasses || desc->nsubs <= 0 ||
        desc->nchans % desc->nsubs != 0)
        return fail(MDSM_EINVAL, "bad arguments");
    std::vector<float> dms(desc->nchans), dmv;
    dmshifts_ref(desc->nchans, desc->fch1, desc->foff, dms.data());
    std::vector<int32_t> a, b;
    const int bsz = desc->passes[pass].binsize > 1 ? desc->passes[pass].binsize : 1;
    subband_tables(desc->passes[pass], desc->nchans, desc->nsubs, desc->tsamp * (float)bsz,
                   desc->use_fma != 0, dms.data(), a, b, dmv);
    if (S1) std::memcpy(S1, a.data(), a.size() * sizeof(int32_t));
    if (S2) std::memcpy(S2, b.data(), b.size() * sizeof(int32_t));
    return MDSM_OK;
}

mdsm_status mdsm_dedisperse_device(mdsm_plan *plan, const void *d_in, long long in_stride,
                                   size_t in_bytes, void *d_out, long long out_stride,
                                   void *stream)
{
    if (!plan || !d_in || !d_out) return fail(MDSM_EINVAL, "null argument");
    return plan_run_device(plan->p, d_in, in_stride, in_bytes, d_out, out_stride,
                           static_cast<cudaStream_t>(stream));
}

mdsm_status mdsm_dedisperse_host(mdsm_plan *plan, const void *h_in, long long h_in_stride,
                                 void *h_out, void *stream)
{
    if (!plan || !h_in || !h_out) return fail(MDSM_EINVAL, "null argument");
    Plan &p = plan->p;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t SZ = dtype_size(p.in_dtype);
    const long long row = (long long)p.nsamp + p.maxshift;
    if (h_in_stride < row)
        return fail(MDSM_ERANGE, "host row pitch smaller than nsamp + maxshift");
    long long need = 0;
    MDSM_TRY(plan_in_requirements(p, p.in_stride, &need));
    MDSM_TRY(ensure(&p.d_in, &p.d_in_bytes, (size_t)need + 256));
    const size_t out_bytes = (size_t)p.ndms * p.nsamp * 4;
    MDSM_TRY(ensure(&p.d_out, &p.d_out_bytes, out_bytes));
    if (p.kind == 1 && p.nsamp >= 2 * kHostSegMin)
        return dedisperse_host_pipelined(p, h_in, h_in_stride, h_out, st);
    MDSM_CUDA_TRY(cudaMemcpy2DAsync(p.d_in, (size_t)p.in_stride * SZ, h_in,
                                    (size_t)h_in_stride * SZ, (size_t)row * SZ,
                                    (size_t)p.nchans, cudaMemcpyHostToDevice, st));
    MDSM_TRY(plan_run_device(p, p.d_in, p.in_stride, p.d_in_bytes, p.d_out, p.nsamp, st));
    MDSM_CUDA_TRY(cudaMemcpyAsync(h_out, p.d_out, out_bytes, cudaMemcpyDeviceToHost, st));
    return check_err_word(p.d_err, st);
}

int mdsm_plan_last_launches(const mdsm_plan *plan) { return plan ? plan->p.last_launches : 0; }

mdsm_status mdsm_plan_check(mdsm_plan *plan, void *stream)
{
    if (!plan) return fail(MDSM_EINVAL, "null argument");
    return check_err_word(plan->p.d_err, static_cast<cudaStream_t>(stream));
}

mdsm_status mdsm_plan_wait_selftest(mdsm_plan *plan, unsigned spin_limit, void *stream)
{
    if (!plan) return fail(MDSM_EINVAL, "null argument");
    if (spin_limit == 0 || spin_limit > (1u << 16))
        return fail(MDSM_EINVAL, "wait self-test: spin limit must be 1..65536");
    return wait_selftest(plan->p.d_err, spin_limit, static_cast<cudaStream_t>(stream));
}

mdsm_status mdsm_plan_set_stage_timing(mdsm_plan *plan, int on)
{
    if (!plan) return fail(MDSM_EINVAL, "null argument");
    Plan &p = plan->p;
    if (on && p.stage_ev.size() < p.stages.size() + 1) {
        while (p.stage_ev.size() < p.stages.size() + 1) {
            cudaEvent_t e = nullptr;
            MDSM_CUDA_TRY(cudaEventCreate(&e));
            p.stage_ev.push_back(e);
        }
    }
    p.stage_timing = on != 0;
    p.stage_ev_used = 0;
    return MDSM_OK;
}

mdsm_status mdsm_plan_stage_times(mdsm_plan *plan, float *ms, int cap, int *n)
{
    if (!plan || !n) return fail(MDSM_EINVAL, "null argument");
    Plan &p = plan->p;
    *n = 0;
    if (p.stage_ev_used < 2) return fail(MDSM_ESTATE, "no timed device-path call on this plan");
    MDSM_CUDA_TRY(cudaEventSynchronize(p.stage_ev[(size_t)p.stage_ev_used - 1]));
    const int k = p.stage_ev_used - 1;
    for (int i = 0; i < k && i < cap; ++i)
        MDSM_CUDA_TRY(cudaEventElapsedTime(&ms[i], p.stage_ev[(size_t)i],
                                           p.stage_ev[(size_t)i + 1]));
    *n = k;
    return MDSM_OK;
}

mdsm_status mdsm_rfi_clip_device(void *d_x, int dtype, int nchans, long long stride,
                                 long long len, double k_chan, double k_spec, void *stream)
{
    if (!d_x || nchans <= 0 || len <= 0 || stride < len)
        return fail(MDSM_EINVAL, "rfi clip: bad geometry");
    return rfi_clip(d_x, dtype, nchans, stride, len, k_chan, k_spec,
                    static_cast<cudaStream_t>(stream));
}

mdsm_status mdsm_ref_detect_device(const float *d_series, int ndms, int nsamp, float lowdm,
                                   float dmstep, float threshold, mdsm_candidate *h_cands,
                                   long long cap, long long *ncand, float *mean, float *rms,
                                   void *stream)
{
    if (!d_series || ndms <= 0 || nsamp < 5 || !ncand)
        return fail(MDSM_EINVAL, "reference detector: bad arguments");
    return ref_detect(d_series, ndms, nsamp, lowdm, dmstep, threshold, h_cands, cap, ncand,
                      mean, rms, static_cast<cudaStream_t>(stream));
}

mdsm_status mdsm_ref_detect_device_noalloc(const float *d_series, int ndms, int nsamp,
                                           float lowdm, float dmstep, float threshold,
                                           mdsm_candidate *h_cands, long long cap,
                                           long long *ncand, float *mean, float *rms,
                                           void *stream)
{
    if (!d_series || ndms <= 0 || nsamp < 5 || !ncand)
        return fail(MDSM_EINVAL, "reference detector: bad arguments");
    return ref_detect_noalloc(d_series, ndms, nsamp, lowdm, dmstep, threshold, h_cands, cap,
                              ncand, mean, rms, static_cast<cudaStream_t>(stream));
}

mdsm_status mdsm_ref_detect_chunked_device(const float *d_series, int ndms, int nsamp,
                                           float lowdm, float dmstep, float threshold,
                                           const float *h_mean, const float *h_rms,
                                           long long nchunks, int spc, mdsm_candidate *h_cands,
                                           long long cap, long long *ncand, void *stream)
{
    if (!d_series || ndms <= 0 || nsamp < 5 || !ncand || !h_mean || !h_rms)
        return fail(MDSM_EINVAL, "chunked detector: bad arguments");
    return ref_detect_chunked(d_series, ndms, nsamp, lowdm, dmstep, threshold, h_mean, h_rms,
                              nchunks, spc, h_cands, cap, ncand,
                              static_cast<cudaStream_t>(stream));
}

mdsm_status mdsm_ref_detect_subband_device(const mdsm_plan *plan, const float *d_series,
                                           long long out_stride, float threshold,
                                           const float *h_mean, const float *h_rms,
                                           long long nchunks, int spc, mdsm_candidate *h_cands,
                                           long long cap, long long *ncand, void *stream)
{
    if (!plan || !d_series || !ncand) return fail(MDSM_EINVAL, "subband detector: bad arguments");
    if (plan->p.out_dtype != MDSM_OUT_F32)
        return fail(MDSM_EINVAL, "subband detector: the reference's detector reads float series");
    if (out_stride < plan->p.nsamp)
        return fail(MDSM_ERANGE, "subband detector: row pitch smaller than nsamp");
    return ref_detect_subband(plan->p, d_series, out_stride, threshold, h_mean, h_rms, nchunks,
                              spc, h_cands, cap, ncand, static_cast<cudaStream_t>(stream));
}

mdsm_status mdsm_boxcar_detect_device(const void *d_series, int series_dtype, int ndms,
                                      int nsamp, int nwidths, double threshold,
                                      mdsm_candidate *h_cands, long long cap, long long *ncand,
                                      void *stream)
{
    if (!d_series || ndms <= 0 || nsamp <= 0 || nwidths < 1 || nwidths > 12 || !ncand)
        return fail(MDSM_EINVAL, "boxcar detector: bad arguments");
    return boxcar_detect(d_series, series_dtype, ndms, nsamp, nwidths, threshold, h_cands, cap,
                         ncand, static_cast<cudaStream_t>(stream));
}

}  // extern "C"
