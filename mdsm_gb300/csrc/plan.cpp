// plan.cpp -- DM plans: per-channel delays, integer shift tables, buffer geometry, and the
// run sequence of a plan on the device.
//
// The integer shift of every (DM trial, channel) pair is formed once here on the host, with the
// same float/double operations the reference evaluates (its delays in
// src/mdsm/dedispersion_manager.cpp:262-289, its shift expressions in
// src/mdsm/dedispersion_kernel.cu:27,36 / :54,70 / :148,163,167 and the host-side arguments in
// src/mdsm/dedispersion_thread.cu:76,85-86,151-205).  The device kernels then index with
// integers only, so shift parity is a property of this file that the CPU tests check in full.
// This file is compiled with -ffp-contract=off: every expression is rounded operation by
// operation as written, and the device-side contractions are spelled out with std::fma.
#include <cmath>
#include <cstring>

#include <algorithm>

#include "internal.h"

namespace mdsm {

// src/mdsm/dedispersion_manager.cpp:262-265 (double arithmetic, float result)
float dmdelay_ref(float f1, float f2)
{
    const double a = 1.0 / (double)f1 / (double)f1;
    const double b = 1.0 / (double)f2 / (double)f2;
    return (float)(4148.741601 * (a - b));
}

// src/mdsm/dedispersion_manager.cpp:286-289: f_c = fch1 + foff*c in float
void dmshifts_ref(int nchans, float fch1, float foff, float *out)
{
    for (int c = 0; c < nchans; ++c) {
        const float fc = fch1 + foff * (float)c;
        out[c] = dmdelay_ref(fc, fch1);
    }
}

// The per-trial factor each mode multiplies the channel delay by (float modes), evaluated as
// the reference evaluates it.  idx is the trial's index inside its segment.
static float trial_factor(float lowdm, float dmstep, int idx, float tsamp, int mode)
{
    switch (mode) {
    case MDSM_SHIFT_L1: {
        const float ms = lowdm / tsamp;   // dedispersion_thread.cu:85
        const float md = dmstep / tsamp;  // dedispersion_thread.cu:86
        return std::fma((float)(unsigned)idx, md, ms);  // dedispersion_kernel.cu:27
    }
    case MDSM_SHIFT_L1_MULADD: {
        const float ms = lowdm / tsamp, md = dmstep / tsamp;
        const float m = (float)(unsigned)idx * md;
        return ms + m;
    }
    case MDSM_SHIFT_OPT:  // dedispersion_kernel.cu:54
        return std::fma((float)(unsigned)idx, dmstep, lowdm) / tsamp;
    case MDSM_SHIFT_OPT_MULADD: {
        const float m = (float)(unsigned)idx * dmstep;
        return (lowdm + m) / tsamp;
    }
    }
    return 0.0f;
}

int32_t shift_of(float dms, double delay64, float lowdm, float dmstep, int idx, float tsamp,
                 int mode)
{
    if (mode == MDSM_SHIFT_FP64_TRUNC || mode == MDSM_SHIFT_FP64_ROUND) {
        const double dm = (double)lowdm + (double)idx * (double)dmstep;
        const double v = delay64 * dm / (double)tsamp;
        return mode == MDSM_SHIFT_FP64_TRUNC ? (int32_t)std::trunc(v)
                                             : (int32_t)std::floor(v + 0.5);
    }
    const float p = dms * trial_factor(lowdm, dmstep, idx, tsamp, mode);
    // dedispersion_kernel.cu:36 truncates (__float2int_rz); :70 floors
    return (mode == MDSM_SHIFT_L1 || mode == MDSM_SHIFT_L1_MULADD) ? (int32_t)std::trunc(p)
                                                                   : (int32_t)std::floor(p);
}

namespace {

// 1: exact INT32 sums, 0: FP32, -1: INT32 asked for float samples, -2: INT32 asked for sums
// that may not fit.  Automatic: INT32 where a sum of nchans samples always fits, else FP32.
int acc_is_int(int in_dtype, int acc, int nchans)
{
    const long long maxabs = in_dtype == MDSM_U8 ? 255 : in_dtype == MDSM_U16 ? 65535
                             : in_dtype == MDSM_I16 ? 32768 : 0;
    const bool fits = maxabs > 0 && (long long)nchans * maxabs <= 0x7fffffffLL;
    if (acc == MDSM_ACC_I32) return in_dtype == MDSM_F32 ? -1 : (fits ? 1 : -2);
    if (acc == MDSM_ACC_F32) return 0;
    return fits ? 1 : 0;
}

long long round_pitch(long long elems, int dtype)
{
    const long long per16 = 16 / (long long)dtype_size(dtype);
    return (elems + per16 - 1) / per16 * per16;
}

mdsm_status alloc_err(Plan &p)
{
    MDSM_CUDA_TRY(cudaMalloc(&p.d_err, sizeof(unsigned)));
    MDSM_CUDA_TRY(cudaMemset(p.d_err, 0, sizeof(unsigned)));
    return MDSM_OK;
}

}  // namespace

// --------------------------------------------------------------------------------------------
// brute force
// --------------------------------------------------------------------------------------------

mdsm_status brute_tables(const mdsm_brute_desc &d, std::vector<float> &dmshifts,
                         std::vector<int32_t> &S, std::vector<float> &dmv)
{
    if (d.nchans <= 0 || d.nsamp <= 0 || d.nsegs <= 0 || !d.segs || !(d.tsamp > 0))
        return fail(MDSM_EINVAL, "brute plan: nchans, nsamp, segments and tsamp are required");
    if (d.shift_mode < MDSM_SHIFT_L1 || d.shift_mode > MDSM_SHIFT_FP64_ROUND)
        return fail(MDSM_EINVAL, "brute plan: unknown shift mode");
    int ndms = 0;
    for (int s = 0; s < d.nsegs; ++s) {
        if (d.segs[s].ndms <= 0) return fail(MDSM_EINVAL, "segment with no DM trials");
        ndms += d.segs[s].ndms;
    }
    dmshifts.resize(d.nchans);
    dmshifts_ref(d.nchans, d.fch1, d.foff, dmshifts.data());
    const double K = d.K > 0 ? d.K : 4148.741601;
    std::vector<double> d64(d.nchans);
    for (int c = 0; c < d.nchans; ++c) {
        const double fc = (double)d.fch1 + (double)d.foff * c, ft = (double)d.fch1;
        d64[c] = K * (1.0 / (fc * fc) - 1.0 / (ft * ft));
    }
    S.resize((size_t)ndms * d.nchans);
    dmv.resize(ndms);
    int row = 0;
    for (int s = 0; s < d.nsegs; ++s)
        for (int i = 0; i < d.segs[s].ndms; ++i, ++row) {
            const float m = (float)(unsigned)i * d.segs[s].dmstep;
            dmv[row] = d.segs[s].lowdm + m;
            int32_t *o = &S[(size_t)row * d.nchans];
            if (d.shift_mode == MDSM_SHIFT_FP64_TRUNC || d.shift_mode == MDSM_SHIFT_FP64_ROUND) {
                for (int c = 0; c < d.nchans; ++c)
                    o[c] = shift_of(dmshifts[c], d64[c], d.segs[s].lowdm, d.segs[s].dmstep, i,
                                    d.tsamp, d.shift_mode);
            } else {
                const float f = trial_factor(d.segs[s].lowdm, d.segs[s].dmstep, i, d.tsamp,
                                             d.shift_mode);
                const bool l1 =
                    d.shift_mode == MDSM_SHIFT_L1 || d.shift_mode == MDSM_SHIFT_L1_MULADD;
                for (int c = 0; c < d.nchans; ++c) {
                    const float pr = dmshifts[c] * f;
                    o[c] = l1 ? (int32_t)std::trunc(pr) : (int32_t)std::floor(pr);
                }
            }
        }
    return MDSM_OK;
}

mdsm_status plan_create_brute(const mdsm_brute_desc &d, Plan &p)
{
    if (d.in_dtype < MDSM_U8 || d.in_dtype > MDSM_F32)
        return fail(MDSM_EINVAL, "brute plan: unknown input dtype");
    const int ai = acc_is_int(d.in_dtype, d.acc, d.nchans);
    if (ai == -2)
        return fail(MDSM_ERANGE, "INT32 accumulation: sums of this many channels may overflow");
    if (ai < 0) return fail(MDSM_EINVAL, "INT32 accumulation needs integer samples");
    MDSM_TRY(brute_tables(d, p.dmshifts, p.S, p.dm_values));
    const int ndms = (int)p.dm_values.size();
    p.kind = 1;
    p.nchans = d.nchans;
    p.nsamp = d.nsamp;
    p.fch1 = d.fch1;
    p.foff = d.foff;
    p.tsamp = d.tsamp;
    p.in_dtype = d.in_dtype;
    p.out_dtype = d.out_dtype;
    p.acc = ai ? MDSM_ACC_I32 : MDSM_ACC_F32;  // the accumulation in effect
    p.ndms = ndms;
    StageGeom g;
    g.nchans = d.nchans;
    g.ndms = ndms;
    g.ngroups = 1;
    g.nsamp = d.nsamp;
    g.in_dtype = d.in_dtype;
    g.acc_int = ai;
    g.out_i32 = d.out_dtype == MDSM_OUT_I32;
    g.DPW = d.dm_block == 16 ? 2 : (d.dm_block == 8 ? 1 : 4);
    g.kernel = d.kernel;
    MDSM_TRY(build_stage_tables(g, p.S));
    p.maxshift = g.max_shift;
    MDSM_TRY(upload_stage(g));
    p.stages.push_back(std::move(g));
    p.in_stride = round_pitch((long long)p.nsamp + p.maxshift, p.in_dtype);
    return alloc_err(p);
}

// --------------------------------------------------------------------------------------------
// two-stage subband
// --------------------------------------------------------------------------------------------

// Stage tables of one subband pass: S1 [ncalls][nchans], S2 [ncalls*calldms][nsubs]; appends
// the pass's fine DM values to dmv.
void subband_tables(const SUBBAND_PASSES &ps, int nchans, int nsubs, float tsamp, bool use_fma,
                    const float *dms, std::vector<int32_t> &S1, std::vector<int32_t> &S2,
                    std::vector<float> &dmv)
{
    struct {
        int nchans;
        float tsamp;
        int use_fma;
    } d{nchans, tsamp, use_fma ? 1 : 0};
    const int cps = nchans / nsubs;
    const int ncalls = ps.ncalls, calldms = ps.calldms;
        // stage 1 shifts (dedispersion_kernel.cu:148,163,167; startdm = lowdm on one device)
        S1.assign((size_t)ncalls * d.nchans, 0);
        for (int j = 0; j < ncalls; ++j) {
            float num;
            if (d.use_fma)
                num = std::fma((float)(unsigned)j, ps.sub_dmstep, ps.lowdm);
            else {
                float m = (float)(unsigned)j * ps.sub_dmstep;
                num = ps.lowdm + m;
            }
            float st = num / d.tsamp;
            for (int b = 0; b < nsubs; ++b) {
                float pl = dms[b * cps] * st;
                const int tv = (int)(float)pl;
                for (int c = b * cps; c < (b + 1) * cps; ++c) {
                    float v;
                    if (d.use_fma)
                        v = std::fma(dms[c], (float)st, -(float)tv);
                    else {
                        float pc = dms[c] * st;
                        v = pc - (float)tv;
                    }
                    S1[(size_t)j * d.nchans + c] = (int32_t)v;
                }
            }
        }
        // stage 2 shifts (dedispersion_thread.cu:197-205, kernel.cu:54,70)
        S2.assign((size_t)ncalls * calldms * nsubs, 0);
        for (int j = 0; j < ncalls; ++j) {
            float half = ((float)calldms * ps.dmstep) / 2.0f;
            float jm = ps.sub_dmstep * (float)j;
            float a = ps.lowdm + jm;
            float dm0 = a - half;
            if (!(dm0 > 0.0f)) dm0 = 0.0f;
            for (int k = 0; k < calldms; ++k) {
                float num;
                if (d.use_fma)
                    num = std::fma((float)(unsigned)k, ps.dmstep, dm0);
                else {
                    float m = (float)(unsigned)k * ps.dmstep;
                    num = dm0 + m;
                }
                float st = num / d.tsamp;
                dmv.push_back(num);
                for (int b = 0; b < nsubs; ++b) {
                    float pp = dms[b * cps] * st;
                    S2[((size_t)j * calldms + k) * nsubs + b] = (int32_t)std::floor((float)pp);
                }
            }
        }
}

mdsm_status plan_create_subband(const mdsm_subband_desc &d, Plan &p)
{
    if (d.nchans <= 0 || d.nsamp <= 0 || d.nsubs <= 0 || d.npasses <= 0 || !d.passes ||
        !(d.tsamp > 0))
        return fail(MDSM_EINVAL, "subband plan: nchans, nsamp, nsubs, passes, tsamp required");
    if (d.nchans % d.nsubs != 0)
        return fail(MDSM_EINVAL, "subband plan: nchans must be a multiple of nsubs");
    const int ai = acc_is_int(d.in_dtype, d.acc, d.nchans);
    if (ai == -2)
        return fail(MDSM_ERANGE, "INT32 accumulation: sums of this many channels may overflow");
    if (ai < 0) return fail(MDSM_EINVAL, "INT32 accumulation needs integer samples");
    p.kind = 2;
    p.nchans = d.nchans;
    p.nsamp = d.nsamp;
    p.fch1 = d.fch1;
    p.foff = d.foff;
    p.tsamp = d.tsamp;
    p.in_dtype = d.in_dtype;
    p.out_dtype = d.out_dtype;
    p.acc = ai ? MDSM_ACC_I32 : MDSM_ACC_F32;  // the accumulation in effect
    p.dmshifts.resize(d.nchans);
    dmshifts_ref(d.nchans, d.fch1, d.foff, p.dmshifts.data());
    const int nsubs = d.nsubs, cps = d.nchans / d.nsubs;
    const float *dms = p.dmshifts.data();
    const int zdtype = ai ? MDSM_I32 : MDSM_F32;
    long long row0 = 0;
    int maxshift = 0;
    size_t zmax = 0;
    for (int pi = 0; pi < d.npasses; ++pi) {
        const SUBBAND_PASSES &ps = d.passes[pi];
        const int bsz = std::max(1, ps.binsize);
        if (d.nsamp % bsz != 0)
            return fail(MDSM_EINVAL, "subband plan: nsamp must be a multiple of each downsample");
        if (ps.ncalls <= 0 || ps.calldms <= 0)
            return fail(MDSM_EINVAL, "subband plan: ncalls and calldms must be positive");
        const int ncalls = ps.ncalls, calldms = ps.calldms;
        // a pass with downsample b dedisperses the block summed over b samples, at tsamp*b
        // (src/mdsm/dedispersion_thread.cu:159-168,192-205)
        const int nsb = d.nsamp / bsz;
        const float tsb = d.tsamp * (float)bsz;
        const int ds_dtype = bsz == 1 ? d.in_dtype
                                      : (d.in_dtype == MDSM_U8 ? MDSM_U16
                                                               : (d.in_dtype == MDSM_F32 ? MDSM_F32
                                                                                         : MDSM_I32));
        if (bsz > 257 && d.in_dtype == MDSM_U8)
            return fail(MDSM_EINVAL, "subband plan: downsample above 257 for uint8 samples");
        std::vector<int32_t> S1, S2;
        subband_tables(ps, d.nchans, nsubs, tsb, d.use_fma != 0, dms, S1, S2, p.dm_values);
        int m2 = 0, m1 = 0;
        for (int32_t v : S2) m2 = std::max(m2, (int)v);
        const long long n1 = (long long)nsb + m2;
        // stage 1: groups = subbands, rows = sub-DMs.  Sums of at most 257 uint8 channels fit
        // uint16: the packed kernel then writes the subband series as uint16 and the second
        // stage reads half the bytes with its packed uint16 kernel.
        StageGeom g1;
        g1.nchans = cps;
        g1.ndms = ncalls;
        g1.ngroups = nsubs;
        g1.nsamp = (int)n1;
        g1.in_dtype = ds_dtype;
        g1.acc_int = ai;
        g1.out_i32 = ai;
        g1.out_u16 = ai && ds_dtype == MDSM_U8 && (long long)cps * 255 <= 65535;
        g1.DPW = 4;
        std::vector<int32_t> S1g((size_t)nsubs * ncalls * cps);
        for (int b = 0; b < nsubs; ++b)
            for (int j = 0; j < ncalls; ++j)
                for (int c = 0; c < cps; ++c)
                    S1g[((size_t)b * ncalls + j) * cps + c] = S1[(size_t)j * d.nchans + b * cps + c];
        MDSM_TRY(build_stage_tables(g1, S1g));
        const int pz = g1.out_u16 ? MDSM_U16 : zdtype;  // the pass's subband series type
        const long long n1p = round_pitch(n1, pz);
        m1 = g1.max_shift;
        g1.out_stride = (long long)nsubs * n1p;  // z[j][b][t]
        g1.out_group_stride = n1p;
        // stage 2: groups = calls, channels = subbands, rows = fine DMs
        StageGeom g2;
        g2.nchans = nsubs;
        g2.ndms = calldms;
        g2.ngroups = ncalls;
        g2.nsamp = nsb;
        g2.in_dtype = pz;
        g2.acc_int = ai;
        g2.out_i32 = d.out_dtype == MDSM_OUT_I32;
        g2.DPW = calldms <= 8 ? 1 : (calldms <= 16 ? 2 : 4);  // DM block no wider than a call
        if (calldms < 10) g2.kernel = 1;  // the packed uint16 kernel's blocks are 16 trials
        MDSM_TRY(build_stage_tables(g2, S2));
        g2.in_stride = n1p;
        g2.in_group_stride = (long long)nsubs * n1p;
        g1.in_group_stride = cps;  // multiplied by the input pitch at run time
        MDSM_TRY(upload_stage(g1));
        MDSM_TRY(upload_stage(g2));
        // z is written for t < n1 and read with the stage-2 tile overrun past its last row
        const size_t zwrite = (size_t)ncalls * nsubs * n1p * dtype_size(pz);
        const size_t zread = (size_t)stage_in_bytes(g2, n1p, (long long)nsubs * n1p);
        zmax = std::max(zmax, std::max(zwrite, zread) + 4096);
        // original samples read: (n1 + m1) downsampled samples of bsz each
        maxshift = std::max(maxshift, (int)((n1 - nsb + m1) * bsz));
        p.stages.push_back(std::move(g1));
        p.stages.push_back(std::move(g2));
        p.pass_row0.push_back(row0);
        p.pass_bin.push_back(bsz);
        p.pass_ds_dtype.push_back(ds_dtype);
        row0 += (long long)ncalls * calldms;
        if (pi == 0) {
            p.S1 = S1;
            p.S2 = S2;
            p.n1 = n1;
        }
    }
    p.ndms = (int)row0;
    p.maxshift = maxshift;
    p.work_bytes = zmax;
    MDSM_CUDA_TRY(cudaMalloc(&p.d_work, p.work_bytes));
    MDSM_CUDA_TRY(cudaMemset(p.d_work, 0, p.work_bytes));
    p.in_stride = round_pitch((long long)p.nsamp + p.maxshift, p.in_dtype);
    // downsampled copies of the block for passes with downsample > 1
    size_t dsmax = 0;
    for (size_t i = 0; i < p.pass_bin.size(); ++i) {
        const int b = p.pass_bin[i];
        const long long len = ((long long)p.nsamp + p.maxshift) / b;
        const long long pitch = b == 1 ? 0 : round_pitch(len, p.pass_ds_dtype[i]);
        p.pass_ds_pitch.push_back(pitch);
        if (b == 1) continue;
        const StageGeom &g1 = p.stages[2 * i];
        const size_t need = (size_t)std::max<long long>(
            stage_in_bytes(g1, pitch, g1.in_group_stride * pitch),
            (long long)p.nchans * pitch * (long long)dtype_size(p.pass_ds_dtype[i]));
        dsmax = std::max(dsmax, need + 4096);
    }
    if (dsmax) {
        MDSM_CUDA_TRY(cudaMalloc(&p.d_ds, dsmax));
        MDSM_CUDA_TRY(cudaMemset(p.d_ds, 0, dsmax));
        p.ds_bytes = dsmax;
        p.work_bytes += dsmax;
    }
    return alloc_err(p);
}

// --------------------------------------------------------------------------------------------
// running a plan
// --------------------------------------------------------------------------------------------

mdsm_status plan_in_requirements(const Plan &p, long long in_stride, long long *in_bytes)
{
    if (in_stride < (long long)p.nsamp + p.maxshift)
        return fail(MDSM_ERANGE, "input row pitch smaller than nsamp + maxshift (" +
                                     std::to_string(p.nsamp + p.maxshift) + ")");
    long long need = 0;
    if (p.kind == 1) {
        need = stage_in_bytes(p.stages[0], in_stride, 0);
    } else {
        for (size_t i = 0; i < p.stages.size(); i += 2) {
            const StageGeom &g1 = p.stages[i];
            if (p.pass_bin[i / 2] == 1)
                need = std::max(need, stage_in_bytes(g1, in_stride, g1.in_group_stride * in_stride));
            else  // the downsampling kernel reads whole rows of nsamp + maxshift samples
                need = std::max(need, ((long long)(p.nchans - 1) * in_stride + p.nsamp +
                                       p.maxshift) * (long long)dtype_size(p.in_dtype));
        }
    }
    *in_bytes = need;
    return MDSM_OK;
}

mdsm_status plan_run_device(Plan &p, const void *d_in, long long in_stride, size_t in_bytes,
                            void *d_out, long long out_stride, cudaStream_t st,
                            unsigned long long *mom, bool *folded)
{
    long long need = 0;
    MDSM_TRY(plan_in_requirements(p, in_stride, &need));
    if ((long long)in_bytes < need)
        return fail(MDSM_ERANGE, "input buffer has " + std::to_string(in_bytes) +
                                     " bytes; the plan reads up to " + std::to_string(need));
    if (out_stride < p.nsamp) return fail(MDSM_ERANGE, "output row pitch smaller than nsamp");
    p.last_launches = 0;
    p.stage_ev_used = 0;
    const bool timed = p.stage_timing && p.stage_ev.size() >= p.stages.size() + 1;
    auto mark = [&]() -> mdsm_status {
        if (timed) MDSM_CUDA_TRY(cudaEventRecord(p.stage_ev[(size_t)p.stage_ev_used++], st));
        return MDSM_OK;
    };
    // row moments folded into the final stages' stores, where all of them can
    bool fold = mom != nullptr;
    for (size_t i = p.kind == 1 ? 0 : 1; fold && i < p.stages.size(); i += p.kind == 1 ? 1 : 2)
        fold = stage_folds_moments(p.stages[i]);
    if (folded) *folded = fold;
    if (fold) MDSM_CUDA_TRY(cudaMemsetAsync(mom, 0, (size_t)p.ndms * 3 * sizeof(*mom), st));
    MDSM_TRY(mark());
    if (p.kind == 1) {
        MDSM_TRY(launch_stage(p.stages[0], d_in, in_stride, 0, d_out, out_stride, 0, p.d_err, st,
                              &p.last_launches, -1, fold ? mom : nullptr, p.ndms));
        return mark();
    }
    const size_t osz = 4;
    for (size_t i = 0; i < p.stages.size(); i += 2) {
        const StageGeom &g1 = p.stages[i];
        const StageGeom &g2 = p.stages[i + 1];
        const int b = p.pass_bin[i / 2];
        const void *src = d_in;
        long long pitch = in_stride;
        if (b > 1) {
            pitch = p.pass_ds_pitch[i / 2];
            MDSM_TRY(downsample(d_in, p.in_dtype, p.nchans, in_stride,
                                (long long)p.nsamp + p.maxshift, b, 0, p.d_ds,
                                p.pass_ds_dtype[i / 2], pitch, st));
            p.last_launches += 1;
            src = p.d_ds;
        }
        MDSM_TRY(launch_stage(g1, src, pitch, g1.in_group_stride * pitch, p.d_work,
                              g1.out_stride, g1.out_group_stride, p.d_err, st, &p.last_launches));
        MDSM_TRY(mark());
        void *o = static_cast<char *>(d_out) + (size_t)p.pass_row0[i / 2] * out_stride * osz;
        MDSM_TRY(launch_stage(g2, p.d_work, g2.in_stride, g2.in_group_stride, o, out_stride,
                              (long long)g2.ndms * out_stride, p.d_err, st, &p.last_launches, -1,
                              fold ? mom + 3 * (size_t)p.pass_row0[i / 2] : nullptr, g2.ndms));
        MDSM_TRY(mark());
    }
    return MDSM_OK;
}

mdsm_status check_err_word(unsigned *d_err, cudaStream_t st)
{
    unsigned h = 0;
    MDSM_CUDA_TRY(cudaMemcpyAsync(&h, d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    MDSM_CUDA_TRY(cudaStreamSynchronize(st));
    if (h & ERR_WAIT_TIMEOUT) {
        cudaMemsetAsync(d_err, 0, sizeof(unsigned), st);
        return fail(MDSM_ETIMEOUT, "a device-side wait ran out; results of this call are invalid");
    }
    return MDSM_OK;
}

}  // namespace mdsm
