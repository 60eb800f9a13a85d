/*
 * ref_gpu_harness.c -- TEST INFRASTRUCTURE ONLY.
 *
 * Runs the reference's own CUDA kernels (src/mdsm/dedispersion_kernel.cu, compiled unmodified
 * for sm_103a into oracle/_ref/ref_kernels.cubin by oracle/Makefile) through the CUDA driver
 * API, launched with the grids and arguments of src/mdsm/dedispersion_thread.cu.  It gives the
 * reference result that the oracle and the product are pinned against on a GPU.
 *
 * Before every launch the host computes the largest element index the kernel will read,
 * replaying the kernel's own index arithmetic (including the float rounding of the opt kernel's
 * index), and refuses the launch (returns RG_EBOUNDS) if it falls outside the allocation.
 */
#include <cuda.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define RG_OK 0
#define RG_ECUDA 1
#define RG_EBOUNDS 2
#define RG_ENOTLOADED 3

static CUmodule g_mod;
static CUfunction g_l1, g_opt, g_sub;
static CUdeviceptr g_shifts;
static size_t g_shifts_bytes;
static int g_loaded;
static char g_err[256];

const char *rg_error(void) { return g_err; }

#define CK(x)                                                                           \
    do {                                                                                \
        CUresult r_ = (x);                                                              \
        if (r_ != CUDA_SUCCESS) {                                                       \
            const char *s_ = 0;                                                         \
            cuGetErrorString(r_, &s_);                                                  \
            snprintf(g_err, sizeof g_err, "%s: %s", #x, s_ ? s_ : "?");                 \
            return RG_ECUDA;                                                            \
        }                                                                               \
    } while (0)

int rg_init(const char *cubin_path)
{
    CUdevice dev;
    CUcontext ctx;
    CK(cuInit(0));
    CK(cuDeviceGet(&dev, 0));
    CK(cuDevicePrimaryCtxRetain(&ctx, dev));
    CK(cuCtxSetCurrent(ctx));
    CK(cuModuleLoad(&g_mod, cubin_path));
    CK(cuModuleGetFunction(&g_l1, g_mod, "_Z31global_for_time_dedisperse_loopPfS_iiffi"));
    CK(cuModuleGetFunction(&g_opt, g_mod, "_Z19opt_dedisperse_loopPfS_iififfiii"));
    CK(cuModuleGetFunction(&g_sub, g_mod, "_Z22opt_dedisperse_subbandPfS_iiifffiii"));
    CK(cuModuleGetGlobal(&g_shifts, &g_shifts_bytes, g_mod, "dm_shifts"));
    g_loaded = 1;
    return RG_OK;
}

/* dedispersion_thread.cu:263 copies nchans*sizeof(int) bytes of the float table. */
static int upload_shifts(const float *dmshifts, int n)
{
    if ((size_t)n * sizeof(float) > g_shifts_bytes) {
        snprintf(g_err, sizeof g_err, "dm_shifts holds %zu bytes", g_shifts_bytes);
        return RG_EBOUNDS;
    }
    CK(cuMemcpyHtoD(g_shifts, dmshifts, (size_t)n * sizeof(float)));
    return RG_OK;
}

/* Largest shift the L1 kernel forms for DMs idx < ndm (both contraction variants). */
static long l1_max_shift(const float *dms, int nchans, float lowdm, float dmstep, float tsamp,
                         int ndm)
{
    float ms = lowdm / tsamp, md = dmstep / tsamp;
    long mx = 0;
    for (int d = 0; d < ndm; d++) {
        float a = fmaf((float)(unsigned)d, md, ms);
        float b = ms + (float)(unsigned)d * md;
        for (int c = 0; c < nchans; c++) {
            long s1 = (long)truncf(dms[c] * a), s2 = (long)truncf(dms[c] * b);
            if (s1 > mx) mx = s1;
            if (s2 > mx) mx = s2;
        }
    }
    return mx;
}

/* Largest element index the opt kernel reads (dedispersion_kernel.cu:70-71), replaying its
 * int + float index sum, for both contraction variants of start + i*step. */
static long opt_max_index(const float *dms, int nchans, int chanfactor, long stride, int nsamp,
                          float startdm, float dmstep, float tsamp, int ndm, long inshift)
{
    long mx = 0;
    for (int d = 0; d < ndm; d++) {
        float sts[2] = {fmaf((float)(unsigned)d, dmstep, startdm) / tsamp,
                        (startdm + (float)(unsigned)d * dmstep) / tsamp};
        for (int v = 0; v < 2; v++)
            for (int c = 0; c < nchans; c++) {
                float f = floorf(dms[c * chanfactor] * sts[v]);
                float sum = (float)(int)((long)c * stride) + f;
                long idx = inshift + (long)(int)sum + nsamp - 1;
                if (idx > mx) mx = idx;
            }
    }
    return mx;
}

static int launch(CUfunction f, unsigned gx, unsigned gy, unsigned bx, unsigned by,
                  unsigned smem, void **args)
{
    CK(cuLaunchKernel(f, gx, gy, 1, bx, by, 1, smem, 0, args, 0));
    return RG_OK;
}

static int timed_begin(CUevent *a, CUevent *b)
{
    CK(cuEventCreate(a, CU_EVENT_DEFAULT));
    CK(cuEventCreate(b, CU_EVENT_DEFAULT));
    CK(cuEventRecord(*a, 0));
    return RG_OK;
}

static int timed_end(CUevent a, CUevent b, float *ms)
{
    CK(cuEventRecord(b, 0));
    CK(cuEventSynchronize(b));
    CK(cuEventElapsedTime(ms, a, b));
    cuEventDestroy(a);
    cuEventDestroy(b);
    return RG_OK;
}

/* Brute force.  kind 0: global_for_time_dedisperse_loop launched as dedispersion_thread.cu:
 * 69-87; kind 1: opt_dedisperse_loop launched as dedispersion_thread.cu:229-234.  Input is
 * channel-major [nchans][nsamp+maxshift]; output [tdms][nsamp], zeroed first (:324). */
int rg_brute(int kind, const float *in, int nsamp, int nchans, int maxshift, float lowdm,
             float dmstep, float tsamp, int tdms, const float *dmshifts, float *out,
             float *kernel_ms)
{
    if (!g_loaded) return RG_ENOTLOADED;
    int rc = upload_shifts(dmshifts, nchans);
    if (rc) return rc;
    long stride = (long)nsamp + maxshift;
    long in_elems = stride * nchans;
    long slack = 1 << 16;
    long need;
    if (kind == 0) {
        long tmax = (long)(nsamp / 210) * 210 - 1;
        need = (long)(nchans - 1) * stride + tmax +
               l1_max_shift(dmshifts, nchans, lowdm, dmstep, tsamp, (tdms / 32) * 32) + 1;
    } else {
        need = opt_max_index(dmshifts, nchans, 1, stride, nsamp, lowdm, dmstep, tsamp, tdms, 0) + 1;
    }
    if (need > in_elems + slack) {
        snprintf(g_err, sizeof g_err, "reads up to %ld of %ld elements", need, in_elems + slack);
        return RG_EBOUNDS;
    }
    CUdeviceptr din, dout;
    size_t out_bytes = (size_t)tdms * (size_t)nsamp * sizeof(float);
    CK(cuMemAlloc(&din, (size_t)(in_elems + slack) * sizeof(float)));
    CK(cuMemAlloc(&dout, out_bytes));
    CK(cuMemsetD8(din, 0, (size_t)(in_elems + slack) * sizeof(float)));
    CK(cuMemcpyHtoD(din, in, (size_t)in_elems * sizeof(float)));
    CK(cuMemsetD8(dout, 0, out_bytes));
    CUevent e0, e1;
    if ((rc = timed_begin(&e0, &e1))) return rc;
    if (kind == 0) {
        int a_nsamp = nsamp, a_nchans = nchans, a_ms = maxshift;
        float a_sd = lowdm / tsamp, a_st = dmstep / tsamp;
        void *args[] = {&dout, &din, &a_nsamp, &a_nchans, &a_sd, &a_st, &a_ms};
        if (nsamp / 210 > 0 && tdms / 32 > 0)
            if ((rc = launch(g_l1, (unsigned)(nsamp / 210), (unsigned)(tdms / 32), 15, 32, 0, args)))
                return rc;
    } else {
        int a_nsamp = nsamp, a_nchans = nchans, a_cf = 1, a_ms = maxshift, a_in = 0, a_out = 0;
        float a_ts = tsamp, a_sd = lowdm, a_st = dmstep;
        void *args[] = {&dout, &din, &a_nsamp, &a_nchans, &a_ts, &a_cf, &a_sd, &a_st, &a_ms,
                        &a_in, &a_out};
        if ((rc = launch(g_opt, (unsigned)(nsamp / 128), (unsigned)tdms, 128, 1, 0, args)))
            return rc;
    }
    if ((rc = timed_end(e0, e1, kernel_ms))) return rc;
    CK(cuMemcpyDtoH(out, dout, out_bytes));
    CK(cuMemFree(din));
    CK(cuMemFree(dout));
    return RG_OK;
}

/* One subband pass with binsize 1 on one device: stage 1 as dedispersion_thread.cu:146-172,
 * stage 2 as :185-210 (the D2D copy at :180 is replaced by reading stage 1's buffer).
 * z: [ncalls][nsubs][nsamp+tempval]; out: [ncalls*calldms][nsamp]. */
int rg_subband(const float *in, int nsamp, int nchans, int maxshift, int nsubs, int tempval,
               float lowdm, float sub_dmstep, int ncalls, float dmstep, int calldms, float tsamp,
               const float *dmshifts, float *z_out, float *out, float *kernel_ms)
{
    if (!g_loaded) return RG_ENOTLOADED;
    int rc = upload_shifts(dmshifts, nchans);
    if (rc) return rc;
    long stride = (long)nsamp + maxshift;
    long in_elems = stride * nchans, slack = 1 << 16;
    long n1 = (long)nsamp + tempval;
    int cps = nchans / nsubs;
    /* stage-1 reads: c*stride + (int)(dms[c]*st - tv) + s, s < n1 */
    long need1 = 0;
    for (int j = 0; j < ncalls; j++) {
        float sts[2] = {fmaf((float)(unsigned)j, sub_dmstep, lowdm) / tsamp,
                        (lowdm + (float)(unsigned)j * sub_dmstep) / tsamp};
        for (int v = 0; v < 2; v++)
            for (int c = 0; c < nchans; c++) {
                int tv = (int)(dmshifts[(c / cps) * cps] * sts[v]);
                float a = fmaf(dmshifts[c], sts[v], -(float)tv);
                float b = dmshifts[c] * sts[v] - (float)tv;
                long s = (long)(int)a > (long)(int)b ? (long)(int)a : (long)(int)b;
                long idx = (long)c * stride + s + n1;
                if (idx > need1) need1 = idx;
            }
    }
    if (need1 > in_elems + slack) {
        snprintf(g_err, sizeof g_err, "stage 1 reads up to %ld of %ld", need1, in_elems + slack);
        return RG_EBOUNDS;
    }
    long z_elems = (long)ncalls * nsubs * n1;
    long need2 = 0;
    for (int j = 0; j < ncalls; j++) {
        float half = ((float)calldms * dmstep) / 2.0f;
        float dm0 = (lowdm + sub_dmstep * (float)j) - half;
        if (!(dm0 > 0.0f)) dm0 = 0.0f;
        long idx = opt_max_index(dmshifts, nsubs, cps, n1, nsamp, dm0, dmstep, tsamp, calldms,
                                 (long)j * n1 * nsubs) + 1;
        if (idx > need2) need2 = idx;
    }
    if (need2 > z_elems + slack) {
        snprintf(g_err, sizeof g_err, "stage 2 reads up to %ld of %ld", need2, z_elems + slack);
        return RG_EBOUNDS;
    }
    CUdeviceptr din, dz, dout;
    size_t out_bytes = (size_t)ncalls * calldms * (size_t)nsamp * sizeof(float);
    CK(cuMemAlloc(&din, (size_t)(in_elems + slack) * sizeof(float)));
    CK(cuMemAlloc(&dz, (size_t)(z_elems + slack) * sizeof(float)));
    CK(cuMemAlloc(&dout, out_bytes));
    CK(cuMemsetD8(din, 0, (size_t)(in_elems + slack) * sizeof(float)));
    CK(cuMemcpyHtoD(din, in, (size_t)in_elems * sizeof(float)));
    CK(cuMemsetD8(dz, 0, (size_t)(z_elems + slack) * sizeof(float)));
    CK(cuMemsetD8(dout, 0, out_bytes));
    CUevent e0, e1;
    if ((rc = timed_begin(&e0, &e1))) return rc;
    {
        int a_n = (int)n1, a_nc = nchans, a_ns = nsubs, a_ms = maxshift - tempval, a_i = 0, a_o = 0;
        float a_sd = lowdm, a_st = sub_dmstep, a_ts = tsamp;
        void *args[] = {&dz, &din, &a_n, &a_nc, &a_ns, &a_sd, &a_st, &a_ts, &a_ms, &a_i, &a_o};
        if ((rc = launch(g_sub, (unsigned)(n1 / 128), (unsigned)ncalls, 128, 1, 0, args)))
            return rc;
    }
    for (int j = 0; j < ncalls; j++) {
        float half = ((float)calldms * dmstep) / 2.0f;
        float dm0 = (lowdm + sub_dmstep * (float)j) - half;
        if (!(dm0 > 0.0f)) dm0 = 0.0f;
        int a_n = nsamp, a_nc = nsubs, a_cf = cps, a_ms = tempval;
        int a_i = (int)((long)j * n1 * nsubs), a_o = (int)((long)j * nsamp * calldms);
        float a_ts = tsamp, a_sd = dm0, a_st = dmstep;
        void *args[] = {&dout, &dz, &a_n, &a_nc, &a_ts, &a_cf, &a_sd, &a_st, &a_ms, &a_i, &a_o};
        if ((rc = launch(g_opt, (unsigned)(nsamp / 128), (unsigned)calldms, 128, 1, 128, args)))
            return rc;
    }
    if ((rc = timed_end(e0, e1, kernel_ms))) return rc;
    if (z_out) CK(cuMemcpyDtoH(z_out, dz, (size_t)z_elems * sizeof(float)));
    CK(cuMemcpyDtoH(out, dout, out_bytes));
    CK(cuMemFree(din));
    CK(cuMemFree(dz));
    CK(cuMemFree(dout));
    return RG_OK;
}

/* ---- prototype kernels (src/prototypes/detrend.cu, src/prototypes/rfi_clipper.cu) ---- */

static CUmodule g_mod_dt, g_mod_rfi;
static CUfunction g_detrend, g_rfi;
static int g_proto_loaded;

/* Loads oracle/_ref/ref_detrend.cubin and oracle/_ref/ref_rfi.cubin (after rg_init). */
int rg_init_proto(const char *detrend_cubin, const char *rfi_cubin)
{
    if (!g_loaded) return RG_ENOTLOADED;
    CK(cuModuleLoad(&g_mod_dt, detrend_cubin));
    CK(cuModuleGetFunction(&g_detrend, g_mod_dt, "_Z17detrend_normalisePfi"));
    CK(cuModuleLoad(&g_mod_rfi, rfi_cubin));
    CK(cuModuleGetFunction(&g_rfi, g_mod_rfi, "_Z12rfi_clippingPfS_ii"));
    g_proto_loaded = 1;
    return RG_OK;
}

/* detrend_normalise launched as detrend.cu:139: grid (nsamp/len, ndms), 256 threads, on
 * y [ndms][nsamp] in place.  Every index the kernel forms, blockIdx.y*gridDim.x*len +
 * blockIdx.x*len + i with i < len, stays below ndms*nsamp when nsamp is a multiple of len;
 * its int index needs ndms*nsamp < 2^31. */
int rg_detrend(float *y, int ndms, int nsamp, int len, float *kernel_ms)
{
    if (!g_proto_loaded) return RG_ENOTLOADED;
    if (len <= 0 || nsamp <= 0 || ndms <= 0 || nsamp % len != 0 ||
        (long)ndms * nsamp >= 2147483647L || nsamp / len > 2147483647 || ndms > 65535) {
        snprintf(g_err, sizeof g_err, "detrend: shape %d x %d, len %d not launchable", ndms,
                 nsamp, len);
        return RG_EBOUNDS;
    }
    size_t bytes = (size_t)ndms * (size_t)nsamp * sizeof(float);
    CUdeviceptr d;
    CK(cuMemAlloc(&d, bytes));
    CK(cuMemcpyHtoD(d, y, bytes));
    int a_len = len;
    void *args[] = {&d, &a_len};
    CUevent e0, e1;
    int rc;
    if ((rc = timed_begin(&e0, &e1))) return rc;
    if ((rc = launch(g_detrend, (unsigned)(nsamp / len), (unsigned)ndms, 256, 1, 0, args)))
        return rc;
    if ((rc = timed_end(e0, e1, kernel_ms))) return rc;
    CK(cuMemcpyDtoH(y, d, bytes));
    CK(cuMemFree(d));
    return RG_OK;
}

/* rfi_clipping launched as rfi_clipper.cu:135: grid (1, nrows), blockdim threads, blockdim*4
 * bytes of dynamic shared memory, on x [nrows][nsamp] in place; means[nrows] receives the row
 * means.  The kernel's clip loop calls __syncthreads() once per iteration, so every thread
 * must run the same number of iterations: nsamp must be a multiple of blockdim (refused
 * otherwise).  Its static shared array holds 1024 entries, one per thread. */
int rg_rfi_clip(float *x, int nrows, int nsamp, int blockdim, float *means, float *kernel_ms)
{
    if (!g_proto_loaded) return RG_ENOTLOADED;
    if (blockdim <= 0 || blockdim > 1024 || (blockdim & 31) || nsamp <= 0 || nrows <= 0 ||
        nsamp % blockdim != 0 || nrows > 65535 || (long)nrows * nsamp >= 2147483647L) {
        snprintf(g_err, sizeof g_err, "rfi: %d rows x %d, %d threads not launchable", nrows,
                 nsamp, blockdim);
        return RG_EBOUNDS;
    }
    size_t bytes = (size_t)nrows * (size_t)nsamp * sizeof(float);
    CUdeviceptr d, dm;
    CK(cuMemAlloc(&d, bytes));
    CK(cuMemAlloc(&dm, (size_t)nrows * sizeof(float)));
    CK(cuMemcpyHtoD(d, x, bytes));
    CK(cuMemsetD8(dm, 0, (size_t)nrows * sizeof(float)));
    int a_n = nsamp, a_r = nrows;
    void *args[] = {&d, &dm, &a_n, &a_r};
    CUevent e0, e1;
    int rc;
    if ((rc = timed_begin(&e0, &e1))) return rc;
    if ((rc = launch(g_rfi, 1, (unsigned)nrows, (unsigned)blockdim, 1, (unsigned)blockdim * 4,
                     args)))
        return rc;
    if ((rc = timed_end(e0, e1, kernel_ms))) return rc;
    CK(cuMemcpyDtoH(x, d, bytes));
    CK(cuMemcpyDtoH(means, dm, (size_t)nrows * sizeof(float)));
    CK(cuMemFree(d));
    CK(cuMemFree(dm));
    return RG_OK;
}
