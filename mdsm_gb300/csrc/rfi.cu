// rfi.cu -- RFI clipping of a channel-major filterbank block, in place on the device.
//
// src/prototypes/rfi_clipper.cu:8-67 clips each row: mean and sigma over the row, then samples
// with |x - mean| >= 4 sigma are replaced by the mean.  Here the same rule runs per channel
// (over time) and then per spectrum (over channels at one time sample).  Two defects of the
// prototype are not reproduced: its accumulators start uninitialised (:33) and it also clips
// |x - mean| <= sigma/4 (:61).  Statistics are exact for integer samples (int64 sums) and use
// a fixed left-to-right order of double sums for float samples, so the device result equals
// the oracle's bit for bit.
#include <cuda_runtime.h>
#include <stdint.h>

#include "internal.h"

namespace mdsm {

template <typename T>
struct Clip;

template <>
struct Clip<uint8_t> {
    static __device__ __forceinline__ uint8_t from(double v)
    {
        int r = __double2int_rn(v);
        return (uint8_t)min(max(r, 0), 255);
    }
};
template <>
struct Clip<uint16_t> {
    static __device__ __forceinline__ uint16_t from(double v)
    {
        int r = __double2int_rn(v);
        return (uint16_t)min(max(r, 0), 65535);
    }
};
template <>
struct Clip<int16_t> {
    static __device__ __forceinline__ int16_t from(double v)
    {
        int r = __double2int_rn(v);
        return (int16_t)min(max(r, -32768), 32767);
    }
};
template <>
struct Clip<float> {
    static __device__ __forceinline__ float from(double v) { return __double2float_rn(v); }
};

template <typename T>
constexpr bool is_int_sample()
{
    return !std::is_same<T, float>::value;
}

__device__ __forceinline__ void mean_sigma_int(long long s1, long long s2, long long n, double *mu,
                                               double *sig)
{
    const double m = __ddiv_rn((double)s1, (double)n);
    const double var = __dadd_rn(__ddiv_rn((double)s2, (double)n), -__dmul_rn(m, m));
    *mu = m;
    *sig = var > 0.0 ? __dsqrt_rn(var) : 0.0;
}

// One CTA per channel: statistics over the row, then the clip.
template <typename T>
__global__ void __launch_bounds__(256)
    k_clip_channels(T *__restrict__ x, long long stride, long long len, double k)
{
    extern __shared__ __align__(16) unsigned char sm[];
    T *row = x + (size_t)blockIdx.x * stride;
    __shared__ double s_mu, s_sig;
    if constexpr (is_int_sample<T>()) {
        __shared__ long long r1[256], r2[256];
        long long a1 = 0, a2 = 0;
        for (long long i = threadIdx.x; i < len; i += blockDim.x) {
            const long long v = (long long)row[i];
            a1 += v;
            a2 += v * v;
        }
        r1[threadIdx.x] = a1;
        r2[threadIdx.x] = a2;
        __syncthreads();
        for (int o = 128; o > 0; o >>= 1) {
            if ((int)threadIdx.x < o) {
                r1[threadIdx.x] += r1[threadIdx.x + o];
                r2[threadIdx.x] += r2[threadIdx.x + o];
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) mean_sigma_int(r1[0], r2[0], len, &s_mu, &s_sig);
    } else {
        // runs of 1024 summed left to right, partials summed left to right
        double2 *part = reinterpret_cast<double2 *>(sm);
        const long long nch = (len + 1023) / 1024;
        for (long long c = threadIdx.x; c < nch; c += blockDim.x) {
            const long long c0 = c * 1024, c1 = min(c0 + 1024, len);
            double p1 = 0.0, p2 = 0.0;
            for (long long i = c0; i < c1; ++i) {
                const double v = (double)row[i];
                p1 = __dadd_rn(p1, v);
                p2 = __fma_rn(v, v, p2);  // v*v exact: same as dmul + dadd
            }
            part[c] = make_double2(p1, p2);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double s1 = 0.0, s2 = 0.0;
            for (long long c = 0; c < nch; ++c) {
                s1 = __dadd_rn(s1, part[c].x);
                s2 = __dadd_rn(s2, part[c].y);
            }
            const double m = __ddiv_rn(s1, (double)len);
            const double var = __dadd_rn(__ddiv_rn(s2, (double)len), -__dmul_rn(m, m));
            s_mu = m;
            s_sig = var > 0.0 ? __dsqrt_rn(var) : 0.0;
        }
    }
    __syncthreads();
    const double mu = s_mu, lim = __dmul_rn(k, s_sig);
    const T rep = Clip<T>::from(mu);
    for (long long i = threadIdx.x; i < len; i += blockDim.x) {
        const double v = (double)row[i];
        if (fabs(__dadd_rn(v, -mu)) >= lim) row[i] = rep;
    }
}

// One thread per time sample: statistics over the channels, then the clip.
template <typename T>
__global__ void k_clip_spectra(T *__restrict__ x, int nchans, long long stride, long long len,
                               double k)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= len) return;
    double mu, sig;
    if constexpr (is_int_sample<T>()) {
        long long s1 = 0, s2 = 0;
        for (int c = 0; c < nchans; ++c) {
            const long long v = (long long)x[(size_t)c * stride + t];
            s1 += v;
            s2 += v * v;
        }
        mean_sigma_int(s1, s2, nchans, &mu, &sig);
    } else {
        double s1 = 0.0, s2 = 0.0;
        for (int c0 = 0; c0 < nchans; c0 += 1024) {
            const int c1 = min(c0 + 1024, nchans);
            double p1 = 0.0, p2 = 0.0;
            for (int c = c0; c < c1; ++c) {
                const double v = (double)x[(size_t)c * stride + t];
                p1 = __dadd_rn(p1, v);
                p2 = __fma_rn(v, v, p2);  // v*v exact: same as dmul + dadd
            }
            s1 = __dadd_rn(s1, p1);
            s2 = __dadd_rn(s2, p2);
        }
        mu = __ddiv_rn(s1, (double)nchans);
        const double var = __dadd_rn(__ddiv_rn(s2, (double)nchans), -__dmul_rn(mu, mu));
        sig = var > 0.0 ? __dsqrt_rn(var) : 0.0;
    }
    const double lim = __dmul_rn(k, sig);
    const T rep = Clip<T>::from(mu);
    for (int c = 0; c < nchans; ++c) {
        T *p = x + (size_t)c * stride + t;
        if (fabs(__dadd_rn((double)*p, -mu)) >= lim) *p = rep;
    }
}

template <typename T>
static mdsm_status clip_t(T *x, int nchans, long long stride, long long len, double kc, double ks,
                          cudaStream_t st)
{
    if (kc > 0.0) {
        size_t smem = 0;
        if (!is_int_sample<T>()) {
            smem = (size_t)((len + 1023) / 1024) * sizeof(double2);
            if (smem > 200 * 1024) return fail(MDSM_EINVAL, "rfi clip: row too long");
            MDSM_CUDA_TRY(cudaFuncSetAttribute(k_clip_channels<T>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)smem));
        }
        k_clip_channels<T><<<nchans, 256, smem, st>>>(x, stride, len, kc);
        MDSM_CUDA_TRY(cudaGetLastError());
    }
    if (ks > 0.0) {
        k_clip_spectra<T><<<(unsigned)((len + 255) / 256), 256, 0, st>>>(x, nchans, stride, len, ks);
        MDSM_CUDA_TRY(cudaGetLastError());
    }
    return MDSM_OK;
}

mdsm_status rfi_clip(void *d_x, int dtype, int nchans, long long stride, long long len,
                     double k_chan, double k_spec, cudaStream_t st)
{
    switch (dtype) {
    case MDSM_U8: return clip_t(static_cast<uint8_t *>(d_x), nchans, stride, len, k_chan, k_spec, st);
    case MDSM_U16:
        return clip_t(static_cast<uint16_t *>(d_x), nchans, stride, len, k_chan, k_spec, st);
    case MDSM_I16:
        return clip_t(static_cast<int16_t *>(d_x), nchans, stride, len, k_chan, k_spec, st);
    case MDSM_F32: return clip_t(static_cast<float *>(d_x), nchans, stride, len, k_chan, k_spec, st);
    }
    return fail(MDSM_EINVAL, "rfi clip: unknown sample type");
}

}  // namespace mdsm
