// binning.cu -- time downsampling of channel-major blocks for downsampled DM passes.
//
// The reference downsamples with src/mdsm/dedispersion_kernel.cu:203-264 (mean of binsize
// samples, launched at src/mdsm/dedispersion_thread.cu:116-144) and the prototype
// src/prototypes/binner.cu:13-71 (sum / sqrt(binsize)), but both index the buffer as
// interleaved [t][c] while MDSM's blocks are channel-major [c][t], so passes with binsize > 1
// do not dedisperse the right samples there.  Here out[c][t] = f(sum_{k<b} in[c][t*b + k])
// on the channel-major layout, with f the plain sum (exact: integer samples widen to uint16 or
// int32), the mean, or sum / sqrt(b).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <type_traits>

#include "internal.h"

namespace mdsm {

template <typename TIn, typename TOut>
__global__ void k_downsample(const TIn *__restrict__ in, long long in_stride, long long nout,
                             int b, int mode, float scale, TOut *__restrict__ out,
                             long long out_stride)
{
    const int c = blockIdx.y;
    const TIn *r = in + (size_t)c * in_stride;
    TOut *o = out + (size_t)c * out_stride;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < nout;
         t += (long long)gridDim.x * blockDim.x) {
        const TIn *p = r + t * b;
        if (mode == 0) {
            long long acc = 0;
            double facc = 0.0;
            if (std::is_floating_point<TIn>::value) {
                for (int k = 0; k < b; ++k) facc = __dadd_rn(facc, (double)p[k]);
                o[t] = (TOut)facc;
            } else {
                for (int k = 0; k < b; ++k) acc += (long long)p[k];
                o[t] = (TOut)acc;
            }
        } else {
            float acc = 0.0f;
            for (int k = 0; k < b; ++k) acc = __fadd_rn(acc, (float)p[k]);
            o[t] = (TOut)__fmul_rn(acc, scale);
        }
    }
}

template <typename TIn, typename TOut>
static void launch_ds(const void *in, long long in_stride, int nchans, long long nout, int b,
                      int mode, float scale, void *out, long long out_stride, cudaStream_t st)
{
    dim3 grid((unsigned)std::min<long long>((nout + 255) / 256, 1024), (unsigned)nchans);
    k_downsample<TIn, TOut><<<grid, 256, 0, st>>>(static_cast<const TIn *>(in), in_stride, nout,
                                                  b, mode, scale, static_cast<TOut *>(out),
                                                  out_stride);
}

mdsm_status downsample(const void *in, int in_dtype, int nchans, long long in_stride,
                       long long len, int b, int mode, void *out, int out_dtype,
                       long long out_stride, cudaStream_t st)
{
    if (b < 1 || nchans <= 0 || len < 0) return fail(MDSM_EINVAL, "downsample: bad arguments");
    const long long nout = len / b;
    if (out_stride < nout) return fail(MDSM_ERANGE, "downsample: output pitch too small");
    if (nout == 0) return MDSM_OK;
    const float scale = mode == 1 ? 1.0f / (float)b : (mode == 2 ? 1.0f / sqrtf((float)b) : 1.0f);
    if (mode != 0 && out_dtype != MDSM_F32)
        return fail(MDSM_EINVAL, "downsample: mean and 1/sqrt(b) outputs are float32");
    if (mode == 0 && in_dtype == MDSM_U8 && out_dtype == MDSM_U16 && b > 257)
        return fail(MDSM_ERANGE, "downsample: uint16 sums hold at most 257 uint8 samples");
#define DS(TI, TO) launch_ds<TI, TO>(in, in_stride, nchans, nout, b, mode, scale, out, out_stride, st)
    if (in_dtype == MDSM_U8 && out_dtype == MDSM_U16) DS(uint8_t, uint16_t);
    else if (in_dtype == MDSM_U8 && out_dtype == MDSM_I32) DS(uint8_t, int32_t);
    else if (in_dtype == MDSM_U8 && out_dtype == MDSM_F32) DS(uint8_t, float);
    else if (in_dtype == MDSM_U16 && out_dtype == MDSM_I32) DS(uint16_t, int32_t);
    else if (in_dtype == MDSM_U16 && out_dtype == MDSM_F32) DS(uint16_t, float);
    else if (in_dtype == MDSM_I16 && out_dtype == MDSM_I32) DS(int16_t, int32_t);
    else if (in_dtype == MDSM_I16 && out_dtype == MDSM_F32) DS(int16_t, float);
    else if (in_dtype == MDSM_F32 && out_dtype == MDSM_F32) DS(float, float);
    else return fail(MDSM_EINVAL, "downsample: unsupported sample types");
#undef DS
    MDSM_CUDA_TRY(cudaGetLastError());
    return MDSM_OK;
}

}  // namespace mdsm

extern "C" mdsm_status mdsm_downsample_device(const void *d_in, int in_dtype, int nchans,
                                              long long in_stride, long long len, int binsize,
                                              int mode, void *d_out, int out_dtype,
                                              long long out_stride, void *stream)
{
    if (!d_in || !d_out) return mdsm::fail(MDSM_EINVAL, "null argument");
    return mdsm::downsample(d_in, in_dtype, nchans, in_stride, len, binsize, mode, d_out,
                            out_dtype, out_stride, static_cast<cudaStream_t>(stream));
}
