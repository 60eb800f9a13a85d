// sigproc.cu -- sigproc filterbank ingest: header reader and writer, and the device kernel that
// unpacks time-major spectra and corner-turns them into the channel-major block the
// dedispersion kernels read.
//
// Reference: header parsing src/mdsm/file_handler.cpp:33-187, sample unpack :193-290 (1/2/4-bit
// samples least-significant field first, 16-bit read unsigned), the host corner turn of
// src/MDSM.cpp:100-125 and src/pelican-mdsm/modules/MdsmModule.cpp:135-151 (with optional
// channel inversion), and the series header of
// src/pelican-mdsm/modules/DedispersedDataWriter.cpp:49-63.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <type_traits>

#include "internal.h"

namespace mdsm {

// Float rows to uint8 rows where every value is an integer 0..255 (the float blocks of the
// stage interface usually hold 8-bit samples): four columns per thread, float4 loads and
// 4-byte stores where the row allows.
__global__ void __launch_bounds__(256)
    k_pack_u8_rows(const float *__restrict__ in, long long in_stride, int nrows, long long ncols,
                   uint8_t *__restrict__ out, long long out_stride, unsigned *__restrict__ flag)
{
    const int r = blockIdx.y;
    const long long t = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * 4;
    if (r >= nrows || t >= ncols) return;
    const float *row = in + (size_t)r * in_stride;
    float v[4];
    if (t + 3 < ncols) {
        const float4 q = *reinterpret_cast<const float4 *>(row + t);
        v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
    } else {
        for (int e = 0; e < 4; ++e) v[e] = t + e < ncols ? row[t + e] : 0.0f;
    }
    uint32_t packed = 0;
    bool bad = false;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const unsigned u = __float2uint_rz(v[e]);
        // bit-exact round trip: rejects fractions, -0, NaN and values past 255
        bad |= u > 255u || __float_as_uint(v[e]) != __float_as_uint(__uint2float_rn(u));
        packed |= (u & 0xFFu) << (8 * e);
    }
    if (bad) atomicOr(flag, 1u);
    uint8_t *orow = out + (size_t)r * out_stride;
    if (t + 3 < ncols) {
        *reinterpret_cast<uint32_t *>(orow + t) = packed;
    } else {
        for (int e = 0; e < 4 && t + e < ncols; ++e) orow[t + e] = (uint8_t)(packed >> (8 * e));
    }
}

mdsm_status pack_u8_rows(const float *in, long long in_stride, int nrows, long long ncols,
                         uint8_t *out, long long out_stride, unsigned *flag, cudaStream_t st)
{
    if (nrows <= 0 || ncols <= 0) return MDSM_OK;
    if (((uintptr_t)in & 15) || (in_stride & 3) || ((uintptr_t)out & 3) || (out_stride & 3))
        return fail(MDSM_EINVAL, "pack_u8_rows: rows must be 16-byte (float) / 4-byte aligned");
    const long long quads = (ncols + 3) / 4;
    if (nrows > 65535) return fail(MDSM_EINVAL, "pack_u8_rows: too many rows");
    dim3 grid((unsigned)((quads + 255) / 256), (unsigned)nrows);
    k_pack_u8_rows<<<grid, 256, 0, st>>>(in, in_stride, nrows, ncols, out, out_stride, flag);
    MDSM_CUDA_TRY(cudaGetLastError());
    return MDSM_OK;
}

// One CTA moves a tile of 32 spectra x 32 channels: loads walk channels (consecutive in the
// raw stream), stores walk time (consecutive in the output rows).
template <int NBITS, typename TOut>
__global__ void __launch_bounds__(256)
    k_unpack_transpose(const uint8_t *__restrict__ raw, long long nspectra, int nchans, int invert,
                       TOut *__restrict__ out, long long out_stride, long long col0)
{
    __shared__ TOut tile[32][33];
    const long long t0 = (long long)blockIdx.x * 32;
    const int c0 = blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const long long t = t0 + ty + 8 * i;
        const int c = c0 + tx;
        TOut v = TOut(0);
        if (t < nspectra && c < nchans) {
            const long long idx = t * nchans + c;  // sample index in the stream
            if constexpr (NBITS == 8) {
                v = (TOut)raw[idx];
            } else if constexpr (NBITS == 16) {
                const uint16_t s = (uint16_t)(raw[2 * idx] | ((uint16_t)raw[2 * idx + 1] << 8));
                if constexpr (std::is_same<TOut, int16_t>::value)
                    v = (int16_t)((int32_t)s - ((s & 0x8000u) ? 65536 : 0));  // two's complement
                else
                    v = (TOut)s;
            } else if constexpr (NBITS == 32) {
                float f;
                memcpy(&f, raw + 4 * idx, 4);
                v = (TOut)f;
            } else {
                const long long bit = idx * NBITS;
                const unsigned b = raw[bit >> 3];
                v = (TOut)((b >> (bit & 7)) & ((1u << NBITS) - 1u));
            }
        }
        tile[ty + 8 * i][tx] = v;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int c = c0 + ty + 8 * i;
        const long long t = t0 + tx;
        if (t < nspectra && c < nchans) {
            const int co = invert ? nchans - 1 - c : c;
            out[(size_t)co * out_stride + col0 + t] = tile[tx][ty + 8 * i];
        }
    }
}

template <int NBITS>
static mdsm_status launch_unpack(const void *raw, long long nspectra, int nchans, int invert,
                                 void *out, int out_dtype, long long out_stride, long long col0,
                                 cudaStream_t st)
{
    dim3 grid((unsigned)((nspectra + 31) / 32), (unsigned)((nchans + 31) / 32));
    dim3 block(32, 8);
    const uint8_t *r = static_cast<const uint8_t *>(raw);
    switch (out_dtype) {
    case MDSM_U8:
        k_unpack_transpose<NBITS, uint8_t><<<grid, block, 0, st>>>(
            r, nspectra, nchans, invert, static_cast<uint8_t *>(out), out_stride, col0);
        break;
    case MDSM_U16:
        k_unpack_transpose<NBITS, uint16_t><<<grid, block, 0, st>>>(
            r, nspectra, nchans, invert, static_cast<uint16_t *>(out), out_stride, col0);
        break;
    case MDSM_I16:  // 16-bit samples read as two's-complement int16 (the int16 data form)
        if (NBITS == 32) return fail(MDSM_EINVAL, "unpack: float samples to int16 output");
        k_unpack_transpose<NBITS, int16_t><<<grid, block, 0, st>>>(
            r, nspectra, nchans, invert, static_cast<int16_t *>(out), out_stride, col0);
        break;
    case MDSM_F32:
        k_unpack_transpose<NBITS, float><<<grid, block, 0, st>>>(
            r, nspectra, nchans, invert, static_cast<float *>(out), out_stride, col0);
        break;
    default:
        return fail(MDSM_EINVAL, "unpack: output must be uint8, uint16, int16 or float32");
    }
    MDSM_CUDA_TRY(cudaGetLastError());
    return MDSM_OK;
}

}  // namespace mdsm

using namespace mdsm;

namespace {

// file_handler.cpp:33-49: an int32 length then that many characters; lengths outside 1..80
// give the string "ERROR".
bool get_string(FILE *f, std::string &s, long long &nbytes)
{
    int32_t n = 0;
    if (fread(&n, sizeof n, 1, f) != 1) return false;
    s = "ERROR";
    nbytes = 4;
    if (n > 80 || n < 1) return true;
    char buf[81];
    if (fread(buf, 1, (size_t)n, f) != (size_t)n) return false;
    buf[n] = 0;
    s = buf;
    nbytes += n;
    return true;
}

template <typename T>
bool get_val(FILE *f, T *v, long long &total)
{
    if (fread(v, sizeof(T), 1, f) != 1) return false;
    total += (long long)sizeof(T);
    return true;
}

void put_string(FILE *f, const char *s)
{
    const int32_t n = (int32_t)strlen(s);
    fwrite(&n, sizeof n, 1, f);
    fwrite(s, 1, (size_t)n, f);
}

template <typename T>
void put_val(FILE *f, const char *name, T v)
{
    put_string(f, name);
    fwrite(&v, sizeof(T), 1, f);
}

}  // namespace

extern "C" {

mdsm_status mdsm_sigproc_read_header(const char *path, mdsm_sigproc_header *h)
{
    if (!path || !h) return fail(MDSM_EINVAL, "null argument");
    FILE *f = fopen(path, "rb");
    if (!f) return fail(MDSM_EIO, std::string("cannot open ") + path);
    std::memset(h, 0, sizeof(*h));
    std::string s;
    long long nb = 0, total = 0;
    if (!get_string(f, s, nb) || s != "HEADER_START") {
        fclose(f);
        return fail(MDSM_EPARSE, "not a sigproc file (no HEADER_START)");
    }
    total = nb;
    bool raw_next = false, src_next = false;
    int chan_index = 0;
    bool ok = true;
    for (;;) {
        if (!get_string(f, s, nb)) {
            ok = false;
            break;
        }
        if (s == "HEADER_END") break;
        total += nb;
        const char *k = s.c_str();
        if (s == "rawdatafile") raw_next = true;
        else if (s == "source_name") src_next = true;
        else if (s == "FREQUENCY_START") chan_index = 0;
        else if (s == "FREQUENCY_END") {}
        else if (!strcmp(k, "az_start")) ok = get_val(f, &h->az_start, total);
        else if (!strcmp(k, "za_start")) ok = get_val(f, &h->za_start, total);
        else if (!strcmp(k, "src_raj")) ok = get_val(f, &h->src_raj, total);
        else if (!strcmp(k, "src_dej")) ok = get_val(f, &h->src_dej, total);
        else if (!strcmp(k, "tstart")) ok = get_val(f, &h->tstart, total);
        else if (!strcmp(k, "tsamp")) ok = get_val(f, &h->tsamp, total);
        else if (!strcmp(k, "period")) ok = get_val(f, &h->period, total);
        else if (!strcmp(k, "fch1")) ok = get_val(f, &h->fch1, total);
        else if (!strcmp(k, "fchannel")) {
            double v;
            ok = get_val(f, &v, total);
            chan_index++;
            h->fch1 = h->foff = 0.0;  // a frequency table is in use (file_handler.cpp:116-120)
            h->nfchannels = chan_index;
        } else if (!strcmp(k, "foff")) ok = get_val(f, &h->foff, total);
        else if (!strcmp(k, "nchans")) ok = get_val(f, &h->nchans, total);
        else if (!strcmp(k, "telescope_id")) ok = get_val(f, &h->telescope_id, total);
        else if (!strcmp(k, "machine_id")) ok = get_val(f, &h->machine_id, total);
        else if (!strcmp(k, "Telescope")) {
            long long n2 = 0;
            ok = get_string(f, s, n2);  // value skipped, not counted (as the reference)
        } else if (!strcmp(k, "data_type")) ok = get_val(f, &h->data_type, total);
        else if (!strcmp(k, "ibeam")) ok = get_val(f, &h->ibeam, total);
        else if (!strcmp(k, "nbeams")) ok = get_val(f, &h->nbeams, total);
        else if (!strcmp(k, "nbits")) ok = get_val(f, &h->nbits, total);
        else if (!strcmp(k, "barycentric")) ok = get_val(f, &h->barycentric, total);
        else if (!strcmp(k, "pulsarcentric")) ok = get_val(f, &h->pulsarcentric, total);
        else if (!strcmp(k, "nbins")) ok = get_val(f, &h->nbins, total);
        else if (!strcmp(k, "nsamples")) ok = get_val(f, &h->nsamples, total);
        else if (!strcmp(k, "nifs")) ok = get_val(f, &h->nifs, total);
        else if (!strcmp(k, "npuls")) {
            long v = 0;  // a C long in the file (file_handler.cpp:163-165)
            ok = get_val(f, &v, total);
            h->npuls = v;
        }
        else if (!strcmp(k, "refdm")) ok = get_val(f, &h->refdm, total);
        else if (raw_next) {
            snprintf(h->rawdatafile, sizeof h->rawdatafile, "%.80s", k);
            raw_next = false;
        } else if (src_next) {
            snprintf(h->source_name, sizeof h->source_name, "%.80s", k);
            src_next = false;
        } else {
            fclose(f);
            return fail(MDSM_EPARSE, std::string("sigproc header: unknown parameter ") + k);
        }
        if (!ok) break;
    }
    fclose(f);
    if (!ok) return fail(MDSM_EPARSE, "sigproc header: truncated");
    h->header_bytes = total + nb;  // file_handler.cpp:181-182
    return MDSM_OK;
}

// The header of a dedispersed-series file: one summed channel of 32-bit samples
// (DedispersedDataWriter.cpp:49-63).  Samples are appended by the caller.
mdsm_status mdsm_sigproc_write_series_header(const char *path, double fch1, double foff,
                                             double tsamp, double tstart)
{
    if (!path) return fail(MDSM_EINVAL, "null argument");
    FILE *f = fopen(path, "wb");
    if (!f) return fail(MDSM_EIO, std::string("cannot create ") + path);
    put_string(f, "HEADER_START");
    put_val<int32_t>(f, "machine_id", 0);
    put_val<int32_t>(f, "telescope_id", 0);
    put_val<int32_t>(f, "data_type", 1);
    put_val<double>(f, "fch1", fch1);
    put_val<double>(f, "foff", foff);
    put_val<int32_t>(f, "nchans", 1);
    put_val<double>(f, "tsamp", tsamp);
    put_val<int32_t>(f, "nbits", 32);
    put_val<double>(f, "tstart", tstart);
    put_val<int32_t>(f, "nifs", 1);
    put_string(f, "HEADER_END");
    const bool ok = fflush(f) == 0;
    fclose(f);
    return ok ? MDSM_OK : fail(MDSM_EIO, "write failed");
}

mdsm_status mdsm_unpack_device(const void *d_raw, long long nspectra, int nchans, int nbits,
                               int invert, void *d_out, int out_dtype, long long out_stride,
                               long long col0, void *stream)
{
    if (!d_raw || !d_out || nspectra < 0 || nchans <= 0 || col0 < 0)
        return fail(MDSM_EINVAL, "unpack: bad arguments");
    if ((long long)nchans * nbits % 8 != 0)
        return fail(MDSM_EINVAL, "unpack: a spectrum must fill whole bytes");
    if (nspectra == 0) return MDSM_OK;
    if (nspectra > 65535LL * 32 * 65535LL) return fail(MDSM_EINVAL, "unpack: block too long");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    switch (nbits) {
    case 1: return launch_unpack<1>(d_raw, nspectra, nchans, invert, d_out, out_dtype, out_stride, col0, st);
    case 2: return launch_unpack<2>(d_raw, nspectra, nchans, invert, d_out, out_dtype, out_stride, col0, st);
    case 4: return launch_unpack<4>(d_raw, nspectra, nchans, invert, d_out, out_dtype, out_stride, col0, st);
    case 8: return launch_unpack<8>(d_raw, nspectra, nchans, invert, d_out, out_dtype, out_stride, col0, st);
    case 16: return launch_unpack<16>(d_raw, nspectra, nchans, invert, d_out, out_dtype, out_stride, col0, st);
    case 32: return launch_unpack<32>(d_raw, nspectra, nchans, invert, d_out, out_dtype, out_stride, col0, st);
    }
    return fail(MDSM_EINVAL, "unpack: nbits must be 1, 2, 4, 8, 16 or 32");
}

}  // extern "C"
