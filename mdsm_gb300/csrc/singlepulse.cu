// singlepulse.cu -- the single-pulse prototype's search (src/prototypes/singlepulse.cpp:148-300)
// on the device, in its template form.
//
// For every DM row, in chunks of chunk_len samples, and every width of {1} + the downfactor
// ladder {2, 3, 4, 6, 9, 14, 20, 30, 45, 70, 100, 150} up to max_downfact (:20,161-164): the
// response of the centred boxcar template (:41-67; window [t - w/2, t - w/2 + w), scaled by
// 1/sqrt(w)), thresholded (:240-245,261-270); each width's list of a chunk is pruned by
// pruneRelated as the prototype writes it (:90-120), and one DM's survivors, in (chunk, width,
// sample) order, by pruneRelatedDownfactors (:122-146).  The prototype convolves by FFT; here the
// response is the exact template sum, in FP32, left to right from the window's first sample
// (zero outside the series), then (sum - w*mean) * 1/(sigma*sqrt(w)) with mean 0 and sigma 1
// unless the row's statistics are asked for.  The prototype's main loop has defects that are
// not reproduced (its first chunk reads DM row 0, it searches each chunk's samples only up to
// chunk_len - overlap, drops a trailing partial chunk, stores the value of the wrong list entry
// and the list index as the sample, and keeps the candidates its downfactor mask marks as
// pruned); the two prune functions are reproduced as written.
//
// Device part: one CTA per (chunk, DM).  The chunk's samples plus the widest template's halo are
// staged in shared memory; each thread sums four consecutive window starts at once, reading one
// new sample per step, and emits the response of every ladder width as its window length is
// reached; responses over the threshold set bits in per-width masks.  Then one lane per width
// walks its mask in sample order and applies pruneRelated (a crossing is pruned iff an earlier
// kept crossing within w/2 samples is not both at a list index that is a multiple of 256 and no
// stronger than it: the prototype's `mask[j] = i`).  Survivors go to a global list; the host
// sorts that short list and applies pruneRelatedDownfactors, which depends on list order across
// chunks.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <vector>

#include "internal.h"

namespace mdsm {

namespace {

constexpr int kSpThreads = 256;
constexpr int kSpR = 4;          // window starts per thread per pass
constexpr int kSpMaxWidths = 13; // 1 + the 12 downfactors
constexpr int kSpMaxChunk = 32768;
const int kSpLadder[12] = {2, 3, 4, 6, 9, 14, 20, 30, 45, 70, 100, 150};

struct SpWidths {
    int nw;
    int w[kSpMaxWidths];
};

template <typename T>
__device__ __forceinline__ float sp_load(const T *r, long long t, long long n)
{
    if (t < 0 || t >= n) return 0.0f;
    if constexpr (std::is_same<T, float>::value)
        return __ldg(r + t);
    else
        return (float)__ldg(r + t);
}

// Response of width w at chunk position p (xs[p + hmax] is the sample at the chunk's start +
// p): the same additions in the same order as the sweep.
__device__ __forceinline__ float sp_value(const float *xs, int p, int hmax, int w, float mu_f,
                                          float inv)
{
    const int s = p + hmax - w / 2;
    float acc = xs[s];
    for (int k = 1; k < w; ++k) acc = __fadd_rn(acc, xs[s + k]);
    return __fmul_rn(__fadd_rn(acc, -__fmul_rn((float)w, mu_f)), inv);
}

template <typename T>
__global__ void __launch_bounds__(kSpThreads)
    k_singlepulse(const T *__restrict__ y, long long n, int chunk_len, SpWidths W,
                  double threshold, const double2 *__restrict__ musig,
                  DevCand *__restrict__ cands, unsigned long long *__restrict__ count,
                  long long cap)
{
    extern __shared__ __align__(16) unsigned char sm[];
    const int nw = W.nw, wmax = W.w[nw - 1], hmax = wmax / 2;
    const int d = blockIdx.y;
    const long long c0 = (long long)blockIdx.x * chunk_len;
    const int lc = (int)min((long long)chunk_len, n - c0);  // positions of this chunk
    const int nwords = (chunk_len + 31) / 32;
    const int nstart = lc + hmax;                           // window starts of the chunk
    // staged samples: xs[i] = sample c0 - hmax + i, i < nstart + wmax + kSpR (0 outside)
    const int nx = nstart + wmax + kSpR;
    float *xs = reinterpret_cast<float *>(sm);
    unsigned *bits = reinterpret_cast<unsigned *>(xs + ((nx + 3) & ~3));

    double mu = 0.0, sig = 1.0;
    if (musig) {
        mu = musig[d].x;
        sig = musig[d].y;
        if (!(sig > 0.0)) return;
    }
    const float mu_f = __double2float_rn(mu);
    const float thr = __double2float_rn(threshold);
    __shared__ float inv_w[kSpMaxWidths];
    if (threadIdx.x < nw)
        inv_w[threadIdx.x] = __double2float_rn(
            __ddiv_rn(1.0, __dmul_rn(sig, __dsqrt_rn((double)W.w[threadIdx.x]))));
    const T *r = y + (size_t)d * (size_t)n;
    for (int i = threadIdx.x; i < nx; i += kSpThreads) xs[i] = sp_load(r, c0 - hmax + i, n);
    for (int i = threadIdx.x; i < nw * nwords; i += kSpThreads) bits[i] = 0u;
    __syncthreads();

    // sweep: thread handles starts s0 .. s0 + 3; at step k every accumulator holds the sum of
    // k + 1 samples from its start, which is the response window of width k + 1
    for (int s0 = threadIdx.x * kSpR; s0 < nstart; s0 += kSpThreads * kSpR) {
        float win[kSpR], acc[kSpR];
#pragma unroll
        for (int j = 0; j < kSpR; ++j) acc[j] = win[j] = xs[s0 + j];
        int li = 0;
        for (int k = 0; k < wmax; ++k) {
            if (k > 0) {
#pragma unroll
                for (int j = 0; j < kSpR - 1; ++j) win[j] = win[j + 1];
                win[kSpR - 1] = xs[s0 + kSpR - 1 + k];
#pragma unroll
                for (int j = 0; j < kSpR; ++j) acc[j] = __fadd_rn(acc[j], win[j]);
            }
            if (k + 1 == W.w[li]) {
                const int w = k + 1;
                const float wm = __fmul_rn((float)w, mu_f), inv = inv_w[li];
#pragma unroll
                for (int j = 0; j < kSpR; ++j) {
                    const int p = s0 + j - hmax + w / 2;  // chunk position of this window
                    if (p < 0 || p >= lc) continue;
                    const float v = __fmul_rn(__fadd_rn(acc[j], -wm), inv);
                    if (v >= thr) atomicOr(&bits[li * nwords + (p >> 5)], 1u << (p & 31));
                }
                ++li;
            }
        }
    }
    __syncthreads();

    // per width: pruneRelated in list order (lane 0 of one warp per width)
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int li = warp; li < nw; li += kSpThreads / 32) {
        if (lane != 0) continue;
        const int w = W.w[li], h = w / 2;
        const float inv = inv_w[li];
        // kept crossings within h samples behind the current one: (position, list index, value)
        int kp[80], ki[80];
        float kv[80];
        int head = 0, tail = 0;  // ring [head, tail) over 80 entries (h + 1 <= 76 live)
        int idx = 0;
        for (int wd = 0; wd < nwords; ++wd) {
            unsigned m = bits[li * nwords + wd];
            while (m) {
                const int b = __ffs(m) - 1;
                m &= m - 1;
                const int p = wd * 32 + b;
                const float v = sp_value(xs, p, hmax, w, mu_f, inv);
                bool pruned = false;
                if (li > 0) {
                    while (head != tail && kp[head % 80] < p - h) ++head;
                    for (int e = head; e != tail && !pruned; ++e) {
                        const int q = e % 80;
                        if (!((ki[q] & 255) == 0 && v >= kv[q])) pruned = true;
                    }
                    if (!pruned) {
                        kp[tail % 80] = p;
                        ki[tail % 80] = idx;
                        kv[tail % 80] = v;
                        ++tail;
                    }
                }
                ++idx;
                if (pruned || v == 0.0f) continue;
                const unsigned long long at = atomicAdd(count, 1ull);
                if ((long long)at < cap) cands[at] = DevCand{d, (int32_t)(c0 + p), w, v};
            }
        }
    }
}

template <typename T>
cudaError_t launch_sp(const T *y, int ndms, long long n, int chunk_len, const SpWidths &W,
                      double threshold, const double2 *musig, DevCand *cands,
                      unsigned long long *count, long long cap, cudaStream_t st)
{
    const int wmax = W.w[W.nw - 1];
    const int nx = chunk_len + wmax / 2 + wmax + kSpR;
    const size_t smem = (size_t)((nx + 3) & ~3) * 4 + (size_t)W.nw * ((chunk_len + 31) / 32) * 4;
    cudaError_t e = cudaFuncSetAttribute(k_singlepulse<T>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const long long nchunks = (n + chunk_len - 1) / chunk_len;
    dim3 grid((unsigned)nchunks, (unsigned)ndms);
    k_singlepulse<T><<<grid, kSpThreads, smem, st>>>(y, n, chunk_len, W, threshold, musig, cands,
                                                     count, cap);
    return cudaGetLastError();
}

}  // namespace

// pruneRelatedDownfactors (singlepulse.cpp:122-146) as written, over one DM's list, mask
// starting at zero; mask[i] != 0 marks a pruned candidate.
static void prune_downfactors(const std::vector<DevCand> &c, size_t a, size_t b, int maxdf,
                              std::vector<unsigned char> &mask)
{
    for (size_t i = a; i < b; ++i) {
        if (mask[i]) continue;
        for (size_t j = i + 1; j < b; ++j) {
            const long long dist = std::llabs((long long)c[j].sample - (long long)c[i].sample);
            if (dist > (long long)((unsigned)maxdf / 2u)) break;
            if (mask[j]) continue;
            unsigned prox = std::max((unsigned)c[i].width / 2u, (unsigned)c[j].width / 2u);
            prox = prox > 1u ? prox : 1u;
            if (dist <= (long long)prox) {
                if (c[i].snr > c[j].snr) mask[j] = 1;
                else mask[i] = 1;
            }
        }
    }
}

mdsm_status singlepulse_detect(const void *d_series, int dtype, int ndms, int nsamp,
                               int max_downfact, int chunk_len, int normalise, double threshold,
                               mdsm_candidate *h_cands, long long cap, long long *ncand,
                               cudaStream_t st)
{
    if (dtype != MDSM_OUT_F32 && dtype != MDSM_OUT_I32)
        return fail(MDSM_EINVAL, "single-pulse search: series must be float32 or int32");
    if (!d_series || ndms <= 0 || nsamp <= 0 || !ncand)
        return fail(MDSM_EINVAL, "single-pulse search: bad arguments");
    if (ndms > 65535) return fail(MDSM_EINVAL, "single-pulse search: at most 65535 DM rows");
    if (max_downfact < 2)
        return fail(MDSM_EINVAL, "single-pulse search: max_downfact must be at least 2");
    if (chunk_len < 32 || chunk_len > kSpMaxChunk)
        return fail(MDSM_EINVAL, "single-pulse search: chunk_len must be 32..32768");
    if (cap < 0) cap = 0;
    SpWidths W{};
    W.nw = 0;
    W.w[W.nw++] = 1;
    for (int i = 0; i < 12 && kSpLadder[i] <= max_downfact; ++i) W.w[W.nw++] = kSpLadder[i];
    const int maxdf = W.w[W.nw - 1];
    if (chunk_len < maxdf) return fail(MDSM_EINVAL, "single-pulse search: chunk_len < widest template");
    // device list of the per-width survivors: room for at least 2^18 of them
    const long long dcap = std::max<long long>(std::max<long long>(4 * cap, 1LL << 18), 1);
    const size_t off_part = 256;
    const size_t part_bytes = normalise ? series_stats_part_bytes(ndms, nsamp) : 0;
    const size_t off_ms = off_part + (part_bytes + 255) / 256 * 256;
    const size_t off_c = off_ms + ((size_t)ndms * sizeof(double2) + 255) / 256 * 256;
    const size_t bytes = off_c + (size_t)dcap * sizeof(DevCand);
    void *sc = nullptr;
    std::unique_lock<std::mutex> lease;
    MDSM_TRY(scratch_get(bytes, &sc, &lease));
    char *base = static_cast<char *>(sc);
    auto *d_count = reinterpret_cast<unsigned long long *>(base);
    auto *d_part = reinterpret_cast<double2 *>(base + off_part);
    auto *d_ms = reinterpret_cast<double2 *>(base + off_ms);
    auto *d_c = reinterpret_cast<DevCand *>(base + off_c);
    MDSM_CUDA_TRY(cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), st));
    if (normalise) MDSM_TRY(series_stats_launch(d_series, dtype, ndms, nsamp, d_part, d_ms, st));
    const double2 *ms = normalise ? d_ms : nullptr;
    if (dtype == MDSM_OUT_F32)
        MDSM_CUDA_TRY(launch_sp(static_cast<const float *>(d_series), ndms, nsamp, chunk_len, W,
                                threshold, ms, d_c, d_count, dcap, st));
    else
        MDSM_CUDA_TRY(launch_sp(static_cast<const int32_t *>(d_series), ndms, nsamp, chunk_len,
                                W, threshold, ms, d_c, d_count, dcap, st));
    unsigned long long n = 0;
    MDSM_CUDA_TRY(cudaMemcpyAsync(&n, d_count, sizeof(n), cudaMemcpyDeviceToHost, st));
    MDSM_CUDA_TRY(cudaStreamSynchronize(st));
    if ((long long)n > dcap) {
        *ncand = (long long)n;
        return fail(MDSM_ERANGE, "single-pulse search: " + std::to_string(n) +
                                     " crossings survive the per-width pruning (room for " +
                                     std::to_string(dcap) + "); raise the threshold or cap");
    }
    std::vector<DevCand> c((size_t)n);
    if (n) MDSM_CUDA_TRY(cudaMemcpy(c.data(), d_c, (size_t)n * sizeof(DevCand),
                                    cudaMemcpyDeviceToHost));
    lease.unlock();
    // the prototype's list order: DM, chunk, width (ladder order), sample
    auto wi = [&](int w) {
        for (int i = 0; i < W.nw; ++i)
            if (W.w[i] == w) return i;
        return W.nw;
    };
    std::sort(c.begin(), c.end(), [&](const DevCand &a, const DevCand &b) {
        if (a.dm_idx != b.dm_idx) return a.dm_idx < b.dm_idx;
        const int ca = a.sample / chunk_len, cb = b.sample / chunk_len;
        if (ca != cb) return ca < cb;
        if (a.width != b.width) return wi(a.width) < wi(b.width);
        return a.sample < b.sample;
    });
    std::vector<unsigned char> mask(c.size(), 0);
    for (size_t a = 0; a < c.size();) {
        size_t b = a;
        while (b < c.size() && c[b].dm_idx == c[a].dm_idx) ++b;
        prune_downfactors(c, a, b, maxdf, mask);
        a = b;
    }
    long long k = 0;
    for (size_t i = 0; i < c.size(); ++i) {
        if (mask[i]) continue;
        if (k < cap && h_cands) {
            h_cands[k].dm_idx = c[i].dm_idx;
            h_cands[k].sample = c[i].sample;
            h_cands[k].width = c[i].width;
            h_cands[k].snr = c[i].snr;
        }
        ++k;
    }
    *ncand = k;
    return MDSM_OK;
}

}  // namespace mdsm

extern "C" mdsm_status mdsm_singlepulse_detect_device(const void *d_series, int series_dtype,
                                                      int ndms, int nsamp, int max_downfact,
                                                      int chunk_len, int normalise,
                                                      double threshold, mdsm_candidate *h_cands,
                                                      long long cap, long long *ncand,
                                                      void *stream)
{
    return mdsm::singlepulse_detect(d_series, series_dtype, ndms, nsamp, max_downfact, chunk_len,
                                    normalise, threshold, h_cands, cap, ncand,
                                    static_cast<cudaStream_t>(stream));
}
