// dedisp.cu -- the shift-and-sum kernel shared by brute-force dedispersion and both subband
// stages, and the host code that tiles a shift table for it.
//
// What it computes (src/mdsm/dedispersion_kernel.cu:11-48 and :51-77, :144-175):
//     out[g][d][t] = sum_{c < nchans} in[g][c][t + S[g][d][c]],   t < nsamp
// with the channels summed in increasing c from zero, so float results are bit-identical to
// the reference kernels' sequential per-thread sums.
//
// How (GB300): one CTA owns a block of Db DM trials x a tile of T samples.  For every channel
// the CTA needs one contiguous segment of the input row, [t0 + smin, t0 + T + smax), where
// smin/smax are the smallest/largest shift of its DMs in that channel.  Warp 0 stages CC such
// segments at a time into shared memory with 1-D bulk copies (the TMA engine) completing on an
// mbarrier, NST stages deep, while all warps accumulate from the previous stage: each lane
// holds DPW DMs x R samples (strided by 32) in registers, so every staged sample is reused
// by up to Db DM trials and all shared-memory reads are bank-conflict free.
//
// Integer samples with FP32 accumulation (the precision form's path for sums that may not fit
// INT32): each staged chunk of CC channels is summed exactly in INT32 and the chunk sums are
// added into the FP32 result with Kahan compensation, so the error stays within about
// 2 * 2^-24 * sum_c |x| however many channels are summed.  Float samples keep the plain
// sequential FP32 sum of the reference kernels.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstring>
#include <type_traits>

#include "internal.h"
#include "box.cuh"
#include "ptx.cuh"

namespace mdsm {


__device__ __forceinline__ unsigned warp_sum_u32(unsigned v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <typename TAcc>
__device__ __forceinline__ void store_out(unsigned char *orow, int t, TAcc v, int out_i32)
{
    if (out_i32)
        reinterpret_cast<int32_t *>(orow)[t] = static_cast<int32_t>(v);
    else
        reinterpret_cast<float *>(orow)[t] = static_cast<float>(v);
}

template <typename TIn, typename TAcc, int R, int DPW, int NW, int CC>
__global__ void __launch_bounds__(NW * 32) k_shift_sum(KArgs a)
{
    constexpr int T = 32 * R;
    constexpr int DB = NW * DPW;
    constexpr int SZ = (int)sizeof(TIn);
    extern __shared__ __align__(128) unsigned char smem[];

    const int nst = a.nst;
    const int rowbytes = a.rowcap * SZ;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem);                     // nst x 8 B
    unsigned char *rows = smem + 128;                                         // nst*CC rows
    int32_t *relsm = reinterpret_cast<int32_t *>(rows + (size_t)nst * CC * rowbytes);
    int32_t *basesm = relsm + nst * CC * DB;

    const int blk = blockIdx.x, g = blockIdx.z;
    const long long t0 = (long long)blockIdx.y * T;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned char *in_g = a.in + (size_t)(g * a.in_group_stride) * SZ;
    const size_t bofs = (size_t)(g * a.nblk + blk) * a.nchans;
    const int32_t *rel_b = a.rel + bofs * DB;
    const int32_t *ss_b = a.sminspan + bofs * 2;
    const int nchunks = (a.nchans + CC - 1) / CC;

    if (threadIdx.x == 0) {
        for (int s = 0; s < nst; ++s) mbar_init(&bars[s], 1);
        fence_mbar_init();
    }
    __syncthreads();

    // Warp 0 stages chunk k (channels k*CC ..) into stage s.
    auto fill = [&](int s, int k) {
        const int c0 = k * CC;
        const int nc = min(CC, a.nchans - c0);
        unsigned bytes = 0;
        const unsigned char *src = nullptr;
        if (lane < nc) {
            const int c = c0 + lane;
            const long long start = t0 + ss_b[2 * c];
            const long long end = start + T + ss_b[2 * c + 1];
            const long long sb = (start * SZ) & ~15LL;
            const long long eb = (end * SZ + 15) & ~15LL;
            bytes = (unsigned)(eb - sb);
            basesm[s * CC + lane] = (int)(start - sb / SZ);
            src = in_g + (size_t)c * (size_t)a.in_stride * SZ + sb;
        }
        const unsigned relbytes = (unsigned)(nc * DB * 4);
        const unsigned total = warp_sum_u32(bytes) + relbytes;
        __syncwarp();
        if (lane == 0) mbar_arrive_expect_tx(&bars[s], total);
        __syncwarp();
        if (lane < nc) bulk_g2s(rows + (size_t)(s * CC + lane) * rowbytes, src, bytes, &bars[s]);
        if (lane == 0) bulk_g2s(relsm + s * CC * DB, rel_b + (size_t)c0 * DB, relbytes, &bars[s]);
    };

    if (warp == 0)
        for (int s = 0; s < nst && s < nchunks; ++s) fill(s, s);

    // Integer samples summed in FP32: exact INT32 chunk sums, Kahan-compensated across chunks.
    constexpr bool kSplit = std::is_same<TAcc, float>::value && !std::is_same<TIn, float>::value;
    using TPart = typename std::conditional<kSplit, int, TAcc>::type;
    TPart acc[DPW][R];
    float ksum[kSplit ? DPW : 1][R], kcomp[kSplit ? DPW : 1][R];
#pragma unroll
    for (int j = 0; j < DPW; ++j)
#pragma unroll
        for (int r = 0; r < R; ++r) acc[j][r] = TPart(0);
    if constexpr (kSplit) {
#pragma unroll
        for (int j = 0; j < DPW; ++j)
#pragma unroll
            for (int r = 0; r < R; ++r) ksum[j][r] = kcomp[j][r] = 0.0f;
    }

    int k = 0;
    bool aborted = false;
    for (; k < nchunks; ++k) {
        const int s = k % nst;
        const unsigned par = (unsigned)(k / nst) & 1u;
        const bool ok = mbar_wait_bounded(&bars[s], par, a.err, ERR_WAIT_TIMEOUT);
        if (ok) {
            const int nc = min(CC, a.nchans - k * CC);
            const unsigned char *rb = rows + (size_t)s * CC * rowbytes;
            const int32_t *rs = relsm + s * CC * DB + warp * DPW;
            const int32_t *bs = basesm + s * CC;
#pragma unroll 2
            for (int ci = 0; ci < nc; ++ci) {
                const TIn *row = reinterpret_cast<const TIn *>(rb + (size_t)ci * rowbytes) +
                                 bs[ci] + lane;
#pragma unroll
                for (int j = 0; j < DPW; ++j) {
                    const TIn *p = row + rs[ci * DB + j];
#pragma unroll
                    for (int r = 0; r < R; ++r) acc[j][r] += static_cast<TPart>(p[32 * r]);
                }
            }
            if constexpr (kSplit) {
#pragma unroll
                for (int j = 0; j < DPW; ++j)
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        const float y = __fsub_rn((float)acc[j][r], kcomp[j][r]);
                        const float t = __fadd_rn(ksum[j][r], y);
                        kcomp[j][r] = __fsub_rn(__fsub_rn(t, ksum[j][r]), y);
                        ksum[j][r] = t;
                        acc[j][r] = 0;
                    }
            }
        }
        if (__syncthreads_or(!ok)) {
            aborted = true;
            break;
        }
        if (warp == 0 && k + nst < nchunks) {
            fence_proxy_async_smem();
            fill(s, k + nst);
        }
    }

    if (aborted) {
        // Let this CTA's copies still in flight land before it exits (bounded as well).
        for (int kk = k; kk < nchunks && kk < k + nst; ++kk)
            mbar_wait_bounded(&bars[kk % nst], (unsigned)(kk / nst) & 1u, nullptr, 0);
        return;
    }

    const int osz = 4;  // int32 and float32 outputs alike
#pragma unroll
    for (int j = 0; j < DPW; ++j) {
        const int d = blk * DB + warp * DPW + j;
        if (d >= a.ndms) continue;
        unsigned char *orow =
            a.out + (size_t)(g * a.out_group_stride + (long long)d * a.out_stride) * osz;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const long long t = t0 + lane + 32 * r;
            if (t >= a.nsamp) continue;
            if constexpr (kSplit)
                store_out<float>(orow, (int)t, __fsub_rn(ksum[j][r], kcomp[j][r]), a.out_i32);
            else
                store_out<TAcc>(orow, (int)t, acc[j][r], a.out_i32);
        }
    }
}

// ------------------------------------------------------------------------------------------
// Packed kernels (uint8 and uint16 samples, exact integer sums).
//
// The generic kernel spends one shared-memory load per add, which caps it at 32 adds per
// clock per SM (the 128 B/clk shared-memory port).  Here one 32-bit load brings several
// consecutive samples (4 uint8 or 2 uint16):
//  * each staged row is expanded once into phase copies, P_a[j] = the word starting at sample
//    (words per sample) * j + a, so any run of samples starting at any offset is one aligned
//    word, and a warp's 32 lanes read 32 consecutive words (no bank conflicts);
//  * the raw words are summed as 32-bit integers, A = sum w (mod 2^32), and one extraction per
//    word sums the odd samples separately: uint8, O = sum (s1 | s3 << 16) by one PRMT; uint16,
//    O = sum s1 by one shift;
//  * w = (even lanes) + 2^(8*bytes) O, so E = A - 2^(8*bytes) O (mod 2^32) are the even lanes'
//    sums; over at most 256 channels every uint8 lane sum is <= 256 * 255 < 2^16 and every
//    uint16 one < 2^32, so E and O hold the sums exactly; they are added into int32 every
//    256 channels;
//  * two channels share each 3-input integer add (A += wa + wz, O += odd(wa) + odd(wz)).
// Per word (4 or 2 sample-adds) and channel: 1 LDS, 1 PRMT or shift, one 3-input add.
// A CTA is NW compute warps of DPW DM trials each and one producer warp that only issues the
// copies, so no compute warp carries the copy latency into the per-chunk barrier; uint8 uses
// 19 x 2 (38 trials a tile; 20 warps keep 96 registers a thread), uint16 (the second subband
// stage, 16 trials per call) 16 x 1.  One CTA per SM (the staging takes ~200 KB).
// ------------------------------------------------------------------------------------------
constexpr int kPCC = 16;         // channels per stage
constexpr int kPNR = 3;          // raw stages in flight
constexpr int kPT = 512;         // samples per tile (wider where no flush registers are kept)

template <int SW_, int NW_, int DPW_, bool U16OUT_ = false, int PT_ = kPT, bool SIGNED_ = false>
struct PackedCfg {
    static constexpr bool U16OUT = U16OUT_;       // store the sums as uint16
    // int16 samples: the expansion flips each sample's sign bit (x + 32768, offset binary), the
    // store takes 32768 per channel off again
    static constexpr bool SIGNED = SIGNED_;
    static constexpr int SW = SW_;                // bytes per sample
    static constexpr int SPW = 4 / SW;            // samples per word = phase copies
    static constexpr int NW = NW_;                // compute warps (the producer is warp NW)
    static constexpr int DPW = DPW_;              // DM trials per compute warp
    static constexpr int PT = PT_;                // samples per tile
    static constexpr int PRW = PT / (32 * SPW);   // words per lane per DM trial
    static constexpr int DB = NW * DPW;           // DM trials per tile
    static constexpr int DBS = (DB + 3) / 4 * 4;  // offsets per channel as stored (16-byte rows)
    static constexpr int THREADS = (NW + 1) * 32;
    static_assert(NW * 32 >= kPCC * DB, "the compute threads copy a chunk's offsets");
    static_assert(DPW == 1 || DPW == 2, "one or two DM trials per warp");
    static_assert(!U16OUT || SW == 1, "uint16 output from uint8 samples");
    static_assert(PT % (32 * SPW) == 0, "whole words per lane");
    static_assert(!SIGNED || (SW == 2 && !U16OUT), "signed samples are int16");
};
using CfgU8 = PackedCfg<1, 19, 2>;
using CfgU8w16 = PackedCfg<1, 16, 2>;         // 32-trial blocks, for trial counts of 32 k
// The first subband stage (uint16 subband series): without the int32 flush registers there
// is room for 1024-sample tiles, which halve the per-chunk costs per add; 768- or 512-sample
// tiles where the wider staging does not fit in shared memory.
template <int NW, int PT>
using CfgU8to16T = PackedCfg<1, NW, 2, true, PT>;
// uint16 samples (no flush registers either): 768- or 512-sample tiles as the staging fits
// shared memory (1024-sample rows of uint16 never fit with their two phase copies).
template <int PT>
using CfgU16T = PackedCfg<2, 16, 1, false, PT>;
template <int PT>
using CfgI16T = PackedCfg<2, 16, 1, false, PT, true>;

// Work items of the packed kernels are (beam, DM block, time tile, group) tiles; a CTA runs a
// stream of them.  The producer warp stages the stream's chunks (16 channels of one item) into
// a ring of kPNR stages, running ahead across item boundaries, and writes each chunk's
// (item, chunk index, channels, flags) beside it; the compute warps take the chunks in order,
// start an item's sums on its first chunk and store them after its last.  So short items
// (few channels, as in the subband stages) keep the copies in flight between items.
constexpr int kChunkFirst = 1, kChunkLast = 2, kChunkStop = 4;  // chunk flags (bits 0-2)

// CTA barrier 0 returning whether any thread passed true.  The producer and the compute warps
// reach it from their own loops, once per chunk each (a barrier counts warps, so the program
// locations may differ between warps).
__device__ __forceinline__ bool cta_any(bool pred)
{
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.or.pred q, 0, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)pred)
        : "memory");
    return r != 0;
}

// Items of one plan, (DM block fastest, time tile, group); CTA b takes b, b + G, b + 2G, ...
struct OnePlanItems {
    const KArgs *a;
    int ntiles, nitems;
    int next_it;
    __device__ int grab()
    {
        const int it = next_it;
        next_it += gridDim.x;
        return it < nitems ? it : -1;
    }
    __device__ int4 item(int it) const
    {
        const int blk = it % a->nblk, rest = it / a->nblk;
        return make_int4(0, blk, rest % ntiles, rest / ntiles);
    }
    __device__ const KArgs &args(int) const { return *a; }
    __device__ void item_done(int) const {}
    static constexpr bool kBeamStride = false;  // every chunk has the kernel's phase stride
};

// Items of several plans from a list, taken from a global counter.
struct ListItems {
    const KArgs *beams;
    const int4 *items;
    int nitems;
    unsigned *counter;
    __device__ int grab()
    {
        const int it = (int)atomicAdd(counter, 1u);
        return it < nitems ? it : -1;
    }
    __device__ int4 item(int it) const { return items[it]; }
    __device__ const KArgs &args(int beam) const { return beams[beam]; }
    __device__ void item_done(int) const {}
    static constexpr bool kBeamStride = true;  // each beam's chunks with its own phase stride
};

// The odd samples of a word as 32-bit lanes: uint8, (s1, s3) as uint16 lanes; uint16, s1.
template <int SW>
__device__ __forceinline__ uint32_t odd_lanes(uint32_t w)
{
    if constexpr (SW == 1)
        return __byte_perm(w, 0u, 0x4341);
    else
        return w >> 16;
}

// o + (w >> 16) as (w * 2^16) >> 32 + o: one integer multiply-add, issued on the FMA pipe, so
// that the uint16 kernel's odd-lane sums leave the ALU pipe to the raw-word sums.
__device__ __forceinline__ uint32_t add_hi16(uint32_t w, uint32_t o)
{
    uint32_t d;
    asm("mad.hi.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(w), "r"(0x10000u), "r"(o));
    return d;
}

template <class Cfg, class Src>
__device__ __forceinline__ void packed_stream(Src &src, unsigned char *smem, int rawcap, int ps,
                                              unsigned *err)
{
    constexpr int SW = Cfg::SW, SPW = Cfg::SPW, NW = Cfg::NW, DPW = Cfg::DPW, PRW = Cfg::PRW;
    constexpr int DB = Cfg::DB, DBS = Cfg::DBS;
    const int nwp = ps >> 2;  // words per phase copy
    const int nq = nwp >> 2;  // 16-byte quads per phase copy
    // ceil(2^20 / nq): (q * nq_inv) >> 20 == q / nq for q < 16 nq, nq < 256 (the host keeps
    // rows below 4096 bytes)
    const unsigned nq_inv = ((1u << 20) + (unsigned)nq - 1) / (unsigned)nq;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem);
    int4 *meta = reinterpret_cast<int4 *>(smem + 64);  // kPNR entries
    unsigned char *raw = smem + 128;
    int32_t *offsm = reinterpret_cast<int32_t *>(raw + (size_t)kPNR * kPCC * rawcap);
    int32_t *offcur = offsm + kPNR * kPCC * DBS;                 // 2 x kPCC x DBS
    uint32_t *P = reinterpret_cast<uint32_t *>(offcur + 2 * kPCC * DBS);  // 2 x kPCC x SPW x nwp
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (warp == NW) {
        // ---- producer: the item being staged, its next chunk, and the lane's (smin, span)
        // for that chunk, loaded one fill ahead so that no fill waits on a global load
        int p_it = -1, p_k = 0, p_nchunks = 0;
        int4 p_w = make_int4(0, 0, 0, 0);
        int2 p_ss = make_int2(0, 0);
        // the item's beam fields the fills use, in registers (the barrier and copy asm clobber
        // memory, which would otherwise reload them from the argument list at every fill)
        struct {
            const unsigned char *in;
            long long in_stride, in_group_stride;
            const int32_t *rel, *sminspan;
            int nchans, nblk;
        } a{};
        auto p_next_item = [&]() {
            int it = 0;
            if (lane == 0) it = src.grab();
            p_it = __shfl_sync(0xffffffffu, it, 0);
            p_k = 0;
            if (p_it >= 0) {
                p_w = src.item(p_it);
                const KArgs &b = src.args(p_w.x);
                a.in = b.in;
                a.in_stride = b.in_stride;
                a.in_group_stride = b.in_group_stride;
                a.rel = b.rel;
                a.sminspan = b.sminspan;
                a.nchans = b.nchans;
                a.nblk = b.nblk;
                p_nchunks = (a.nchans + kPCC - 1) / kPCC;
            }
        };
        auto p_load_ss = [&]() {
            if (p_it < 0) return;
            const int c = p_k * kPCC + lane;
            if (c < a.nchans) {
                const size_t bofs = (size_t)(p_w.w * a.nblk + p_w.y) * a.nchans;
                p_ss = __ldg(reinterpret_cast<const int2 *>(a.sminspan + bofs * 2) + c);
            }
        };
        // Stage the next chunk of the stream into stage s (or mark the end of the stream).
        auto fill_next = [&](int s) {
            if (p_it < 0) {
                if (lane == 0) {
                    meta[s] = make_int4(-1, 0, 0, kChunkStop);
                    mbar_arrive(&bars[s]);
                }
                __syncwarp();
                return;
            }
            const long long t0 = (long long)p_w.z * Cfg::PT;
            const size_t bofs = (size_t)(p_w.w * a.nblk + p_w.y) * a.nchans;
            const int c0 = p_k * kPCC;
            const int nc = min(kPCC, a.nchans - c0);
            unsigned bytes = 0;
            const unsigned char *src_row = nullptr;
            if (lane < nc) {
                const int c = c0 + lane;
                const long long start = t0 + p_ss.x;
                const long long end = start + Cfg::PT + p_ss.y;
                const long long sb = (start * SW) & ~15LL;  // bytes
                const long long eb = (end * SW + 15) & ~15LL;
                bytes = (unsigned)(eb - sb);
                src_row = a.in + (size_t)(p_w.w * a.in_group_stride) * SW +
                          (size_t)c * (size_t)a.in_stride * SW + sb;
            }
            const unsigned offbytes = (unsigned)(nc * DBS * 4);
            const unsigned total = warp_sum_u32(bytes) + offbytes;
            __syncwarp();
            if (lane == 0) {
                meta[s] = make_int4(p_it, p_k, nc,
                                    (p_k == 0 ? kChunkFirst : 0) |
                                        (p_k == p_nchunks - 1 ? kChunkLast : 0) |
                                        (p_w.x << 8));  // the item's beam above the flags
                mbar_arrive_expect_tx(&bars[s], total);  // releases the meta entry with the phase
            }
            __syncwarp();
            if (lane < nc)
                bulk_g2s(raw + (size_t)(s * kPCC + lane) * rawcap, src_row, bytes, &bars[s]);
            if (lane == 0)
                bulk_g2s(offsm + s * kPCC * DBS, a.rel + (bofs + (size_t)c0) * DBS, offbytes,
                         &bars[s]);
            if (++p_k == p_nchunks) p_next_item();
            p_load_ss();
        };
        // One CTA barrier per chunk, as the compute warps', then the refill of the stage every
        // warp has just finished expanding.
        p_next_item();
        p_load_ss();
        for (int i = 0; i < kPNR; ++i) fill_next(i);
        for (unsigned gk = 0;; ++gk) {
            const int s = (int)(gk % kPNR);
            const bool stop = (meta[s].w & kChunkStop) != 0;  // written by this warp
            if (cta_any(false)) {
                for (unsigned q = gk; q < gk + kPNR; ++q)
                    mbar_wait_bounded(&bars[q % kPNR], (q / kPNR) & 1u, nullptr, 0);
                return;
            }
            if (stop) return;
            fence_proxy_async_smem();
            fill_next(s);
        }
    }

    // ---- compute warps ----
    uint32_t A[DPW][PRW];        // raw words summed mod 2^32 (<= 256 channels)
    uint32_t O[DPW][PRW];        // odd lanes summed (<= 256 channels)
    int32_t f[DPW][PRW][SPW];    // int32 sums
    // The lane sums are final (no int32 flush) for uint16 output (an item has at most 257
    // channels, so the 16-bit lanes do not carry) and for uint16 samples (E and O are then
    // 32-bit sums, exact while nchans * 65535 < 2^31, which the host checks).
    constexpr bool kDirect = Cfg::U16OUT || SW == 2;

    unsigned gk = 0;  // chunk sequence number
    bool aborted = false;
    // the chunk's phase stride (words), quads per row and their reciprocal: the kernel's, or,
    // for sources whose beams keep their own strides, those of the last chunk's beam
    int nwc = nwp, nqc = nq, sb_beam = -1;
    unsigned nqc_inv = nq_inv;
    int done_beam = -1;  // beam of an item whose stores are not yet published
    for (;; ++gk) {
        const int s = (int)(gk % kPNR);
        const int pb = (int)(gk & 1u);  // phase buffer of this chunk
        const unsigned par = (gk / kPNR) & 1u;
        const bool ok = mbar_wait_bounded(&bars[s], par, err, ERR_WAIT_TIMEOUT);
        const int4 m = ok ? meta[s] : make_int4(-1, 0, 0, 0);
        if (ok) {
            // Expand the staged rows into their phase copies (16-byte loads and stores), the
            // 16 rows' quads spread over all compute threads.  P[pb] was last read for chunk
            // gk-2, before the barrier of chunk gk-1.  All 16 rows are expanded whatever the
            // chunk holds (rows past its channels, or the whole stage at the end of the
            // stream, hold earlier data nobody reads), so the expansion does not wait for the
            // chunk's entry.
            if constexpr (Src::kBeamStride) {
                const int beam = m.w >> 8;
                if (m.x >= 0 && beam != sb_beam) {  // (consecutive chunks mostly share a beam)
                    sb_beam = beam;
                    nwc = src.args(beam).ps >> 2;
                    nqc = nwc >> 2;
                    nqc_inv = ((1u << 20) + (unsigned)nqc - 1) / (unsigned)nqc;
                }
            }
            for (int q = tid; q < kPCC * nqc; q += NW * 32) {
                const int row = (int)(((unsigned)q * nqc_inv) >> 20);  // q / nqc
                const int i = q - row * nqc;
                const uint32_t *W =
                    reinterpret_cast<const uint32_t *>(raw + (size_t)(s * kPCC + row) * rawcap);
                // phase-major: copy a of row r at (a * 16 + r) * nwc from the phase buffer's
                // start (buffers kPCC * SPW * nwp words apart), so a warp whose quads cross from
                // one row into the next stores to consecutive addresses
                uint32_t *Pr = P + (size_t)pb * SPW * kPCC * nwp + (size_t)row * nwc;
                {
                    uint4 w = reinterpret_cast<const uint4 *>(W)[i];
                    uint32_t w4 = W[4 * i + 4];
                    if constexpr (Cfg::SIGNED) {
                        w.x ^= 0x80008000u;
                        w.y ^= 0x80008000u;
                        w.z ^= 0x80008000u;
                        w.w ^= 0x80008000u;
                        w4 ^= 0x80008000u;
                    }
                    reinterpret_cast<uint4 *>(Pr)[i] = w;
#pragma unroll
                    for (int a = 1; a < SPW; ++a)
                        reinterpret_cast<uint4 *>(Pr + a * kPCC * nwc)[i] =
                            make_uint4(__funnelshift_r(w.x, w.y, 8 * SW * a),
                                       __funnelshift_r(w.y, w.z, 8 * SW * a),
                                       __funnelshift_r(w.z, w.w, 8 * SW * a),
                                       __funnelshift_r(w.w, w4, 8 * SW * a));
                }
            }
            if (tid < kPCC * DB) {  // one real entry per thread (the row padding is not read)
                const int i = tid / DB * DBS + tid % DB;
                offcur[pb * kPCC * DBS + i] = offsm[s * kPCC * DBS + i];
            }
        }
        // Every thread that waited saw the same entry, so the stop flag agrees across the CTA
        // when no wait ran out.
        if (cta_any(!ok)) {
            aborted = true;
            break;
        }
        // The previous item's rows were all stored before this barrier: one thread publishes
        // that (its fence is cumulative over the CTA's writes ordered by the barrier).
        if (done_beam >= 0) {
            if (tid == 0) src.item_done(done_beam);
            done_beam = -1;
        }
        if (m.w & kChunkStop) break;
        const int nc = m.z;
        if (m.w & kChunkFirst) {
#pragma unroll
            for (int j = 0; j < DPW; ++j)
#pragma unroll
                for (int r = 0; r < PRW; ++r) {
                    A[j][r] = O[j][r] = 0u;
                    if constexpr (!kDirect)
#pragma unroll
                        for (int e = 0; e < SPW; ++e) f[j][r][e] = 0;
                }
        }
        const unsigned char *pbase =
            reinterpret_cast<const unsigned char *>(P + (size_t)pb * kPCC * SPW * nwp) + lane * 4;
        const int32_t *oc = offcur + pb * kPCC * DBS + warp * DPW;
        // this warp's DM trials' word offsets (bytes) in channel c's phase-expanded row
        auto offs = [&](int c, int (&o)[DPW]) {
            if constexpr (DPW == 2) {
                const int2 v = *reinterpret_cast<const int2 *>(oc + c * DBS);
                o[0] = v.x;
                o[1] = v.y;
            } else {
                o[0] = oc[c * DBS];
            }
        };
        // Two channels per step: A += wa + wz and O += odd(wa) + odd(wz) are one 3-input
        // integer add each.
        auto pair = [&](int c) {
            const unsigned char *pa = pbase, *pz = pbase;  // the offsets select the rows
            int oa[DPW], oz[DPW];
            offs(c, oa);
            offs(c + 1, oz);
#pragma unroll
            for (int r = 0; r < PRW; ++r) {
                uint32_t wa[DPW], wz[DPW];
#pragma unroll
                for (int j = 0; j < DPW; ++j) {
                    wa[j] = reinterpret_cast<const uint32_t *>(pa + oa[j])[32 * r];
                    wz[j] = reinterpret_cast<const uint32_t *>(pz + oz[j])[32 * r];
                }
#pragma unroll
                for (int j = 0; j < DPW; ++j) {
                    A[j][r] = A[j][r] + wa[j] + wz[j];
                    if constexpr (SW == 2)
                        O[j][r] = add_hi16(wz[j], add_hi16(wa[j], O[j][r]));
                    else
                        O[j][r] += odd_lanes<SW>(wa[j]) + odd_lanes<SW>(wz[j]);
                }
            }
        };
        int ci = 0;
        if (nc == kPCC) {
#pragma unroll
            for (int c = 0; c < kPCC; c += 2) pair(c);
            ci = kPCC;
        } else {
#pragma unroll 1
            for (; ci + 1 < nc; ci += 2) pair(ci);
        }
        if (ci < nc) {  // odd channel count: the last channel alone
            const unsigned char *pa = pbase;
            int oa[DPW];
            offs(ci, oa);
#pragma unroll
            for (int r = 0; r < PRW; ++r)
#pragma unroll
                for (int j = 0; j < DPW; ++j) {
                    const uint32_t wa = reinterpret_cast<const uint32_t *>(pa + oa[j])[32 * r];
                    A[j][r] += wa;
                    if constexpr (SW == 2)
                        O[j][r] = add_hi16(wa, O[j][r]);
                    else
                        O[j][r] += odd_lanes<SW>(wa);
                }
        }
        const bool last = (m.w & kChunkLast) != 0;
        if (!kDirect && (((m.y + 1) & 15) == 0 || last)) {
            // A = E + 2^(8 SW) O (mod 2^32): E and O hold the lane sums exactly
#pragma unroll
            for (int j = 0; j < DPW; ++j)
#pragma unroll
                for (int r = 0; r < PRW; ++r) {
                    const uint32_t E = A[j][r] - (O[j][r] << (8 * SW));
                    if constexpr (SW == 1) {
                        f[j][r][0] += (int32_t)(E & 0xFFFFu);
                        f[j][r][2] += (int32_t)(E >> 16);
                        f[j][r][1] += (int32_t)(O[j][r] & 0xFFFFu);
                        f[j][r][3] += (int32_t)(O[j][r] >> 16);
                    }
                    A[j][r] = O[j][r] = 0u;
                }
        }
        if (!last) continue;
        // the item's sums are complete: store them (int32, float32 or, for the uint16 subband
        // series of the first stage, uint16)
        const int4 w = src.item(m.x);
        const KArgs &a = src.args(w.x);
        const long long t0 = (long long)w.z * Cfg::PT;
        constexpr bool U16OUT = Cfg::U16OUT;
        constexpr int osz = U16OUT ? 2 : 4;
#pragma unroll
        for (int j = 0; j < DPW; ++j) {
            const int d = w.y * DB + warp * DPW + j;
            if (d >= a.ndms) continue;
            unsigned char *orow =
                a.out + (size_t)(w.w * a.out_group_stride + (long long)d * a.out_stride) * osz;
            long long m1 = 0;                    // this lane's share of the row's moments
            unsigned long long m2lo = 0, m2hi = 0;
#pragma unroll
            for (int r = 0; r < PRW; ++r) {
                const long long t = t0 + SPW * (lane + 32 * r);
                const bool whole = t + SPW - 1 < a.nsamp &&
                                   ((((uintptr_t)orow) | (t * osz)) & (SPW * osz - 1)) == 0;
                if constexpr (U16OUT) {
                    // samples 0 and 2 are E's lanes, 1 and 3 O's
                    const uint32_t E = A[j][r] - (O[j][r] << 8);
                    const uint32_t w01 = __byte_perm(E, O[j][r], 0x5410);
                    const uint32_t w23 = __byte_perm(E, O[j][r], 0x7632);
                    if (whole) {
                        *reinterpret_cast<uint2 *>(orow + t * 2) = make_uint2(w01, w23);
                    } else {
                        const uint32_t v[4] = {w01 & 0xFFFFu, w01 >> 16, w23 & 0xFFFFu, w23 >> 16};
#pragma unroll
                        for (int e = 0; e < 4; ++e)
                            if (t + e < a.nsamp) reinterpret_cast<uint16_t *>(orow)[t + e] = (uint16_t)v[e];
                    }
                    continue;
                }
                int32_t v[SPW];
                if constexpr (SW == 2) {
                    // offset-binary sums less 32768 per channel (exact: the host keeps
                    // nchans * 65535 below 2^31)
                    const uint32_t bias = Cfg::SIGNED ? 32768u * (uint32_t)a.nchans : 0u;
                    v[0] = (int32_t)(A[j][r] - (O[j][r] << 16) - bias);
                    v[SPW - 1] = (int32_t)(O[j][r] - bias);
                } else {
#pragma unroll
                    for (int e = 0; e < SPW; ++e) v[e] = f[j][r][e];
                }
                if (a.mom) {
#pragma unroll
                    for (int e = 0; e < SPW; ++e)
                        if (t + e < a.nsamp) {
                            const unsigned long long q =
                                (unsigned long long)((long long)v[e] * (long long)v[e]);
                            m1 += v[e];
                            m2lo += q;
                            m2hi += (m2lo < q);
                        }
                }
                if (whole && a.out_i32) {
                    if constexpr (SPW == 4)
                        *reinterpret_cast<int4 *>(orow + t * 4) = make_int4(v[0], v[1], v[2], v[3]);
                    else
                        *reinterpret_cast<int2 *>(orow + t * 4) = make_int2(v[0], v[SPW - 1]);
                } else if (whole) {
                    if constexpr (SPW == 4)
                        *reinterpret_cast<float4 *>(orow + t * 4) =
                            make_float4((float)v[0], (float)v[1], (float)v[2], (float)v[3]);
                    else
                        *reinterpret_cast<float2 *>(orow + t * 4) =
                            make_float2((float)v[0], (float)v[SPW - 1]);
                } else {
#pragma unroll
                    for (int e = 0; e < SPW; ++e)
                        if (t + e < a.nsamp) store_out<int>(orow, (int)(t + e), v[e], a.out_i32);
                }
            }
            if (!U16OUT && a.mom) {
                // the row's share of this item: warp sum (128-bit with carries), then one
                // atomic per word; integer sums do not depend on their order
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    m1 += __shfl_xor_sync(0xffffffffu, m1, o);
                    const unsigned long long lo = __shfl_xor_sync(0xffffffffu, m2lo, o);
                    const unsigned long long hi = __shfl_xor_sync(0xffffffffu, m2hi, o);
                    const unsigned long long nl = m2lo + lo;
                    m2hi += hi + (nl < m2lo);
                    m2lo = nl;
                }
                if (lane == 0) {
                    unsigned long long *mp = a.mom + 3 * (size_t)(w.w * a.mom_group_rows + d);
                    atomicAdd(mp, (unsigned long long)m1);
                    const unsigned long long old = atomicAdd(mp + 1, m2lo);
                    atomicAdd(mp + 2, m2hi + (old + m2lo < old ? 1ull : 0ull));
                }
            }
        }
        done_beam = w.x;  // published after the next chunk's barrier
    }
    if (aborted) {
        // let the copies already issued land before the CTA exits (bounded as well)
        for (unsigned q = gk; q < gk + kPNR; ++q)
            mbar_wait_bounded(&bars[q % kPNR], (q / kPNR) & 1u, nullptr, 0);
    }
}

__device__ __forceinline__ void packed_init_barriers(unsigned char *smem)
{
    if (threadIdx.x == 0) {
        uint64_t *bars = reinterpret_cast<uint64_t *>(smem);
        for (int s = 0; s < kPNR; ++s) mbar_init(&bars[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
}

// One plan: a persistent grid of at most one CTA per SM over the plan's items.
template <class Cfg>
__global__ void __launch_bounds__(Cfg::THREADS, 1)
    k_shift_sum_packed(const __grid_constant__ KArgs a, int ntiles, int nitems)
{
    extern __shared__ __align__(128) unsigned char smem[];
    packed_init_barriers(smem);
    OnePlanItems src{&a, ntiles, nitems, (int)blockIdx.x};
    packed_stream<Cfg>(src, smem, a.rowcap, a.ps, a.err);
}

// Several uint8 plans (beams that may differ in channels, samples and DM plan) from one work
// list, sharing one staging geometry (rowcap, ps) so the shared-memory layout is the same for
// every item.
__global__ void __launch_bounds__(CfgU8::THREADS, 1)
    k_shift_sum_u8x4_batch(const KArgs *__restrict__ beams, const int4 *__restrict__ items,
                           int nitems, unsigned *__restrict__ counter, int rawcap, int ps,
                           unsigned *err)
{
    extern __shared__ __align__(128) unsigned char smem[];
    packed_init_barriers(smem);
    ListItems src{beams, items, nitems, counter};
    packed_stream<CfgU8>(src, smem, rawcap, ps, err);
}

// ------------------------------------------------------------------------------------------
// fused batched launch: RFI clip, dedispersion and boxcar search of several uint8 beams in one
// persistent launch
// ------------------------------------------------------------------------------------------
// Four phases over four work lists, each item taken from its own global counter: (1) clip one
// channel of one beam; (2) clip one run of columns (spectra) of one beam; (3) dedisperse one
// (beam, DM block, time tile) through the packed stream, storing int32 series and folding
// each row's exact moments when a search follows; (4) boxcar-search one run of tiles of one
// row, in one of several independent thread groups of the CTA.  Each item first waits
// (bounded) for its beam's items of the phase before: a count in `done` that one thread
// raises, after a CTA barrier and a fence, once the item's results are written.  A CTA leaves a
// phase only when that phase's list is exhausted, so every item an item waits for has already
// been taken by a running CTA, which depends only on earlier phases: the waits always end.
constexpr int kFusedSpecCols = kFusedSpecColsHost;  // columns of one phase-2 item (a thread each)
constexpr int kFusedBoxThreads = 128;  // threads of one search group (4 warps)
constexpr int kFusedBoxWidths = 9;     // widths 1..256
constexpr int kFusedBoxK = 19;         // positions per thread
using FusedBoxGeom = BoxGeom<kFusedBoxWidths, kFusedBoxThreads, kFusedBoxK>;
// shared memory of one search group (16-byte multiple)
constexpr size_t kFusedBoxSmem = (FusedBoxGeom::SMEM + 15) / 16 * 16;

// Bounded wait until *ctr >= target (raised by other CTAs after a fence): polling with
// backoff, about 4 s at most; on timeout sets ERR_WAIT_TIMEOUT and returns false.
__device__ __forceinline__ bool wait_count(const unsigned *ctr, unsigned target, unsigned *err)
{
    for (unsigned i = 0; i < (1u << 22); ++i) {
        if (*reinterpret_cast<const volatile unsigned *>(ctr) >= target) {
            __threadfence();
            return true;
        }
        __nanosleep(i < 64 ? 32 : 1000);
    }
    atomicOr(err, ERR_WAIT_TIMEOUT);
    return false;
}

// The whole CTA's next item of a list: thread 0 takes it from the counter.
__device__ __forceinline__ int cta_grab(unsigned *counter, int n, int *slot)
{
    __syncthreads();  // everyone is done with the previous item and with *slot
    if (threadIdx.x == 0) *slot = (int)atomicAdd(counter, 1u);
    __syncthreads();
    const int it = *slot;
    return it < n ? it : -1;
}

// Marks an item of `phase` of beam b done, after this CTA's writes.
__device__ __forceinline__ void cta_done(unsigned *done, int b, int phase)
{
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(&done[3 * b + phase], 1u);
}

// The clip test of the standalone clip (rfi.cu), fabs(v - mean) >= lim in double, is monotone
// in v on each side of the mean (the rounded difference is monotone), so for integer samples
// it holds exactly for v >= hi when v >= ceil(mean) and for v <= lo below: the bounds are found
// from the real-valued estimates and corrected with that same test.
__device__ __forceinline__ void clip_bounds_u8(double mu, double lim, int *cm, int *lo, int *hi)
{
    auto clipped = [&](int v) { return fabs(__dadd_rn((double)v, -mu)) >= lim; };
    const int c = (int)ceil(mu);
    int h = (int)fmin(fmax(ceil(mu + lim), (double)c), 256.0);
    while (h > c && clipped(h - 1)) --h;
    while (h <= 255 && !clipped(h)) ++h;
    int l = (int)fmax(fmin(floor(mu - lim), (double)(c - 1)), -1.0);
    while (l < c - 1 && clipped(l + 1)) ++l;
    while (l >= 0 && !clipped(l)) --l;
    *cm = c;
    *lo = l;
    *hi = h;
}

__device__ __forceinline__ uint8_t clip_rep_u8(double mu)
{
    const int r = __double2int_rn(mu);
    return (uint8_t)min(max(r, 0), 255);
}

__device__ __forceinline__ void mean_sigma_ll(long long s1, long long s2, long long n, double *mu,
                                              double *sig)
{
    const double m = __ddiv_rn((double)s1, (double)n);
    const double var = __dadd_rn(__ddiv_rn((double)s2, (double)n), -__dmul_rn(m, m));
    *mu = m;
    *sig = var > 0.0 ? __dsqrt_rn(var) : 0.0;
}

// Phase 3's item source: the dedispersion list, each item waiting for its beam's clip (when
// there is one), each compute warp counting its stores (when a search follows).
struct FusedItems {
    const KArgs *beams;
    const int4 *items;
    int nitems;
    unsigned *counter;
    const FusedBeam *fb;
    unsigned *done;
    unsigned *err;
    bool count;  // phase 4 waits on the stores
    bool clip;   // the items wait for their beam's spectrum clips
    __device__ int grab()
    {
        const int it = (int)atomicAdd(counter, 1u);
        if (it >= nitems) return -1;
        if (clip) {
            const int b = items[it].x;
            wait_count(&done[3 * b + 1], fb[b].nspec_items, err);  // (a timeout is recorded)
        }
        return it;
    }
    __device__ int4 item(int it) const { return items[it]; }
    __device__ const KArgs &args(int beam) const { return beams[beam]; }
    __device__ void item_done(int beam) const
    {
        if (!count) return;
        __threadfence();
        atomicAdd(&done[3 * beam + 2], 1u);
    }
    // each beam's chunks are expanded with the beam's own phase stride (KArgs::ps, at most
    // the kernel's), so a narrow beam does not expand the widest beam's row length
    static constexpr bool kBeamStride = true;
};

template <class Cfg>
__global__ void __launch_bounds__(Cfg::THREADS, 1)
    k_batch_fused(const FusedArgs f, const KArgs *__restrict__ beams,
                  const int4 *__restrict__ dd_items, int n_dd, int rawcap, int ps)
{
    static_assert(Cfg::THREADS >= kFusedSpecCols && Cfg::THREADS >= kFusedBoxThreads,
                  "CTA too narrow for the clip and search phases");
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ int slot;
    __shared__ long long red[2][Cfg::THREADS / 32];
    __shared__ double s_mu, s_sig;
    __shared__ int s_ok;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int NWARP = Cfg::THREADS / 32;

    // ---- phase 1: clip each channel over its row ----
    if (f.k_chan > 0.0)
        for (int it; (it = cta_grab(&f.counters[0], f.n_cc, &slot)) >= 0;) {
            const int2 w = f.cc_items[it];
            const FusedBeam &B = f.fb[w.x];
            uint8_t *row = B.in + (size_t)w.y * (size_t)B.in_stride;
            long long a1 = 0, a2 = 0;
            for (long long i = tid; i < B.ncols; i += Cfg::THREADS) {
                const long long v = row[i];
                a1 += v;
                a2 += v * v;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                a1 += __shfl_xor_sync(0xffffffffu, a1, o);
                a2 += __shfl_xor_sync(0xffffffffu, a2, o);
            }
            if (lane == 0) {
                red[0][warp] = a1;
                red[1][warp] = a2;
            }
            __syncthreads();
            if (tid == 0) {
                long long s1 = 0, s2 = 0;
                for (int k = 0; k < NWARP; ++k) {
                    s1 += red[0][k];
                    s2 += red[1][k];
                }
                mean_sigma_ll(s1, s2, B.ncols, &s_mu, &s_sig);
            }
            __syncthreads();
            int cm, lo, hi;
            clip_bounds_u8(s_mu, __dmul_rn(f.k_chan, s_sig), &cm, &lo, &hi);
            const uint8_t rep = clip_rep_u8(s_mu);
            for (long long i = tid; i < B.ncols; i += Cfg::THREADS) {
                const int v = row[i];
                if (v >= cm ? v >= hi : v <= lo) row[i] = rep;
            }
            cta_done(f.done, w.x, 0);
        }

    // ---- phase 2: clip each spectrum over the channels (one column per thread) ----
    for (int it; (it = cta_grab(&f.counters[1], f.n_cs, &slot)) >= 0;) {
        const int2 w = f.cs_items[it];
        const FusedBeam &B = f.fb[w.x];
        if (tid == 0)
            s_ok = wait_count(&f.done[3 * w.x + 0], f.k_chan > 0.0 ? (unsigned)B.nchans : 0u, f.err);
        __syncthreads();
        const long long t = (long long)w.y + tid;
        if (f.k_spec > 0.0 && s_ok && tid < kFusedSpecCols && t < B.ncols) {
            long long s1 = 0, s2 = 0;
            const uint8_t *col = B.in + t;
            for (int c = 0; c < B.nchans; ++c) {
                const long long v = col[(size_t)c * (size_t)B.in_stride];
                s1 += v;
                s2 += v * v;
            }
            double mu, sig;
            mean_sigma_ll(s1, s2, B.nchans, &mu, &sig);
            int cm, lo, hi;
            clip_bounds_u8(mu, __dmul_rn(f.k_spec, sig), &cm, &lo, &hi);
            const uint8_t rep = clip_rep_u8(mu);
            uint8_t *cw = B.in + t;
            for (int c = 0; c < B.nchans; ++c) {
                uint8_t *p = cw + (size_t)c * (size_t)B.in_stride;
                const int v = *p;
                if (v >= cm ? v >= hi : v <= lo) *p = rep;
            }
        }
        cta_done(f.done, w.x, 1);
    }

    // ---- phase 3: dedispersion through the packed stream ----
    __syncthreads();
    packed_init_barriers(smem);
    {
        FusedItems src{beams, dd_items, n_dd, &f.counters[2], f.fb, f.done, f.err, f.n_bx > 0,
                       f.n_cs > 0};
        packed_stream<Cfg>(src, smem, rawcap, ps, f.err);
    }
    __syncthreads();
    if (tid == 0) {  // the barriers' memory is used for other data from here on
        uint64_t *bars = reinterpret_cast<uint64_t *>(smem);
        for (int k = 0; k < kPNR; ++k) mbar_inval(&bars[k]);
    }

    // ---- phase 4: boxcar search, one run of tiles of one row per item ----
    // The CTA splits into groups of kFusedBoxThreads threads, each taking items on its own
    // (named barrier 1 + group, its own shared memory), so that one group's barriers overlap
    // the others' work; warps past the last whole group have nothing to do.
    constexpr int NG = Cfg::THREADS / kFusedBoxThreads;
    static_assert(NG >= 1 && NG <= 8, "search groups");
    __shared__ int g_item[NG], g_ok[NG];
    __shared__ double g_mu[NG], g_sig[NG];
    const int grp = tid / kFusedBoxThreads, gt = tid % kFusedBoxThreads;
    __syncthreads();  // the barriers are invalidated before their memory is reused
    if (grp >= NG) return;
    const BoxBarGroup gbar{1 + grp, kFusedBoxThreads};
    unsigned char *gsm = smem + (size_t)grp * kFusedBoxSmem;
    for (;;) {
        gbar.sync();  // the group is done with its previous item and with g_*[grp]
        if (gt == 0) {
            const int it = (int)atomicAdd(&f.counters[3], 1u);
            g_item[grp] = it;
            if (it < f.n_bx) {
                const int4 w = f.bx_items[it];
                const FusedBeam &B = f.fb[w.x];
                g_ok[grp] = wait_count(&f.done[3 * w.x + 2], B.ndd_done, f.err);
                // the row's mean and sigma from its folded moments (k_mom_finish's conversion)
                const unsigned long long *m = B.mom + 3 * (size_t)w.y;
                const long long s1 = (long long)m[0];
                const double e2 =
                    __ddiv_rn(__dadd_rn(__dmul_rn((double)m[2], 18446744073709551616.0),
                                        (double)m[1]),
                              (double)B.nsamp);
                const double mm = __ddiv_rn((double)s1, (double)B.nsamp);
                const double var = __dadd_rn(e2, -__dmul_rn(mm, mm));
                g_mu[grp] = mm;
                g_sig[grp] = var > 0.0 ? __dsqrt_rn(var) : 0.0;
            }
        }
        gbar.sync();
        const int it = g_item[grp];
        if (it >= f.n_bx) break;
        const double mu = g_mu[grp], sig = g_sig[grp];
        if (!g_ok[grp] || !(sig > 0.0)) continue;  // (uniform across the group)
        const int4 w = f.bx_items[it];
        const FusedBeam &B = f.fb[w.x];
        box_run<int32_t, kFusedBoxWidths, kFusedBoxThreads, kFusedBoxK>(
            B.out + (size_t)w.y * (size_t)B.out_stride, B.nsamp, w.z, w.w, mu, sig, f.threshold,
            w.y, B.cands, B.count, f.cap, gsm, gbar, gt, true);
    }
}

// ------------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------------

namespace {

constexpr int kR = 8;
constexpr int kNW = 8;

template <typename TIn, typename TAcc, int DPW, int CC>
void *kernel_ptr()
{
    return reinterpret_cast<void *>(&k_shift_sum<TIn, TAcc, kR, DPW, kNW, CC>);
}

template <typename TIn, typename TAcc, int CC>
void *pick_dpw(int dpw)
{
    switch (dpw) {
    case 4: return kernel_ptr<TIn, TAcc, 4, CC>();
    case 2: return kernel_ptr<TIn, TAcc, 2, CC>();
    default: return kernel_ptr<TIn, TAcc, 1, CC>();
    }
}

void *select_kernel(int in_dtype, int acc_int, int dpw, int cc)
{
    // 1- and 2-byte samples stage 16 channels per step, 4-byte samples 8.
    switch (in_dtype) {
    case MDSM_U8:
        return acc_int ? pick_dpw<uint8_t, int, 16>(dpw) : pick_dpw<uint8_t, float, 16>(dpw);
    case MDSM_U16:
        return acc_int ? pick_dpw<uint16_t, int, 16>(dpw) : pick_dpw<uint16_t, float, 16>(dpw);
    case MDSM_I16:
        return acc_int ? pick_dpw<int16_t, int, 16>(dpw) : pick_dpw<int16_t, float, 16>(dpw);
    case MDSM_I32:
        return pick_dpw<int32_t, int, 8>(dpw);
    case MDSM_F32:
    default:
        return pick_dpw<float, float, 8>(dpw);
    }
    (void)cc;
}

size_t smem_for(const StageGeom &g)
{
    const size_t SZ = dtype_size(g.in_dtype);
    return 128 + (size_t)g.nst * g.cc * g.rowcap * SZ + (size_t)g.nst * g.cc * g.Db * 4 +
           (size_t)g.nst * g.cc * 4;
}

}  // namespace

size_t dtype_size(int dtype)
{
    switch (dtype) {
    case MDSM_U8: return 1;
    case MDSM_U16:
    case MDSM_I16: return 2;
    default: return 4;
    }
}

namespace {

// Per-block (smin, span) and relative shifts of S[g][d][c] for DM blocks of g.Db.
int tile_tables(StageGeom &g, const std::vector<int32_t> &S)
{
    g.nblk = (g.ndms + g.Db - 1) / g.Db;
    g.rel.assign((size_t)g.ngroups * g.nblk * g.nchans * g.Db, 0);
    g.sminspan.assign((size_t)g.ngroups * g.nblk * g.nchans * 2, 0);
    int maxspan = 0;
    for (int gi = 0; gi < g.ngroups; ++gi)
        for (int b = 0; b < g.nblk; ++b) {
            const int d0 = b * g.Db, d1 = std::min(g.ndms, d0 + g.Db);
            for (int c = 0; c < g.nchans; ++c) {
                int lo = INT32_MAX, hi = INT32_MIN;
                for (int d = d0; d < d1; ++d) {
                    const int v = S[((size_t)gi * g.ndms + d) * g.nchans + c];
                    lo = std::min(lo, v);
                    hi = std::max(hi, v);
                }
                const size_t o = (((size_t)gi * g.nblk + b) * g.nchans + c);
                g.sminspan[o * 2] = lo;
                g.sminspan[o * 2 + 1] = hi - lo;
                maxspan = std::max(maxspan, hi - lo);
                for (int d = d0; d < d1; ++d)
                    g.rel[o * g.Db + (d - d0)] = S[((size_t)gi * g.ndms + d) * g.nchans + c] - lo;
            }
        }
    return maxspan;
}

// Dynamic shared memory a packed CTA may take: the device's opt-in limit per block (227 KB on
// GB300; the packed kernels declare no static shared memory), 220 KB if it cannot be read.
size_t packed_smem_limit()
{
    static size_t lim = 0;
    if (!lim) {
        int dev = 0, v = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) ==
                cudaSuccess &&
            v > 0)
            lim = (size_t)v;
        else
            lim = 220 * 1024;
    }
    return lim;
}

template <class Cfg>
size_t packed_smem(int rawcap, int ps)
{
    return 128 + (size_t)kPNR * kPCC * rawcap + (size_t)kPNR * kPCC * Cfg::DBS * 4 +
           (size_t)2 * kPCC * Cfg::DBS * 4 + (size_t)2 * kPCC * Cfg::SPW * ps;
}

// Packed tables for configuration Cfg: offsets (bytes) of (c, d)'s first word from the start
// of the chunk's phase-expanded rows (phase copy, row c % 16, the word; the copies are stored
// phase-major), stored DBS per channel (the padding stays 0).  False if the
// staging does not fit in shared memory.
template <class Cfg>
bool packed_tables(StageGeom &g, const std::vector<int32_t> &S, int kernel_id)
{
    g.Db = Cfg::DB;
    g.T = Cfg::PT;
    g.R = Cfg::PRW * Cfg::SPW;
    g.DPW = Cfg::DPW;
    g.cc = kPCC;
    g.nst = kPNR;
    const int maxspan = tile_tables(g, S);
    // raw row: the tile plus the span, from the 16-byte boundary below smin, in bytes
    const int rawcap =
        (int)(((long long)(Cfg::PT + maxspan) * Cfg::SW + 32 + 15) / 16 * 16) + 16;
    const int ps = rawcap - 16;  // nwp = ps/4 words; the expansion reads word nwp too
    if (packed_smem<Cfg>(rawcap, ps) > packed_smem_limit() || ps >= 4096) return false;
    g.max_span = maxspan;
    g.rowcap = rawcap;
    g.ps = ps;
    const int lomask = 16 / Cfg::SW - 1;  // samples before smin in its 16-byte unit
    std::vector<int32_t> off(g.sminspan.size() / 2 * Cfg::DBS, 0);
    for (size_t o = 0; o < g.sminspan.size() / 2; ++o) {
        const int lo = g.sminspan[o * 2] & lomask;
        const int row = (int)(o % (size_t)g.nchans) % kPCC;  // the channel's row in its chunk
        for (int j = 0; j < g.Db; ++j) {
            const int e = lo + g.rel[o * g.Db + j];  // samples from the staged row's start
            off[o * Cfg::DBS + j] = ((e % Cfg::SPW) * kPCC + row) * ps + (e / Cfg::SPW) * 4;
        }
    }
    g.rel.swap(off);
    g.smem_bytes = packed_smem<Cfg>(rawcap, ps);
    g.kernel = kernel_id;
    return true;
}

}  // namespace

// ---- fused batched launch: its tile shapes, tables and launch ----
namespace {
using FusedCfg0 = CfgU8;                               // 19 warps x 2 trials, 512 samples
using FusedCfg1 = CfgU8w16;                            // 16 x 2, 512
using FusedCfg2 = PackedCfg<1, 19, 2, false, 256>;     // 19 x 2, 256
using FusedCfg3 = PackedCfg<1, 16, 2, false, 768>;     // 16 x 2, 768

template <class Cfg>
size_t fused_smem_t(int rawcap, int ps)
{
    return std::max(packed_smem<Cfg>(rawcap, ps),
                    (size_t)(Cfg::THREADS / kFusedBoxThreads) * kFusedBoxSmem);
}

template <class Cfg>
mdsm_status fused_launch_t(const FusedArgs &f, const KArgs *kargs, const int4 *items, int n_dd,
                           int rawcap, int ps, cudaStream_t st)
{
    const size_t smem = fused_smem_t<Cfg>(rawcap, ps);
    cudaFuncAttributes at;
    MDSM_CUDA_TRY(cudaFuncGetAttributes(&at, k_batch_fused<Cfg>));
    if (smem + at.sharedSizeBytes > packed_smem_limit())
        return fail(MDSM_EINVAL, "fused batch: staging does not fit this tile shape");
    MDSM_CUDA_TRY(cudaFuncSetAttribute(k_batch_fused<Cfg>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int dev = 0, sms = 0;
    MDSM_CUDA_TRY(cudaGetDevice(&dev));
    MDSM_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    k_batch_fused<Cfg><<<sms, Cfg::THREADS, smem, st>>>(f, kargs, items, n_dd, rawcap, ps);
    MDSM_CUDA_TRY(cudaGetLastError());
    return MDSM_OK;
}
}  // namespace

int fused_num_shapes() { return 4; }

int fused_box_tile() { return FusedBoxGeom::TILE; }

FusedShapeInfo fused_shape_info(int shape)
{
    switch (shape) {
    case 0: return {FusedCfg0::DB, FusedCfg0::PT, FusedCfg0::NW};
    case 1: return {FusedCfg1::DB, FusedCfg1::PT, FusedCfg1::NW};
    case 2: return {FusedCfg2::DB, FusedCfg2::PT, FusedCfg2::NW};
    default: return {FusedCfg3::DB, FusedCfg3::PT, FusedCfg3::NW};
    }
}

// g: a copy of a uint8 brute-force plan's stage (its geometry); S: the plan's shift table.
mdsm_status fused_tables(int shape, StageGeom &g, const std::vector<int32_t> &S)
{
    g.out_u16 = 0;
    g.out_i32 = 1;
    g.d_rel = nullptr;
    g.d_sminspan = nullptr;
    bool ok = false;
    switch (shape) {
    case 0: ok = packed_tables<FusedCfg0>(g, S, 2); break;
    case 1: ok = packed_tables<FusedCfg1>(g, S, 2); break;
    case 2: ok = packed_tables<FusedCfg2>(g, S, 2); break;
    default: ok = packed_tables<FusedCfg3>(g, S, 2); break;
    }
    if (!ok) return fail(MDSM_EINVAL, "fused batch: a beam's staging does not fit this shape");
    return upload_stage(g);
}

mdsm_status fused_launch(int shape, const FusedArgs &f, const KArgs *d_kargs, const int4 *d_items,
                         int n_dd, int rawcap, int ps, cudaStream_t st)
{
    switch (shape) {
    case 0: return fused_launch_t<FusedCfg0>(f, d_kargs, d_items, n_dd, rawcap, ps, st);
    case 1: return fused_launch_t<FusedCfg1>(f, d_kargs, d_items, n_dd, rawcap, ps, st);
    case 2: return fused_launch_t<FusedCfg2>(f, d_kargs, d_items, n_dd, rawcap, ps, st);
    default: return fused_launch_t<FusedCfg3>(f, d_kargs, d_items, n_dd, rawcap, ps, st);
    }
}

// KArgs of one beam of the fused launch (with the launch's common staging geometry)
KArgs fused_kargs(const StageGeom &g, const void *d_rel_common, const unsigned char *in,
                  long long in_stride, int32_t *out, long long out_stride, int rawcap, int ps,
                  unsigned long long *mom, unsigned *err)
{
    KArgs a;
    std::memset(&a, 0, sizeof a);
    a.in = in;
    a.in_stride = in_stride;
    a.out = reinterpret_cast<unsigned char *>(out);
    a.out_stride = out_stride;
    a.rel = static_cast<const int32_t *>(d_rel_common);
    a.sminspan = g.d_sminspan;
    a.nchans = g.nchans;
    a.ndms = g.ndms;
    a.nsamp = g.nsamp;
    a.nblk = g.nblk;
    a.rowcap = rawcap;
    a.nst = g.nst;
    a.out_i32 = 1;
    a.ps = ps;
    a.err = err;
    a.mom = mom;
    a.mom_group_rows = g.ndms;
    return a;
}

// Tile S[g][d][c] for the kernel.  Fails if any shift is negative.  uint8 and uint16 samples
// use the packed kernels (Db 38 / 16, T 512) unless g.kernel == 1 asks for the generic one or
// their staging does not fit; everything else uses the generic kernel with Db 32/16/8.
mdsm_status build_stage_tables(StageGeom &g, const std::vector<int32_t> &S)
{
    const int SZ = (int)dtype_size(g.in_dtype);
    const long long need = (long long)g.ngroups * g.ndms * g.nchans;
    if ((long long)S.size() != need) return fail(MDSM_EINVAL, "shift table size mismatch");
    int mx = 0;
    for (long long i = 0; i < need; ++i) {
        if (S[(size_t)i] < 0)
            return fail(MDSM_EINVAL,
                        "negative sample shift: channel 0 must be the highest frequency");
        mx = std::max(mx, (int)S[(size_t)i]);
    }
    g.max_shift = mx;
    // the packed kernels sum exactly in int32: only where every sum fits
    if (g.kernel != 1) {
        if (g.in_dtype == MDSM_U8 && (long long)g.nchans * 255 <= 0x7fffffffLL) {
            // 38-trial blocks run ~5 % faster per trial than 32-trial ones; take 32 where the
            // last 38-trial block would leave more than that idle (e.g. 64 or 128 trials)
            const int n38 = (g.ndms + CfgU8::DB - 1) / CfgU8::DB * CfgU8::DB;
            const int n32 = (g.ndms + CfgU8w16::DB - 1) / CfgU8w16::DB * CfgU8w16::DB;
            const bool w38 = n38 <= 1.05 * n32;
            if (g.out_u16) {
                if (w38 && (packed_tables<CfgU8to16T<19, 1024>>(g, S, 2) ||
                            packed_tables<CfgU8to16T<19, 768>>(g, S, 2) ||
                            packed_tables<CfgU8to16T<19, 512>>(g, S, 2)))
                    return MDSM_OK;
                if (packed_tables<CfgU8to16T<16, 1024>>(g, S, 2) ||
                    packed_tables<CfgU8to16T<16, 768>>(g, S, 2) ||
                    packed_tables<CfgU8to16T<16, 512>>(g, S, 2))
                    return MDSM_OK;
            } else {
                if (w38 && packed_tables<CfgU8>(g, S, 2)) return MDSM_OK;
                if (packed_tables<CfgU8w16>(g, S, 2)) return MDSM_OK;
            }
        }
        if ((g.in_dtype == MDSM_U16 || g.in_dtype == MDSM_I16) && !g.out_u16 &&
            (long long)g.nchans * 65535 <= 0x7fffffffLL &&
            (packed_tables<CfgU16T<768>>(g, S, 3) || packed_tables<CfgU16T<512>>(g, S, 3)))
            return MDSM_OK;
    }
    g.out_u16 = 0;  // only the uint8 packed kernel writes uint16 sums
    g.kernel = 1;
    g.R = kR;
    g.T = 32 * kR;
    g.cc = SZ == 4 ? 8 : 16;
    // Try Db = 32, 16, 8 until the staged rows fit in shared memory.
    const int dpws[3] = {4, 2, 1};
    int first = g.DPW == 4 ? 0 : (g.DPW == 2 ? 1 : 2);
    for (int i = first; i < 3; ++i) {
        g.DPW = dpws[i];
        g.Db = kNW * g.DPW;
        const int maxspan = tile_tables(g, S);
        g.max_span = maxspan;
        const long long bytes = (long long)(g.T + maxspan) * SZ + 32;
        g.rowcap = (int)(((bytes + 15) / 16) * 16 / SZ);
        g.nst = 3;
        g.smem_bytes = smem_for(g);
        if (g.smem_bytes > 200 * 1024) {
            g.nst = 2;
            g.smem_bytes = smem_for(g);
        }
        if (g.smem_bytes <= 200 * 1024) return MDSM_OK;
    }
    return fail(MDSM_EINVAL, "DM plan too wide for shared-memory staging (shift span " +
                                 std::to_string(g.max_span) + " per 8 DM trials)");
}

mdsm_status upload_stage(StageGeom &g)
{
    free_stage(g);
    MDSM_CUDA_TRY(cudaMalloc(&g.d_rel, g.rel.size() * sizeof(int32_t)));
    MDSM_CUDA_TRY(cudaMalloc(&g.d_sminspan, g.sminspan.size() * sizeof(int32_t)));
    MDSM_CUDA_TRY(cudaMemcpy(g.d_rel, g.rel.data(), g.rel.size() * sizeof(int32_t),
                             cudaMemcpyHostToDevice));
    MDSM_CUDA_TRY(cudaMemcpy(g.d_sminspan, g.sminspan.data(),
                             g.sminspan.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    return MDSM_OK;
}

void free_stage(StageGeom &g)
{
    if (g.d_rel) cudaFree(g.d_rel);
    if (g.d_sminspan) cudaFree(g.d_sminspan);
    g.d_rel = nullptr;
    g.d_sminspan = nullptr;
}

long long stage_in_bytes(const StageGeom &g, long long in_stride, long long in_group_stride)
{
    const long long SZ = (long long)dtype_size(g.in_dtype);
    const long long ntiles = (g.nsamp + g.T - 1) / g.T;
    const long long last = ((ntiles * g.T + g.max_shift) * SZ + 15) / 16 * 16;
    return ((long long)(g.ngroups - 1) * in_group_stride + (long long)(g.nchans - 1) * in_stride) *
               SZ + last;
}

mdsm_status launch_stage(const StageGeom &g, const void *in, long long in_stride,
                         long long in_group_stride, void *out, long long out_stride,
                         long long out_group_stride, unsigned *d_err, cudaStream_t st,
                         int *launches, long long nsamp_run, unsigned long long *mom,
                         long long mom_group_rows)
{
    const int SZ = (int)dtype_size(g.in_dtype);
    const long long nsamp = nsamp_run >= 0 ? std::min<long long>(nsamp_run, g.nsamp) : g.nsamp;
    if (nsamp == 0) return MDSM_OK;
    if (((uintptr_t)in & 15) != 0) return fail(MDSM_EINVAL, "input must be 16-byte aligned");
    if ((in_stride * SZ) % 16 != 0)
        return fail(MDSM_EINVAL, "input row pitch must be a multiple of 16 bytes");
    if ((in_group_stride * SZ) % 16 != 0)
        return fail(MDSM_EINVAL, "input group pitch must be a multiple of 16 bytes");
    void *fn = select_kernel(g.in_dtype, g.acc_int, g.DPW, g.cc);
    unsigned threads = kNW * 32;
    bool persistent = true;  // the packed kernels: a persistent grid over (block, tile, group)
    if (g.kernel == 2 && g.Db == CfgU8::DB) {
        fn = !g.out_u16     ? reinterpret_cast<void *>(&k_shift_sum_packed<CfgU8>)
             : g.T == 1024 ? reinterpret_cast<void *>(&k_shift_sum_packed<CfgU8to16T<19, 1024>>)
             : g.T == 768  ? reinterpret_cast<void *>(&k_shift_sum_packed<CfgU8to16T<19, 768>>)
                           : reinterpret_cast<void *>(&k_shift_sum_packed<CfgU8to16T<19, 512>>);
        threads = CfgU8::THREADS;
    } else if (g.kernel == 2) {
        fn = !g.out_u16     ? reinterpret_cast<void *>(&k_shift_sum_packed<CfgU8w16>)
             : g.T == 1024 ? reinterpret_cast<void *>(&k_shift_sum_packed<CfgU8to16T<16, 1024>>)
             : g.T == 768  ? reinterpret_cast<void *>(&k_shift_sum_packed<CfgU8to16T<16, 768>>)
                           : reinterpret_cast<void *>(&k_shift_sum_packed<CfgU8to16T<16, 512>>);
        threads = CfgU8w16::THREADS;
    } else if (g.kernel == 3) {
        const bool sgn = g.in_dtype == MDSM_I16;
        fn = g.T == 768 ? (sgn ? reinterpret_cast<void *>(&k_shift_sum_packed<CfgI16T<768>>)
                               : reinterpret_cast<void *>(&k_shift_sum_packed<CfgU16T<768>>))
                        : (sgn ? reinterpret_cast<void *>(&k_shift_sum_packed<CfgI16T<512>>)
                               : reinterpret_cast<void *>(&k_shift_sum_packed<CfgU16T<512>>));
        threads = CfgU16T<512>::THREADS;
    } else {
        persistent = false;
    }
    MDSM_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)g.smem_bytes));
    KArgs a;
    a.in = static_cast<const unsigned char *>(in);
    a.in_stride = in_stride;
    a.in_group_stride = in_group_stride;
    a.out = static_cast<unsigned char *>(out);
    a.out_stride = out_stride;
    a.out_group_stride = out_group_stride;
    a.rel = g.d_rel;
    a.sminspan = g.d_sminspan;
    a.nchans = g.nchans;
    a.ndms = g.ndms;
    a.nsamp = (int)nsamp;
    a.nblk = g.nblk;
    a.rowcap = g.rowcap;
    a.nst = g.nst;
    a.out_i32 = g.out_i32;
    a.ps = g.ps;
    a.err = d_err;
    a.mom = (mom && stage_folds_moments(g)) ? mom : nullptr;
    a.mom_group_rows = mom_group_rows;
    const long long ntiles = (nsamp + g.T - 1) / g.T;
    if (persistent) {
        // at most one CTA per SM walks the (DM block, tile, group) items
        const long long nitems = (long long)g.nblk * ntiles * g.ngroups;
        if (nitems > 0x7fffffffLL) return fail(MDSM_EINVAL, "block too long for one launch");
        int dev = 0, sms = 0;
        MDSM_CUDA_TRY(cudaGetDevice(&dev));
        MDSM_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        int nt = (int)ntiles, ni = (int)nitems;
        void *args[] = {&a, &nt, &ni};
        const unsigned grid = (unsigned)std::min<long long>(sms, nitems);
        MDSM_CUDA_TRY(cudaLaunchKernel(fn, dim3(grid), dim3(threads), args, g.smem_bytes, st));
    } else {
        if (ntiles > 65535 || g.ngroups > 65535)
            return fail(MDSM_EINVAL, "block too long for one launch");
        dim3 grid((unsigned)g.nblk, (unsigned)ntiles, (unsigned)g.ngroups);
        void *args[] = {&a};
        MDSM_CUDA_TRY(cudaLaunchKernel(fn, grid, dim3(threads), args, g.smem_bytes, st));
    }
    if (launches) *launches += 1;
    return MDSM_OK;
}

// ------------------------------------------------------------------------------------------
// batched persistent launch over several brute-force plans
// ------------------------------------------------------------------------------------------

namespace {
// beams the persistent batch kernel (38-trial uint8 blocks) runs; others launch alone
bool in_batch_kernel(const StageGeom &g)
{
    return g.kernel == 2 && g.Db == CfgU8::DB && !g.out_u16;
}
}  // namespace

mdsm_status batch_prepare(BatchState &b, const std::vector<BatchBeam> &beams)
{
    batch_release(b);
    b.beams = beams;
    int rawcap = 0, ps = 0;
    for (const BatchBeam &bb : beams)
        if (in_batch_kernel(*bb.g)) {
            rawcap = std::max(rawcap, bb.g->rowcap);
            ps = std::max(ps, bb.g->ps);
        }
    b.rawcap = rawcap;
    b.ps = ps;
    b.smem = rawcap ? packed_smem<CfgU8>(rawcap, ps) : 0;
    if (b.smem > packed_smem_limit())
        return fail(MDSM_EINVAL, "batch: common staging does not fit");
    // (each packed beam keeps its plan's offsets and phase stride: the launch expands a beam's
    // chunks with its own stride; the shared-memory buffers are sized for the widest)
    MDSM_CUDA_TRY(cudaMalloc(&b.d_counter, sizeof(unsigned)));
    MDSM_CUDA_TRY(cudaMalloc(&b.d_kargs, std::max<size_t>(1, beams.size()) * sizeof(KArgs)));
    return MDSM_OK;
}

// Items of the packed beams, largest channel count first; within a beam all DM blocks of a
// time tile are adjacent (tile_major) so the tile's rows are reused from L2, or all tiles of a
// DM block are adjacent (!tile_major).
mdsm_status batch_set_buffers(BatchState &b, const std::vector<const void *> &in,
                              const std::vector<long long> &in_stride,
                              const std::vector<void *> &out,
                              const std::vector<long long> &out_stride, unsigned *d_err,
                              int tile_major)
{
    if (in.size() != b.beams.size() || out.size() != b.beams.size())
        return fail(MDSM_EINVAL, "batch: one input and one output per beam");
    std::vector<KArgs> ka(b.beams.size());
    std::vector<int> order(b.beams.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        return b.beams[x].g->nchans > b.beams[y].g->nchans;
    });
    std::vector<int4> items;
    for (size_t i = 0; i < b.beams.size(); ++i) {
        const StageGeom &g = *b.beams[i].g;
        b.beams[i].in = in[i];
        b.beams[i].in_stride = in_stride[i];
        b.beams[i].out = out[i];
        b.beams[i].out_stride = out_stride[i];
        if (((uintptr_t)in[i] & 15) != 0 || (in_stride[i] * (long long)dtype_size(g.in_dtype)) % 16)
            return fail(MDSM_EINVAL, "batch: inputs must be 16-byte aligned with 16-byte pitches");
        KArgs &a = ka[i];
        std::memset(&a, 0, sizeof a);
        a.in = static_cast<const unsigned char *>(in[i]);
        a.in_stride = in_stride[i];
        a.in_group_stride = 0;
        a.out = static_cast<unsigned char *>(out[i]);
        a.out_stride = out_stride[i];
        a.out_group_stride = 0;
        a.rel = g.d_rel;
        a.sminspan = g.d_sminspan;
        a.nchans = g.nchans;
        a.ndms = g.ndms;
        a.nsamp = g.nsamp;
        a.nblk = g.nblk;
        a.rowcap = in_batch_kernel(g) ? b.rawcap : g.rowcap;
        a.nst = g.nst;
        a.out_i32 = g.out_i32;
        a.ps = g.ps;
        a.err = d_err;
    }
    for (int i : order) {
        const StageGeom &g = *b.beams[i].g;
        if (!in_batch_kernel(g)) continue;
        const int ntiles = (g.nsamp + g.T - 1) / g.T;
        if (tile_major) {
            for (int t = 0; t < ntiles; ++t)
                for (int k = 0; k < g.nblk; ++k) items.push_back(make_int4(i, k, t, 0));
        } else {
            for (int k = 0; k < g.nblk; ++k)
                for (int t = 0; t < ntiles; ++t) items.push_back(make_int4(i, k, t, 0));
        }
    }
    b.tile_major = tile_major;
    b.nitems = (int)items.size();
    if (b.d_items) cudaFree(b.d_items);
    b.d_items = nullptr;
    if (!items.empty()) {
        MDSM_CUDA_TRY(cudaMalloc(&b.d_items, items.size() * sizeof(int4)));
        MDSM_CUDA_TRY(cudaMemcpy(b.d_items, items.data(), items.size() * sizeof(int4),
                                 cudaMemcpyHostToDevice));
    }
    MDSM_CUDA_TRY(cudaMemcpy(b.d_kargs, ka.data(), ka.size() * sizeof(KArgs),
                             cudaMemcpyHostToDevice));
    b.d_err = d_err;
    return MDSM_OK;
}

// mode 0: one persistent launch for the packed beams (plus separate launches for the others);
// mode 1: every beam its own launch.
mdsm_status batch_launch(BatchState &b, int mode, cudaStream_t st, int *launches)
{
    if (mode == 0 && b.nitems > 0) {
        MDSM_CUDA_TRY(cudaMemsetAsync(b.d_counter, 0, sizeof(unsigned), st));
        MDSM_CUDA_TRY(cudaFuncSetAttribute(k_shift_sum_u8x4_batch,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)b.smem));
        int dev = 0, sms = 0;
        MDSM_CUDA_TRY(cudaGetDevice(&dev));
        MDSM_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        const int grid = std::min(sms, b.nitems);
        k_shift_sum_u8x4_batch<<<grid, CfgU8::THREADS, b.smem, st>>>(
            reinterpret_cast<const KArgs *>(b.d_kargs), reinterpret_cast<const int4 *>(b.d_items),
            b.nitems, b.d_counter, b.rawcap, b.ps, b.d_err);
        MDSM_CUDA_TRY(cudaGetLastError());
        if (launches) *launches += 1;
    }
    for (const BatchBeam &bb : b.beams) {
        if (mode == 0 && in_batch_kernel(*bb.g)) continue;
        MDSM_TRY(launch_stage(*bb.g, bb.in, bb.in_stride, 0, bb.out, bb.out_stride, 0, b.d_err, st,
                              launches));
    }
    return MDSM_OK;
}

void batch_release(BatchState &b)
{
    if (b.d_items) cudaFree(b.d_items);
    if (b.d_counter) cudaFree(b.d_counter);
    if (b.d_kargs) cudaFree(b.d_kargs);
    b.d_items = nullptr;
    b.d_counter = nullptr;
    b.d_kargs = nullptr;
    b.nitems = 0;
}

// Self-test of the bounded-wait path: thread 0 waits, with the wait the kernels above use, on
// an mbarrier nothing arrives at; after `limit` try_waits the wait gives up, records
// ERR_WAIT_TIMEOUT in *err as a starved wait in a dedispersion kernel would, and the kernel
// returns.  No copy is in flight, so nothing writes the barrier's shared memory afterwards.
__global__ void k_wait_selftest(unsigned *err, uint32_t limit)
{
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) mbar_wait_bounded(&bar, 0u, err, ERR_WAIT_TIMEOUT, limit);
}

mdsm_status wait_selftest(unsigned *d_err, unsigned limit, cudaStream_t st)
{
    k_wait_selftest<<<1, 32, 0, st>>>(d_err, limit);
    MDSM_CUDA_TRY(cudaGetLastError());
    return MDSM_OK;
}

}  // namespace mdsm
