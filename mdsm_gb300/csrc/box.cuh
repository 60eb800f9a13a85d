// box.cuh -- the boxcar single-pulse search's tile loop as a device function, shared by the
// standalone search kernel (detect.cu) and the fused batched launch (dedisp.cu).
//
// Widths 1, 2, 4, ..., 2^(NW-1); per DM row the mean and sigma come from the caller.  A run of
// consecutive 2048-sample tiles of one row is searched by a group of THREADS threads: the
// whole CTA (BoxBarCta) or one of several groups of a CTA, each with its own named barrier and
// shared memory (BoxBarGroup), so that one wide CTA runs several searches whose barriers
// overlap.  The samples of the next tile are copied into shared memory
// (cp.async) while the current one is searched.  Arithmetic per sample and width is FP32,
// explicitly rounded, in the oracle's order; each thread owns the position pairs
// (2 tid + 2 THREADS q, +1), keeps their boxcar sums and best SNR in registers across the
// widths and reads only partner sums from shared memory: two widths per step (B_2u and B_4u
// from B_u, three 8-byte loads per pair), so two widths cost per pair three shared loads, one
// shared store, one barrier (the sums alternate between two buffers), and per width three
// paired FP32 operations and two maxima.  Which
// width gave the best SNR is needed only where the best passes the threshold (few
// positions): there box_best_at forms it again, with the same sums.  Candidates are local
// maxima of the best SNR over max(w/2, 1) samples on each side.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "internal.h"
#include "ptx.cuh"

namespace mdsm {

constexpr int kBoxTile = 2048;   // output samples per tile

// Two FP32 lanes at once (Blackwell add/mul.f32x2, each lane rounded to nearest as the scalar
// operation would be).  The operands are formed as register pairs (mov.b64 of two .f32), so
// packing costs no integer instructions.
__device__ __forceinline__ float2 add_f2(float2 a, float2 b)
{
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\t"
        "mov.b64 rb, {%4, %5};\n\t"
        "add.rn.f32x2 rd, ra, rb;\n\t"
        "mov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
__device__ __forceinline__ float2 mul_f2(float2 a, float2 b)
{
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\t"
        "mov.b64 rb, {%4, %5};\n\t"
        "mul.rn.f32x2 rd, ra, rb;\n\t"
        "mov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}

// max(a, b, c) in one instruction (three-input max.f32, sm_100 and later); for values that
// are not NaN the same as two two-input maxima.
__device__ __forceinline__ float fmax3(float a, float b, float c)
{
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// Staged samples for NW widths: the region [t0 - HL, t0 + TILE + HL + wmax - 1), rounded up to
// whole pairs of positions per thread; each sum buffer has wmax floats more so that partner
// reads past the region stay inside it (those positions feed no kept boxcar).
template <int NW, int THREADS>
struct BoxGeom {
    static constexpr int WMAX = 1 << (NW - 1);
    static constexpr int HL = WMAX / 2 > 1 ? WMAX / 2 : 1;
    static constexpr int SPAN = kBoxTile + 2 * HL + WMAX;  // samples a kept boxcar can touch
    static constexpr int NBEST = kBoxTile + 2 * HL;        // positions with a best value
    static constexpr int PAIRS = (SPAN + 2 * THREADS - 1) / (2 * THREADS);  // per thread
    // floats; even, so the second buffer and the pairs in it stay 8-byte aligned
    static constexpr int BUF = PAIRS * 2 * THREADS + (WMAX < 2 ? 2 : WMAX);
    // shared memory of box_run: two sum buffers, the best SNR of NBEST positions, the next
    // tile's samples, 1 / (sigma sqrt(w)) per width (16 floats)
    static constexpr size_t SMEM =
        (size_t)BUF * 8 + (size_t)NBEST * 4 + (size_t)PAIRS * 2 * THREADS * 4 + 64;
    static_assert(NW <= 16, "widths");
    static_assert(BUF % 2 == 0 && NBEST % 2 == 0, "pairs of positions");
    static_assert((THREADS & (THREADS - 1)) == 0, "power-of-two thread count");
};

// Best SNR over the widths 1, 2, ..., 2^(NW-1) at series position t (0 <= t < n) and the first
// width reaching it, for a position that passed the threshold.  The sums are formed in the
// order of the tile loop (B_w[t] = B_{w/2}[t] + B_{w/2}[t + w/2]): a pairwise sum over the
// samples in order, merging equal-sized partial sums as a binary counter carries, completes
// the width-w sum exactly when w samples have been added.
template <typename T, int NW>
__device__ __noinline__ void box_best_at(const T *__restrict__ r, long long t, long long n,
                                         float mu_f, const float *inv_w, float *bv, int *bw)
{
    float st[NW];
    int sp = 0;
    float best = -INFINITY;
    int width = 0;
    for (int j = 0; j < (1 << (NW - 1)) && t + j < n; ++j) {
        st[sp++] = (float)__ldg(r + t + j);
        for (int k = j + 1; (k & 1) == 0; k >>= 1) {
            st[sp - 2] = __fadd_rn(st[sp - 2], st[sp - 1]);
            --sp;
        }
        if (((j + 1) & j) == 0) {  // j + 1 = w, a power of two: st[0] is the width-w sum
            const int w = j + 1;
            const int l = 31 - __clz(w);
            const float sv = __fmul_rn(__fadd_rn(st[0], -__fmul_rn((float)w, mu_f)), inv_w[l]);
            if (sv > best) {
                best = sv;
                width = w;
            }
        }
    }
    *bv = best;
    *bw = width;
}

// Asynchronous copy of one tile's samples into NB: this thread's pairs
// (r0 + 2 tid + 2 THREADS q, +1), zero outside the series.  Only the issuing thread reads
// them back, so its own wait is the only synchronisation.
template <typename T, int PAIRS, int THREADS>
__device__ __forceinline__ void box_prefetch(uint32_t *NB, const T *__restrict__ r, long long r0,
                                             long long n, int tid)
{
    static_assert(sizeof(T) == 4, "4-byte samples");
    const bool inside = r0 >= 0 && r0 + PAIRS * 2 * THREADS <= n;
    if (inside && ((uintptr_t)(r + r0) & 7) == 0) {
        // the whole region inside the series, pairs 8-byte aligned: one 8-byte copy a pair
        const T *base = r + r0;
#pragma unroll
        for (int q = 0; q < PAIRS; ++q) {
            const int i = 2 * tid + 2 * THREADS * q;
            cp_async8(NB + i, base + i);
        }
    } else {
#pragma unroll
        for (int q = 0; q < PAIRS; ++q)
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int i = 2 * tid + 2 * THREADS * q + e;
                const long long t = r0 + i;
                const bool in = t >= 0 && t < n;
                cp_async4(NB + i, in ? r + t : r, in ? 4u : 0u);
            }
    }
    cp_async_commit();
}

// The search group's barriers.  BoxBarCta: the group is the whole CTA (threads at or past
// the group's size only take part in the barriers).  BoxBarGroup: named barrier `id` (1..15)
// of `count` threads, a multiple of 32 (whole warps).
struct BoxBarCta {
    __device__ __forceinline__ void sync() const { __syncthreads(); }
    __device__ __forceinline__ bool any(bool p) const { return __syncthreads_or(p) != 0; }
};
struct BoxBarGroup {
    int id, count;
    __device__ __forceinline__ void sync() const
    {
        asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
    }
    __device__ __forceinline__ bool any(bool p) const
    {
        unsigned r;
        asm volatile(
            "{\n\t.reg .pred p, q;\n\t"
            "setp.ne.u32 p, %1, 0;\n\t"
            "bar.red.or.pred q, %2, %3, p;\n\t"
            "selp.u32 %0, 1, 0, q;\n\t}"
            : "=r"(r)
            : "r"((unsigned)p), "r"(id), "r"(count)
            : "memory");
        return r != 0;
    }
};

template <typename T>
__device__ __forceinline__ float box_value(uint32_t raw)
{
    if constexpr (std::is_same<T, float>::value)
        return __uint_as_float(raw);
    else
        return (float)(int32_t)raw;
}

// Tiles [tile_lo, tile_hi) of row r (n samples, DM index d) with the row's mean and sigma
// (sigma > 0), searched by the calling group: `active` threads with group index tid in
// [0, THREADS) (every thread of the group's barrier calls it); sm holds
// BoxGeom<NW, THREADS>::SMEM bytes of the group's own.  Candidates (d, sample, width, snr) go
// to cands[atomicAdd(count)] below cap.  When it returns, no copy is in flight (the last tile
// prefetches nothing); the caller synchronises the group before sm is written again.
template <typename T, int NW, int THREADS, class Bar>
__device__ __forceinline__ void box_run(const T *__restrict__ r, long long n, long long tile_lo,
                                        long long tile_hi, double mu, double sig, double threshold,
                                        int d, DevCand *__restrict__ cands,
                                        unsigned long long *__restrict__ count, long long cap,
                                        unsigned char *sm, const Bar &bar, int tid_in, bool active)
{
    using G = BoxGeom<NW, THREADS>;
    constexpr int HL = G::HL, NBEST = G::NBEST, PAIRS = G::PAIRS;
    float *B0 = reinterpret_cast<float *>(sm), *B1 = B0 + G::BUF;
    float *best_s = B1 + G::BUF;
    uint32_t *NB = reinterpret_cast<uint32_t *>(best_s + NBEST);  // next tile's samples
    float *inv_w = reinterpret_cast<float *>(NB + PAIRS * 2 * THREADS);
    // (the mask tells the compiler tid < THREADS, so range tests fold at compile time for all
    // but the last pair)
    const int tid = tid_in & (THREADS - 1);
    const float mu_f = __double2float_rn(mu);
    const float thr = __double2float_rn(threshold);
    // 1 / (sigma sqrt(w)) in FP64, rounded to FP32, once per width (FP64 is a slow pipe here)
    if (active && tid < NW)
        inv_w[tid] = __double2float_rn(__ddiv_rn(1.0, __dmul_rn(sig, __dsqrt_rn((double)(1 << tid)))));
    // every staged sample and every boxcar of the tile inside the series: no per-element tests
    auto inside = [&](long long tile) {
        const long long r0 = tile * kBoxTile - HL;
        return r0 >= 0 && r0 + PAIRS * 2 * THREADS <= n;
    };
    if (active) box_prefetch<T, PAIRS, THREADS>(NB, r, tile_lo * kBoxTile - HL, n, tid);
    for (long long tile = tile_lo; tile < tile_hi; ++tile) {
        const long long t0 = tile * kBoxTile;
        const long long r0 = t0 - HL;  // series index of B[0] and best[0]
        const bool interior = inside(tile);  // (uniform across the group)
        float2 b[PAIRS], best[PAIRS];
        if (active) {
            cp_async_wait_all();
#pragma unroll
            for (int q = 0; q < PAIRS; ++q) {
                const int i = 2 * tid + 2 * THREADS * q;
                const uint2 raw = *reinterpret_cast<const uint2 *>(NB + i);
                b[q] = make_float2(box_value<T>(raw.x), box_value<T>(raw.y));
                *reinterpret_cast<float2 *>(B0 + i) = b[q];
                best[q] = make_float2(-INFINITY, -INFINITY);
            }
        }
        if (active && tile + 1 < tile_hi)  // in flight while this tile is searched
            box_prefetch<T, PAIRS, THREADS>(NB, r, r0 + kBoxTile, n, tid);
        bar.sync();  // B0 (and inv_w) written (each thread reads back only its own NB words)
        // The widths of this tile, compiled twice: for tiles whose every staged sample and
        // boxcar lies inside the series (no per-position range tests) and for the edges.
        auto widths = [&](auto interior_tag) {
            constexpr bool INTERIOR = decltype(interior_tag)::value;
            // SNR of the pair's width-2^l sums v
            auto snr = [&](float2 v, int l) {
                const float wm = __fmul_rn((float)(1 << l), mu_f);
                const float inv = inv_w[l];
                return mul_f2(add_f2(v, make_float2(-wm, -wm)), make_float2(inv, inv));
            };
            // best SNR of pair q over widths 2^l (sums v) and, when l4 >= 0, 2^l4 (sums v4).
            // Interior tiles need no range tests and keep values at positions past NBEST
            // (never read); edge tiles take each width where its boxcar lies in the series.
            auto score = [&](int q, float2 v, int l, float2 v4, int l4) {
                const int i = 2 * tid + 2 * THREADS * q;
                if (INTERIOR) {
                    const float2 sv = snr(v, l);
                    if (l4 >= 0) {
                        const float2 s4 = snr(v4, l4);
                        best[q].x = fmax3(best[q].x, sv.x, s4.x);
                        best[q].y = fmax3(best[q].y, sv.y, s4.y);
                    } else {
                        best[q].x = fmaxf(best[q].x, sv.x);
                        best[q].y = fmaxf(best[q].y, sv.y);
                    }
                    return;
                }
                if (i >= NBEST) return;  // i even and NBEST even: i + 1 < NBEST too
                const long long t = r0 + i;
#pragma unroll
                for (int k = 0; k < 2; ++k) {
                    const int lk = k ? l4 : l;
                    if (lk < 0) continue;
                    const int w = 1 << lk;
                    const float2 sv = snr(k ? v4 : v, lk);
                    if (t >= 0 && t + w <= n) best[q].x = fmaxf(best[q].x, sv.x);
                    if (t + 1 >= 0 && t + 1 + w <= n) best[q].y = fmaxf(best[q].y, sv.y);
                }
            };
            if (active) {
#pragma unroll
                for (int q = 0; q < PAIRS; ++q) {
                    if (INTERIOR)
                        best[q] = snr(b[q], 0);  // (best starts at -inf: max(-inf, x) = x)
                    else
                        score(q, b[q], 0, b[q], -1);
                }
            }
            // Two widths per step: from B_u (u = 4^(s-1), in B0 for odd s, else B1)
            //   B_2u[i] = B_u[i] + B_u[i + u]
            //   B_4u[i] = B_2u[i] + B_2u[i + 2u],  B_2u[i + 2u] = B_u[i + 2u] + B_u[i + 3u]
            // the same roundings, operands and order as one width per step, with three
            // partner loads, one store and one barrier per two widths.
#pragma unroll
            for (int s = 1; 2 * s - 1 < NW; ++s) {
                const int u = 1 << (2 * s - 2);
                const bool two = 2 * s < NW;       // width 4u searched too
                const bool more = 2 * s + 1 < NW;  // a further step reads B_4u
                const float *cur = (s & 1) ? B0 : B1;
                float *nxt = (s & 1) ? B1 : B0;
                if (active) {
#pragma unroll
                    for (int q = 0; q < PAIRS; ++q) {
                        const int i = 2 * tid + 2 * THREADS * q;
                        float2 p1, p23 = make_float2(0.f, 0.f);
                        if (u == 1) {
                            const float2 c = *reinterpret_cast<const float2 *>(cur + i + 2);
                            p1 = make_float2(b[q].y, c.x);
                            if (two) p23 = add_f2(c, make_float2(c.y, cur[i + 4]));
                        } else {
                            p1 = *reinterpret_cast<const float2 *>(cur + i + u);
                            if (two)
                                p23 = add_f2(*reinterpret_cast<const float2 *>(cur + i + 2 * u),
                                             *reinterpret_cast<const float2 *>(cur + i + 3 * u));
                        }
                        const float2 v2 = add_f2(b[q], p1);
                        b[q] = two ? add_f2(v2, p23) : v2;
                        score(q, v2, 2 * s - 1, b[q], two ? 2 * s : -1);
                        if (more) *reinterpret_cast<float2 *>(nxt + i) = b[q];
                    }
                }
                if (more) bar.sync();
            }
        };
        if (interior)
            widths(std::true_type{});
        else
            widths(std::false_type{});
        bool any = false;
        if (active) {
#pragma unroll
            for (int q = 0; q < PAIRS; ++q)
                if (2 * tid + 2 * THREADS * q < NBEST) any |= best[q].x >= thr || best[q].y >= thr;
        }
        // most tiles hold no sample over the threshold: skip the neighbourhood test there
        if (!bar.any(any)) continue;
        if (active) {
#pragma unroll
            for (int q = 0; q < PAIRS; ++q) {
                const int i = 2 * tid + 2 * THREADS * q;
                if (i < NBEST) *reinterpret_cast<float2 *>(best_s + i) = best[q];
            }
        }
        bar.sync();
        if (active) {
            for (int q = tid; q < kBoxTile; q += THREADS) {
                const long long t = t0 + q;
                if (t >= n) break;
                const int i = q + HL;
                const float bv = best_s[i];
                if (!(bv >= thr)) continue;
                float snr;
                int width;
                box_best_at<T, NW>(r, t, n, mu_f, inv_w, &snr, &width);
                const int h = max(width / 2, 1);
                bool keep = true;
                for (int u = 1; u <= h && keep; ++u)
                    if (t - u >= 0 && !(best_s[i - u] < bv)) keep = false;
                for (int u = 1; u <= h && keep; ++u)
                    if (t + u <= n - 1 && !(best_s[i + u] <= bv)) keep = false;
                if (!keep) continue;
                const unsigned long long at = atomicAdd(count, 1ull);
                if ((long long)at < cap) cands[at] = DevCand{d, (int32_t)t, width, snr};
            }
        }
        // (the next tile writes best_s only after its own barriers)
    }
}

}  // namespace mdsm
