// box.cuh -- the boxcar single-pulse search's tile loop as a device function, shared by the
// standalone search kernel (detect.cu) and the fused batched launch (dedisp.cu).
//
// Widths 1, 2, 4, ..., 2^(NW-1); per DM row the mean and sigma come from the caller.  A run of
// consecutive tiles of one row is searched by a group of THREADS threads: the whole CTA
// (BoxBarCta) or one of several groups of a CTA, each with its own named barrier and shared
// memory (BoxBarGroup), so that one wide CTA runs several searches whose barriers overlap.
// The next tile's samples are copied into shared memory (one bulk copy on an mbarrier, or
// per-thread cp.async) while the current one is searched.  Arithmetic per sample and width is
// FP32, explicitly rounded, in the oracle's
// order: B_2w[i] = B_w[i] + B_w[i + w] (a pairwise tree over each boxcar), and the SNR
// (B_w - w mu) / (sigma sqrt w) with 1 / (sigma sqrt w) rounded once per width.
//
// Two paths (box_run): a fast path that only decides whether a tile reaches the threshold,
// over chains of one residue class of each step's stride per thread, keeping the largest sum
// of each width; and an exact path (box_tile_exact) for the tiles it flags: every position's
// best SNR over the widths, then the candidates, local maxima of the best SNR over
// max(w/2, 1) samples on each side, with the width that gave the best formed again for those
// few positions (box_best_at).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "internal.h"
#include "ptx.cuh"

namespace mdsm {

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

// Tile geometry of the search for NW widths (1 .. WMAX = 2^(NW-1)) by a group of THREADS
// threads, each owning K positions of a region of N = THREADS * K samples (K odd).
//
// A tile's output samples are [t0, t0 + TILE).  The fast path stages the region [t0, t0 + N),
// which holds every boxcar that starts in the tile (TILE <= N - WMAX + 1).  The exact path
// searches a tile in parts of ETILE output samples [a, a + ETILE), each from a region of
// NE = THREADS * KE samples [a - HL, a + ETILE + HL + WMAX) that also holds the neighbourhoods
// of the kept boxcars; NBEST = ETILE + 2 HL positions carry a best SNR.
template <int NW, int THREADS, int K, int KE = K>
struct BoxGeom {
    static_assert(NW >= 1 && NW <= 9, "widths 1 .. 256");
    static_assert(K % 2 == 1, "odd positions per thread (no bank conflicts in the chains)");
    static_assert(KE >= 1 && KE <= K, "the exact path's region within the fast path's");
    static_assert((THREADS & (THREADS - 1)) == 0, "power-of-two thread count");
    static constexpr int WMAX = 1 << (NW - 1);
    static constexpr int HL = WMAX / 2 > 1 ? WMAX / 2 : 1;
    static constexpr int N = THREADS * K;
    static constexpr int NE = THREADS * KE;
    static constexpr int TILE = (N - WMAX + 1) & ~3;  // (a multiple of 4: aligned copies)
    static constexpr int ETILE = (NE - 2 * HL - WMAX) & ~3;
    static constexpr int NBEST = ETILE + 2 * HL;
    static_assert(ETILE >= THREADS && TILE >= ETILE, "tile");
    // The fast path's chain steps: step s reads B_u (u = 8^(s-1)) and forms up to three
    // doublings (widths 2u, 4u, 8u); ND(s) of them, LA(s) = 2^ND - 1 chain elements of lookahead.
    static constexpr int STEPS = (NW + 1) / 3;  // widths 2 .. 2^(NW-1) in steps of three
    static_assert(STEPS <= 3, "three chain steps at most");
    static constexpr int nd(int s) { return NW - 1 - 3 * (s - 1) < 3 ? NW - 1 - 3 * (s - 1) : 3; }
    static constexpr int la(int s) { return (1 << nd(s)) - 1; }
    static constexpr int UMAX = STEPS > 0 ? 1 << (3 * (STEPS - 1)) : 1;  // widest chain stride
    static_assert(UMAX <= THREADS, "a chain stride per residue class");
    // zeros past N that the chains of steps 2.. read: u LA(s) floats
    static constexpr int pad_sums()
    {
        int p = 0;
        for (int s = 2; s <= STEPS; ++s) {
            const int q = (1 << (3 * (s - 1))) * la(s);
            p = q > p ? q : p;
        }
        return p;
    }
    // the exact path: position pairs (2 tid + 2 THREADS q, +1)
    static constexpr int PAIRS = (NE + 2 * THREADS - 1) / (2 * THREADS);
    // floats of each sum buffer: the exact path's pairs plus WMAX of partner reads past them,
    // and the chains' reads past N; even (8-byte aligned pairs)
    static constexpr int BUF0 = PAIRS * 2 * THREADS + (WMAX < 2 ? 2 : WMAX);
    static constexpr int BUF1 = N + pad_sums();
    static constexpr int BUF = ((BUF0 > BUF1 ? BUF0 : BUF1) + 3) / 4 * 4;
    static constexpr int NBF = N + 8;  // staged samples, 7 zeros of step 1's reads past them
    // shared memory of box_run: the staged samples, two sum buffers, the best SNR of NBEST
    // positions (exact path), 1 / (sigma sqrt(w)) per width (16 floats), the bulk-copy
    // mbarrier (16 bytes)
    static constexpr size_t SMEM = (size_t)NBF * 4 + (size_t)BUF * 8 + (size_t)NBEST * 4 + 80;
    static_assert(NBEST % 2 == 0 && NBF % 4 == 0, "alignment");
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

// Output samples [t0, t0 + cnt) (cnt <= ETILE) exactly: the width ladder with every
// position's best SNR and the range tests of the series' ends, then the candidates; for the
// tiles the fast path flags.  The samples are read from the series (zero outside it).  B0, B1:
// BUF floats each; best_s: NBEST.  Every thread of the group calls it.
template <typename T, int NW, int THREADS, int K, class Bar>
__device__ __noinline__ void box_tile_exact(const T *__restrict__ r, long long n, long long t0,
                                            int cnt, float mu_f, float thr, const float *inv_w,
                                            int d, DevCand *__restrict__ cands,
                                            unsigned long long *__restrict__ count, long long cap,
                                            float *B0, float *B1, float *best_s, const Bar &bar,
                                            int tid, bool active)
{
    using G = BoxGeom<NW, THREADS, K>;
    constexpr int HL = G::HL, NBEST = G::NBEST, PAIRS = G::PAIRS;
    const long long r0 = t0 - HL;  // series index of B[0] and best[0]
    float2 b[PAIRS], best[PAIRS];
    if (active) {
#pragma unroll
        for (int q = 0; q < PAIRS; ++q) {
            const int i = 2 * tid + 2 * THREADS * q;
            float v[2];
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const long long t = r0 + i + e;
                v[e] = t >= 0 && t < n ? (float)__ldg(r + t) : 0.f;
            }
            b[q] = make_float2(v[0], v[1]);
            *reinterpret_cast<float2 *>(B0 + i) = b[q];
            best[q] = make_float2(-INFINITY, -INFINITY);
        }
    }
    bar.sync();
    // best SNR of pair q over width 2^l (sums v), where the boxcar lies in the series
    auto score = [&](int q, float2 v, int l) {
        const int i = 2 * tid + 2 * THREADS * q;
        if (i >= NBEST) return;  // i even and NBEST even: i + 1 < NBEST too
        const int w = 1 << l;
        const float wm = __fmul_rn((float)w, mu_f);
        const float2 sv = mul_f2(add_f2(v, make_float2(-wm, -wm)), make_float2(inv_w[l], inv_w[l]));
        const long long t = r0 + i;
        if (t >= 0 && t + w <= n) best[q].x = fmaxf(best[q].x, sv.x);
        if (t + 1 >= 0 && t + 1 + w <= n) best[q].y = fmaxf(best[q].y, sv.y);
    };
    if (active) {
#pragma unroll
        for (int q = 0; q < PAIRS; ++q) score(q, b[q], 0);
    }
    // two widths per step, as the fast path's chains: B_2u[i] = B_u[i] + B_u[i + u],
    // B_4u[i] = B_2u[i] + (B_u[i + 2u] + B_u[i + 3u])
#pragma unroll
    for (int s = 1; 2 * s - 1 < NW; ++s) {
        const int u = 1 << (2 * s - 2);
        const bool two = 2 * s < NW;
        const bool more = 2 * s + 1 < NW;
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
                score(q, v2, 2 * s - 1);
                b[q] = v2;
                if (two) {
                    b[q] = add_f2(v2, p23);
                    score(q, b[q], 2 * s);
                }
                if (more) *reinterpret_cast<float2 *>(nxt + i) = b[q];
            }
        }
        if (more) bar.sync();
    }
    bool any = false;
    if (active) {
#pragma unroll
        for (int q = 0; q < PAIRS; ++q)
            if (2 * tid + 2 * THREADS * q < NBEST) any |= best[q].x >= thr || best[q].y >= thr;
    }
    if (!bar.any(any)) return;
    if (active) {
#pragma unroll
        for (int q = 0; q < PAIRS; ++q) {
            const int i = 2 * tid + 2 * THREADS * q;
            if (i < NBEST) *reinterpret_cast<float2 *>(best_s + i) = best[q];
        }
    }
    bar.sync();
    if (active) {
        for (int q = tid; q < cnt; q += THREADS) {
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
}

// Asynchronous copy of the fast path's region [t0, t0 + N) of tile `tile` into NB by the group:
// 16-byte copies where the region lies inside the series and starts 16-byte aligned, else
// 4-byte copies with zeros past the series.  Each thread waits for its own copies
// (cp_async_wait_all); a group barrier then makes all of them visible.
template <typename T, int NW, int THREADS, int K>
__device__ __forceinline__ void box_stage(uint32_t *NB, const T *__restrict__ r, long long n,
                                          long long tile, int tid)
{
    using G = BoxGeom<NW, THREADS, K>;
    static_assert(sizeof(T) == 4, "4-byte samples");
    const long long r0 = tile * G::TILE;
    if (r0 + G::N <= n && ((uintptr_t)(r + r0) & 15) == 0) {
        const T *base = r + r0;
        for (int q = tid; q < G::N / 4; q += THREADS) cp_async16(NB + 4 * q, base + 4 * q);
    } else {
        for (int i = tid; i < G::N; i += THREADS) {
            const long long t = r0 + i;
            const bool in = t < n;
            cp_async4(NB + i, in ? r + t : r, in ? 4u : 0u);
        }
    }
    cp_async_commit();
}

// m = max(m, c[0], .., c[K - 1]) in three-input maxima.
template <int K>
__device__ __forceinline__ void box_fold(float &m, const float *c)
{
#pragma unroll
    for (int j = 0; j + 1 < K; j += 2) m = fmax3(m, c[j], c[j + 1]);
    if (K & 1) m = fmaxf(m, c[K - 1]);
}

// c[j] = c[j] + c[j + H] for j < CNT, in place in ascending j (the partners are not yet
// updated); for H >= 2 the operand pairs (j, j + 1) and (j + H, j + H + 1) are register pairs,
// added in FP32x2.
template <int CNT, int H>
__device__ __forceinline__ void box_double(float *c)
{
    if constexpr (H == 1) {
#pragma unroll
        for (int j = 0; j < CNT; ++j) c[j] = __fadd_rn(c[j], c[j + 1]);
    } else {
#pragma unroll
        for (int j = 0; j + 1 < CNT; j += 2) {
            const float2 v = add_f2(make_float2(c[j], c[j + 1]), make_float2(c[j + H], c[j + H + 1]));
            c[j] = v.x;
            c[j + 1] = v.y;
        }
        if constexpr ((CNT & 1) != 0) c[CNT - 1] = __fadd_rn(c[CNT - 1], c[CNT - 1 + H]);
    }
}

// Step S of the fast path's chains for one thread (see box_run): B_u (u = 8^(S-1)) of its chain
// and LA(S) further chain elements from the staged samples (S = 1) or the previous step's
// buffer, ND(S) doublings in registers with the largest sum of each width folded into M, and
// the last doubling stored for the next step.
template <typename T, int NW, int THREADS, int K, int S>
__device__ __forceinline__ void box_chain_step(const uint32_t *NB, float *A, float *Bf, float *M,
                                               int tid)
{
    using G = BoxGeom<NW, THREADS, K>;
    constexpr int u = 1 << (3 * (S - 1)), nd = G::nd(S), la = G::la(S);
    const int p0 = (tid & (u - 1)) + u * K * (tid / u);  // chain element 0
    float c[K + la];
    const float *src = (S & 1) ? Bf : A;
#pragma unroll
    for (int j = 0; j < K + la; ++j) c[j] = S == 1 ? box_value<T>(NB[p0 + j]) : src[p0 + u * j];
    if constexpr (S == 1) box_fold<K>(M[0], c);
    // c[j] = B_{2^e u}[j] for j < K + la + 1 - 2^e after doubling e
    if constexpr (nd >= 1) {
        box_double<K + la - 1, 1>(c);
        box_fold<K>(M[3 * (S - 1) + 1], c);
    }
    if constexpr (nd >= 2) {
        box_double<K + la - 3, 2>(c);
        box_fold<K>(M[3 * (S - 1) + 2], c);
    }
    if constexpr (nd >= 3) {
        box_double<K + la - 7, 4>(c);
        box_fold<K>(M[3 * (S - 1) + 3], c);
    }
    if constexpr (S < G::STEPS) {  // a further step reads B_8u
        float *nxt = (S & 1) ? A : Bf;
#pragma unroll
        for (int j = 0; j < K; ++j) nxt[p0 + u * j] = c[j];
    }
}

// Tiles [tile_lo, tile_hi) of row r (n samples, DM index d) with the row's mean and sigma
// (sigma > 0), searched by the calling group: `active` threads with group index tid in
// [0, THREADS) (every thread of the group's barrier calls it); sm holds
// BoxGeom<NW, THREADS, K, KE>::SMEM bytes of the group's own.  Candidates (d, sample, width, snr)
// go to cands[atomicAdd(count)] below cap.  When it returns, no copy is in flight and no
// mbarrier lives in sm; the caller synchronises the group before sm is written again.
//
// Staging (kBulk): a tile whose region lies inside the series and starts 16-byte aligned
// arrives by one bulk copy (cp.async.bulk, issued by the group's thread 0 on an mbarrier in
// sm), and every thread waits on the mbarrier's phase, bounded, instead of at a group barrier.
// A wait that runs out sets kBoxCountLate in *count (the search's results are then void); the
// group learns of it at the tile's closing vote and leaves the run together, after a bounded
// wait for a copy still in flight.  Other tiles, and every tile without kBulk, arrive by
// per-thread cp.async.
//
// Fast path (every tile): only whether a boxcar that starts in the tile reaches the threshold
// at some width is needed, so no position keeps a best SNR.  Step s (chain stride u = 8^(s-1))
// gives each thread the residue class tid mod u, block b = tid / u: the K positions
// p_j = (tid mod u) + u (K b + j) and, from the previous step's buffer (the staged samples for
// s = 1), B_u at p_j for j < K + LA(s).  In registers it forms up to three doublings over the
// chain, B_2u[j] = B_u[j] + B_u[j + 1], B_4u[j] = B_2u[j] + B_2u[j + 2] and
// B_8u[j] = B_4u[j] + B_4u[j + 4] (the exact path's operands and order), keeps the largest sum
// of each width over its K positions and stores the last for the next step.  Reads and stores
// are conflict-free (K odd).  The SNR (v - w mu) / (sigma sqrt w), rounded as the exact path
// rounds it, does not decrease with v, so the largest SNR of a width is the SNR of its largest
// sum.  Positions whose boxcars reach past the region (or past the series, staged as zeros)
// take part too: their sums hold real samples and zeros, and a tile they flag is only searched
// exactly, where the range tests apply.  A flagged tile is searched exactly in parts of ETILE
// output samples.
template <typename T, int NW, int THREADS, int K, int KE = K, bool kBulk = false,
          class Bar = BoxBarCta>
__device__ __forceinline__ void box_run(const T *__restrict__ r, long long n, long long tile_lo,
                                        long long tile_hi, double mu, double sig, double threshold,
                                        int d, DevCand *__restrict__ cands,
                                        unsigned long long *__restrict__ count, long long cap,
                                        unsigned char *sm, const Bar &bar, int tid_in, bool active)
{
    using G = BoxGeom<NW, THREADS, K, KE>;
    constexpr int N = G::N;
    uint32_t *NB = reinterpret_cast<uint32_t *>(sm);  // staged samples of the current tile
    float *A = reinterpret_cast<float *>(NB + G::NBF);
    float *Bf = A + G::BUF;
    float *best_s = Bf + G::BUF;
    float *inv_w = best_s + G::NBEST;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(inv_w + 16);
    const int tid = tid_in & (THREADS - 1);
    if (kBulk && active && tid == 0) {
        mbar_init(mbar, 1);
        fence_mbar_init();
    }
    const float mu_f = __double2float_rn(mu);
    const float thr = __double2float_rn(threshold);
    // 1 / (sigma sqrt(w)) in FP64, rounded to FP32, once per width (FP64 is a slow pipe here)
    if (active && tid < NW)
        inv_w[tid] = __double2float_rn(__ddiv_rn(1.0, __dmul_rn(sig, __dsqrt_rn((double)(1 << tid)))));
    // zeros past the region: the chains read up to 7 positions past NB and LA u past N
    auto zero_pads = [&]() {
        if (!active) return;
        for (int i = N + tid; i < G::BUF; i += THREADS) A[i] = Bf[i] = 0.f;
        if (tid < G::NBF - N) NB[N + tid] = 0u;
    };
    zero_pads();
    // SNR at width 2^l of sums v
    auto snr = [&](float v, int l) {
        const float wm = __fmul_rn((float)(1 << l), mu_f);
        return __fmul_rn(__fadd_rn(v, -wm), inv_w[l]);
    };
    // whether tile `tile` arrives by one bulk copy (uniform across the group)
    auto bulk = [&](long long tile) {
        const long long r0 = tile * G::TILE;
        return kBulk && r0 + N <= n && ((uintptr_t)(r + r0) & 15) == 0;
    };
    uint32_t nwait = 0;  // bulk-copy phases waited for (the next copy's phase parity: nwait & 1)
    int tail = -1;       // thread 0: the parity of a copy it issued and has not seen complete
    bool late = false;   // a bulk-copy wait of this thread ran out
    auto stage = [&](long long tile) {
        if (!active) return;
        if (bulk(tile)) {
            if (tid == 0 && !late) {  // (never an arrival on a phase that may be incomplete)
                fence_proxy_async_smem();  // (after the group's reads of NB, at a barrier)
                mbar_arrive_expect_tx(mbar, (uint32_t)N * 4u);
                bulk_g2s(NB, r + tile * G::TILE, (uint32_t)N * 4u, mbar);
                tail = (int)(nwait & 1u);
            }
        } else {
            box_stage<T, NW, THREADS, K>(NB, r, n, tile, tid);
        }
    };
    if (kBulk) bar.sync();  // the mbarrier initialised (before any thread waits on it)
    if (tile_lo < tile_hi) stage(tile_lo);  // (no copy is left in flight for an empty run)
    for (long long tile = tile_lo; tile < tile_hi; ++tile) {
        const long long t0 = tile * G::TILE;
        if (bulk(tile)) {
            // the bulk copy's bytes are visible to each thread that sees the phase complete;
            // inv_w is visible since the barrier before the loop; every thread is past the
            // previous tile's reads of the sum buffers (its last barrier)
            if (active) {
                if (mbar_wait_bounded(mbar, nwait & 1u, nullptr, 0)) {
                    if (tid == 0) tail = -1;
                } else {
                    late = true;
                    atomicOr(count, kBoxCountLate);
                }
            }
            ++nwait;
        } else {
            if (active) cp_async_wait_all();
            bar.sync();  // the tile's samples (every thread's copies), inv_w and the pads visible
        }
        float M[NW];
#pragma unroll
        for (int l = 0; l < NW; ++l) M[l] = -INFINITY;
        bool staged = false;  // the next tile's copies issued
        auto stage_next = [&]() {
            if (tile + 1 < tile_hi) stage(tile + 1);
            staged = true;
        };
        if (G::STEPS == 0 && active) {  // width 1 alone
            float c[K];
#pragma unroll
            for (int j = 0; j < K; ++j) c[j] = box_value<T>(NB[K * tid + j]);
            box_fold<K>(M[0], c);
        }
        if constexpr (G::STEPS >= 1) {
            if (active) box_chain_step<T, NW, THREADS, K, 1>(NB, A, Bf, M, tid);
            if constexpr (G::STEPS >= 2) {
                bar.sync();
                stage_next();  // the samples are read: copies overlap the search
                if (active) box_chain_step<T, NW, THREADS, K, 2>(NB, A, Bf, M, tid);
                if constexpr (G::STEPS >= 3) {
                    bar.sync();
                    if (active) box_chain_step<T, NW, THREADS, K, 3>(NB, A, Bf, M, tid);
                }
            }
        }
        bool hit = false;
        if (active) {
#pragma unroll
            for (int l = 0; l < NW; ++l) hit |= snr(M[l], l) >= thr;
        }
        const bool flagged = bar.any(hit || late);
        if (kBulk && flagged && bar.any(late)) break;  // a wait ran out: the group stops together
        if (!staged) stage_next();
        if (flagged) {
            // (every thread is past the fast path's reads of the sum buffers)
            for (int a = 0; a < G::TILE && t0 + a < n; a += G::ETILE) {
                if (a > 0) bar.sync();  // the previous part's candidate reads done
                box_tile_exact<T, NW, THREADS, KE>(r, n, t0 + a, min(G::ETILE, G::TILE - a),
                                                  mu_f, thr, inv_w, d, cands, count, cap, A,
                                                  Bf, best_s, bar, tid, active);
            }
            bar.sync();
            zero_pads();  // (visible to the chains' reads past the next tile's first barrier)
        }
    }
    if (active) cp_async_wait_all();
    if (kBulk && active && tid == 0) {
        // a copy still in flight (the group stopped after a wait ran out): one more bounded wait
        if (tail >= 0) mbar_wait_bounded(mbar, (uint32_t)tail, nullptr, 0);
        mbar_inval(mbar);  // (every thread's waits are behind the last group barrier)
    }
}

}  // namespace mdsm
