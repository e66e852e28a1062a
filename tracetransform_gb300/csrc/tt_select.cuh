// tt_select.cuh -- weighted selection used by T6 and T7.
//
// TFunctional6/7 (c++/src/functionals.cpp:226-276) sort a key sequence,
// accumulate sqrt-weights in sorted order and return the key at the first
// index where twice the cumulative weight reaches the total.  That key is
// the smallest key k with 2 * W(<= k) >= W, so no sort is needed:
//
//   1. weights become u32 fixed point (2^-30 of a power-of-two bound on the
//      total), summed exactly and deterministically by integer atomics;
//   2. a 256-bin histogram linear in the key over [klo, khi] locates the bin
//      holding the crossing (bins are monotone in the key);
//   3. the keys of that bin are compacted into a 64-entry list, sorted by a
//      warp bitonic network and scanned exactly; if the bin holds more than
//      64 keys the interval shrinks to that bin's key range and step 2
//      repeats (a bin whose keys are all equal is the answer).
//
// One warp per line.  Elements are the line's stored rows [b, e) at
// x[row - jlo]; every other row is a zero sample (key 0, weight 0), which
// cannot move the crossing unless all weights are zero, in which case the
// reference returns its smallest key, 0.
#pragma once

#include "tt_common.cuh"

namespace tt {

constexpr int kSelBins = 256;
constexpr int kSelList = 64;

struct SelScratch {
    unsigned hist[kSelBins];
    unsigned key[kSelList];
    unsigned w[kSelList];
};

// Smallest bin d with 2 * (below + sum_{d' <= d} h[d']) >= total; adds the
// weight of the bins before d to *below.
__device__ __forceinline__ int sel_pick_bin(const unsigned *h, unsigned long long *below,
                                            unsigned long long total, int lane) {
    constexpr int per = kSelBins / 32;
    unsigned run = 0;
#pragma unroll
    for (int k = 0; k < per; k++)
        run += h[lane * per + k];
    unsigned long long inc = run;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned long long t = __shfl_up_sync(TT_FULL_MASK, inc, d);
        if (lane >= d)
            inc += t;
    }
    unsigned long long cum = *below + inc - run;
    int kfirst = per;
    unsigned long long before = cum, last_before = cum;
#pragma unroll
    for (int k = 0; k < per; k++) {
        const unsigned hk = h[lane * per + k];
        if (k == per - 1)
            last_before = cum;
        if (kfirst == per && 2ull * (cum + hk) >= total) {
            kfirst = k;
            before = cum;
        }
        cum += hk;
    }
    const unsigned ball = __ballot_sync(TT_FULL_MASK, kfirst < per);
    const int ln = ball ? __ffs(ball) - 1 : 31;
    const int kk = __shfl_sync(TT_FULL_MASK, ball ? kfirst : per - 1, ln);
    *below = __shfl_sync(TT_FULL_MASK, ball ? before : last_before, ln);
    return ln * per + kk;
}

// Bitonic sort of 64 (key, weight) pairs held two per lane (element i in
// lane i % 32, register i / 32), ascending by key.
__device__ __forceinline__ void sel_sort64(unsigned &k0, unsigned &w0, unsigned &k1,
                                           unsigned &w1, int lane) {
#pragma unroll
    for (int k = 2; k <= 64; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            if (j == 32) {
                // partners i and i + 32 sit in the same lane (k == 64: ascending)
                if (k0 > k1) {
                    unsigned t = k0; k0 = k1; k1 = t;
                    t = w0; w0 = w1; w1 = t;
                }
            } else {
                const unsigned ok0 = __shfl_xor_sync(TT_FULL_MASK, k0, j);
                const unsigned ow0 = __shfl_xor_sync(TT_FULL_MASK, w0, j);
                const unsigned ok1 = __shfl_xor_sync(TT_FULL_MASK, k1, j);
                const unsigned ow1 = __shfl_xor_sync(TT_FULL_MASK, w1, j);
                const bool lower = (lane & j) == 0;
                const bool up0 = (lane & k) == 0, up1 = ((lane + 32) & k) == 0;
                // the lower element of an ascending pair keeps the smaller key
                const bool take0 = lower == up0 ? (ok0 < k0) : (ok0 > k0);
                const bool take1 = lower == up1 ? (ok1 < k1) : (ok1 > k1);
                if (take0) { k0 = ok0; w0 = ow0; }
                if (take1) { k1 = ok1; w1 = ow1; }
            }
        }
    }
}

// Exact answer from a compacted list of at most 64 (key, weight) entries.
__device__ __forceinline__ float sel_finish(const SelScratch *sc, int count,
                                            unsigned long long below,
                                            unsigned long long total, float fallback,
                                            int lane) {
    unsigned k0 = lane < count ? sc->key[lane] : 0xffffffffu;
    unsigned w0 = lane < count ? sc->w[lane] : 0u;
    unsigned k1 = lane + 32 < count ? sc->key[lane + 32] : 0xffffffffu;
    unsigned w1 = lane + 32 < count ? sc->w[lane + 32] : 0u;
    sel_sort64(k0, w0, k1, w1, lane);
    unsigned long long c0 = w0, c1 = w1;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned long long t0 = __shfl_up_sync(TT_FULL_MASK, c0, d);
        const unsigned long long t1 = __shfl_up_sync(TT_FULL_MASK, c1, d);
        if (lane >= d) {
            c0 += t0;
            c1 += t1;
        }
    }
    const unsigned long long half0 = __shfl_sync(TT_FULL_MASK, c0, 31);
    c0 += below;
    c1 += below + half0;
    const unsigned b0 = __ballot_sync(TT_FULL_MASK, lane < count && 2ull * c0 >= total);
    const unsigned b1 = __ballot_sync(TT_FULL_MASK, lane + 32 < count && 2ull * c1 >= total);
    if (b0)
        return __uint_as_float(__shfl_sync(TT_FULL_MASK, k0, __ffs(b0) - 1));
    if (b1)
        return __uint_as_float(__shfl_sync(TT_FULL_MASK, k1, __ffs(b1) - 1));
    return fallback; // rounding guard: the bin's largest key
}

// Append (key, weight) of the lanes with `in` set to the list.
__device__ __forceinline__ void sel_append(SelScratch *sc, int *count, bool in, float k,
                                           unsigned wq, int lane) {
    const unsigned m = __ballot_sync(TT_FULL_MASK, in);
    if (in) {
        const int pos = *count + __popc(m & ((1u << lane) - 1u));
        if (pos < kSelList) {
            sc->key[pos] = __float_as_uint(k);
            sc->w[pos] = wq;
        }
    }
    *count += __popc(m);
}

// Histogram bin of key k in [klo, klo + 256 / bs]: monotone in k, and always a
// valid bin: keys below klo (negative samples of an image with negative
// pixels) go to bin 0 and NaN keys convert to 0, so no input can index
// outside the histogram.
__device__ __forceinline__ int sel_bin(float k, float klo, float bs) {
    return min(kSelBins - 1, max(0, (int)((k - klo) * bs)));
}

// Weighted selection over a list of keys stored in shared memory whose
// weights are sqrt(key) (T7: the keys are the samples themselves).  The list
// is refined in place: each round histograms [klo, khi], keeps the crossing
// bin's keys (a strided sweep, so every write lands on an already-read slot)
// until at most 64 remain or they are all equal.
inline __device__ float sel_list_sqrt(float *keys, int count, float klo, float khi, float qs,
                               unsigned long long below, unsigned long long total,
                               SelScratch *sc, int lane) {
    for (int level = 0; level < 16 && count > kSelList; level++) {
        if (!(khi > klo))
            return klo;
        const float bs = (float)kSelBins / (khi - klo);
        for (int i = lane; i < kSelBins; i += 32)
            sc->hist[i] = 0u;
        __syncwarp();
        for (int i = lane; i < count; i += 32) {
            const float k = keys[i];
            atomicAdd(sc->hist + sel_bin(k, klo, bs), __float2uint_rn(sqrt_nn(k) * qs));
        }
        __syncwarp();
        const int d = sel_pick_bin(sc->hist, &below, total, lane);
        __syncwarp();
        int nc = 0;
        float mn = __int_as_float(0x7f800000), mx = 0.f;
        for (int i0 = 0; i0 < count; i0 += 32) {
            const int i = i0 + lane;
            const float k = i < count ? keys[i] : 0.f;
            const bool in = i < count && sel_bin(k, klo, bs) == d;
            const unsigned m = __ballot_sync(TT_FULL_MASK, in);
            __syncwarp();
            if (in) {
                keys[nc + __popc(m & ((1u << lane) - 1u))] = k;
                mn = fminf(mn, k);
                mx = fmaxf(mx, k);
            }
            nc += __popc(m);
            __syncwarp();
        }
        count = nc;
        klo = __int_as_float(warp_min(__float_as_int(mn)));
        khi = __int_as_float(warp_max(__float_as_int(mx)));
    }
    if (count > kSelList)
        return klo;
    for (int i = lane; i < count; i += 32) {
        sc->key[i] = __float_as_uint(keys[i]);
        sc->w[i] = __float2uint_rn(sqrt_nn(keys[i]) * qs);
    }
    __syncwarp();
    return sel_finish(sc, count, below, total, khi, lane);
}

// Fixed-point weight of a sample v: sqrt(v) (T6, T7) or v itself (P2).
struct SqrtWeight {
    float qs;
    __device__ __forceinline__ unsigned operator()(float v) const {
        return __float2uint_rn(sqrt_nn(v) * qs);
    }
};
struct LinearWeight {
    float qs;
    __device__ __forceinline__ unsigned operator()(float v) const {
        return __float2uint_rn(v * qs);
    }
};

// Interval refinement for a crossing bin that held more than 64 keys:
// repeat histogram + compaction over [klo, khi] (the bin's key range).
template <class KeyFn, class WFn = SqrtWeight>
__device__ float sel_refine(const float *x, int jlo, int j0, int j1, int per, KeyFn keyfn,
                            float qs, float klo, float khi, unsigned long long below,
                            unsigned long long total, SelScratch *sc, int lane,
                            WFn wfn = WFn{0.f}) {
    if (wfn.qs == 0.f)
        wfn.qs = qs;
    for (int level = 0; level < 8; level++) {
        if (!(khi > klo))
            return klo;
        const float bs = (float)kSelBins / (khi - klo);
        for (int i = lane; i < kSelBins; i += 32)
            sc->hist[i] = 0u;
        __syncwarp();
        for (int i = 0; i < per; i++) { // warp-uniform trip count
            const int j = j0 + i;
            const float v = j < j1 ? x[j - jlo] : 0.f;
            const float k = keyfn(j, v);
            if (j < j1 && k >= klo && k <= khi)
                atomicAdd(sc->hist + sel_bin(k, klo, bs), wfn(v));
        }
        __syncwarp();
        const int d = sel_pick_bin(sc->hist, &below, total, lane);
        __syncwarp();
        int count = 0;
        float bmin = __int_as_float(0x7f800000), bmax = 0.f;
        for (int i = 0; i < per; i++) {
            const int j = j0 + i;
            const float v = j < j1 ? x[j - jlo] : 0.f;
            const float k = keyfn(j, v);
            const bool in = j < j1 && k >= klo && k <= khi && sel_bin(k, klo, bs) == d;
            const unsigned wq = in ? wfn(v) : 0u;
            bmin = in ? fminf(bmin, k) : bmin;
            bmax = in ? fmaxf(bmax, k) : bmax;
            sel_append(sc, &count, in, k, wq, lane);
        }
        bmin = __int_as_float(warp_min(__float_as_int(bmin)));
        bmax = __int_as_float(warp_max(__float_as_int(bmax)));
        __syncwarp();
        if (count <= kSelList)
            return sel_finish(sc, count, below, total, bmax, lane);
        klo = bmin;
        khi = bmax;
        __syncwarp();
    }
    return klo;
}

// T6 and T7 of one line (c++/src/functionals.cpp:226-276).  T6: keys
// r1 * x[m2 + r1], r1 in [0, N - m2); T7: keys x[m1 ..]; both weighted by
// sqrt(x).  One histogram pass serves both (a chunked sweep: far-apart
// elements in flight, so fewer atomic collisions); T6 then compacts its bin
// into a 64-entry list, and T7 -- last, because it overwrites the line --
// compacts its bin in place and refines on that list.  xmax and qtot (the
// line's largest sample and sum of square roots) bound every key and weight
// total, so no separate range pass is needed.
inline __device__ void select_t67(float *x, int jlo, int jhi, int m1, int m2, bool want6,
                           bool want7, float xmax, float qtot, SelScratch *s6, SelScratch *s7,
                           int lane, float *r6, float *r7) {
    *r6 = 0.f;
    *r7 = 0.f;
    const int b7 = max(m1, jlo), b6 = max(m2, jlo);
    const int b = min(want7 ? b7 : jhi, want6 ? b6 : jhi);
    const int cnt = jhi - b;
    if (cnt <= 0 || !(xmax > 0.f) || !(qtot > 0.f))
        return;
    const int per = ((cnt + 31) >> 5) | 1; // odd: conflict-free chunks
    const int j0 = min(b + lane * per, jhi), j1 = min(j0 + per, jhi);
    // u32 fixed-point weights: q = 2^(30 - E), every weight total < 2^E
    const float qb = qtot * 1.001f;
    const int E = ((__float_as_int(qb) >> 23) & 0xff) - 126;
    const float qs = __int_as_float((127 + 30 - E) << 23);
    const float k6max = __fmul_rn((float)max(jhi - 1 - m2, 0), xmax);
    want6 = want6 && k6max > 0.f; // otherwise every T6 key is 0
    const float bs7 = (float)kSelBins / xmax, bs6 = want6 ? (float)kSelBins / k6max : 0.f;
    auto key6 = [b6, m2](int j, float v) { return j >= b6 ? __fmul_rn((float)(j - m2), v) : -1.f; };

    for (int i = lane; i < kSelBins; i += 32) {
        s6->hist[i] = 0u;
        s7->hist[i] = 0u;
    }
    __syncwarp();
    unsigned l6 = 0, l7 = 0, l7max = 0;
    // a warp-uniform trip count (per), lanes past their chunk predicated off
    for (int i0 = 0; i0 < per; i0 += 4) {
        float vb[4]; // four loads in flight before the atomics
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int j = j0 + i0 + u;
            vb[u] = j < j1 ? x[j - jlo] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int j = j0 + i0 + u;
            const float v = vb[u];
            const unsigned wq = __float2uint_rn(sqrt_nn(v) * qs);
            const bool in7 = want7 && j >= b7 && j < j1, in6 = want6 && j >= b6 && j < j1;
            l7 += in7 ? wq : 0u;
            l7max += in7 && v == xmax ? wq : 0u;
            l6 += in6 ? wq : 0u;
            if (in7)
                atomicAdd(s7->hist + sel_bin(v, 0.f, bs7), wq);
            if (in6)
                atomicAdd(s6->hist + sel_bin(key6(j, v), 0.f, bs6), wq);
        }
    }
    const unsigned long long W7 = __reduce_add_sync(TT_FULL_MASK, l7);
    const unsigned long long W6 = __reduce_add_sync(TT_FULL_MASK, l6);
    // Saturated lines (samples clipped at the image's maximum) put the
    // crossing on the largest key: when the keys below the maximum weigh less
    // than half the total, 2 W(< xmax) < W, the answer is xmax -- exact in
    // the fixed-point weights, no compaction or refinement needed.
    const unsigned long long W7max = __reduce_add_sync(TT_FULL_MASK, l7max);
    if (want7 && W7max > 0 && 2ull * (W7 - W7max) < W7) {
        *r7 = xmax;
        want7 = false;
    }
    __syncwarp();

    if (want6) {
        unsigned long long below = 0;
        const int d = sel_pick_bin(s6->hist, &below, W6, lane);
        __syncwarp();
        int c = 0;
        float mn = __int_as_float(0x7f800000), mx = 0.f;
        for (int i = 0; i < per; i++) {
            const int j = j0 + i;
            const float v = j < j1 ? x[j - jlo] : 0.f;
            const float k = key6(j, v);
            const bool in = j < j1 && j >= b6 && sel_bin(k, 0.f, bs6) == d;
            const unsigned wq = in ? __float2uint_rn(sqrt_nn(v) * qs) : 0u;
            mn = in ? fminf(mn, k) : mn;
            mx = in ? fmaxf(mx, k) : mx;
            sel_append(s6, &c, in, k, wq, lane);
        }
        mn = __int_as_float(warp_min(__float_as_int(mn)));
        mx = __int_as_float(warp_max(__float_as_int(mx)));
        __syncwarp();
        if (c <= kSelList)
            *r6 = sel_finish(s6, c, below, W6, mx, lane);
        else
            *r6 = sel_refine(x, jlo, j0, j1, per, key6, qs, mn, mx, below, W6, s6, lane);
    }

    if (want7) {
        unsigned long long below = 0;
        const int d = sel_pick_bin(s7->hist, &below, W7, lane);
        __syncwarp();
        // in-place compaction: the write index never passes the read index
        int c = 0;
        float mn = __int_as_float(0x7f800000), mx = 0.f;
        for (int js = b7; js < jhi; js += 32) {
            const int j = js + lane;
            const float v = j < jhi ? x[j - jlo] : 0.f;
            const bool in = j < jhi && sel_bin(v, 0.f, bs7) == d;
            const unsigned m = __ballot_sync(TT_FULL_MASK, in);
            __syncwarp();
            if (in) {
                x[c + __popc(m & ((1u << lane) - 1u))] = v;
                mn = fminf(mn, v);
                mx = fmaxf(mx, v);
            }
            c += __popc(m);
            __syncwarp();
        }
        mn = __int_as_float(warp_min(__float_as_int(mn)));
        mx = __int_as_float(warp_max(__float_as_int(mx)));
        *r7 = sel_list_sqrt(x, c, mn, mx, qs, below, W7, s7, lane);
    }
}

// PFunctional2 of one non-negative column (c++/src/functionals.cpp:303-311):
// the column sorted, weighted by itself, its weighted median -- the smallest
// value v with 2 * sum(x <= v) >= sum(x), found without sorting.  x: the
// column in shared memory, n values, xmax their maximum, xsum their sum (a
// bound for the fixed-point scale).  One warp.
inline __device__ float select_p2(const float *x, int n, float xmax, float xsum, SelScratch *sc,
                           int lane) {
    if (n <= 0)
        return 0.f;
    if (!(xmax > 0.f) || !(xsum > 0.f))
        return 0.f; // all zero: the first sorted value
    const int per = ((n + 31) >> 5) | 1;
    const int j0 = min(lane * per, n), j1 = min(j0 + per, n);
    const float qb = xsum * 1.001f;
    const int E = ((__float_as_int(qb) >> 23) & 0xff) - 126;
    const float qs = __int_as_float((127 + 30 - E) << 23);
    const LinearWeight wfn{qs};
    const float bs = (float)kSelBins / xmax;
    for (int i = lane; i < kSelBins; i += 32)
        sc->hist[i] = 0u;
    __syncwarp();
    unsigned lw = 0;
    for (int i0 = 0; i0 < per; i0 += 4) { // warp-uniform trip count
        float vb[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int j = j0 + i0 + u;
            vb[u] = j < j1 ? x[j] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const bool in = j0 + i0 + u < j1;
            const unsigned wq = wfn(vb[u]);
            lw += in ? wq : 0u;
            if (in)
                atomicAdd(sc->hist + sel_bin(vb[u], 0.f, bs), wq);
        }
    }
    const unsigned long long W = __reduce_add_sync(TT_FULL_MASK, lw);
    __syncwarp();
    unsigned long long below = 0;
    const int d = sel_pick_bin(sc->hist, &below, W, lane);
    __syncwarp();
    int c = 0;
    float mn = __int_as_float(0x7f800000), mx = 0.f;
    for (int i = 0; i < per; i++) {
        const int j = j0 + i;
        const float k = j < j1 ? x[j] : 0.f;
        const bool in = j < j1 && sel_bin(k, 0.f, bs) == d;
        const unsigned wq = in ? wfn(k) : 0u;
        mn = in ? fminf(mn, k) : mn;
        mx = in ? fmaxf(mx, k) : mx;
        sel_append(sc, &c, in, k, wq, lane);
    }
    mn = __int_as_float(warp_min(__float_as_int(mn)));
    mx = __int_as_float(warp_max(__float_as_int(mx)));
    __syncwarp();
    if (c <= kSelList)
        return sel_finish(sc, c, below, W, mx, lane);
    auto key = [](int, float v) { return v; };
    return sel_refine(x, 0, j0, j1, per, key, qs, mn, mx, below, W, sc, lane, wfn);
}

} // namespace tt
