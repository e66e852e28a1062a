// tt_sinogram.cu -- fused rotate + T-functional kernel.
//
// One CTA owns L adjacent columns ("trace lines") of one angle.  It samples
// the rotated image along those lines straight from the source image (no
// rotated image is written anywhere), keeps the samples of its lines in
// shared memory, and then reduces each line with one warp into every
// requested T-functional (c++/src/sinogram.cpp:67-178 with the functionals of
// c++/src/functionals.cpp:21-276).
//
// Sampling.  The source region sits in a block-linear CUDA array read through
// a texture object in border mode (texels outside the region read 0, which
// is exactly the reference's zero padding).  One 2x2 gather (tld4) fetches
// the bilinear stencil; coordinates and weights are then combined in the
// reference's order with scalar round-to-nearest operations, so every
// rotated sample is bit-identical to rotate()/interpolate()
// (c++/src/auxiliary.cpp:182-196, 223-255): the host rounds cos/sin as the
// reference does and no multiply-add is fused.  (Packed f32x2 multiply + add
// measured fused on this part, so they are not used here.)  Each thread keeps
// four gathers in flight.  Only rows whose stencil can touch the image are
// sampled; all others are exact zeros in the reference too.
//
// Reductions run in warp order rather than the reference's sequential order,
// so sums agree to rounding and a weighted median can move by one row where
// the reference's cumulative sum ties the half-total to within rounding.
// T6 and T7 need no sort: their weighted medians come from a histogram
// selection with exact fixed-point weights (tt_select.cuh).
#include <climits>
#include <map>
#include <mutex>
#include <utility>

#include "tt_common.cuh"
#include "tt_internal.h"
#include "tt_select.cuh"

namespace tt {
namespace {

// Rows [lo, hi) of a line whose samples can be non-zero: the reference's
// bounds test 0 <= q < n-1 intersected with the band where the 2x2 stencil
// overlaps the source region, widened by a row on each side.
__device__ __forceinline__ void line_support(float X, float c, float s, float o,
                                             int n, float xlo, float xhi,
                                             float ylo, float yhi, int *lo,
                                             int *hi) {
    // qx(j) = X c + o + (j - o) s ;  qy(j) = -X s + o + (j - o) c
    float jl = 0.f, jh = (float)(n - 1);
    const float bx = X * c + o, by = -X * s + o;
    if (fabsf(s) > 1e-7f) {
        float a0 = o + __fdividef(xlo - bx, s), a1 = o + __fdividef(xhi - bx, s);
        jl = fmaxf(jl, fminf(a0, a1));
        jh = fminf(jh, fmaxf(a0, a1));
    } else if (bx < xlo || bx > xhi) {
        jh = -1.f;
    }
    if (fabsf(c) > 1e-7f) {
        float a0 = o + __fdividef(ylo - by, c), a1 = o + __fdividef(yhi - by, c);
        jl = fmaxf(jl, fminf(a0, a1));
        jh = fminf(jh, fmaxf(a0, a1));
    } else if (by < ylo || by > yhi) {
        jh = -1.f;
    }
    if (jh < jl) {
        *lo = n;
        *hi = 0;
        return;
    }
    *lo = max(0, (int)floorf(jl) - 1);
    *hi = min(n, (int)ceilf(jh) + 2);
}

// First crossing -> weighted-median row, following findWeightedMedian
// (c++/src/functionals.cpp:21-30) over the full column: rows before jlo and
// from jhi on are zeros.
__device__ __forceinline__ int resolve_median(int found, float total, int jlo,
                                              int jhi, int len, int n) {
    if (jlo > 0 && 0.f >= total)
        return 0;
    if (found != INT_MAX) {
        int m = jlo + min(found, len);
        return m < n ? m : n - 1;
    }
    if (jhi < n && 2.f * total >= total)
        return jhi;
    return n - 1;
}

template <bool kSqrt>
__device__ __forceinline__ float elem(const float *x, int i) {
    return kSqrt ? sqrt_nn(x[i]) : x[i];
}

// First element i (of the chunked line) with 2 * prefix_i >= total, given the
// per-lane chunk sums: the warp jumps to the first chunk whose inclusive sum
// crosses and scans that chunk cooperatively (continuing into the next chunk
// if rounding put the crossing there).  Valid for non-negative data.
template <bool kSqrt>
__device__ int find_crossing(const float *x, int C, float inc, float exc, float total, int lane) {
    const unsigned ball = __ballot_sync(TT_FULL_MASK, 2.f * inc >= total);
    if (!ball)
        return INT_MAX;
    for (int ln = __ffs(ball) - 1; ln < 32; ln++) {
        float basev = __shfl_sync(TT_FULL_MASK, exc, ln);
        for (int t0 = 0; t0 < C; t0 += 32) {
            const int t = t0 + lane;
            const float v = t < C ? elem<kSqrt>(x, ln * C + t) : 0.f;
            const float p = warp_incl_scan(v, lane) + basev;
            const unsigned b = __ballot_sync(TT_FULL_MASK, t < C && 2.f * p >= total);
            if (b)
                return ln * C + t0 + __ffs(b) - 1;
            basev = __shfl_sync(TT_FULL_MASK, p, 31);
        }
    }
    return INT_MAX;
}

// Sequential per-lane walk (any sign): the first crossing as the reference
// defines it even when the prefix is not monotone.
__device__ int find_crossing_walk(const float *x, int C, float exc, float total, int lane) {
    float run = exc;
    int f = INT_MAX;
    for (int k = 0; k < C; k++) {
        run += x[lane * C + k];
        if (f == INT_MAX && 2.f * run >= total)
            f = lane * C + k;
    }
    return warp_min(f);
}

// One CTA's unit of work: L adjacent lines (columns col0 ..) of one angle of
// one image.
struct BlockJob {
    cudaTextureObject_t tex;
    float tu, tv;     // texel coordinate = frame coordinate + (tu, tv)
    int n, col0, angle;
    float c, s;       // cos(-theta), sin(-theta) as the host rounded them
    int roff, coff, rr, rc; // support region inside the frame
    const float2 *tab;      // T3, T4, T5 kernels of this n
    float *out;             // this image's n_t x n_angles x n sinogram stack
    int32_t *medians;       // optional, same shape
    size_t plane;           // n_angles * n
};

// The fused body: support, sampling, T-functionals of one BlockJob.  Every
// thread of the CTA (W >= L warps) calls it; it synchronises the CTA but
// never returns early.  All W warps sample; warps 0..L-1 then take one line
// each.  tf_code holds the T-functional id of output t in bits [3t, 3t + 3).
template <int L, bool kSel, bool kInterior, int W = L>
__device__ __forceinline__ void sino_block(const BlockJob &J, unsigned long long tf_code,
                                           int n_t, unsigned need, int stride, float *sm,
                                           int *s_range) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int angle = J.angle;
    const int col0 = J.col0;
    const int n = J.n;
    const float c = J.c, s = J.s;
    const float o = (float)(n - 1) * 0.5f;
    const float nm1 = (float)(n - 1);
    const int roff = J.roff, coff = J.coff;
    const int rr = max(J.rr, 0), rc = max(J.rc, 0);

    // 1. Row range shared by the CTA's lines.
    if (warp == 0) {
        int lo = n, hi = 0;
        if (lane < L && col0 + lane < n && rr > 0 && rc > 0) {
            const float X = (float)(col0 + lane) - o;
            line_support(X, c, s, o, n, (float)coff - 2.f, (float)(coff + rc) + 1.f,
                         (float)roff - 2.f, (float)(roff + rr) + 1.f, &lo, &hi);
        }
        lo = warp_min(lo);
        hi = warp_max(hi);
        if (lane == 0) {
            if (hi <= lo) {
                lo = 0;
                hi = 0;
            }
            s_range[0] = lo;
            s_range[1] = hi;
        }
    }
    __syncthreads();
    const int jlo = s_range[0], jhi = s_range[1];
    const int len = jhi - jlo;
    const int C = max((len + 31) >> 5, 1) | 1; // odd: conflict-free chunks


    // 2. Sample the lines into shared memory (zeros past len, rows < 32 C).
    {
        constexpr int RS = 32 * W / L; // row streams per line
        const int l = lane % L, r = (warp * 32 + lane) / L;
        const int col = col0 + l;
        const bool colok = col < n;
        const float X = (float)col - o;
        const float Xc = __fmul_rn(X, c), Xms = __fmul_rn(X, -s);
        const float tu = J.tu, tv = J.tv;
        float *dst = sm + l * stride;
        const int rows = 32 * C, iters = (rows + RS - 1) / RS; // this thread: r + RS i
        constexpr int U = 4;                                   // gathers in flight per thread
        for (int i0 = 0; i0 < iters; i0 += U) {
            float4 g[U];
            float xf[U], yf[U];
            bool ok[U];
#pragma unroll
            for (int u = 0; u < U; u++) {
                const int jr = r + RS * (i0 + u);
                const float Y = (float)(jlo + jr) - o;
                // (x c + y s) + o and (x (-s) + y c) + o, each operation rounded
                const float qx = __fadd_rn(__fadd_rn(Xc, __fmul_rn(Y, s)), o);
                const float qy = __fadd_rn(__fadd_rn(Xms, __fmul_rn(Y, c)), o);
                ok[u] = colok && jr < len;
                if (!kInterior) // see warp_sample: border texels answer the test
                    ok[u] = ok[u] && qx >= 0.f && qx < nm1 && qy >= 0.f && qy < nm1;
                const float xi = truncf(qx), yi = truncf(qy);
                xf[u] = __fsub_rn(qx, xi);
                yf[u] = __fsub_rn(qy, yi);
                // texel (u, v) = image (row, col); w/z/x/y = s00, s10, s01, s11
                g[u] = tex2Dgather<float4>(J.tex, yi + tu, xi + tv, 0);
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
                const float omx = __fsub_rn(1.f, xf[u]), omy = __fsub_rn(1.f, yf[u]);
                const float t0 = __fmul_rn(__fmul_rn(g[u].w, omx), omy);
                const float t1 = __fmul_rn(__fmul_rn(g[u].x, xf[u]), omy);
                const float t2 = __fmul_rn(__fmul_rn(g[u].z, omx), yf[u]);
                const float t3 = __fmul_rn(__fmul_rn(g[u].y, xf[u]), yf[u]);
                const float v = __fadd_rn(__fadd_rn(__fadd_rn(t0, t1), t2), t3);
                const int jr = r + RS * (i0 + u);
                if (jr < rows)
                    dst[jr] = ok[u] ? v : 0.f;
            }
        }
    }
    __syncthreads();

    // 3. One warp per line: T-functionals.
    const int col = col0 + warp;
    if (warp < L && col < n) {
    float *x = sm + warp * stride;
    const bool need_m1 = need & ((1u << 1) | (1u << 2) | (1u << 7));
    const bool need_m2 = need & ((1u << 3) | (1u << 4) | (1u << 5) | (1u << 6));
    const bool need_sq = need_m2 || (need & (1u << 7)); // sum of sqrt(x) wanted
    const int base = lane * C;

    float tot = 0.f, totq = 0.f, lmax = 0.f;
    bool neg = false;
#pragma unroll 4
    for (int k = 0; k < C; k++) {
        const float v = x[base + k];
        tot += v;
        neg |= v < 0.f;
        if (kSel)
            lmax = fmaxf(lmax, v);
        if (need_sq)
            totq += sqrt_nn(v);
    }
    const float inc = warp_incl_scan(tot, lane);
    const float S = __shfl_sync(TT_FULL_MASK, inc, 31);
    float exc = __shfl_up_sync(TT_FULL_MASK, inc, 1);
    float Q = 0.f, incq = 0.f, excq = 0.f;
    if (need_sq) {
        incq = warp_incl_scan(totq, lane);
        Q = __shfl_sync(TT_FULL_MASK, incq, 31);
        excq = __shfl_up_sync(TT_FULL_MASK, incq, 1);
    }
    if (lane == 0) {
        exc = 0.f;
        excq = 0.f;
    }
    const bool any_neg = __any_sync(TT_FULL_MASK, neg);

    int m1 = 0, m2 = 0;
    if (need_m1) {
        const int f = any_neg ? find_crossing_walk(x, C, exc, S, lane)
                              : find_crossing<false>(x, C, inc, exc, S, lane);
        m1 = resolve_median(f, S, jlo, jhi, len, n);
    }
    if (need_m2)
        m2 = resolve_median(find_crossing<true>(x, C, incq, excq, Q, lane), Q, jlo, jhi, len, n);

    float r1v = 0.f, r2v = 0.f;
    if (need & ((1u << 1) | (1u << 2))) {
        float t1 = 0.f, t2 = 0.f;
#pragma unroll 4
        for (int j = max(m1, jlo) + lane; j < jhi; j += 32) {
            const float v = x[j - jlo];
            const float r = (float)(j - m1);
            const float vr = v * r;
            t1 += vr;
            t2 = fmaf(vr, r, t2);
        }
        r1v = warp_sum(t1);
        r2v = warp_sum(t2);
    }

    float r345[3] = {0.f, 0.f, 0.f};
    if (need & ((1u << 3) | (1u << 4) | (1u << 5))) {
        const bool w3 = need & (1u << 3), w4 = need & (1u << 4), w5 = need & (1u << 5);
        const float2 *tab3 = J.tab, *tab4 = J.tab + n, *tab5 = J.tab + 2 * n;
        float re3 = 0.f, im3 = 0.f, re4 = 0.f, im4 = 0.f, re5 = 0.f, im5 = 0.f;
        const int lo = max(1, jlo - m2), hi = min(n - m2, jhi - m2);
#pragma unroll 4
        for (int q = lo + lane; q < hi; q += 32) {
            const float v = x[m2 + q - jlo];
            if (w3) {
                const float2 w = __ldg(tab3 + q);
                re3 = fmaf(w.x, v, re3);
                im3 = fmaf(w.y, v, im3);
            }
            if (w4) {
                const float2 w = __ldg(tab4 + q);
                re4 = fmaf(w.x, v, re4);
                im4 = fmaf(w.y, v, im4);
            }
            if (w5) {
                const float2 w = __ldg(tab5 + q);
                re5 = fmaf(w.x, v, re5);
                im5 = fmaf(w.y, v, im5);
            }
        }
        // hypot of the two float integrals (CUDA's hypotf: no FP64, whose
        // narrow pipe every lane of every line would otherwise queue on)
        if (w3)
            r345[0] = hypotf(warp_sum(re3), warp_sum(im3));
        if (w4)
            r345[1] = hypotf(warp_sum(re4), warp_sum(im4));
        if (w5)
            r345[2] = hypotf(warp_sum(re5), warp_sum(im5));
    }

    float r6v = 0.f, r7v = 0.f;
    if (kSel) {
        SelScratch *scr = reinterpret_cast<SelScratch *>(sm + L * stride) + 2 * warp;
        const float xmax = __int_as_float(warp_max(__float_as_int(lmax)));
        // T6: keys r1 * x[m2 + r1], r1 in [0, N - m2); T7: keys x[m1 ..]
        select_t67(x, jlo, jhi, m1, m2, need & (1u << 6), need & (1u << 7), xmax, Q, scr,
                   scr + 1, lane, &r6v, &r7v);
    }

    if (lane == 0) {
        const size_t plane = J.plane;
        const size_t at = (size_t)angle * n + col;
        for (int t = 0; t < n_t; t++) {
            const int f = (int)((tf_code >> (3 * t)) & 7ull);
            float v;
            int med;
            switch (f) {
            case 0: v = S; med = -1; break;
            case 1: v = r1v; med = m1; break;
            case 2: v = r2v; med = m1; break;
            case 3: v = r345[0]; med = m2; break;
            case 4: v = r345[1]; med = m2; break;
            case 5: v = r345[2]; med = m2; break;
            case 6: v = r6v; med = m2; break;
            default: v = r7v; med = m1; break;
            }
            J.out[t * plane + at] = v;
            if (J.medians)
                J.medians[t * plane + at] = med;
        }
    }
    } // col < n
}

template <int L, bool kSel, bool kInterior, int W = L>
__global__ void __launch_bounds__(32 * W, W > L ? 2 : 1)
    sino_kernel(const SinoArgs a) {
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ int s_range[2];
    __shared__ int s_region[4];
    // support region: static, or the non-zero box found on the device
    if (threadIdx.x == 0) {
        if (a.dyn_region) {
            s_region[0] = a.dyn_region[0];
            s_region[1] = a.dyn_region[1];
            s_region[2] = a.dyn_region[2];
            s_region[3] = a.dyn_region[3];
        } else {
            s_region[0] = a.row_off;
            s_region[1] = a.col_off;
            s_region[2] = a.src_rows;
            s_region[3] = a.src_cols;
        }
    }
    __syncthreads();
    BlockJob J;
    J.tex = a.tex;
    J.tu = 1.f - (float)a.tex_row_off;
    J.tv = 1.f - (float)a.tex_col_off;
    J.n = a.n;
    J.col0 = blockIdx.x * L;
    J.angle = blockIdx.y;
    const float2 cs = a.trig[blockIdx.y];
    J.c = cs.x;
    J.s = cs.y;
    J.roff = s_region[0];
    J.coff = s_region[1];
    J.rr = s_region[2];
    J.rc = s_region[3];
    J.tab = a.tab;
    J.out = a.out;
    J.medians = a.medians;
    J.plane = (size_t)a.n_angles * a.n;
    unsigned long long code = 0;
    for (int t = 0; t < a.n_t; t++)
        code |= (unsigned long long)(a.tf[t] & 7) << (3 * t);
    sino_block<L, kSel, kInterior, W>(J, code, a.n_t, a.need, a.stride,
                                      reinterpret_cast<float *>(smraw), s_range);
}

// Persistent kernel over a batch of images of different sizes and angle
// counts: each CTA claims work items (image, angle, line block) from a
// counter until all are taken; items are numbered largest image first.
template <int L, bool kSel, bool kInterior>
__global__ void __launch_bounds__(32 * L)
    sino_batch_kernel(const BatchSinoArgs b) {
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ int s_range[2];
    __shared__ int s_item;
    for (;;) {
        __syncthreads(); // the previous item is done with shared memory
        if (threadIdx.x == 0)
            s_item = (int)atomicAdd(b.counter, 1u);
        __syncthreads();
        const int item = s_item;
        if (item >= b.total_items)
            break;
        int lo = 0, hi = b.n_img - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(&b.img[mid].items_begin) <= item)
                lo = mid;
            else
                hi = mid - 1;
        }
        const BatchImage &im = b.img[lo];
        const int k = item - im.items_begin;
        BlockJob J;
        J.tex = im.tex;
        J.tu = 1.f - (float)im.row_off;
        J.tv = 1.f - (float)im.col_off;
        J.n = im.n;
        J.angle = k / im.blocks;
        J.col0 = (k - J.angle * im.blocks) * L;
        const float2 cs = b.trig[im.trig_off + J.angle];
        J.c = cs.x;
        J.s = cs.y;
        J.roff = im.row_off;
        J.coff = im.col_off;
        J.rr = im.rows;
        J.rc = im.cols;
        J.tab = b.tab + im.tab_off;
        J.out = b.sino + im.sino_off;
        J.medians = nullptr;
        J.plane = (size_t)im.n_angles * im.n;
        sino_block<L, kSel, kInterior>(J, b.tf_code, b.n_t, b.need, b.stride,
                                       reinterpret_cast<float *>(smraw), s_range);
    }
}

// ---- warp-autonomous lines (T0-T5) -------------------------------------------
//
// A warp owns LPW adjacent lines of one angle: each segment of SW = 32 / LPW
// lanes samples its line into its own shared-memory row and reduces it, with
// segment-wide (width SW) shuffles, so a warp's fixed per-line work -- scans,
// crossing searches, reductions, the output writes -- is shared by LPW lines
// when lines are short.  Warps never wait for one another (no CTA barrier);
// the lines' rows are laid out so that the sampling stores (LPW lines x SW
// consecutive rows per instruction) and the chunked reads (chunk length C odd,
// line rows SW banks apart) are free of bank conflicts.

template <int SW> __device__ __forceinline__ float seg_sum(float v) {
#pragma unroll
    for (int d = SW / 2; d > 0; d >>= 1)
        v += __shfl_xor_sync(TT_FULL_MASK, v, d);
    return v;
}

template <int SW> __device__ __forceinline__ int seg_min(int v) {
#pragma unroll
    for (int d = SW / 2; d > 0; d >>= 1)
        v = min(v, __shfl_xor_sync(TT_FULL_MASK, v, d));
    return v;
}

template <int SW> __device__ __forceinline__ float seg_incl_scan(float v, int sub) {
#pragma unroll
    for (int d = 1; d < SW; d <<= 1) {
        const float t = __shfl_up_sync(TT_FULL_MASK, v, d, SW);
        if (sub >= d)
            v += t;
    }
    return v;
}

// The ballot bits of segment s (bit i: lane i of the segment).
template <int SW> __device__ __forceinline__ unsigned seg_ballot(bool p, int s) {
    const unsigned b = __ballot_sync(TT_FULL_MASK, p);
    return SW == 32 ? b : (b >> (s * SW)) & ((1u << (SW & 31)) - 1u);
}

// find_crossing per segment; every lane runs the same (warp-uniform) loops.
template <bool kSqrt, int SW>
__device__ int seg_find_crossing(const float *x, int C, float inc, float exc, float total, int s,
                                 int sub) {
    const unsigned ball = seg_ballot<SW>(2.f * inc >= total, s);
    int ln = ball ? __ffs(ball) - 1 : SW;
    int found = INT_MAX;
    bool active = ln < SW;
    while (__any_sync(TT_FULL_MASK, active)) {
        float basev = __shfl_sync(TT_FULL_MASK, exc, s * SW + min(ln, SW - 1));
        for (int t0 = 0; t0 < C; t0 += SW) {
            const int t = t0 + sub;
            const bool in = active && t < C;
            const float v = in ? elem<kSqrt>(x, ln * C + t) : 0.f;
            const float p = seg_incl_scan<SW>(v, sub) + basev;
            const unsigned b = seg_ballot<SW>(in && 2.f * p >= total, s);
            if (active && b) {
                found = ln * C + t0 + __ffs(b) - 1;
                active = false;
            }
            basev = __shfl_sync(TT_FULL_MASK, p, s * SW + SW - 1);
        }
        if (active && ++ln >= SW)
            active = false;
    }
    return found;
}

// Both crossings of a segment's line at once: the plain values' (total
// tot1, chunk prefix sums inc1 / exc1) and their square roots' (tot2, inc2 /
// exc2); the same result as two seg_find_crossing calls, in one loop.
template <int SW>
__device__ void seg_find_crossing2(const float *x, int C, float inc1, float exc1, float tot1,
                                   float inc2, float exc2, float tot2, int s, int sub, int &f1,
                                   int &f2) {
    const unsigned b1 = seg_ballot<SW>(2.f * inc1 >= tot1, s);
    const unsigned b2 = seg_ballot<SW>(2.f * inc2 >= tot2, s);
    int ln1 = b1 ? __ffs(b1) - 1 : SW, ln2 = b2 ? __ffs(b2) - 1 : SW;
    f1 = INT_MAX;
    f2 = INT_MAX;
    bool a1 = ln1 < SW, a2 = ln2 < SW;
    while (__any_sync(TT_FULL_MASK, a1 || a2)) {
        float base1 = __shfl_sync(TT_FULL_MASK, exc1, s * SW + min(ln1, SW - 1));
        float base2 = __shfl_sync(TT_FULL_MASK, exc2, s * SW + min(ln2, SW - 1));
        for (int t0 = 0; t0 < C; t0 += SW) {
            const int t = t0 + sub;
            const bool in1 = a1 && t < C, in2 = a2 && t < C;
            const float v1 = in1 ? x[ln1 * C + t] : 0.f;
            const float v2 = in2 ? sqrt_nn(x[ln2 * C + t]) : 0.f;
            const float p1 = seg_incl_scan<SW>(v1, sub) + base1;
            const float p2 = seg_incl_scan<SW>(v2, sub) + base2;
            const unsigned c1 = seg_ballot<SW>(in1 && 2.f * p1 >= tot1, s);
            const unsigned c2 = seg_ballot<SW>(in2 && 2.f * p2 >= tot2, s);
            if (a1 && c1) {
                f1 = ln1 * C + t0 + __ffs(c1) - 1;
                a1 = false;
            }
            if (a2 && c2) {
                f2 = ln2 * C + t0 + __ffs(c2) - 1;
                a2 = false;
            }
            base1 = __shfl_sync(TT_FULL_MASK, p1, s * SW + SW - 1);
            base2 = __shfl_sync(TT_FULL_MASK, p2, s * SW + SW - 1);
        }
        if (a1 && ++ln1 >= SW)
            a1 = false;
        if (a2 && ++ln2 >= SW)
            a2 = false;
    }
}

// Eight sums over a segment of SW >= 8 lanes, transposed: three halving
// exchanges (each lane keeps the half of the values its offset bit selects
// and adds its partner's copy of it), then plain butterflies over the rest;
// lane sub ends with sum k = (sub / (SW / 8)) % 8 of (a0, ..., a7).
template <int SW>
__device__ __forceinline__ float seg_sum8(float a0, float a1, float a2, float a3, float a4,
                                          float a5, float a6, float a7, int sub) {
    static_assert(SW >= 8, "eight sums need eight lanes");
    constexpr int d1 = SW / 2, d2 = SW / 4, d3 = SW / 8;
    bool hi = sub & d1; // keep a4..a7
    float k0 = hi ? a4 : a0, k1 = hi ? a5 : a1, k2 = hi ? a6 : a2, k3 = hi ? a7 : a3;
    const float s0 = hi ? a0 : a4, s1 = hi ? a1 : a5, s2 = hi ? a2 : a6, s3 = hi ? a3 : a7;
    k0 += __shfl_xor_sync(TT_FULL_MASK, s0, d1);
    k1 += __shfl_xor_sync(TT_FULL_MASK, s1, d1);
    k2 += __shfl_xor_sync(TT_FULL_MASK, s2, d1);
    k3 += __shfl_xor_sync(TT_FULL_MASK, s3, d1);
    hi = sub & d2; // keep k2, k3
    float m0 = hi ? k2 : k0, m1 = hi ? k3 : k1;
    const float t0 = hi ? k0 : k2, t1 = hi ? k1 : k3;
    m0 += __shfl_xor_sync(TT_FULL_MASK, t0, d2);
    m1 += __shfl_xor_sync(TT_FULL_MASK, t1, d2);
    hi = sub & d3; // keep m1
    float r = hi ? m1 : m0;
    r += __shfl_xor_sync(TT_FULL_MASK, hi ? m0 : m1, d3);
#pragma unroll
    for (int d = d3 / 2; d > 0; d >>= 1)
        r += __shfl_xor_sync(TT_FULL_MASK, r, d);
    return r;
}

// find_crossing_walk per segment (values of any sign).
template <int SW>
__device__ int seg_walk(const float *x, int C, float exc, float total, int sub) {
    float run = exc;
    int f = INT_MAX;
    for (int k = 0; k < C; k++) {
        run += x[sub * C + k];
        if (f == INT_MAX && 2.f * run >= total)
            f = sub * C + k;
    }
    return seg_min<SW>(f);
}

// Floats per line row of the warp-autonomous layout: room for SW chunks of
// the longest chunk length, then SW more so that rows sit SW banks apart.
__host__ __device__ constexpr int warp_line_stride(int n, int lpw) {
    return 32 * ((32 / lpw * (((n + 32 / lpw - 1) / (32 / lpw)) | 1) + 31) / 32) +
           (32 / lpw) % 32;
}

// Sampling of the warp-autonomous path: lane (s, sub) takes rows sub + SW i
// of line s into x.  kBounds = false when the texture's region sits at least
// two texels inside the frame on every side (interior_source): a sample the
// reference's bounds test rejects then has a stencil of border texels only,
// whose bilinear combination is +0, the value the test would give.
template <int SW, bool kBounds>
__device__ __forceinline__ void warp_sample(const BlockJob &J, float *x, int col, bool colok,
                                            int jlo, int len, int C, int sub) {
    const int n = J.n;
    const float c = J.c, sn = J.s;
    const float o = (float)(n - 1) * 0.5f, nm1 = (float)(n - 1);
    const float X = (float)col - o;
    const float Xc = __fmul_rn(X, c), Xms = __fmul_rn(X, -sn);
    const float tu = J.tu, tv = J.tv;
    constexpr int U = 4;
    float Y0 = (float)(jlo + sub) - o; // exact: integers below 2^24
    for (int i0 = 0; i0 < C; i0 += U) {
        float4 g[U];
        float xf[U], yf[U];
        bool ok[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int jr = sub + SW * (i0 + u);
            const float Y = Y0 + (float)(SW * u);
            const float qx = __fadd_rn(__fadd_rn(Xc, __fmul_rn(Y, sn)), o);
            const float qy = __fadd_rn(__fadd_rn(Xms, __fmul_rn(Y, c)), o);
            ok[u] = colok && jr < len;
            if (kBounds)
                ok[u] = ok[u] && qx >= 0.f && qx < nm1 && qy >= 0.f && qy < nm1;
            const float xi = truncf(qx), yi = truncf(qy);
            xf[u] = __fsub_rn(qx, xi);
            yf[u] = __fsub_rn(qy, yi);
            g[u] = tex2Dgather<float4>(J.tex, yi + tu, xi + tv, 0);
        }
        Y0 += (float)(SW * U);
#pragma unroll
        for (int u = 0; u < U; u++) {
            const float omx = __fsub_rn(1.f, xf[u]), omy = __fsub_rn(1.f, yf[u]);
            const float t0 = __fmul_rn(__fmul_rn(g[u].w, omx), omy);
            const float t1 = __fmul_rn(__fmul_rn(g[u].x, xf[u]), omy);
            const float t2 = __fmul_rn(__fmul_rn(g[u].z, omx), yf[u]);
            const float t3 = __fmul_rn(__fmul_rn(g[u].y, xf[u]), yf[u]);
            const float v = __fadd_rn(__fadd_rn(__fadd_rn(t0, t1), t2), t3);
            if (i0 + u < C)
                x[sub + SW * (i0 + u)] = ok[u] ? v : 0.f;
        }
    }
}

template <int LPW, bool kInterior>
__device__ void warp_lines(const BlockJob &J, unsigned long long tf_code, int n_t,
                           unsigned need, int stride, float *xw) {
    constexpr int SW = 32 / LPW;
    const int lane = threadIdx.x & 31, s = lane / SW, sub = lane % SW;
    const int n = J.n, angle = J.angle;
    const float c = J.c, sn = J.s;
    const float o = (float)(n - 1) * 0.5f;
    const int col = J.col0 + s;
    const bool colok = col < n;
    const int rr = max(J.rr, 0), rc = max(J.rc, 0);

    // 1. rows of the warp's lines whose stencil can touch the image
    int lo = n, hi = 0;
    if (colok && rr > 0 && rc > 0)
        line_support((float)col - o, c, sn, o, n, (float)J.coff - 2.f,
                     (float)(J.coff + rc) + 1.f, (float)J.roff - 2.f,
                     (float)(J.roff + rr) + 1.f, &lo, &hi);
    lo = warp_min(lo);
    hi = warp_max(hi);
    if (hi <= lo) {
        lo = 0;
        hi = 0;
    }
    const int jlo = lo, jhi = hi, len = jhi - jlo;
    const int C = max((len + SW - 1) / SW, 1) | 1; // odd: conflict-free chunks
    float *x = xw + s * stride;

    // 2. sampling
    warp_sample<SW, !kInterior>(J, x, col, colok, jlo, len, C, sub);
    __syncwarp();

    // 3. T0-T5 of each segment's line
    const bool need_m1 = need & ((1u << 1) | (1u << 2));
    const bool need_m2 = need & ((1u << 3) | (1u << 4) | (1u << 5));
    const int base = sub * C;
    float tot = 0.f, totq = 0.f;
    bool neg = false;
    for (int k = 0; k < C; k++) {
        const float v = x[base + k];
        tot += v;
        neg |= v < 0.f;
        if (need_m2)
            totq += sqrt_nn(v);
    }
    const float inc = seg_incl_scan<SW>(tot, sub);
    const float S = __shfl_sync(TT_FULL_MASK, inc, s * SW + SW - 1);
    float exc = __shfl_up_sync(TT_FULL_MASK, inc, 1, SW);
    float Q = 0.f, incq = 0.f, excq = 0.f;
    if (need_m2) {
        incq = seg_incl_scan<SW>(totq, sub);
        Q = __shfl_sync(TT_FULL_MASK, incq, s * SW + SW - 1);
        excq = __shfl_up_sync(TT_FULL_MASK, incq, 1, SW);
    }
    if (sub == 0) {
        exc = 0.f;
        excq = 0.f;
    }
    const bool any_neg = __any_sync(TT_FULL_MASK, neg);
    int m1 = 0, m2 = 0;
    if (need_m1 && need_m2 && !any_neg) {
        int f1, f2;
        seg_find_crossing2<SW>(x, C, inc, exc, S, incq, excq, Q, s, sub, f1, f2);
        m1 = resolve_median(f1, S, jlo, jhi, len, n);
        m2 = resolve_median(f2, Q, jlo, jhi, len, n);
    } else {
        if (need_m1) {
            const int f = any_neg ? seg_walk<SW>(x, C, exc, S, sub)
                                  : seg_find_crossing<false, SW>(x, C, inc, exc, S, s, sub);
            m1 = resolve_median(f, S, jlo, jhi, len, n);
        }
        if (need_m2)
            m2 = resolve_median(seg_find_crossing<true, SW>(x, C, incq, excq, Q, s, sub), Q, jlo,
                                jhi, len, n);
    }

    float t1 = 0.f, t2 = 0.f;
    if (need_m1) {
        int j = max(m1, jlo) + sub;
        float r = (float)(j - m1); // exact: integers below 2^24
        for (; j < jhi; j += SW, r += (float)SW) {
            const float vr = x[j - jlo] * r;
            t1 += vr;
            t2 = fmaf(vr, r, t2);
        }
    }
    float re3 = 0.f, im3 = 0.f, re4 = 0.f, im4 = 0.f, re5 = 0.f, im5 = 0.f;
    if (need_m2) {
        const bool w3 = need & (1u << 3), w4 = need & (1u << 4), w5 = need & (1u << 5);
        const float2 *tab3 = J.tab, *tab4 = J.tab + n, *tab5 = J.tab + 2 * n;
        const int qlo = max(1, jlo - m2), qhi = min(n - m2, jhi - m2);
        for (int q = qlo + sub; q < qhi; q += SW) {
            const float v = x[m2 + q - jlo];
            if (w3) {
                const float2 w = __ldg(tab3 + q);
                re3 = fmaf(w.x, v, re3);
                im3 = fmaf(w.y, v, im3);
            }
            if (w4) {
                const float2 w = __ldg(tab4 + q);
                re4 = fmaf(w.x, v, re4);
                im4 = fmaf(w.y, v, im4);
            }
            if (w5) {
                const float2 w = __ldg(tab5 + q);
                re5 = fmaf(w.x, v, re5);
                im5 = fmaf(w.y, v, im5);
            }
        }
    }

    // 4. the eight sums of a segment reduced transposed: after the halving
    // exchanges lane (s, sub) holds sum k = (sub / (SW / 8)) % 8 of
    // (t1, t2, re3, im3, re4, im4, re5, im5), the moduli |re + i im| are
    // taken once per lane, and lane t writes output t (T0's sum S and the
    // medians are held by every lane of the segment)
    const float v8 = seg_sum8<SW>(t1, t2, re3, im3, re4, im4, re5, im5, sub);
    constexpr int unit = SW / 8;
    const int k8 = (sub / unit) & 7;
    const float other = __shfl_xor_sync(TT_FULL_MASK, v8, unit);
    const float res = k8 >= 2 ? hypotf(k8 & 1 ? other : v8, k8 & 1 ? v8 : other) : v8;
    // n_t <= kWarpMaxOutputs <= SW (the hosts' choice of this path)
    const size_t plane = J.plane;
    const size_t at = (size_t)angle * n + col;
    const int t = sub < n_t ? sub : 0;
    const int f = (int)((tf_code >> (3 * t)) & 7ull);
    const int kf = f == 1 ? 0 : f == 2 ? 1 : f == 3 ? 2 : f == 4 ? 4 : 6;
    const float got = __shfl_sync(TT_FULL_MASK, res, s * SW + kf * unit);
    if (colok && sub < n_t) {
        J.out[t * plane + at] = f == 0 ? S : got;
        if (J.medians)
            J.medians[t * plane + at] = f == 0 ? -1 : f <= 2 ? m1 : m2;
    }
}

// One image: warp w of CTA (bx, angle) takes lines (bx W + w) LPW ..
template <int LPW, int W, bool kInterior>
__global__ void __launch_bounds__(32 * W, 32 / W) sino_warp_kernel(const SinoArgs a) {
    extern __shared__ __align__(16) float smw[];
    const int warp = threadIdx.x >> 5;
    BlockJob J;
    J.n = a.n;
    J.col0 = (blockIdx.x * W + warp) * LPW;
    if (J.col0 >= a.n)
        return; // whole warps: no CTA barrier below
    J.tex = a.tex;
    J.tu = 1.f - (float)a.tex_row_off;
    J.tv = 1.f - (float)a.tex_col_off;
    J.angle = blockIdx.y;
    const float2 cs = a.trig[blockIdx.y];
    J.c = cs.x;
    J.s = cs.y;
    if (a.dyn_region) {
        J.roff = a.dyn_region[0];
        J.coff = a.dyn_region[1];
        J.rr = a.dyn_region[2];
        J.rc = a.dyn_region[3];
    } else {
        J.roff = a.row_off;
        J.coff = a.col_off;
        J.rr = a.src_rows;
        J.rc = a.src_cols;
    }
    J.tab = a.tab;
    J.out = a.out;
    J.medians = a.medians;
    J.plane = (size_t)a.n_angles * a.n;
    unsigned long long code = 0;
    for (int t = 0; t < a.n_t; t++)
        code |= (unsigned long long)(a.tf[t] & 7) << (3 * t);
    warp_lines<LPW, kInterior>(J, code, a.n_t, a.need, a.stride,
                               smw + (size_t)warp * LPW * a.stride);
}

// Batch: every warp claims (image, angle, LPW-line block) items from the
// counter until all are taken (items numbered largest image first).
template <int LPW, int W, bool kInterior>
__global__ void __launch_bounds__(32 * W, 32 / W) sino_batch_warp_kernel(const BatchSinoArgs b) {
    extern __shared__ __align__(16) float smw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float *xw = smw + (size_t)warp * LPW * b.stride;
    int lo = 0; // image of the warp's previous item: claims only grow
    for (;;) {
        int item = 0;
        if (lane == 0)
            item = (int)atomicAdd(b.counter, 1u);
        item = __shfl_sync(TT_FULL_MASK, item, 0);
        if (item >= b.total_items)
            break;
        if (lo + 1 < b.n_img && __ldg(&b.img[lo + 1].items_begin) <= item) {
            int hi = b.n_img - 1; // a later image: search [lo + 1, n_img)
            ++lo;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (__ldg(&b.img[mid].items_begin) <= item)
                    lo = mid;
                else
                    hi = mid - 1;
            }
        }
        const BatchImage &im = b.img[lo];
        const int k = item - im.items_begin;
        BlockJob J;
        J.tex = im.tex;
        J.tu = 1.f - (float)im.row_off;
        J.tv = 1.f - (float)im.col_off;
        J.n = im.n;
        J.angle = k / im.blocks;
        J.col0 = (k - J.angle * im.blocks) * LPW;
        const float2 cs = b.trig[im.trig_off + J.angle];
        J.c = cs.x;
        J.s = cs.y;
        J.roff = im.row_off;
        J.coff = im.col_off;
        J.rr = im.rows;
        J.rc = im.cols;
        J.tab = b.tab + im.tab_off;
        J.out = b.sino + im.sino_off;
        J.medians = nullptr;
        J.plane = (size_t)im.n_angles * im.n;
        warp_lines<LPW, kInterior>(J, b.tf_code, b.n_t, b.need, b.stride, xw);
        __syncwarp(); // the line rows are rewritten by the next item
    }
}

// rotate() of c++/src/auxiliary.cpp:223-255 about ((cols-1)/2, (rows-1)/2),
// writing the rotated image (used to check the sampling arithmetic; the
// fused kernel never materialises it).  Same texture path as the fused kernel.
__global__ void rotate_kernel(cudaTextureObject_t tex, int rows, int cols, float2 cs,
                              float *__restrict__ out) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= (long long)rows * cols)
        return;
    const int row = (int)(i % rows), col = (int)(i / rows);
    const float ox = (float)(cols - 1) * 0.5f, oy = (float)(rows - 1) * 0.5f;
    const float X = (float)col - ox, Y = (float)row - oy;
    const float qx = __fadd_rn(__fadd_rn(__fmul_rn(X, cs.x), __fmul_rn(Y, cs.y)), ox);
    const float qy = __fadd_rn(__fadd_rn(__fmul_rn(X, -cs.y), __fmul_rn(Y, cs.x)), oy);
    float v = 0.f;
    if (qx >= 0.f && qx < (float)(cols - 1) && qy >= 0.f && qy < (float)(rows - 1)) {
        const float xi = truncf(qx), yi = truncf(qy);
        const float xf = __fsub_rn(qx, xi), yf = __fsub_rn(qy, yi);
        const float4 g = tex2Dgather<float4>(tex, yi + 1.f, xi + 1.f, 0);
        const float omx = __fsub_rn(1.f, xf), omy = __fsub_rn(1.f, yf);
        const float t0 = __fmul_rn(__fmul_rn(g.w, omx), omy);
        const float t1 = __fmul_rn(__fmul_rn(g.x, xf), omy);
        const float t2 = __fmul_rn(__fmul_rn(g.z, omx), yf);
        const float t3 = __fmul_rn(__fmul_rn(g.y, xf), yf);
        v = __fadd_rn(__fadd_rn(__fadd_rn(t0, t1), t2), t3);
    }
    out[i] = v;
}

// resize() of c++/src/auxiliary.cpp:198-221: the output pixel (row, col)
// samples the input at ((col + 0.5) t00 - 0.5, (row + 0.5) t11 - 0.5) with
// t00 = in_rows / rows, t11 = in_cols / cols (the reference scales x by the
// row ratio and y by the column ratio; the orthonormal mode only resizes
// square images to squares).  The outermost rows and columns stay zero, as
// do samples outside the interpolation domain.  Column-major in and out, one
// thread per output pixel; rounding and operation order as interpolate().
__global__ void resize_kernel(const float *__restrict__ in, int in_rows, int in_cols, int rows,
                              int cols, float t00, float t11, float *__restrict__ out) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= (long long)rows * cols)
        return;
    const int row = (int)(i % rows), col = (int)(i / rows);
    float v = 0.f;
    if (row >= 1 && row < rows - 1 && col >= 1 && col < cols - 1) {
        const float qx = __fsub_rn(__fmul_rn((float)col + 0.5f, t00), 0.5f);
        const float qy = __fsub_rn(__fmul_rn((float)row + 0.5f, t11), 0.5f);
        if (qx >= 0.f && qy >= 0.f && qx < (float)(in_cols - 1) && qy < (float)(in_rows - 1)) {
            const float xi = truncf(qx), yi = truncf(qy);
            const float xf = __fsub_rn(qx, xi), yf = __fsub_rn(qy, yi);
            const size_t x0 = (size_t)xi, y0 = (size_t)yi;
            const float *c0 = in + x0 * in_rows + y0, *c1 = c0 + in_rows;
            const float omx = __fsub_rn(1.f, xf), omy = __fsub_rn(1.f, yf);
            const float t0 = __fmul_rn(__fmul_rn(__ldg(c0), omx), omy);
            const float t1 = __fmul_rn(__fmul_rn(__ldg(c1), xf), omy);
            const float t2 = __fmul_rn(__fmul_rn(__ldg(c0 + 1), omx), yf);
            const float t3 = __fmul_rn(__fmul_rn(__ldg(c1 + 1), xf), yf);
            v = __fadd_rn(__fadd_rn(__fadd_rn(t0, t1), t2), t3);
        }
    }
    out[i] = v;
}

// Bounding box of the non-zero pixels of an n x n frame.
__global__ void bbox_init(int *r) {
    r[0] = INT_MAX; // min row
    r[1] = INT_MAX; // min col
    r[2] = -1;      // max row
    r[3] = -1;      // max col
}

__global__ void bbox_kernel(const float *__restrict__ f, int n, int *r) {
    int mnr = INT_MAX, mnc = INT_MAX, mxr = -1, mxc = -1;
    const long long total = (long long)n * n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        if (f[i] != 0.f) {
            const int row = (int)(i % n), col = (int)(i / n);
            mnr = min(mnr, row);
            mxr = max(mxr, row);
            mnc = min(mnc, col);
            mxc = max(mxc, col);
        }
    }
    mnr = warp_min(mnr);
    mnc = warp_min(mnc);
    mxr = warp_max(mxr);
    mxc = warp_max(mxc);
    if ((threadIdx.x & 31) == 0 && mxr >= 0) {
        atomicMin(r + 0, mnr);
        atomicMin(r + 1, mnc);
        atomicMax(r + 2, mxr);
        atomicMax(r + 3, mxc);
    }
}

// {min row, min col, max row, max col} -> {row0, col0, rows, cols}
__global__ void bbox_finish(int *r) {
    if (r[2] < 0) {
        r[0] = 0;
        r[1] = 0;
        r[2] = 0;
        r[3] = 0;
    } else {
        r[2] = r[2] - r[0] + 1;
        r[3] = r[3] - r[1] + 1;
    }
}

template <int L, bool kSel>
cudaError_t launch_one(const SinoArgs &a, size_t smem, cudaStream_t stream) {
    // 4 lines per CTA (long lines: 2 CTAs per SM by shared memory) are
    // sampled by 16 warps, so that more gathers are in flight per SM
    constexpr int W = L == 4 ? 16 : L;
    const void *k = a.interior ? (const void *)sino_kernel<L, kSel, true, W>
                               : (const void *)sino_kernel<L, kSel, false, W>;
    const size_t limit = opt_in_smem(k);
    if (limit == 0)
        return cudaErrorInvalidValue;
    if (smem > limit)
        return cudaErrorInvalidValue;
    dim3 grid((a.n + L - 1) / L, a.n_angles);
    void *args[] = {(void *)&a};
    return cudaLaunchKernel(k, grid, dim3(32 * W), args, smem, stream);
}

} // namespace

size_t dynamic_smem_limit(const void *kernel) {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa{};
    cudaFuncGetAttributes(&fa, kernel);
    return optin > (int)fa.sharedSizeBytes ? (size_t)optin - fa.sharedSizeBytes : 0;
}

size_t opt_in_smem(const void *kernel) {
    static std::mutex mu;
    static std::map<std::pair<int, const void *>, size_t> done; // (device, kernel) -> limit
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
        return 0;
    std::lock_guard<std::mutex> lock(mu);
    const auto key = std::make_pair(dev, kernel);
    const auto it = done.find(key);
    if (it != done.end())
        return it->second;
    const size_t limit = dynamic_smem_limit(kernel);
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)limit) !=
        cudaSuccess)
        return 0;
    done.emplace(key, limit);
    return limit;
}

int sino_lines_per_block(int n, unsigned need) {
    // eight lines per CTA unless the line buffers (+ T6/T7 histograms) would
    // leave room for a single CTA per SM
    return sino_smem_bytes(n, 8, need) > 110 * 1024 ? 4 : 8;
}

int sino_stride(int n, int lines) {
    const int cmax = (((n + 31) >> 5) | 1);
    return 32 * cmax + 32 / lines;
}

size_t sino_smem_bytes(int n, int lines, unsigned need) {
    size_t bytes = sizeof(float) * (size_t)lines * sino_stride(n, lines);
    if (need & ((1u << 6) | (1u << 7)))
        bytes = ((bytes + 15) & ~size_t(15)) + 2 * sizeof(SelScratch) * lines;
    return bytes;
}

cudaError_t launch_sinograms(const SinoArgs &a, int lines, cudaStream_t stream) {
    const size_t smem = sino_smem_bytes(a.n, lines, a.need);
    const bool sel = a.need & ((1u << 6) | (1u << 7));
    if (lines == 8)
        return sel ? launch_one<8, true>(a, smem, stream) : launch_one<8, false>(a, smem, stream);
    return sel ? launch_one<4, true>(a, smem, stream) : launch_one<4, false>(a, smem, stream);
}

namespace {
const void *batch_cta_kernel(int lines, bool sel, bool in) {
    if (lines == 8)
        return sel ? (in ? (const void *)sino_batch_kernel<8, true, true>
                         : (const void *)sino_batch_kernel<8, true, false>)
                   : (in ? (const void *)sino_batch_kernel<8, false, true>
                         : (const void *)sino_batch_kernel<8, false, false>);
    return sel ? (in ? (const void *)sino_batch_kernel<4, true, true>
                     : (const void *)sino_batch_kernel<4, true, false>)
               : (in ? (const void *)sino_batch_kernel<4, false, true>
                     : (const void *)sino_batch_kernel<4, false, false>);
}
} // namespace

cudaError_t prepare_sino_batch(int lines, bool sel, bool interior, size_t smem) {
    const size_t limit = opt_in_smem(batch_cta_kernel(lines, sel, interior));
    if (limit == 0)
        return cudaErrorInvalidValue;
    return smem > limit ? cudaErrorInvalidValue : cudaSuccess;
}

int sino_batch_occupancy(int lines, bool sel, bool interior, size_t smem) {
    if (prepare_sino_batch(lines, sel, interior, smem) != cudaSuccess)
        return 0;
    int blocks = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, batch_cta_kernel(lines, sel, interior),
                                                  32 * lines, smem);
    return blocks;
}

cudaError_t launch_sino_batch(const BatchSinoArgs &a, int lines, int grid, size_t smem,
                              cudaStream_t stream) {
    if (grid <= 0 || a.total_items <= 0)
        return cudaSuccess;
    const bool sel = a.need & ((1u << 6) | (1u << 7));
    void *args[] = {(void *)&a};
    return cudaLaunchKernel(batch_cta_kernel(lines, sel, a.all_interior), dim3(grid),
                            dim3(32 * lines), args, smem, stream);
}

// ---- warp-autonomous variants (T0-T5) ------------------------------------------

namespace {
constexpr int kWarpCtaWarps = 4; // warps per CTA of the warp-autonomous kernels

template <int LPW, bool kI> cudaError_t launch_warp_one(const SinoArgs &a, size_t smem,
                                                        cudaStream_t stream) {
    const size_t limit = opt_in_smem((const void *)sino_warp_kernel<LPW, kWarpCtaWarps, kI>);
    if (limit == 0 || smem > limit)
        return cudaErrorInvalidValue;
    constexpr int L = LPW * kWarpCtaWarps;
    dim3 grid((a.n + L - 1) / L, a.n_angles);
    sino_warp_kernel<LPW, kWarpCtaWarps, kI><<<grid, 32 * kWarpCtaWarps, smem, stream>>>(a);
    return cudaGetLastError();
}

template <int LPW, bool kI> const void *batch_warp_fn() {
    return (const void *)sino_batch_warp_kernel<LPW, kWarpCtaWarps, kI>;
}

const void *batch_warp_kernel(int lpw, bool interior) {
    if (lpw == 1)
        return interior ? batch_warp_fn<1, true>() : batch_warp_fn<1, false>();
    if (lpw == 2)
        return interior ? batch_warp_fn<2, true>() : batch_warp_fn<2, false>();
    return interior ? batch_warp_fn<4, true>() : batch_warp_fn<4, false>();
}
} // namespace

int sino_warp_stride(int n, int lpw) { return warp_line_stride(n, lpw); }

size_t sino_warp_smem_bytes(int n, int lpw) {
    return sizeof(float) * (size_t)kWarpCtaWarps * lpw * warp_line_stride(n, lpw);
}

cudaError_t launch_sinograms_warp(const SinoArgs &a, int lpw, cudaStream_t stream) {
    if (a.need & ((1u << 6) | (1u << 7)))
        return cudaErrorInvalidValue; // T6 / T7 take the CTA kernels
    const size_t smem = sino_warp_smem_bytes(a.n, lpw);
    const bool in = a.interior;
    if (lpw == 1)
        return in ? launch_warp_one<1, true>(a, smem, stream)
                  : launch_warp_one<1, false>(a, smem, stream);
    if (lpw == 2)
        return in ? launch_warp_one<2, true>(a, smem, stream)
                  : launch_warp_one<2, false>(a, smem, stream);
    return in ? launch_warp_one<4, true>(a, smem, stream)
              : launch_warp_one<4, false>(a, smem, stream);
}

int sino_batch_warp_occupancy(int lpw, bool interior, size_t smem) {
    const void *k = batch_warp_kernel(lpw, interior);
    const size_t limit = opt_in_smem(k);
    if (limit == 0 || smem > limit)
        return 0;
    int blocks = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k, 32 * kWarpCtaWarps, smem);
    return blocks;
}

int sino_warp_cta_warps() { return kWarpCtaWarps; }

cudaError_t launch_sino_batch_warp(const BatchSinoArgs &a, int lpw, int grid, size_t smem,
                                   cudaStream_t stream) {
    if (grid <= 0 || a.total_items <= 0)
        return cudaSuccess;
    if (a.need & ((1u << 6) | (1u << 7)))
        return cudaErrorInvalidValue;
    if (sino_batch_warp_occupancy(lpw, a.all_interior, smem) <= 0)
        return cudaErrorInvalidValue;
    void *args[] = {(void *)&a};
    return cudaLaunchKernel(batch_warp_kernel(lpw, a.all_interior), dim3(grid),
                            dim3(32 * kWarpCtaWarps), args, smem, stream);
}

cudaError_t launch_rotate(cudaTextureObject_t tex, int rows, int cols, float c, float s,
                          float *out, cudaStream_t stream) {
    const long long total = (long long)rows * cols;
    if (total == 0)
        return cudaSuccess;
    rotate_kernel<<<(unsigned)((total + 255) / 256), 256, 0, stream>>>(tex, rows, cols,
                                                                       make_float2(c, s), out);
    return cudaGetLastError();
}

cudaError_t launch_resize(const float *in, int in_rows, int in_cols, int rows, int cols,
                          float *out, cudaStream_t stream) {
    const long long total = (long long)rows * cols;
    if (total == 0)
        return cudaSuccess;
    const float t00 = (float)in_rows / (float)rows, t11 = (float)in_cols / (float)cols;
    resize_kernel<<<(unsigned)((total + 255) / 256), 256, 0, stream>>>(in, in_rows, in_cols, rows,
                                                                       cols, t00, t11, out);
    return cudaGetLastError();
}

cudaError_t launch_region_bbox(const float *frame, int n, int *d_region,
                               cudaStream_t stream) {
    bbox_init<<<1, 1, 0, stream>>>(d_region);
    long long total = (long long)n * n;
    int blocks = (int)std::min<long long>((total + 255) / 256, 152 * 8);
    if (blocks < 1)
        blocks = 1;
    bbox_kernel<<<blocks, 256, 0, stream>>>(frame, n, d_region);
    bbox_finish<<<1, 1, 0, stream>>>(d_region);
    return cudaGetLastError();
}

} // namespace tt
