// tt_sinogram.cu -- fused rotate + T-functional kernel.
//
// One CTA owns L adjacent columns ("trace lines") of one angle.  It samples
// the rotated image along those lines straight from the source image (no
// rotated image is written anywhere), keeps the samples of its lines in
// shared memory, and then reduces each line with one warp into every
// requested T-functional (c++/src/sinogram.cpp:67-178 with the functionals of
// c++/src/functionals.cpp:21-276).
//
// Rotated samples are bit-identical to the reference's rotate()/interpolate()
// (c++/src/auxiliary.cpp:182-196, 223-255): the host rounds cos/sin exactly as
// the reference does, and the coordinate transform and bilinear expression
// are evaluated with explicit round-to-nearest intrinsics in the reference's
// order, so no multiply-add is fused.  Only rows whose 2x2 stencil can touch
// the image are sampled; all others are exact zeros in the reference too.
//
// Reductions run in warp order rather than the reference's sequential order,
// so sums agree to rounding and a weighted median can move by one row where
// the reference's cumulative sum ties the half-total to within rounding.
#include <climits>

#include "tt_common.cuh"
#include "tt_internal.h"

namespace tt {
namespace {

constexpr int kLines = 8; // lines (warps) per CTA

// Bilinear sample at frame coordinates (qx, qy), reference order.  The
// reference samples only where 0 <= qx < xmax and 0 <= qy < ymax (frame
// columns - 1, rows - 1); the source region is rr x rc at (roff, coff).
__device__ __forceinline__ float sample(const float *__restrict__ src, int ld,
                                        int rr, int rc, int roff, int coff,
                                        float xmax, float ymax, float qx, float qy) {
    if (!(qx >= 0.f && qx < xmax && qy >= 0.f && qy < ymax))
        return 0.f;
    const float xi = truncf(qx), yi = truncf(qy);
    const float xf = __fsub_rn(qx, xi), yf = __fsub_rn(qy, yi);
    const int cx = (int)xi - coff, cy = (int)yi - roff;
    const bool x0 = (unsigned)cx < (unsigned)rc;
    const bool x1 = (unsigned)(cx + 1) < (unsigned)rc;
    const bool y0 = (unsigned)cy < (unsigned)rr;
    const bool y1 = (unsigned)(cy + 1) < (unsigned)rr;
    const long long o00 = (long long)cx * ld + cy;
    const float s00 = (x0 && y0) ? __ldg(src + o00) : 0.f;
    const float s10 = (x0 && y1) ? __ldg(src + o00 + 1) : 0.f;
    const float s01 = (x1 && y0) ? __ldg(src + o00 + ld) : 0.f;
    const float s11 = (x1 && y1) ? __ldg(src + o00 + ld + 1) : 0.f;
    const float omx = __fsub_rn(1.f, xf), omy = __fsub_rn(1.f, yf);
    const float t0 = __fmul_rn(__fmul_rn(s00, omx), omy);
    const float t1 = __fmul_rn(__fmul_rn(s01, xf), omy);
    const float t2 = __fmul_rn(__fmul_rn(s10, omx), yf);
    const float t3 = __fmul_rn(__fmul_rn(s11, xf), yf);
    return __fadd_rn(__fadd_rn(__fadd_rn(t0, t1), t2), t3);
}

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
        float a0 = o + (xlo - bx) / s, a1 = o + (xhi - bx) / s;
        jl = fmaxf(jl, fminf(a0, a1));
        jh = fminf(jh, fmaxf(a0, a1));
    } else if (bx < xlo || bx > xhi) {
        jh = -1.f;
    }
    if (fabsf(c) > 1e-7f) {
        float a0 = o + (ylo - by) / c, a1 = o + (yhi - by) / c;
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

// Smallest key k (a non-negative float) with 2 * sum(weights of keys <= k) >=
// sum(weights): the weighted median of a sorted sequence as TFunctional6 /
// TFunctional7 take it (c++/src/functionals.cpp:226-276), found by bisection
// on the key's bit pattern.  Elements are the stored rows [b, jhi) of a line.
template <bool kT6>
__device__ float weighted_select(const float *x, int jlo, int jhi, int b,
                                 int m, int lane) {
    float wt = 0.f;
    for (int j = b + lane; j < jhi; j += 32)
        wt += __fsqrt_rn(x[j - jlo]);
    wt = warp_sum(wt);
    unsigned lo = 0u, hi = 0x7f800000u;
    while (lo < hi) {
        const unsigned mid = lo + ((hi - lo) >> 1);
        float f = 0.f;
        for (int j = b + lane; j < jhi; j += 32) {
            const float v = x[j - jlo];
            const float key = kT6 ? __fmul_rn((float)(j - m), v) : v;
            if (__float_as_uint(key) <= mid)
                f += __fsqrt_rn(v);
        }
        f = warp_sum(f);
        if (2.f * f >= wt)
            hi = mid;
        else
            lo = mid + 1u;
    }
    return __uint_as_float(lo);
}

template <int L>
__global__ void __launch_bounds__(32 * L)
    sino_kernel(const SinoArgs a) {
    extern __shared__ float sm[];
    __shared__ int s_range[2];
    __shared__ int s_region[4];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int angle = blockIdx.y;
    const int col0 = blockIdx.x * L;
    const int n = a.n;
    const float2 cs = a.trig[angle];
    const float c = cs.x, s = cs.y, ms = -cs.y;
    const float o = (float)(n - 1) * 0.5f;
    const float nm1 = (float)(n - 1);

    // Source region (static or computed on the device).
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
    const int roff = s_region[0], coff = s_region[1];
    const int rr = max(s_region[2], 0), rc = max(s_region[3], 0);
    const float *src = a.dyn_region ? a.src + (long long)coff * a.src_ld + roff : a.src;

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
    const int span = 32 * C;

    // 2. Sample the lines into shared memory (zeros past len).
    {
        constexpr int RPW = 32 / L;
        const int l = lane % L, r = lane / L;
        const int col = col0 + l;
        const float X = (float)col - o;
        const float Xc = __fmul_rn(X, c), Xms = __fmul_rn(X, ms);
        float *dst = sm + l * a.stride;
#pragma unroll 4
        for (int jr = warp * RPW + r; jr < span; jr += 32) {
            float v = 0.f;
            if (jr < len && col < n) {
                const float Y = (float)(jlo + jr) - o;
                const float qx = __fadd_rn(__fadd_rn(Xc, __fmul_rn(Y, s)), o);
                const float qy = __fadd_rn(__fadd_rn(Xms, __fmul_rn(Y, c)), o);
                v = sample(src, a.src_ld, rr, rc, roff, coff, nm1, nm1, qx, qy);
            }
            dst[jr] = v;
        }
    }
    __syncthreads();

    // 3. One warp per line: T-functionals.
    const int col = col0 + warp;
    if (col >= n)
        return;
    const float *x = sm + warp * a.stride;
    const unsigned need = a.need;
    const bool need_m1 = need & ((1u << 1) | (1u << 2) | (1u << 7));
    const bool need_m2 = need & ((1u << 3) | (1u << 4) | (1u << 5) | (1u << 6));
    const int base = lane * C;

    float tot = 0.f, totq = 0.f;
    for (int k = 0; k < C; k++) {
        const float v = x[base + k];
        tot += v;
        if (need_m2)
            totq += __fsqrt_rn(v);
    }
    const float inc = warp_incl_scan(tot, lane);
    const float S = __shfl_sync(TT_FULL_MASK, inc, 31);
    float ps = __shfl_up_sync(TT_FULL_MASK, inc, 1);
    float Q = 0.f, pq = 0.f;
    if (need_m2) {
        const float incq = warp_incl_scan(totq, lane);
        Q = __shfl_sync(TT_FULL_MASK, incq, 31);
        pq = __shfl_up_sync(TT_FULL_MASK, incq, 1);
    }
    if (lane == 0) {
        ps = 0.f;
        pq = 0.f;
    }

    int m1 = 0, m2 = 0;
    if (need_m1 || need_m2) {
        int f1 = INT_MAX, f2 = INT_MAX;
        for (int k = 0; k < C; k++) {
            const float v = x[base + k];
            ps += v;
            if (f1 == INT_MAX && 2.f * ps >= S)
                f1 = base + k;
            if (need_m2) {
                pq += __fsqrt_rn(v);
                if (f2 == INT_MAX && 2.f * pq >= Q)
                    f2 = base + k;
            }
        }
        m1 = resolve_median(warp_min(f1), S, jlo, jhi, len, n);
        if (need_m2)
            m2 = resolve_median(warp_min(f2), Q, jlo, jhi, len, n);
    }

    float r1v = 0.f, r2v = 0.f;
    if (need & ((1u << 1) | (1u << 2))) {
        float t1 = 0.f, t2 = 0.f;
        for (int k = 0; k < C; k++) {
            const int j = jlo + base + k;
            const float v = x[base + k];
            if (j >= m1) {
                const float r = (float)(j - m1);
                const float vr = v * r;
                t1 += vr;
                t2 += vr * r;
            }
        }
        r1v = warp_sum(t1);
        r2v = warp_sum(t2);
    }

    float r345[3] = {0.f, 0.f, 0.f};
    if (need & ((1u << 3) | (1u << 4) | (1u << 5))) {
        const bool w3 = need & (1u << 3), w4 = need & (1u << 4), w5 = need & (1u << 5);
        const float2 *tab3 = a.tab, *tab4 = a.tab + n, *tab5 = a.tab + 2 * n;
        float re3 = 0.f, im3 = 0.f, re4 = 0.f, im4 = 0.f, re5 = 0.f, im5 = 0.f;
        const int lo = max(1, jlo - m2), hi = min(n - m2, jhi - m2);
        for (int q = lo + lane; q < hi; q += 32) {
            const float v = x[m2 + q - jlo];
            if (w3) {
                const float2 w = __ldg(tab3 + q);
                re3 += w.x * v;
                im3 += w.y * v;
            }
            if (w4) {
                const float2 w = __ldg(tab4 + q);
                re4 += w.x * v;
                im4 += w.y * v;
            }
            if (w5) {
                const float2 w = __ldg(tab5 + q);
                re5 += w.x * v;
                im5 += w.y * v;
            }
        }
        // hypot of the two float integrals in double, as C's hypot does
        if (w3) {
            const double re = warp_sum(re3), im = warp_sum(im3);
            r345[0] = (float)sqrt(re * re + im * im);
        }
        if (w4) {
            const double re = warp_sum(re4), im = warp_sum(im4);
            r345[1] = (float)sqrt(re * re + im * im);
        }
        if (w5) {
            const double re = warp_sum(re5), im = warp_sum(im5);
            r345[2] = (float)sqrt(re * re + im * im);
        }
    }

    float r6v = 0.f, r7v = 0.f;
    if (need & (1u << 6))
        r6v = weighted_select<true>(x, jlo, jhi, max(m2, jlo), m2, lane);
    if (need & (1u << 7))
        r7v = weighted_select<false>(x, jlo, jhi, max(m1, jlo), m1, lane);

    if (lane == 0) {
        const size_t plane = (size_t)a.n_angles * n;
        const size_t at = (size_t)angle * n + col;
        for (int t = 0; t < a.n_t; t++) {
            const int f = a.tf[t];
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
            a.out[t * plane + at] = v;
            if (a.medians)
                a.medians[t * plane + at] = med;
        }
    }
}

// rotate() of c++/src/auxiliary.cpp:223-255 about ((cols-1)/2, (rows-1)/2),
// writing the rotated image (used to check the sampling arithmetic; the
// fused kernel never materialises it).
__global__ void rotate_kernel(const float *__restrict__ src, int rows, int cols, float2 cs,
                              float *__restrict__ out) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= (long long)rows * cols)
        return;
    const int row = (int)(i % rows), col = (int)(i / rows);
    const float ox = (float)(cols - 1) * 0.5f, oy = (float)(rows - 1) * 0.5f;
    const float X = (float)col - ox, Y = (float)row - oy;
    const float qx = __fadd_rn(__fadd_rn(__fmul_rn(X, cs.x), __fmul_rn(Y, cs.y)), ox);
    const float qy = __fadd_rn(__fadd_rn(__fmul_rn(X, -cs.y), __fmul_rn(Y, cs.x)), oy);
    out[i] = sample(src, rows, rows, cols, 0, 0, (float)(cols - 1), (float)(rows - 1), qx, qy);
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

} // namespace

int sino_lines_per_block() { return kLines; }

int sino_stride(int n, int lines) {
    const int cmax = (((n + 31) >> 5) | 1);
    return 32 * cmax + 32 / lines;
}

size_t sino_smem_bytes(int n, int lines) {
    return sizeof(float) * (size_t)lines * sino_stride(n, lines);
}

size_t dynamic_smem_limit(const void *kernel) {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa{};
    cudaFuncGetAttributes(&fa, kernel);
    return optin > (int)fa.sharedSizeBytes ? (size_t)optin - fa.sharedSizeBytes : 0;
}

cudaError_t launch_sinograms(const SinoArgs &a, cudaStream_t stream) {
    const int L = kLines;
    const size_t smem = sino_smem_bytes(a.n, L);
    static size_t limit = 0;
    if (limit == 0) {
        limit = dynamic_smem_limit((const void *)sino_kernel<kLines>);
        cudaError_t e = cudaFuncSetAttribute(sino_kernel<kLines>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)limit);
        if (e != cudaSuccess)
            return e;
    }
    if (smem > limit)
        return cudaErrorInvalidValue;
    dim3 grid((a.n + L - 1) / L, a.n_angles);
    sino_kernel<kLines><<<grid, 32 * L, smem, stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_rotate(const float *src, int rows, int cols, float c, float s, float *out,
                          cudaStream_t stream) {
    const long long total = (long long)rows * cols;
    if (total == 0)
        return cudaSuccess;
    rotate_kernel<<<(unsigned)((total + 255) / 256), 256, 0, stream>>>(src, rows, cols,
                                                                       make_float2(c, s), out);
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
