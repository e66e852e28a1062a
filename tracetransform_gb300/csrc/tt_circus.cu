// tt_circus.cu -- P-functional (circus) kernels and z-score kernel
// (c++/src/circus.cpp:104-177 with c++/src/functionals.cpp:287-386).
//
// P1-P3 over stacks of sinogram columns (every call without Hermite, and
// the batched engine), three launches:
//   p3_dft_kernel      P3: the real DFT of every column as a GEMM-shaped
//                      direct sum F = W^T X with |F_k / N|^4 and the trapz
//                      weights folded into the epilogue (partial sums per
//                      64-frequency tile, added in tile order: deterministic)
//   circus_p12_kernel  one warp per column: P1 = sum |x[p] - x[p-1]|, P2 = the
//                      weighted median of the column weighted by itself by
//                      selection (tt_select.cuh, no sort), P3's tile sums
//   p2_sort_kernel     P2 by an exact bitonic sort for the columns the
//                      selection cannot take (negative or non-finite values)
// circus_kernel (one CTA per column) serves calls with Hermite
// P-functionals: P1, P2 by bitonic sort, P3 by the chirp-z (Bluestein)
// identity on a power-of-two shared-memory FFT, and the Hermite projections
// on a host-built basis psi_order(z(p)).
// zscore_kernel follows c++/src/auxiliary.cpp:277-318 in the reference's own
// order: a float mean, a double sum of squared float differences, n - 1.
#include <climits>

#include "tt_common.cuh"
#include "tt_internal.h"
#include "tt_select.cuh"

namespace tt {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// z-score of one vector by one block, in the reference's order.
__device__ __forceinline__ void zscore_vector(const float *__restrict__ x, int len,
                                              float *__restrict__ z) {
    __shared__ float s_mean, s_std;
    if (threadIdx.x == 0) {
        float sum = 0.f;
        for (int i = 0; i < len; i++)
            sum = __fadd_rn(sum, x[i]);
        const float mean = __fdiv_rn(sum, (float)len);
        double acc = 0.0;
        for (int i = 0; i < len; i++) {
            const double d = (double)__fsub_rn(x[i], mean);
            acc = __dadd_rn(acc, __dmul_rn(d, d));
        }
        s_mean = mean;
        s_std = (float)sqrt(acc / (double)(len - 1));
    }
    __syncthreads();
    for (int i = threadIdx.x; i < len; i += blockDim.x)
        z[i] = __fdiv_rn(__fsub_rn(x[i], s_mean), s_std);
}

// All requested P-functionals of column colidx of sinogram sidx.  Every thread
// of the block calls it (it synchronises the block); smraw is the dynamic
// shared memory sized by circus_smem_bytes.
__device__ __forceinline__ void circus_column(const CircusArgs &a, int sidx, int colidx,
                                              unsigned char *smraw, float *red, int *redi) {
    const int tid = threadIdx.x, bd = blockDim.x;
    const int rows = a.rows, M = a.M, P = a.sort_len;
    const bool need_p2 = a.need & (1u << 2), need_p3 = a.need & (1u << 3);

    float2 *fft = reinterpret_cast<float2 *>(smraw);              // M (P3)
    float *colv = reinterpret_cast<float *>(fft + (need_p3 ? M : 0)); // rows
    float *srt = colv + ((rows + 3) & ~3);                         // P (P2, P3)

    const float *src = a.sino + ((size_t)sidx * a.cols + colidx) * rows;
    for (int i = tid; i < rows; i += bd)
        colv[i] = src[i];
    __syncthreads();

    float res[kMaxP];
#pragma unroll
    for (int p = 0; p < kMaxP; p++)
        res[p] = 0.f;

    // P1
    if (a.need & (1u << 1)) {
        float acc = 0.f;
        for (int i = 1 + tid; i < rows; i += bd)
            acc += fabsf(colv[i - 1] - colv[i]);
        const float v = block_sum(acc, red);
        for (int p = 0; p < a.n_p; p++)
            if (a.kind[p] == 1)
                res[p] = v;
    }

    // P2
    if (need_p2) {
        for (int i = tid; i < P; i += bd)
            srt[i] = i < rows ? colv[i] : __int_as_float(0x7f800000);
        __syncthreads();
        for (int k = 2; k <= P; k <<= 1) {
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int i = tid; i < P; i += bd) {
                    const int ixj = i ^ j;
                    if (ixj > i) {
                        const float u = srt[i], w = srt[ixj];
                        const bool up = (i & k) == 0;
                        if ((u > w) == up) {
                            srt[i] = w;
                            srt[ixj] = u;
                        }
                    }
                }
                __syncthreads();
            }
        }
        // weighted median of the sorted column, weights = values
        const int per = (rows + bd - 1) / bd;
        const int beg = min(tid * per, rows), end = min(beg + per, rows);
        float loc = 0.f;
        for (int i = beg; i < end; i++)
            loc += srt[i];
        float total;
        float run = block_excl_scan(loc, red, &total);
        int found = INT_MAX;
        for (int i = beg; i < end; i++) {
            run += srt[i];
            if (2.f * run >= total) {
                found = i;
                break;
            }
        }
        found = block_min(found, redi);
        const float v = srt[found == INT_MAX ? rows - 1 : found];
        for (int p = 0; p < a.n_p; p++)
            if (a.kind[p] == 2)
                res[p] = v;
        __syncthreads();
    }

    // P3
    if (need_p3) {
        const int logM = 31 - __clz(M);
        for (int i = tid; i < M; i += bd)
            fft[i] = make_float2(0.f, 0.f);
        __syncthreads();
        for (int j = tid; j < rows; j += bd) {
            const float2 w = __ldg(a.chirp + j);
            const float v = colv[j];
            fft[__brev(j) >> (32 - logM)] = make_float2(v * w.x, v * w.y);
        }
        __syncthreads();
        // forward radix-2 DIT, natural-order output
        for (int h = 1; h < M; h <<= 1) {
            const int tstep = M / (2 * h);
            for (int i = tid; i < M / 2; i += bd) {
                const int pos = i & (h - 1);
                const int ia = ((i - pos) << 1) + pos, ib = ia + h;
                const float2 t = cmul(fft[ib], __ldg(a.twid + pos * tstep));
                const float2 u = fft[ia];
                fft[ia] = make_float2(u.x + t.x, u.y + t.y);
                fft[ib] = make_float2(u.x - t.x, u.y - t.y);
            }
            __syncthreads();
        }
        for (int i = tid; i < M; i += bd)
            fft[i] = cmul(fft[i], __ldg(a.filt + i));
        __syncthreads();
        // inverse radix-2 DIF (conjugate twiddles), bit-reversed output
        for (int h = M / 2; h >= 1; h >>= 1) {
            const int tstep = M / (2 * h);
            for (int i = tid; i < M / 2; i += bd) {
                const int pos = i & (h - 1);
                const int ia = ((i - pos) << 1) + pos, ib = ia + h;
                const float2 u = fft[ia], w = fft[ib];
                const float2 tw = __ldg(a.twid + pos * tstep);
                fft[ia] = make_float2(u.x + w.x, u.y + w.y);
                fft[ib] = cmul(make_float2(u.x - w.x, u.y - w.y), make_float2(tw.x, -tw.y));
            }
            __syncthreads();
        }
        // (|F_k| / N)^4 for k <= N/2 into srt
        const float fn = (float)rows;
        const int nb = rows / 2 + 1;
        for (int k = tid; k < nb; k += bd) {
            const float2 F = cmul(fft[__brev(k) >> (32 - logM)], __ldg(a.chirp + k));
            const double fr = (double)(F.x / fn), fi = (double)(F.y / fn);
            const double h2 = fr * fr + fi * fi;
            srt[k] = (float)(h2 * h2);
        }
        __syncthreads();
        // trapz over p = 0 .. rows-1 with the mirror y[p] = y[rows - p]
        float acc = 0.f;
        for (int i = tid; i < rows - 1; i += bd) {
            const int p0 = i <= rows / 2 ? i : rows - i;
            const int p1 = (i + 1) <= rows / 2 ? i + 1 : rows - (i + 1);
            acc += (__ldg(a.lin + i + 1) - __ldg(a.lin + i)) * (srt[p1] + srt[p0]);
        }
        const float v = (float)((double)block_sum(acc, red) * 0.5);
        for (int p = 0; p < a.n_p; p++)
            if (a.kind[p] == 3)
                res[p] = v;
        __syncthreads();
    }

    // Hermite projections
    if (a.need & 1u) {
        for (int p = 0; p < a.n_p; p++) {
            if (a.kind[p] != 0)
                continue;
            const float *basis = a.herm[(size_t)sidx * a.n_p + p];
            float acc = 0.f;
            for (int i = tid; i < rows; i += bd)
                acc += colv[i] * __ldg(basis + i);
            res[p] = block_sum(acc, red);
        }
    }

    if (tid == 0) {
        for (int p = 0; p < a.n_p; p++)
            if (a.need & (1u << a.kind[p])) // kinds left to another kernel stay as they are
                a.out[((size_t)sidx * a.n_p + p) * a.cols + colidx] = res[p];
    }
}

__global__ void __launch_bounds__(kThreads) circus_kernel(const CircusArgs a) {
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ float red[kThreads / 32];
    __shared__ int redi[kThreads / 32];
    circus_column(a, blockIdx.y, blockIdx.x, smraw, red, redi);
}

// z-score of vectors of varying length: vector v is in[off[v] .. off[v] + len[v]).
__global__ void zscore_batch_kernel(const float *__restrict__ in, const long long *__restrict__ off,
                                    const int *__restrict__ len, float *__restrict__ out) {
    const long long o = off[blockIdx.x];
    zscore_vector(in + o, len[blockIdx.x], out + o);
}

__global__ void zscore_kernel(const float *__restrict__ in, int len,
                              float *__restrict__ out) {
    zscore_vector(in + (size_t)blockIdx.x * len, len, out + (size_t)blockIdx.x * len);
}

// ---- P-stage over stacks --------------------------------------------------
//
// P3 as a direct DFT computed like a GEMM.  For a stack of columns X (n x
// cols), F = W^T X with W[p][2k] = cos(2 pi k p / n), W[p][2k+1] =
// -sin(2 pi k p / n), k <= n/2; the epilogue folds |F_k / n|^4 and the trapz
// weights ck[k] into one partial sum per (64-frequency tile, column), which
// the per-column kernel adds in tile order (deterministic).  A CTA computes a
// 128 x 128 tile of F (64 frequencies as re/im rows x 128 columns) with an
// 8 x 8 register tile per thread, samples staged 16 at a time through shared
// memory (next step's global loads in flight during the current step's
// FMAs); W is generated from the n-entry twiddle table with an incremental
// (k p) mod n index.  The O(n^2) DFT replaces the Bluestein FFT's two
// power-of-two transforms in shared memory: at these lengths the FMA pipe
// runs it faster than the FFT's barrier-bound butterflies, and its float
// error (accumulated over n terms) stays far inside the 1e-4 tolerance.
constexpr int kDftBM = 128, kDftBN = 128, kDftBK = 16, kFreqTile = kDftBM / 2;

__device__ __forceinline__ const CircusStack &stack_at(const CircusStackArgs &a, int i) {
    return a.st ? a.st[i] : a.one;
}

__device__ __forceinline__ int stack_of(const CircusStack *st, int n_st, int v, bool by_tile) {
    int lo = 0, hi = n_st - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        const int b = by_tile ? __ldg(&st[mid].tile_begin) : __ldg(&st[mid].col_begin);
        if (b <= v)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

__global__ void __launch_bounds__(256, 2) p3_dft_kernel(const CircusStackArgs a) {
    __shared__ __align__(16) float Ws[kDftBK][kDftBM];
    __shared__ __align__(16) float Xs[kDftBK][kDftBN];
    __shared__ float Red[16][kDftBN];
    const int tile = blockIdx.x;
    const CircusStack &S = stack_at(a, stack_of(a.st, a.n_st, tile, true));
    const int n = S.n, cols = S.cols, K = n / 2 + 1;
    const int local = tile - S.tile_begin;
    const int mt = local % S.mtiles, ct = local / S.mtiles;
    const int k0 = mt * kFreqTile, c0 = ct * kDftBN;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const float2 *tw = S.tw;
    const float *x = S.sino;
    // twiddles: frequency kk of the tile, samples pw .. pw + 3 of each step
    const int kk = tid & 63, pw = (tid >> 6) * 4;
    const int kg = k0 + kk;
    const bool kval = kg < K;
    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; i++)
#pragma unroll
        for (int j = 0; j < 8; j++)
            acc[i][j] = 0.f;
    float xr[8];
    float2 wr[4];
    auto load = [&](int p0) {
        // (kg p) mod n for p = p0 + pw, then stepped by kg (kg < n, n < 46341)
        unsigned idx = kval ? ((unsigned)kg * (unsigned)(p0 + pw)) % (unsigned)n : 0u;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int p = p0 + pw + j;
            wr[j] = (kval && p < n) ? __ldg(tw + idx) : make_float2(0.f, 0.f);
            idx += (unsigned)kg;
            if (idx >= (unsigned)n)
                idx -= (unsigned)n;
        }
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const int e = tid + 256 * j;
            const int col = e >> 4, p = p0 + (e & 15), gc = c0 + col;
            xr[j] = (gc < cols && p < n) ? __ldg(x + (size_t)gc * n + p) : 0.f;
        }
    };
    load(0);
    for (int p0 = 0; p0 < n; p0 += kDftBK) {
        __syncthreads(); // the previous step is done with Ws / Xs
#pragma unroll
        for (int j = 0; j < 4; j++) {
            Ws[pw + j][2 * kk] = wr[j].x;
            Ws[pw + j][2 * kk + 1] = wr[j].y;
        }
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const int e = tid + 256 * j;
            Xs[e & 15][e >> 4] = xr[j];
        }
        __syncthreads();
        if (p0 + kDftBK < n)
            load(p0 + kDftBK);
#pragma unroll
        for (int q = 0; q < kDftBK; q++) {
            const float4 a0 = *reinterpret_cast<const float4 *>(&Ws[q][ty * 4]);
            const float4 a1 = *reinterpret_cast<const float4 *>(&Ws[q][64 + ty * 4]);
            const float4 b0 = *reinterpret_cast<const float4 *>(&Xs[q][tx * 4]);
            const float4 b1 = *reinterpret_cast<const float4 *>(&Xs[q][64 + tx * 4]);
            const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
            for (int i = 0; i < 8; i++)
#pragma unroll
                for (int j = 0; j < 8; j++)
                    acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
        }
    }
    // epilogue: rows (2f, 2f + 1) of the register tile are (re, im) of one
    // frequency; ck |F / n|^4 summed over the thread's 4 frequencies
    const float invn = 1.f / (float)n;
#pragma unroll
    for (int j = 0; j < 8; j++) {
        float part = 0.f;
#pragma unroll
        for (int f = 0; f < 4; f++) {
            const int freq = k0 + (f < 2 ? 0 : 32) + ty * 2 + (f & 1);
            if (freq < K) {
                const float re = acc[2 * f][j] * invn, im = acc[2 * f + 1][j] * invn;
                const float s2 = re * re + im * im;
                part = fmaf(__ldg(S.ck + freq), s2 * s2, part);
            }
        }
        Red[ty][j < 4 ? tx * 4 + j : 64 + tx * 4 + (j - 4)] = part;
    }
    __syncthreads();
    if (tid < kDftBN) {
        float sum = 0.f;
#pragma unroll
        for (int t = 0; t < 16; t++)
            sum += Red[t][tid];
        const int gc = c0 + tid;
        if (gc < cols)
            S.partial[(size_t)mt * cols + gc] = sum;
    }
}

// P1, P2 and the P3 total of one column per warp (8 columns per CTA).  P2 is
// the weighted selection of tt_select.cuh (no sort) for columns of finite,
// non-negative values; any other column is listed for p2_sort_kernel.
__global__ void __launch_bounds__(256) circus_p12_kernel(const CircusStackArgs a) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int gcol = blockIdx.x * 8 + warp;
    if (gcol >= a.total_cols)
        return; // whole warps only: no CTA-wide barrier below
    const int si = stack_of(a.st, a.n_st, gcol, false);
    const CircusStack &S = stack_at(a, si);
    const int c = gcol - S.col_begin, n = S.n;
    const float *xg = S.sino + (size_t)c * n;
    float *x = reinterpret_cast<float *>(smraw) + (size_t)warp * a.stride;
    SelScratch *sc =
        reinterpret_cast<SelScratch *>(reinterpret_cast<float *>(smraw) + 8 * (size_t)a.stride) +
        warp;
    float lsum = 0.f, lmax = 0.f;
    bool bad = false;
    for (int i = lane; i < n; i += 32) {
        const float v = __ldg(xg + i);
        x[i] = v;
        lsum += v;
        lmax = fmaxf(lmax, v);
        bad |= !(v >= 0.f);
    }
    __syncwarp();
    float v1 = 0.f, v2 = 0.f, v3 = 0.f;
    if (a.need & (1u << 1)) {
        float acc = 0.f;
        for (int p = 1 + lane; p < n; p += 32)
            acc += fabsf(x[p - 1] - x[p]);
        v1 = warp_sum(acc);
    }
    if (a.need & (1u << 2)) {
        const float xsum = warp_sum(lsum);
        const float xmax = __int_as_float(warp_max(__float_as_int(lmax)));
        if (__any_sync(TT_FULL_MASK, bad) || !(xsum < __int_as_float(0x7f800000))) {
            if (lane == 0) {
                const unsigned pos = atomicAdd(a.fb_count, 1u);
                if (pos < (unsigned)a.fb_capacity)
                    a.fb_list[pos] = make_int2(si, c);
            }
        } else {
            v2 = select_p2(x, n, xmax, xsum, sc, lane);
        }
    }
    if (lane == 0) {
        if (a.need & (1u << 3)) {
            float t = 0.f;
            for (int m = 0; m < S.mtiles; m++)
                t += S.partial[(size_t)m * S.cols + c];
            v3 = n > 1 ? t * 0.5f : 0.f;
        }
        const int s = c / S.angles, ang = c - s * S.angles;
        for (int p = 0; p < a.n_p; p++) {
            const int k = a.kind[p];
            if (k < 1 || (k == 2 && bad))
                continue; // written by another kernel (P2: p2_sort_kernel)
            S.out[((size_t)s * a.n_p + p) * S.angles + ang] = k == 1 ? v1 : k == 2 ? v2 : v3;
        }
    }
}

// PFunctional2 by an exact sort for the listed columns (values of any sign:
// the reference sorts and walks the cumulative sum from the first element).
__global__ void __launch_bounds__(kThreads) p2_sort_kernel(const CircusStackArgs a) {
    extern __shared__ __align__(16) float srt[];
    __shared__ float red[kThreads / 32];
    __shared__ int redi[kThreads / 32];
    const unsigned cnt = min(*a.fb_count, (unsigned)a.fb_capacity);
    const int tid = threadIdx.x, bd = blockDim.x;
    for (unsigned e = blockIdx.x; e < cnt; e += gridDim.x) {
        const int2 it = a.fb_list[e];
        const CircusStack &S = stack_at(a, it.x);
        const int n = S.n, c = it.y;
        int P = 1;
        while (P < n)
            P <<= 1;
        const float *xg = S.sino + (size_t)c * n;
        for (int i = tid; i < P; i += bd)
            srt[i] = i < n ? xg[i] : __int_as_float(0x7f800000);
        __syncthreads();
        for (int k = 2; k <= P; k <<= 1) {
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int i = tid; i < P; i += bd) {
                    const int ixj = i ^ j;
                    if (ixj > i) {
                        const float u = srt[i], w = srt[ixj];
                        const bool up = (i & k) == 0;
                        if ((u > w) == up) {
                            srt[i] = w;
                            srt[ixj] = u;
                        }
                    }
                }
                __syncthreads();
            }
        }
        const int per = (n + bd - 1) / bd;
        const int beg = min(tid * per, n), end = min(beg + per, n);
        float loc = 0.f;
        for (int i = beg; i < end; i++)
            loc += srt[i];
        float total;
        float run = block_excl_scan(loc, red, &total);
        int found = INT_MAX;
        for (int i = beg; i < end; i++) {
            run += srt[i];
            if (2.f * run >= total) {
                found = i;
                break;
            }
        }
        found = block_min(found, redi);
        if (tid == 0) {
            const float v = srt[found == INT_MAX ? n - 1 : found];
            const int s = c / S.angles, ang = c - s * S.angles;
            for (int p = 0; p < a.n_p; p++)
                if (a.kind[p] == 2)
                    S.out[((size_t)s * a.n_p + p) * S.angles + ang] = v;
        }
        __syncthreads();
    }
}

} // namespace

size_t circus_smem_bytes(const CircusArgs &a) {
    const bool need_p2 = a.need & (1u << 2), need_p3 = a.need & (1u << 3);
    size_t bytes = (need_p3 ? sizeof(float2) * (size_t)a.M : 0) +
                   sizeof(float) * (size_t)((a.rows + 3) & ~3);
    if (need_p2 || need_p3)
        bytes += sizeof(float) * (size_t)a.sort_len;
    return bytes;
}

cudaError_t launch_circus(const CircusArgs &a, cudaStream_t stream) {
    const size_t limit = opt_in_smem((const void *)circus_kernel);
    if (limit == 0)
        return cudaErrorInvalidValue;
    const size_t smem = circus_smem_bytes(a);
    if (smem > limit)
        return cudaErrorInvalidValue;
    dim3 grid(a.cols, a.n_sino);
    circus_kernel<<<grid, kThreads, smem, stream>>>(a);
    return cudaGetLastError();
}

// Tables of the direct-DFT P3, built on the device so that every path (plans,
// batches, the allocation-free entry point) uses bit-identical values:
// tw[j] = (cos, -sin)(2 pi j / n) from sincospi in double, rounded to float;
// ck[k] = the trapz weight of bin k summed over the positions that read it
// (the reference's mirror reads bin n - p for p > n/2), each position's
// weight (lin[p] - lin[p-1]) + (lin[p+1] - lin[p]) with the reference's
// float linspace (c++/src/functionals.cpp:332-356); P3 = 0.5 sum_k ck |F_k/n|^4.
__global__ void p3_dft_tables_kernel(int n, float2 *__restrict__ tw, float *__restrict__ ck) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) {
        double sv, cv;
        sincospi(2.0 * (double)j / (double)n, &sv, &cv);
        tw[j] = make_float2((float)cv, (float)-sv);
    }
    if (j <= n / 2) {
        double acc = 0.0;
        if (n > 1) {
            auto lin = [n](int p) { return (float)(-1 + p * 2.0 / (n - 1)); };
            const int pos[2] = {j, n - j};
            for (int q = 0; q < 2; q++) {
                const int p = pos[q];
                if (p >= n || (q == 1 && p == j))
                    continue;
                if (p > 0)
                    acc += (double)__fsub_rn(lin(p), lin(p - 1));
                if (p + 1 < n)
                    acc += (double)__fsub_rn(lin(p + 1), lin(p));
            }
        }
        ck[j] = (float)acc;
    }
}

cudaError_t launch_p3_dft_tables(int n, float2 *tw, float *ck, cudaStream_t st) {
    if (n <= 0)
        return cudaSuccess;
    p3_dft_tables_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, tw, ck);
    return cudaGetLastError();
}

int p3_freq_tiles(int n) { return (n / 2 + 1 + kFreqTile - 1) / kFreqTile; }

int circus_warp_stride(int n_max) { return (n_max + 3) & ~3; }

size_t circus_warp_smem_bytes(int n_max) {
    return 8 * (sizeof(float) * (size_t)circus_warp_stride(n_max) + sizeof(SelScratch));
}

cudaError_t launch_circus_stacks(const CircusStackArgs &a, size_t smem, cudaStream_t st) {
    if (a.total_cols <= 0 || a.n_p <= 0)
        return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(a.fb_count, 0, sizeof(unsigned), st);
    if (e != cudaSuccess)
        return e;
    if ((a.need & (1u << 3)) && a.total_tiles > 0) {
        p3_dft_kernel<<<a.total_tiles, 256, 0, st>>>(a);
        if ((e = cudaGetLastError()) != cudaSuccess)
            return e;
    }
    const size_t limit = opt_in_smem((const void *)circus_p12_kernel);
    if (limit == 0 || smem > limit)
        return cudaErrorInvalidValue;
    circus_p12_kernel<<<(a.total_cols + 7) / 8, 256, smem, st>>>(a);
    if ((e = cudaGetLastError()) != cudaSuccess)
        return e;
    if (a.need & (1u << 2)) {
        const size_t sm2 = sizeof(float) * (size_t)a.sort_len_max;
        const size_t lim2 = opt_in_smem((const void *)p2_sort_kernel);
        if (lim2 == 0 || sm2 > lim2)
            return cudaErrorInvalidValue;
        p2_sort_kernel<<<a.fb_grid, kThreads, sm2, st>>>(a);
        e = cudaGetLastError();
    }
    return e;
}

cudaError_t launch_zscore(const float *in, int n_vec, int len, float *out,
                          cudaStream_t stream) {
    if (n_vec <= 0 || len <= 0)
        return cudaSuccess;
    zscore_kernel<<<n_vec, 128, 0, stream>>>(in, len, out);
    return cudaGetLastError();
}

cudaError_t launch_zscore_batch(const float *in, const long long *off, const int *len,
                                int n_vec, float *out, cudaStream_t stream) {
    if (n_vec <= 0)
        return cudaSuccess;
    zscore_batch_kernel<<<n_vec, 128, 0, stream>>>(in, off, len, out);
    return cudaGetLastError();
}

} // namespace tt
