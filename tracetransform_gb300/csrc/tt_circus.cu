// tt_circus.cu -- P-functional (circus) kernels and z-score kernel
// (c++/src/circus.cpp:104-177 with c++/src/functionals.cpp:287-386).
//
// P1-P3 over stacks of sinogram columns (every call without Hermite, and
// the batched engine), three launches:
//   p3_dft_tc_kernel   P3: the real DFT of every column as a GEMM on the
//                      tensor cores (tcgen05, TF32 split in three products,
//                      the accumulator in tensor memory), F = W^T X with
//                      |F_k / N|^4 and the trapz weights folded into the
//                      epilogue (partial sums per 64-frequency tile, added in
//                      tile order: deterministic)
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
// the per-column kernel adds in tile order (deterministic).  W is generated
// from the n-entry twiddle table with an incremental (k p) mod n index.  The
// O(n^2) DFT replaces the Bluestein FFT's two power-of-two transforms in
// shared memory: as a GEMM it runs on the tensor cores, and its error
// (accumulated in FP32 over n terms) stays far inside the 1e-4 tolerance.
constexpr int kFreqTile = 64; // frequencies per partial sum

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

// ---- P3 DFT on the tensor cores (tcgen05, kind::tf32, three products) -------
//
// Per CTA, F^T = X^T W^T for 128 sinogram columns (M: the accumulator's
// tensor memory lanes) x one 64-frequency tile as (re, im) pairs (N <= 128
// tensor memory columns), over the columns' n samples in stages of 32.  TF32
// keeps 10 mantissa bits, so each operand is split x = hi + lo (hi rounded to
// TF32, lo = x - hi exact in FP32) and F sums hi.hi + hi.lo + lo.hi: ~2^-21
// relative per product.  The tensor cores' FP32 accumulation rounds at every
// MMA, and that rounding, not the split, bounds the error: hi.hi goes to
// three accumulators in turn (stage s to accumulator s mod 3) and the small
// cross terms to a fourth, so that each accumulator takes a third of the
// big products' roundings; the epilogue adds the four in FP32.  All 256
// threads stage the operands into shared memory in the canonical K-major
// layout without swizzle, one block per 8-sample MMA slice: core matrices of
// 8 rows x 16 bytes (4 samples), the slice's second 4 samples 128 bytes on
// (LBO), the next 8 rows 256 bytes on (SBO) -- every descriptor stays inside
// its slice's block -- into two stage buffers, each released by the commit
// of the MMAs that read it; one thread issues a stage's 12 MMAs (4 slices x
// 3 products).  The twiddle operand depends only on (n, frequency tile,
// stage): with kPre its hi / lo blocks come precomputed in that layout
// (p3_tc_tables_kernel) and one bulk asynchronous copy per stage brings them
// in, completing on an mbarrier, so that the threads only split and store
// the sinogram operand; without (the allocation-free entry point) the
// threads gather the twiddles from the n-entry table one stage ahead.  The epilogue: warps 0-3 read their 32 lanes' accumulator rows
// (one sinogram column per thread) and fold ck |F/n|^4 into the tile's
// partial sum.  Every wait is bounded: a barrier that never completes (which
// the commit protocol rules out) makes the tile's partial sums NaN instead
// of hanging the GPU.
constexpr int kTcCols = 128, kTcKT = 32, kTcThreads = 256, kTcN = 2 * kFreqTile;
constexpr int kTcAcc = 4; // accumulators of kTcN columns: hi.hi x 3, cross terms
constexpr int kTcAFloats = kTcCols * kTcKT, kTcBFloats = kTcN * kTcKT;
constexpr size_t kTcBufFloats = 2 * (size_t)kTcAFloats + 2 * (size_t)kTcBFloats;
constexpr int kTcRing = 3; // stage buffers
constexpr size_t kTcSmem = kTcRing * kTcBufFloats * sizeof(float); // 192 KB

__device__ __forceinline__ unsigned smem_addr(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}
// x rounded to TF32 (10 mantissa bits); infinities and NaN unchanged
__device__ __forceinline__ float tf32_hi(float x) {
    const unsigned u = __float_as_uint(x);
    return __uint_as_float((u & 0x7f800000u) == 0x7f800000u ? u : (u + 0x1000u) & 0xffffe000u);
}
// Shared-memory matrix descriptor: start, leading (K) and stride (M/N) byte
// offsets in 16-byte units, the descriptor version bit, no swizzle.
__device__ __forceinline__ unsigned long long umma_desc(unsigned addr, unsigned lbo,
                                                        unsigned sbo) {
    return (unsigned long long)((addr & 0x3ffffu) >> 4) |
           ((unsigned long long)((lbo >> 4) & 0x3fffu) << 16) |
           ((unsigned long long)((sbo >> 4) & 0x3fffu) << 32) | (1ull << 46);
}
__device__ __forceinline__ void umma_tf32(unsigned d, unsigned long long a, unsigned long long b,
                                          unsigned idesc, unsigned accumulate) {
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
                 "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
                 : "memory");
}
__device__ __forceinline__ void tmem_ld32(unsigned ta, float (&o)[32]) {
    unsigned v[32];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, "
                 "%8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, "
                 "%22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
                   "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]),
                   "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]),
                   "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
                   "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]),
                   "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                 : "r"(ta));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++)
        o[i] = __uint_as_float(v[i]);
}
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity) {
    for (int it = 0; it < (1 << 22); it++) {
        unsigned ok;
        asm volatile("{\n\t.reg .pred p;\n\t"
                     "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(ok)
                     : "r"(bar), "r"(parity)
                     : "memory");
        if (ok)
            return true;
    }
    return false;
}

// The precomputed twiddle operand of n: for each (64-frequency tile mt,
// stage of 32 samples), a hi block then a lo block of 128 component rows x 32
// samples in the layout the kernel stages (p3_tc_table_floats(n) floats).
__global__ void p3_tc_tables_kernel(int n, const float2 *__restrict__ tw, float *__restrict__ out) {
    const int K = n / 2 + 1, stages = (n + kTcKT - 1) / kTcKT;
    const long long total = (long long)((K + kFreqTile - 1) / kFreqTile) * stages * kTcBFloats;
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= total)
        return;
    const int blk = (int)(e / kTcBFloats), w = (int)(e % kTcBFloats);
    const int mt = blk / stages, st = blk % stages;
    const int row = w / kTcKT, k = w % kTcKT;
    const int f = mt * kFreqTile + (row >> 1), p = st * kTcKT + k;
    float v = 0.f;
    if (f < K && p < n) {
        const float2 t = tw[(int)(((long long)f * p) % n)];
        v = (row & 1) ? t.y : t.x;
    }
    const float hi = tf32_hi(v);
    const int off = (k >> 3) * (kTcN * 8) + (row >> 3) * 64 + ((k >> 2) & 1) * 32 + (row & 7) * 4 + (k & 3);
    float *b = out + (size_t)blk * 2 * kTcBFloats;
    b[off] = hi;
    b[kTcBFloats + off] = v - hi;
}

// grid: one CTA per (64-frequency tile, 128 columns) over the stacks.
// Warp-specialised: warps 0-7 produce the stages into a ring of kTcRing
// buffers (each thread its 16 sinogram samples, hi / lo split and stored;
// with kPre one thread also starts the bulk copy of the twiddle blocks) and
// arrive on the slot's `full` barrier (256 arrivals plus the copy's bytes);
// warp 8 waits on `full`, issues the slot's 12 MMAs and commits them to the
// slot's `empty` barrier, which the producers wait on before refilling it.
// No CTA barrier inside the stage loop: producers run up to kTcRing stages
// ahead of the MMAs.  Warps 0-3 then read the accumulators.
template <bool kPre>
__global__ void __launch_bounds__(kTcThreads + 32, 1) p3_dft_tc_kernel(const CircusStackArgs a) {
    extern __shared__ __align__(1024) float tsm[];
    __shared__ __align__(8) unsigned long long s_full[kTcRing], s_empty[kTcRing], s_done;
    __shared__ unsigned s_tmem;
    const int tile = blockIdx.x;
    const CircusStack &S = stack_at(a, stack_of(a.st, a.n_st, tile, true));
    const int local = tile - S.tile_begin;
    const int mt = local % S.mtiles, ct = local / S.mtiles;
    const int n = S.n, cols = S.cols, K = n / 2 + 1;
    const int k0 = mt * kFreqTile, c0 = ct * kTcCols;
    const int nfreq = min(kFreqTile, K - k0);
    const int N = (2 * nfreq + 15) & ~15;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int stages = (n + kTcKT - 1) / kTcKT;
    constexpr int kMmaWarp = kTcThreads / 32;
    if (warp == kMmaWarp) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_addr(&s_tmem)),
                     "r"((unsigned)(kTcAcc * kTcN))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int i = 0; i < kTcRing; i++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(&s_full[i])),
                         "r"((unsigned)kTcThreads)
                         : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(&s_empty[i])),
                         "r"(1u)
                         : "memory");
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(&s_done)), "r"(1u)
                     : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const unsigned tmem = s_tmem;
    bool ok = true;

    if (warp == kMmaWarp) {
        if (lane == 0) {
            const unsigned idesc = (1u << 4) | (2u << 7) | (2u << 10) |
                                   ((unsigned)(N >> 3) << 17) | ((unsigned)(kTcCols >> 4) << 24);
            const unsigned slice = kTcCols * 32; // bytes per 8-sample block (A and B: 128 rows)
            for (int s = 0; s < stages; s++) {
                const int b = s % kTcRing;
                ok &= mbar_wait(smem_addr(&s_full[b]), (unsigned)(s / kTcRing) & 1u);
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                float *Ahi = tsm + b * kTcBufFloats, *Alo = Ahi + kTcAFloats;
                float *Bhi = Alo + kTcAFloats, *Blo = Bhi + kTcBFloats;
                const unsigned ahi = smem_addr(Ahi), alo = smem_addr(Alo);
                const unsigned bhi = smem_addr(Bhi), blo = smem_addr(Blo);
                const unsigned dbig = tmem + (unsigned)(s % 3) * kTcN, dsmall = tmem + 3u * kTcN;
#pragma unroll
                for (int j = 0; j < kTcKT / 8; j++) {
                    const unsigned long long dah = umma_desc(ahi + j * slice, 128, 256);
                    const unsigned long long dal = umma_desc(alo + j * slice, 128, 256);
                    const unsigned long long dbh = umma_desc(bhi + j * slice, 128, 256);
                    const unsigned long long dbl = umma_desc(blo + j * slice, 128, 256);
                    umma_tf32(dbig, dah, dbh, idesc, (s >= 3 || j > 0) ? 1u : 0u);
                    umma_tf32(dsmall, dah, dbl, idesc, (s > 0 || j > 0) ? 1u : 0u);
                    umma_tf32(dsmall, dal, dbh, idesc, 1u);
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 smem_addr(&s_empty[b]))
                             : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_addr(&s_done))
                         : "memory");
        }
    } else {
        // producers: column / component row r = tid & 127, sample chunks
        // (4 samples) h, h + 2, h + 4, h + 6 of a stage, h = tid / 128
        const int r = tid & 127, h = tid >> 7;
        const int gcol = c0 + r;
        const float *xcol = S.sino + (size_t)min(gcol, cols - 1) * n;
        const bool acol = gcol < cols;
        const int bf = r >> 1, be = r & 1;
        const bool brow = bf < nfreq;
        const unsigned f = (unsigned)(k0 + bf) % (unsigned)n;
        const unsigned f4 = (4u * f) % (unsigned)n, f32 = (32u * f) % (unsigned)n;
        unsigned idx = (f4 * (unsigned)h) % (unsigned)n; // (f p) mod n at p = p0 + 4 h
        float va[16], vb[16];
        auto fetch = [&](int p0) {
            unsigned ib = idx;
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int kq = h + 2 * u;
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const int p = p0 + 4 * kq + e;
                    va[4 * u + e] = acol && p < n ? __ldg(xcol + p) : 0.f;
                    if (!kPre) {
                        float w = 0.f;
                        if (brow && p < n) {
                            const float2 t = __ldg(S.tw + ib);
                            w = be ? t.y : t.x;
                        }
                        vb[4 * u + e] = w;
                    }
                    ib += f;
                    if (ib >= (unsigned)n)
                        ib -= (unsigned)n;
                }
                ib += f4; // skip the other half's 4 samples
                if (ib >= (unsigned)n)
                    ib -= (unsigned)n;
            }
            idx += f32;
            if (idx >= (unsigned)n)
                idx -= (unsigned)n;
        };
        fetch(0);
        for (int s = 0; s < stages; s++) {
            const int b = s % kTcRing;
            float *Ahi = tsm + b * kTcBufFloats, *Alo = Ahi + kTcAFloats;
            float *Bhi = Alo + kTcAFloats, *Blo = Bhi + kTcBFloats;
            float ca[16], cb[16];
#pragma unroll
            for (int i = 0; i < 16; i++) {
                ca[i] = va[i];
                cb[i] = vb[i];
            }
            if (s + 1 < stages)
                fetch((s + 1) * kTcKT);
            if (s >= kTcRing)
                ok &= mbar_wait(smem_addr(&s_empty[b]), (unsigned)(s / kTcRing - 1) & 1u);
            if (kPre && tid == 0) { // the stage's twiddle blocks (hi, lo: contiguous here and there)
                const unsigned bytes = (unsigned)(2 * kTcBFloats * sizeof(float));
                asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(
                                 smem_addr(&s_full[b])),
                             "r"(bytes)
                             : "memory");
                const float *src = S.wtc + ((size_t)mt * stages + s) * 2 * kTcBFloats;
                asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                                 smem_addr(Bhi)),
                             "l"(src), "r"(bytes), "r"(smem_addr(&s_full[b]))
                             : "memory");
            }
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int kq = h + 2 * u;
                const int off = (kq >> 1) * (kTcCols * 8) + (r >> 3) * 64 + (kq & 1) * 32 + (r & 7) * 4;
                const float4 ah = make_float4(tf32_hi(ca[4 * u]), tf32_hi(ca[4 * u + 1]),
                                              tf32_hi(ca[4 * u + 2]), tf32_hi(ca[4 * u + 3]));
                *reinterpret_cast<float4 *>(Ahi + off) = ah;
                *reinterpret_cast<float4 *>(Alo + off) =
                    make_float4(ca[4 * u] - ah.x, ca[4 * u + 1] - ah.y, ca[4 * u + 2] - ah.z,
                                ca[4 * u + 3] - ah.w);
                if (!kPre) {
                    const float4 bh = make_float4(tf32_hi(cb[4 * u]), tf32_hi(cb[4 * u + 1]),
                                                  tf32_hi(cb[4 * u + 2]), tf32_hi(cb[4 * u + 3]));
                    *reinterpret_cast<float4 *>(Bhi + off) = bh;
                    *reinterpret_cast<float4 *>(Blo + off) =
                        make_float4(cb[4 * u] - bh.x, cb[4 * u + 1] - bh.y, cb[4 * u + 2] - bh.z,
                                    cb[4 * u + 3] - bh.w);
                }
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            unsigned long long state;
            asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 %0, [%1];"
                         : "=l"(state)
                         : "r"(smem_addr(&s_full[b]))
                         : "memory");
        }
        // epilogue: warp w < 4 holds columns c0 + 32 w + lane
        if (warp < 4) {
            ok &= mbar_wait(smem_addr(&s_done), 0u);
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const float invn = 1.f / (float)n;
            float part = 0.f;
            const unsigned row = tmem + ((unsigned)(32 * warp) << 16);
            const int chunks = (2 * nfreq + 31) / 32;
            for (int q = 0; q < chunks; q++) {
                float v[32], t[32];
                tmem_ld32(row + 32u * q, v);
                for (int d = 1; d < 4; d++) {
                    if (d < 3 && d >= stages)
                        continue; // an accumulator no stage wrote
                    tmem_ld32(row + (unsigned)d * kTcN + 32u * q, t);
#pragma unroll
                    for (int i = 0; i < 32; i++)
                        v[i] += t[i];
                }
#pragma unroll
                for (int i = 0; i < 16; i++) {
                    const int fl = 16 * q + i;
                    if (fl < nfreq) {
                        const float re = v[2 * i] * invn, im = v[2 * i + 1] * invn;
                        const float s2 = re * re + im * im;
                        part = fmaf(__ldg(S.ck + k0 + fl), s2 * s2, part);
                    }
                }
            }
            const int gc = c0 + 32 * warp + lane;
            if (gc < cols)
                S.partial[(size_t)mt * cols + gc] = ok ? part : __int_as_float(0x7fc00000);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == kMmaWarp) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"((unsigned)(kTcAcc * kTcN))
                     : "memory");
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

size_t p3_tc_table_floats(int n) {
    return (size_t)p3_freq_tiles(n) * ((n + kTcKT - 1) / kTcKT) * 2 * kTcBFloats;
}

cudaError_t launch_p3_tc_tables(int n, const float2 *tw, float *out, cudaStream_t st) {
    const long long total = (long long)p3_tc_table_floats(n) / 2;
    if (n <= 0 || total <= 0)
        return cudaSuccess;
    p3_tc_tables_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(n, tw, out);
    return cudaGetLastError();
}

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
        const void *k = a.tc_tables ? (const void *)p3_dft_tc_kernel<true>
                                    : (const void *)p3_dft_tc_kernel<false>;
        if (opt_in_smem(k) < kTcSmem)
            return cudaErrorInvalidValue;
        if (a.tc_tables)
            p3_dft_tc_kernel<true><<<a.total_tiles, kTcThreads + 32, kTcSmem, st>>>(a);
        else
            p3_dft_tc_kernel<false><<<a.total_tiles, kTcThreads + 32, kTcSmem, st>>>(a);
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
