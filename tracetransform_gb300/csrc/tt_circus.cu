// tt_circus.cu -- P-functional (circus) kernel and z-score kernel.
//
// One CTA per sinogram column (one angle of one sinogram) computes every
// requested P-functional of that column (c++/src/circus.cpp:104-177 with
// c++/src/functionals.cpp:287-386):
//   P1       sum |x[p] - x[p-1]|
//   P2       bitonic sort in shared memory, weighted median of the sorted
//            column weighted by itself
//   P3       DFT of the real column by the chirp-z (Bluestein) identity on a
//            power-of-two shared-memory FFT, then trapz(linspace(-1, 1),
//            (|F_p| / N)^4) with the reference's mirror for p > N/2
//   Hermite  projection on a host-built basis psi_order(z(p)) (the basis is
//            evaluated on the host exactly as hermite_function does)
// zscore_kernel follows c++/src/auxiliary.cpp:277-318 in the reference's own
// order: a float mean, a double sum of squared float differences, n - 1.
#include <climits>

#include "tt_common.cuh"
#include "tt_internal.h"

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
            a.out[((size_t)sidx * a.n_p + p) * a.cols + colidx] = res[p];
    }
}

__global__ void __launch_bounds__(kThreads) circus_kernel(const CircusArgs a) {
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ float red[kThreads / 32];
    __shared__ int redi[kThreads / 32];
    circus_column(a, blockIdx.y, blockIdx.x, smraw, red, redi);
}

// Batched P-stage: block b handles one column of one sinogram of one image;
// images differ in sinogram length (rows), angle count (cols) and tables.
__global__ void __launch_bounds__(kThreads) circus_batch_kernel(const BatchCircusArgs b) {
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ float red[kThreads / 32];
    __shared__ int redi[kThreads / 32];
    const int blk = blockIdx.x;
    int lo = 0, hi = b.n_img - 1; // image whose column range holds blk
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (b.img[mid].col_begin <= blk)
            lo = mid;
        else
            hi = mid - 1;
    }
    const BatchCircusImage im = b.img[lo];
    const int k = blk - im.col_begin; // = sinogram * cols + column
    CircusArgs a{};
    a.sino = b.sino + im.sino_off;
    a.rows = im.rows;
    a.cols = im.cols;
    a.n_sino = b.n_sino;
    a.n_p = b.n_p;
    for (int p = 0; p < b.n_p; p++)
        a.kind[p] = b.kind[p];
    a.chirp = b.tables + im.chirp_off;
    a.filt = b.tables + im.filt_off;
    a.twid = b.tables + im.twid_off;
    a.lin = b.lin + im.lin_off;
    a.M = im.M;
    a.sort_len = im.sort_len;
    a.need = b.need;
    a.out = b.out + im.out_off;
    circus_column(a, k / im.cols, k % im.cols, smraw, red, redi);
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

cudaError_t launch_zscore(const float *in, int n_vec, int len, float *out,
                          cudaStream_t stream) {
    if (n_vec <= 0 || len <= 0)
        return cudaSuccess;
    zscore_kernel<<<n_vec, 128, 0, stream>>>(in, len, out);
    return cudaGetLastError();
}

cudaError_t prepare_circus_batch(size_t smem) {
    const size_t limit = opt_in_smem((const void *)circus_batch_kernel);
    if (limit == 0)
        return cudaErrorInvalidValue;
    return smem > limit ? cudaErrorInvalidValue : cudaSuccess;
}

cudaError_t launch_circus_batch(const BatchCircusArgs &a, int blocks, size_t smem,
                                cudaStream_t stream) {
    if (blocks <= 0)
        return cudaSuccess;
    circus_batch_kernel<<<blocks, kThreads, smem, stream>>>(a);
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
