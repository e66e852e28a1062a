// tt_nos.cu -- nearest orthonormal sinogram on the device.
//
// The reference's orthonormal mode (c++/src/circus.cpp:68-102) shifts every
// sinogram column by its weighted-median offset into an m x A matrix
// (m = N + padding) and replaces it by the polar factor U V^T of its SVD,
// computed by Eigen's float JacobiSVD with a column-pivoting Householder QR
// preconditioner.  Here, for n_sino sinograms at once, the same structure
// with the precision split that GB300's rates call for: no FP64 at all
// (its pipe is narrow enough that a few scalar FP64 operations per step
// dominate), double-float pairs on the FP32 pipes where float is too short:
//
//   nos_offsets   per column: weighted median row - center, with the
//                 reference's sequential float sums (one thread per column)
//   nos_align     the shifted columns into a zeroed m x A matrix of
//                 double-float pairs (hi + lo, ~48 significant bits)
//   QR            column-pivoting Householder QR, A P = Q R, in double-float
//                 (the only stage beyond float precision: it fixes the small
//                 singular directions that a float factorisation would lose;
//                 the O(m A) work per step runs on the FP32 pipes); one
//                 launch per column step, in which every CTA picks the pivot
//                 itself and applies the reflector to its own columns,
//                 LAPACK-style otherwise (tau, partial column norms downdated
//                 and recomputed when cancellation sets in)
//   Jacobi        one-sided Jacobi on X = R^T in float (R^T of a pivoted QR is
//                 graded, so float rotations keep relative accuracy), block-
//                 cyclic: round-robin rounds of 12-column block pairs, each
//                 pair rotated in one CTA's shared memory with V updated once
//                 per round through the accumulated rotation;
//                 X V = U_X S, so polar(R) = V U_X^T
//   assemble      P = V U_X^T (float) with one Newton-Schulz step to clean
//                 its orthogonality, then polar(A P) = Q [P; 0] applied
//                 reflector by reflector to groups of columns held in
//                 registers (up to 4096 aligned rows) or by blocks of 32
//                 reflectors in compact-WY form (above), straight into the
//                 result columns, which undoes the column permutation
//
// Against the oracle's double one-sided Jacobi on the aligned matrix the
// result agrees to ~3e-5 absolute (entries up to ~0.7) for condition numbers
// up to ~1e6; Eigen's float SVD of the same matrices is far less accurate.
// Every launch is bounded; there is no grid-wide wait.
#include "tt_common.cuh"
#include "tt_internal.h"

namespace tt {
namespace {

__global__ void nos_offsets_kernel(const float *__restrict__ sino, int rows, int n_cols,
                                   int center, int *__restrict__ offsets) {
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (idx >= n_cols)
        return;
    const float *x = sino + (size_t)idx * rows;
    float sum = 0.f;
    for (int i = 0; i < rows; i++)
        sum = __fadd_rn(sum, x[i]);
    float integral = 0.f;
    int m = rows - 1;
    for (int i = 0; i < rows; i++) {
        integral = __fadd_rn(integral, x[i]);
        if (2.f * integral >= sum) {
            m = i;
            break;
        }
    }
    offsets[idx] = m - center;
}

// ---- double-float arithmetic -------------------------------------------------
//
// The aligned matrices hold each element as an unevaluated sum hi + lo of two
// floats (~48 significant bits).  The QR's O(m n) work -- dot products and
// trailing updates -- runs on these pairs with error-free float transforms
// (Knuth's two-sum, the FMA two-product, Dekker's renormalisation; the
// products that feed a two-sum are __fmul_rn, which the compiler never
// contracts into a fused multiply-add), i.e. on
// the FP32 pipes, which GB300 runs far faster than FP64; so do the scalars
// (norms, reflector coefficients, with double-float division and square
// root): a handful of FP64 operations per column step, each waiting on the
// narrow FP64 pipe, cost more than the step's O(m n) double-float work.

__device__ __forceinline__ float2 df_quick(float a, float b) { // |a| >= |b|
    const float s = a + b;
    return make_float2(s, b - (s - a));
}
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
    const float s = a.x + b.x, bb = s - a.x;
    const float e = (a.x - (s - bb)) + (b.x - bb);
    return df_quick(s, e + a.y + b.y);
}
__device__ __forceinline__ float2 df_mul(float2 a, float2 b) {
    const float p = __fmul_rn(a.x, b.x); // never contracted into a later add
    float e = fmaf(a.x, b.x, -p);
    e = fmaf(a.x, b.y, e);
    e = fmaf(a.y, b.x, e);
    return df_quick(p, e);
}
// acc + a b with the product's rounding error carried into the low word
// instead of renormalising the product first
__device__ __forceinline__ float2 df_fma(float2 a, float2 b, float2 acc) {
    const float p = __fmul_rn(a.x, b.x); // never contracted into a later add
    float e = fmaf(a.x, b.x, -p);
    e = fmaf(a.x, b.y, e);
    e = fmaf(a.y, b.x, e);
    const float s = acc.x + p, bb = s - acc.x;
    const float err = (acc.x - (s - bb)) + (p - bb);
    return df_quick(s, err + e + acc.y);
}
// Compensated dot product of double-float vectors (Ogita, Rump and Oishi's
// Dot2, extended by the low-word cross terms): the high words' products go
// into s with Knuth's two-sum, whose errors, the products' FMA rounding
// errors and the cross terms collect in e; only s + p is on the dependent
// path per element.  df_dot_end renormalises.
struct DfDot {
    float s = 0.f, e = 0.f;
};
__device__ __forceinline__ void df_dot_add(DfDot &d, float2 a, float2 b) {
    const float p = __fmul_rn(a.x, b.x); // never contracted into a later add
    const float pe = fmaf(a.x, b.x, -p);
    const float t = d.s + p, bb = t - d.s;
    const float err = (d.s - (t - bb)) + (p - bb);
    d.e += (err + pe) + fmaf(a.x, b.y, a.y * b.x);
    d.s = t;
}
__device__ __forceinline__ float2 df_dot_end(DfDot d) { return df_quick(d.s, d.e); }
__device__ __forceinline__ float2 df_neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 df_sub(float2 a, float2 b) { return df_add(a, df_neg(b)); }
// a / b: float quotient, corrected once by the double-float remainder
__device__ __forceinline__ float2 df_div(float2 a, float2 b) {
    const float q1 = a.x / b.x;
    const float2 r = df_sub(a, df_mul(make_float2(q1, 0.f), b));
    return df_quick(q1, r.x / b.x);
}
// sqrt(a), a >= 0: float root, corrected once by the double-float residual
__device__ __forceinline__ float2 df_sqrt(float2 a) {
    if (!(a.x > 0.f))
        return make_float2(0.f, 0.f);
    const float r0 = sqrtf(a.x);
    const float2 res = df_sub(a, df_mul(make_float2(r0, 0.f), make_float2(r0, 0.f)));
    return df_quick(r0, res.x / (2.f * r0));
}
__device__ __forceinline__ float2 df_shfl_xor(float2 v, int o) {
    return make_float2(__shfl_xor_sync(TT_FULL_MASK, v.x, o),
                       __shfl_xor_sync(TT_FULL_MASK, v.y, o));
}

// grid (cols, n_sino); A_s must be zeroed before.
__global__ void nos_align_kernel(const float *__restrict__ sino, int rows, int cols,
                                 const NosDesc *__restrict__ desc,
                                 const int *__restrict__ offsets, float2 *__restrict__ A) {
    const int col = blockIdx.x, s = blockIdx.y;
    const NosDesc d = desc[s];
    const int shift = d.mx - offsets[(size_t)s * cols + col];
    const float *src = sino + ((size_t)s * cols + col) * rows;
    float2 *dst = A + d.a_off + (size_t)col * d.m + shift;
    for (int r = threadIdx.x; r < rows; r += blockDim.x)
        dst[r] = make_float2(src[r], 0.f);
}

template <int kThreads> __device__ __forceinline__ float2 block_sum_df(float2 v, float2 *red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v = df_add(v, df_shfl_xor(v, o));
    if (lane == 0)
        red[warp] = v;
    __syncthreads();
    float2 t = red[0];
#pragma unroll
    for (int w = 1; w < kThreads / 32; w++)
        t = df_add(t, red[w]);
    __syncthreads();
    return t;
}

// ---- column-pivoting Householder QR (double-float) ---------------------------

constexpr int kQrThreads = 256;

// Squared column norms (partial, by position, in the step-0 half of the
// double buffer, double-float; and the reference copy, by stored column,
// float) and the identity position map.  grid (n, n_sino).
__global__ void __launch_bounds__(kQrThreads)
qr_init_kernel(const float2 *__restrict__ A, const NosDesc *__restrict__ desc, int n,
               NosWork w) {
    __shared__ float2 red[kQrThreads / 32];
    const int j = blockIdx.x, s = blockIdx.y;
    const NosDesc d = desc[s];
    const float2 *a = A + d.a_off + (size_t)j * d.m;
    float2 v = make_float2(0.f, 0.f);
    for (int i = threadIdx.x; i < d.m; i += kQrThreads)
        v = df_fma(a[i], a[i], v);
    v = block_sum_df<kQrThreads>(v, red);
    if (threadIdx.x == 0) {
        w.norms[(size_t)s * n + j] = v;
        w.orig[(size_t)s * n + j] = v.x;
        w.cmap[(size_t)s * n + j] = j;
    }
}

// Most positions one CTA of the column step handles.
constexpr int kQrMaxCols = 64;

// Warp-then-block double-float sum through red[T / 32]; one barrier.
// Consecutive calls must alternate between two red buffers.
template <int T> __device__ __forceinline__ float2 qr_block_sum(float2 v, float2 *red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v = df_add(v, df_shfl_xor(v, o));
    if (lane == 0)
        red[warp] = v;
    __syncthreads();
    v = red[0];
#pragma unroll
    for (int u = 1; u < T / 32; u++)
        v = df_add(v, red[u]);
    return v;
}

// Column step k of the pivoted QR in one launch, grid (G, n_sino): CTA b
// handles positions k + b, k + b + G, ... (G is chosen so that the grid is one
// wave, and each CTA prefetches its next column while it reduces the current
// one).
//
// Every CTA picks the pivot itself -- the remaining position of largest
// partial norm, lowest position on ties -- and reads the pivot column
// x = A[k:, c_p].  The CTA owning position p stores the reflector's scalars
// (beta = R[k, k], scale = 1 / (alpha - beta), tau); every other column gets
// H = I - tau v v^T, v = (1, x[k+1:] scale), in place, with
// v . a = a[k] + scale (x[k+1:] . a[k+1:]), and then its partial norm loses
// a[k]^2 (recomputed from the column when that leaves less than ~sqrt(eps)
// of the norm at the last recompute, as LAPACK does).
//
// Columns never move: cmap maps positions to stored columns and the pivot
// swap exchanges two of its entries.  The pivot column is left as it is (its
// rows above k are R[:k, k], those below k the reflector up to `scale`), so
// no CTA writes what another reads in the same step; the partial norms (by
// position) and cmap are double-buffered by step parity.  perm[k] receives
// the stored column that ends at position k.
//
// Element slots: thread t holds rows k + 1 + t + kQrThreads u (u < K, K kQrThreads >=
// m) of a column in registers, so each column is read once with all loads in
// flight and written once.  Sums, updates and scalars are all double-float;
// the scalars are computed by one lane per warp.
// At 16 rows per thread and 128 threads the next column is not prefetched:
// that leaves 96 registers and 5 CTAs per SM instead of 128 and 4 (at
// 8 x 1843 x 360: 4.32 against 4.50 ms for the 360 steps, same results).
template <int K, int T>
__global__ void __launch_bounds__(T, K == 32                ? 1
                                     : K == 16 && T == 128 ? 5
                                                           : 512 / T) // no spills below K = 32
qr_step_kernel(float2 *__restrict__ A, const NosDesc *__restrict__ desc, int n, int n_sino,
               int k, NosWork w) {
    constexpr int kW = T / 32;
    constexpr bool kPrefetch = K <= 12 || (K == 16 && T == 256); // registers for a second column
    __shared__ int s_bv[kW];
    __shared__ int s_bi[kW];
    __shared__ float2 s_red[2][kW];
    __shared__ float2 s_red2[kW];
    __shared__ int s_col[kQrMaxCols];
    __shared__ float2 s_nr[kQrMaxCols];
    __shared__ float s_og[kQrMaxCols];
    const int s = blockIdx.y, G = gridDim.x, b = blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const NosDesc d = desc[s];
    const int m = d.m;
    // slot (t, u) of a column holds row k + 1 + t + T u; keff slots
    // cover the rows below the diagonal
    const int keff = (m - k - 1 + T - 1) / T;
    float2 *As = A + d.a_off;
    const size_t cur = (size_t)(k & 1) * n_sino + s, nxt = (size_t)((k + 1) & 1) * n_sino + s;
    const float2 *nr = w.norms + cur * n;
    const int *cm = w.cmap + cur * n;
    const int j0 = k + b;
    const int cnt = min((n - j0 + G - 1) / G, kQrMaxCols);
    // per own column: stored column, partial norm and recompute threshold
    for (int t = threadIdx.x; t < cnt; t += T) {
        const int c = cm[j0 + t * G];
        s_col[t] = c;
        s_nr[t] = nr[j0 + t * G];
        s_og[t] = w.orig[(size_t)s * n + c];
    }

    // first own column, loaded while the pivot is chosen
    const int c0 = cm[j0];
    float2 cv[K];
    {
        const float2 *c = As + (size_t)c0 * m;
#pragma unroll
        for (int u = 0; u < K; u++) {
            const int i = k + 1 + threadIdx.x + T * u;
            cv[u] = u < keff && i < m ? c[i] : make_float2(0.f, 0.f);
        }
    }
    float2 ck = As[(size_t)c0 * m + k];

    // pivot: argmax of the partial norms over positions k..n-1, compared as
    // the bit patterns of their (non-negative) high words on the integer
    // pipe; a NaN or negative norm counts as 0
    int best = -1;
    int bidx = n;
    for (int jj = k + threadIdx.x; jj < n; jj += T) {
        int v = __float_as_int(nr[jj].x);
        if (v < 0 || v > 0x7F800000)
            v = 0;
        if (v > best) { // positions rise per thread: the first maximum stays
            best = v;
            bidx = jj;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const int ov = __shfl_xor_sync(TT_FULL_MASK, best, o);
        const int oi = __shfl_xor_sync(TT_FULL_MASK, bidx, o);
        if (ov > best || (ov == best && oi < bidx)) {
            best = ov;
            bidx = oi;
        }
    }
    if (lane == 0) {
        s_bv[warp] = best;
        s_bi[warp] = bidx;
    }
    __syncthreads(); // also publishes s_col
    best = s_bv[0];
    bidx = s_bi[0];
#pragma unroll
    for (int u = 1; u < kW; u++)
        if (s_bv[u] > best || (s_bv[u] == best && s_bi[u] < bidx)) {
            best = s_bv[u];
            bidx = s_bi[u];
        }
    const int p = bidx < n ? bidx : k;
    const int cp = cm[p];
    const float2 *x = As + (size_t)cp * m;
    float2 xv[K];
#pragma unroll
    for (int u = 0; u < K; u++) {
        const int i = k + 1 + threadIdx.x + T * u;
        xv[u] = u < keff && i < m ? x[i] : make_float2(0.f, 0.f);
    }
    const float2 xk = x[k];

    // |x[k+1:]|^2 and, for the first own column, x[k+1:] . a[k+1:]
    float2 xn, xa;
    {
        DfDot dn[2], da[2];
#pragma unroll
        for (int u = 0; u < K; u++)
            if (u < keff) {
                df_dot_add(dn[u & 1], xv[u], xv[u]);
                df_dot_add(da[u & 1], xv[u], cv[u]);
            }
        xn = df_add(df_dot_end(dn[0]), df_dot_end(dn[1]));
        xa = df_add(df_dot_end(da[0]), df_dot_end(da[1]));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        xn = df_add(xn, df_shfl_xor(xn, o));
        xa = df_add(xa, df_shfl_xor(xa, o));
    }
    if (lane == 0) {
        s_red[0][warp] = xn;
        s_red2[warp] = xa;
    }
    __syncthreads();
    xn = s_red[0][0];
    xa = s_red2[0];
#pragma unroll
    for (int u = 1; u < kW; u++) {
        xn = df_add(xn, s_red[0][u]);
        xa = df_add(xa, s_red2[u]);
    }
    int rb = 1; // s_red[rb] is the next free reduction buffer
    const bool zero = xn.x == 0.f; // uniform: H = I, x stays as it is

    // reflector scalars (double-float, no FP64: GB300's FP64 pipe would
    // serialise them) by lane 0 of each warp, broadcast by shuffle
    float2 scale_df = make_float2(0.f, 0.f), tau_df = make_float2(0.f, 0.f);
    if (lane == 0) {
        float2 beta = xk;
        if (!zero) {
            const float2 root = df_sqrt(df_fma(xk, xk, xn));
            beta = xk.x >= 0.f ? df_neg(root) : root;
            scale_df = df_div(make_float2(1.f, 0.f), df_sub(xk, beta));
            tau_df = df_div(df_sub(beta, xk), beta);
        }
        if (warp == 0 && (p - k) % G == b) {
            const size_t o = (size_t)s * n + k;
            w.beta[o] = beta;
            w.scale[o] = scale_df;
            w.tau[o] = tau_df;
            w.perm[o] = cp;
        }
    }
    scale_df = make_float2(__shfl_sync(TT_FULL_MASK, scale_df.x, 0),
                           __shfl_sync(TT_FULL_MASK, scale_df.y, 0));
    tau_df = make_float2(__shfl_sync(TT_FULL_MASK, tau_df.x, 0),
                         __shfl_sync(TT_FULL_MASK, tau_df.y, 0));
    float *og = w.orig + (size_t)s * n;

    for (int t = 0; t < cnt; t++) {
        const int j = j0 + t * G, cj = s_col[t];
        float2 cn[kPrefetch ? K : 1];
        float2 ckn = make_float2(0.f, 0.f);
        if (kPrefetch && t + 1 < cnt) {
            const float2 *c = As + (size_t)s_col[t + 1] * m;
#pragma unroll
            for (int u = 0; u < (kPrefetch ? K : 1); u++) {
                const int i = k + 1 + threadIdx.x + T * u;
                cn[u] = u < keff && i < m ? c[i] : make_float2(0.f, 0.f);
            }
            ckn = c[k];
        }
        if (j != p) { // uniform
            float2 *c = As + (size_t)cj * m;
            if (t > 0) {
                DfDot dv[2];
#pragma unroll
                for (int u = 0; u < K; u++)
                    if (u < keff)
                        df_dot_add(dv[u & 1], xv[u], cv[u]);
                xa = qr_block_sum<T>(df_add(df_dot_end(dv[0]), df_dot_end(dv[1])), s_red[rb]);
                rb ^= 1;
            }
            if (!zero) {
                // a -= tau v (v . a), v . a = a[k] + scale (x[k+1:] . a[k+1:])
                const float2 vc = df_add(ck, df_mul(scale_df, xa));
                const float2 ntw = df_neg(df_mul(tau_df, vc));
                const float2 ntws = df_mul(ntw, scale_df);
#pragma unroll
                for (int u = 0; u < K; u++) {
                    const int i = k + 1 + threadIdx.x + T * u;
                    if (u < keff)
                        cv[u] = df_fma(ntws, xv[u], cv[u]);
                    if (u < keff && i < m)
                        c[i] = cv[u];
                }
                ck = df_add(ck, ntw);
                if (threadIdx.x == 0)
                    c[k] = ck;
            }
            // partial norm for step k + 1, decided by lane 0 of each warp
            float2 n2 = make_float2(0.f, 0.f);
            int recompute = 0;
            if (lane == 0) {
                n2 = df_sub(s_nr[t], df_mul(ck, ck));
                recompute = n2.x <= 1.5e-8f * s_og[t];
            }
            if (__shfl_sync(TT_FULL_MASK, recompute, 0)) { // uniform
                DfDot dr[2];
#pragma unroll
                for (int u = 0; u < K; u++)
                    if (u < keff)
                        df_dot_add(dr[u & 1], cv[u], cv[u]);
                const float2 r = qr_block_sum<T>(df_add(df_dot_end(dr[0]), df_dot_end(dr[1])), s_red[rb]);
                rb ^= 1;
                n2 = r;
                if (threadIdx.x == 0)
                    og[cj] = n2.x;
            }
            if (threadIdx.x == 0) {
                const int dest = j == k ? p : j;
                w.norms[nxt * n + dest] = n2;
                w.cmap[nxt * n + dest] = cj;
            }
        }
        if (t + 1 < cnt) {
            if (kPrefetch) {
#pragma unroll
                for (int u = 0; u < (kPrefetch ? K : 1); u++)
                    cv[u] = cn[u];
                ck = ckn;
            } else {
                const float2 *c = As + (size_t)s_col[t + 1] * m;
#pragma unroll
                for (int u = 0; u < K; u++) {
                    const int i = k + 1 + threadIdx.x + T * u;
                    cv[u] = u < keff && i < m ? c[i] : make_float2(0.f, 0.f);
                }
                ck = c[k];
            }
        }
    }
}

// ---- one-sided Jacobi on X = R^T (float) ----------------------------------

// Directions of R whose norm is below kNullRel |R[0, 0]| (|R[0, 0]| is the
// largest column norm of the aligned matrix) are below the double precision
// of the input: they take no rotations and no part in U, as the oracle
// treats exactly-zero directions.
constexpr float kNullRel = 1e-15f;

// X[i + j n] = R[j, i] (upper triangle of the QR result), V = I, and the
// null-direction bound tiny[s] = (kNullRel R[0, 0])^2.
// grid (ceil(n * n / 256), n_sino).
__global__ void nos_rt_kernel(const float2 *__restrict__ A, const NosDesc *__restrict__ desc,
                              int n, NosWork w) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long nn = (long long)n * n;
    if (e >= nn)
        return;
    const int s = blockIdx.y, i = (int)(e % n), j = (int)(e / n);
    const NosDesc d = desc[s];
    const float2 *beta = w.beta + (size_t)s * n;
    if (e == 0) {
        const float r = kNullRel * (beta[0].x + beta[0].y);
        w.tiny[s] = r * r;
    }
    // R[j, i]: the diagonal from beta, above it the stored column of position i
    float r = 0.f;
    if (j == i)
        r = beta[i].x + beta[i].y;
    else if (j < i) {
        const float2 a = A[d.a_off + j + (size_t)w.perm[(size_t)s * n + i] * d.m];
        r = a.x + a.y;
    }
    w.X[s * nn + e] = r;
    w.V[s * nn + e] = i == j ? 1.f : 0.f;
}

// A pair is rotated when |x_p . x_q| > kJacTol |x_p| |x_q| -- a few times the
// rounding of a float dot product over n terms split across a warp -- and a
// sweep that rotates none (or whose largest rotated pair is below
// kJacDone) ends the iteration.  Near convergence the cyclic method is
// quadratic (measured at 1449 x 360: 7.6e-4, 2.1e-5, then 1.0e-6, the float
// floor), so a sweep whose largest rotated cosine is below 1e-4 leaves every
// pair at that floor and the next sweep would only confirm it.
constexpr float kJacTol = 1e-6f, kJacDone = 1e-4f;

// Two-level (block) Jacobi.  The n columns form blocks of kBJ, and a sweep
// visits every column pair once, in nbp - 1 launches (rounds of a
// round-robin tournament of the nbp blocks, a dummy block making nbp even):
// in each round a CTA copies its block pair -- 2 kBJ columns of X -- into
// shared memory and rotates the kBJ^2 pairs across the two blocks in kBJ
// inner rounds of kBJ disjoint pairs (one warp per pair, __syncthreads
// between inner rounds); the first round of a sweep first rotates the pairs
// inside each of its two blocks (kBJ - 1 more inner rounds).  A block-cyclic
// ordering of the cyclic Jacobi method.
//
// V does not take part in the inner rounds: their rotations are accumulated
// into a 2 kBJ x 2 kBJ orthogonal J (in shared memory), and the block's
// columns of V are multiplied by J once per round, in row chunks staged
// through shared memory.  Columns sit in shared memory zero-padded to a
// multiple of 128 rows, so a lane moves 4 consecutive rows per 128-bit
// access and no row needs a bounds test.  Blocks of 12 (measured at 8
// sinograms of 1449 x 360 and 5795 x 720: 11 % and 29 % faster sweeps than
// blocks of 16, whose inner rounds are longer; blocks of 8 took one sweep
// more) give a round of 8 x 360-angle sinograms 120 CTAs.
constexpr int kBJ = 12, kBCols = 2 * kBJ, kBThreads = 32 * kBJ;
constexpr int kVRows = 256; // rows of V per chunk: 64 groups of 4 rows x kBCols / 4 of 4 columns
static_assert(kBJ % 2 == 0 && kBCols <= 32, "whole pairs per block; a J row per lane");
static_assert(kBThreads == (kVRows / 4) * (kBCols / 4), "one 4 x 4 tile of V J per thread");

__device__ __forceinline__ void round_robin(int players, int round, int k, int &p, int &q) {
    const int P1 = players - 1;
    if (k == 0) {
        p = P1;
        q = round;
    } else {
        p = (round + k) % P1;
        q = (round - k + P1) % P1;
    }
    if (p > q) {
        const int t = p;
        p = q;
        q = t;
    }
}

// The V block sits whole in shared memory up to 4 slots of 128 rows; larger
// ones go through a kVRows chunk.
__host__ __device__ constexpr bool block_round_whole_v(int k4) { return k4 <= 4; }

// Dynamic shared memory of the round kernel with K4 slots of 128 rows
// (floats): the X block, the V block (or chunk, leading dimension rows + 4)
// and the two copies of J.
__host__ __device__ constexpr size_t block_round_smem_floats(int k4) {
    return (size_t)kBCols * 128 * k4 +
           (size_t)kBCols * ((block_round_whole_v(k4) ? 128 * k4 : kVRows) + 4) +
           kBCols * (kBCols + 1) + kBCols * kBCols;
}

__device__ __forceinline__ float4 f4_lin(float a, float4 x, float b, float4 y) {
    return make_float4(a * x.x + b * y.x, a * x.y + b * y.y, a * x.z + b * y.z, a * x.w + b * y.w);
}

// 4-byte asynchronous global -> shared copy; src_bytes 0 writes a zero
// without reading src.
__device__ __forceinline__ void cp_async4(float *dst, const float *src, int src_bytes) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(src),
                 "r"(src_bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
    asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N> __device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// 16-byte asynchronous copy of src_bytes (0 or 16) bytes, zero-filling the rest.
__device__ __forceinline__ void cp_async16(float *dst, const float *src, int src_bytes) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(src),
                 "r"(src_bytes)
                 : "memory");
}

// Rows [r0, r0 + rows) of the 2 kBJ columns of the block (global column
// gcol(c), none past n) into a shared column-major block with leading
// dimension ld, zero-filled past n, as asynchronous copies: warp w takes
// local columns w and w + kBJ, its lanes consecutive rows -- 16 bytes at a
// time when n is a multiple of 4 (every column then starts 16-byte
// aligned, given a 16-byte aligned matrix), else 4.  rows and r0 are
// multiples of 4.
template <typename G>
__device__ __forceinline__ void stage_cols_async(float *dst, int ld, const float *src, int n,
                                                 int r0, int rows, G gcol) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool vec = (n & 3) == 0 && ((uintptr_t)src & 15) == 0;
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int c = warp + kBJ * h, gc = gcol(c);
        float *d = dst + (size_t)c * ld;
        const float *g = src + (size_t)(gc < n ? gc : 0) * n;
        if (vec) {
            for (int q = lane; q < rows / 4; q += 32) {
                const int r = r0 + 4 * q;
                const bool ok = gc < n && r < n;
                cp_async16(d + 4 * q, ok ? g + r : src, ok ? 16 : 0);
            }
        } else {
            for (int q = lane; q < rows; q += 32) {
                const int r = r0 + q;
                const bool ok = gc < n && r < n;
                cp_async4(d + q, ok ? g + r : src, ok ? 4 : 0);
            }
        }
    }
}

// The inverse of stage_cols_async (plain stores, none past n).
template <typename G>
__device__ __forceinline__ void store_cols(float *dst, const float *sm, int ld, int n, int r0,
                                           int rows, G gcol) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool vec = (n & 3) == 0 && ((uintptr_t)dst & 15) == 0;
    const int lim = min(rows, n - r0); // rows of the block inside the matrix
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int c = warp + kBJ * h, gc = gcol(c);
        if (gc >= n)
            continue;
        const float *l = sm + (size_t)c * ld;
        float *g = dst + (size_t)gc * n + r0;
        if (vec) {
            for (int q = lane; 4 * q < lim; q += 32)
                *reinterpret_cast<float4 *>(g + 4 * q) = *reinterpret_cast<const float4 *>(l + 4 * q);
        } else {
            for (int q = lane; q < lim; q += 32)
                g[q] = l[q];
        }
    }
}

// One Jacobi rotation of the column pair (x, y) held by a warp (lane l
// holds rows 4 l + 128 u .. + 3): cos of the pair = |x . y| / (|x| |y|);
// rotated (x and y replaced) unless a column is null (norm^2 <= tn, or a zero
// column past n) or the pair is already orthogonal to kJacTol.  The
// rotation parameters come from the (2-ulp) hardware reciprocal square root:
// the rotation only has to be orthogonal (c^2 + s^2 = 1 to float precision),
// not exact.  Returns the pair's cos when rotated, else 0.
template <int K4>
__device__ __forceinline__ float jacobi_pair(float4 (&x)[K4], float4 (&y)[K4], float tn,
                                             float &c, float &sn) {
    float al = 0.f, be = 0.f, ga = 0.f;
#pragma unroll
    for (int u = 0; u < K4; u++) {
        al = fmaf(x[u].x, x[u].x, al);
        be = fmaf(y[u].x, y[u].x, be);
        ga = fmaf(x[u].x, y[u].x, ga);
        al = fmaf(x[u].y, x[u].y, al);
        be = fmaf(y[u].y, y[u].y, be);
        ga = fmaf(x[u].y, y[u].y, ga);
        al = fmaf(x[u].z, x[u].z, al);
        be = fmaf(y[u].z, y[u].z, be);
        ga = fmaf(x[u].z, y[u].z, ga);
        al = fmaf(x[u].w, x[u].w, al);
        be = fmaf(y[u].w, y[u].w, be);
        ga = fmaf(x[u].w, y[u].w, ga);
    }
    al = warp_sum(al);
    be = warp_sum(be);
    ga = warp_sum(ga);
    const float cosv = fabsf(ga) * (rsqrtf(al) * rsqrtf(be));
    if (!(al > tn && be > tn && ga != 0.f && cosv > kJacTol))
        return 0.f; // uniform across the warp
    const float zeta = __fdividef(be - al, 2.f * ga);
    const float az = fabsf(zeta);
    float t;
    if (az < 1e15f) {
        const float z2 = fmaf(zeta, zeta, 1.f);
        t = __fdividef(1.f, az + z2 * rsqrtf(z2));
    } else {
        t = __fdividef(0.5f, az);
    }
    t = zeta >= 0.f ? t : -t;
    c = rsqrtf(fmaf(t, t, 1.f));
    sn = c * t;
#pragma unroll
    for (int u = 0; u < K4; u++) {
        const float4 xo = x[u];
        x[u] = f4_lin(c, xo, -sn, y[u]);
        y[u] = f4_lin(sn, xo, c, y[u]);
    }
    return cosv;
}

// grid (nbp / 2, n_sino), kBThreads threads, dynamic shared memory
// block_round_smem_floats(K4) floats, 128 K4 >= n: lane l holds rows
// 4 l + 128 u .. + 3 (u < K4) of a column.
template <int K4>
__global__ void __launch_bounds__(kBThreads)
rt_block_round_kernel(float *__restrict__ X, float *__restrict__ V, int n, int nbp, int round,
                      unsigned *__restrict__ off_bits, const float *__restrict__ tiny) {
    extern __shared__ __align__(16) float bsm[];
    constexpr int NP = 128 * K4; // padded rows
    constexpr bool kWholeV = block_round_whole_v(K4);
    constexpr int VR = kWholeV ? NP : kVRows; // rows of the V buffer
    constexpr int VLD = VR + 4;               // its leading dimension (bank spread)
    float *Xl = bsm;                          // kBCols x NP
    float *Vb = Xl + (size_t)kBCols * NP;     // kBCols x VLD
    float(*Jt)[kBCols + 1] = reinterpret_cast<float(*)[kBCols + 1]>(Vb + kBCols * VLD);
    float(*Jr)[kBCols] = reinterpret_cast<float(*)[kBCols]>(&Jt[kBCols][0]); // row-major J
    const int s = blockIdx.y, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nb = (n + kBJ - 1) / kBJ;
    int bp, bq;
    round_robin(nbp, round, blockIdx.x, bp, bq);
    const bool intra = round == 0; // the sweep's first round also rotates within blocks
    if (bq >= nb && !intra)
        return; // the bye (the dummy block's columns are zeros and never rotate)
    const size_t nn = (size_t)n * n;
    float *Xg = X + s * nn, *Vg = V + s * nn;
    // global column of local column c
    auto gcol = [&](int c) { return c < kBJ ? bp * kBJ + c : bq * kBJ + c - kBJ; };
    // X block (zero-padded to NP rows), then -- in flight during the inner
    // rounds -- the V block (or its first chunk); J = I
    stage_cols_async(Xl, NP, Xg, n, 0, NP, gcol);
    cp_async_commit();
    stage_cols_async(Vb, VLD, Vg, n, 0, VR, gcol);
    cp_async_commit();
    for (int e = threadIdx.x; e < kBCols * kBCols; e += kBThreads)
        Jt[e / kBCols][e % kBCols] = e / kBCols == e % kBCols ? 1.f : 0.f;
    cp_async_wait<1>();
    __syncthreads();
    const float tn = tiny[s];
    float wmax = 0.f;
    // J <- J G on columns p, q (row `lane` of each)
    auto j_rotate = [&](int p, int q, float c, float sn) {
        if (kBCols < 32 && lane >= kBCols)
            return;
        const float a = Jt[p][lane], b = Jt[q][lane];
        Jt[p][lane] = c * a - sn * b;
        Jt[q][lane] = sn * a + c * b;
    };
    float4 x[K4], y[K4];
    if (intra) {
        // pairs within each block: warps 0 .. kBJ / 2 - 1 block bp, the rest block bq
        const int half = warp / (kBJ / 2);
        for (int ir = 0; ir < kBJ - 1; ir++) {
            int p, q;
            round_robin(kBJ, ir, warp % (kBJ / 2), p, q);
            p += half * kBJ;
            q += half * kBJ;
            float4 *xp = reinterpret_cast<float4 *>(Xl + (size_t)p * NP);
            float4 *xq = reinterpret_cast<float4 *>(Xl + (size_t)q * NP);
#pragma unroll
            for (int u = 0; u < K4; u++) {
                x[u] = xp[lane + 32 * u];
                y[u] = xq[lane + 32 * u];
            }
            float c, sn;
            const float cosv = jacobi_pair<K4>(x, y, tn, c, sn);
            if (cosv > 0.f) {
                wmax = fmaxf(wmax, cosv);
#pragma unroll
                for (int u = 0; u < K4; u++) {
                    xp[lane + 32 * u] = x[u];
                    xq[lane + 32 * u] = y[u];
                }
                j_rotate(p, q, c, sn);
            }
            __syncthreads();
        }
    }
    // pairs across the blocks: in inner round r warp w pairs column w of bp
    // (kept in registers throughout) with column (w + r) % kBJ of bq
    float4 *xw = reinterpret_cast<float4 *>(Xl + (size_t)warp * NP);
#pragma unroll
    for (int u = 0; u < K4; u++)
        x[u] = xw[lane + 32 * u];
    for (int r = 0; r < kBJ; r++) {
        const int q = kBJ + (warp + r) % kBJ;
        float4 *xq = reinterpret_cast<float4 *>(Xl + (size_t)q * NP);
#pragma unroll
        for (int u = 0; u < K4; u++)
            y[u] = xq[lane + 32 * u];
        float c, sn;
        const float cosv = jacobi_pair<K4>(x, y, tn, c, sn);
        if (cosv > 0.f) {
            wmax = fmaxf(wmax, cosv);
#pragma unroll
            for (int u = 0; u < K4; u++)
                xq[lane + 32 * u] = y[u];
            j_rotate(warp, q, c, sn);
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < K4; u++)
        xw[lane + 32 * u] = x[u];
    __syncthreads();
    if (lane == 0 && wmax > 0.f)
        atomicMax(off_bits + s, __float_as_uint(wmax));
    // X block back
    store_cols(Xg, Xl, NP, n, 0, NP, gcol);
    for (int e = threadIdx.x; e < kBCols * kBCols; e += kBThreads)
        Jr[e / kBCols][e % kBCols] = Jt[e % kBCols][e / kBCols];

    // V block <- V block J, kVRows rows per pass: thread t computes rows
    // 4 (t / G) .. + 3 and columns 4 (t % G) .. + 3 of each pass, G = kBCols / 4
    constexpr int kCG = kBCols / 4;
    const int cg = (threadIdx.x % kCG) * 4, rg = (threadIdx.x / kCG) * 4;
    auto vj_tile = [&](const float *vb, int ld, float (&acc)[4][4]) {
#pragma unroll
        for (int u = 0; u < 4; u++)
#pragma unroll
            for (int v = 0; v < 4; v++)
                acc[u][v] = 0.f;
#pragma unroll 8
        for (int i = 0; i < kBCols; i++) {
            const float4 vin = *reinterpret_cast<const float4 *>(vb + (size_t)i * ld + rg);
            const float4 jr = *reinterpret_cast<const float4 *>(&Jr[i][cg]);
            const float vi[4] = {vin.x, vin.y, vin.z, vin.w}, ji[4] = {jr.x, jr.y, jr.z, jr.w};
#pragma unroll
            for (int u = 0; u < 4; u++)
#pragma unroll
                for (int v = 0; v < 4; v++)
                    acc[u][v] = fmaf(vi[u], ji[v], acc[u][v]);
        }
    };
    auto put_tile = [&](float *vb, int ld, const float (&acc)[4][4]) {
#pragma unroll
        for (int v = 0; v < 4; v++)
            *reinterpret_cast<float4 *>(vb + (size_t)(cg + v) * ld + rg) =
                make_float4(acc[0][v], acc[1][v], acc[2][v], acc[3][v]);
    };
    if constexpr (kWholeV) {
        constexpr int kPasses = (NP + kVRows - 1) / kVRows; // 1 or 2
        cp_async_wait<0>();
        __syncthreads(); // V block and Jr in place
        float acc[kPasses][4][4];
#pragma unroll
        for (int ps = 0; ps < kPasses; ps++)
            if (ps * kVRows + rg < NP)
                vj_tile(Vb + ps * kVRows, VLD, acc[ps]);
        __syncthreads(); // every thread has read Vb
#pragma unroll
        for (int ps = 0; ps < kPasses; ps++)
            if (ps * kVRows + rg < NP)
                put_tile(Vb + ps * kVRows, VLD, acc[ps]);
        __syncthreads();
        store_cols(Vg, Vb, VLD, n, 0, NP, gcol);
    } else {
        for (int r0 = 0; r0 < n; r0 += kVRows) {
            if (r0 > 0) {
                __syncthreads(); // the previous chunk is written out
                stage_cols_async(Vb, VLD, Vg, n, r0, kVRows, gcol);
                cp_async_commit();
            }
            cp_async_wait<0>();
            __syncthreads(); // chunk and Jr in place
            float acc[4][4];
            vj_tile(Vb, VLD, acc);
            __syncthreads(); // every thread has read the chunk
            put_tile(Vb, VLD, acc);
            __syncthreads();
            store_cols(Vg, Vb, VLD, n, r0, kVRows, gcol);
        }
    }
}

// ---- assembly ---------------------------------------------------------------

// 1 / |x_k| per column of the converged X (0 for a null direction).  grid
// (ceil(n / 4), n_sino), one warp per column.
__global__ void rt_invnorm_kernel(const float *__restrict__ X, int n, const float *__restrict__ tiny,
                                  float *__restrict__ inv) {
    const int k = blockIdx.x * 4 + (threadIdx.x >> 5), s = blockIdx.y, lane = threadIdx.x & 31;
    if (k >= n)
        return;
    const float *x = X + (size_t)s * n * n + (size_t)k * n;
    float v = 0.f;
    for (int i = lane; i < n; i += 32)
        v = fmaf(x[i], x[i], v);
    v = warp_sum(v);
    if (lane == 0)
        inv[(size_t)s * n + k] = v > tiny[s] ? rsqrtf(v) : 0.f;
}

// X[:, k] *= inv[k]: the columns of X become U_X.  grid (ceil(n n / 256), n_sino).
__global__ void rt_scale_kernel(float *__restrict__ X, const float *__restrict__ inv, int n) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long nn = (long long)n * n;
    if (e < nn)
        X[blockIdx.y * nn + e] *= inv[(size_t)blockIdx.y * n + (int)(e / n)];
}

// C = alpha op(A) op(B) + beta D for n x n column-major float matrices per
// sinogram, op given by strides: op(A)(i, k) = A[i ai + k ak], op(B)(k, j) =
// B[k bk + j bj].  32 x 32 output tiles (256 threads, 4 outputs each), k in
// shared-memory steps of 32.  grid (ceil(n / 32), ceil(n / 32), n_sino).
__global__ void __launch_bounds__(256)
rt_gemm_kernel(const float *__restrict__ A, int ai, int ak, const float *__restrict__ B, int bk,
               int bj, const float *__restrict__ D, float alpha, float beta, int n,
               float *__restrict__ C) {
    __shared__ float as[32][33], bs[32][33];
    const int ti = threadIdx.x & 31, tj = threadIdx.x >> 5; // tj 0..7
    const int i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
    const size_t off = (size_t)blockIdx.z * n * n;
    A += off;
    B += off;
    C += off;
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    for (int k0 = 0; k0 < n; k0 += 32) {
        __syncthreads();
        for (int e = threadIdx.x; e < 32 * 32; e += 256) {
            const int r = e & 31, kk = e >> 5, k = k0 + kk;
            as[kk][r] = (k < n && i0 + r < n) ? A[(size_t)(i0 + r) * ai + (size_t)k * ak] : 0.f;
            bs[kk][r] = (k < n && j0 + r < n) ? B[(size_t)k * bk + (size_t)(j0 + r) * bj] : 0.f;
        }
        __syncthreads();
#pragma unroll 8
        for (int kk = 0; kk < 32; kk++) {
            const float a = as[kk][ti];
#pragma unroll
            for (int u = 0; u < 4; u++)
                acc[u] = fmaf(a, bs[kk][tj + 8 * u], acc[u]);
        }
    }
    const int i = i0 + ti;
#pragma unroll
    for (int u = 0; u < 4; u++) {
        const int j = j0 + tj + 8 * u;
        if (i < n && j < n) {
            const size_t e = i + (size_t)j * n;
            C[e] = beta != 0.f ? alpha * acc[u] + beta * D[off + e] : alpha * acc[u];
        }
    }
}

// Y = Q [P; 0] = H_0 H_1 ... H_{n-1} [P; 0], out[:, perm[j]] = Y[:, j]:
// one reflector at a time with Y in registers while the aligned columns fit
// (m <= 16 kQThreads), by blocks of reflectors above.
constexpr int kQThreads = 256, kQCols = 4; // columns of Y per CTA
constexpr int kNosMaxCols = 1024;              // angles the orthonormal circus takes

// The product with Y held in registers, for m <= K kQThreads: thread t
// owns rows t + kQThreads u (u < K) of the kQCols columns, so applying a
// reflector needs one block reduction (double-buffered: one barrier) and no
// other exchange; the next reflector's column is loaded while the current
// one is applied, and the reflector scalars sit in shared memory.  Slot
// (t, u) of reflector k holds v_i for i = t + kQThreads u: 1 at i = k, the
// scaled pivot column below it, 0 above.
template <int K>
__global__ void __launch_bounds__(kQThreads, K == 8 ? 3 : 1) // 3 CTAs per SM fit K = 8 unspilled
nos_apply_q_reg_kernel(const float2 *__restrict__ A, const NosDesc *__restrict__ desc,
                       const float2 *__restrict__ tau, const float2 *__restrict__ scale,
                       const int *__restrict__ perm, const float *__restrict__ P, int n,
                       float *__restrict__ out) {
    __shared__ float s_t[kNosMaxCols], s_vs[kNosMaxCols];
    __shared__ int s_pm[kNosMaxCols];
    __shared__ float red[2][kQThreads / 32][kQCols];
    const int s = blockIdx.y, j0 = blockIdx.x * kQCols;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const NosDesc d = desc[s];
    const int m = d.m, nc = min(kQCols, n - j0);
    const size_t nn = (size_t)n * n;
    for (int k = threadIdx.x; k < n; k += kQThreads) {
        const float2 t = tau[(size_t)s * n + k], v = scale[(size_t)s * n + k];
        s_t[k] = t.x + t.y;
        s_vs[k] = v.x + v.y;
        s_pm[k] = perm[(size_t)s * n + k];
    }
    float y[kQCols][K];
#pragma unroll
    for (int u = 0; u < K; u++) {
        const int i = threadIdx.x + kQThreads * u;
#pragma unroll
        for (int c = 0; c < kQCols; c++)
            y[c][u] = (c < nc && i < n) ? P[s * nn + i + (size_t)(j0 + c) * n] : 0.f;
    }
    __syncthreads(); // scalars in place
    const float2 *As = A + d.a_off;
    auto load_v = [&](int k, float(&v)[K]) {
        const float2 *x = As + (size_t)s_pm[k] * m;
        const float vs = s_vs[k];
#pragma unroll
        for (int u = 0; u < K; u++) {
            const int i = threadIdx.x + kQThreads * u;
            float vi = 0.f;
            if (i > k && i < m) {
                const float2 xi = x[i];
                vi = (xi.x + xi.y) * vs;
            } else if (i == k) {
                vi = 1.f;
            }
            v[u] = vi;
        }
    };
    float v[K], vn[K];
    load_v(n - 1, v);
    int rb = 0;
    for (int k = n - 1; k >= 0; k--) {
        if (k > 0)
            load_v(k - 1, vn);
        const float t = s_t[k];
        if (t != 0.f) { // uniform
            float w[kQCols];
#pragma unroll
            for (int c = 0; c < kQCols; c++) {
                w[c] = 0.f;
#pragma unroll
                for (int u = 0; u < K; u++)
                    w[c] = fmaf(v[u], y[c][u], w[c]);
                w[c] = warp_sum(w[c]);
            }
            if (lane == 0)
#pragma unroll
                for (int c = 0; c < kQCols; c++)
                    red[rb][warp][c] = w[c];
            __syncthreads();
#pragma unroll
            for (int c = 0; c < kQCols; c++) {
                float tot = 0.f;
#pragma unroll
                for (int q = 0; q < kQThreads / 32; q++)
                    tot += red[rb][q][c];
                w[c] = t * tot;
            }
            rb ^= 1;
#pragma unroll
            for (int u = 0; u < K; u++)
#pragma unroll
                for (int c = 0; c < kQCols; c++)
                    y[c][u] = fmaf(-w[c], v[u], y[c][u]);
        }
#pragma unroll
        for (int u = 0; u < K; u++)
            v[u] = vn[u];
    }
    for (int c = 0; c < nc; c++) {
        float *o = out + d.out_off + (size_t)s_pm[j0 + c] * m;
#pragma unroll
        for (int u = 0; u < K; u++) {
            const int i = threadIdx.x + kQThreads * u;
            if (i < m)
                o[i] = y[c][u];
        }
    }
}

// Y = Q [P; 0] = H_0 H_1 ... H_{n-1} [P; 0] by blocks of kWyB reflectors in
// compact WY form (the LAPACK larft / larfb scheme): the product of reflectors
// k0 .. k0 + b - 1 is I - V T V^T with V = [v_k0 .. v_k0+b-1] (v_k: 1 at row
// k, the scaled stored pivot column below it, 0 above) and T upper
// triangular, T[i, i] = tau_i, T[0:i, i] = -tau_i T[0:i, 0:i] V[:, 0:i]^T v_i.
// The blocks apply last to first, each as Y <- Y - V (T (V^T Y)) over rows
// k0.. (V is zero above): V^T Y by row chunks into partial sums, T times
// their sum, then the rank-b update -- float GEMM tiles instead of one
// latency-bound pass over Y per reflector.  Y lives in the output: its
// column j is out[:, perm[j]].
constexpr int kWyB = 32;          // reflectors per block
constexpr int kWyThreads = 256;   // threads of every WY kernel
constexpr int kWyCols = 128;      // columns of Y per CTA of the GEMM passes
constexpr int kWyVLd = 36;        // V tile row stride (float4 rows, conflict-free fill)
constexpr int kWyYLd = 132;       // Y / W tile row stride
constexpr int kWyGramRows = 128;  // rows per pass of the T kernel

// out[:, perm[j]] = [P[:, j]; 0].  grid (n, n_sino).
__global__ void __launch_bounds__(kWyThreads)
wy_init_kernel(const float *__restrict__ P, const NosDesc *__restrict__ desc,
               const int *__restrict__ perm, int n, float *__restrict__ out) {
    const int j = blockIdx.x, s = blockIdx.y;
    const NosDesc d = desc[s];
    float *o = out + d.out_off + (size_t)perm[(size_t)s * n + j] * d.m;
    const float *p = P + (size_t)s * n * n + (size_t)j * n;
    for (int i = threadIdx.x; i < d.m; i += kWyThreads)
        o[i] = i < n ? p[i] : 0.f;
}

// Per-block reflector data in shared memory: stored column, float scale and
// tau (0 past n, which makes those columns of V and T zero).
struct WyRefl {
    int pm[kWyB];
    float vs[kWyB], t[kWyB];
};
__device__ __forceinline__ void wy_load_refl(WyRefl &R, const float2 *tau, const float2 *scale,
                                             const int *perm, int n, int s, int k0) {
    if (threadIdx.x < kWyB) {
        const int k = k0 + threadIdx.x;
        const bool ok = k < n;
        const size_t o = (size_t)s * n + k;
        R.pm[threadIdx.x] = ok ? perm[o] : 0;
        R.vs[threadIdx.x] = ok ? scale[o].x + scale[o].y : 0.f;
        R.t[threadIdx.x] = ok ? tau[o].x + tau[o].y : 0.f;
    }
}
// v_{k0 + r}[row] for a row inside the matrix (row < m).
__device__ __forceinline__ float wy_v(const float2 *As, int m, const WyRefl &R, int n, int k0,
                                      int r, int row) {
    const int k = k0 + r;
    if (k >= n || row < k)
        return 0.f;
    if (row == k)
        return 1.f;
    const float2 x = As[(size_t)R.pm[r] * m + row];
    return (x.x + x.y) * R.vs[r];
}

// T of every block: the Gram matrix G = V^T V over rows k0..m-1 (kWyGramRows
// rows of V staged per pass; thread t accumulates G[t / 32 + 8 q][t % 32]),
// then the recurrence on one warp.  grid (blocks, n_sino); T row-major,
// 32 x 32 per (sinogram, block).
__global__ void __launch_bounds__(kWyThreads)
wy_t_kernel(const float2 *__restrict__ A, const NosDesc *__restrict__ desc,
            const float2 *__restrict__ tau, const float2 *__restrict__ scale,
            const int *__restrict__ perm, int n, float *__restrict__ T) {
    __shared__ float Vs[kWyGramRows][kWyB + 1];
    __shared__ float Gs[kWyB][kWyB + 1];
    __shared__ float Ts[kWyB][kWyB + 1];
    __shared__ WyRefl R;
    const int jb = blockIdx.x, s = blockIdx.y, k0 = jb * kWyB;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const NosDesc d = desc[s];
    const int m = d.m;
    const float2 *As = A + d.a_off;
    wy_load_refl(R, tau, scale, perm, n, s, k0);
    __syncthreads(); // R in place
    constexpr int kPer = kWyGramRows * kWyB / kWyThreads;
    float vr[kPer]; // the next pass, fetched while the current one is reduced
    auto fetch = [&](int row0) {
#pragma unroll
        for (int q = 0; q < kPer; q++) {
            const int e = threadIdx.x + kWyThreads * q;
            const int i = e % kWyGramRows, r = e / kWyGramRows, row = row0 + i;
            vr[q] = row < m ? wy_v(As, m, R, n, k0, r, row) : 0.f;
        }
    };
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    if (k0 < m)
        fetch(k0);
    for (int row0 = k0; row0 < m; row0 += kWyGramRows) {
        __syncthreads(); // the previous pass is read
#pragma unroll
        for (int q = 0; q < kPer; q++) {
            const int e = threadIdx.x + kWyThreads * q;
            Vs[e % kWyGramRows][e / kWyGramRows] = vr[q];
        }
        __syncthreads();
        if (row0 + kWyGramRows < m)
            fetch(row0 + kWyGramRows);
#pragma unroll 4
        for (int i = 0; i < kWyGramRows; i++) {
            const float b = Vs[i][lane];
#pragma unroll
            for (int q = 0; q < 4; q++)
                acc[q] = fmaf(Vs[i][warp + 8 * q], b, acc[q]);
        }
    }
#pragma unroll
    for (int q = 0; q < 4; q++)
        Gs[warp + 8 * q][lane] = acc[q];
    __syncthreads();
    if (warp == 0) {
        for (int c = 0; c < kWyB; c++)
            Ts[lane][c] = 0.f;
        __syncwarp();
        for (int i = 0; i < kWyB; i++) {
            float v = 0.f;
            if (lane < i) {
                for (int c = lane; c < i; c++)
                    v = fmaf(Ts[lane][c], Gs[c][i], v);
                v *= -R.t[i];
            }
            __syncwarp();
            if (lane < i)
                Ts[lane][i] = v;
            else if (lane == i)
                Ts[i][i] = R.t[i];
            __syncwarp();
        }
        float *o = T + ((size_t)s * gridDim.x + jb) * kWyB * kWyB;
        for (int r = 0; r < kWyB; r++)
            o[r * kWyB + lane] = Ts[r][lane];
    }
}

// Column offsets of the CTA's kWyCols columns of Y in out (-1 past n).
__device__ __forceinline__ void wy_load_cols(long long *cols, const NosDesc &d, const int *perm,
                                             int n, int s, int j0) {
    if (threadIdx.x < kWyCols) {
        const int j = j0 + threadIdx.x;
        cols[threadIdx.x] = j < n ? d.out_off + (long long)perm[(size_t)s * n + j] * d.m : -1;
    }
}

// Partial W = V^T Y over rows [k0 + c R, k0 + (c + 1) R) of each sinogram
// (R = 32 ns rows; none past m): part[s][c][r][j], 32 x kWyCols per CTA,
// thread (warp, lane) owning reflectors 4 warp .. + 3 and columns 4 lane ..
// + 3.  Rows are staged 32 at a time; the fills map a warp to 8 rows x 4
// columns, which makes their shared-memory stores conflict-free.
// grid (ceil(n / kWyCols), nchunk, n_sino).
__global__ void __launch_bounds__(kWyThreads)
wy_vty_kernel(const float2 *__restrict__ A, const NosDesc *__restrict__ desc,
              const float2 *__restrict__ tau, const float2 *__restrict__ scale,
              const int *__restrict__ perm, int n, int k0, int ns,
              const float *__restrict__ out, float *__restrict__ part) {
    __shared__ __align__(16) float Vs[32 * kWyVLd];
    __shared__ __align__(16) float Ys[32 * kWyYLd];
    __shared__ long long cols[kWyCols];
    __shared__ WyRefl R;
    const int j0 = blockIdx.x * kWyCols, c = blockIdx.y, s = blockIdx.z;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const NosDesc d = desc[s];
    const int m = d.m;
    const float2 *As = A + d.a_off;
    const int rb = k0 + c * 32 * ns, re = min(rb + 32 * ns, m);
    wy_load_refl(R, tau, scale, perm, n, s, k0);
    wy_load_cols(cols, d, perm, n, s, j0);
    __syncthreads(); // R and cols in place
    constexpr int kPV = 32 * kWyB / kWyThreads, kPY = 32 * kWyCols / kWyThreads;
    float vr[kPV], yr[kPY]; // the next 32 rows, fetched during the current ones
    auto fetch = [&](int row0) {
#pragma unroll
        for (int q = 0; q < kPV; q++) {
            const int e = threadIdx.x + kWyThreads * q;
            const int i = (e >> 8) * 8 + (e & 7), r = (e >> 3) & 31, row = row0 + i;
            vr[q] = row < re ? wy_v(As, m, R, n, k0, r, row) : 0.f;
        }
#pragma unroll
        for (int q = 0; q < kPY; q++) {
            const int e = threadIdx.x + kWyThreads * q;
            const int i = (e >> 10) * 8 + (e & 7), col = (e >> 3) & 127, row = row0 + i;
            const long long o = cols[col];
            yr[q] = o >= 0 && row < re ? out[o + row] : 0.f;
        }
    };
    float acc[4][4];
#pragma unroll
    for (int u = 0; u < 4; u++)
#pragma unroll
        for (int v = 0; v < 4; v++)
            acc[u][v] = 0.f;
    if (rb < re)
        fetch(rb);
    for (int row0 = rb; row0 < re; row0 += 32) {
        __syncthreads(); // the previous tiles are read
#pragma unroll
        for (int q = 0; q < kPV; q++) {
            const int e = threadIdx.x + kWyThreads * q;
            Vs[((e >> 8) * 8 + (e & 7)) * kWyVLd + ((e >> 3) & 31)] = vr[q];
        }
#pragma unroll
        for (int q = 0; q < kPY; q++) {
            const int e = threadIdx.x + kWyThreads * q;
            Ys[((e >> 10) * 8 + (e & 7)) * kWyYLd + ((e >> 3) & 127)] = yr[q];
        }
        __syncthreads();
        if (row0 + 32 < re)
            fetch(row0 + 32);
#pragma unroll 8
        for (int i = 0; i < 32; i++) {
            const float4 a = *reinterpret_cast<const float4 *>(&Vs[i * kWyVLd + 4 * warp]);
            const float4 y = *reinterpret_cast<const float4 *>(&Ys[i * kWyYLd + 4 * lane]);
            const float av[4] = {a.x, a.y, a.z, a.w}, yv[4] = {y.x, y.y, y.z, y.w};
#pragma unroll
            for (int u = 0; u < 4; u++)
#pragma unroll
                for (int v = 0; v < 4; v++)
                    acc[u][v] = fmaf(av[u], yv[v], acc[u][v]);
        }
    }
    float *p = part + ((size_t)s * gridDim.y + c) * kWyB * n;
#pragma unroll
    for (int u = 0; u < 4; u++)
#pragma unroll
        for (int v = 0; v < 4; v++) {
            const int j = j0 + 4 * lane + v;
            if (j < n)
                p[(size_t)(4 * warp + u) * n + j] = acc[u][v];
        }
}

// W2 = T (sum of the nchunk partials), 32 x n per sinogram.  grid
// (ceil(n / 32), n_sino).
__global__ void __launch_bounds__(kWyThreads)
wy_w2_kernel(const float *__restrict__ T, const float *__restrict__ part, int nchunk, int n,
             int jb, int nbk, float *__restrict__ W2) {
    __shared__ float Ws[kWyB][33];
    __shared__ float Tt[kWyB][kWyB + 1];
    const int j0 = blockIdx.x * 32, s = blockIdx.y;
    const float *Tb = T + ((size_t)s * nbk + jb) * kWyB * kWyB;
    for (int e = threadIdx.x; e < kWyB * 32; e += kWyThreads) {
        const int r = e >> 5, jj = e & 31, j = j0 + jj;
        // four independent sums, so that the chunks' loads overlap
        float s4[4] = {0.f, 0.f, 0.f, 0.f};
        if (j < n) {
            const float *q = part + ((size_t)s * nchunk * kWyB + r) * n + j;
            const size_t step = (size_t)kWyB * n;
            int c = 0;
#pragma unroll 2
            for (; c + 4 <= nchunk; c += 4)
#pragma unroll
                for (int h = 0; h < 4; h++)
                    s4[h] += q[(c + h) * step];
            for (; c < nchunk; c++)
                s4[0] += q[c * step];
        }
        Ws[r][jj] = (s4[0] + s4[1]) + (s4[2] + s4[3]);
        Tt[r][jj] = Tb[r * kWyB + jj];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < kWyB * 32; e += kWyThreads) {
        const int r = e >> 5, jj = e & 31, j = j0 + jj;
        float v = 0.f;
        for (int c = r; c < kWyB; c++)
            v = fmaf(Tt[r][c], Ws[c][jj], v);
        if (j < n)
            W2[((size_t)s * kWyB + r) * n + j] = v;
    }
}

// Y[rows, cols] -= V[rows, :] W2[:, cols] over rows [k0 + c R, .. + R)
// (none past m): W2's 32 x kWyCols tile staged once, V 32 rows at a time;
// lane = row, warp w = columns 16 w .. + 15, so each column's 32 rows are
// one coalesced read-modify-write.  grid (ceil(n / kWyCols), nchunk, n_sino).
__global__ void __launch_bounds__(kWyThreads)
wy_update_kernel(const float2 *__restrict__ A, const NosDesc *__restrict__ desc,
                 const float2 *__restrict__ tau, const float2 *__restrict__ scale,
                 const int *__restrict__ perm, int n, int k0, int ns,
                 const float *__restrict__ W2, float *__restrict__ out) {
    __shared__ __align__(16) float Ws[kWyB * kWyYLd];
    __shared__ float Vs[32 * 33];
    __shared__ long long cols[kWyCols];
    __shared__ WyRefl R;
    const int j0 = blockIdx.x * kWyCols, c = blockIdx.y, s = blockIdx.z;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const NosDesc d = desc[s];
    const int m = d.m;
    const int rb = k0 + c * 32 * ns, re = min(rb + 32 * ns, m);
    if (rb >= re)
        return; // uniform: no rows of this sinogram here
    const float2 *As = A + d.a_off;
    wy_load_refl(R, tau, scale, perm, n, s, k0);
    wy_load_cols(cols, d, perm, n, s, j0);
    for (int e = threadIdx.x; e < kWyB * kWyCols; e += kWyThreads) {
        const int r = e >> 7, q = e & 127, j = j0 + q;
        Ws[r * kWyYLd + q] = j < n ? W2[((size_t)s * kWyB + r) * n + j] : 0.f;
    }
    const int cw = 16 * warp;
    constexpr int kPV = 32 * kWyB / kWyThreads;
    float vr[kPV]; // the next 32 rows of V, fetched during the current ones
    auto fetch = [&](int row0) {
#pragma unroll
        for (int q = 0; q < kPV; q++) {
            const int e = threadIdx.x + kWyThreads * q;
            const int i = e & 31, r = e >> 5, row = row0 + i;
            vr[q] = row < re ? wy_v(As, m, R, n, k0, r, row) : 0.f;
        }
    };
    __syncthreads(); // R, cols and Ws in place
    fetch(rb);
    for (int row0 = rb; row0 < re; row0 += 32) {
        __syncthreads(); // the previous V tile is read
#pragma unroll
        for (int q = 0; q < kPV; q++) {
            const int e = threadIdx.x + kWyThreads * q;
            Vs[(e & 31) * 33 + (e >> 5)] = vr[q];
        }
        __syncthreads();
        if (row0 + 32 < re)
            fetch(row0 + 32);
        const int row = row0 + lane;
        float yo[16]; // the rows' current values, loaded ahead of the FMAs
#pragma unroll
        for (int v = 0; v < 16; v++) {
            const long long o = cols[cw + v];
            yo[v] = o >= 0 && row < re ? out[o + row] : 0.f;
        }
        float acc[16];
#pragma unroll
        for (int v = 0; v < 16; v++)
            acc[v] = 0.f;
#pragma unroll 4
        for (int r = 0; r < kWyB; r++) {
            const float a = Vs[lane * 33 + r];
            const float4 *w = reinterpret_cast<const float4 *>(&Ws[r * kWyYLd + cw]);
#pragma unroll
            for (int h = 0; h < 4; h++) {
                const float4 x = w[h];
                acc[4 * h] = fmaf(a, x.x, acc[4 * h]);
                acc[4 * h + 1] = fmaf(a, x.y, acc[4 * h + 1]);
                acc[4 * h + 2] = fmaf(a, x.z, acc[4 * h + 2]);
                acc[4 * h + 3] = fmaf(a, x.w, acc[4 * h + 3]);
            }
        }
        if (row < re)
#pragma unroll
            for (int v = 0; v < 16; v++) {
                const long long o = cols[cw + v];
                if (o >= 0)
                    out[o + row] = yo[v] - acc[v];
            }
    }
}

// The stop rule after a sweep: the largest rotated cosine over the
// sinograms below kJacDone, or below 1e-3 and no longer falling by 4x (the
// float rounding floor of the rotated columns, which grows with sqrt(n) --
// near convergence the cyclic method is quadratic, so a real decrease is by
// orders of magnitude), or max_sweeps done.  state = {previous sweep's
// largest cosine (float bits; 1 before the first), sweeps done}.
__global__ void nos_sweep_check_kernel(const unsigned *__restrict__ off_bits, int n_sino,
                                       unsigned *__restrict__ state, int max_sweeps,
                                       cudaGraphConditionalHandle loop) {
    float worst = 0.f;
    for (int i = threadIdx.x; i < n_sino; i += 32)
        worst = fmaxf(worst, __uint_as_float(off_bits[i]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        worst = fmaxf(worst, __shfl_xor_sync(TT_FULL_MASK, worst, o));
    if (threadIdx.x != 0)
        return;
    const unsigned done = state[1] + 1;
    const float prev = done == 1 ? 1.f : __uint_as_float(state[0]);
    state[0] = __float_as_uint(worst);
    state[1] = done;
    const bool stop = worst < kJacDone || (worst < 1e-3f && worst > 0.25f * prev) ||
                      (int)done >= max_sweeps;
    cudaGraphSetConditional(loop, stop ? 0u : 1u);
}

} // namespace

cudaError_t launch_nos_offsets(const float *sino, int rows, int cols, int n_sino, int center,
                               int *offsets, cudaStream_t st) {
    const long long n = (long long)cols * n_sino;
    if (n <= 0)
        return cudaSuccess;
    nos_offsets_kernel<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(sino, rows, (int)n, center,
                                                                      offsets);
    return cudaGetLastError();
}

cudaError_t launch_nos_align(const float *sino, int rows, int cols, int n_sino,
                             const NosDesc *desc, const int *offsets, float2 *A, size_t a_elems,
                             cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(A, 0, sizeof(float2) * a_elems, st);
    if (e != cudaSuccess)
        return e;
    nos_align_kernel<<<dim3(cols, n_sino), 128, 0, st>>>(sino, rows, cols, desc, offsets, A);
    return cudaGetLastError();
}

template <int K, int T>
static void qr_steps(float2 *A, const NosDesc *desc, int n, int n_sino, const NosWork &w,
                     cudaStream_t st) {
    // CTAs per sinogram: one wave over all sinograms, at most kQrMaxCols
    // positions per CTA
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, qr_step_kernel<K, T>, T, 0);
    const int wave = std::max(1, sms * std::max(per_sm, 1) / std::max(n_sino, 1));
    for (int k = 0; k < n; k++) {
        const int left = n - k;
        const int g = std::min(left, std::max(wave, (left + kQrMaxCols - 1) / kQrMaxCols));
        qr_step_kernel<K, T><<<dim3(g, n_sino), T, 0, st>>>(A, desc, n, n_sino, k, w);
    }
}

int nos_max_rows() { return 32 * kQrThreads; }

cudaError_t launch_nos_factor(float2 *A, const NosDesc *desc, int n, int n_sino, int max_m,
                              const NosWork &w, cudaStream_t st) {
    if (max_m > nos_max_rows())
        return cudaErrorInvalidValue;
    qr_init_kernel<<<dim3(n, n_sino), kQrThreads, 0, st>>>(A, desc, n, w);
    // 128-thread CTAs up to 2048 rows (more CTAs, and so more column chains,
    // in flight per SM), 256 above
    if (max_m <= 12 * 128)
        qr_steps<12, 128>(A, desc, n, n_sino, w, st);
    else if (max_m <= 16 * 128)
        qr_steps<16, 128>(A, desc, n, n_sino, w, st);
    else if (max_m <= 16 * kQrThreads)
        qr_steps<16, kQrThreads>(A, desc, n, n_sino, w, st);
    else if (max_m <= 24 * kQrThreads)
        qr_steps<24, kQrThreads>(A, desc, n, n_sino, w, st);
    else
        qr_steps<32, kQrThreads>(A, desc, n, n_sino, w, st);
    const long long nn = (long long)n * n;
    nos_rt_kernel<<<dim3((unsigned)((nn + 255) / 256), n_sino), 256, 0, st>>>(A, desc, n, w);
    return cudaGetLastError();
}

template <int K4>
static cudaError_t block_rounds(int n, int n_sino, const NosWork &w, cudaStream_t st) {
    const int nb = (n + kBJ - 1) / kBJ, nbp = nb + (nb & 1);
    const size_t smem = sizeof(float) * block_round_smem_floats(K4);
    if (128 * K4 < n)
        return cudaErrorInvalidValue;
    if (smem > opt_in_smem((const void *)rt_block_round_kernel<K4>))
        return cudaErrorInvalidValue;
    for (int r = 0; r < nbp - 1; r++)
        rt_block_round_kernel<K4><<<dim3(nbp / 2, n_sino), kBThreads, smem, st>>>(
            w.X, w.V, n, nbp, r, w.off_bits, w.tiny);
    return cudaGetLastError();
}

cudaError_t launch_nos_sweep(int n, int n_sino, const NosWork &w, int max_sweeps,
                             cudaGraphConditionalHandle loop, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(w.off_bits, 0, sizeof(unsigned) * n_sino, st);
    if (e != cudaSuccess)
        return e;
    if (n <= 128)
        e = block_rounds<1>(n, n_sino, w, st);
    else if (n <= 256)
        e = block_rounds<2>(n, n_sino, w, st);
    else if (n <= 384)
        e = block_rounds<3>(n, n_sino, w, st);
    else if (n <= 512)
        e = block_rounds<4>(n, n_sino, w, st);
    else if (n <= 768)
        e = block_rounds<6>(n, n_sino, w, st);
    else if (n <= 1024)
        e = block_rounds<8>(n, n_sino, w, st);
    else
        e = cudaErrorInvalidValue; // more than 1024 angles
    if (e != cudaSuccess)
        return e;
    nos_sweep_check_kernel<<<1, 32, 0, st>>>(w.off_bits, n_sino, w.sweep_state, max_sweeps,
                                             loop);
    return cudaGetLastError();
}

// Shape of the blocked Q application: row chunks of 32 ns rows, ns halved
// from 8 until the GEMM passes have at least 3 CTAs per SM (or ns is 1).
struct WyShape {
    int nbk, tiles, ns, nchunk0;
    size_t t_floats, part_floats, w2_floats;
};
static WyShape wy_shape(int n, int n_sino, int max_m) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    WyShape w;
    w.nbk = (n + kWyB - 1) / kWyB;
    w.tiles = (n + kWyCols - 1) / kWyCols;
    w.ns = 8;
    auto chunks = [&](int ns) { return (max_m + 32 * ns - 1) / (32 * ns); };
    while (w.ns > 1 && (long long)w.tiles * chunks(w.ns) * n_sino < 3LL * std::max(sms, 1))
        w.ns /= 2;
    w.nchunk0 = chunks(w.ns);
    w.t_floats = (size_t)n_sino * w.nbk * kWyB * kWyB;
    w.part_floats = (size_t)n_sino * w.nchunk0 * kWyB * n;
    w.w2_floats = (size_t)n_sino * kWyB * n;
    return w;
}

// The blocked application takes over from the register kernel where the
// aligned columns no longer fit its registers (measured on 8 sinograms of
// 5795 x 720: the whole assembly 9.5 ms against 32.4 ms with a shared-memory
// form of the one-reflector-at-a-time kernel; on 1843 x 360 the register
// kernel is the faster, 1.04 against 1.33 ms).
static bool wy_path(int n, int max_m) { return n > kNosMaxCols || max_m > 16 * kQThreads; }

size_t nos_assemble_floats(int n, int n_sino, int max_m) {
    if (!wy_path(n, max_m))
        return 0;
    const WyShape w = wy_shape(n, n_sino, max_m);
    return w.t_floats + w.part_floats + w.w2_floats;
}

cudaError_t launch_nos_assemble(const float2 *A, const NosDesc *desc, int n, int n_sino,
                                int max_m, const NosWork &w, float *out, cudaStream_t st) {
    const long long nn = (long long)n * n;
    const dim3 ge((unsigned)((nn + 255) / 256), n_sino), gt((n + 31) / 32, (n + 31) / 32, n_sino);
    rt_invnorm_kernel<<<dim3((n + 3) / 4, n_sino), 128, 0, st>>>(w.X, n, w.tiny, w.inv);
    rt_scale_kernel<<<ge, 256, 0, st>>>(w.X, w.inv, n);
    // P = V U^T, then one Newton-Schulz step P <- P (3 I - P^T P) / 2 (in the
    // V buffer), which removes the symmetric part of P's distance from
    // orthogonality left by the float sweeps' stopping bound; S = P^T P goes
    // to the X buffer
    rt_gemm_kernel<<<gt, 256, 0, st>>>(w.V, 1, n, w.X, n, 1, nullptr, 1.f, 0.f, n, w.P);
    rt_gemm_kernel<<<gt, 256, 0, st>>>(w.P, n, 1, w.P, 1, n, nullptr, 1.f, 0.f, n, w.X);
    rt_gemm_kernel<<<gt, 256, 0, st>>>(w.P, 1, n, w.X, 1, n, w.P, -0.5f, 1.5f, n, w.V);
    const dim3 gq((n + kQCols - 1) / kQCols, n_sino);
    if (!wy_path(n, max_m) && max_m <= 8 * kQThreads) {
        nos_apply_q_reg_kernel<8><<<gq, kQThreads, 0, st>>>(A, desc, w.tau, w.scale, w.perm,
                                                             w.V, n, out);
        return cudaGetLastError();
    }
    if (!wy_path(n, max_m)) {
        nos_apply_q_reg_kernel<16><<<gq, kQThreads, 0, st>>>(A, desc, w.tau, w.scale, w.perm,
                                                              w.V, n, out);
        return cudaGetLastError();
    }
    // Y = Q [P; 0] in the output, block by block (last block first)
    const WyShape sh = wy_shape(n, n_sino, max_m);
    float *T = w.wy, *part = T + sh.t_floats, *W2 = part + sh.part_floats;
    wy_init_kernel<<<dim3(n, n_sino), kWyThreads, 0, st>>>(w.V, desc, w.perm, n, out);
    wy_t_kernel<<<dim3(sh.nbk, n_sino), kWyThreads, 0, st>>>(A, desc, w.tau, w.scale, w.perm,
                                                              n, T);
    for (int jb = sh.nbk - 1; jb >= 0; jb--) {
        const int k0 = jb * kWyB;
        const int nch = (max_m - k0 + 32 * sh.ns - 1) / (32 * sh.ns);
        const dim3 g(sh.tiles, nch, n_sino);
        wy_vty_kernel<<<g, kWyThreads, 0, st>>>(A, desc, w.tau, w.scale, w.perm, n, k0, sh.ns,
                                                 out, part);
        wy_w2_kernel<<<dim3((n + 31) / 32, n_sino), kWyThreads, 0, st>>>(T, part, nch, n, jb,
                                                                         sh.nbk, W2);
        wy_update_kernel<<<g, kWyThreads, 0, st>>>(A, desc, w.tau, w.scale, w.perm, n, k0,
                                                    sh.ns, W2, out);
    }
    return cudaGetLastError();
}

} // namespace tt
