// tt_nos.cu -- nearest orthonormal sinogram on the device.
//
// The reference's orthonormal mode (c++/src/circus.cpp:68-102) shifts every
// sinogram column by its weighted-median offset into an m x A matrix
// (m = N + padding) and replaces it by the polar factor U V^T of its SVD,
// computed by Eigen's float JacobiSVD with a column-pivoting Householder QR
// preconditioner.  Here, for n_sino sinograms at once, the same structure
// with the precision split that GB300's rates call for (FP64 ~1/64 of FP32):
//
//   nos_offsets   per column: weighted median row - center, with the
//                 reference's sequential float sums (one thread per column)
//   nos_align     the shifted columns into a zeroed m x A matrix of
//                 double-float pairs (hi + lo, ~48 significant bits)
//   QR            column-pivoting Householder QR, A P = Q R, in double-float
//                 (the only stage beyond float precision: it fixes the small
//                 singular directions that a float factorisation would lose;
//                 the O(m A) work per step runs on the FP32 pipes); per
//                 column step one pivot/reflector launch and one trailing-
//                 update launch, LAPACK-style (reflector below the diagonal,
//                 tau, partial column norms downdated and recomputed when
//                 cancellation sets in)
//   Jacobi        one-sided Jacobi on X = R^T in float (R^T of a pivoted QR is
//                 graded, so float rotations keep relative accuracy), two-
//                 level: round-robin rounds of column-block pairs, each pair
//                 swept in one CTA's shared memory, V accumulated;
//                 X V = U_X S, so polar(R) = V U_X^T
//   assemble      P = V U_X^T (float) with one Newton-Schulz step to clean
//                 its orthogonality, then polar(A P) = Q [P; 0] applied
//                 reflector by reflector per group of columns in shared
//                 memory, and the column permutation undone
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
// (Knuth's two-sum, the FMA two-product, Dekker's renormalisation), i.e. on
// the FP32 pipes, which GB300 runs far faster than FP64.  Scalars (norms,
// reflector coefficients) stay in double.

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
    const float p = a.x * b.x;
    float e = fmaf(a.x, b.x, -p);
    e = fmaf(a.x, b.y, e);
    e = fmaf(a.y, b.x, e);
    return df_quick(p, e);
}
__device__ __forceinline__ float2 df_neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ double df_to_d(float2 a) { return (double)a.x + (double)a.y; }
__device__ __forceinline__ float2 d_to_df(double d) {
    const float hi = __double2float_rn(d);
    return make_float2(hi, __double2float_rn(d - (double)hi));
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

template <typename T, int kThreads> __device__ __forceinline__ T block_sum(T v, T *red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(TT_FULL_MASK, v, o);
    if (lane == 0)
        red[warp] = v;
    __syncthreads();
    T t = 0;
#pragma unroll
    for (int w = 0; w < kThreads / 32; w++)
        t += red[w];
    __syncthreads();
    return t;
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

// Squared column norms (partial and reference copy, double) and the identity
// permutation.  grid (n, n_sino).
__global__ void __launch_bounds__(kQrThreads)
qr_init_kernel(const float2 *__restrict__ A, const NosDesc *__restrict__ desc, int n,
               double *__restrict__ norms, double *__restrict__ orig, int *__restrict__ perm) {
    __shared__ double red[kQrThreads / 32];
    const int j = blockIdx.x, s = blockIdx.y;
    const NosDesc d = desc[s];
    const float2 *a = A + d.a_off + (size_t)j * d.m;
    double v = 0;
    for (int i = threadIdx.x; i < d.m; i += kQrThreads) {
        const double x = df_to_d(a[i]);
        v += x * x;
    }
    v = block_sum<double, kQrThreads>(v, red);
    if (threadIdx.x == 0) {
        norms[(size_t)s * n + j] = v;
        orig[(size_t)s * n + j] = v;
        perm[(size_t)s * n + j] = j;
    }
}

// Element slots: thread t holds rows t + kQrThreads u (u < K, K kQrThreads >=
// m) of a column in registers, so a column is read once with all loads in
// flight and written once.

// Step k, one CTA per sinogram: pivot = the remaining column of largest
// partial norm (lowest index on ties), swapped into place; then the
// reflector H = I - tau v v^T with H A[k:, k] = (beta, 0, ...): beta on the
// diagonal, v[1:] below it (v[0] = 1 implicit).  Per step this is O(m), so
// its arithmetic is plain double.
template <int K>
__global__ void __launch_bounds__(kQrThreads)
qr_pivot_kernel(float2 *__restrict__ A, const NosDesc *__restrict__ desc, int n, int k,
                double *__restrict__ norms, double *__restrict__ orig, int *__restrict__ perm,
                double *__restrict__ tau) {
    __shared__ double red[kQrThreads / 32];
    __shared__ double bv[kQrThreads / 32];
    __shared__ int bi[kQrThreads / 32];
    __shared__ int piv;
    __shared__ double s_alpha;
    const int s = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const NosDesc d = desc[s];
    const int m = d.m;
    float2 *As = A + d.a_off;
    double *nr = norms + (size_t)s * n, *og = orig + (size_t)s * n;
    int *pm = perm + (size_t)s * n;
    // argmax of the partial norms over j >= k
    double best = -1;
    int bidx = n;
    for (int j = k + threadIdx.x; j < n; j += kQrThreads) {
        const double v = nr[j];
        if (v > best || (v == best && j < bidx)) {
            best = v;
            bidx = j;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double ov = __shfl_xor_sync(TT_FULL_MASK, best, o);
        const int oi = __shfl_xor_sync(TT_FULL_MASK, bidx, o);
        if (ov > best || (ov == best && oi < bidx)) {
            best = ov;
            bidx = oi;
        }
    }
    if (lane == 0) {
        bv[warp] = best;
        bi[warp] = bidx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = bv[0];
        int ix = bi[0];
        for (int w = 1; w < kQrThreads / 32; w++)
            if (bv[w] > b || (bv[w] == b && bi[w] < ix)) {
                b = bv[w];
                ix = bi[w];
            }
        piv = ix < n ? ix : k;
    }
    __syncthreads();
    const int jp = piv;
    float2 *x = As + (size_t)k * m;
    float2 xv[K];
    if (jp != k) {
        float2 *cb = As + (size_t)jp * m;
        float2 ov[K];
#pragma unroll
        for (int u = 0; u < K; u++) {
            const int i = threadIdx.x + kQrThreads * u;
            xv[u] = i < m ? cb[i] : make_float2(0.f, 0.f);
            ov[u] = i < m ? x[i] : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < K; u++) {
            const int i = threadIdx.x + kQrThreads * u;
            if (i < m) {
                x[i] = xv[u];
                cb[i] = ov[u];
            }
        }
        if (threadIdx.x == 0) {
            double t = nr[k];
            nr[k] = nr[jp];
            nr[jp] = t;
            t = og[k];
            og[k] = og[jp];
            og[jp] = t;
            const int q = pm[k];
            pm[k] = pm[jp];
            pm[jp] = q;
        }
    } else {
#pragma unroll
        for (int u = 0; u < K; u++) {
            const int i = threadIdx.x + kQrThreads * u;
            xv[u] = i < m ? x[i] : make_float2(0.f, 0.f);
        }
    }
    // reflector of x = A[k:m, k]
    double xn = 0;
#pragma unroll
    for (int u = 0; u < K; u++) {
        const int i = threadIdx.x + kQrThreads * u;
        const double xd = df_to_d(xv[u]);
        if (i > k && i < m)
            xn += xd * xd;
        if (i == k)
            s_alpha = xd;
    }
    xn = block_sum<double, kQrThreads>(xn, red); // its barriers publish s_alpha
    const double alpha = s_alpha;
    if (xn == 0) { // already (alpha, 0, ...): H = I
        if (threadIdx.x == 0)
            tau[(size_t)s * n + k] = 0;
        return;
    }
    const double beta = -copysign(sqrt(alpha * alpha + xn), alpha);
    const double scale = 1 / (alpha - beta);
#pragma unroll
    for (int u = 0; u < K; u++) {
        const int i = threadIdx.x + kQrThreads * u;
        if (i > k && i < m)
            x[i] = d_to_df(df_to_d(xv[u]) * scale);
        if (i == k)
            x[i] = d_to_df(beta);
    }
    if (threadIdx.x == 0)
        tau[(size_t)s * n + k] = (beta - alpha) / beta;
}

// Step k, one CTA per trailing column j = k + 1 + blockIdx.x: A[k:, j] -=
// tau v (v . A[k:, j]) in double-float, then the partial norm loses
// A[k, j]^2 -- recomputed from the column when that leaves less than
// ~sqrt(eps) of the original.
template <int K>
__global__ void __launch_bounds__(kQrThreads)
qr_update_kernel(float2 *__restrict__ A, const NosDesc *__restrict__ desc, int n, int k,
                 double *__restrict__ norms, double *__restrict__ orig,
                 const double *__restrict__ tau) {
    __shared__ float2 red[kQrThreads / 32];
    __shared__ double redd[kQrThreads / 32];
    const int j = k + 1 + blockIdx.x, s = blockIdx.y;
    const NosDesc d = desc[s];
    const int m = d.m;
    float2 *As = A + d.a_off;
    const float2 *v = As + (size_t)k * m;
    float2 *c = As + (size_t)j * m;
    const double t = tau[(size_t)s * n + k];
    float2 vv[K], cv[K];
#pragma unroll
    for (int u = 0; u < K; u++) {
        const int i = threadIdx.x + kQrThreads * u;
        const bool in = i > k && i < m;
        vv[u] = in ? v[i] : make_float2(0.f, 0.f);
        cv[u] = in ? c[i] : make_float2(0.f, 0.f);
    }
    float2 ck = c[k];
    if (t != 0) { // uniform
        float2 w = make_float2(0.f, 0.f);
#pragma unroll
        for (int u = 0; u < K; u++)
            w = df_add(w, df_mul(vv[u], cv[u]));
        w = df_add(block_sum_df<kQrThreads>(w, red), ck);
        const float2 ntw = df_neg(df_mul(d_to_df(t), w));
#pragma unroll
        for (int u = 0; u < K; u++) {
            const int i = threadIdx.x + kQrThreads * u;
            cv[u] = df_add(cv[u], df_mul(ntw, vv[u]));
            if (i > k && i < m)
                c[i] = cv[u];
        }
        ck = df_add(ck, ntw);
        if (threadIdx.x == 0)
            c[k] = ck;
    }
    double *nr = norms + (size_t)s * n, *og = orig + (size_t)s * n;
    const double ckd = df_to_d(ck);
    double n2 = nr[j] - ckd * ckd;
    if (n2 <= 1.5e-8 * og[j]) { // uniform: every thread holds the same values
        double r = 0;
#pragma unroll
        for (int u = 0; u < K; u++) {
            const double cd = df_to_d(cv[u]);
            r += cd * cd;
        }
        n2 = block_sum<double, kQrThreads>(r, redd);
        if (threadIdx.x == 0)
            og[j] = n2;
    }
    if (threadIdx.x == 0)
        nr[j] = n2;
}

// ---- one-sided Jacobi on X = R^T (float) ----------------------------------

// Directions of R whose norm is below kNullRel |R[0, 0]| (|R[0, 0]| is the
// largest column norm of the aligned matrix) are below the double precision
// of the input: they take no rotations and no part in U, as the oracle
// treats exactly-zero directions.
constexpr double kNullRel = 1e-15;

// X[i + j n] = R[j, i] (upper triangle of the QR result), V = I, and the
// null-direction bound tiny[s] = (kNullRel R[0, 0])^2.
// grid (ceil(n * n / 256), n_sino).
__global__ void nos_rt_kernel(const float2 *__restrict__ A, const NosDesc *__restrict__ desc,
                              int n, float *__restrict__ X, float *__restrict__ V,
                              float *__restrict__ tiny) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long nn = (long long)n * n;
    if (e >= nn)
        return;
    const int s = blockIdx.y, i = (int)(e % n), j = (int)(e / n);
    const NosDesc d = desc[s];
    if (e == 0) {
        const double r = kNullRel * df_to_d(A[d.a_off]);
        tiny[s] = (float)(r * r);
    }
    X[s * nn + e] = j <= i ? (float)df_to_d(A[d.a_off + j + (size_t)i * d.m]) : 0.f;
    V[s * nn + e] = i == j ? 1.f : 0.f;
}

// A pair is rotated when |x_p . x_q| > kJacTol |x_p| |x_q| -- a few times the
// rounding of a float dot product over n terms split across a warp -- and a
// sweep that rotates none (or whose largest rotated pair is below
// kJacDone) ends the iteration.
constexpr float kJacTol = 1e-6f, kJacDone = 1e-5f;

// Two-level (block) Jacobi.  The n columns form blocks of kBJ; a sweep is a
// round-robin tournament of the blocks (nbp - 1 rounds for nbp blocks, a bye
// when odd), and in each outer round a CTA copies its block pair -- 2 kBJ
// columns of X and of V -- into shared memory and runs one inner sweep over
// all their pairs (2 kBJ - 1 inner rounds of kBJ disjoint pairs, one warp per
// pair, __syncthreads between rounds) before writing them back.  A sweep is
// nbp - 1 launches instead of n - 1, and the rotations are those of the
// cyclic Jacobi method.
constexpr int kBJ = 8, kBCols = 2 * kBJ, kBThreads = 32 * kBJ;

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

// grid (nbp / 2, n_sino), kBThreads threads, dynamic shared memory 2 kBCols n
// floats.  Lane l holds elements l + 32 u (u < K, 32 K >= n) of a column.
template <int K>
__global__ void __launch_bounds__(kBThreads)
rt_block_round_kernel(float *__restrict__ X, float *__restrict__ V, int n, int nbp, int round,
                      unsigned *__restrict__ off_bits, const float *__restrict__ tiny) {
    extern __shared__ __align__(16) float bsm[];
    float *Xl = bsm, *Vl = bsm + (size_t)kBCols * n;
    const int s = blockIdx.y, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nb = (n + kBJ - 1) / kBJ;
    int bp, bq;
    round_robin(nbp, round, blockIdx.x, bp, bq);
    if (bq >= nb)
        return; // the bye
    const size_t nn = (size_t)n * n;
    float *Xg = X + s * nn, *Vg = V + s * nn;
    // warp w stages local columns w (block bp) and w + kBJ (block bq) of X and
    // V, all 4 K loads of a lane in flight at once
    const int c0 = bp * kBJ + warp, c1 = bq * kBJ + warp;
    {
        float a[K], b[K], c[K], d[K];
#pragma unroll
        for (int u = 0; u < K; u++) {
            const int i = lane + 32 * u;
            a[u] = (i < n && c0 < n) ? Xg[(size_t)c0 * n + i] : 0.f;
            b[u] = (i < n && c1 < n) ? Xg[(size_t)c1 * n + i] : 0.f;
            c[u] = (i < n && c0 < n) ? Vg[(size_t)c0 * n + i] : 0.f;
            d[u] = (i < n && c1 < n) ? Vg[(size_t)c1 * n + i] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < K; u++) {
            const int i = lane + 32 * u;
            if (i < n) {
                Xl[(size_t)warp * n + i] = a[u];
                Xl[(size_t)(warp + kBJ) * n + i] = b[u];
                Vl[(size_t)warp * n + i] = c[u];
                Vl[(size_t)(warp + kBJ) * n + i] = d[u];
            }
        }
    }
    __syncthreads();
    const float tn = tiny[s];
    float wmax = 0.f;
    for (int ir = 0; ir < kBCols - 1; ir++) {
        int p, q;
        round_robin(kBCols, ir, warp, p, q);
        float *xp = Xl + (size_t)p * n, *xq = Xl + (size_t)q * n;
        float x[K], y[K];
#pragma unroll
        for (int u = 0; u < K; u++) {
            const int i = lane + 32 * u;
            x[u] = i < n ? xp[i] : 0.f;
            y[u] = i < n ? xq[i] : 0.f;
        }
        float al = 0.f, be = 0.f, ga = 0.f;
#pragma unroll
        for (int u = 0; u < K; u++) {
            al = fmaf(x[u], x[u], al);
            be = fmaf(y[u], y[u], be);
            ga = fmaf(x[u], y[u], ga);
        }
        al = warp_sum(al);
        be = warp_sum(be);
        ga = warp_sum(ga);
        // cos of the pair = |ga| / (|x_p| |x_q|); rotation parameters from
        // the (2-ulp) hardware reciprocal square root: the rotation only has
        // to be orthogonal (c^2 + s^2 = 1 to float precision), not exact
        const float cosv = fabsf(ga) * (rsqrtf(al) * rsqrtf(be));
        // a null direction (or an empty slot past n), or already orthogonal
        if (al > tn && be > tn && ga != 0.f && cosv > kJacTol) {
            wmax = fmaxf(wmax, cosv);
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
            const float c = rsqrtf(fmaf(t, t, 1.f)), sn = c * t;
            float *vp = Vl + (size_t)p * n, *vq = Vl + (size_t)q * n;
#pragma unroll
            for (int u = 0; u < K; u++) {
                const int i = lane + 32 * u;
                if (i < n) {
                    const float a = vp[i], b = vq[i];
                    xp[i] = c * x[u] - sn * y[u];
                    xq[i] = sn * x[u] + c * y[u];
                    vp[i] = c * a - sn * b;
                    vq[i] = sn * a + c * b;
                }
            }
        }
        __syncthreads();
    }
    if (lane == 0 && wmax > 0.f)
        atomicMax(off_bits + s, __float_as_uint(wmax));
#pragma unroll
    for (int u = 0; u < K; u++) {
        const int i = lane + 32 * u;
        if (i < n) {
            if (c0 < n) {
                Xg[(size_t)c0 * n + i] = Xl[(size_t)warp * n + i];
                Vg[(size_t)c0 * n + i] = Vl[(size_t)warp * n + i];
            }
            if (c1 < n) {
                Xg[(size_t)c1 * n + i] = Xl[(size_t)(warp + kBJ) * n + i];
                Vg[(size_t)c1 * n + i] = Vl[(size_t)(warp + kBJ) * n + i];
            }
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

constexpr int kQThreads = 256, kQCols = 4; // columns of Y per CTA

// Y = Q [P; 0] = H_0 H_1 ... H_{n-1} [P; 0] for kQCols columns of P per CTA
// (shared memory: kQCols x m floats), then out[:, perm[j]] = Y[:, j].
// grid (ceil(n / kQCols), n_sino).
__global__ void __launch_bounds__(kQThreads)
nos_apply_q_kernel(const float2 *__restrict__ A, const NosDesc *__restrict__ desc,
                   const double *__restrict__ tau, const int *__restrict__ perm,
                   const float *__restrict__ P, int n, float *__restrict__ out) {
    extern __shared__ __align__(16) unsigned char smraw[];
    float *y = reinterpret_cast<float *>(smraw);
    __shared__ float red[kQThreads / 32][kQCols];
    const int s = blockIdx.y, j0 = blockIdx.x * kQCols;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const NosDesc d = desc[s];
    const int m = d.m, nc = min(kQCols, n - j0);
    const size_t nn = (size_t)n * n;
    for (int c = 0; c < kQCols; c++)
        for (int i = threadIdx.x; i < m; i += kQThreads)
            y[c * m + i] = (c < nc && i < n) ? P[s * nn + i + (size_t)(j0 + c) * n] : 0.f;
    const float2 *As = A + d.a_off;
    const double *ts = tau + (size_t)s * n;
    for (int k = n - 1; k >= 0; k--) {
        const float t = (float)ts[k];
        if (t == 0.f)
            continue; // uniform
        const float2 *v = As + (size_t)k * m;
        __syncthreads();
        float w[kQCols];
#pragma unroll
        for (int c = 0; c < kQCols; c++)
            w[c] = 0.f;
        for (int i = k + 1 + threadIdx.x; i < m; i += kQThreads) {
            const float vi = (v[i].x + v[i].y);
#pragma unroll
            for (int c = 0; c < kQCols; c++)
                w[c] = fmaf(vi, y[c * m + i], w[c]);
        }
#pragma unroll
        for (int c = 0; c < kQCols; c++) {
            w[c] = warp_sum(w[c]);
            if (lane == 0)
                red[warp][c] = w[c];
        }
        __syncthreads();
#pragma unroll
        for (int c = 0; c < kQCols; c++) {
            float tot = y[c * m + k];
            for (int u = 0; u < kQThreads / 32; u++)
                tot += red[u][c];
            w[c] = t * tot;
        }
        __syncthreads(); // everyone has read y[.., k] and red
        for (int i = k + 1 + threadIdx.x; i < m; i += kQThreads) {
            const float vi = (v[i].x + v[i].y);
#pragma unroll
            for (int c = 0; c < kQCols; c++)
                y[c * m + i] = fmaf(-w[c], vi, y[c * m + i]);
        }
        if (threadIdx.x < kQCols)
            y[threadIdx.x * m + k] -= w[threadIdx.x];
    }
    __syncthreads();
    const int *pm = perm + (size_t)s * n;
    for (int c = 0; c < nc; c++) {
        float *o = out + d.out_off + (size_t)pm[j0 + c] * m;
        for (int i = threadIdx.x; i < m; i += kQThreads)
            o[i] = y[c * m + i];
    }
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

template <int K>
static void qr_steps(float2 *A, const NosDesc *desc, int n, int n_sino, const NosWork &w,
                     cudaStream_t st) {
    for (int k = 0; k < n; k++) {
        qr_pivot_kernel<K><<<n_sino, kQrThreads, 0, st>>>(A, desc, n, k, w.norms, w.orig, w.perm,
                                                          w.tau);
        if (k + 1 < n)
            qr_update_kernel<K><<<dim3(n - k - 1, n_sino), kQrThreads, 0, st>>>(
                A, desc, n, k, w.norms, w.orig, w.tau);
    }
}

int nos_max_rows() { return 32 * kQrThreads; }

cudaError_t launch_nos_factor(float2 *A, const NosDesc *desc, int n, int n_sino, int max_m,
                              const NosWork &w, cudaStream_t st) {
    if (max_m > nos_max_rows())
        return cudaErrorInvalidValue;
    qr_init_kernel<<<dim3(n, n_sino), kQrThreads, 0, st>>>(A, desc, n, w.norms, w.orig, w.perm);
    if (max_m <= 8 * kQrThreads)
        qr_steps<8>(A, desc, n, n_sino, w, st);
    else if (max_m <= 16 * kQrThreads)
        qr_steps<16>(A, desc, n, n_sino, w, st);
    else
        qr_steps<32>(A, desc, n, n_sino, w, st);
    const long long nn = (long long)n * n;
    nos_rt_kernel<<<dim3((unsigned)((nn + 255) / 256), n_sino), 256, 0, st>>>(A, desc, n, w.X,
                                                                              w.V, w.tiny);
    return cudaGetLastError();
}

template <int K> static cudaError_t block_rounds(int n, int n_sino, const NosWork &w,
                                                 cudaStream_t st) {
    const int nb = (n + kBJ - 1) / kBJ, nbp = nb + (nb & 1);
    const size_t smem = sizeof(float) * 2 * kBCols * (size_t)n;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(rt_block_round_kernel<K>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)dynamic_smem_limit(
                                                 (const void *)rt_block_round_kernel<K>));
        if (e != cudaSuccess)
            return e;
        attr = true;
    }
    if (smem > dynamic_smem_limit((const void *)rt_block_round_kernel<K>))
        return cudaErrorInvalidValue;
    for (int r = 0; r < nbp - 1; r++)
        rt_block_round_kernel<K><<<dim3(nbp / 2, n_sino), kBThreads, smem, st>>>(
            w.X, w.V, n, nbp, r, w.off_bits, w.tiny);
    return cudaGetLastError();
}

cudaError_t launch_nos_sweep(int n, int n_sino, const NosWork &w, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(w.off_bits, 0, sizeof(unsigned) * n_sino, st);
    if (e != cudaSuccess)
        return e;
    if (n <= 256)
        return block_rounds<8>(n, n_sino, w, st);
    if (n <= 384)
        return block_rounds<12>(n, n_sino, w, st);
    if (n <= 512)
        return block_rounds<16>(n, n_sino, w, st);
    if (n <= 768)
        return block_rounds<24>(n, n_sino, w, st);
    if (n <= 1024)
        return block_rounds<32>(n, n_sino, w, st);
    return cudaErrorInvalidValue; // more than 1024 angles
}

float nos_sweep_done_bound() { return kJacDone; }

size_t nos_apply_smem(int max_m) { return sizeof(float) * (size_t)kQCols * max_m; }

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
    static size_t limit = 0;
    if (limit == 0) {
        limit = dynamic_smem_limit((const void *)nos_apply_q_kernel);
        cudaError_t e = cudaFuncSetAttribute(nos_apply_q_kernel,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)limit);
        if (e != cudaSuccess)
            return e;
    }
    const size_t smem = nos_apply_smem(max_m);
    if (smem > limit)
        return cudaErrorInvalidValue;
    nos_apply_q_kernel<<<dim3((n + kQCols - 1) / kQCols, n_sino), kQThreads, smem, st>>>(
        A, desc, w.tau, w.perm, w.V, n, out);
    return cudaGetLastError();
}

} // namespace tt
