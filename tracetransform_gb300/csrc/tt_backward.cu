// tt_backward.cu -- gradients of circus functions with respect to the image.
//
// The reference has no derivative; this is the hand-written adjoint of the
// forward path for the functionals config 4 differentiates: T0, T1, T2
// (c++/src/functionals.cpp:95-129) and P1, P3 (:287-360), through the
// bilinear rotation (c++/src/auxiliary.cpp:182-255).
//
//   circus_backward   P-stage adjoint per sinogram column:
//                       P1:  d/dx_n sum|x_p - x_{p-1}| = sgn(x_n - x_{n-1}) - sgn(x_{n+1} - x_n)
//                       P3:  y_p = |F_m(p)|^4 / N^4 with the reference's mirror m(p),
//                            P3 = trapz(lin, y), so with w_p the trapz weights and
//                            d_k = 2 |F_k|^2 / N^4 sum_{m(p) = k} w_p,
//                            dP3/dx_n = sum_{k <= N/2} 2 d_k Re(conj(F_k) e^{-2 pi i k n / N})
//                     (float: both DFTs of a column by the chirp-z FFT on the
//                     forward's tables, O(M log M); double, and float columns
//                     whose FFT buffer exceeds shared memory: direct sums with an
//                     exact twiddle index)
//   line_params       per line (angle, column): (G0, G1, G2, m) with G_t the
//                     gradient of sinogram t at that entry and m the weighted
//                     median the forward used -- dT1/dx_j = (j - m)+,
//                     dT2/dx_j = (j - m)+^2, dT0/dx_j = 1
//   adjoint_gather    rotation adjoint in gather form: one thread per image
//                     pixel enumerates, per angle, the 3 x 3 rotated-grid
//                     points around its inverse-rotated position, recomputes
//                     their coordinates exactly as the forward did, and adds
//                     bilinear weight x line gradient for the points whose
//                     stencil holds the pixel (no atomics, deterministic;
//                     rotations are recomputed, never stored)
//
// Everything is templated on float / double.  The double instantiation, with
// the plain double forward below (sino_f64_kernel, circus_f64_kernel), is what
// the finite-difference check runs in.
#include <climits>

#include "tt_common.cuh"
#include "tt_internal.h"

namespace tt {
namespace {

template <typename T> struct Coord;
// The forward's coordinate arithmetic, bit for bit: q = (X c + Y s) + o,
// products and sums rounded one at a time (no contraction into FMAs), so the
// adjoint can hoist X c / Y s and still reproduce every coordinate.
template <> struct Coord<float> {
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ void q(float X, float Y, float c, float s, float o,
                                             float &qx, float &qy) {
        qx = add(add(mul(X, c), mul(Y, s)), o);
        qy = add(add(mul(X, -s), mul(Y, c)), o);
    }
};
template <> struct Coord<double> {
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ void q(double X, double Y, double c, double s, double o,
                                             double &qx, double &qy) {
        qx = add(add(mul(X, c), mul(Y, s)), o);
        qy = add(add(mul(X, -s), mul(Y, c)), o);
    }
};

template <typename T> __device__ __forceinline__ T sgn(T v) {
    return (T)((v > (T)0) - (v < (T)0));
}

template <typename T> __device__ __forceinline__ T block_sum_t(T v, T *red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1)
        v += __shfl_xor_sync(TT_FULL_MASK, v, d);
    __syncthreads();
    if (lane == 0)
        red[warp] = v;
    __syncthreads();
    T t = 0;
    for (int w = 0; w < nw; w++)
        t += red[w];
    return t;
}

template <typename T> struct CS {
    T c, s;
};

// P-stage adjoint.  Block per column (sinogram s, column a); dynamic shared
// memory: x (rows), F (2 * (rows / 2 + 1)), the weighted coefficients
// (2 * (rows / 2 + 1)), all of T, then -- when they fit -- the (cos, sin)
// twiddle pairs (2 * rows).  grad_circus: n_sino x n_p x cols; out: n_sino x
// cols x rows.
template <typename T>
__global__ void circus_backward_kernel(const T *__restrict__ sino, int rows, int cols,
                                       int n_sino, const int *__restrict__ kinds, int n_p,
                                       const T *__restrict__ grad_circus,
                                       const T *__restrict__ cosv, const T *__restrict__ sinv,
                                       const T *__restrict__ lin, bool tab_in_smem,
                                       T *__restrict__ out) {
    extern __shared__ __align__(16) unsigned char smraw[];
    T *x = reinterpret_cast<T *>(smraw);
    const int nb = rows / 2 + 1;
    T *Fr = x + rows, *Fi = Fr + nb, *wr = Fi + nb, *wi = wr + nb;
    const int a = blockIdx.x, s = blockIdx.y, tid = threadIdx.x, bd = blockDim.x;
    const T *col = sino + ((size_t)s * cols + a) * rows;
    for (int i = tid; i < rows; i += bd)
        x[i] = col[i];
    // twiddles (cos, sin)(2 pi i / rows), paired in shared memory when they fit
    const int tw_off = (rows + 4 * nb + 1) & ~1; // pairs start at an even T
    CS<T> *tw = reinterpret_cast<CS<T> *>(x + tw_off);
    if (tab_in_smem)
        for (int i = tid; i < rows; i += bd)
            tw[i] = CS<T>{cosv[i], sinv[i]};
    auto twid = [&](long idx) {
        return tab_in_smem ? tw[idx] : CS<T>{__ldg(cosv + idx), __ldg(sinv + idx)};
    };
    T g1 = 0, g3 = 0;
    for (int p = 0; p < n_p; p++) {
        const T g = grad_circus[((size_t)s * n_p + p) * cols + a];
        if (kinds[p] == 1)
            g1 += g;
        else if (kinds[p] == 3)
            g3 += g;
    }
    __syncthreads();
    if (g3 != (T)0) {
        // F_k, k <= N/2 (twiddle index k n mod N)
        for (int k = tid; k < nb; k += bd) {
            T re = 0, im = 0;
            long idx = 0;
            for (int n = 0; n < rows; n++) {
                const CS<T> w = twid(idx);
                re += x[n] * w.c;
                im -= x[n] * w.s;
                idx += k;
                if (idx >= rows)
                    idx -= rows;
            }
            Fr[k] = re;
            Fi[k] = im;
        }
        __syncthreads();
        // d_k = 2 |F_k|^2 / N^4 * sum of trapz weights of the p that read bin k;
        // the inverse sum below takes 2 d_k F_k
        const T n4 = (T)rows * rows * rows * rows;
        for (int k = tid; k < nb; k += bd) {
            T wsum = 0;
            const int ps[2] = {k, rows - k};
            for (int u = 0; u < 2; u++) {
                const int p = ps[u];
                if (p < 0 || p >= rows || (u == 1 && (p <= rows / 2 || p == k)))
                    continue;
                T w = 0;
                if (p + 1 <= rows - 1)
                    w += (T)0.5 * (lin[p + 1] - lin[p]);
                if (p >= 1)
                    w += (T)0.5 * (lin[p] - lin[p - 1]);
                wsum += w;
            }
            const T dk = (T)2 * (Fr[k] * Fr[k] + Fi[k] * Fi[k]) / n4 * wsum;
            wr[k] = (T)2 * dk * Fr[k];
            wi[k] = (T)2 * dk * Fi[k];
        }
        __syncthreads();
    }
    for (int n = tid; n < rows; n += bd) {
        T g = 0;
        if (g1 != (T)0) {
            T v = 0;
            if (n >= 1)
                v += sgn(x[n] - x[n - 1]);
            if (n + 1 < rows)
                v -= sgn(x[n + 1] - x[n]);
            g += g1 * v;
        }
        if (g3 != (T)0) {
            // sum_k 2 d_k Re(conj(F_k) e^{-2 pi i k n / N})
            //     = sum_k 2 d_k (Fr cos(2 pi k n / N) - Fi sin(2 pi k n / N))
            T acc = 0;
            long idx = 0;
            for (int k = 0; k < nb; k++) {
                const CS<T> w = twid(idx);
                acc += wr[k] * w.c - wi[k] * w.s;
                idx += n;
                if (idx >= rows)
                    idx -= rows;
            }
            g += g3 * acc;
        }
        out[((size_t)s * cols + a) * rows + n] = g;
    }
}

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// In-place chirp-z convolution step on M = 2^logM points: forward radix-2
// DIT of the bit-reversed input (natural-order result), times the filter,
// inverse radix-2 DIF with conjugate twiddles (bit-reversed result).  The
// input must be scattered to fft[brev(j)] before; every thread calls it.
__device__ void chirp_convolve(float2 *fft, int M, const float2 *__restrict__ twid,
                               const float2 *__restrict__ filt) {
    const int tid = threadIdx.x, bd = blockDim.x;
    for (int h = 1; h < M; h <<= 1) {
        const int tstep = M / (2 * h);
        for (int i = tid; i < M / 2; i += bd) {
            const int pos = i & (h - 1);
            const int ia = ((i - pos) << 1) + pos, ib = ia + h;
            const float2 t = cmulf(fft[ib], __ldg(twid + pos * tstep));
            const float2 u = fft[ia];
            fft[ia] = make_float2(u.x + t.x, u.y + t.y);
            fft[ib] = make_float2(u.x - t.x, u.y - t.y);
        }
        __syncthreads();
    }
    for (int i = tid; i < M; i += bd)
        fft[i] = cmulf(fft[i], __ldg(filt + i));
    __syncthreads();
    for (int h = M / 2; h >= 1; h >>= 1) {
        const int tstep = M / (2 * h);
        for (int i = tid; i < M / 2; i += bd) {
            const int pos = i & (h - 1);
            const int ia = ((i - pos) << 1) + pos, ib = ia + h;
            const float2 u = fft[ia], w = fft[ib];
            const float2 tw = __ldg(twid + pos * tstep);
            fft[ia] = make_float2(u.x + w.x, u.y + w.y);
            fft[ib] = cmulf(make_float2(u.x - w.x, u.y - w.y), make_float2(tw.x, -tw.y));
        }
        __syncthreads();
    }
}

// The float P-stage adjoint with both DFTs of a column by the chirp-z
// identity (the forward's tables: chirp w_j = exp(-i pi j^2 / N), the
// M-point filter and twiddles, M >= 2N - 1 a power of two), O(M log M) per
// column instead of the direct sums' O(N^2):
//   F_k = w_k conv(x w, conj w)_k                     (k <= N/2)
//   W_k = 2 d_k F_k,  dP3/dx_n = Re sum_k W_k e^{2 pi i k n / N}
//       = Re w_n conv(conj(W) w, conj w)_n            (n < N)
// Block per column; dynamic shared memory: the M-point buffer, x (rows) and
// W (N/2 + 1 pairs).
__global__ void circus_backward_fft_kernel(const float *__restrict__ sino, int rows, int cols,
                                           const int *__restrict__ kinds, int n_p,
                                           const float *__restrict__ grad_circus,
                                           const float2 *__restrict__ chirp,
                                           const float2 *__restrict__ filt,
                                           const float2 *__restrict__ twid, int M,
                                           const float *__restrict__ lin,
                                           float *__restrict__ out) {
    extern __shared__ __align__(16) unsigned char smraw[];
    float2 *fft = reinterpret_cast<float2 *>(smraw);
    const int nb = rows / 2 + 1;
    float2 *W = fft + M;
    float *x = reinterpret_cast<float *>(W + nb);
    const int a = blockIdx.x, s = blockIdx.y, tid = threadIdx.x, bd = blockDim.x;
    const int logM = 31 - __clz(M);
    const float *col = sino + ((size_t)s * cols + a) * rows;
    for (int i = tid; i < rows; i += bd)
        x[i] = col[i];
    float g1 = 0.f, g3 = 0.f;
    for (int p = 0; p < n_p; p++) {
        const float g = grad_circus[((size_t)s * n_p + p) * cols + a];
        if (kinds[p] == 1)
            g1 += g;
        else if (kinds[p] == 3)
            g3 += g;
    }
    if (g3 != 0.f) {
        for (int i = tid; i < M; i += bd)
            fft[i] = make_float2(0.f, 0.f);
        __syncthreads();
        for (int j = tid; j < rows; j += bd) {
            const float2 w = __ldg(chirp + j);
            fft[__brev(j) >> (32 - logM)] = make_float2(x[j] * w.x, x[j] * w.y);
        }
        __syncthreads();
        chirp_convolve(fft, M, twid, filt);
        const float n4 = (float)rows * rows * (float)rows * rows;
        for (int k = tid; k < nb; k += bd) {
            const float2 F = cmulf(fft[__brev(k) >> (32 - logM)], __ldg(chirp + k));
            float wsum = 0.f;
            const int ps[2] = {k, rows - k};
            for (int u = 0; u < 2; u++) {
                const int p = ps[u];
                if (p < 0 || p >= rows || (u == 1 && (p <= rows / 2 || p == k)))
                    continue;
                if (p + 1 <= rows - 1)
                    wsum += 0.5f * (__ldg(lin + p + 1) - __ldg(lin + p));
                if (p >= 1)
                    wsum += 0.5f * (__ldg(lin + p) - __ldg(lin + p - 1));
            }
            const float dk2 = 4.f * (F.x * F.x + F.y * F.y) / n4 * wsum; // 2 d_k
            W[k] = make_float2(dk2 * F.x, dk2 * F.y);
        }
        __syncthreads();
        for (int i = tid; i < M; i += bd)
            fft[i] = make_float2(0.f, 0.f);
        __syncthreads();
        for (int k = tid; k < nb; k += bd) {
            const float2 w = __ldg(chirp + k);
            fft[__brev(k) >> (32 - logM)] = cmulf(make_float2(W[k].x, -W[k].y), w);
        }
        __syncthreads();
        chirp_convolve(fft, M, twid, filt);
    } else {
        __syncthreads();
    }
    for (int n = tid; n < rows; n += bd) {
        float g = 0.f;
        if (g1 != 0.f) {
            float v = 0.f;
            if (n >= 1)
                v += sgn(x[n] - x[n - 1]);
            if (n + 1 < rows)
                v -= sgn(x[n + 1] - x[n]);
            g += g1 * v;
        }
        if (g3 != 0.f)
            g += g3 * cmulf(fft[__brev(n) >> (32 - logM)], __ldg(chirp + n)).x;
        out[((size_t)s * cols + a) * rows + n] = g;
    }
}

// (G0, G1, G2, m) per line (image, angle a, column col): grad_sino holds
// n_images stacks of n_t x A x n, medians the same (the forward's
// weighted-median rows); params: n_images x A x n x 4.
template <typename T>
__global__ void line_params_kernel(const T *__restrict__ grad_sino,
                                   const int *__restrict__ medians, int n_images, int n,
                                   int n_angles, unsigned long long tf_code, int n_t,
                                   T *__restrict__ params) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long plane = (long long)n * n_angles;
    if (i >= plane * n_images)
        return;
    const long long img = i / plane, at = i - img * plane;
    const long long base = img * n_t * plane + at;
    T g[3] = {0, 0, 0};
    int m = 0;
    for (int t = 0; t < n_t; t++) {
        const int f = (int)((tf_code >> (3 * t)) & 7ull);
        g[f] += grad_sino[base + t * plane];
        if (f == 1 || f == 2)
            m = medians[base + t * plane];
    }
    params[4 * i + 0] = g[0];
    params[4 * i + 1] = g[1];
    params[4 * i + 2] = g[2];
    params[4 * i + 3] = (T)m;
}

template <typename T> struct Quad;
template <> struct Quad<float> {
    static __device__ __forceinline__ void load(const float *p, float &a, float &b, float &c,
                                                float &d) {
        const float4 v = __ldg(reinterpret_cast<const float4 *>(p));
        a = v.x; b = v.y; c = v.z; d = v.w;
    }
};
template <> struct Quad<double> {
    static __device__ __forceinline__ void load(const double *p, double &a, double &b,
                                                double &c, double &d) {
        const double2 u = __ldg(reinterpret_cast<const double2 *>(p));
        const double2 v = __ldg(reinterpret_cast<const double2 *>(p) + 1);
        a = u.x; b = u.y; c = v.x; d = v.y;
    }
};

constexpr int kAdjWarps = 8; // angle groups per pixel group

// Rotation adjoint by gathering.  Pixel (r, c) of a rows x cols image sits at
// frame point (px, py) = (c + col_off, r + row_off).  A rotated-grid point
// (column cc, sample j) with frame coordinates q = (qx, qy) feeds it the
// bilinear weight (1 - |qx - px|)+ (1 - |qy - py|)+ -- the forward's
// (1 - xf) or xf factor exactly, since qx - px and 1 - |qx - px| are exact in
// floating point for |qx - px| < 1 -- provided the forward sampled q at all
// (0 <= qx, qy < n - 1).  Such points lie within sqrt(2) of the pixel's
// inverse-rotated position, i.e. in the 3 x 3 lattice block around its
// nearest lattice point; each is recomputed with the forward's arithmetic.
//
// kInterior: the image lies at least two pixels inside its frame, so a
// candidate with non-zero weight (within a unit of the pixel on both axes)
// lies inside [1, n - 2] and always passed the forward's bounds test; only
// the grid indices still need their range checks.
//
// CTA: 32 consecutive pixels (lanes) x kAdjWarps warps; warp w sums the angles
// a = w (mod kAdjWarps) in increasing order and the warps' partial sums are
// added in warp order, so the result is deterministic.  blockIdx.y = image.
template <typename T, bool kInterior>
__global__ void __launch_bounds__(32 * kAdjWarps)
adjoint_gather_kernel(int rows, int cols, int row_off, int col_off, int n, int n_angles,
                      const T *__restrict__ cs, const T *__restrict__ params,
                      T *__restrict__ grad_img) {
    using C = Coord<T>;
    __shared__ T part[kAdjWarps][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long pix = (long long)rows * cols;
    const long long i = (long long)blockIdx.x * 32 + lane;
    params += (size_t)blockIdx.y * 4 * (size_t)n * n_angles;
    T acc = 0;
    const unsigned live = __ballot_sync(TT_FULL_MASK, i < pix);
    if (i < pix) {
        const int r = (int)(i % rows), c = (int)(i / rows);
        const T fpx = (T)(c + col_off), fpy = (T)(r + row_off);
        const T o = (T)(n - 1) * (T)0.5, nm1 = (T)(n - 1);
        const T dx = fpx - o, dy = fpy - o;
        for (int a = warp; a < n_angles; a += kAdjWarps) {
            const T ca = __ldg(cs + 2 * a), sa = __ldg(cs + 2 * a + 1);
            // inverse of (X, Y) -> (X c + Y s, -X s + Y c), nearest lattice point
            const int c0 = (int)rint(ca * dx - sa * dy + o);
            const int j0 = (int)rint(sa * dx + ca * dy + o);
            T ys[3], yc[3];
#pragma unroll
            for (int u = 0; u < 3; u++) {
                const T Y = (T)(j0 - 1 + u) - o;
                ys[u] = C::mul(Y, sa);
                yc[u] = C::mul(Y, ca);
            }
            const T *pa = params + (size_t)4 * a * n;
            // every lane's 3 x 3 block inside the lattice (all but the frame's
            // corners): no per-candidate index checks
            const bool inner = (unsigned)(c0 - 1) < (unsigned)(n - 2) &&
                               (unsigned)(j0 - 1) < (unsigned)(n - 2);
            if (kInterior && __all_sync(live, inner)) {
#pragma unroll
                for (int v = 0; v < 3; v++) {
                    const int cc = c0 - 1 + v;
                    T g0, g1, g2, mf;
                    Quad<T>::load(pa + 4 * cc, g0, g1, g2, mf);
                    const T X = (T)cc - o;
                    const T xc = C::mul(X, ca), xs = C::mul(X, -sa);
#pragma unroll
                    for (int u = 0; u < 3; u++) {
                        const T qx = C::add(C::add(xc, ys[u]), o);
                        const T qy = C::add(C::add(xs, yc[u]), o);
                        const T wx = fmax((T)1 - fabs(qx - fpx), (T)0);
                        const T wy = fmax((T)1 - fabs(qy - fpy), (T)0);
                        const T rr = (T)(j0 - 1 + u) - mf;
                        const T g = rr >= (T)0 ? g0 + rr * (g1 + rr * g2) : g0;
                        acc += wx * wy * g;
                    }
                }
                continue;
            }
#pragma unroll
            for (int v = 0; v < 3; v++) {
                const int cc = c0 - 1 + v;
                if (cc < 0 || cc >= n)
                    continue;
                T g0, g1, g2, mf;
                Quad<T>::load(pa + 4 * cc, g0, g1, g2, mf);
                const T X = (T)cc - o;
                const T xc = C::mul(X, ca), xs = C::mul(X, -sa);
#pragma unroll
                for (int u = 0; u < 3; u++) {
                    const int j = j0 - 1 + u;
                    const T qx = C::add(C::add(xc, ys[u]), o);
                    const T qy = C::add(C::add(xs, yc[u]), o);
                    // (1 - |qx - px|)+ (1 - |qy - py|)+: zero outside the stencil
                    const T wx = fmax((T)1 - fabs(qx - fpx), (T)0);
                    const T wy = fmax((T)1 - fabs(qy - fpy), (T)0);
                    const T rr = (T)j - mf;
                    const T g = rr >= (T)0 ? g0 + rr * (g1 + rr * g2) : g0;
                    if (kInterior) {
                        acc += (j >= 0 && j < n) ? wx * wy * g : (T)0;
                    } else {
                        const bool in = j >= 0 && j < n && qx >= (T)0 && qx < nm1 &&
                                        qy >= (T)0 && qy < nm1;
                        acc += in ? wx * wy * g : (T)0;
                    }
                }
            }
        }
    }
    part[warp][lane] = acc;
    __syncthreads();
    if (warp == 0 && i < pix) {
        T t = part[0][lane];
#pragma unroll
        for (int w = 1; w < kAdjWarps; w++)
            t += part[w][lane];
        grad_img[(size_t)blockIdx.y * pix + i] = t;
    }
}

// ---- plain double-precision forward (for the finite-difference check) ----

// Sinograms T0, T1, T2 of a rows x cols double image in its pad() frame,
// computed in double: block per line (angle, column), samples in shared
// memory (n doubles), one thread sums.  out / medians: n_t x A x n.
__global__ void sino_f64_kernel(const double *__restrict__ img, int rows, int cols,
                                int row_off, int col_off, int n, const double *__restrict__ cs,
                                unsigned long long tf_code, int n_t, int n_angles,
                                double *__restrict__ out, int *__restrict__ medians) {
    extern __shared__ __align__(16) unsigned char smraw[];
    double *x = reinterpret_cast<double *>(smraw);
    const int col = blockIdx.x, a = blockIdx.y;
    const double o = (n - 1) * 0.5, nm1 = n - 1;
    const double ca = cs[2 * a], sa = cs[2 * a + 1];
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        double qx, qy;
        Coord<double>::q(col - o, j - o, ca, sa, o, qx, qy);
        double v = 0;
        if (qx >= 0 && qx < nm1 && qy >= 0 && qy < nm1) {
            const double xi = trunc(qx), yi = trunc(qy), xf = qx - xi, yf = qy - yi;
            const int x0 = (int)xi - col_off, y0 = (int)yi - row_off;
            double tap[4] = {0, 0, 0, 0};
            for (int u = 0; u < 4; u++) {
                const int xx = x0 + (u & 1), yy = y0 + (u >> 1);
                if (xx >= 0 && xx < cols && yy >= 0 && yy < rows)
                    tap[u] = img[yy + (size_t)xx * rows];
            }
            v = tap[0] * (1 - xf) * (1 - yf) + tap[1] * xf * (1 - yf) + tap[2] * (1 - xf) * yf +
                tap[3] * xf * yf;
        }
        x[j] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double S = 0;
        for (int j = 0; j < n; j++)
            S += x[j];
        int m = n - 1;
        double run = 0;
        for (int j = 0; j < n; j++) {
            run += x[j];
            if (2 * run >= S) {
                m = j;
                break;
            }
        }
        double t1 = 0, t2 = 0;
        for (int j = m; j < n; j++) {
            t1 += x[j] * (j - m);
            t2 += x[j] * (double)(j - m) * (j - m);
        }
        const size_t plane = (size_t)n_angles * n, at = (size_t)a * n + col;
        for (int t = 0; t < n_t; t++) {
            const int f = (int)((tf_code >> (3 * t)) & 7ull);
            out[t * plane + at] = f == 0 ? S : f == 1 ? t1 : t2;
            medians[t * plane + at] = f == 0 ? -1 : m;
        }
    }
}

// P1 and P3 of double sinogram columns (direct DFT), block per column.
__global__ void circus_f64_kernel(const double *__restrict__ sino, int rows, int cols,
                                  const int *__restrict__ kinds, int n_p,
                                  const double *__restrict__ cosv, const double *__restrict__ sinv,
                                  const double *__restrict__ lin, double *__restrict__ out) {
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ double red[8];
    double *x = reinterpret_cast<double *>(smraw);
    double *y = x + rows;
    const int a = blockIdx.x, s = blockIdx.y, tid = threadIdx.x, bd = blockDim.x;
    const double *colp = sino + ((size_t)s * cols + a) * rows;
    for (int i = tid; i < rows; i += bd)
        x[i] = colp[i];
    __syncthreads();
    const int nb = rows / 2 + 1;
    for (int k = tid; k < nb; k += bd) {
        double re = 0, im = 0;
        long idx = 0;
        for (int j = 0; j < rows; j++) {
            re += x[j] * cosv[idx];
            im -= x[j] * sinv[idx];
            idx += k;
            if (idx >= rows)
                idx -= rows;
        }
        const double h2 = (re * re + im * im) / ((double)rows * rows);
        y[k] = h2 * h2;
    }
    __syncthreads();
    double p1 = 0, p3 = 0;
    for (int i = tid; i < rows; i += bd) {
        if (i >= 1)
            p1 += fabs(x[i] - x[i - 1]);
        if (i + 1 < rows) {
            const int m0 = i <= rows / 2 ? i : rows - i;
            const int m1 = i + 1 <= rows / 2 ? i + 1 : rows - (i + 1);
            p3 += 0.5 * (lin[i + 1] - lin[i]) * (y[m1] + y[m0]);
        }
    }
    p1 = block_sum_t(p1, red);
    p3 = block_sum_t(p3, red);
    if (tid == 0)
        for (int p = 0; p < n_p; p++)
            out[((size_t)s * n_p + p) * cols + a] = kinds[p] == 1 ? p1 : kinds[p] == 3 ? p3 : 0;
}

} // namespace

template <typename T>
cudaError_t launch_circus_backward(const T *sino, int rows, int cols, int n_sino,
                                   const int *d_kinds, int n_p, const T *grad_circus,
                                   const T *cosv, const T *sinv, const T *lin, T *out,
                                   cudaStream_t st) {
    if (rows <= 0 || cols <= 0 || n_sino <= 0)
        return cudaSuccess;
    // x, F (re, im), 2 d F (re, im); the twiddle pairs after, at an even offset
    const size_t head = (size_t)rows + 4 * (size_t)(rows / 2 + 1);
    const size_t base = sizeof(T) * ((head + 1) & ~size_t(1));
    const size_t with_tab = base + sizeof(T) * 2 * (size_t)rows;
    const size_t limit = opt_in_smem((const void *)circus_backward_kernel<T>);
    if (limit == 0)
        return cudaErrorInvalidValue;
    const bool tab = with_tab <= limit;
    const size_t smem = tab ? with_tab : base;
    if (smem > limit)
        return cudaErrorInvalidValue;
    circus_backward_kernel<T><<<dim3(cols, n_sino), 256, smem, st>>>(
        sino, rows, cols, n_sino, d_kinds, n_p, grad_circus, cosv, sinv, lin, tab, out);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_sino_backward(const T *grad_sino, const int *medians, int n_images, int n,
                                 int n_angles, unsigned long long tf_code, int n_t, T *params,
                                 int rows, int cols, int row_off, int col_off, const T *cs,
                                 T *grad_img, cudaStream_t st) {
    if (n_images <= 0)
        return cudaSuccess;
    const long long lines = (long long)n * n_angles * n_images, pix = (long long)rows * cols;
    if (lines > 0)
        line_params_kernel<T><<<(unsigned)((lines + 255) / 256), 256, 0, st>>>(
            grad_sino, medians, n_images, n, n_angles, tf_code, n_t, params);
    if (pix > 0) {
        const dim3 grid((unsigned)((pix + 31) / 32), n_images);
        if (interior_source(n, row_off, col_off, rows, cols))
            adjoint_gather_kernel<T, true><<<grid, 32 * kAdjWarps, 0, st>>>(
                rows, cols, row_off, col_off, n, n_angles, cs, params, grad_img);
        else
            adjoint_gather_kernel<T, false><<<grid, 32 * kAdjWarps, 0, st>>>(
                rows, cols, row_off, col_off, n, n_angles, cs, params, grad_img);
    }
    return cudaGetLastError();
}

cudaError_t launch_sino_f64(const double *img, int rows, int cols, int row_off, int col_off,
                            int n, const double *cs, unsigned long long tf_code, int n_t,
                            int n_angles, double *out, int *medians, cudaStream_t st) {
    if (n <= 0 || n_angles <= 0)
        return cudaSuccess;
    const size_t smem = sizeof(double) * (size_t)n;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(sino_f64_kernel,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess)
            return e;
    }
    sino_f64_kernel<<<dim3(n, n_angles), 128, smem, st>>>(img, rows, cols, row_off, col_off, n,
                                                           cs, tf_code, n_t, n_angles, out,
                                                           medians);
    return cudaGetLastError();
}

cudaError_t launch_circus_f64(const double *sino, int rows, int cols, int n_sino,
                              const int *d_kinds, int n_p, const double *cosv,
                              const double *sinv, const double *lin, double *out,
                              cudaStream_t st) {
    if (rows <= 0 || cols <= 0 || n_sino <= 0)
        return cudaSuccess;
    const size_t smem = sizeof(double) * ((size_t)rows + rows / 2 + 1);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(circus_f64_kernel,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess)
            return e;
    }
    circus_f64_kernel<<<dim3(cols, n_sino), 256, smem, st>>>(sino, rows, cols, d_kinds, n_p, cosv,
                                                             sinv, lin, out);
    return cudaGetLastError();
}

cudaError_t launch_circus_backward_fft(const float *sino, int rows, int cols, int n_sino,
                                       const int *d_kinds, int n_p, const float *grad_circus,
                                       const float2 *chirp, const float2 *filt,
                                       const float2 *twid, int M, const float *lin, float *out,
                                       cudaStream_t st) {
    if (rows <= 0 || cols <= 0 || n_sino <= 0)
        return cudaSuccess;
    const size_t smem = circus_backward_fft_smem(rows, M);
    const size_t limit = opt_in_smem((const void *)circus_backward_fft_kernel);
    if (limit == 0 || smem > limit || M < 2 * rows - 1 || (M & (M - 1)))
        return cudaErrorInvalidValue;
    circus_backward_fft_kernel<<<dim3(cols, n_sino), 512, smem, st>>>(
        sino, rows, cols, d_kinds, n_p, grad_circus, chirp, filt, twid, M, lin, out);
    return cudaGetLastError();
}

size_t circus_backward_fft_smem(int rows, int M) {
    return sizeof(float2) * ((size_t)M + rows / 2 + 1) + sizeof(float) * (size_t)rows;
}

bool circus_backward_fft_fits(int rows, int M) {
    return circus_backward_fft_smem(rows, M) <=
           opt_in_smem((const void *)circus_backward_fft_kernel);
}

template cudaError_t launch_circus_backward<float>(const float *, int, int, int, const int *, int,
                                                   const float *, const float *, const float *,
                                                   const float *, float *, cudaStream_t);
template cudaError_t launch_circus_backward<double>(const double *, int, int, int, const int *,
                                                    int, const double *, const double *,
                                                    const double *, const double *, double *,
                                                    cudaStream_t);
template cudaError_t launch_sino_backward<float>(const float *, const int *, int, int, int,
                                                 unsigned long long, int, float *, int, int, int,
                                                 int, const float *, float *, cudaStream_t);
template cudaError_t launch_sino_backward<double>(const double *, const int *, int, int, int,
                                                  unsigned long long, int, double *, int, int, int,
                                                  int, const double *, double *, cudaStream_t);

} // namespace tt
