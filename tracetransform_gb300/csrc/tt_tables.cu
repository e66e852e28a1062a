// tt_tables.cu -- host-side tables of the P3 functional (no device code).
//
// PFunctional3 (c++/src/functionals.cpp:318-360) needs |F_p| of each
// sinogram column, F its real DFT.  The device computes the DFT of length N
// by the chirp-z identity on a power-of-two FFT of length M >= 2N - 1:
//   F_k = w_k sum_j (x_j w_j) conj(w_{k-j}),   w_j = exp(-i pi j^2 / N),
// so it needs the chirp w (N), the M-point FFT of the conjugate chirp divided
// by M (the convolution filter), the FFT twiddles exp(-2 pi i k / M) (M / 2)
// and the reference's linspace(-1, 1, N) rounded as it rounds it.  All are
// computed here in double and rounded once to float.
#include <cmath>
#include <complex>

#include "tt_internal.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

namespace tt {

int p3_fft_length(int n) {
    int m = 2;
    while (m < 2 * n - 1)
        m <<= 1;
    return m;
}

void fft_pow2(std::complex<double> *a, int n, int sign) {
    for (int i = 1, j = 0; i < n; i++) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1)
            j ^= bit;
        j ^= bit;
        if (i < j)
            std::swap(a[i], a[j]);
    }
    for (int len = 2; len <= n; len <<= 1) {
        for (int i = 0; i < n; i += len) {
            for (int k = 0; k < len / 2; k++) {
                const double ang = sign * 2.0 * M_PI * k / len;
                const std::complex<double> w(std::cos(ang), std::sin(ang));
                const std::complex<double> u = a[i + k], v = a[i + k + len / 2] * w;
                a[i + k] = u + v;
                a[i + k + len / 2] = u - v;
            }
        }
    }
}

void p3_tables(int n, float2 *chirp, float2 *filt, float2 *twid, float *lin,
               std::complex<double> *work) {
    const int m = p3_fft_length(n);
    for (int i = 0; i < m; i++)
        work[i] = 0.0;
    for (int j = 0; j < n; j++) {
        const long q = ((long)j * j) % (2L * n);
        const std::complex<double> w(std::cos(M_PI * q / n), -std::sin(M_PI * q / n));
        chirp[j] = make_float2((float)w.real(), (float)w.imag());
        work[j] = std::conj(w);
        if (j > 0)
            work[m - j] = std::conj(w);
    }
    fft_pow2(work, m, -1);
    for (int i = 0; i < m; i++)
        filt[i] = make_float2((float)(work[i].real() / m), (float)(work[i].imag() / m));
    for (int k = 0; k < m / 2; k++)
        twid[k] = make_float2((float)std::cos(-2.0 * M_PI * k / m),
                              (float)std::sin(-2.0 * M_PI * k / m));
    for (int p = 0; p < n; p++)
        lin[p] = (float)(-1 + p * 2.0 / (n - 1));
}

// pad() of c++/src/auxiliary.cpp:257-275: side N of the zero frame that holds
// every rotation of a rows x cols image, and the image's offset inside it
// (the reference's float origin and hypot arithmetic).
void pad_geometry(int rows, int cols, int *n, int *row_off, int *col_off) {
    const float ox = (float)(std::floor((cols + 1) / 2.0) - 1);
    const float oy = (float)(std::floor((rows + 1) / 2.0) - 1);
    const float hx = (float)(cols - 1) - ox - 1;
    const float hy = (float)(rows - 1) - oy - 1;
    const int r_last = (int)std::ceil(std::hypot(hx, hy)) + 1;
    const int nb = 2 * r_last + 1;
    const float opad = (float)(std::floor((nb + 1) / 2.0) - 1);
    *n = nb;
    *col_off = (int)(opad - ox);
    *row_off = (int)(opad - oy);
}

// (cos(-theta), sin(-theta)) of an angle in degrees, rounded as the reference
// rounds them: deg2rad on a float in double arithmetic (c++/src/auxiliary.cpp:
// 180), then std::cos / std::sin of the float (auxiliary.cpp:227-237).
float2 rotation(float degrees) {
    const float ang = (float)(degrees * M_PI / 180);
    return make_float2(std::cos(-ang), std::sin(-ang));
}

// T3, T4, T5 kernels r^k exp(i m log r), r = 1 .. n-1, in double and rounded
// once (c++/src/functionals.cpp:136-198); out holds 3 n entries, T3 first.
void t345_tables(int n, float2 *out) {
    for (int i = 0; i < 3 * n; i++)
        out[i] = make_float2(0.f, 0.f);
    for (int r = 1; r < n; r++) {
        out[r] = make_float2((float)(r * std::cos(5.0 * std::log((double)r))),
                             (float)(r * std::sin(5.0 * std::log((double)r))));
        out[n + r] = make_float2((float)std::cos(3.0 * std::log((double)r)),
                                 (float)std::sin(3.0 * std::log((double)r)));
        out[2 * n + r] =
            make_float2((float)(std::sqrt((double)r) * std::cos(4.0 * std::log((double)r))),
                        (float)(std::sqrt((double)r) * std::sin(4.0 * std::log((double)r))));
    }
}

} // namespace tt
