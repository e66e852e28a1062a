/*
 * tt_oracle.c -- CPU restatement of the reference trace-transform float path.
 *
 * TEST INFRASTRUCTURE ONLY (parity checker and timed CPU baseline).  The
 * product never links it.  Build with -ffp-contract=off so that no multiply
 * and add are fused: the reference's x86-64 build has no FMA contraction.
 *
 * Citations are file:line in maleadt/tracetransform.
 */
#include "tt_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------------
 * auxiliary.cpp
 * ---------------------------------------------------------------------- */

/* c++/src/auxiliary.cpp:180 -- float in, double arithmetic, float out. */
float tto_deg2rad(float degrees) { return (float)(degrees * M_PI / 180); }

/* c++/src/auxiliary.cpp:227-237 -- the matrix [[c, -s], [s, c]] is built
 * from std::cos(-angle) / std::sin(-angle) on a float, i.e. cosf / sinf. */
void tto_rotation(float angle, float *c, float *s) {
    *c = cosf(-angle);
    *s = sinf(-angle);
}

/* c++/src/auxiliary.cpp:257-275 */
void tto_pad_geometry(int rows, int cols, int *n, int *row_off, int *col_off) {
    float ox = (float)(floor((cols + 1) / 2.0) - 1);
    float oy = (float)(floor((rows + 1) / 2.0) - 1);
    /* Eigen Index minus float: float arithmetic, then float hypot/ceil. */
    float hx = (float)(cols - 1) - ox - 1;
    float hy = (float)(rows - 1) - oy - 1;
    int r_last = (int)ceilf(hypotf(hx, hy)) + 1;
    int n_bins = 2 * r_last + 1;
    float opad = (float)(floor((n_bins + 1) / 2.0) - 1);
    *n = n_bins;
    *col_off = (int)(opad - ox);
    *row_off = (int)(opad - oy);
}

void tto_pad(const float *image, int rows, int cols, float *out) {
    int n, ro, co;
    tto_pad_geometry(rows, cols, &n, &ro, &co);
    memset(out, 0, sizeof(float) * (size_t)n * n);
    for (int c = 0; c < cols; c++)
        for (int r = 0; r < rows; r++)
            out[(size_t)(r + ro) + (size_t)(c + co) * n] =
                image[(size_t)r + (size_t)c * rows];
}

/* c++/src/auxiliary.cpp:182-196 -- modf split, then the four-term bilinear
 * expression evaluated left to right. */
static float interpolate(const float *src, int rows, float px, float py) {
    float xi, yi;
    float xf = modff(px, &xi);
    float yf = modff(py, &yi);
    size_t x0 = (size_t)xi, y0 = (size_t)yi;
    float s00 = src[y0 + x0 * rows];
    float s01 = src[y0 + (x0 + 1) * rows];
    float s10 = src[(y0 + 1) + x0 * rows];
    float s11 = src[(y0 + 1) + (x0 + 1) * rows];
    return s00 * (1 - xf) * (1 - yf) + s01 * xf * (1 - yf) +
           s10 * (1 - xf) * yf + s11 * xf * yf;
}

/* c++/src/auxiliary.cpp:198-221 (square transform as the reference builds it:
 * the x coordinate is scaled by the row ratio, y by the column ratio). */
void tto_resize(const float *in, int in_rows, int in_cols, int rows, int cols,
                float *out) {
    float t00 = ((float)in_rows) / rows;
    float t11 = ((float)in_cols) / cols;
    memset(out, 0, sizeof(float) * (size_t)rows * cols);
    for (int col = 1; col < cols - 1; col++) {
        for (int row = 1; row < rows - 1; row++) {
            float px = (float)col + 0.5f, py = (float)row + 0.5f;
            /* row vector times [[t00, 0], [0, t11]] */
            float qx = px * t00 + py * 0.0f;
            float qy = px * 0.0f + py * t11;
            qx = qx - 0.5f;
            qy = qy - 0.5f;
            if (qx < 0 || qy < 0 || qx >= in_cols - 1 || qy >= in_rows - 1) {
                /* outside the reference's asserted domain: never produced for
                 * down-scaling or up-scaling below 3x */
                continue;
            }
            out[(size_t)row + (size_t)col * rows] =
                interpolate(in, in_rows, qx, qy);
        }
    }
}

/* c++/src/auxiliary.cpp:223-255, origin ((cols-1)/2, (rows-1)/2) as
 * getSinograms passes it (c++/src/sinogram.cpp:73-74). */
void tto_rotate(const float *in, int rows, int cols, float angle, float *out) {
    float c, s;
    tto_rotation(angle, &c, &s);
    float ms = -s;
    float ox = (float)((cols - 1) / 2.0), oy = (float)((rows - 1) / 2.0);
    for (int col = 0; col < cols; col++) {
        for (int row = 0; row < rows; row++) {
            float x = (float)col - ox, y = (float)row - oy;
            float qx = x * c + y * s;
            float qy = x * ms + y * c;
            qx = qx + ox;
            qy = qy + oy;
            float v = 0;
            if (qx >= 0 && qx < cols - 1 && qy >= 0 && qy < rows - 1)
                v = interpolate(in, rows, qx, qy);
            out[(size_t)row + (size_t)col * rows] = v;
        }
    }
}

/* c++/src/auxiliary.cpp:277-287 */
float tto_arithmetic_mean(const float *x, int n) {
    if (n == 0)
        return NAN;
    float sum = 0;
    for (int i = 0; i < n; i++)
        sum += x[i];
    return sum / (float)n;
}

/* c++/src/auxiliary.cpp:289-303 */
float tto_standard_deviation(const float *x, int n) {
    if (n <= 0)
        return NAN;
    float mean = tto_arithmetic_mean(x, n);
    double sum = 0;
    for (int i = 0; i < n; i++) {
        double diff = x[i] - mean;
        sum += diff * diff;
    }
    return (float)sqrt(sum / (n - 1));
}

/* c++/src/auxiliary.cpp:305-318 */
void tto_zscore(const float *x, int n, float *out) {
    if (n == 0)
        return;
    float mean = tto_arithmetic_mean(x, n);
    float stdev = tto_standard_deviation(x, n);
    for (int i = 0; i < n; i++)
        out[i] = (x[i] - mean) / stdev;
}

/* ------------------------------------------------------------------------
 * functionals.cpp
 * ---------------------------------------------------------------------- */

/* Sum in storage order.  The reference calls Eigen's data.sum(); Eigen is not
 * available here, and its vectorised reduction order is not reproduced. */
static float seq_sum(const float *x, int n) {
    float s = 0;
    for (int i = 0; i < n; i++)
        s += x[i];
    return s;
}

/* c++/src/functionals.cpp:21-30 */
int tto_find_weighted_median(const float *x, int n) {
    float sum = seq_sum(x, n);
    float integral = 0;
    for (int i = 0; i < n; i++) {
        integral += x[i];
        if (2 * integral >= sum)
            return i;
    }
    return n - 1;
}

static int weighted_median_sqrt(const float *x, int n, float *scratch) {
    for (int i = 0; i < n; i++)
        scratch[i] = sqrtf(x[i]);
    return tto_find_weighted_median(scratch, n);
}

/* c++/src/functionals.cpp:95-97 */
float tto_t_radon(const float *x, int n) { return seq_sum(x, n); }

/* c++/src/functionals.cpp:104-113 */
static float t1_at(const float *x, int n, int median) {
    float integral = 0;
    for (int r = 0; r < n - median; r++)
        integral += x[r + median] * (float)r;
    return integral;
}
float tto_t1(const float *x, int n) {
    return t1_at(x, n, tto_find_weighted_median(x, n));
}

/* c++/src/functionals.cpp:120-129 */
static float t2_at(const float *x, int n, int median) {
    float integral = 0;
    for (int r = 0; r < n - median; r++)
        integral += x[r + median] * (float)r * (float)r;
    return integral;
}
float tto_t2(const float *x, int n) {
    return t2_at(x, n, tto_find_weighted_median(x, n));
}

/* c++/src/functionals.cpp:136-198 (the GCC branch: double arithmetic, one
 * rounding to float on store).  which = 3, 4 or 5; index 0 is unused. */
void tto_t345_prepare(int which, int rows, float *re, float *im) {
    if (rows > 0) {
        re[0] = 0;
        im[0] = 0;
    }
    for (int r = 1; r < rows; r++) {
        if (which == 3) {
            re[r] = (float)(r * cos(5.0 * log(r)));
            im[r] = (float)(r * sin(5.0 * log(r)));
        } else if (which == 4) {
            re[r] = (float)cos(3.0 * log(r));
            im[r] = (float)sin(3.0 * log(r));
        } else {
            re[r] = (float)(sqrt(r) * cos(4.0 * log(r)));
            im[r] = (float)(sqrt(r) * sin(4.0 * log(r)));
        }
    }
}

/* c++/src/functionals.cpp:200-213; the unqualified hypot there is C's
 * double hypot applied to the two float integrals. */
static float t345_at(const float *x, int n, int sqmedian, const float *re,
                     const float *im) {
    float ir = 0, ii = 0;
    for (int r1 = 1; r1 < n - sqmedian; r1++) {
        ir += re[r1] * x[r1 + sqmedian];
        ii += im[r1] * x[r1 + sqmedian];
    }
    return (float)hypot(ir, ii);
}
float tto_t345(const float *x, int n, const float *re, const float *im) {
    float *tmp = (float *)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1));
    int m = weighted_median_sqrt(x, n, tmp);
    free(tmp);
    return t345_at(x, n, m, re, im);
}

/* Stable merge sort helpers (the reference uses glibc qsort / qsort_r; the
 * order among equal keys only changes float rounding of tied groups). */
static void msort_idx(int *idx, int *tmp, int n, const float *key) {
    if (n < 2)
        return;
    int h = n / 2;
    msort_idx(idx, tmp, h, key);
    msort_idx(idx + h, tmp, n - h, key);
    int i = 0, j = h, k = 0;
    while (i < h && j < n) {
        if (key[idx[j]] < key[idx[i]])
            tmp[k++] = idx[j++];
        else
            tmp[k++] = idx[i++];
    }
    while (i < h)
        tmp[k++] = idx[i++];
    while (j < n)
        tmp[k++] = idx[j++];
    memcpy(idx, tmp, sizeof(int) * (size_t)n);
}
static void msort_float(float *x, float *tmp, int n) {
    if (n < 2)
        return;
    int h = n / 2;
    msort_float(x, tmp, h);
    msort_float(x + h, tmp, n - h);
    int i = 0, j = h, k = 0;
    while (i < h && j < n) {
        if (x[j] < x[i])
            tmp[k++] = x[j++];
        else
            tmp[k++] = x[i++];
    }
    while (i < h)
        tmp[k++] = x[i++];
    while (j < n)
        tmp[k++] = x[j++];
    memcpy(x, tmp, sizeof(float) * (size_t)n);
}

/* c++/src/functionals.cpp:226-255 */
static float t6_at(const float *x, int n, int sqmedian) {
    int len = n - sqmedian;
    float *w = (float *)calloc((size_t)len, sizeof(float));
    float *srt = (float *)malloc(sizeof(float) * (size_t)len);
    int *idx = (int *)malloc(sizeof(int) * (size_t)len);
    int *tmp = (int *)malloc(sizeof(int) * (size_t)len);
    for (int r1 = 0; r1 < len; r1++) {
        w[r1] = (float)r1 * x[r1 + sqmedian];
        idx[r1] = r1;
    }
    msort_idx(idx, tmp, len, (const float *)w);
    for (int r1 = 0; r1 < len; r1++)
        srt[r1] = sqrtf(x[sqmedian + idx[r1]]);
    int index = tto_find_weighted_median(srt, len);
    float result = w[idx[index]];
    free(w);
    free(srt);
    free(idx);
    free(tmp);
    return result;
}
float tto_t6(const float *x, int n) {
    float *tmp = (float *)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1));
    int m = weighted_median_sqrt(x, n, tmp);
    free(tmp);
    return t6_at(x, n, m);
}

/* c++/src/functionals.cpp:262-276 */
static float t7_at(const float *x, int n, int median) {
    int len = n - median;
    float *d = (float *)malloc(sizeof(float) * (size_t)len);
    float *tmp = (float *)malloc(sizeof(float) * (size_t)len);
    memcpy(d, x + median, sizeof(float) * (size_t)len);
    msort_float(d, tmp, len);
    for (int i = 0; i < len; i++)
        tmp[i] = sqrtf(d[i]);
    int index = tto_find_weighted_median(tmp, len);
    float result = d[index];
    free(d);
    free(tmp);
    return result;
}
float tto_t7(const float *x, int n) {
    return t7_at(x, n, tto_find_weighted_median(x, n));
}

/* T-functional f of column x with its weighted median held at row median
 * (the *_at bodies above; T0 ignores median).  Test infrastructure: the
 * parity checker evaluates the reference's arithmetic at the row the engine
 * chose when the reference's own crossing is a rounding tie. */
float tto_t_at(int f, const float *x, int n, int median) {
    if (f == TTO_RADON)
        return tto_t_radon(x, n);
    if (median < 0 || median >= n)
        return NAN;
    switch (f) {
    case TTO_T1: return t1_at(x, n, median);
    case TTO_T2: return t2_at(x, n, median);
    case TTO_T3:
    case TTO_T4:
    case TTO_T5: {
        float *re = (float *)malloc(sizeof(float) * (size_t)n);
        float *im = (float *)malloc(sizeof(float) * (size_t)n);
        tto_t345_prepare(f, n, re, im);
        float r = t345_at(x, n, median, re, im);
        free(re);
        free(im);
        return r;
    }
    case TTO_T6: return t6_at(x, n, median);
    case TTO_T7: return t7_at(x, n, median);
    default: return NAN;
    }
}

/* c++/src/functionals.cpp:287-296; fabs there is C's double fabs. */
float tto_p1(const float *x, int n) {
    float sum = 0;
    float previous = x[0];
    for (int p = 1; p < n; p++) {
        float current = x[p];
        sum = (float)((double)sum + fabs((double)(previous - current)));
        previous = current;
    }
    return sum;
}

/* c++/src/functionals.cpp:303-311 */
float tto_p2(const float *x, int n) {
    float *s = (float *)malloc(sizeof(float) * (size_t)n);
    float *tmp = (float *)malloc(sizeof(float) * (size_t)n);
    memcpy(s, x, sizeof(float) * (size_t)n);
    msort_float(s, tmp, n);
    int m = tto_find_weighted_median(s, n);
    float result = s[m];
    free(s);
    free(tmp);
    return result;
}

/* Radix-2 complex FFT in double (in place, n a power of two, sign -1 forward). */
static void fft_pow2(double *re, double *im, int n, int sign) {
    for (int i = 1, j = 0; i < n; i++) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1)
            j ^= bit;
        j ^= bit;
        if (i < j) {
            double t = re[i]; re[i] = re[j]; re[j] = t;
            t = im[i]; im[i] = im[j]; im[j] = t;
        }
    }
    for (int len = 2; len <= n; len <<= 1) {
        double ang = sign * 2 * M_PI / len;
        for (int i = 0; i < n; i += len) {
            for (int k = 0; k < len / 2; k++) {
                double wr = cos(ang * k), wi = sin(ang * k);
                int a = i + k, b = i + k + len / 2;
                double xr = re[b] * wr - im[b] * wi;
                double xi = re[b] * wi + im[b] * wr;
                re[b] = re[a] - xr; im[b] = im[a] - xi;
                re[a] += xr; im[a] += xi;
            }
        }
    }
}

/* Real-input DFT in double, bins 0..n/2, rounded once to float.  Direct
 * summation with exact twiddle index (k*j mod n) up to 2048 points, chirp-z
 * (Bluestein) above. */
void tto_dft_r2c(const float *x, int n, float *ore, float *oim) {
    int nb = n / 2 + 1;
    if (n <= 2048) {
        double *cs = (double *)malloc(sizeof(double) * (size_t)n);
        double *sn = (double *)malloc(sizeof(double) * (size_t)n);
        for (int j = 0; j < n; j++) {
            cs[j] = cos(2 * M_PI * j / n);
            sn[j] = sin(2 * M_PI * j / n);
        }
        for (int k = 0; k < nb; k++) {
            double ar = 0, ai = 0;
            long idx = 0;
            for (int j = 0; j < n; j++) {
                ar += x[j] * cs[idx];
                ai -= x[j] * sn[idx];
                idx += k;
                if (idx >= n)
                    idx -= n;
            }
            ore[k] = (float)ar;
            oim[k] = (float)ai;
        }
        free(cs);
        free(sn);
        return;
    }
    int m = 1;
    while (m < 2 * n - 1)
        m <<= 1;
    double *wr = (double *)malloc(sizeof(double) * (size_t)n);
    double *wi = (double *)malloc(sizeof(double) * (size_t)n);
    double *ar = (double *)calloc((size_t)m, sizeof(double));
    double *ai = (double *)calloc((size_t)m, sizeof(double));
    double *br = (double *)calloc((size_t)m, sizeof(double));
    double *bi = (double *)calloc((size_t)m, sizeof(double));
    for (int j = 0; j < n; j++) {
        long q = ((long)j * j) % (2L * n); /* exp(-i pi j^2 / n) */
        wr[j] = cos(M_PI * q / n);
        wi[j] = -sin(M_PI * q / n);
    }
    for (int j = 0; j < n; j++) {
        ar[j] = x[j] * wr[j];
        ai[j] = x[j] * wi[j];
    }
    br[0] = wr[0];
    bi[0] = -wi[0];
    for (int j = 1; j < n; j++) {
        br[j] = br[m - j] = wr[j];
        bi[j] = bi[m - j] = -wi[j];
    }
    fft_pow2(ar, ai, m, -1);
    fft_pow2(br, bi, m, -1);
    for (int j = 0; j < m; j++) {
        double r = ar[j] * br[j] - ai[j] * bi[j];
        double i = ar[j] * bi[j] + ai[j] * br[j];
        ar[j] = r;
        ai[j] = i;
    }
    fft_pow2(ar, ai, m, +1);
    for (int k = 0; k < nb; k++) {
        double r = ar[k] / m, i = ai[k] / m;
        ore[k] = (float)(r * wr[k] - i * wi[k]);
        oim[k] = (float)(r * wi[k] + i * wr[k]);
    }
    free(wr); free(wi); free(ar); free(ai); free(br); free(bi);
}

/* c++/src/functionals.cpp:53-60 */
static float trapz(const float *x, const float *y, int n) {
    float sum = 0;
    for (int i = 0; i < n - 1; i++)
        sum += (x[i + 1] - x[i]) * (y[i + 1] + y[i]);
    return (float)(sum * 0.5);
}

/* c++/src/functionals.cpp:332-360; hypot and pow there are C's double
 * versions applied to float quotients. */
float tto_p3(const float *x, int n) {
    int nb = n / 2 + 1;
    float *fr = (float *)malloc(sizeof(float) * (size_t)nb);
    float *fi = (float *)malloc(sizeof(float) * (size_t)nb);
    float *lin = (float *)malloc(sizeof(float) * (size_t)n);
    float *mod = (float *)malloc(sizeof(float) * (size_t)n);
    tto_dft_r2c(x, n, fr, fi);
    float fn = (float)n;
    for (int p = 0; p < n / 2 + 1; p++) {
        mod[p] = (float)pow(hypot(fr[p] / fn, fi[p] / fn), 4);
        lin[p] = (float)(-1 + p * 2.0 / (n - 1));
    }
    for (int p = n / 2 + 1; p < n; p++) {
        mod[p] = (float)pow(hypot(fr[n - p] / fn, fi[n - p] / fn), 4);
        lin[p] = (float)(-1 + p * 2.0 / (n - 1));
    }
    float result = trapz(lin, mod, n);
    free(fr); free(fi); free(lin); free(mod);
    return result;
}

/* c++/src/functionals.cpp:62-74 -- float return, double intermediates. */
float tto_hermite_polynomial(unsigned order, float x) {
    switch (order) {
    case 0:
        return 1.0f;
    case 1:
        return (float)(2.0 * x);
    default:
        return (float)(2.0 * x * tto_hermite_polynomial(order - 1, x) -
                       2.0 * (order - 1) * tto_hermite_polynomial(order - 2, x));
    }
}

static unsigned factorial(unsigned n) {
    return (n == 1 || n == 0) ? 1 : factorial(n - 1) * n;
}

/* c++/src/functionals.cpp:80-84 */
float tto_hermite_function(unsigned order, float x) {
    float half_sq = x * x / 2;
    return (float)(tto_hermite_polynomial(order, x) /
                   (sqrt(pow(2, order) * factorial(order) * sqrt(M_PI)) *
                    exp(half_sq)));
}

/* c++/src/functionals.cpp:369-386 */
float tto_p_hermite(const float *x, int n, unsigned order, int center) {
    float lower = (float)(10.0 / center);
    float upper = (float)(10.0 / (n - 1 - center));
    float integral = 0;
    for (int p = 0; p < n; p++) {
        float z;
        if (p < center)
            z = p * lower - 10;
        else
            z = (p - center) * upper;
        integral += x[p] * tto_hermite_function(order, z);
    }
    return integral;
}

/* ------------------------------------------------------------------------
 * sinogram.cpp / circus.cpp
 * ---------------------------------------------------------------------- */

/* c++/src/sinogram.cpp:67-178; the angle loop is the one openmp/src/
 * sinogram.cpp:110 parallelises. */
void tto_sinograms(const float *padded, int n, const float *angles_deg,
                   int n_angles, const int *tfuncs, int n_t, float *out,
                   int *medians, int threads) {
    float *tab_re[8] = {0}, *tab_im[8] = {0};
    for (int t = 0; t < n_t; t++) {
        int f = tfuncs[t];
        if (f >= TTO_T3 && f <= TTO_T5 && !tab_re[f]) {
            tab_re[f] = (float *)malloc(sizeof(float) * (size_t)n);
            tab_im[f] = (float *)malloc(sizeof(float) * (size_t)n);
            tto_t345_prepare(f, n, tab_re[f], tab_im[f]);
        }
    }
    size_t plane = (size_t)n * n_angles;
#ifdef _OPENMP
    int nthr = threads > 0 ? threads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthr)
#else
    (void)threads;
#endif
    for (int a = 0; a < n_angles; a++) {
        float *rot = (float *)malloc(sizeof(float) * (size_t)n * n);
        float *sq = (float *)malloc(sizeof(float) * (size_t)n);
        tto_rotate(padded, n, n, tto_deg2rad(angles_deg[a]), rot);
        for (int col = 0; col < n; col++) {
            const float *x = rot + (size_t)col * n;
            int m1 = -2, m2 = -2;
            for (int t = 0; t < n_t; t++) {
                int f = tfuncs[t];
                float r = 0;
                int med = -1;
                if (f == TTO_T1 || f == TTO_T2 || f == TTO_T7) {
                    if (m1 == -2)
                        m1 = tto_find_weighted_median(x, n);
                    med = m1;
                } else if (f >= TTO_T3 && f <= TTO_T6) {
                    if (m2 == -2)
                        m2 = weighted_median_sqrt(x, n, sq);
                    med = m2;
                }
                switch (f) {
                case TTO_RADON: r = tto_t_radon(x, n); break;
                case TTO_T1: r = t1_at(x, n, med); break;
                case TTO_T2: r = t2_at(x, n, med); break;
                case TTO_T3:
                case TTO_T4:
                case TTO_T5: r = t345_at(x, n, med, tab_re[f], tab_im[f]); break;
                case TTO_T6: r = t6_at(x, n, med); break;
                case TTO_T7: r = t7_at(x, n, med); break;
                default: r = NAN; break;
                }
                out[(size_t)t * plane + (size_t)col + (size_t)a * n] = r;
                if (medians)
                    medians[(size_t)t * plane + (size_t)col + (size_t)a * n] = med;
            }
        }
        free(rot);
        free(sq);
    }
    for (int f = 0; f < 8; f++) {
        free(tab_re[f]);
        free(tab_im[f]);
    }
}

/* c++/src/circus.cpp:104-177; the column loop is the one openmp/src/
 * circus.cpp:129 parallelises. */
void tto_circus(const float *sino, int rows, int cols, const int *kinds,
                const int *orders, const int *centers, int n_p, float *out,
                int threads) {
#ifdef _OPENMP
    int nthr = threads > 0 ? threads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthr)
#else
    (void)threads;
#endif
    for (int col = 0; col < cols; col++) {
        const float *x = sino + (size_t)col * rows;
        for (int p = 0; p < n_p; p++) {
            float r;
            switch (kinds[p]) {
            case TTO_P1: r = tto_p1(x, rows); break;
            case TTO_P2: r = tto_p2(x, rows); break;
            case TTO_P3: r = tto_p3(x, rows); break;
            case TTO_HERMITE:
                r = tto_p_hermite(x, rows, (unsigned)orders[p], centers[p]);
                break;
            default: r = NAN; break;
            }
            out[(size_t)p * cols + col] = r;
        }
    }
}

/* ------------------------------------------------------------------------
 * Nearest orthonormal sinogram (c++/src/circus.cpp:68-102).  The reference
 * takes U[:, :cols] * V^T from Eigen's float JacobiSVD; here the same polar
 * factor comes from a one-sided Jacobi SVD in double.
 * ---------------------------------------------------------------------- */
static void polar_factor(const float *a_in, int m, int n, float *out) {
    double *a = (double *)malloc(sizeof(double) * (size_t)m * n);
    double *v = (double *)calloc((size_t)n * n, sizeof(double));
    for (size_t i = 0; i < (size_t)m * n; i++)
        a[i] = a_in[i];
    for (int i = 0; i < n; i++)
        v[i + (size_t)i * n] = 1;
    for (int sweep = 0; sweep < 60; sweep++) {
        double off = 0;
        for (int p = 0; p < n - 1; p++) {
            for (int q = p + 1; q < n; q++) {
                double *ap = a + (size_t)p * m, *aq = a + (size_t)q * m;
                double alpha = 0, beta = 0, gamma = 0;
                for (int i = 0; i < m; i++) {
                    alpha += ap[i] * ap[i];
                    beta += aq[i] * aq[i];
                    gamma += ap[i] * aq[i];
                }
                if (gamma == 0 || fabs(gamma) <= 1e-15 * sqrt(alpha * beta))
                    continue;
                double r = fabs(gamma) / sqrt(alpha * beta);
                if (r > off)
                    off = r;
                double zeta = (beta - alpha) / (2 * gamma);
                double t = (zeta >= 0 ? 1.0 : -1.0) /
                           (fabs(zeta) + sqrt(1 + zeta * zeta));
                double c = 1 / sqrt(1 + t * t), s = c * t;
                for (int i = 0; i < m; i++) {
                    double x = ap[i], y = aq[i];
                    ap[i] = c * x - s * y;
                    aq[i] = s * x + c * y;
                }
                double *vp = v + (size_t)p * n, *vq = v + (size_t)q * n;
                for (int i = 0; i < n; i++) {
                    double x = vp[i], y = vq[i];
                    vp[i] = c * x - s * y;
                    vq[i] = s * x + c * y;
                }
            }
        }
        if (off < 1e-15)
            break;
    }
    /* U[:, k] = a[:, k] / sigma_k; polar = U V^T */
    for (int k = 0; k < n; k++) {
        double nrm = 0;
        double *ak = a + (size_t)k * m;
        for (int i = 0; i < m; i++)
            nrm += ak[i] * ak[i];
        nrm = sqrt(nrm);
        for (int i = 0; i < m; i++)
            ak[i] = nrm > 0 ? ak[i] / nrm : 0;
    }
    for (int j = 0; j < n; j++) {
        for (int i = 0; i < m; i++) {
            double acc = 0;
            for (int k = 0; k < n; k++)
                acc += a[i + (size_t)k * m] * v[j + (size_t)k * n];
            out[i + (size_t)j * m] = (float)acc;
        }
    }
    free(a);
    free(v);
}

int tto_nos(const float *sino, int rows, int cols, float *out, int *out_rows,
            int *new_center) {
    if (rows <= 0 || cols <= 0)
        return -1;
    int center = (int)floor((rows - 1) / 2.0);
    int *offset = (int *)malloc(sizeof(int) * (size_t)cols);
    for (int p = 0; p < cols; p++)
        offset[p] = tto_find_weighted_median(sino + (size_t)p * rows, rows) -
                    center;
    int mn = offset[0], mx = offset[0];
    for (int p = 1; p < cols; p++) {
        if (offset[p] < mn)
            mn = offset[p];
        if (offset[p] > mx)
            mx = offset[p];
    }
    int padding = abs(mx) + abs(mn);
    int m = rows + padding;
    *new_center = center + mx;
    *out_rows = m;
    float *aligned = (float *)calloc((size_t)m * cols, sizeof(float));
    for (int col = 0; col < cols; col++)
        for (int row = 0; row < rows; row++)
            aligned[(size_t)(mx + row - offset[col]) + (size_t)col * m] =
                sino[(size_t)row + (size_t)col * rows];
    int rc = 0;
    if (m >= cols)
        polar_factor(aligned, m, cols, out);
    else
        rc = -2; /* the reference's U.block(0, 0, m, cols) needs m >= cols */
    free(aligned);
    free(offset);
    return rc;
}
