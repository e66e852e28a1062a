/*
 * tt_oracle.h -- CPU restatement of the reference trace-transform float path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the CUDA
 * engine and the timed CPU baseline ("port").  Nothing in the product path
 * (tracetransform_gb300/) may link, load or call it.
 *
 * Every function restates one routine of maleadt/tracetransform's C++ port
 * (c++/src/..., the OpenMP port openmp/src/... adds only loop pragmas) with the
 * same float/double evaluation order, so that it agrees bit for bit with the
 * reference sources compiled against the API-subset stand-ins in oracle/shim/.
 *
 * Layout conventions follow Eigen's default: column-major, element (row, col)
 * of an R x C matrix lives at [row + col * R].
 */
#ifndef TT_ORACLE_H
#define TT_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* T-functional ids, as parsed by c++/src/sinogram.cpp:34-65 ("0".."7"). */
enum { TTO_RADON = 0, TTO_T1, TTO_T2, TTO_T3, TTO_T4, TTO_T5, TTO_T6, TTO_T7 };
/* P-functional kinds, as parsed by c++/src/circus.cpp:33-66. */
enum { TTO_HERMITE = 0, TTO_P1 = 1, TTO_P2 = 2, TTO_P3 = 3 };

/* ---- auxiliary.cpp ---------------------------------------------------- */
float tto_deg2rad(float degrees);                               /* :180 */
void tto_rotation(float angle, float *c, float *s);             /* :227-237 */
void tto_pad_geometry(int rows, int cols, int *n, int *row_off, /* :257-275 */
                      int *col_off);
void tto_pad(const float *image, int rows, int cols, float *out);
void tto_resize(const float *in, int in_rows, int in_cols,      /* :198-221 */
                int rows, int cols, float *out);
void tto_rotate(const float *in, int rows, int cols, float angle, /* :223-255 */
                float *out);
float tto_arithmetic_mean(const float *x, int n);               /* :277-287 */
float tto_standard_deviation(const float *x, int n);            /* :289-303 */
void tto_zscore(const float *x, int n, float *out);             /* :305-318 */

/* ---- functionals.cpp -------------------------------------------------- */
int tto_find_weighted_median(const float *x, int n);            /* :21-30 */
float tto_t_radon(const float *x, int n);                       /* :95-97 */
float tto_t1(const float *x, int n);                            /* :104-113 */
float tto_t2(const float *x, int n);                            /* :120-129 */
void tto_t345_prepare(int which, int rows, float *re, float *im); /* :136-198 */
float tto_t345(const float *x, int n, const float *re, const float *im); /* :200-213 */
float tto_t6(const float *x, int n);                            /* :226-255 */
float tto_t7(const float *x, int n);                            /* :262-276 */
float tto_t_at(int f, const float *x, int n, int median);      /* *_at above */
float tto_p1(const float *x, int n);                            /* :287-296 */
float tto_p2(const float *x, int n);                            /* :303-311 */
float tto_p3(const float *x, int n);                            /* :332-360 */
float tto_hermite_polynomial(unsigned order, float x);          /* :62-74 */
float tto_hermite_function(unsigned order, float x);            /* :80-84 */
float tto_p_hermite(const float *x, int n, unsigned order, int center); /* :369-386 */

/* Real-input DFT, bins 0..n/2, computed in double and rounded to float (the
 * stand-in for FFTW's fftwf_plan_dft_r2c_1d used by PFunctional3). */
void tto_dft_r2c(const float *x, int n, float *re, float *im);

/* ---- sinogram.cpp / circus.cpp / transform.cpp ------------------------ */
/* getSinograms (c++/src/sinogram.cpp:67-178) over an explicit angle list in
 * degrees (the reference uses a_step * angle_stepsize).  out is
 * n_t x (n x n_angles), each sinogram column-major with one column per angle.
 * medians (optional, may be NULL): n_t x n x n_angles int32, the weighted
 * median index each T-functional used (-1 for Radon).  threads <= 0: all. */
void tto_sinograms(const float *padded, int n, const float *angles_deg,
                   int n_angles, const int *tfuncs, int n_t, float *out,
                   int *medians, int threads);
/* getCircusFunctions (c++/src/circus.cpp:104-177): sino is rows x cols,
 * out is n_p x cols. */
void tto_circus(const float *sino, int rows, int cols, const int *kinds,
                const int *orders, const int *centers, int n_p, float *out,
                int threads);
/* nearest_orthonormal_sinogram (c++/src/circus.cpp:68-102).  out must hold
 * (rows + rows) x cols floats; *out_rows receives rows + padding. */
int tto_nos(const float *sino, int rows, int cols, float *out, int *out_rows,
            int *new_center);

#ifdef __cplusplus
}
#endif
#endif
