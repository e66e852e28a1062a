/* fftw3.h stand-in: the single-precision real-to-complex 1-D plan that
 * maleadt/tracetransform's PFunctional3 uses (c++/src/functionals.cpp:318-360)
 * plus the threading calls of its OpenMP port.  Plans compute the DFT in
 * double precision and round each output bin once to float. */
#ifndef TT_SHIM_FFTW3_H
#define TT_SHIM_FFTW3_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef float fftwf_complex[2];
typedef double fftw_complex[2];
typedef struct tt_fftwf_plan_s *fftwf_plan;
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)
fftwf_plan fftwf_plan_dft_r2c_1d(int n, float *in, fftwf_complex *out,
                                 unsigned flags);
void fftwf_execute(const fftwf_plan p);
void fftwf_destroy_plan(fftwf_plan p);
void *fftwf_malloc(size_t n);
void fftwf_free(void *p);
int fftw_init_threads(void);
void fftw_plan_with_nthreads(int nthreads);
void fftw_cleanup_threads(void);
#ifdef __cplusplus
}
#endif
#endif
