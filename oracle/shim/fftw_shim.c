/* Implementation of the fftw3.h stand-in: direct real-input DFT in double
 * with exact twiddle index (k*j mod n), each bin rounded once to float. */
#include "fftw3.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
struct tt_fftwf_plan_s {
    int n;
    float *in;
    fftwf_complex *out;
};
fftwf_plan fftwf_plan_dft_r2c_1d(int n, float *in, fftwf_complex *out,
                                 unsigned flags) {
    fftwf_plan p = (fftwf_plan)malloc(sizeof(*p));
    p->n = n;
    p->in = in;
    p->out = out;
    if (!(flags & FFTW_ESTIMATE)) /* measuring planners may clobber arrays */
        memset(in, 0, sizeof(float) * (size_t)n);
    return p;
}
void fftwf_execute(const fftwf_plan p) {
    int n = p->n, nb = n / 2 + 1;
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
            ar += p->in[j] * cs[idx];
            ai -= p->in[j] * sn[idx];
            idx += k;
            if (idx >= n)
                idx -= n;
        }
        p->out[k][0] = (float)ar;
        p->out[k][1] = (float)ai;
    }
    free(cs);
    free(sn);
}
void fftwf_destroy_plan(fftwf_plan p) { free(p); }
void *fftwf_malloc(size_t n) { return malloc(n); }
void fftwf_free(void *p) { free(p); }
int fftw_init_threads(void) { return 1; }
void fftw_plan_with_nthreads(int nthreads) { (void)nthreads; }
void fftw_cleanup_threads(void) {}
