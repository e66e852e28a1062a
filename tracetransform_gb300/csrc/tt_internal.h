// tt_internal.h -- argument blocks and launchers shared by the engine's
// translation units (not part of the public ABI).
#pragma once

#include <complex>

#include <cuda_runtime.h>
#include <stdint.h>

namespace tt {

constexpr int kMaxT = 16; // T-functional entries per call
constexpr int kMaxP = 16; // P-functional entries per call

// Fused rotate + T-functional sweep over one image.
struct SinoArgs {
    cudaTextureObject_t tex; // source pixels (border mode: 0 outside)
    int tex_row_off, tex_col_off; // frame position of texel (0, 0)
    int src_rows, src_cols;       // support region: rows x cols at
    int row_off, col_off;         // (row_off, col_off) of the frame
    const int *dyn_region; // optional device int4 {row0, col0, rows, cols}
                           // replacing the support region
    int n;                 // padded side N
    int n_angles;
    const float2 *trig; // per angle (cos(-theta), sin(-theta)), host-rounded
    const float2 *tab;  // 3 x n complex kernels of T3, T4, T5
    float *out;         // n_t x n_angles x n
    int32_t *medians;   // optional, same shape as out
    int n_t;
    int tf[kMaxT];
    unsigned need;      // bit f set when T-functional f is requested
    int stride;         // floats per line in shared memory
};

// P-functionals over stacked sinograms.
struct CircusArgs {
    const float *sino; // n_sino x cols x rows
    int rows, cols, n_sino;
    int n_p;
    int kind[kMaxP];
    const float *const *herm; // n_sino x n_p basis pointers (Hermite kinds)
    const float2 *chirp;  // rows: exp(-i pi j^2 / rows)
    const float2 *filt;   // M: FFT of the conjugate chirp, divided by M
    const float2 *twid;   // M / 2: exp(-2 pi i k / M)
    const float *lin;     // rows: linspace(-1, 1, rows) as the reference rounds it
    int M, sort_len;      // FFT length, power-of-two sort length
    unsigned need;        // bit k set when P kind k is requested
    float *out;           // n_sino x n_p x cols
};

// P3 tables (tt_tables.cu): FFT length M for a column of n samples, and the
// chirp (n), filter (M), twiddles (M / 2) and linspace (n); work holds M.
int p3_fft_length(int n);
void p3_tables(int n, float2 *chirp, float2 *filt, float2 *twid, float *lin,
               std::complex<double> *work);

// Record a failure for tt_last_error() on this thread; returns status.
int record_error(int status, const char *message);

// Opt-in shared memory per block minus the kernel's static shared memory.
size_t dynamic_smem_limit(const void *kernel);

int sino_lines_per_block(int n, unsigned need);
size_t sino_smem_bytes(int n, int lines, unsigned need);
int sino_stride(int n, int lines);
cudaError_t launch_sinograms(const SinoArgs &a, int lines, cudaStream_t stream);
cudaError_t launch_rotate(cudaTextureObject_t tex, int rows, int cols, float c, float s,
                          float *out, cudaStream_t stream);
cudaError_t launch_region_bbox(const float *frame, int n, int *d_region,
                               cudaStream_t stream);
cudaError_t launch_circus(const CircusArgs &a, cudaStream_t stream);
size_t circus_smem_bytes(const CircusArgs &a);
cudaError_t launch_zscore(const float *in, int n_vec, int len, float *out,
                          cudaStream_t stream);

} // namespace tt
