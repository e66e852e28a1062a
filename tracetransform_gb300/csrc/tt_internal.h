// tt_internal.h -- argument blocks and launchers shared by the engine's
// translation units (not part of the public ABI).
#pragma once

#include <complex>

#include <cuda_runtime.h>
#include <stdint.h>

#include "tracetransform.h"

namespace tt {

constexpr int kMaxT = 16; // T-functional entries per call
constexpr int kMaxP = 16; // P-functional entries per call
// Sinograms per line the warp-autonomous kernels write (one lane each; at
// most 4 lines per warp, so a line has 8 lanes or more): calls with more
// T-functional entries take the CTA kernels.
constexpr int kWarpMaxOutputs = 8;

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
    bool interior;      // the texture region lies >= 2 texels inside the frame
};

// Does a texture region of rows x cols at (row_off, col_off) lie at least two
// texels inside the n x n frame on every side?  Then a rotated sample outside
// [0, n-1) only ever reads border texels (value 0), and the sampler can skip
// the reference's bounds test without changing any result.
inline bool interior_source(int n, int row_off, int col_off, int rows, int cols) {
    return row_off >= 2 && col_off >= 2 && row_off + rows <= n - 1 && col_off + cols <= n - 1;
}

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

// P-stage over stacks of columns (P1, P2, P3; no Hermite): P3 as a direct
// DFT computed like a GEMM (F = W^T X per stack, |F|^4 and the trapz weights
// folded into its epilogue), P1 and P2 one warp per column.
struct CircusStack {
    const float *sino;  // cols columns of n floats (n_sino sinograms x angles)
    float *out;         // n_sino x n_p x angles
    float *partial;     // P3: mtiles x cols partial sums of ck |F_k / n|^4
    const float2 *tw;   // n twiddles (cos, -sin)(2 pi j / n)
    const float *ck;    // n / 2 + 1 trapz weights
    const float *wtc;   // the tensor cores' twiddle blocks of n (p3_tc_table_floats)
    int n, angles, cols;
    int mtiles;         // frequency tiles of 64 (P3)
    int tile_begin;     // first P3 tile of this stack (flat over stacks)
    int col_begin;      // first column (flat over stacks)
};

struct CircusStackArgs {
    const CircusStack *st; // n_st descriptors in device memory, or NULL: `one`
    CircusStack one;
    int n_st;
    int total_tiles, total_cols;
    int n_p;
    int kind[kMaxP];
    unsigned need;      // bit k: P kind k requested
    int stride;         // floats of shared memory per warp's column buffer
    unsigned *fb_count; // P2 columns left to the exact sort (negative / non-finite)
    int2 *fb_list;      // (stack, column) of those columns
    int fb_capacity;
    int sort_len_max;   // power of two >= the longest column (exact-sort fallback)
    int fb_grid;        // CTAs of the exact-sort fallback
    int tc_tables;      // every stack has wtc (else the kernel gathers the twiddles)
};

// Device tables of the direct-DFT P3: tw (n), ck (n / 2 + 1), built on stream.
cudaError_t launch_p3_dft_tables(int n, float2 *tw, float *ck, cudaStream_t st);
// The tensor-core P3's precomputed twiddle blocks of n, from its twiddles.
size_t p3_tc_table_floats(int n);
cudaError_t launch_p3_tc_tables(int n, const float2 *tw, float *out, cudaStream_t st);
// Longest column whose P3 the direct DFT computes (longer ones: the FFT kernel).
constexpr int kP3DftMaxRows = 2048;
// P3 frequency tiles of a column length n.
int p3_freq_tiles(int n);
size_t circus_warp_smem_bytes(int n_max);
int circus_warp_stride(int n_max);
// The three launches of the P-stage over stacks (fb_count zeroed on stream).
cudaError_t launch_circus_stacks(const CircusStackArgs &a, size_t smem, cudaStream_t st);

// P3 tables (tt_tables.cu): FFT length M for a column of n samples, and the
// chirp (n), filter (M), twiddles (M / 2) and linspace (n); work holds M.
int p3_fft_length(int n);
void p3_tables(int n, float2 *chirp, float2 *filt, float2 *twid, float *lin,
               std::complex<double> *work);

// Rotation (cos(-theta), sin(-theta)) of an angle in degrees and the T3-T5
// kernels (3 n entries) as the reference rounds them (tt_tables.cu).
float2 rotation(float degrees);
void t345_tables(int n, float2 *out);

// pad() geometry of c++/src/auxiliary.cpp:257-275 (tt_tables.cu).
void pad_geometry(int rows, int cols, int *n, int *row_off, int *col_off);

// The batched engine (tt_batch.cu): one per plan, rebuilt when the batch shape
// changes.  batch_run returns a tt_status.
class BatchEngine;
BatchEngine *batch_create(int device);
void batch_destroy(BatchEngine *b);
int batch_run(BatchEngine *b, const float *d_images, const long long *offsets, const int *rows,
              const int *cols, const int *steps, int n_img, const int32_t *tfuncs, int n_t,
              const tt_pfunctional *pf, int n_p, float *d_circus, float *d_sig,
              cudaStream_t st);
// Copies the last batch's sinograms (input order, each n_t x A_i x N_i);
// *count receives their float count (0 before the first batch).
int batch_sinograms(BatchEngine *b, float *d_out, size_t capacity, size_t *count,
                    cudaStream_t st);
// Device milliseconds of the last replay's three kernels (sinograms,
// P-functionals, z-scores), from events recorded inside the graph.
int batch_stage_ms(BatchEngine *b, float ms[3]);
// The persistent kernel's tile {lines per CTA, CTAs per SM, lines per warp
// (0: one per warp)}; pinning one with CTAs per SM > 0 replaces the tuner.
void batch_tile(BatchEngine *b, int out[3]);
void batch_pin_tile(BatchEngine *b, const int t[3]);

// Backward pass (tt_backward.cu), T = float or double.  cs: (cos, sin) per
// angle as the forward used them; cosv / sinv: cos, sin(2 pi j / rows);
// params: scratch of 4 T per line (n x n_angles).
template <typename T>
cudaError_t launch_circus_backward(const T *sino, int rows, int cols, int n_sino,
                                   const int *d_kinds, int n_p, const T *grad_circus,
                                   const T *cosv, const T *sinv, const T *lin, T *out,
                                   cudaStream_t st);
// The float P-stage adjoint by the chirp-z identity on the forward's FFT
// tables (chirp, filter, twiddles of length M); cudaErrorInvalidValue when
// its shared memory (circus_backward_fft_smem) exceeds the device's.
cudaError_t launch_circus_backward_fft(const float *sino, int rows, int cols, int n_sino,
                                       const int *d_kinds, int n_p, const float *grad_circus,
                                       const float2 *chirp, const float2 *filt,
                                       const float2 *twid, int M, const float *lin, float *out,
                                       cudaStream_t st);
size_t circus_backward_fft_smem(int rows, int M);
bool circus_backward_fft_fits(int rows, int M);
template <typename T>
cudaError_t launch_sino_backward(const T *grad_sino, const int *medians, int n_images, int n,
                                 int n_angles, unsigned long long tf_code, int n_t, T *params,
                                 int rows, int cols, int row_off, int col_off, const T *cs,
                                 T *grad_img, cudaStream_t st);
cudaError_t launch_sino_f64(const double *img, int rows, int cols, int row_off, int col_off,
                            int n, const double *cs, unsigned long long tf_code, int n_t,
                            int n_angles, double *out, int *medians, cudaStream_t st);
cudaError_t launch_circus_f64(const double *sino, int rows, int cols, int n_sino,
                              const int *d_kinds, int n_p, const double *cosv,
                              const double *sinv, const double *lin, double *out,
                              cudaStream_t st);

// Nearest orthonormal sinogram (tt_nos.cu): one aligned matrix per sinogram.
struct NosDesc {
    long long a_off;   // into the double-float m x cols matrices
    long long out_off; // into the float results
    int m;             // rows + |max offset| + |min offset|
    int mx;            // max offset
};
// Per-call scratch of the nearest orthonormal sinogram (n = angles).
struct NosWork {
    float2 *norms;              // 2 x n_sino x n: QR partial norms by position, by step parity
    float *orig;                // n_sino x n: norm at the last recompute, by stored column
    float2 *tau, *beta, *scale; // n_sino x n each: the reflectors (double-float)
    int *cmap;                  // 2 x n_sino x n: position -> stored column, by step parity
    int *perm;                  // n_sino x n: stored column that ends at each position
    float *X, *V, *P;           // n_sino x n x n each (R^T, Jacobi V, polar(R))
    float *inv;                 // n_sino x n
    unsigned *off_bits;         // n_sino: largest rotated |cos| of a sweep (float bits)
    float *tiny;                // n_sino: squared column norm below which a direction is null
    unsigned *sweep_state;      // 2: the last sweep's largest cos (float bits), sweeps done
    float *wy;                  // nos_assemble_floats(): the blocked Q application's T
                                // factors, partial products and T W
};
cudaError_t launch_nos_offsets(const float *sino, int rows, int cols, int n_sino, int center,
                               int *offsets, cudaStream_t st);
cudaError_t launch_nos_align(const float *sino, int rows, int cols, int n_sino,
                             const NosDesc *desc, const int *offsets, float2 *A, size_t a_elems,
                             cudaStream_t st);
// QR of the aligned matrices and X = R^T, V = I (n + 2 launches).
cudaError_t launch_nos_factor(float2 *A, const NosDesc *desc, int n, int n_sino, int max_m,
                              const NosWork &w, cudaStream_t st);
int nos_max_rows(); // aligned rows the QR kernels hold in registers
// One Jacobi sweep on X (n - 1 + (n & 1) launches), then the stop rule on
// the device: the sweep sets the while-loop condition `loop` to 0 when the
// iteration has converged or max_sweeps sweeps are done (w.sweep_state,
// zeroed before the loop, counts them).
cudaError_t launch_nos_sweep(int n, int n_sino, const NosWork &w, int max_sweeps,
                             cudaGraphConditionalHandle loop, cudaStream_t st);
// Scratch floats (NosWork.wy) of launch_nos_assemble.
size_t nos_assemble_floats(int n, int n_sino, int max_m);
// The nearest orthonormal sinograms from the converged sweeps:
// Q [V U^T; 0] by blocks of reflectors, into out.
cudaError_t launch_nos_assemble(const float2 *A, const NosDesc *desc, int n, int n_sino,
                                int max_m, const NosWork &w, float *out, cudaStream_t st);

// Record a failure for tt_last_error() on this thread; returns status.
int record_error(int status, const char *message);

// Every device allocation of the library goes through these: cudaMalloc /
// cudaMallocArray, unless tt_debug_fail_allocations armed a simulated
// failure, which they report as cudaErrorMemoryAllocation without touching
// the device.
cudaError_t dev_malloc(void **p, size_t bytes);
cudaError_t dev_malloc_array(cudaArray_t *a, const cudaChannelFormatDesc *desc, size_t w,
                             size_t h, unsigned flags);

// Opt-in shared memory per block minus the kernel's static shared memory.
size_t dynamic_smem_limit(const void *kernel);
// Raises the kernel's dynamic shared memory cap to dynamic_smem_limit on the
// current device (once per device and kernel, thread-safe); returns the cap,
// 0 on failure.
size_t opt_in_smem(const void *kernel);

// Batched sinograms: one image of a batch (device descriptor).
struct BatchImage {
    cudaTextureObject_t tex; // the image, texel (u, v) = (row, col)
    int rows, cols, n, row_off, col_off;
    int n_angles, blocks;    // angles; CTA line blocks per angle, ceil(n / L)
    int items_begin;         // first work item (angle * blocks + block)
    int trig_off, tab_off;   // into trig (per angle) and tab (3 n)
    long long sino_off;      // into sino (n_t x n_angles x n floats)
};

struct BatchSinoArgs {
    const BatchImage *img;
    int n_img, total_items;
    const float2 *trig, *tab;
    float *sino;
    unsigned *counter;       // work counter, zero before the launch
    unsigned long long tf_code; // T id of output t in bits [3t, 3t + 3)
    int n_t;
    unsigned need;
    int stride;              // floats per line buffer (for the largest n)
    bool all_interior;       // every image passes interior_source
};

int sino_lines_per_block(int n, unsigned need);
size_t sino_smem_bytes(int n, int lines, unsigned need);
int sino_stride(int n, int lines);
cudaError_t launch_sinograms(const SinoArgs &a, int lines, cudaStream_t stream);
// Warp-autonomous sinogram kernels for T0-T5: each warp samples and reduces
// lpw (1, 2 or 4) lines of its own; the CTA kernels above serve T6 / T7.
int sino_warp_stride(int n, int lpw);
size_t sino_warp_smem_bytes(int n, int lpw);
int sino_warp_cta_warps();
cudaError_t launch_sinograms_warp(const SinoArgs &a, int lpw, cudaStream_t stream);
int sino_batch_warp_occupancy(int lpw, bool interior, size_t smem);
cudaError_t launch_sino_batch_warp(const BatchSinoArgs &a, int lpw, int grid, size_t smem,
                                   cudaStream_t stream);
cudaError_t launch_rotate(cudaTextureObject_t tex, int rows, int cols, float c, float s,
                          float *out, cudaStream_t stream);
// resize() of the orthonormal mode; column-major device buffers.
cudaError_t launch_resize(const float *in, int in_rows, int in_cols, int rows, int cols,
                          float *out, cudaStream_t stream);
cudaError_t launch_region_bbox(const float *frame, int n, int *d_region,
                               cudaStream_t stream);
cudaError_t launch_circus(const CircusArgs &a, cudaStream_t stream);
size_t circus_smem_bytes(const CircusArgs &a);
cudaError_t launch_zscore(const float *in, int n_vec, int len, float *out,
                          cudaStream_t stream);

// Batched engine kernels.  The persistent sinogram kernel runs `grid` CTAs
// that claim work items from *counter; lines = 4 or 8.
cudaError_t prepare_sino_batch(int lines, bool sel, bool interior, size_t smem);
int sino_batch_occupancy(int lines, bool sel, bool interior, size_t smem);
cudaError_t launch_sino_batch(const BatchSinoArgs &a, int lines, int grid, size_t smem,
                              cudaStream_t stream);
cudaError_t launch_zscore_batch(const float *in, const long long *off, const int *len,
                                int n_vec, float *out, cudaStream_t stream);

} // namespace tt
