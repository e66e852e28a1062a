/*
 * tracetransform.h -- C ABI of the GB300 trace-transform engine
 * (libtt_gb300.so).
 *
 * The engine is a drop-in for the sinogram + circus-function path of
 * maleadt/tracetransform's C++ implementation: a padded image is rotated over
 * a set of angles, every rotated column is reduced by T-functionals into
 * sinograms, every sinogram column by P-functionals into circus functions,
 * and each circus function is z-scored into the signature matrix.
 *
 * Conventions (those of the reference's Eigen matrices):
 *   - matrices are float32, column-major: element (row, col) of an R x C
 *     matrix is at [row + col * R];
 *   - a stack of nT sinograms is nT consecutive N x A matrices, column a
 *     holding angle a;
 *   - circus functions are nT x nP consecutive vectors of length A (T-major);
 *   - the signature matrix is A x (nT * nP), column t * nP + p being the
 *     z-scored circus function of (T t, P p) -- the same bytes as the circus
 *     stack, z-scored.
 *
 * Every call returns a tt_status; on failure tt_last_error() describes the
 * error of the calling thread.  Host-pointer calls are synchronous; *_device
 * calls take device pointers and are ordered on the given CUDA stream (NULL:
 * the plan's own stream) and return before the work completes.
 */
#ifndef TRACETRANSFORM_H
#define TRACETRANSFORM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    TT_OK = 0,
    TT_ERR_INVALID_ARG = 1, /* bad size, id or pointer (reference: assert /
                               boost::program_options::validation_error) */
    TT_ERR_UNSUPPORTED = 2, /* valid request this build does not handle */
    TT_ERR_CUDA = 3,        /* CUDA runtime error (reference: CUDAHelper::Error) */
    TT_ERR_TIMEOUT = 4,     /* reserved: no entry point waits on the device (the
                               engine's kernels contain no spin-waits), so none
                               returns it */
    TT_ERR_OOM = 5          /* device or host allocation failed */
} tt_status;

/* T-functional ids: the strings "0".."7" of c++/src/sinogram.cpp:34-65
 * (enum class TFunctional, c++/src/sinogram.hpp:22-31). */
enum {
    TT_T_RADON = 0,
    TT_T1 = 1,
    TT_T2 = 2,
    TT_T3 = 3,
    TT_T4 = 4,
    TT_T5 = 5,
    TT_T6 = 6,
    TT_T7 = 7
};

/* P-functional kinds: "1", "2", "3" and "H<order>" of c++/src/circus.cpp:33-66
 * (enum class PFunctional, c++/src/circus.hpp:27-32). */
enum { TT_P_HERMITE = 0, TT_P1 = 1, TT_P2 = 2, TT_P3 = 3 };

/* PFunctionalWrapper + PFunctionalArguments{order, center}
 * (c++/src/circus.hpp:34-57).  order and center are used by TT_P_HERMITE
 * only; center < 0 means "not set". */
typedef struct {
    int32_t kind;
    int32_t order;
    int32_t center;
} tt_pfunctional;

#define TT_MAX_TFUNCTIONALS 8
#define TT_MAX_PFUNCTIONALS 16

/* Opaque engine state: device tables (T3-T5 kernels, FFT chirps, Hermite
 * bases), staging buffers and streams of one device.  Re-entrant per plan;
 * one plan must not be used by two threads at once. */
typedef struct tt_plan tt_plan;

/* ---- plans and errors ------------------------------------------------ */
tt_status tt_plan_create(tt_plan **plan, int device);
tt_status tt_plan_destroy(tt_plan *plan);
/* Message for the last failed call on this thread ("" if none). */
const char *tt_last_error(void);
/* Library version string. */
const char *tt_version(void);

/* ---- geometry (host only) -------------------------------------------- */
/* Side N of the padded square and the offset of the image inside it:
 * pad() of c++/src/auxiliary.cpp:257-275. */
tt_status tt_pad_geometry(int rows, int cols, int *n, int *row_off, int *col_off);
/* Side the orthonormal (Hermite) mode stretches the image to before padding:
 * Transformer::Transformer, c++/src/transform.cpp:35-41. */
tt_status tt_ortho_size(unsigned angle_stepsize, int *side);
/* Angles a_step * step, a_step in [0, floor(360 / step)), in degrees
 * (c++/src/sinogram.cpp:77, 112).  *count receives the number of angles;
 * angles may be NULL to query it. */
tt_status tt_angles_from_step(unsigned angle_stepsize, float *angles, int capacity,
                              int *count);

/* ---- drop-in entry points (host buffers, synchronous) ----------------- */
/* Replaces getSinograms(const Eigen::MatrixXf& padded, unsigned
 * angle_stepsize, const std::vector<TFunctionalWrapper>&)
 * (c++/src/sinogram.hpp:57-59, c++/src/sinogram.cpp:67-178).
 * padded: rows x cols, must be square (the reference asserts it).
 * out: n_t x (rows x floor(360 / angle_stepsize)). plan may be NULL (the
 * process-wide plan of the current device is used). */
tt_status tt_sinograms(tt_plan *plan, const float *padded, int rows, int cols,
                       unsigned angle_stepsize, const int32_t *tfuncs, int n_t,
                       float *out);

/* Replaces getCircusFunctions(const Eigen::MatrixXf& sinogram, const
 * std::vector<PFunctionalWrapper>&) (c++/src/circus.hpp:69-71,
 * c++/src/circus.cpp:104-177).  sinogram: rows x cols; out: n_p x cols.
 * Hermite entries need center >= 0 (the reference dereferences the optional). */
tt_status tt_circus(tt_plan *plan, const float *sinogram, int rows, int cols,
                    const tt_pfunctional *pfuncs, int n_p, float *out);

/* Replaces rotate(input, origin, deg2rad(angle)) with the origin
 * ((cols-1)/2, (rows-1)/2) that getSinograms uses (c++/src/auxiliary.cpp:
 * 223-255, c++/src/sinogram.cpp:73-74, c++/src/rottest.cpp:46-49).  The
 * rotated image is bit-identical to the reference's; it uses the sampling
 * code of the fused sinogram kernel, which never writes it out. */
tt_status tt_rotate(tt_plan *plan, const float *image, int rows, int cols, float angle_deg,
                    float *out);

/* Replaces resize(input, rows, cols) (c++/src/auxiliary.cpp:198-221), the
 * orthonormal mode's stretch (c++/src/transform.cpp:35-41).  image:
 * in_rows x in_cols, out: rows x cols, both column-major; bit-identical to
 * the reference, whose outermost output rows and columns stay zero.  Needs
 * rows, cols >= 1 and in_rows, in_cols >= 1. */
tt_status tt_resize(tt_plan *plan, const float *image, int in_rows, int in_cols, int rows,
                    int cols, float *out);

/* Replaces zscore(const Eigen::VectorXf&) (c++/src/auxiliary.cpp:305-318)
 * applied to n_vec consecutive vectors of length len. */
tt_status tt_zscore(tt_plan *plan, const float *in, int n_vec, int len, float *out);

/* Replaces Transformer(image, basename, angle_step, orthonormal) +
 * getTransform(T, P, write_data) (c++/src/transform.cpp:28-112) without the
 * file output: image is the unpadded rows x cols image (values as gray2mat
 * gives them).  Orthonormal mode is selected as demo.cpp:153-169 does: all P
 * Hermite -> orthonormal, none -> regular, mixed -> TT_ERR_INVALID_ARG.
 * circus (may be NULL): n_t x n_p x A raw circus functions.
 * signatures (may be NULL): A x (n_t * n_p) z-scored.
 * In orthonormal mode the Hermite centers come from the nearest orthonormal
 * sinogram; the centers of pfuncs are ignored (the reference overwrites
 * them). */
tt_status tt_transform(tt_plan *plan, const float *image, int rows, int cols,
                       unsigned angle_stepsize, const int32_t *tfuncs, int n_t,
                       const tt_pfunctional *pfuncs, int n_p, float *circus,
                       float *signatures);

/* Transformer's two modes over the same sinograms in one call, from host
 * buffers.  The reference computes P1-P3 (regular mode) and the Hermite
 * circus (orthonormal mode) in separate Transformer runs, the latter on the
 * image stretched to tt_ortho_size (c++/src/transform.cpp:28-112,
 * demo.cpp:153-169 rejects mixing them); this call computes, for the
 * unstretched image and an explicit angle list (degrees, any values),
 * every T-functional's sinogram once, the regular circus functions of pfuncs
 * (P1-P3 only) and the Hermite circus of hermite_orders on each sinogram's
 * nearest orthonormal sinogram (c++/src/circus.cpp:68-102, centers as
 * transform.cpp:75-85 sets them).  circus / signatures (may be NULL):
 * n_t x n_p x n_angles as tt_transform; hermite_circus / hermite_signatures
 * (may be NULL): n_t x n_h x n_angles; centers (may be NULL): n_t. */
tt_status tt_transform_extended(tt_plan *plan, const float *image, int rows, int cols,
                                const float *angles_deg, int n_angles, const int32_t *tfuncs,
                                int n_t, const tt_pfunctional *pfuncs, int n_p,
                                const int32_t *hermite_orders, int n_h, float *circus,
                                float *signatures, float *hermite_circus,
                                float *hermite_signatures, int32_t *centers);

/* ---- device entry points (stream ordered) ----------------------------- */
/* Fused rotate + T-functional sweep over an explicit angle list (degrees;
 * the integer-step list of the reference is tt_angles_from_step).
 * src: src_rows x src_cols image with leading dimension src_ld, placed at
 * (row_off, col_off) inside an n x n zero frame (row_off = col_off = 0 and
 * src_rows = src_cols = n for an already padded image).
 * d_out: n_t x n x n_angles.  d_medians (may be NULL): n_t x n x n_angles
 * int32, the weighted-median row each T-functional used (-1 for Radon). */
tt_status tt_sinograms_device(tt_plan *plan, const float *d_src, int src_rows,
                              int src_cols, int src_ld, int n, int row_off,
                              int col_off, const float *angles_deg, int n_angles,
                              const int32_t *tfuncs, int n_t, float *d_out,
                              int32_t *d_medians, void *stream);

/* P-functionals over n_sino stacked rows x cols sinograms.  d_out:
 * n_sino x n_p x cols.  Hermite centers: centers[s] (host array of n_sino
 * entries) when not NULL, else each pfunctional's own center. */
tt_status tt_circus_device(tt_plan *plan, const float *d_sino, int rows, int cols,
                           int n_sino, const tt_pfunctional *pfuncs, int n_p,
                           const int32_t *centers, float *d_out, void *stream);

/* Orthonormal (Hermite) circus functions of n_sino stacked rows x cols
 * sinograms (as tt_sinograms_device wrote them): each sinogram's nearest
 * orthonormal sinogram (c++/src/circus.cpp:68-102; here a column-pivoting
 * QR in double-float, a one-sided Jacobi SVD of R^T in float and Q applied on
 * the device), then the Hermite P-functionals with the center it yields
 * (c++/src/transform.cpp:75-85).  pfuncs must all be TT_P_HERMITE (their
 * centers are ignored).  d_out: n_sino x n_p x cols; centers (host, may be
 * NULL): the n_sino centers used.  The reference runs this only on images
 * stretched to tt_ortho_size; here it takes sinograms of any size, so a
 * Hermite circus can sit beside P1-P3 of the regular sinograms.
 * Synchronises the stream once (the aligned matrices' sizes depend on the
 * weighted medians); the Jacobi sweeps loop on the device (a conditional
 * graph node whose stop rule runs after each sweep).  *sweeps (may be NULL)
 * receives the number of sweeps -- asking for it adds a synchronisation at
 * the end.  TT_ERR_UNSUPPORTED for more than 1024 angles, for more than 8192
 * aligned rows (rows plus the spread of the weighted-median offsets), or when
 * the aligned rows are fewer than the angles. */
tt_status tt_circus_orthonormal_device(tt_plan *plan, const float *d_sino, int rows, int cols,
                                       int n_sino, const tt_pfunctional *pfuncs, int n_p,
                                       float *d_out, int32_t *centers, int32_t *sweeps,
                                       void *stream);

/* Replaces nearest_orthonormal_sinogram(const Eigen::MatrixXf&, unsigned
 * int& new_center) (c++/src/circus.cpp:68-102) for one rows x cols host
 * sinogram.  out must hold 2 rows x cols floats; *out_rows receives the
 * aligned row count m (out is m x cols), *new_center the center.
 * TT_ERR_UNSUPPORTED when m < cols (the reference's U.block needs m >= cols). */
tt_status tt_nos(tt_plan *plan, const float *sinogram, int rows, int cols, float *out,
                 int32_t *out_rows, int32_t *new_center);

/* z-score of n_vec consecutive vectors of length len (device). */
tt_status tt_zscore_device(tt_plan *plan, const float *d_in, int n_vec, int len,
                           float *d_out, void *stream);

/* Synchronise the plan's stream. */
tt_status tt_plan_synchronize(tt_plan *plan);

/* ---- backward pass -------------------------------------------------------- */
/* The reference has no derivatives; these are the adjoints of the forward
 * path for T0, T1, T2 (c++/src/functionals.cpp:95-129), P1 and P3
 * (:287-360) and the bilinear rotation (c++/src/auxiliary.cpp:182-255).
 * The weighted median of T1/T2 is held at the row the forward chose (pass
 * the d_medians the forward wrote).  Other functionals are
 * TT_ERR_UNSUPPORTED. */
/* d_grad_circus: n_sino x n_p x cols -> d_grad_sino: n_sino x cols x rows. */
tt_status tt_circus_backward_device(tt_plan *plan, const float *d_sino, int rows, int cols,
                                    int n_sino, const tt_pfunctional *pfuncs, int n_p,
                                    const float *d_grad_circus, float *d_grad_sino,
                                    void *stream);
/* n_images images of one size at a time: d_grad_sino, d_medians: n_images
 * stacks of n_t x n x n_angles (as tt_sinograms_device wrote them) ->
 * d_grad_image: n_images column-major src_rows x src_cols images (the
 * rotation adjoint, gathered per pixel; rotations are recomputed, not
 * stored).  Scratch of 16 n n_angles n_images bytes (32 for f64) is held by
 * the plan. */
tt_status tt_sinograms_backward_device(tt_plan *plan, int n_images, int src_rows, int src_cols,
                                       int n,
                                       int row_off, int col_off, const float *angles_deg,
                                       int n_angles, const int32_t *tfuncs, int n_t,
                                       const float *d_grad_sino, const int32_t *d_medians,
                                       float *d_grad_image, void *stream);
/* Double-precision forward (T0-T2 on a rows x cols image in its pad() frame,
 * with exact double coordinates; P1, P3) and backward, for finite-difference
 * checks. */
tt_status tt_sinograms_f64_device(tt_plan *plan, const double *d_img, int rows, int cols,
                                  const float *angles_deg, int n_angles, const int32_t *tfuncs,
                                  int n_t, double *d_out, int32_t *d_medians, void *stream);
tt_status tt_circus_f64_device(tt_plan *plan, const double *d_sino, int rows, int cols,
                               int n_sino, const tt_pfunctional *pfuncs, int n_p, double *d_out,
                               void *stream);
tt_status tt_circus_backward_f64_device(tt_plan *plan, const double *d_sino, int rows, int cols,
                                        int n_sino, const tt_pfunctional *pfuncs, int n_p,
                                        const double *d_grad_circus, double *d_grad_sino,
                                        void *stream);
tt_status tt_sinograms_backward_f64_device(tt_plan *plan, int n_images, int src_rows,
                                           int src_cols, int n,
                                           int row_off, int col_off, const float *angles_deg,
                                           int n_angles, const int32_t *tfuncs, int n_t,
                                           const double *d_grad_sino, const int32_t *d_medians,
                                           double *d_grad_image, void *stream);

/* ---- batched engine ------------------------------------------------------ */
/* Many images of uneven sizes and angle counts in one pass: the reference
 * transforms its inputs one after another (the demo's loop over files and
 * components, c++/src/demo.cpp:179-254, each a Transformer::getTransform,
 * c++/src/transform.cpp:49-112; the CUDA port gives each GPU thread one
 * image, cuda/src/demo.cpp:258-266).  Image i is rows[i] x cols[i],
 * column-major, at images + offsets[i] (elements); it is transformed with
 * 360 / angle_steps[i] angles (integer degrees), the T- and P-functionals
 * given (P1-P3; Hermite is TT_ERR_UNSUPPORTED here).  circus and signatures
 * receive, image after image, each image's n_t x n_p x A_i block (the layout
 * of tt_transform).  The first call for a batch shape (sizes, steps,
 * functionals, input pointer) builds per-image textures and per-size tables,
 * times the persistent kernel's tile shapes on the batch (the choice is kept
 * in $TT_AUTOTUNE_CACHE, default ~/.cache/tracetransform_gb300_autotune.json)
 * and captures one CUDA graph: work-counter reset, image copies, a persistent
 * sinogram kernel, the batched P-functional kernel and the batched z-score;
 * later calls of that shape replay the graph. */
tt_status tt_transform_batch(tt_plan *plan, const float *images, const int64_t *offsets,
                             const int32_t *rows, const int32_t *cols, const int32_t *angle_steps,
                             int n_images, const int32_t *tfuncs, int n_t,
                             const tt_pfunctional *pfuncs, int n_p, float *circus,
                             float *signatures);
/* The same on device buffers, ordered on stream (NULL: the plan's stream);
 * d_circus / d_signatures may be NULL. */
tt_status tt_transform_batch_device(tt_plan *plan, const float *d_images, const int64_t *offsets,
                                    const int32_t *rows, const int32_t *cols,
                                    const int32_t *angle_steps, int n_images,
                                    const int32_t *tfuncs, int n_t, const tt_pfunctional *pfuncs,
                                    int n_p, float *d_circus, float *d_signatures, void *stream);

/* The sinograms behind the plan's last tt_transform_batch[_device] call,
 * image after image in input order, each n_t x A_i x N_i as
 * tt_sinograms_device writes them (N_i from tt_pad_geometry): the per-image
 * sinograms the reference writes in its debug output
 * (Transformer::getTransform with write_data, c++/src/transform.cpp:61-72).
 * *count (may be NULL) receives the float count, 0 before the first batch;
 * d_out may be NULL to query it, else it must hold capacity >= *count floats.
 * Ordered on stream (NULL: the plan's stream) after the last batch. */
tt_status tt_transform_batch_sinograms_device(tt_plan *plan, float *d_out, int64_t capacity,
                                              int64_t *count, void *stream);

/* Device time, in milliseconds, of the three kernels of the plan's last
 * batched call (ms[0] sinograms, ms[1] P-functionals, ms[2] z-scores), from
 * CUDA events recorded inside the captured graph; waits for that call. */
tt_status tt_transform_batch_stage_ms(tt_plan *plan, float *ms);

/* The persistent sinogram kernel's tile shape, tile = {lines per CTA, CTAs
 * per SM, lines per warp}: lines per warp 0 is the CTA kernel (one warp per
 * line, 8 or 4 lines per CTA, every T-functional); 1, 2 or 4 the
 * warp-autonomous kernel (each warp samples and reduces that many lines of
 * its own; T0-T5 only).  pin = 0: reads the shape the last batch used (the
 * autotuner's choice).  pin != 0: fixes *tile for the following batches
 * instead of tuning (CTAs per SM 0 returns to the tuner). */
tt_status tt_transform_batch_tile(tt_plan *plan, int32_t *tile, int32_t pin);

/* Testing aid (no counterpart in the reference): the next `count` device
 * allocations the library makes fail as if the device were out of memory,
 * without touching the device, so callers can test their handling of
 * TT_ERR_OOM (the reference's CUDAHelper::Error on cudaMalloc,
 * cuda/src/cudahelper/errorhandling.hpp:24-31).  count = 0 disarms it. */
tt_status tt_debug_fail_allocations(int count);

/* ---- allocation-free entry point ---------------------------------------- */
/* No counterpart in the reference.  P1 / P2 / P3 circus functions of n_sino
 * stacked rows x cols sinograms (device), z-scored into d_signatures
 * (n_sino x n_p x cols, the layout of tt_circus_device + tt_zscore_device),
 * for callers that cannot allocate device memory while they run -- a plugin
 * whose host application's allocator owns all device memory, or a loop that
 * cannot afford cudaMalloc/cudaFree stalls.  It runs the kernels of
 * tt_circus_device (same results, bit for bit) and allocates nothing: their
 * scratch -- raw circus values, P3 partial sums and tables, the P2 sort list --
 * lives in one file-scope device array of 1048576 floats (4 MiB) that every
 * GPU loading the library holds until the process exits.  Requests whose
 * scratch exceeds it fail with TT_ERR_INVALID_ARG (about n_sino * cols *
 * (n_p + 2) floats, plus with P3 n_sino * cols * ceil((rows / 2 + 1) / 64) +
 * 2.5 rows); P3 needs rows <= 2048 (TT_ERR_INVALID_ARG beyond); Hermite is
 * TT_ERR_UNSUPPORTED (use tt_circus_device).  The first call on a device
 * looks up the array's device address; with CUDA's lazy module loading it is
 * also where the array is allocated, so make that first call before any
 * region that must not allocate (or set CUDA_MODULE_LOADING=EAGER), and
 * before any stream capture.  cudaDeviceReset between calls is not supported.
 * Every call shares the array and it keeps the last call's contents (the one
 * counter that must start at zero is cleared by each call on its stream);
 * calls that overlap on the GPU race on it.  stream: a CUDA stream handle,
 * NULL for the legacy default stream. */
tt_status tt_circus_zscore_noalloc(const float *d_sino, int rows, int cols, int n_sino,
                                   const tt_pfunctional *pfuncs, int n_p, float *d_signatures,
                                   void *stream);

#ifdef __cplusplus
}
#endif
#endif
