// tt_noalloc.cu -- circus functions and signatures without any allocation.
//
// Some callers cannot allocate device memory when they run the P-stage: a
// plugin inside a host application whose own allocator owns every byte of
// device memory (a fixed budget that a stray cudaMalloc would break), or a
// latency-critical loop where cudaMalloc / cudaFree would stall the device.
// tt_circus_zscore_noalloc serves them: the caller passes the sinograms and
// the signature buffer, and the only other device memory it touches is the
// file-scope array below, which every GPU that loads this library holds
// until the process exits.
//
// It runs the same kernels as the allocating path (tt_circus_device: the
// direct-DFT P3, the warp-per-column P1/P2, the exact-sort fallback of P2,
// then the z-scores), with their scratch carved out of the array: the raw
// circus functions, the P3 partial sums, the P3 tables (built on the device
// by a kernel, so nothing is copied from the host) and the P2 fallback list.
// Every call shares the array and it keeps the last call's contents: the
// fallback counter, the only part that must start at zero, is cleared by the
// call on its stream before use; calls that overlap on the GPU -- on
// different streams, or from different host threads -- race on it.
//
// The array's device address is looked up once per device (the first call
// made with that device current); with CUDA's lazy module loading that first
// call is also where the CUDA driver loads this module and allocates the array,
// so make it before any region that must not allocate (or run with
// CUDA_MODULE_LOADING=EAGER).  The cached address does not survive
// cudaDeviceReset.
#include <cstdio>
#include <mutex>

#include "tracetransform.h"
#include "tt_internal.h"

namespace {

constexpr size_t kScratchFloats = size_t(1) << 20; // 4 MiB
constexpr int kMaxDevices = 64;

__device__ __align__(256) float g_noalloc_scratch[kScratchFloats];

std::mutex g_setup_mu;
float *g_scratch_addr[kMaxDevices]; // device address of the array, per device

size_t align64(size_t floats) { return (floats + 63) & ~size_t(63); } // 256 bytes

tt_status fail(tt_status st, const char *fmt, int a = 0, int b = 0, long c = 0) {
    char buf[320];
    snprintf(buf, sizeof buf, fmt, a, b, c);
    tt::record_error((int)st, buf);
    return st;
}

tt_status cuda_fail(cudaError_t e, const char *what) {
    char buf[320];
    snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
    tt::record_error((int)TT_ERR_CUDA, buf);
    return TT_ERR_CUDA;
}

} // namespace

extern "C" tt_status tt_circus_zscore_noalloc(const float *d_sino, int rows, int cols,
                                              int n_sino, const tt_pfunctional *pfuncs,
                                              int n_p, float *d_signatures, void *stream) {
    if (rows <= 0 || cols < 0 || n_sino < 0 || n_p < 0 || n_p > tt::kMaxP)
        return fail(TT_ERR_INVALID_ARG, "bad sizes: %d rows, %d columns, %ld P-functionals",
                    rows, cols, n_p);
    if ((size_t)n_sino * n_p * cols == 0)
        return TT_OK;
    if (!d_sino || !d_signatures || !pfuncs)
        return fail(TT_ERR_INVALID_ARG, "NULL sinogram, signature or P-functional pointer");
    unsigned need = 0;
    for (int p = 0; p < n_p; p++) {
        if (pfuncs[p].kind == TT_P_HERMITE)
            return fail(TT_ERR_UNSUPPORTED,
                        "Hermite P-functionals need per-sinogram bases: use tt_circus_device");
        if (pfuncs[p].kind < TT_P1 || pfuncs[p].kind > TT_P3)
            return fail(TT_ERR_INVALID_ARG, "invalid P-functional kind %d", pfuncs[p].kind);
        need |= 1u << pfuncs[p].kind;
    }
    const bool p3 = need & (1u << TT_P3);
    if (p3 && rows > tt::kP3DftMaxRows)
        return fail(TT_ERR_INVALID_ARG,
                    "P3 without allocation supports sinograms of at most %d rows, got %d",
                    tt::kP3DftMaxRows, rows);
    const size_t total_cols = (size_t)n_sino * cols;
    if (total_cols > 0x7fffffffu / 8)
        return fail(TT_ERR_INVALID_ARG, "%d sinograms of %d columns exceed the column limit",
                    n_sino, cols);
    if (tt::circus_warp_smem_bytes(rows) > 227 * 1024)
        return fail(TT_ERR_UNSUPPORTED, "sinogram length %d exceeds the shared-memory buffers",
                    rows);
    const int mtiles = p3 ? tt::p3_freq_tiles(rows) : 0;
    // layout (256-byte aligned): circus | P3 partials | twiddles | trapz
    // weights | P2 fallback count + list (int2)
    const size_t circ_floats = (size_t)n_sino * n_p * cols;
    const size_t off_part = align64(circ_floats);
    const size_t off_tw = off_part + (p3 ? align64((size_t)mtiles * total_cols) : 0);
    const size_t off_ck = off_tw + (p3 ? align64(2 * (size_t)rows) : 0);
    const size_t off_fb = off_ck + (p3 ? align64((size_t)rows / 2 + 1) : 0);
    const size_t total = off_fb + align64(2 * (total_cols + 1));
    if (total > kScratchFloats)
        return fail(TT_ERR_INVALID_ARG,
                    "%d x %d circus values plus scratch need %ld floats; the "
                    "allocation-free limit is 1048576 floats (4 MiB)",
                    n_sino * n_p, cols, (long)total);
    int sl = 1;
    while (sl < rows)
        sl <<= 1;
    if (sizeof(float) * (size_t)sl > 227 * 1024)
        return fail(TT_ERR_UNSUPPORTED, "sinogram length %d exceeds the sort buffer", rows);

    // one-time set-up per device: the array's device address
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices)
        return fail(TT_ERR_UNSUPPORTED, "device %d beyond the %d supported", dev, kMaxDevices);
    float *scratch;
    int sms = 0;
    {
        std::lock_guard<std::mutex> lock(g_setup_mu);
        if (!g_scratch_addr[dev]) {
            void *ptr = nullptr;
            e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
            if (e != cudaSuccess)
                return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
            g_scratch_addr[dev] = static_cast<float *>(ptr);
        }
        scratch = g_scratch_addr[dev];
    }
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaDeviceGetAttribute");
    cudaStream_t st = (cudaStream_t)stream;

    tt::CircusStackArgs a{};
    tt::CircusStack &S = a.one;
    S.sino = d_sino;
    S.out = scratch;
    S.n = rows;
    S.angles = cols;
    S.cols = (int)total_cols;
    S.mtiles = mtiles;
    S.partial = scratch + off_part;
    if (p3) {
        float2 *tw = reinterpret_cast<float2 *>(scratch + off_tw);
        float *ck = scratch + off_ck;
        e = tt::launch_p3_dft_tables(rows, tw, ck, st);
        if (e != cudaSuccess)
            return cuda_fail(e, "P3 table kernel");
        S.tw = tw;
        S.ck = ck;
    }
    a.st = nullptr;
    a.n_st = 1;
    a.total_tiles = mtiles * (int)((total_cols + 127) / 128);
    a.total_cols = (int)total_cols;
    a.n_p = n_p;
    for (int p = 0; p < n_p; p++)
        a.kind[p] = pfuncs[p].kind;
    a.need = need;
    a.stride = tt::circus_warp_stride(rows);
    a.fb_count = reinterpret_cast<unsigned *>(scratch + off_fb);
    a.fb_list = reinterpret_cast<int2 *>(scratch + off_fb) + 1;
    a.fb_capacity = (int)total_cols;
    a.sort_len_max = sl;
    a.fb_grid = 2 * sms;
    e = tt::launch_circus_stacks(a, tt::circus_warp_smem_bytes(rows), st);
    if (e != cudaSuccess)
        return cuda_fail(e, "circus kernels");
    e = tt::launch_zscore(scratch, n_sino * n_p, cols, d_signatures, st);
    if (e != cudaSuccess)
        return cuda_fail(e, "z-score kernel");
    return TT_OK;
}
