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
// The array holds the raw circus functions (the intermediate between the
// P-functional kernel and the z-score kernel) and, when P3 is requested, the
// P3 tables.  Every call shares it and it keeps the last call's contents:
// nothing in it needs to start at zero (every element is written before it is
// read), but calls that overlap on the GPU -- on different streams, or from
// different host threads -- race on it.
#include <complex>
#include <cstdio>
#include <mutex>

#include "tracetransform.h"
#include "tt_internal.h"

namespace {

constexpr size_t kScratchFloats = size_t(1) << 20; // 4 MiB
constexpr int kMaxRowsP3 = 8192;                    // P3 FFT length <= 16384
constexpr int kMaxDevices = 64;

__device__ __align__(256) float g_noalloc_scratch[kScratchFloats];

std::mutex g_setup_mu;
float *g_scratch_addr[kMaxDevices]; // device address of the array, per device

// host staging for the P3 tables (static: the call allocates nothing)
std::mutex g_tables_mu;
float2 g_chirp[kMaxRowsP3], g_filt[2 * kMaxRowsP3], g_twid[kMaxRowsP3];
float g_lin[kMaxRowsP3];
std::complex<double> g_work[2 * kMaxRowsP3];

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
    if (p3 && rows > kMaxRowsP3)
        return fail(TT_ERR_INVALID_ARG,
                    "P3 without allocation supports sinograms of at most %d rows, got %d",
                    kMaxRowsP3, rows);
    const int M = p3 ? tt::p3_fft_length(rows) : 0;
    // layout: circus | chirp | filter | twiddles | linspace (256-byte aligned)
    const size_t circ_floats = (size_t)n_sino * n_p * cols;
    const size_t off_chirp = align64(circ_floats);
    const size_t off_filt = off_chirp + (p3 ? align64(2 * (size_t)rows) : 0);
    const size_t off_twid = off_filt + (p3 ? align64(2 * (size_t)M) : 0);
    const size_t off_lin = off_twid + (p3 ? align64((size_t)M) : 0);
    const size_t total = off_lin + (p3 ? align64((size_t)rows) : 0);
    if (total > kScratchFloats)
        return fail(TT_ERR_INVALID_ARG,
                    "%d x %d circus values plus tables need %ld floats of scratch; the "
                    "allocation-free limit is 1048576 floats (4 MiB)",
                    n_sino * n_p, cols, (long)total);

    // one-time set-up per device: the array's device address
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices)
        return fail(TT_ERR_UNSUPPORTED, "device %d beyond the %d supported", dev, kMaxDevices);
    float *scratch;
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
    cudaStream_t st = (cudaStream_t)stream;

    tt::CircusArgs a{};
    a.sino = d_sino;
    a.rows = rows;
    a.cols = cols;
    a.n_sino = n_sino;
    a.n_p = n_p;
    for (int p = 0; p < n_p; p++)
        a.kind[p] = pfuncs[p].kind;
    a.need = need;
    a.out = scratch;
    int sl = 1;
    while (sl < rows)
        sl <<= 1;
    a.sort_len = sl;
    if (p3) {
        a.M = M;
        a.chirp = reinterpret_cast<const float2 *>(scratch + off_chirp);
        a.filt = reinterpret_cast<const float2 *>(scratch + off_filt);
        a.twid = reinterpret_cast<const float2 *>(scratch + off_twid);
        a.lin = scratch + off_lin;
        // copies from pageable host memory return once the source is staged,
        // so the static staging buffers may be reused right after
        std::lock_guard<std::mutex> lock(g_tables_mu);
        tt::p3_tables(rows, g_chirp, g_filt, g_twid, g_lin, g_work);
        const struct {
            size_t off, bytes;
            const void *src;
        } copies[4] = {{off_chirp, sizeof(float2) * rows, g_chirp},
                       {off_filt, sizeof(float2) * M, g_filt},
                       {off_twid, sizeof(float2) * (M / 2), g_twid},
                       {off_lin, sizeof(float) * rows, g_lin}};
        for (const auto &c : copies) {
            e = cudaMemcpyAsync(scratch + c.off, c.src, c.bytes, cudaMemcpyHostToDevice, st);
            if (e != cudaSuccess)
                return cuda_fail(e, "cudaMemcpyAsync(P3 tables)");
        }
    }
    if (tt::circus_smem_bytes(a) > 227 * 1024)
        return fail(TT_ERR_UNSUPPORTED, "sinogram length %d exceeds the shared-memory buffers",
                    rows);
    e = tt::launch_circus(a, st);
    if (e != cudaSuccess)
        return cuda_fail(e, "circus kernel");
    e = tt::launch_zscore(scratch, n_sino * n_p, cols, d_signatures, st);
    if (e != cudaSuccess)
        return cuda_fail(e, "z-score kernel");
    return TT_OK;
}
