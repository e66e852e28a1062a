// tt_api.cu -- C ABI of the trace-transform engine: plans, host-side tables,
// and the drop-in and device entry points declared in include/tracetransform.h.
//
// Host-side tables are evaluated with the reference's own expressions so that
// the device kernels see the reference's float values:
//   rotation      cos/sin of -deg2rad(a) on a float   (c++/src/auxiliary.cpp:180, 227-237)
//   T3, T4, T5    r^k * exp(i m log r) in double, rounded once (c++/src/functionals.cpp:136-198)
//   P3 linspace   -1 + p * 2.0 / (N - 1) in double, rounded once (c++/src/functionals.cpp:346-355)
//   Hermite       hermite_function with its double intermediates (c++/src/functionals.cpp:62-84, 369-386)
#include <algorithm>
#include <atomic>
#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "tracetransform.h"
#include "tt_internal.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

using tt::CircusArgs;
using tt::CircusStack;
using tt::CircusStackArgs;
using tt::NosDesc;
using tt::SinoArgs;

namespace {

thread_local std::string g_error;

tt_status fail(tt_status st, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_error = buf;
    return st;
}

#define TT_CUDA(call)                                                          \
    do {                                                                       \
        cudaError_t e_ = (call);                                               \
        if (e_ != cudaSuccess)                                                 \
            return fail(e_ == cudaErrorMemoryAllocation ? TT_ERR_OOM           \
                                                        : TT_ERR_CUDA,         \
                        "%s: %s (%s:%d)", #call, cudaGetErrorString(e_),       \
                        __FILE__, __LINE__);                                   \
    } while (0)

#define TT_CHECK(expr)                                                         \
    do {                                                                       \
        tt_status s_ = (expr);                                                 \
        if (s_ != TT_OK)                                                       \
            return s_;                                                         \
    } while (0)

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
};

struct FftTables {
    int M = 0;
    float2 *chirp = nullptr, *filt = nullptr, *twid = nullptr;
    float *lin = nullptr;
};

// A gather-capable CUDA array holding a source image (texel (u, v) = image
// row u, column v) and its border-mode texture object.
struct SourceTexture {
    cudaArray_t arr = nullptr;
    cudaTextureObject_t tex = 0;
    int rows = 0, cols = 0;

    void release() {
        if (tex)
            cudaDestroyTextureObject(tex);
        if (arr)
            cudaFreeArray(arr);
        tex = 0;
        arr = nullptr;
        rows = cols = 0;
    }
};

// ---- host math -----------------------------------------------------------

float deg2rad(float degrees) { return (float)(degrees * M_PI / 180); }

float hermite_polynomial(unsigned order, float x) {
    switch (order) {
    case 0:
        return 1.0f;
    case 1:
        return (float)(2.0 * x);
    default:
        return (float)(2.0 * x * hermite_polynomial(order - 1, x) -
                       2.0 * (order - 1) * hermite_polynomial(order - 2, x));
    }
}

unsigned factorial(unsigned n) { return (n == 1 || n == 0) ? 1 : factorial(n - 1) * n; }

float hermite_function(unsigned order, float x) {
    const float half_sq = x * x / 2;
    return (float)(hermite_polynomial(order, x) /
                   (std::sqrt(std::pow(2.0, (double)order) * factorial(order) *
                              std::sqrt(M_PI)) *
                    std::exp((double)half_sq)));
}

// The basis psi(order, z(p)) that PFunctionalHermite multiplies the column by.
std::vector<float> hermite_basis(int n, unsigned order, int center) {
    std::vector<float> b(n);
    const float lower = (float)(10.0 / center);
    const float upper = (float)(10.0 / (n - 1 - center));
    for (int p = 0; p < n; p++) {
        float z;
        if (p < center)
            z = p * lower - 10;
        else
            z = (p - center) * upper;
        b[p] = hermite_function(order, z);
    }
    return b;
}

using tt::pad_geometry;

int ortho_side(unsigned step) {
    const size_t ndiag = (int)std::ceil(360.0 / step);
    return (int)std::ceil(ndiag / std::sqrt(2));
}


} // namespace

// ---- the plan ----------------------------------------------------------------

struct tt_plan {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::map<int, float2 *> t345;                       // n -> 3 x n
    std::map<int, FftTables> fft;                       // n -> P3 tables
    std::map<std::tuple<int, int, int>, float *> herm;  // (n, order, center)
    std::map<std::vector<float>, float2 *> trig;        // angle list -> (c, s)
    std::map<std::vector<long>, const float **> herm_ptrs;
    DevBuf in, stretch, sino, circ, sig, region, nos, batch_in, batch_out, params;
    // P-stage scratch: P3 partial sums, the exact-sort list of P2 (count + entries)
    DevBuf cpart, cfb;
    std::map<int, std::pair<float2 *, float *>> p3dft; // n -> twiddles, trapz weights
    std::map<int, float *> p3tc;                        // n -> tensor-core twiddle blocks
    int sms = 0;
    // nearest orthonormal sinogram scratch (double matrices, V, norms, ...)
    DevBuf nos_a, nos_work, nos_desc, nos_off;
    // the QR and one Jacobi sweep as graphs, for the buffers and sizes they
    // were captured with
    struct Graph {
        cudaGraphExec_t exec = nullptr;
        std::vector<const void *> key;
    } nos_factor_graph, nos_sweep_graph;
    cudaStream_t capture_stream = nullptr;
    SourceTexture src;
    tt::BatchEngine *batch = nullptr;
    // backward / double-precision tables
    std::map<int, float *> dft32;                  // n -> cos, sin(2 pi j / n), 2 n
    std::map<int, double *> dft64, lin64;
    std::map<std::vector<float>, double *> trig64; // angle list -> (cos, sin) in double
    std::map<std::vector<int>, int *> kinds;

    template <typename T> tt_status get_dft(int n, const T **cosv, const T **sinv) {
        std::map<int, T *> &cache = dft_cache((T *)nullptr);
        auto it = cache.find(n);
        if (it == cache.end()) {
            std::vector<T> h(2 * (size_t)n);
            for (int j = 0; j < n; j++) {
                h[j] = (T)std::cos(2 * M_PI * j / n);
                h[n + j] = (T)std::sin(2 * M_PI * j / n);
            }
            T *d;
            TT_CHECK(upload(&d, h));
            it = cache.emplace(n, d).first;
        }
        *cosv = it->second;
        *sinv = it->second + n;
        return TT_OK;
    }
    std::map<int, float *> &dft_cache(float *) { return dft32; }
    std::map<int, double *> &dft_cache(double *) { return dft64; }

    tt_status get_lin64(int n, const double **out) {
        auto it = lin64.find(n);
        if (it == lin64.end()) {
            std::vector<double> h(n);
            for (int p = 0; p < n; p++)
                h[p] = -1 + p * 2.0 / (n - 1);
            double *d;
            TT_CHECK(upload(&d, h));
            it = lin64.emplace(n, d).first;
        }
        *out = it->second;
        return TT_OK;
    }

    tt_status get_trig64(const float *angles, int n_angles, const double **out) {
        std::vector<float> key(angles, angles + n_angles);
        auto it = trig64.find(key);
        if (it == trig64.end()) {
            std::vector<double> h(2 * (size_t)n_angles);
            for (int a = 0; a < n_angles; a++) {
                const double th = angles[a] * M_PI / 180;
                h[2 * a] = std::cos(-th);
                h[2 * a + 1] = std::sin(-th);
            }
            double *d;
            TT_CHECK(upload(&d, h));
            it = trig64.emplace(key, d).first;
        }
        *out = it->second;
        return TT_OK;
    }

    tt_status get_kinds(const tt_pfunctional *pf, int n_p, const int **out) {
        std::vector<int> key;
        for (int p = 0; p < n_p; p++)
            key.push_back(pf[p].kind);
        auto it = kinds.find(key);
        if (it == kinds.end()) {
            int *d;
            TT_CHECK(upload(&d, key.empty() ? std::vector<int>{0} : key));
            it = kinds.emplace(key, d).first;
        }
        *out = it->second;
        return TT_OK;
    }
    std::vector<void *> owned;

    ~tt_plan() {
        int prev = 0;
        cudaGetDevice(&prev);
        cudaSetDevice(device);
        if (stream)
            cudaStreamSynchronize(stream);
        cudaDeviceSynchronize();
        tt::batch_destroy(batch);
        src.release();
        for (void *p : owned)
            cudaFree(p);
        for (DevBuf *b : {&in, &sino, &circ, &sig, &region, &nos, &batch_in, &batch_out, &params,
                          &nos_a, &nos_work, &nos_desc, &nos_off, &cpart, &cfb})
            cudaFree(b->p);
        for (Graph *g : {&nos_factor_graph, &nos_sweep_graph})
            if (g->exec)
                cudaGraphExecDestroy(g->exec);
        if (capture_stream)
            cudaStreamDestroy(capture_stream);
        if (stream)
            cudaStreamDestroy(stream);
        cudaSetDevice(prev);
    }

    tt_status alloc(void **p, size_t bytes) {
        TT_CUDA(tt::dev_malloc(p, bytes > 0 ? bytes : 1));
        owned.push_back(*p);
        return TT_OK;
    }
    // Capture fn's launches on the plan's capture stream as g (unless g was
    // captured with the same key) so that they replay as one graph launch.
    template <typename F> tt_status graph(Graph &g, const std::vector<const void *> &key, F fn) {
        if (g.exec && g.key == key)
            return TT_OK;
        if (g.exec) {
            TT_CUDA(cudaGraphExecDestroy(g.exec));
            g.exec = nullptr;
        }
        if (!capture_stream)
            TT_CUDA(cudaStreamCreateWithFlags(&capture_stream, cudaStreamNonBlocking));
        TT_CUDA(cudaStreamBeginCapture(capture_stream, cudaStreamCaptureModeThreadLocal));
        const cudaError_t le = fn(capture_stream);
        cudaGraph_t gr = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(capture_stream, &gr);
        cudaError_t ie = cudaSuccess;
        if (le == cudaSuccess && ce == cudaSuccess)
            ie = cudaGraphInstantiate(&g.exec, gr, 0);
        if (gr)
            cudaGraphDestroy(gr);
        TT_CUDA(le);
        TT_CUDA(ce);
        TT_CUDA(ie);
        g.key = key;
        return TT_OK;
    }
    // A graph that runs the body fn captures while the body keeps its
    // condition set (cudaGraphSetConditional from a body kernel); each
    // launch of the graph starts with the condition at 1, so the body runs
    // at least once.
    template <typename F>
    tt_status while_graph(Graph &g, const std::vector<const void *> &key, F fn) {
        if (g.exec && g.key == key)
            return TT_OK;
        if (g.exec) {
            TT_CUDA(cudaGraphExecDestroy(g.exec));
            g.exec = nullptr;
        }
        if (!capture_stream)
            TT_CUDA(cudaStreamCreateWithFlags(&capture_stream, cudaStreamNonBlocking));
        cudaGraph_t gr = nullptr;
        TT_CUDA(cudaGraphCreate(&gr, 0));
        cudaGraphConditionalHandle loop = 0;
        cudaError_t e = cudaGraphConditionalHandleCreate(&loop, gr, 1, cudaGraphCondAssignDefault);
        cudaGraphNodeParams np{};
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = loop;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        cudaGraphNode_t node = nullptr;
        if (e == cudaSuccess)
            e = cudaGraphAddNode(&node, gr, nullptr, nullptr, 0, &np);
        if (e == cudaSuccess)
            e = cudaStreamBeginCaptureToGraph(capture_stream, np.conditional.phGraph_out[0],
                                              nullptr, nullptr, 0,
                                              cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            const cudaError_t le = fn(capture_stream, loop);
            cudaGraph_t body = nullptr;
            const cudaError_t ce = cudaStreamEndCapture(capture_stream, &body);
            e = le != cudaSuccess ? le : ce;
        }
        if (e == cudaSuccess)
            e = cudaGraphInstantiate(&g.exec, gr, 0);
        cudaGraphDestroy(gr);
        TT_CUDA(e);
        g.key = key;
        return TT_OK;
    }
    tt_status ensure(DevBuf &b, size_t bytes) {
        if (b.bytes >= bytes && b.p)
            return TT_OK;
        if (b.p) {
            TT_CUDA(cudaStreamSynchronize(stream));
            cudaFree(b.p);
            b.p = nullptr;
            b.bytes = 0;
        }
        TT_CUDA(tt::dev_malloc(&b.p, bytes > 0 ? bytes : 1));
        b.bytes = bytes;
        return TT_OK;
    }
    // Tables are created once and read by kernels on any stream, so the copy
    // completes before the table is handed out.
    template <typename T> tt_status upload(T **dst, const std::vector<T> &h) {
        TT_CHECK(alloc((void **)dst, sizeof(T) * h.size()));
        TT_CUDA(cudaMemcpyAsync(*dst, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, stream));
        TT_CUDA(cudaStreamSynchronize(stream));
        return TT_OK;
    }

    // Copy a rows x cols column-major device image (leading dimension ld)
    // into the source texture, stream ordered.  The array is reallocated only
    // when the size changes (after the device has drained: kernels in flight
    // may still read the old texture).
    tt_status load_source(const float *d_img, int rows, int cols, int ld, cudaStream_t st,
                          cudaTextureObject_t *tex) {
        if (rows > 32768 || cols > 32768)
            return fail(TT_ERR_UNSUPPORTED, "image %dx%d exceeds the 32768 texture-gather limit",
                        rows, cols);
        if (src.rows != rows || src.cols != cols) {
            TT_CUDA(cudaDeviceSynchronize());
            src.release();
            cudaChannelFormatDesc desc = cudaCreateChannelDesc<float>();
            TT_CUDA(tt::dev_malloc_array(&src.arr, &desc, rows, cols, cudaArrayTextureGather));
            cudaResourceDesc res{};
            res.resType = cudaResourceTypeArray;
            res.res.array.array = src.arr;
            cudaTextureDesc td{};
            td.addressMode[0] = cudaAddressModeBorder;
            td.addressMode[1] = cudaAddressModeBorder;
            td.filterMode = cudaFilterModePoint;
            td.readMode = cudaReadModeElementType;
            td.normalizedCoords = 0;
            TT_CUDA(cudaCreateTextureObject(&src.tex, &res, &td, nullptr));
            src.rows = rows;
            src.cols = cols;
        }
        if (d_img)
            TT_CUDA(cudaMemcpy2DToArrayAsync(src.arr, 0, 0, d_img, sizeof(float) * (size_t)ld,
                                             sizeof(float) * (size_t)rows, cols,
                                             cudaMemcpyDeviceToDevice, st));
        *tex = src.tex;
        return TT_OK;
    }

    tt_status get_trig(const float *angles, int n_angles, const float2 **out) {
        std::vector<float> key(angles, angles + n_angles);
        auto it = trig.find(key);
        if (it != trig.end()) {
            *out = it->second;
            return TT_OK;
        }
        std::vector<float2> h(n_angles);
        for (int a = 0; a < n_angles; a++) {
            h[a] = tt::rotation(angles[a]);
        }
        float2 *d;
        TT_CHECK(upload(&d, h));
        trig[key] = d;
        *out = d;
        return TT_OK;
    }

    tt_status get_t345(int n, const float2 **out) {
        auto it = t345.find(n);
        if (it != t345.end()) {
            *out = it->second;
            return TT_OK;
        }
        std::vector<float2> h((size_t)3 * n);
        tt::t345_tables(n, h.data());
        float2 *d;
        TT_CHECK(upload(&d, h));
        t345[n] = d;
        *out = d;
        return TT_OK;
    }

    tt_status get_fft(int n, const FftTables **out) {
        auto it = fft.find(n);
        if (it != fft.end()) {
            *out = &it->second;
            return TT_OK;
        }
        FftTables t;
        const int M = tt::p3_fft_length(n);
        t.M = M;
        std::vector<float2> chirp(n), filt(M), twid(M / 2);
        std::vector<float> lin(n);
        std::vector<std::complex<double>> work(M);
        tt::p3_tables(n, chirp.data(), filt.data(), twid.data(), lin.data(), work.data());
        TT_CHECK(upload(&t.chirp, chirp));
        TT_CHECK(upload(&t.filt, filt));
        TT_CHECK(upload(&t.twid, twid));
        TT_CHECK(upload(&t.lin, lin));
        fft[n] = t;
        *out = &fft[n];
        return TT_OK;
    }

    tt_status get_p3dft(int n, const float2 **tw, const float **ck) {
        auto it = p3dft.find(n);
        if (it == p3dft.end()) {
            float2 *dt;
            float *dc;
            TT_CHECK(upload(&dt, std::vector<float2>(n)));
            TT_CHECK(upload(&dc, std::vector<float>(n / 2 + 1)));
            TT_CUDA(tt::launch_p3_dft_tables(n, dt, dc, stream));
            TT_CUDA(cudaStreamSynchronize(stream));
            it = p3dft.emplace(n, std::make_pair(dt, dc)).first;
        }
        *tw = it->second.first;
        *ck = it->second.second;
        return TT_OK;
    }

    // The tensor-core P3's twiddle blocks of n (built once from the twiddles).
    tt_status get_p3tc(int n, const float2 *tw, const float **out) {
        auto it = p3tc.find(n);
        if (it == p3tc.end()) {
            float *d;
            TT_CHECK(alloc((void **)&d, sizeof(float) * tt::p3_tc_table_floats(n)));
            TT_CUDA(tt::launch_p3_tc_tables(n, tw, d, stream));
            TT_CUDA(cudaStreamSynchronize(stream));
            it = p3tc.emplace(n, d).first;
        }
        *out = it->second;
        return TT_OK;
    }

    tt_status get_herm(int n, int order, int center, const float **out) {
        auto key = std::make_tuple(n, order, center);
        auto it = herm.find(key);
        if (it != herm.end()) {
            *out = it->second;
            return TT_OK;
        }
        float *d;
        TT_CHECK(upload(&d, hermite_basis(n, (unsigned)order, center)));
        herm[key] = d;
        *out = d;
        return TT_OK;
    }
};

namespace {

std::mutex g_default_mu;
std::map<int, tt_plan *> g_default;

tt_status resolve_plan(tt_plan *plan, tt_plan **out) {
    if (plan) {
        *out = plan;
        TT_CUDA(cudaSetDevice(plan->device));
        return TT_OK;
    }
    int dev = 0;
    TT_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(g_default_mu);
    auto it = g_default.find(dev);
    if (it == g_default.end()) {
        tt_plan *p = nullptr;
        TT_CHECK(tt_plan_create(&p, dev));
        g_default[dev] = p;
        *out = p;
    } else {
        *out = it->second;
    }
    return TT_OK;
}

cudaStream_t pick_stream(tt_plan *p, void *stream) {
    return stream ? (cudaStream_t)stream : p->stream;
}

tt_status check_tfuncs(const int32_t *tfuncs, int n_t, unsigned *need) {
    if (n_t < 0 || n_t > tt::kMaxT)
        return fail(TT_ERR_INVALID_ARG, "between 0 and %d T-functionals are supported, got %d",
                    tt::kMaxT, n_t);
    if (n_t > 0 && !tfuncs)
        return fail(TT_ERR_INVALID_ARG, "tfuncs is NULL");
    *need = 0;
    for (int t = 0; t < n_t; t++) {
        if (tfuncs[t] < 0 || tfuncs[t] > 7)
            return fail(TT_ERR_INVALID_ARG, "invalid T-functional id %d (valid: 0..7)", tfuncs[t]);
        *need |= 1u << tfuncs[t];
    }
    return TT_OK;
}

tt_status check_pfuncs(const tt_pfunctional *pf, int n_p, bool need_center, unsigned *need) {
    if (n_p < 0 || n_p > tt::kMaxP)
        return fail(TT_ERR_INVALID_ARG, "between 0 and %d P-functionals are supported, got %d",
                    tt::kMaxP, n_p);
    if (n_p > 0 && !pf)
        return fail(TT_ERR_INVALID_ARG, "pfuncs is NULL");
    *need = 0;
    for (int p = 0; p < n_p; p++) {
        if (pf[p].kind < 0 || pf[p].kind > 3)
            return fail(TT_ERR_INVALID_ARG, "invalid P-functional kind %d", pf[p].kind);
        if (pf[p].kind == TT_P_HERMITE) {
            if (pf[p].order < 0)
                return fail(TT_ERR_INVALID_ARG, "Hermite P-functional needs an order >= 0");
            if (need_center && pf[p].center < 0)
                return fail(TT_ERR_INVALID_ARG, "Hermite P-functional needs a center");
        }
        *need |= 1u << pf[p].kind;
    }
    return TT_OK;
}

std::vector<float> step_angles(unsigned step) {
    const int k = (int)std::floor(360 / step);
    std::vector<float> a(k);
    for (int i = 0; i < k; i++)
        a[i] = (float)(i * step);
    return a;
}

// Sinograms of a region placed in an n x n frame (device pointers).
tt_status run_sinograms(tt_plan *p, const float *d_src, int src_rows, int src_cols, int src_ld,
                        int n, int row_off, int col_off, const int *d_region,
                        const float *angles, int n_angles, const int32_t *tfuncs, int n_t,
                        unsigned need, float *d_out, int32_t *d_medians, cudaStream_t st) {
    if (n_angles == 0 || n_t == 0 || n == 0)
        return TT_OK;
    SinoArgs a{};
    if (src_rows > 0 && src_cols > 0) {
        TT_CHECK(p->load_source(d_src, src_rows, src_cols, src_ld, st, &a.tex));
    } else {
        src_rows = src_cols = 0; // nothing to sample: every line is zero
        TT_CHECK(p->load_source(nullptr, 1, 1, 1, st, &a.tex));
    }
    a.tex_row_off = row_off;
    a.tex_col_off = col_off;
    a.src_rows = src_rows;
    a.src_cols = src_cols;
    a.interior = src_rows > 0 && src_cols > 0 &&
                 tt::interior_source(n, row_off, col_off, src_rows, src_cols);
    a.row_off = row_off;
    a.col_off = col_off;
    a.dyn_region = d_region;
    a.n = n;
    a.n_angles = n_angles;
    TT_CHECK(p->get_trig(angles, n_angles, &a.trig));
    a.tab = nullptr;
    if (need & ((1u << 3) | (1u << 4) | (1u << 5)))
        TT_CHECK(p->get_t345(n, &a.tab));
    a.out = d_out;
    a.medians = d_medians;
    a.n_t = n_t;
    for (int t = 0; t < n_t; t++)
        a.tf[t] = tfuncs[t];
    a.need = need;
    if (!(need & ((1u << 6) | (1u << 7))) && n <= 1024 && n_t <= tt::kWarpMaxOutputs) {
        // T0-T5 of short lines: two lines per warp (the shape the batch tuner
        // picks for lines of this length)
        a.stride = tt::sino_warp_stride(n, 2);
        TT_CUDA(tt::launch_sinograms_warp(a, 2, st));
        return TT_OK;
    }
    const int L = tt::sino_lines_per_block(n, need);
    a.stride = tt::sino_stride(n, L);
    if (tt::sino_smem_bytes(n, L, need) > 227 * 1024)
        return fail(TT_ERR_UNSUPPORTED, "padded side %d exceeds the shared-memory line buffer", n);
    TT_CUDA(tt::launch_sinograms(a, L, st));
    return TT_OK;
}

// P1-P3 without Hermite: P3 as a DFT computed like a GEMM, P1 / P2 one warp
// per column (launch_circus_stacks), the stack descriptor passed by value.
tt_status run_circus_stacks(tt_plan *p, const float *d_sino, int rows, int cols, int n_sino,
                            const tt_pfunctional *pf, int n_p, unsigned need, float *d_out,
                            cudaStream_t st) {
    if ((need & (1u << 3)) && rows > tt::kP3DftMaxRows) {
        // P3 of long columns: the chirp-z FFT kernel (its accumulation error
        // does not grow with the column as the direct DFT's does), the rest here
        CircusArgs a{};
        a.sino = d_sino;
        a.rows = rows;
        a.cols = cols;
        a.n_sino = n_sino;
        a.n_p = n_p;
        for (int i = 0; i < n_p; i++)
            a.kind[i] = pf[i].kind;
        a.need = 1u << 3;
        a.out = d_out;
        int sl = 1;
        while (sl < rows)
            sl <<= 1;
        a.sort_len = sl;
        const FftTables *f;
        TT_CHECK(p->get_fft(rows, &f));
        a.M = f->M;
        a.chirp = f->chirp;
        a.filt = f->filt;
        a.twid = f->twid;
        a.lin = f->lin;
        if (tt::circus_smem_bytes(a) > 227 * 1024)
            return fail(TT_ERR_UNSUPPORTED, "sinogram length %d exceeds the FFT buffers", rows);
        TT_CUDA(tt::launch_circus(a, st));
        need &= ~(1u << 3);
        if (!(need & ((1u << 1) | (1u << 2))))
            return TT_OK;
    }
    if (tt::circus_warp_smem_bytes(rows) > 227 * 1024)
        return fail(TT_ERR_UNSUPPORTED, "sinogram length %d exceeds the shared-memory column "
                                        "buffers", rows);
    CircusStackArgs a{};
    CircusStack &S = a.one;
    S.sino = d_sino;
    S.out = d_out;
    S.n = rows;
    S.angles = cols;
    S.cols = cols * n_sino;
    S.mtiles = (need & (1u << 3)) ? tt::p3_freq_tiles(rows) : 0;
    if (need & (1u << 3)) {
        TT_CHECK(p->get_p3dft(rows, &S.tw, &S.ck));
        TT_CHECK(p->get_p3tc(rows, S.tw, &S.wtc));
        a.tc_tables = 1;
    }
    const size_t part = (size_t)S.mtiles * S.cols;
    TT_CHECK(p->ensure(p->cpart, sizeof(float) * std::max<size_t>(part, 1)));
    TT_CHECK(p->ensure(p->cfb, sizeof(int2) * ((size_t)S.cols + 1)));
    S.partial = (float *)p->cpart.p;
    a.st = nullptr;
    a.n_st = 1;
    a.total_tiles = S.mtiles * ((S.cols + 127) / 128);
    a.total_cols = S.cols;
    a.n_p = n_p;
    for (int i = 0; i < n_p; i++)
        a.kind[i] = (need & (1u << pf[i].kind)) ? pf[i].kind : -1; // -1: written elsewhere
    a.need = need;
    a.stride = tt::circus_warp_stride(rows);
    a.fb_count = (unsigned *)p->cfb.p;
    a.fb_list = (int2 *)p->cfb.p + 1;
    a.fb_capacity = S.cols;
    int sl = 1;
    while (sl < rows)
        sl <<= 1;
    a.sort_len_max = sl;
    if (!p->sms)
        TT_CUDA(cudaDeviceGetAttribute(&p->sms, cudaDevAttrMultiProcessorCount, p->device));
    a.fb_grid = 2 * p->sms;
    if (sizeof(float) * (size_t)sl > 227 * 1024)
        return fail(TT_ERR_UNSUPPORTED, "sinogram length %d exceeds the sort buffer", rows);
    TT_CUDA(tt::launch_circus_stacks(a, tt::circus_warp_smem_bytes(rows), st));
    return TT_OK;
}

tt_status run_circus(tt_plan *p, const float *d_sino, int rows, int cols, int n_sino,
                     const tt_pfunctional *pf, int n_p, const int32_t *centers, unsigned need,
                     float *d_out, cudaStream_t st) {
    if (n_p == 0 || cols == 0 || n_sino == 0)
        return TT_OK;
    if (rows <= 0)
        return fail(TT_ERR_INVALID_ARG, "sinograms need at least one row");
    if (!(need & 1u) && (size_t)cols * n_sino <= 0x7fffffff / 8)
        return run_circus_stacks(p, d_sino, rows, cols, n_sino, pf, n_p, need, d_out, st);
    CircusArgs a{};
    a.sino = d_sino;
    a.rows = rows;
    a.cols = cols;
    a.n_sino = n_sino;
    a.n_p = n_p;
    for (int i = 0; i < n_p; i++)
        a.kind[i] = pf[i].kind;
    a.need = need;
    a.out = d_out;
    int sl = 1;
    while (sl < rows)
        sl <<= 1;
    a.sort_len = sl;
    if (need & (1u << 3)) {
        const FftTables *f;
        TT_CHECK(p->get_fft(rows, &f));
        a.M = f->M;
        a.chirp = f->chirp;
        a.filt = f->filt;
        a.twid = f->twid;
        a.lin = f->lin;
    }
    if (need & 1u) {
        std::vector<long> key;
        key.push_back(rows);
        std::vector<const float *> ptrs((size_t)n_sino * n_p, nullptr);
        for (int s = 0; s < n_sino; s++)
            for (int i = 0; i < n_p; i++) {
                if (pf[i].kind != TT_P_HERMITE)
                    continue;
                const int center = centers ? centers[s] : pf[i].center;
                if (center < 0)
                    return fail(TT_ERR_INVALID_ARG, "Hermite P-functional needs a center");
                const float *b;
                TT_CHECK(p->get_herm(rows, pf[i].order, center, &b));
                ptrs[(size_t)s * n_p + i] = b;
                key.push_back(((long)s * n_p + i) * 1000003L + pf[i].order * 100003L + center);
            }
        auto it = p->herm_ptrs.find(key);
        if (it == p->herm_ptrs.end()) {
            const float **d;
            TT_CHECK(p->upload(&d, ptrs));
            p->herm_ptrs[key] = d;
            a.herm = d;
        } else {
            a.herm = it->second;
        }
    }
    if (tt::circus_smem_bytes(a) > 227 * 1024)
        return fail(TT_ERR_UNSUPPORTED, "sinogram length %d exceeds the shared-memory column buffers",
                    rows);
    TT_CUDA(tt::launch_circus(a, st));
    return TT_OK;
}

// Nearest orthonormal sinograms (c++/src/circus.cpp:68-102) of n_sino device
// sinograms of rows x cols: results in p->nos, desc[s].out_off / .m per
// sinogram, centers[s] the new Hermite centers.  One host synchronisation:
// the aligned matrices' sizes depend on the weighted medians (a second, at
// the end, only when *sweeps is asked for).
tt_status run_nos(tt_plan *p, const float *d_sino, int rows, int cols, int n_sino,
                  cudaStream_t st, std::vector<NosDesc> &desc, std::vector<int> &centers,
                  int *sweeps = nullptr) {
    const int center = (int)std::floor((rows - 1) / 2.0);
    const size_t ncol = (size_t)cols * n_sino;
    TT_CHECK(p->ensure(p->nos_off, sizeof(int) * std::max<size_t>(ncol, 1)));
    TT_CUDA(tt::launch_nos_offsets(d_sino, rows, cols, n_sino, center, (int *)p->nos_off.p, st));
    std::vector<int> off(ncol);
    TT_CUDA(cudaMemcpyAsync(off.data(), p->nos_off.p, sizeof(int) * ncol, cudaMemcpyDeviceToHost,
                            st));
    TT_CUDA(cudaStreamSynchronize(st));
    desc.assign(n_sino, NosDesc{});
    centers.assign(n_sino, 0);
    size_t a_elems = 0;
    int max_m = 0;
    for (int s = 0; s < n_sino; s++) {
        const int *o = off.data() + (size_t)s * cols;
        const int mn = *std::min_element(o, o + cols), mx = *std::max_element(o, o + cols);
        const int m = rows + std::abs(mx) + std::abs(mn);
        if (m < cols)
            return fail(TT_ERR_UNSUPPORTED,
                        "nearest orthonormal sinogram needs at least as many rows (%d) as angles "
                        "(%d)", m, cols);
        desc[s].a_off = desc[s].out_off = (long long)a_elems;
        desc[s].m = m;
        desc[s].mx = mx;
        centers[s] = center + mx;
        a_elems += (size_t)m * cols;
        max_m = std::max(max_m, m);
    }
    TT_CHECK(p->ensure(p->nos_a, sizeof(float2) * a_elems));
    TT_CHECK(p->ensure(p->nos_desc, sizeof(NosDesc) * n_sino));
    TT_CHECK(p->ensure(p->nos, sizeof(float) * a_elems));
    if (max_m > tt::nos_max_rows())
        return fail(TT_ERR_UNSUPPORTED,
                    "nearest orthonormal sinogram of %d aligned rows exceeds %d", max_m,
                    tt::nos_max_rows());
    if (cols > 1024)
        return fail(TT_ERR_UNSUPPORTED, "orthonormal circus of %d angles exceeds 1024", cols);
    // scratch: 5 double-float + 3 int vectors of n, 3 float n x n matrices,
    // 2 float vectors, the sweep loop's state, then (256-byte aligned) the
    // blocked Q application's
    const size_t nv = ncol, nm = (size_t)cols * cols * n_sino;
    const size_t head = sizeof(float2) * 5 * nv + sizeof(int) * 3 * nv +
                        sizeof(float) * (3 * nm + 2 * nv) + sizeof(unsigned) * n_sino +
                        sizeof(float) * n_sino + sizeof(unsigned) * 2;
    const size_t wy_at = (head + 255) & ~size_t(255);
    TT_CHECK(p->ensure(p->nos_work,
                       wy_at + sizeof(float) * tt::nos_assemble_floats(cols, n_sino, max_m)));
    tt::NosWork w;
    {
        char *q = (char *)p->nos_work.p;
        w.norms = (float2 *)q;
        w.tau = w.norms + 2 * nv;
        w.beta = w.tau + nv;
        w.scale = w.beta + nv;
        w.orig = (float *)(w.scale + nv);
        w.X = w.orig + nv;
        w.V = w.X + nm;
        w.P = w.V + nm;
        w.inv = w.P + nm;
        w.cmap = (int *)(w.inv + nv);
        w.perm = w.cmap + 2 * nv;
        w.off_bits = (unsigned *)(w.perm + nv);
        w.tiny = (float *)(w.off_bits + n_sino);
        w.sweep_state = (unsigned *)(w.tiny + n_sino);
        w.wy = (float *)((char *)p->nos_work.p + wy_at);
    }
    TT_CUDA(cudaMemcpyAsync(p->nos_desc.p, desc.data(), sizeof(NosDesc) * n_sino,
                            cudaMemcpyHostToDevice, st));
    float2 *A = (float2 *)p->nos_a.p; // double-float pairs
    const NosDesc *d_desc = (const NosDesc *)p->nos_desc.p;
    TT_CUDA(tt::launch_nos_align(d_sino, rows, cols, n_sino, d_desc, (const int *)p->nos_off.p,
                                 A, a_elems, st));
    // QR (cols + 2 launches) and one Jacobi sweep (about cols / 16 launches),
    // each captured once per buffer set and size and replayed
    const std::vector<const void *> key = {A, d_desc, p->nos_work.p,
                                           (const void *)(size_t)cols,
                                           (const void *)(size_t)n_sino,
                                           (const void *)(size_t)(max_m <= 2048   ? 0
                                                                  : max_m <= 4096 ? 1
                                                                                  : 2)};
    TT_CHECK(p->graph(p->nos_factor_graph, key, [&](cudaStream_t cs) {
        return tt::launch_nos_factor(A, d_desc, cols, n_sino, max_m, w, cs);
    }));
    // the sweeps: a device-side while loop (the stop rule runs after each
    // sweep on the device), at most 40
    TT_CHECK(p->while_graph(p->nos_sweep_graph, key,
                            [&](cudaStream_t cs, cudaGraphConditionalHandle loop) {
                                return tt::launch_nos_sweep(cols, n_sino, w, 40, loop, cs);
                            }));
    TT_CUDA(cudaGraphLaunch(p->nos_factor_graph.exec, st));
    TT_CUDA(cudaMemsetAsync(w.sweep_state, 0, sizeof(unsigned) * 2, st));
    TT_CUDA(cudaGraphLaunch(p->nos_sweep_graph.exec, st));
    TT_CUDA(tt::launch_nos_assemble(A, d_desc, cols, n_sino, max_m, w, (float *)p->nos.p, st));
    if (sweeps) { // the count is read back only when asked for
        unsigned done = 0;
        TT_CUDA(cudaMemcpyAsync(&done, w.sweep_state + 1, sizeof done, cudaMemcpyDeviceToHost,
                                st));
        TT_CUDA(cudaStreamSynchronize(st));
        *sweeps = (int)done;
    }
    return TT_OK;
}

} // namespace

namespace {
std::atomic<int> g_fail_allocs{0};
}

cudaError_t tt::dev_malloc(void **p, size_t bytes) {
    int left = g_fail_allocs.load();
    while (left > 0 && !g_fail_allocs.compare_exchange_weak(left, left - 1)) {
    }
    if (left > 0) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMalloc(p, bytes);
}

cudaError_t tt::dev_malloc_array(cudaArray_t *a, const cudaChannelFormatDesc *desc, size_t w,
                                 size_t h, unsigned flags) {
    int left = g_fail_allocs.load();
    while (left > 0 && !g_fail_allocs.compare_exchange_weak(left, left - 1)) {
    }
    if (left > 0) {
        *a = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMallocArray(a, desc, w, h, flags);
}

int tt::record_error(int status, const char *message) {
    g_error = message;
    return status;
}

// ---- C ABI ---------------------------------------------------------------------

extern "C" {

const char *tt_last_error(void) { return g_error.c_str(); }

const char *tt_version(void) { return "tracetransform-gb300 0.1 (sm_103a)"; }

tt_status tt_plan_create(tt_plan **plan, int device) {
    if (!plan)
        return fail(TT_ERR_INVALID_ARG, "plan is NULL");
    int count = 0;
    TT_CUDA(cudaGetDeviceCount(&count));
    if (device < 0 || device >= count)
        return fail(TT_ERR_INVALID_ARG, "device %d out of range (%d devices)", device, count);
    TT_CUDA(cudaSetDevice(device));
    tt_plan *p = new tt_plan();
    p->device = device;
    cudaError_t e = cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete p;
        return fail(TT_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
    }
    *plan = p;
    return TT_OK;
}

tt_status tt_plan_destroy(tt_plan *plan) {
    if (!plan)
        return TT_OK;
    {
        std::lock_guard<std::mutex> lock(g_default_mu);
        for (auto it = g_default.begin(); it != g_default.end(); ++it)
            if (it->second == plan) {
                g_default.erase(it);
                break;
            }
    }
    delete plan;
    return TT_OK;
}

static tt_status check_batch(const int64_t *offsets, const int32_t *rows, const int32_t *cols,
                             const int32_t *steps, int n_images, const int32_t *tfuncs, int n_t,
                             const tt_pfunctional *pfuncs, int n_p, size_t *in_elems,
                             size_t *out_elems) {
    if (n_images < 0 || (n_images > 0 && (!offsets || !rows || !cols || !steps)))
        return fail(TT_ERR_INVALID_ARG, "bad batch description");
    unsigned need;
    TT_CHECK(check_tfuncs(tfuncs, n_t, &need));
    TT_CHECK(check_pfuncs(pfuncs, n_p, false, &need));
    for (int p = 0; p < n_p; p++)
        if (pfuncs[p].kind == TT_P_HERMITE)
            return fail(TT_ERR_UNSUPPORTED,
                        "the batched engine computes P1-P3; Hermite needs tt_transform");
    size_t in = 0, out = 0;
    for (int i = 0; i < n_images; i++) {
        if (rows[i] <= 0 || cols[i] <= 0 || offsets[i] < 0 || steps[i] <= 0 || steps[i] > 360)
            return fail(TT_ERR_INVALID_ARG, "batch image %d: %dx%d at %lld, step %d", i, rows[i],
                        cols[i], (long long)offsets[i], steps[i]);
        in = std::max(in, (size_t)offsets[i] + (size_t)rows[i] * cols[i]);
        out += (size_t)n_t * n_p * (360 / steps[i]);
    }
    *in_elems = in;
    *out_elems = out;
    return TT_OK;
}

tt_status tt_transform_batch_device(tt_plan *plan, const float *d_images, const int64_t *offsets,
                                    const int32_t *rows, const int32_t *cols,
                                    const int32_t *angle_steps, int n_images,
                                    const int32_t *tfuncs, int n_t, const tt_pfunctional *pfuncs,
                                    int n_p, float *d_circus, float *d_signatures, void *stream) {
    tt_plan *p;
    TT_CHECK(resolve_plan(plan, &p));
    size_t in_elems, out_elems;
    TT_CHECK(check_batch(offsets, rows, cols, angle_steps, n_images, tfuncs, n_t, pfuncs, n_p,
                         &in_elems, &out_elems));
    if (n_images == 0 || out_elems == 0)
        return TT_OK;
    if (!d_images)
        return fail(TT_ERR_INVALID_ARG, "NULL image buffer");
    if (!p->batch)
        p->batch = tt::batch_create(p->device);
    std::vector<long long> off(offsets, offsets + n_images);
    const int st = tt::batch_run(p->batch, d_images, off.data(), rows, cols, angle_steps,
                                 n_images, tfuncs, n_t, pfuncs, n_p, d_circus, d_signatures,
                                 pick_stream(p, stream));
    return (tt_status)st;
}

tt_status tt_transform_batch(tt_plan *plan, const float *images, const int64_t *offsets,
                             const int32_t *rows, const int32_t *cols, const int32_t *angle_steps,
                             int n_images, const int32_t *tfuncs, int n_t,
                             const tt_pfunctional *pfuncs, int n_p, float *circus,
                             float *signatures) {
    tt_plan *p;
    TT_CHECK(resolve_plan(plan, &p));
    size_t in_elems, out_elems;
    TT_CHECK(check_batch(offsets, rows, cols, angle_steps, n_images, tfuncs, n_t, pfuncs, n_p,
                         &in_elems, &out_elems));
    if (n_images == 0 || out_elems == 0)
        return TT_OK;
    if (!images)
        return fail(TT_ERR_INVALID_ARG, "NULL image buffer");
    cudaStream_t st = p->stream;
    TT_CHECK(p->ensure(p->batch_in, sizeof(float) * in_elems));
    TT_CHECK(p->ensure(p->batch_out, sizeof(float) * 2 * out_elems));
    TT_CUDA(cudaMemcpyAsync(p->batch_in.p, images, sizeof(float) * in_elems,
                            cudaMemcpyHostToDevice, st));
    float *d_circ = (float *)p->batch_out.p, *d_sig = d_circ + out_elems;
    TT_CHECK(tt_transform_batch_device(p, (const float *)p->batch_in.p, offsets, rows, cols,
                                       angle_steps, n_images, tfuncs, n_t, pfuncs, n_p, d_circ,
                                       d_sig, st));
    if (circus)
        TT_CUDA(cudaMemcpyAsync(circus, d_circ, sizeof(float) * out_elems, cudaMemcpyDeviceToHost,
                                st));
    if (signatures)
        TT_CUDA(cudaMemcpyAsync(signatures, d_sig, sizeof(float) * out_elems,
                                cudaMemcpyDeviceToHost, st));
    TT_CUDA(cudaStreamSynchronize(st));
    return TT_OK;
}

tt_status tt_transform_extended(tt_plan *plan, const float *image, int rows, int cols,
                                const float *angles_deg, int n_angles, const int32_t *tfuncs,
                                int n_t, const tt_pfunctional *pfuncs, int n_p,
                                const int32_t *hermite_orders, int n_h, float *circus,
                                float *signatures, float *hermite_circus,
                                float *hermite_signatures, int32_t *centers) {
    tt_plan *p;
    TT_CHECK(resolve_plan(plan, &p));
    if (rows <= 0 || cols <= 0 || !image)
        return fail(TT_ERR_INVALID_ARG, "empty image");
    if (n_angles < 0 || (n_angles > 0 && !angles_deg))
        return fail(TT_ERR_INVALID_ARG, "bad angle list");
    if (n_h < 0 || n_h > TT_MAX_PFUNCTIONALS || (n_h > 0 && !hermite_orders))
        return fail(TT_ERR_INVALID_ARG, "bad Hermite order list");
    unsigned tneed, pneed;
    TT_CHECK(check_tfuncs(tfuncs, n_t, &tneed));
    TT_CHECK(check_pfuncs(pfuncs, n_p, false, &pneed));
    for (int i = 0; i < n_p; i++)
        if (pfuncs[i].kind == TT_P_HERMITE)
            return fail(TT_ERR_INVALID_ARG, "pfuncs are the regular P-functionals; Hermite orders "
                                            "go in hermite_orders");
    std::vector<tt_pfunctional> hpf(n_h);
    for (int i = 0; i < n_h; i++)
        hpf[i] = tt_pfunctional{TT_P_HERMITE, hermite_orders[i], -1};
    unsigned hneed = 0;
    TT_CHECK(check_pfuncs(hpf.data(), n_h, false, &hneed));
    int n, ro, co;
    pad_geometry(rows, cols, &n, &ro, &co);
    const int A = n_angles;
    const size_t sino_elems = (size_t)n_t * n * A, circ_elems = (size_t)n_t * n_p * A,
                 herm_elems = (size_t)n_t * n_h * A;
    cudaStream_t st = p->stream;
    TT_CHECK(p->ensure(p->in, sizeof(float) * (size_t)rows * cols));
    TT_CHECK(p->ensure(p->sino, sizeof(float) * std::max<size_t>(sino_elems, 1)));
    TT_CHECK(p->ensure(p->circ, sizeof(float) * std::max<size_t>(circ_elems + herm_elems, 1)));
    TT_CHECK(p->ensure(p->sig, sizeof(float) * std::max<size_t>(circ_elems + herm_elems, 1)));
    TT_CUDA(cudaMemcpyAsync(p->in.p, image, sizeof(float) * (size_t)rows * cols,
                            cudaMemcpyHostToDevice, st));
    TT_CHECK(run_sinograms(p, (const float *)p->in.p, rows, cols, rows, n, ro, co, nullptr,
                           angles_deg, A, tfuncs, n_t, tneed, (float *)p->sino.p, nullptr, st));
    float *d_circ = (float *)p->circ.p, *d_herm = d_circ + circ_elems;
    float *d_sig = (float *)p->sig.p, *d_hsig = d_sig + circ_elems;
    if (A > 0 && n_t > 0) {
        TT_CHECK(run_circus(p, (const float *)p->sino.p, n, A, n_t, pfuncs, n_p, nullptr, pneed,
                            d_circ, st));
        if (n_h > 0) {
            std::vector<NosDesc> desc;
            std::vector<int> c;
            TT_CHECK(run_nos(p, (const float *)p->sino.p, n, A, n_t, st, desc, c));
            for (int t = 0; t < n_t; t++) {
                const int32_t c32 = c[t];
                TT_CHECK(run_circus(p, (const float *)p->nos.p + desc[t].out_off, desc[t].m, A,
                                    1, hpf.data(), n_h, &c32, hneed,
                                    d_herm + (size_t)t * n_h * A, st));
                if (centers)
                    centers[t] = c32;
            }
        }
        if (circ_elems + herm_elems > 0)
            TT_CUDA(tt::launch_zscore(d_circ, n_t * (n_p + n_h), A, d_sig, st));
    }
    if (circus && circ_elems)
        TT_CUDA(cudaMemcpyAsync(circus, d_circ, sizeof(float) * circ_elems,
                                cudaMemcpyDeviceToHost, st));
    if (signatures && circ_elems)
        TT_CUDA(cudaMemcpyAsync(signatures, d_sig, sizeof(float) * circ_elems,
                                cudaMemcpyDeviceToHost, st));
    if (hermite_circus && herm_elems)
        TT_CUDA(cudaMemcpyAsync(hermite_circus, d_herm, sizeof(float) * herm_elems,
                                cudaMemcpyDeviceToHost, st));
    if (hermite_signatures && herm_elems)
        TT_CUDA(cudaMemcpyAsync(hermite_signatures, d_hsig, sizeof(float) * herm_elems,
                                cudaMemcpyDeviceToHost, st));
    TT_CUDA(cudaStreamSynchronize(st));
    return TT_OK;
}

tt_status tt_transform_batch_sinograms_device(tt_plan *plan, float *d_out, int64_t capacity,
                                              int64_t *count, void *stream) {
    tt_plan *p;
    TT_CHECK(resolve_plan(plan, &p));
    if (capacity < 0)
        return fail(TT_ERR_INVALID_ARG, "negative capacity");
    size_t n = 0;
    if (p->batch) {
        const int st = tt::batch_sinograms(p->batch, d_out, (size_t)capacity, &n,
                                           pick_stream(p, stream));
        if (st != TT_OK)
            return (tt_status)st;
    }
    if (count)
        *count = (int64_t)n;
    return TT_OK;
}

tt_status tt_transform_batch_stage_ms(tt_plan *plan, float *ms) {
    tt_plan *p;
    TT_CHECK(resolve_plan(plan, &p));
    if (!ms)
        return fail(TT_ERR_INVALID_ARG, "NULL output");
    if (!p->batch)
        return fail(TT_ERR_INVALID_ARG, "no batch has run on this plan");
    return (tt_status)tt::batch_stage_ms(p->batch, ms);
}

tt_status tt_transform_batch_tile(tt_plan *plan, int32_t *tile, int32_t pin) {
    tt_plan *p;
    TT_CHECK(resolve_plan(plan, &p));
    if (!tile)
        return fail(TT_ERR_INVALID_ARG, "NULL tile");
    if (!p->batch)
        p->batch = tt::batch_create(p->device);
    int t[3] = {tile[0], tile[1], tile[2]};
    if (pin) {
        if (t[1] > 0 && !((t[2] == 0 && (t[0] == 8 || t[0] == 4)) ||
                          t[2] == 1 || t[2] == 2 || t[2] == 4))
            return fail(TT_ERR_INVALID_ARG, "tile: lines per CTA 8 or 4 (lines per warp 0), or "
                                            "lines per warp 1, 2 or 4");
        tt::batch_pin_tile(p->batch, t);
        return TT_OK;
    }
    tt::batch_tile(p->batch, t);
    for (int i = 0; i < 3; i++)
        tile[i] = t[i];
    return TT_OK;
}

// ---- backward ------------------------------------------------------------

static tt_status check_grad_funcs(const int32_t *tfuncs, int n_t, const tt_pfunctional *pf,
                                  int n_p, unsigned long long *code) {
    unsigned need;
    if (tfuncs || n_t) {
        TT_CHECK(check_tfuncs(tfuncs, n_t, &need));
        *code = 0;
        for (int t = 0; t < n_t; t++) {
            if (tfuncs[t] > 2)
                return fail(TT_ERR_UNSUPPORTED, "gradients exist for T0, T1 and T2, not T%d",
                            tfuncs[t]);
            *code |= (unsigned long long)tfuncs[t] << (3 * t);
        }
    }
    if (pf || n_p) {
        TT_CHECK(check_pfuncs(pf, n_p, false, &need));
        for (int p = 0; p < n_p; p++)
            if (pf[p].kind != TT_P1 && pf[p].kind != TT_P3)
                return fail(TT_ERR_UNSUPPORTED, "gradients exist for P1 and P3 only");
    }
    return TT_OK;
}

extern "C++" {
template <typename T>
static tt_status circus_backward_impl(tt_plan *plan, const T *d_sino, int rows, int cols,
                                      int n_sino, const tt_pfunctional *pf, int n_p,
                                      const T *d_grad_circus, T *d_grad_sino, void *stream) {
    tt_plan *p;
    TT_CHECK(resolve_plan(plan, &p));
    unsigned long long code;
    TT_CHECK(check_grad_funcs(nullptr, 0, pf, n_p, &code));
    if (rows <= 0 || cols < 0 || n_sino < 0 || !d_sino || !d_grad_circus || !d_grad_sino)
        return fail(TT_ERR_INVALID_ARG, "bad sinogram stack for the backward pass");
    const T *cosv, *sinv, *lin;
    const int *kinds;
    TT_CHECK(p->get_kinds(pf, n_p, &kinds));
    if (sizeof(T) == sizeof(float)) {
        const FftTables *f;
        TT_CHECK(p->get_fft(rows, &f)); // the forward's float linspace and FFT tables
        lin = (const T *)f->lin;
        // both DFTs of a column by the chirp-z FFT where its M-point buffer
        // fits in shared memory, else the direct sums below
        if (tt::circus_backward_fft_fits(rows, f->M)) {
            TT_CUDA(tt::launch_circus_backward_fft(
                (const float *)d_sino, rows, cols, n_sino, kinds, n_p,
                (const float *)d_grad_circus, f->chirp, f->filt, f->twid, f->M, f->lin,
                (float *)d_grad_sino, pick_stream(p, stream)));
            return TT_OK;
        }
        TT_CHECK(p->get_dft<T>(rows, &cosv, &sinv));
    } else {
        const double *l;
        TT_CHECK(p->get_lin64(rows, &l));
        lin = (const T *)l;
        TT_CHECK(p->get_dft<T>(rows, &cosv, &sinv));
    }
    TT_CUDA(tt::launch_circus_backward<T>(d_sino, rows, cols, n_sino, kinds, n_p, d_grad_circus,
                                          cosv, sinv, lin, d_grad_sino, pick_stream(p, stream)));
    return TT_OK;
}

template <typename T>
static tt_status sino_backward_impl(tt_plan *plan, int n_images, int src_rows, int src_cols,
                                    int n, int row_off,
                                    int col_off, const float *angles_deg, int n_angles,
                                    const int32_t *tfuncs, int n_t, const T *d_grad_sino,
                                    const int32_t *d_medians, T *d_grad_image, void *stream) {
    tt_plan *p;
    TT_CHECK(resolve_plan(plan, &p));
    unsigned long long code;
    TT_CHECK(check_grad_funcs(tfuncs, n_t, nullptr, 0, &code));
    if (n_images < 0 || n <= 0 || src_rows <= 0 || src_cols <= 0 || row_off < 0 || col_off < 0 ||
        row_off + src_rows > n || col_off + src_cols > n || n_angles < 0 || !angles_deg ||
        !d_grad_sino || !d_medians || !d_grad_image)
        return fail(TT_ERR_INVALID_ARG, "bad geometry or buffers for the backward pass");
    const T *cs;
    if (sizeof(T) == sizeof(float)) {
        const float2 *t;
        TT_CHECK(p->get_trig(angles_deg, n_angles, &t));
        cs = (const T *)t;
    } else {
        const double *t;
        TT_CHECK(p->get_trig64(angles_deg, n_angles, &t));
        cs = (const T *)t;
    }
    if (n_images == 0)
        return TT_OK;
    TT_CHECK(p->ensure(p->params,
                       sizeof(T) * 4 * (size_t)n * std::max(n_angles, 1) * (size_t)n_images));
    TT_CUDA(tt::launch_sino_backward<T>(d_grad_sino, d_medians, n_images, n, n_angles, code, n_t,
                                        (T *)p->params.p, src_rows, src_cols, row_off, col_off,
                                        cs, d_grad_image, pick_stream(p, stream)));
    return TT_OK;
}
} // extern "C++"

tt_status tt_circus_backward_device(tt_plan *plan, const float *d_sino, int rows, int cols,
                                    int n_sino, const tt_pfunctional *pfuncs, int n_p,
                                    const float *d_grad_circus, float *d_grad_sino,
                                    void *stream) {
    return circus_backward_impl<float>(plan, d_sino, rows, cols, n_sino, pfuncs, n_p,
                                       d_grad_circus, d_grad_sino, stream);
}

tt_status tt_sinograms_backward_device(tt_plan *plan, int n_images, int src_rows, int src_cols,
                                       int n, int row_off, int col_off, const float *angles_deg,
                                       int n_angles, const int32_t *tfuncs, int n_t,
                                       const float *d_grad_sino, const int32_t *d_medians,
                                       float *d_grad_image, void *stream) {
    return sino_backward_impl<float>(plan, n_images, src_rows, src_cols, n, row_off, col_off, angles_deg,
                                     n_angles, tfuncs, n_t, d_grad_sino, d_medians,
                                     d_grad_image, stream);
}

tt_status tt_circus_backward_f64_device(tt_plan *plan, const double *d_sino, int rows, int cols,
                                        int n_sino, const tt_pfunctional *pfuncs, int n_p,
                                        const double *d_grad_circus, double *d_grad_sino,
                                        void *stream) {
    return circus_backward_impl<double>(plan, d_sino, rows, cols, n_sino, pfuncs, n_p,
                                        d_grad_circus, d_grad_sino, stream);
}

tt_status tt_sinograms_backward_f64_device(tt_plan *plan, int n_images, int src_rows,
                                           int src_cols, int n, int row_off, int col_off, const float *angles_deg,
                                           int n_angles, const int32_t *tfuncs, int n_t,
                                           const double *d_grad_sino, const int32_t *d_medians,
                                           double *d_grad_image, void *stream) {
    return sino_backward_impl<double>(plan, n_images, src_rows, src_cols, n, row_off, col_off, angles_deg,
                                      n_angles, tfuncs, n_t, d_grad_sino, d_medians,
                                      d_grad_image, stream);
}

tt_status tt_sinograms_f64_device(tt_plan *plan, const double *d_img, int rows, int cols,
                                  const float *angles_deg, int n_angles, const int32_t *tfuncs,
                                  int n_t, double *d_out, int32_t *d_medians, void *stream) {
    tt_plan *p;
    TT_CHECK(resolve_plan(plan, &p));
    unsigned long long code;
    TT_CHECK(check_grad_funcs(tfuncs, n_t, nullptr, 0, &code));
    if (rows <= 0 || cols <= 0 || n_angles < 0 || !d_img || !d_out || !d_medians || !angles_deg)
        return fail(TT_ERR_INVALID_ARG, "bad double-precision sinogram arguments");
    int n, ro, co;
    pad_geometry(rows, cols, &n, &ro, &co);
    const double *cs;
    TT_CHECK(p->get_trig64(angles_deg, n_angles, &cs));
    TT_CUDA(tt::launch_sino_f64(d_img, rows, cols, ro, co, n, cs, code, n_t, n_angles, d_out,
                                d_medians, pick_stream(p, stream)));
    return TT_OK;
}

tt_status tt_circus_f64_device(tt_plan *plan, const double *d_sino, int rows, int cols,
                               int n_sino, const tt_pfunctional *pfuncs, int n_p, double *d_out,
                               void *stream) {
    tt_plan *p;
    TT_CHECK(resolve_plan(plan, &p));
    unsigned long long code;
    TT_CHECK(check_grad_funcs(nullptr, 0, pfuncs, n_p, &code));
    if (rows <= 0 || cols < 0 || n_sino < 0 || !d_sino || !d_out)
        return fail(TT_ERR_INVALID_ARG, "bad double-precision sinogram stack");
    const double *cosv, *sinv, *lin;
    const int *kinds;
    TT_CHECK(p->get_dft<double>(rows, &cosv, &sinv));
    TT_CHECK(p->get_lin64(rows, &lin));
    TT_CHECK(p->get_kinds(pfuncs, n_p, &kinds));
    TT_CUDA(tt::launch_circus_f64(d_sino, rows, cols, n_sino, kinds, n_p, cosv, sinv, lin, d_out,
                                  pick_stream(p, stream)));
    return TT_OK;
}

tt_status tt_debug_fail_allocations(int count) {
    if (count < 0)
        return fail(TT_ERR_INVALID_ARG, "negative count");
    g_fail_allocs.store(count);
    return TT_OK;
}

tt_status tt_plan_synchronize(tt_plan *plan) {
    tt_plan *p;
    TT_CHECK(resolve_plan(plan, &p));
    TT_CUDA(cudaStreamSynchronize(p->stream));
    return TT_OK;
}

tt_status tt_pad_geometry(int rows, int cols, int *n, int *row_off, int *col_off) {
    if (rows <= 0 || cols <= 0 || !n || !row_off || !col_off)
        return fail(TT_ERR_INVALID_ARG, "pad geometry needs a non-empty image and output pointers");
    pad_geometry(rows, cols, n, row_off, col_off);
    return TT_OK;
}

tt_status tt_ortho_size(unsigned step, int *side) {
    if (step == 0 || !side)
        return fail(TT_ERR_INVALID_ARG, "angle step must be >= 1");
    *side = ortho_side(step);
    return TT_OK;
}

tt_status tt_angles_from_step(unsigned step, float *angles, int capacity, int *count) {
    if (step == 0 || !count)
        return fail(TT_ERR_INVALID_ARG, "angle step must be >= 1");
    std::vector<float> a = step_angles(step);
    *count = (int)a.size();
    if (angles) {
        if (capacity < (int)a.size())
            return fail(TT_ERR_INVALID_ARG, "angle buffer holds %d, need %d", capacity, (int)a.size());
        std::copy(a.begin(), a.end(), angles);
    }
    return TT_OK;
}

tt_status tt_sinograms_device(tt_plan *plan, const float *d_src, int src_rows, int src_cols,
                              int src_ld, int n, int row_off, int col_off,
                              const float *angles_deg, int n_angles, const int32_t *tfuncs,
                              int n_t, float *d_out, int32_t *d_medians, void *stream) {
    tt_plan *p;
    TT_CHECK(resolve_plan(plan, &p));
    unsigned need;
    TT_CHECK(check_tfuncs(tfuncs, n_t, &need));
    if (n <= 0 || src_rows < 0 || src_cols < 0 || src_ld < src_rows || row_off < 0 || col_off < 0 ||
        row_off + src_rows > n || col_off + src_cols > n)
        return fail(TT_ERR_INVALID_ARG, "source region %dx%d at (%d,%d) does not fit a %dx%d frame",
                    src_rows, src_cols, row_off, col_off, n, n);
    if (n_angles < 0 || (n_angles > 0 && !angles_deg))
        return fail(TT_ERR_INVALID_ARG, "bad angle list");
    if (!d_out || (src_rows * src_cols > 0 && !d_src))
        return fail(TT_ERR_INVALID_ARG, "NULL device buffer");
    return run_sinograms(p, d_src, src_rows, src_cols, src_ld, n, row_off, col_off, nullptr,
                         angles_deg, n_angles, tfuncs, n_t, need, d_out, d_medians,
                         pick_stream(p, stream));
}

tt_status tt_circus_device(tt_plan *plan, const float *d_sino, int rows, int cols, int n_sino,
                           const tt_pfunctional *pfuncs, int n_p, const int32_t *centers,
                           float *d_out, void *stream) {
    tt_plan *p;
    TT_CHECK(resolve_plan(plan, &p));
    unsigned need;
    TT_CHECK(check_pfuncs(pfuncs, n_p, centers == nullptr, &need));
    if (rows <= 0 || cols < 0 || n_sino < 0 || !d_sino || !d_out)
        return fail(TT_ERR_INVALID_ARG, "bad sinogram stack %dx%dx%d", n_sino, rows, cols);
    return run_circus(p, d_sino, rows, cols, n_sino, pfuncs, n_p, centers, need, d_out,
                      pick_stream(p, stream));
}

tt_status tt_circus_orthonormal_device(tt_plan *plan, const float *d_sino, int rows, int cols,
                                       int n_sino, const tt_pfunctional *pfuncs, int n_p,
                                       float *d_out, int32_t *centers, int32_t *sweeps,
                                       void *stream) {
    tt_plan *p;
    TT_CHECK(resolve_plan(plan, &p));
    unsigned need;
    TT_CHECK(check_pfuncs(pfuncs, n_p, false, &need));
    for (int i = 0; i < n_p; i++)
        if (pfuncs[i].kind != TT_P_HERMITE)
            return fail(TT_ERR_INVALID_ARG, "the orthonormal circus takes Hermite P-functionals "
                                            "only");
    if (rows <= 0 || cols < 0 || n_sino < 0 || !d_sino || (n_p > 0 && !d_out))
        return fail(TT_ERR_INVALID_ARG, "bad sinogram stack %dx%dx%d", n_sino, rows, cols);
    if (n_sino == 0 || cols == 0)
        return TT_OK;
    cudaStream_t st = pick_stream(p, stream);
    std::vector<NosDesc> desc;
    std::vector<int> c;
    TT_CHECK(run_nos(p, d_sino, rows, cols, n_sino, st, desc, c, sweeps));
    for (int s = 0; s < n_sino; s++) {
        const int32_t c32 = c[s];
        TT_CHECK(run_circus(p, (const float *)p->nos.p + desc[s].out_off, desc[s].m, cols, 1,
                            pfuncs, n_p, &c32, need, d_out + (size_t)s * n_p * cols, st));
        if (centers)
            centers[s] = c32;
    }
    return TT_OK;
}

tt_status tt_nos(tt_plan *plan, const float *sinogram, int rows, int cols, float *out,
                 int32_t *out_rows, int32_t *new_center) {
    tt_plan *p;
    TT_CHECK(resolve_plan(plan, &p));
    if (rows <= 0 || cols <= 0 || !sinogram || !out || !out_rows || !new_center)
        return fail(TT_ERR_INVALID_ARG, "bad sinogram %dx%d or NULL output", rows, cols);
    cudaStream_t st = p->stream;
    TT_CHECK(p->ensure(p->sino, sizeof(float) * (size_t)rows * cols));
    TT_CUDA(cudaMemcpyAsync(p->sino.p, sinogram, sizeof(float) * (size_t)rows * cols,
                            cudaMemcpyHostToDevice, st));
    std::vector<NosDesc> desc;
    std::vector<int> c;
    TT_CHECK(run_nos(p, (const float *)p->sino.p, rows, cols, 1, st, desc, c));
    TT_CUDA(cudaMemcpyAsync(out, p->nos.p, sizeof(float) * (size_t)desc[0].m * cols,
                            cudaMemcpyDeviceToHost, st));
    TT_CUDA(cudaStreamSynchronize(st));
    *out_rows = desc[0].m;
    *new_center = c[0];
    return TT_OK;
}

tt_status tt_zscore_device(tt_plan *plan, const float *d_in, int n_vec, int len, float *d_out,
                           void *stream) {
    tt_plan *p;
    TT_CHECK(resolve_plan(plan, &p));
    if (n_vec < 0 || len < 0 || (n_vec * len > 0 && (!d_in || !d_out)))
        return fail(TT_ERR_INVALID_ARG, "bad z-score arguments");
    TT_CUDA(tt::launch_zscore(d_in, n_vec, len, d_out, pick_stream(p, stream)));
    return TT_OK;
}

tt_status tt_sinograms(tt_plan *plan, const float *padded, int rows, int cols,
                       unsigned angle_stepsize, const int32_t *tfuncs, int n_t, float *out) {
    tt_plan *p;
    TT_CHECK(resolve_plan(plan, &p));
    if (rows != cols)
        return fail(TT_ERR_INVALID_ARG, "getSinograms needs a square (padded) image, got %dx%d",
                    rows, cols);
    if (rows <= 0 || !padded || !out)
        return fail(TT_ERR_INVALID_ARG, "empty image or NULL buffer");
    if (angle_stepsize == 0)
        return fail(TT_ERR_INVALID_ARG, "angle step must be >= 1");
    unsigned need;
    TT_CHECK(check_tfuncs(tfuncs, n_t, &need));
    const int n = rows;
    std::vector<float> ang = step_angles(angle_stepsize);
    const size_t out_elems = (size_t)n_t * n * ang.size();
    TT_CHECK(p->ensure(p->in, sizeof(float) * (size_t)n * n));
    TT_CHECK(p->ensure(p->sino, sizeof(float) * std::max<size_t>(out_elems, 1)));
    TT_CHECK(p->ensure(p->region, 4 * sizeof(int)));
    cudaStream_t st = p->stream;
    TT_CUDA(cudaMemcpyAsync(p->in.p, padded, sizeof(float) * (size_t)n * n, cudaMemcpyHostToDevice, st));
    // sample only where the padded frame holds non-zero pixels
    TT_CUDA(tt::launch_region_bbox((const float *)p->in.p, n, (int *)p->region.p, st));
    TT_CHECK(run_sinograms(p, (const float *)p->in.p, n, n, n, n, 0, 0, (const int *)p->region.p,
                           ang.data(), (int)ang.size(), tfuncs, n_t, need, (float *)p->sino.p,
                           nullptr, st));
    TT_CUDA(cudaMemcpyAsync(out, p->sino.p, sizeof(float) * out_elems, cudaMemcpyDeviceToHost, st));
    TT_CUDA(cudaStreamSynchronize(st));
    return TT_OK;
}

tt_status tt_circus(tt_plan *plan, const float *sinogram, int rows, int cols,
                    const tt_pfunctional *pfuncs, int n_p, float *out) {
    tt_plan *p;
    TT_CHECK(resolve_plan(plan, &p));
    unsigned need;
    TT_CHECK(check_pfuncs(pfuncs, n_p, true, &need));
    if (rows <= 0 || cols < 0 || !sinogram || !out)
        return fail(TT_ERR_INVALID_ARG, "bad sinogram %dx%d", rows, cols);
    cudaStream_t st = p->stream;
    TT_CHECK(p->ensure(p->sino, sizeof(float) * std::max<size_t>((size_t)rows * cols, 1)));
    TT_CHECK(p->ensure(p->circ, sizeof(float) * std::max<size_t>((size_t)n_p * cols, 1)));
    TT_CUDA(cudaMemcpyAsync(p->sino.p, sinogram, sizeof(float) * (size_t)rows * cols,
                            cudaMemcpyHostToDevice, st));
    TT_CHECK(run_circus(p, (const float *)p->sino.p, rows, cols, 1, pfuncs, n_p, nullptr, need,
                        (float *)p->circ.p, st));
    TT_CUDA(cudaMemcpyAsync(out, p->circ.p, sizeof(float) * (size_t)n_p * cols, cudaMemcpyDeviceToHost, st));
    TT_CUDA(cudaStreamSynchronize(st));
    return TT_OK;
}

tt_status tt_rotate(tt_plan *plan, const float *image, int rows, int cols, float angle_deg,
                    float *out) {
    tt_plan *p;
    TT_CHECK(resolve_plan(plan, &p));
    if (rows <= 0 || cols <= 0 || !image || !out)
        return fail(TT_ERR_INVALID_ARG, "bad image %dx%d", rows, cols);
    const size_t elems = (size_t)rows * cols;
    cudaStream_t st = p->stream;
    TT_CHECK(p->ensure(p->in, sizeof(float) * elems));
    TT_CHECK(p->ensure(p->sino, sizeof(float) * elems));
    TT_CUDA(cudaMemcpyAsync(p->in.p, image, sizeof(float) * elems, cudaMemcpyHostToDevice, st));
    const float ang = deg2rad(angle_deg);
    cudaTextureObject_t tex;
    TT_CHECK(p->load_source((const float *)p->in.p, rows, cols, rows, st, &tex));
    TT_CUDA(tt::launch_rotate(tex, rows, cols, std::cos(-ang), std::sin(-ang), (float *)p->sino.p,
                              st));
    TT_CUDA(cudaMemcpyAsync(out, p->sino.p, sizeof(float) * elems, cudaMemcpyDeviceToHost, st));
    TT_CUDA(cudaStreamSynchronize(st));
    return TT_OK;
}

tt_status tt_resize(tt_plan *plan, const float *image, int in_rows, int in_cols, int rows,
                    int cols, float *out) {
    tt_plan *p;
    TT_CHECK(resolve_plan(plan, &p));
    if (in_rows <= 0 || in_cols <= 0 || rows <= 0 || cols <= 0 || !image || !out)
        return fail(TT_ERR_INVALID_ARG, "bad resize %dx%d -> %dx%d", in_rows, in_cols, rows,
                    cols);
    const size_t in_elems = (size_t)in_rows * in_cols, elems = (size_t)rows * cols;
    cudaStream_t st = p->stream;
    TT_CHECK(p->ensure(p->in, sizeof(float) * in_elems));
    TT_CHECK(p->ensure(p->stretch, sizeof(float) * elems));
    TT_CUDA(cudaMemcpyAsync(p->in.p, image, sizeof(float) * in_elems, cudaMemcpyHostToDevice, st));
    TT_CUDA(tt::launch_resize((const float *)p->in.p, in_rows, in_cols, rows, cols,
                              (float *)p->stretch.p, st));
    TT_CUDA(cudaMemcpyAsync(out, p->stretch.p, sizeof(float) * elems, cudaMemcpyDeviceToHost, st));
    TT_CUDA(cudaStreamSynchronize(st));
    return TT_OK;
}

tt_status tt_zscore(tt_plan *plan, const float *in, int n_vec, int len, float *out) {
    tt_plan *p;
    TT_CHECK(resolve_plan(plan, &p));
    if (n_vec < 0 || len < 0 || (n_vec * len > 0 && (!in || !out)))
        return fail(TT_ERR_INVALID_ARG, "bad z-score arguments");
    const size_t elems = (size_t)n_vec * len;
    if (elems == 0)
        return TT_OK;
    cudaStream_t st = p->stream;
    TT_CHECK(p->ensure(p->circ, sizeof(float) * elems));
    TT_CHECK(p->ensure(p->sig, sizeof(float) * elems));
    TT_CUDA(cudaMemcpyAsync(p->circ.p, in, sizeof(float) * elems, cudaMemcpyHostToDevice, st));
    TT_CUDA(tt::launch_zscore((const float *)p->circ.p, n_vec, len, (float *)p->sig.p, st));
    TT_CUDA(cudaMemcpyAsync(out, p->sig.p, sizeof(float) * elems, cudaMemcpyDeviceToHost, st));
    TT_CUDA(cudaStreamSynchronize(st));
    return TT_OK;
}

tt_status tt_transform(tt_plan *plan, const float *image, int rows, int cols,
                       unsigned angle_stepsize, const int32_t *tfuncs, int n_t,
                       const tt_pfunctional *pfuncs, int n_p, float *circus, float *signatures) {
    tt_plan *p;
    TT_CHECK(resolve_plan(plan, &p));
    if (rows <= 0 || cols <= 0 || !image)
        return fail(TT_ERR_INVALID_ARG, "empty image");
    if (angle_stepsize == 0)
        return fail(TT_ERR_INVALID_ARG, "angle step must be >= 1");
    unsigned tneed, pneed;
    TT_CHECK(check_tfuncs(tfuncs, n_t, &tneed));
    TT_CHECK(check_pfuncs(pfuncs, n_p, false, &pneed));
    int n_herm = 0;
    for (int i = 0; i < n_p; i++)
        n_herm += pfuncs[i].kind == TT_P_HERMITE;
    if (n_herm != 0 && n_herm != n_p)
        return fail(TT_ERR_INVALID_ARG, "Cannot mix regular and orthonormal P-functionals");
    const bool ortho = n_herm > 0;

    // Transformer::Transformer: optional stretch (on the device), then
    // padding (implicit in the sampling)
    int ir = rows, ic = cols;
    if (ortho)
        ir = ic = ortho_side(angle_stepsize);
    int n, ro, co;
    pad_geometry(ir, ic, &n, &ro, &co);
    std::vector<float> ang = step_angles(angle_stepsize);
    const int A = (int)ang.size();
    const size_t sino_elems = (size_t)n_t * n * A, circ_elems = (size_t)n_t * n_p * A;
    cudaStream_t st = p->stream;
    TT_CHECK(p->ensure(p->in, sizeof(float) * (size_t)rows * cols));
    TT_CHECK(p->ensure(p->sino, sizeof(float) * std::max<size_t>(sino_elems, 1)));
    TT_CHECK(p->ensure(p->circ, sizeof(float) * std::max<size_t>(circ_elems, 1)));
    TT_CHECK(p->ensure(p->sig, sizeof(float) * std::max<size_t>(circ_elems, 1)));
    TT_CUDA(cudaMemcpyAsync(p->in.p, image, sizeof(float) * (size_t)rows * cols,
                            cudaMemcpyHostToDevice, st));
    const float *src = (const float *)p->in.p;
    if (ortho) {
        TT_CHECK(p->ensure(p->stretch, sizeof(float) * (size_t)ir * ic));
        TT_CUDA(tt::launch_resize(src, rows, cols, ir, ic, (float *)p->stretch.p, st));
        src = (const float *)p->stretch.p;
    }
    TT_CHECK(run_sinograms(p, src, ir, ic, ir, n, ro, co, nullptr, ang.data(), A,
                           tfuncs, n_t, tneed, (float *)p->sino.p, nullptr, st));
    if (n_p == 0 || A == 0) {
        TT_CUDA(cudaStreamSynchronize(st));
        return TT_OK;
    }
    if (!ortho) {
        TT_CHECK(run_circus(p, (const float *)p->sino.p, n, A, n_t, pfuncs, n_p, nullptr, pneed,
                            (float *)p->circ.p, st));
    } else {
        // nearest orthonormal sinogram per T (device), then the Hermite circus
        std::vector<NosDesc> desc;
        std::vector<int> centers;
        TT_CHECK(run_nos(p, (const float *)p->sino.p, n, A, n_t, st, desc, centers));
        for (int t = 0; t < n_t; t++) {
            const int32_t c32 = centers[t];
            TT_CHECK(run_circus(p, (const float *)p->nos.p + desc[t].out_off, desc[t].m, A, 1,
                                pfuncs, n_p, &c32, pneed, (float *)p->circ.p + (size_t)t * n_p * A,
                                st));
        }
    }
    if (signatures)
        TT_CUDA(tt::launch_zscore((const float *)p->circ.p, n_t * n_p, A, (float *)p->sig.p, st));
    if (circus)
        TT_CUDA(cudaMemcpyAsync(circus, p->circ.p, sizeof(float) * circ_elems, cudaMemcpyDeviceToHost, st));
    if (signatures)
        TT_CUDA(cudaMemcpyAsync(signatures, p->sig.p, sizeof(float) * circ_elems, cudaMemcpyDeviceToHost, st));
    TT_CUDA(cudaStreamSynchronize(st));
    return TT_OK;
}

} // extern "C"
