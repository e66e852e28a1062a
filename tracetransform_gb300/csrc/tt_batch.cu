// tt_batch.cu -- batched engine: many images of uneven sizes and angle
// counts transformed by one persistent sinogram launch, one batched
// P-functional launch and one batched z-score launch, replayed as a CUDA
// graph.
//
// Per batch shape (image sizes, angle steps, functionals) the engine builds
// once: a gather-capable CUDA array and texture per image, the rotation and
// T3-T5 tables of every distinct angle step and padded size, the P3 tables of
// every distinct size, the work-item and column descriptors, and scratch for
// the sinograms.  An autotuner times the persistent kernel's tile shapes
// (lines per CTA, resident CTAs per SM) on the batch itself and remembers the
// winner in a JSON file.  The graph holds the image copies into the texture
// arrays, the three kernels and the work-counter reset; each call replays it.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include <sys/stat.h>

#include "tracetransform.h"
#include "tt_internal.h"

namespace tt {
namespace {

int berr(int status, const char *msg) { return record_error(status, msg); }

int cuda_err(cudaError_t e, const char *what) {
    char buf[320];
    snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
    return record_error(e == cudaErrorMemoryAllocation ? TT_ERR_OOM : TT_ERR_CUDA, buf);
}

#define B_CUDA(call)                                                           \
    do {                                                                       \
        cudaError_t e_ = (call);                                               \
        if (e_ != cudaSuccess)                                                 \
            return cuda_err(e_, #call);                                        \
    } while (0)

#define B_CHECK(expr)                                                          \
    do {                                                                       \
        int s_ = (expr);                                                       \
        if (s_ != TT_OK)                                                       \
            return s_;                                                         \
    } while (0)

template <typename T> struct DevArray {
    T *p = nullptr;
    size_t n = 0;
    ~DevArray() { cudaFree(p); }
    int resize(size_t count) {
        if (count <= n && p)
            return TT_OK;
        cudaFree(p);
        p = nullptr;
        n = 0;
        B_CUDA(dev_malloc(reinterpret_cast<void **>(&p), sizeof(T) * std::max<size_t>(count, 1)));
        n = count;
        return TT_OK;
    }
    int upload(const std::vector<T> &h, cudaStream_t st) {
        B_CHECK(resize(h.size()));
        if (!h.empty()) {
            B_CUDA(cudaMemcpyAsync(p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, st));
            B_CUDA(cudaStreamSynchronize(st));
        }
        return TT_OK;
    }
};

struct ImageTexture {
    cudaArray_t arr = nullptr;
    cudaTextureObject_t tex = 0;
    void release() {
        if (tex)
            cudaDestroyTextureObject(tex);
        if (arr)
            cudaFreeArray(arr);
        tex = 0;
        arr = nullptr;
    }
};

// The shape a captured graph was built for.
struct Shape {
    std::vector<int> rows, cols, steps;
    std::vector<long long> offsets;
    std::vector<int> tf, pk;
    const float *src = nullptr;
    bool operator==(const Shape &o) const {
        return rows == o.rows && cols == o.cols && steps == o.steps && offsets == o.offsets &&
               tf == o.tf && pk == o.pk && src == o.src;
    }
};

// Tile shape of the persistent sinogram kernel: lpw = 0 -- the CTA kernel
// with `lines` lines per CTA (one warp per line, the CTA sampling them
// together); lpw = 1, 2, 4 -- the warp-autonomous kernel, lpw lines per warp
// (T0-T5 only).  ctas_per_sm sizes the persistent grid.
struct Tune {
    int lines = 8, ctas_per_sm = 0, lpw = 0;
};

std::string tune_cache_path() {
    if (const char *p = getenv("TT_AUTOTUNE_CACHE"))
        return p;
    const char *home = getenv("HOME");
    return std::string(home ? home : "/tmp") + "/.cache/tracetransform_gb300_autotune.json";
}

// The cache is a flat JSON object {"key": [lines, ctas_per_sm, lpw], ...}.
std::map<std::string, Tune> load_tune_cache() {
    std::map<std::string, Tune> m;
    std::ifstream f(tune_cache_path());
    if (!f)
        return m;
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string s = ss.str();
    size_t pos = 0;
    while ((pos = s.find('"', pos)) != std::string::npos) {
        const size_t end = s.find('"', pos + 1);
        if (end == std::string::npos)
            break;
        const std::string key = s.substr(pos + 1, end - pos - 1);
        Tune t;
        if (sscanf(s.c_str() + end + 1, " : [ %d , %d , %d ]", &t.lines, &t.ctas_per_sm,
                   &t.lpw) == 3)
            m[key] = t;
        pos = end + 1;
    }
    return m;
}

void save_tune_cache(const std::map<std::string, Tune> &m) {
    const std::string path = tune_cache_path();
    const size_t slash = path.rfind('/');
    if (slash != std::string::npos)
        mkdir(path.substr(0, slash).c_str(), 0755); // the cache's folder, if missing
    std::ofstream f(path);
    if (!f)
        return;
    f << "{\n";
    size_t i = 0;
    for (const auto &kv : m)
        f << "  \"" << kv.first << "\": [" << kv.second.lines << ", " << kv.second.ctas_per_sm
          << ", " << kv.second.lpw << "]" << (++i < m.size() ? ",\n" : "\n");
    f << "}\n";
}

} // namespace

class BatchEngine {
  public:
    explicit BatchEngine(int device) : device_(device) {}
    ~BatchEngine() {
        release();
        if (ev_in_)
            cudaEventDestroy(ev_in_);
        if (ev_out_)
            cudaEventDestroy(ev_out_);
        for (cudaEvent_t e : stage_ev_)
            if (e)
                cudaEventDestroy(e);
        if (own_)
            cudaStreamDestroy(own_);
    }

    int run(const float *d_images, const long long *offsets, const int *rows, const int *cols,
            const int *steps, int n_img, const int32_t *tfuncs, int n_t,
            const tt_pfunctional *pf, int n_p, float *d_circus, float *d_sig, cudaStream_t st);
    int sinograms(float *d_out, size_t capacity, size_t *count, cudaStream_t st);
    int stage_ms(float ms[3]);
    void tile(int out[3]) const {
        out[0] = tune_.lines;
        out[1] = tune_.ctas_per_sm;
        out[2] = tune_.lpw;
    }
    void pin(const int t[3]) {
        pinned_ = t[1] > 0;
        pin_.lines = t[0];
        pin_.ctas_per_sm = t[1];
        pin_.lpw = t[2];
        built_ = false; // the next call rebuilds and captures with the pinned shape
    }

  private:
    int build(cudaStream_t st);
    int make_desc(int lines, std::vector<BatchImage> &desc, int *total_items) const;
    int set_tile(const Tune &t, cudaStream_t st);
    cudaError_t launch_sino(const Tune &t, int grid, cudaStream_t st);
    int autotune(cudaStream_t st);
    int capture(cudaStream_t st);
    void release();

    int device_;
    Shape shape_;
    bool built_ = false;
    std::vector<ImageTexture> tex_;
    std::vector<int> n_, ro_, co_, na_, order_;
    std::vector<long long> sino_off_, out_off_;
    DevArray<BatchImage> img_;
    DevArray<CircusStack> stacks_;
    DevArray<float2> trig_, tab_, p3tw_;
    DevArray<float> p3ck_, p3tc_, sino_, circ_, sig_, part_;
    DevArray<int2> fb_;
    DevArray<unsigned> counter_;
    DevArray<long long> voff_;
    DevArray<int> vlen_;
    BatchSinoArgs sargs_{};
    CircusStackArgs cargs_{};
    size_t circ_smem_ = 0;
    int n_vec_ = 0, n_max_ = 0;
    size_t out_floats_ = 0, sino_floats_ = 0;
    std::vector<int> trig_off_, tab_off_;
    Tune tune_, pin_;
    bool pinned_ = false;
    size_t sino_smem_ = 0;
    cudaGraphExec_t exec_ = nullptr;
    // the graph is captured on and replayed from the engine's own stream
    // (the legacy default stream cannot be captured), ordered after and
    // before the caller's stream by events
    cudaStream_t own_ = nullptr;
    cudaEvent_t ev_in_ = nullptr, ev_out_ = nullptr;
    // recorded inside the graph around its three kernels (per-stage timing)
    cudaEvent_t stage_ev_[4] = {nullptr, nullptr, nullptr, nullptr};
    bool replayed_ = false;
};

void BatchEngine::release() {
    if (exec_)
        cudaGraphExecDestroy(exec_);
    exec_ = nullptr;
    for (auto &t : tex_)
        t.release();
    tex_.clear();
    built_ = false;
}

// Work-item descriptors for a tile of `lines` lines per CTA, largest image first.
int BatchEngine::make_desc(int lines, std::vector<BatchImage> &desc, int *total_items) const {
    const int n_img = (int)shape_.rows.size();
    desc.resize(n_img);
    long long items = 0;
    for (int k = 0; k < n_img; k++) {
        const int i = order_[k];
        BatchImage &d = desc[k];
        d.tex = tex_[i].tex;
        d.rows = shape_.rows[i];
        d.cols = shape_.cols[i];
        d.n = n_[i];
        d.row_off = ro_[i];
        d.col_off = co_[i];
        d.n_angles = na_[i];
        d.blocks = (n_[i] + lines - 1) / lines;
        d.items_begin = (int)items;
        d.trig_off = trig_off_[i];
        d.tab_off = tab_off_[i];
        d.sino_off = sino_off_[i];
        items += (long long)d.blocks * d.n_angles;
    }
    if (items > 0x7fffffffLL)
        return berr(TT_ERR_UNSUPPORTED, "batch has more than 2^31 work items");
    *total_items = (int)items;
    return TT_OK;
}

int BatchEngine::set_tile(const Tune &t, cudaStream_t st) {
    std::vector<BatchImage> desc;
    int total = 0;
    B_CHECK(make_desc(t.lpw ? t.lpw : t.lines, desc, &total));
    B_CHECK(img_.upload(desc, st));
    if (t.lpw) {
        sino_smem_ = sino_warp_smem_bytes(n_max_, t.lpw);
        if (sino_batch_warp_occupancy(t.lpw, sargs_.all_interior, sino_smem_) <= 0)
            return berr(TT_ERR_UNSUPPORTED, "warp tile does not fit the batch's largest image");
        sargs_.stride = sino_warp_stride(n_max_, t.lpw);
    } else {
        sino_smem_ = sino_smem_bytes(n_max_, t.lines, sargs_.need);
        B_CUDA(prepare_sino_batch(t.lines, sargs_.need & ((1u << 6) | (1u << 7)),
                                  sargs_.all_interior, sino_smem_));
        sargs_.stride = sino_stride(n_max_, t.lines);
    }
    sargs_.img = img_.p;
    sargs_.total_items = total;
    return TT_OK;
}

cudaError_t BatchEngine::launch_sino(const Tune &t, int grid, cudaStream_t st) {
    return t.lpw ? launch_sino_batch_warp(sargs_, t.lpw, grid, sino_smem_, st)
                 : launch_sino_batch(sargs_, t.lines, grid, sino_smem_, st);
}

int BatchEngine::build(cudaStream_t st) {
    const int n_img = (int)shape_.rows.size();
    const int n_t = (int)shape_.tf.size(), n_p = (int)shape_.pk.size();
    n_.resize(n_img);
    ro_.resize(n_img);
    co_.resize(n_img);
    na_.resize(n_img);
    trig_off_.resize(n_img);
    tab_off_.resize(n_img);
    sino_off_.resize(n_img);
    out_off_.resize(n_img);
    n_max_ = 0;
    long long sino_total = 0, out_total = 0;
    for (int i = 0; i < n_img; i++) {
        pad_geometry(shape_.rows[i], shape_.cols[i], &n_[i], &ro_[i], &co_[i]);
        na_[i] = 360 / shape_.steps[i];
        n_max_ = std::max(n_max_, n_[i]);
        sino_off_[i] = sino_total;
        out_off_[i] = out_total;
        sino_total += (long long)n_t * na_[i] * n_[i];
        out_total += (long long)n_t * n_p * na_[i];
    }
    out_floats_ = (size_t)out_total;
    sino_floats_ = (size_t)sino_total;
    // textures (texel (u, v) = image row u, column v; border reads 0)
    tex_.resize(n_img);
    for (int i = 0; i < n_img; i++) {
        if (shape_.rows[i] > 32768 || shape_.cols[i] > 32768)
            return berr(TT_ERR_UNSUPPORTED, "batch image exceeds the 32768 texture-gather limit");
        cudaChannelFormatDesc desc = cudaCreateChannelDesc<float>();
        B_CUDA(dev_malloc_array(&tex_[i].arr, &desc, shape_.rows[i], shape_.cols[i],
                               cudaArrayTextureGather));
        cudaResourceDesc res{};
        res.resType = cudaResourceTypeArray;
        res.res.array.array = tex_[i].arr;
        cudaTextureDesc td{};
        td.addressMode[0] = cudaAddressModeBorder;
        td.addressMode[1] = cudaAddressModeBorder;
        td.filterMode = cudaFilterModePoint;
        td.readMode = cudaReadModeElementType;
        B_CUDA(cudaCreateTextureObject(&tex_[i].tex, &res, &td, nullptr));
    }
    // rotation tables per distinct step, T3-T5 and P3 tables per distinct size
    std::vector<float2> trig, tab, p3tw;
    std::vector<float> p3ck;
    std::map<int, int> step_at, tab_at;
    std::map<int, std::pair<long long, long long>> p3_at;
    const bool p3 = std::find(shape_.pk.begin(), shape_.pk.end(), (int)TT_P3) != shape_.pk.end();
    unsigned pneed = 0;
    for (int k : shape_.pk)
        pneed |= 1u << k;
    std::vector<CircusStack> stacks(n_img);
    int col_begin = 0, tile_begin = 0, sort_len = 1;
    long long part_total = 0;
    for (int i = 0; i < n_img; i++) {
        const int step = shape_.steps[i], n = n_[i];
        if (!step_at.count(step)) {
            step_at[step] = (int)trig.size();
            for (int a = 0; a < 360 / step; a++)
                trig.push_back(rotation((float)(a * step)));
        }
        trig_off_[i] = step_at[step];
        if (!tab_at.count(n)) {
            tab_at[n] = (int)tab.size();
            tab.resize(tab.size() + 3 * (size_t)n);
            t345_tables(n, tab.data() + tab_at[n]);
        }
        tab_off_[i] = tab_at[n];
        if (p3 && !p3_at.count(n)) {
            p3_at[n] = std::make_pair((long long)p3tw.size(), (long long)p3ck.size());
            p3tw.resize(p3tw.size() + n);
            p3ck.resize(p3ck.size() + n / 2 + 1);
        }
        while (sort_len < n)
            sort_len <<= 1;
        CircusStack &c = stacks[i];
        c.n = n;
        c.angles = na_[i];
        c.cols = n_t * na_[i];
        c.mtiles = p3 ? p3_freq_tiles(n) : 0;
        c.col_begin = col_begin;
        c.tile_begin = tile_begin;
        col_begin += c.cols;
        tile_begin += c.mtiles * ((c.cols + 127) / 128);
        part_total += (long long)c.mtiles * c.cols;
    }
    if (p3tw.empty()) {
        p3tw.push_back(make_float2(0.f, 0.f));
        p3ck.push_back(0.f);
    }
    B_CHECK(trig_.upload(trig, st));
    B_CHECK(tab_.upload(tab, st));
    B_CHECK(p3tw_.upload(p3tw, st));
    B_CHECK(p3ck_.upload(p3ck, st));
    for (const auto &kv : p3_at)
        B_CUDA(launch_p3_dft_tables(kv.first, p3tw_.p + kv.second.first,
                                    p3ck_.p + kv.second.second, st));
    // the tensor-core P3's twiddle blocks, one set per distinct n
    std::map<int, size_t> p3tc_at;
    size_t p3tc_total = 0;
    for (const auto &kv : p3_at) {
        p3tc_at[kv.first] = p3tc_total;
        p3tc_total += p3_tc_table_floats(kv.first);
    }
    B_CHECK(p3tc_.resize(std::max<size_t>(p3tc_total, 1)));
    for (const auto &kv : p3_at)
        B_CUDA(launch_p3_tc_tables(kv.first, p3tw_.p + kv.second.first,
                                   p3tc_.p + p3tc_at[kv.first], st));
    B_CUDA(cudaStreamSynchronize(st));
    B_CHECK(sino_.resize((size_t)std::max<long long>(sino_total, 1)));
    B_CHECK(circ_.resize(std::max<size_t>(out_floats_, 1)));
    B_CHECK(sig_.resize(std::max<size_t>(out_floats_, 1)));
    B_CHECK(counter_.resize(1));
    B_CHECK(part_.resize((size_t)std::max<long long>(part_total, 1)));
    B_CHECK(fb_.resize((size_t)col_begin + 1));
    long long part_at = 0;
    for (int i = 0; i < n_img; i++) {
        CircusStack &c = stacks[i];
        c.sino = sino_.p + sino_off_[i];
        c.out = circ_.p + out_off_[i];
        c.partial = part_.p + part_at;
        part_at += (long long)c.mtiles * c.cols;
        c.tw = p3 ? p3tw_.p + p3_at[n_[i]].first : nullptr;
        c.ck = p3 ? p3ck_.p + p3_at[n_[i]].second : nullptr;
        c.wtc = p3 ? p3tc_.p + p3tc_at[n_[i]] : nullptr;
    }
    B_CHECK(stacks_.upload(stacks, st));
    // z-score vectors: n_t x n_p per image, length = its angle count
    std::vector<long long> voff;
    std::vector<int> vlen;
    for (int i = 0; i < n_img; i++)
        for (int v = 0; v < n_t * n_p; v++) {
            voff.push_back(out_off_[i] + (long long)v * na_[i]);
            vlen.push_back(na_[i]);
        }
    n_vec_ = (int)voff.size();
    if (voff.empty()) {
        voff.push_back(0);
        vlen.push_back(0);
    }
    B_CHECK(voff_.upload(voff, st));
    B_CHECK(vlen_.upload(vlen, st));
    // work order: largest image first, for a short tail
    order_.resize(n_img);
    for (int i = 0; i < n_img; i++)
        order_[i] = i;
    std::stable_sort(order_.begin(), order_.end(), [&](int a, int b) {
        return (double)n_[a] * n_[a] * na_[a] > (double)n_[b] * n_[b] * na_[b];
    });
    // kernel arguments (the work-item descriptors depend on the tile: set_tile)
    unsigned tneed = 0;
    unsigned long long code = 0;
    for (int t = 0; t < n_t; t++) {
        tneed |= 1u << shape_.tf[t];
        code |= (unsigned long long)shape_.tf[t] << (3 * t);
    }
    sargs_ = BatchSinoArgs{};
    sargs_.n_img = n_img;
    sargs_.trig = trig_.p;
    sargs_.tab = tab_.p;
    sargs_.sino = sino_.p;
    sargs_.counter = counter_.p;
    sargs_.tf_code = code;
    sargs_.n_t = n_t;
    sargs_.need = tneed;
    sargs_.all_interior = true;
    for (int i = 0; i < n_img; i++)
        sargs_.all_interior = sargs_.all_interior &&
                              interior_source(n_[i], ro_[i], co_[i], shape_.rows[i],
                                              shape_.cols[i]);
    cargs_ = CircusStackArgs{};
    cargs_.st = stacks_.p;
    cargs_.n_st = n_img;
    cargs_.total_tiles = tile_begin;
    cargs_.total_cols = col_begin;
    cargs_.n_p = n_p;
    for (int p = 0; p < n_p; p++)
        cargs_.kind[p] = shape_.pk[p];
    cargs_.need = pneed;
    cargs_.tc_tables = 1;
    cargs_.stride = circus_warp_stride(n_max_);
    cargs_.fb_count = reinterpret_cast<unsigned *>(fb_.p);
    cargs_.fb_list = fb_.p + 1;
    cargs_.fb_capacity = col_begin;
    cargs_.sort_len_max = sort_len;
    int sms = 0;
    B_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_));
    cargs_.fb_grid = 2 * sms;
    if (p3 && n_max_ > kP3DftMaxRows)
        return berr(TT_ERR_UNSUPPORTED, "batched P3 takes padded sides up to 2048 (images up to "
                                        "about 1440 px); transform larger images one by one");
    circ_smem_ = circus_warp_smem_bytes(n_max_);
    if (circ_smem_ > 227 * 1024 || sizeof(float) * (size_t)sort_len > 227 * 1024)
        return berr(TT_ERR_UNSUPPORTED, "batch image too large for the P-stage buffers");
    built_ = true;
    return TT_OK;
}

// Tile shapes: lines per CTA (columns per warp group) in {8, 4} and resident
// CTAs per SM for the persistent grid; each candidate is timed on the batch.
int BatchEngine::autotune(cudaStream_t st) {
    int dev_sms = 0;
    B_CUDA(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, device_));
    cudaDeviceProp prop;
    B_CUDA(cudaGetDeviceProperties(&prop, device_));
    int n_min = n_max_;
    long long angles = 0;
    for (int i = 0; i < (int)n_.size(); i++) {
        n_min = std::min(n_min, n_[i]);
        angles += na_[i];
    }
    if (pinned_) {
        const bool sel = sargs_.need & ((1u << 6) | (1u << 7));
        if (pin_.lpw && (sel || sargs_.n_t > kWarpMaxOutputs))
            return berr(TT_ERR_UNSUPPORTED, "lines-per-warp tiles compute T0-T5, at most 8 "
                                            "sinograms per image");
        tune_ = pin_;
        return set_tile(tune_, st);
    }
    std::ostringstream key;
    key << "v2|" << prop.name << "|n" << n_min << "-" << n_max_ << "|imgs" << n_.size()
        << "|angles" << angles << "|need" << sargs_.need;
    std::map<std::string, Tune> cache = load_tune_cache();
    auto hit = cache.find(key.str());
    if (hit != cache.end()) {
        tune_ = hit->second;
        return set_tile(tune_, st);
    }
    // load the images once so the timed runs see real data
    for (int i = 0; i < (int)n_.size(); i++)
        B_CUDA(cudaMemcpy2DToArrayAsync(tex_[i].arr, 0, 0, shape_.src + shape_.offsets[i],
                                        sizeof(float) * shape_.rows[i],
                                        sizeof(float) * shape_.rows[i], shape_.cols[i],
                                        cudaMemcpyDeviceToDevice, st));
    cudaEvent_t e0, e1;
    B_CUDA(cudaEventCreate(&e0));
    B_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    Tune best_t;
    best_t.ctas_per_sm = 0;
    const bool sel = sargs_.need & ((1u << 6) | (1u << 7));
    // candidates: the CTA kernel with 8 or 4 lines per CTA, and (T0-T5) the
    // warp-autonomous kernel with 1, 2 or 4 lines per warp; each at its
    // occupancy and at half of it
    std::vector<Tune> shapes;
    for (int lines : {8, 4}) {
        Tune t;
        t.lines = lines;
        t.lpw = 0;
        shapes.push_back(t);
    }
    if (!sel && sargs_.n_t <= kWarpMaxOutputs)
        for (int lpw : {1, 2, 4}) {
            Tune t;
            t.lines = lpw * sino_warp_cta_warps();
            t.lpw = lpw;
            shapes.push_back(t);
        }
    for (Tune t : shapes) {
        int occ;
        if (t.lpw) {
            occ = sino_batch_warp_occupancy(t.lpw, sargs_.all_interior,
                                            sino_warp_smem_bytes(n_max_, t.lpw));
        } else {
            const size_t smem = sino_smem_bytes(n_max_, t.lines, sargs_.need);
            occ = sino_batch_occupancy(t.lines, sel, sargs_.all_interior, smem);
        }
        if (occ <= 0)
            continue;
        if (set_tile(t, st) != TT_OK)
            continue;
        for (int per_sm : {occ, std::max(1, occ / 2)}) {
            float ms = 0.f;
            for (int rep = 0; rep < 2; rep++) { // first run warms up
                B_CUDA(cudaMemsetAsync(counter_.p, 0, sizeof(unsigned), st));
                B_CUDA(cudaEventRecord(e0, st));
                B_CUDA(launch_sino(t, per_sm * dev_sms, st));
                B_CUDA(cudaEventRecord(e1, st));
                B_CUDA(cudaEventSynchronize(e1));
                B_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            }
            if (ms < best) {
                best = ms;
                best_t = t;
                best_t.ctas_per_sm = per_sm;
            }
            if (per_sm == 1)
                break;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (best_t.ctas_per_sm == 0)
        return berr(TT_ERR_UNSUPPORTED, "no tile shape fits the batch's largest image");
    tune_ = best_t;
    cache[key.str()] = tune_;
    save_tune_cache(cache);
    return set_tile(tune_, st);
}

int BatchEngine::capture(cudaStream_t st) {
    if (exec_) {
        cudaGraphExecDestroy(exec_);
        exec_ = nullptr;
    }
    int dev_sms = 0;
    B_CUDA(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, device_));
    cudaGraph_t graph = nullptr;
    B_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaMemsetAsync(counter_.p, 0, sizeof(unsigned), st);
    for (int i = 0; e == cudaSuccess && i < (int)n_.size(); i++)
        e = cudaMemcpy2DToArrayAsync(tex_[i].arr, 0, 0, shape_.src + shape_.offsets[i],
                                     sizeof(float) * shape_.rows[i],
                                     sizeof(float) * shape_.rows[i], shape_.cols[i],
                                     cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess)
        e = cudaEventRecordWithFlags(stage_ev_[0], st, cudaEventRecordExternal);
    if (e == cudaSuccess)
        e = launch_sino(tune_, tune_.ctas_per_sm * dev_sms, st);
    if (e == cudaSuccess)
        e = cudaEventRecordWithFlags(stage_ev_[1], st, cudaEventRecordExternal);
    if (e == cudaSuccess)
        e = launch_circus_stacks(cargs_, circ_smem_, st);
    if (e == cudaSuccess)
        e = cudaEventRecordWithFlags(stage_ev_[2], st, cudaEventRecordExternal);
    if (e == cudaSuccess)
        e = launch_zscore_batch(circ_.p, voff_.p, vlen_.p, n_vec_, sig_.p, st);
    if (e == cudaSuccess)
        e = cudaEventRecordWithFlags(stage_ev_[3], st, cudaEventRecordExternal);
    const cudaError_t e_end = cudaStreamEndCapture(st, &graph);
    if (e != cudaSuccess) {
        if (graph)
            cudaGraphDestroy(graph);
        return cuda_err(e, "batch graph capture");
    }
    B_CUDA(e_end);
    e = cudaGraphInstantiate(&exec_, graph, 0);
    cudaGraphDestroy(graph);
    B_CUDA(e);
    return TT_OK;
}

int BatchEngine::run(const float *d_images, const long long *offsets, const int *rows,
                     const int *cols, const int *steps, int n_img, const int32_t *tfuncs,
                     int n_t, const tt_pfunctional *pf, int n_p, float *d_circus, float *d_sig,
                     cudaStream_t st) {
    Shape s;
    s.rows.assign(rows, rows + n_img);
    s.cols.assign(cols, cols + n_img);
    s.steps.assign(steps, steps + n_img);
    s.offsets.assign(offsets, offsets + n_img);
    for (int t = 0; t < n_t; t++)
        s.tf.push_back(tfuncs[t]);
    for (int p = 0; p < n_p; p++)
        s.pk.push_back(pf[p].kind);
    s.src = d_images;
    if (!own_) {
        B_CUDA(cudaStreamCreateWithFlags(&own_, cudaStreamNonBlocking));
        B_CUDA(cudaEventCreateWithFlags(&ev_in_, cudaEventDisableTiming));
        B_CUDA(cudaEventCreateWithFlags(&ev_out_, cudaEventDisableTiming));
        for (cudaEvent_t &ev : stage_ev_)
            B_CUDA(cudaEventCreate(&ev));
    }
    // the engine's stream starts after the caller's pending work (the images)
    B_CUDA(cudaEventRecord(ev_in_, st));
    B_CUDA(cudaStreamWaitEvent(own_, ev_in_, 0));
    if (!built_ || !(s == shape_)) {
        B_CUDA(cudaDeviceSynchronize()); // kernels of the old shape may still read its arrays
        release();
        shape_ = s;
        B_CHECK(build(own_));
        B_CHECK(autotune(own_));
        B_CHECK(capture(own_));
    }
    B_CUDA(cudaGraphLaunch(exec_, own_));
    replayed_ = true;
    if (d_circus)
        B_CUDA(cudaMemcpyAsync(d_circus, circ_.p, sizeof(float) * out_floats_,
                               cudaMemcpyDeviceToDevice, own_));
    if (d_sig)
        B_CUDA(cudaMemcpyAsync(d_sig, sig_.p, sizeof(float) * out_floats_,
                               cudaMemcpyDeviceToDevice, own_));
    // and the caller's stream continues after the results
    B_CUDA(cudaEventRecord(ev_out_, own_));
    B_CUDA(cudaStreamWaitEvent(st, ev_out_, 0));
    return TT_OK;
}

// The last batch's sinograms, image after image in input order (each
// n_t x n_angles x n), ordered after the last replay on the caller's stream.
int BatchEngine::sinograms(float *d_out, size_t capacity, size_t *count, cudaStream_t st) {
    *count = built_ ? sino_floats_ : 0;
    if (!d_out || !built_ || sino_floats_ == 0)
        return TT_OK;
    if (capacity < sino_floats_)
        return berr(TT_ERR_INVALID_ARG, "sinogram buffer smaller than the last batch's sinograms");
    B_CUDA(cudaEventRecord(ev_in_, st));
    B_CUDA(cudaStreamWaitEvent(own_, ev_in_, 0));
    B_CUDA(cudaMemcpyAsync(d_out, sino_.p, sizeof(float) * sino_floats_, cudaMemcpyDeviceToDevice,
                           own_));
    B_CUDA(cudaEventRecord(ev_out_, own_));
    B_CUDA(cudaStreamWaitEvent(st, ev_out_, 0));
    return TT_OK;
}

// Device time of the last replay's sinogram, P-functional and z-score
// kernels (events recorded inside the graph); waits for that replay.
int BatchEngine::stage_ms(float ms[3]) {
    if (!replayed_)
        return berr(TT_ERR_INVALID_ARG, "no batch has run on this plan");
    B_CUDA(cudaEventSynchronize(stage_ev_[3]));
    for (int k = 0; k < 3; k++)
        B_CUDA(cudaEventElapsedTime(&ms[k], stage_ev_[k], stage_ev_[k + 1]));
    return TT_OK;
}

BatchEngine *batch_create(int device) { return new BatchEngine(device); }

void batch_destroy(BatchEngine *b) { delete b; }

int batch_run(BatchEngine *b, const float *d_images, const long long *offsets, const int *rows,
              const int *cols, const int *steps, int n_img, const int32_t *tfuncs, int n_t,
              const tt_pfunctional *pf, int n_p, float *d_circus, float *d_sig,
              cudaStream_t st) {
    return b->run(d_images, offsets, rows, cols, steps, n_img, tfuncs, n_t, pf, n_p, d_circus,
                  d_sig, st);
}

int batch_sinograms(BatchEngine *b, float *d_out, size_t capacity, size_t *count,
                    cudaStream_t st) {
    return b->sinograms(d_out, capacity, count, st);
}

int batch_stage_ms(BatchEngine *b, float ms[3]) { return b->stage_ms(ms); }

void batch_tile(BatchEngine *b, int out[3]) { b->tile(out); }

void batch_pin_tile(BatchEngine *b, const int t[3]) { b->pin(t); }

} // namespace tt
