// rz_api.cu -- host runtime behind the C ABI (include/rasterize_gb300.h).
//
// A context owns a stream and growable device buffers.  Host-memory calls
// stage inputs through pinned memory, launch the band kernel and copy the
// masks back; device-memory batches are launched in place.  A batch plan
// keeps the work list and mask descriptors resident on the device and
// replays the launch from a captured CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <functional>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/rasterize_gb300.h"
#include "rz_host_arc.cpp.inc"
#include "rz_host_scene.cpp.inc"
#include "rz_host_stroke.cpp.inc"
#include "rz_glyph.cuh"
#include "rz_kernels.cuh"
#include "rz_pipeline.cuh"
#include "rz_stroke.cuh"

namespace rz {
cudaError_t init_kernels();
cudaError_t launch_mask_bands(const BatchDev& b, const WorkItem* items, int n_items, int32_t* queue, int grid,
                              cudaStream_t stream);
int mask_bands_occupancy();
int band_floats();
uint64_t band_record_bytes();
cudaError_t launch_band_records(const BatchDev& b, cudaStream_t stream);
cudaError_t launch_band_records(const BatchDev& b, uint32_t seg_lo, uint32_t seg_hi, uint32_t sub_lo, uint32_t sub_hi,
                                cudaStream_t stream);
cudaError_t launch_flatten_counts(const BatchDev& b, uint32_t n_segments, uint32_t n_subpaths, uint32_t* counts,
                                  cudaStream_t stream);
cudaError_t launch_flatten_count(const SceneDev& S, cudaStream_t st);
cudaError_t launch_flatten_emit(const SceneDev& S, cudaStream_t st);
cudaError_t launch_flatten_emit_alloc(const SceneDev& S, uint32_t* n_lines, cudaStream_t st);
cudaError_t launch_bin_scatter(const SceneDev& S, cudaStream_t st);
int composite_smem_bytes(int canvas_w, int band_rows, int max_clip_width, bool paint_mode, int* cov_stride);
cudaError_t launch_composite(const SceneDev& S, int cov_stride, int smem, cudaStream_t st);
uint64_t scan_temp_words(uint64_t n);
int lines_band_floats();
cudaError_t init_lines_kernel();
int mask_lines_occupancy();
cudaError_t launch_mask_lines(const SceneDev& S, const MaskDev* masks, const WorkItem* items, int n_items,
                              int32_t* queue, float* out, int grid, cudaStream_t st);
int diff_smem_bytes(int width, int band_rows, bool backward, int* cov_stride);
cudaError_t launch_diff_segments(const float* ctrl, uint32_t n_paths, uint32_t paths_per_image, int segs, int width,
                                 int height, int rule, uint8_t* kind, double* pts, uint32_t* sub_off, FillDev* fills,
                                 cudaStream_t st);
cudaError_t launch_diff(const DiffDev& D, bool backward, int cov_stride, int smem, cudaStream_t st);
cudaError_t launch_l2_loss(const float* A, const float* T, uint64_t n, double* loss, float* dl, int num_sms,
                           cudaStream_t st);
cudaError_t scan_u32(uint32_t* data, uint64_t n, uint32_t* temp, cudaStream_t stream);
cudaError_t launch_encode_rgba8(const float* in, uint8_t* out, uint64_t n, cudaStream_t st);
cudaError_t launch_encode_mask_rgba8(const void* in, int elem_size, uint8_t* out, uint64_t n, cudaStream_t st);
cudaError_t launch_layer_fill(float* buf, uint64_t n_pixels, const float v[4], cudaStream_t st);
cudaError_t launch_layer_compose(float* dst, const int32_t d[4], const float* src, const int32_t s[4],
                                 const float* mask, const int32_t m[4], float opacity, bool scale_opacity, int x0,
                                 int y0, int x1, int y1, cudaStream_t st);
}  // namespace rz

namespace {


struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        size_t want = std::max<size_t>(bytes, 256);
        want = want + want / 4;
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

struct HostBuf {
    void* p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        size_t want = std::max<size_t>(bytes, 4096);
        want = want + want / 4;
        cudaError_t e = cudaMallocHost(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
    }
};

}  // namespace

struct rz_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    std::string last_error;
    std::mutex mu;
    // device buffers
    DevBuf d_kind, d_pts, d_sub, d_psub, d_tr, d_rule, d_masks, d_items, d_out, d_ctrl, d_counts;
    // line pipeline (large paths, scenes)
    DevBuf p_fills, p_paints, p_slots, p_lines, p_ecount, p_estart, p_ecursor, p_pairs, p_scan, p_canvas;
    // differentiable batch
    DevBuf p_leaf, d_loss;
    // output encode (sRGB8 RGBA) and its input staging
    DevBuf p_rgba8, p_encode_in;
    DevBuf p_recs;  // slot records of the band kernel
    DevBuf p_tasks;  // first flatten task of each slot (adaptive subtree tasks)
    // glyph pipeline of the tuner: records, coefficients, chain offsets, tree codes, path flags, vertices, scan scratch
    DevBuf g_recs, g_coef, g_chain, g_code, g_pflags, g_vtx, g_scan, g_paths;
    // scene-tree layers by nesting depth: colour layers and clip masks
    std::vector<DevBuf> layer_pool, mask_pool;
    // concurrent scene-tree layers: one arena for every layer and mask, a stream pool, events
    DevBuf layer_arena;
    std::vector<cudaStream_t> tree_streams;
    std::vector<cudaEvent_t> tree_events;
    // the device stroker's unit table, counts and offsets, its compact offset
    // pieces, and the merged segment arrays it builds (swapped with d_kind / d_pts)
    DevBuf s_units, s_styles, s_counts, s_off, s_fin, s_tmpk, s_tmpp, s_kind, s_pts, s_order, s_nodes, s_pieces, s_joins;
    // batch tuning (rz_tune_batch / rz_set_tuning): band height cap, resident CTAs per SM (0 = occupancy)
    int tune_rows_cap = 256;
    int tune_ctas = 0;
    int tune_walk = 0;  // slots per lane of the glyph tree walk (0: the default)
    std::string device_name;
    HostBuf h_stage, h_out;
    HostBuf h_plan;   // page-locked mask descriptors and work items of chunked batches
    HostBuf h_order;  // page-locked launch order of the device stroker's OFFSET units
    HostBuf h_outline;  // page-locked host copy of the stroke outlines (their bounding boxes)
    // host-side arc expansion scratch
    std::vector<uint8_t> x_kind;
    std::vector<double> x_pts;
    std::vector<uint32_t> x_sub, x_psub, x_segmap, x_submap;
    bool expanded = false;  // the last stage_host expanded arcs
    // chunked host batches: upload and download streams, and their events
    cudaStream_t s_in = nullptr, s_out = nullptr;
    std::vector<cudaEvent_t> pipe_ev;
};

namespace {

// Host phase timing of an entry point, printed to stderr when RZ_TRACE is set.
struct Trace {
    bool on;
    const char* name;
    std::chrono::steady_clock::time_point t0, t;
    std::string line;
    explicit Trace(const char* n) : on(std::getenv("RZ_TRACE") != nullptr), name(n) {
        if (on) t0 = t = std::chrono::steady_clock::now();
    }
    // with tracing on, waits for the stream first so the phase includes its GPU work
    void gpu_mark(cudaStream_t st, const char* phase) {
        if (!on) return;
        cudaStreamSynchronize(st);
        mark(phase);
    }
    void mark(const char* phase) {
        if (!on) return;
        const auto now = std::chrono::steady_clock::now();
        char buf[96];
        std::snprintf(buf, sizeof(buf), " %s %.3f", phase, std::chrono::duration<double, std::milli>(now - t).count());
        line += buf;
        t = now;
    }
    ~Trace() {
        if (!on) return;
        const double total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        std::fprintf(stderr, "[rz] %s ms:%s | total %.3f\n", name, line.c_str(), total);
    }
};

// A persistent pool of host threads (up to 15 workers besides the caller),
// started on first use, so the host-side parallel loops of every call do not
// pay for thread creation.  run(n, fn) calls fn(i) for every i in [0, n):
// the caller and whichever workers are free take items one at a time, and it
// returns when all are done and no worker still holds the job.  Jobs from
// several threads queue; a worker-run item may start a job of its own (its
// caller works through it, so nothing waits on a busy pool).
struct PoolJob {
    std::function<void(int64_t)> fn;
    int64_t n = 0;
    std::atomic<int64_t> next{0};
    std::atomic<int64_t> done{0};
    int refs = 0;  // workers inside the job (guarded by the pool's mutex)
};

class HostPool {
  public:
    static HostPool& get() {
        static HostPool pool;
        return pool;
    }
    void run(int64_t n, std::function<void(int64_t)> fn) {
        if (n <= 0) return;
        if (workers_.empty() || n == 1) {
            for (int64_t i = 0; i < n; ++i) fn(i);
            return;
        }
        PoolJob job;
        job.fn = std::move(fn);
        job.n = n;
        {
            std::lock_guard<std::mutex> lk(mu_);
            queue_.push_back(&job);
        }
        work_.notify_all();
        for (int64_t i = job.next.fetch_add(1); i < n; i = job.next.fetch_add(1)) {
            job.fn(i);
            job.done.fetch_add(1);
        }
        std::unique_lock<std::mutex> lk(mu_);
        for (auto it = queue_.begin(); it != queue_.end(); ++it)
            if (*it == &job) {
                queue_.erase(it);
                break;
            }
        finished_.wait(lk, [&] { return job.done.load() == n && job.refs == 0; });
    }
    ~HostPool() {
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_ = true;
        }
        work_.notify_all();
        for (auto& t : workers_) t.join();
    }

  private:
    HostPool() {
        const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
        for (int i = 1; i < std::min(hw, 16); ++i) workers_.emplace_back([this] { loop(); });
    }
    void loop() {
        for (;;) {
            PoolJob* j = nullptr;
            {
                std::unique_lock<std::mutex> lk(mu_);
                work_.wait(lk, [&] { return stop_ || !queue_.empty(); });
                if (stop_) return;
                j = queue_.front();
                ++j->refs;
            }
            for (int64_t i = j->next.fetch_add(1); i < j->n; i = j->next.fetch_add(1)) {
                j->fn(i);
                j->done.fetch_add(1);
            }
            {
                std::lock_guard<std::mutex> lk(mu_);
                if (!queue_.empty() && queue_.front() == j) queue_.pop_front();
                --j->refs;
            }
            finished_.notify_all();
        }
    }
    std::mutex mu_;
    std::condition_variable work_, finished_;
    std::deque<PoolJob*> queue_;
    std::vector<std::thread> workers_;
    bool stop_ = false;
};

// Runs fn(lo, hi) over [0, n) split across the host cores (up to 16
// chunks); small ranges run on the calling thread.
template <class F>
void parallel_for(int64_t n, int64_t min_per_thread, F fn) {
    const int64_t hw = std::max<int64_t>(1, (int64_t)std::thread::hardware_concurrency());
    const int64_t t = std::min<int64_t>({hw, 16, n / std::max<int64_t>(min_per_thread, 1)});
    if (t <= 1) {
        fn((int64_t)0, n);
        return;
    }
    const int64_t chunk = (n + t - 1) / t;
    HostPool::get().run(t, [&](int64_t i) {
        const int64_t lo = i * chunk, hi = std::min(n, lo + chunk);
        if (lo < hi) fn(lo, hi);
    });
}

// fn(i) for i in [0, n) on the pool, one item at a time (items of very
// different cost).
template <typename F>
void parallel_each(int64_t n, F fn) {
    HostPool::get().run(n, [&](int64_t i) { fn(i); });
}

// Device address of page-locked host memory the GPU can write directly
// (cudaHostAlloc / cudaHostRegister); null for pageable or device memory.
void* mapped_host(const void* p) {
    if (!p) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

rz_status fail(rz_ctx* c, rz_status st, const std::string& msg) {
    if (c) c->last_error = msg;
    return st;
}

rz_status cuda_fail(rz_ctx* c, cudaError_t e, const char* where) {
    return fail(c, RZ_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define RZ_CUDA(call)                                        \
    do {                                                     \
        cudaError_t e_ = (call);                             \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
    } while (0)

// Device error words use the RZ_ERR_* values.
rz_status status_from_device(rz_ctx* ctx, int32_t code) {
    switch (code) {
        case 0: return RZ_OK;
        case RZ_ERR_NAN: return fail(ctx, RZ_ERR_NAN, "cannot flatten segment with NaN");
        case RZ_ERR_DEPTH: return fail(ctx, RZ_ERR_DEPTH, "a curve needs more than 22 bisection levels");
        case RZ_ERR_ARC: return fail(ctx, RZ_ERR_ARC, "an arc has no finite cubic count");
        default: return fail(ctx, RZ_ERR_CAPACITY, "device error " + std::to_string(code));
    }
}

bool valid_flatness(double f) { return std::isfinite(f) && 16.0 * f * f > 0.0; }

// Band height for a mask: as many rows as fit in the shared band, at most
// `cap` (<= 256: the fixed-point accumulator holds band-relative y below 511).
int band_rows(int clip_width, int height, int cap = 256, int band_floats = 0) {
    const int stride = rz::band_stride(clip_width);
    const int floats = band_floats > 0 ? band_floats : rz::band_floats();
    int rows = std::min(std::min(cap, 256), std::max(1, floats / stride));
    return std::min(rows, std::max(1, height));
}

struct Items {
    std::vector<rz::WorkItem> items;
    std::vector<int> path_first;  // first item of each path (items grouped by path)
};

// Items [0, n) by decreasing band area on a log scale (16 buckets per
// octave), by a stable counting sort: linear time, and path order within a
// bucket.  Persistent CTAs then pick the longest items first (LPT order).
void lpt_sort(rz::WorkItem* items, size_t n, const std::vector<rz::MaskDev>& masks) {
    constexpr int kBuckets = 32 * 16;
    if (n < 2) return;
    thread_local std::vector<uint16_t> key;
    thread_local std::vector<uint32_t> start;
    thread_local std::vector<rz::WorkItem> sorted;
    key.resize(n);
    start.assign(kBuckets + 1, 0);
    sorted.resize(n);
    for (size_t i = 0; i < n; ++i) {
        const rz::WorkItem& w = items[i];
        const uint32_t area = std::max<uint32_t>(1u, (uint32_t)w.rows * (uint32_t)masks[w.path].width);
        const int lz = 31 - __builtin_clz(area);
        const int frac = (int)(((uint64_t)area << (31 - lz)) >> 27) & 15;  // next 4 bits below the leading one
        key[i] = (uint16_t)(kBuckets - 1 - std::min(kBuckets - 1, lz * 16 + frac));
        ++start[key[i] + 1];
    }
    for (int k = 0; k < kBuckets; ++k) start[k + 1] += start[k];
    for (size_t i = 0; i < n; ++i) sorted[start[key[i]]++] = items[i];
    std::copy(sorted.begin(), sorted.begin() + n, items);
}

// Work items sorted by decreasing band area so the persistent CTAs pick the
// longest items first (LPT order); `grouped` keeps path order instead.
void build_items(const std::vector<rz::MaskDev>& masks, bool grouped, Items& out, int rows_cap = 256,
                 int band_floats = 0) {
    out.items.clear();
    out.path_first.assign(masks.size() + 1, 0);
    for (size_t p = 0; p < masks.size(); ++p) {
        out.path_first[p] = (int)out.items.size();
        const rz::MaskDev& m = masks[p];
        if (m.width <= 0 || m.height <= 0) continue;
        const int rows = band_rows(m.clip_width, m.height, rows_cap, band_floats);
        for (int y = 0; y < m.height; y += rows) {
            rz::WorkItem w;
            w.path = (uint32_t)p;
            w.y0 = (uint16_t)y;
            w.rows = (uint16_t)std::min(rows, m.height - y);
            out.items.push_back(w);
        }
    }
    out.path_first[masks.size()] = (int)out.items.size();
    if (!grouped) lpt_sort(out.items.data(), out.items.size(), masks);
}

}  // namespace

extern "C" {

const char* rz_version(void) { return "rasterize_gb300 0.1 (sm_103a)"; }

rz_ctx* rz_create(int device, rz_status* status) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= device || device < 0) {
        cudaGetLastError();
        if (status) *status = RZ_ERR_NO_DEVICE;
        return nullptr;
    }
    rz_ctx* c = new rz_ctx();
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
        rz::init_kernels() != cudaSuccess || rz::init_lines_kernel() != cudaSuccess ||
        rz::init_glyph_kernels() != cudaSuccess) {
        cudaGetLastError();
        delete c;
        if (status) *status = RZ_ERR_NO_DEVICE;
        return nullptr;
    }
    c->stream = c->own_stream;
    if (status) *status = RZ_OK;
    return c;
}

void rz_destroy(rz_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    DevBuf* bufs[] = {&c->d_kind,   &c->d_pts,     &c->d_sub,     &c->d_psub,    &c->d_tr,      &c->d_rule,
                      &c->d_masks,  &c->d_items,   &c->d_out,     &c->d_ctrl,    &c->d_counts,  &c->p_fills,
                      &c->p_paints, &c->p_slots,   &c->p_lines,   &c->p_ecount,  &c->p_estart,  &c->p_ecursor,
                      &c->p_pairs,  &c->p_scan,    &c->p_canvas,  &c->p_leaf,    &c->d_loss,    &c->p_rgba8,
                      &c->p_encode_in, &c->p_recs,  &c->g_recs,    &c->g_coef,    &c->g_chain,   &c->g_code,
                      &c->g_pflags, &c->g_vtx,     &c->g_scan,    &c->g_paths,   &c->p_tasks};
    for (DevBuf* b : bufs) b->release();
    for (DevBuf* b : {&c->s_units, &c->s_styles, &c->s_counts, &c->s_off, &c->s_fin, &c->s_tmpk, &c->s_tmpp, &c->s_order, &c->s_nodes, &c->s_pieces, &c->s_joins,
                      &c->s_kind, &c->s_pts})
        b->release();
    for (cudaStream_t s : c->tree_streams) cudaStreamSynchronize(s), cudaStreamDestroy(s);
    for (cudaEvent_t e : c->tree_events) cudaEventDestroy(e);
    c->layer_arena.release();
    for (DevBuf& b : c->layer_pool) b.release();
    for (DevBuf& b : c->mask_pool) b.release();
    c->h_stage.release();
    c->h_plan.release();
    c->h_order.release();
    c->h_outline.release();
    c->h_out.release();
    if (c->s_in) cudaStreamSynchronize(c->s_in), cudaStreamDestroy(c->s_in);
    if (c->s_out) cudaStreamSynchronize(c->s_out), cudaStreamDestroy(c->s_out);
    for (cudaEvent_t e : c->pipe_ev) cudaEventDestroy(e);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    delete c;
}

const char* rz_last_error(const rz_ctx* c) { return c ? c->last_error.c_str() : "no context"; }

rz_status rz_set_stream(rz_ctx* c, void* stream) {
    if (!c) return RZ_ERR_INVALID;
    c->stream = (cudaStream_t)stream;  // NULL selects the legacy default stream
    return RZ_OK;
}

void* rz_get_stream(const rz_ctx* c) { return c ? (void*)c->stream : nullptr; }

rz_status rz_synchronize(rz_ctx* ctx) {
    if (!ctx) return RZ_ERR_INVALID;
    RZ_CUDA(cudaSetDevice(ctx->device));
    RZ_CUDA(cudaStreamSynchronize(ctx->stream));
    return RZ_OK;
}

}  // extern "C"

namespace {

// Everything a launch needs, resident on the device.
struct Staged {
    rz::BatchDev b;
    std::vector<rz::MaskDev> masks;
    Items items;
    uint32_t n_segments = 0, n_subpaths = 0, n_paths = 0;
};

// Copies a host-memory batch into the context's device buffers (through the
// pinned staging buffer, one async copy per array).
rz_status stage_host(rz_ctx* ctx, const uint8_t* kind, const double* pts, uint32_t n_seg, const uint32_t* sub_off,
                     uint32_t n_sub, const uint32_t* path_sub, uint32_t n_paths, const double* tr,
                     const uint8_t* rule, rz::BatchDev& b, const char** defer_kind = nullptr,
                     const char** defer_pts = nullptr, Trace* trace = nullptr) {
    auto mark = [&](const char* phase) {
        if (trace) trace->mark(phase);
    };
    // arcs are converted to cubics on the host, as PathBuilder::arc_to does
    const bool has_arc = n_seg && std::memchr(kind, RZ_SEG_ARC, n_seg) != nullptr;
    ctx->expanded = has_arc;
    if (has_arc) {
        auto pfor = [](int64_t n, const auto& fn) {
            if (n > 1) parallel_each(n, fn);
            else if (n == 1) fn(0);
        };
        if (!rzhost::expand_batch(kind, pts, sub_off, path_sub, n_paths, ctx->x_kind, ctx->x_pts, ctx->x_sub,
                                  ctx->x_psub, ctx->x_segmap, ctx->x_submap, pfor))
            return fail(ctx, RZ_ERR_ARC, "an arc has no finite cubic count");
        kind = ctx->x_kind.data();
        pts = ctx->x_pts.data();
        n_seg = (uint32_t)ctx->x_kind.size();
        sub_off = ctx->x_sub.data();
        n_sub = (uint32_t)ctx->x_sub.size() - 1;
        path_sub = ctx->x_psub.data();
    }
    const size_t sz_kind = n_seg, sz_pts = (size_t)n_seg * 64, sz_sub = ((size_t)n_sub + 1) * 4,
                 sz_psub = ((size_t)n_paths + 1) * 4, sz_tr = tr ? (size_t)n_paths * 48 : 0,
                 sz_rule = rule ? n_paths : 0;
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    // page-locked sources are copied straight to the device
    auto pinned = [](const void* ptr) {
        if (!ptr) return false;
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        return a.type == cudaMemoryTypeHost;
    };
    mark("arc_scan");
    const bool direct = pinned(kind) && pinned(pts);
    mark("pinned_check");
    const size_t total = (direct ? 0 : al(sz_kind) + al(sz_pts)) + al(sz_sub) + al(sz_psub) + al(sz_tr) + al(sz_rule);
    RZ_CUDA(ctx->h_stage.ensure(total));
    // wait for earlier copies out of the staging buffer before overwriting it
    RZ_CUDA(cudaStreamSynchronize(ctx->stream));
    mark("stage_sync");
    char* h = (char*)ctx->h_stage.p;
    size_t o = 0;
    auto put = [&](const void* src, size_t n) {  // large arrays are copied by all host threads
        char* dst = h + o;
        if (n) {
            const int64_t chunks = (int64_t)((n + (1u << 20) - 1) >> 20);
            parallel_for(chunks, 2, [&](int64_t c0, int64_t c1) {
                const size_t b0 = (size_t)c0 << 20, b1 = std::min(n, (size_t)c1 << 20);
                std::memcpy(dst + b0, (const char*)src + b0, b1 - b0);
            });
        }
        o += al(n);
        return dst;
    };
    const char* hk = direct ? (const char*)kind : put(kind, sz_kind);
    const char* hp = direct ? (const char*)pts : put(pts, sz_pts);
    char* hs = put(sub_off, sz_sub);
    char* hq = put(path_sub, sz_psub);
    char* ht = tr ? put(tr, sz_tr) : nullptr;
    char* hr = rule ? put(rule, sz_rule) : nullptr;
    mark("put");
    RZ_CUDA(ctx->d_kind.ensure(sz_kind + 1));
    RZ_CUDA(ctx->d_pts.ensure(sz_pts + 8));
    RZ_CUDA(ctx->d_sub.ensure(sz_sub));
    RZ_CUDA(ctx->d_psub.ensure(sz_psub));
    if (defer_kind && defer_pts) {  // the caller uploads the segments in chunks
        *defer_kind = hk;
        *defer_pts = hp;
    } else {
        if (sz_kind) RZ_CUDA(cudaMemcpyAsync(ctx->d_kind.p, hk, sz_kind, cudaMemcpyHostToDevice, ctx->stream));
        if (sz_pts) RZ_CUDA(cudaMemcpyAsync(ctx->d_pts.p, hp, sz_pts, cudaMemcpyHostToDevice, ctx->stream));
    }
    RZ_CUDA(cudaMemcpyAsync(ctx->d_sub.p, hs, sz_sub, cudaMemcpyHostToDevice, ctx->stream));
    RZ_CUDA(cudaMemcpyAsync(ctx->d_psub.p, hq, sz_psub, cudaMemcpyHostToDevice, ctx->stream));
    b.n_segments = n_seg;
    b.n_subpaths = n_sub;
    b.kind = (const uint8_t*)ctx->d_kind.p;
    b.pts = (const double*)ctx->d_pts.p;
    b.sub_off = (const uint32_t*)ctx->d_sub.p;
    b.path_sub = (const uint32_t*)ctx->d_psub.p;
    b.tr = nullptr;
    b.rule = nullptr;
    if (tr) {
        RZ_CUDA(ctx->d_tr.ensure(sz_tr));
        RZ_CUDA(cudaMemcpyAsync(ctx->d_tr.p, ht, sz_tr, cudaMemcpyHostToDevice, ctx->stream));
        b.tr = (const double*)ctx->d_tr.p;
    }
    if (rule) {
        RZ_CUDA(ctx->d_rule.ensure(sz_rule));
        RZ_CUDA(cudaMemcpyAsync(ctx->d_rule.p, hr, sz_rule, cudaMemcpyHostToDevice, ctx->stream));
        b.rule = (const uint8_t*)ctx->d_rule.p;
    }
    return RZ_OK;
}

// Uploads mask descriptors + work items, sets error/queue words.
rz_status stage_plan(rz_ctx* ctx, const std::vector<rz::MaskDev>& masks, const Items& items, rz::BatchDev& b) {
    const size_t sz_m = masks.size() * sizeof(rz::MaskDev);
    const size_t sz_i = std::max<size_t>(items.items.size(), 1) * sizeof(rz::WorkItem);
    RZ_CUDA(ctx->d_masks.ensure(sz_m + 16));
    RZ_CUDA(ctx->d_items.ensure(sz_i));
    RZ_CUDA(ctx->d_ctrl.ensure(256));
    if (sz_m) RZ_CUDA(cudaMemcpyAsync(ctx->d_masks.p, masks.data(), sz_m, cudaMemcpyHostToDevice, ctx->stream));
    if (!items.items.empty())
        RZ_CUDA(cudaMemcpyAsync(ctx->d_items.p, items.items.data(), items.items.size() * sizeof(rz::WorkItem),
                                cudaMemcpyHostToDevice, ctx->stream));
    RZ_CUDA(cudaMemsetAsync(ctx->d_ctrl.p, 0, 256, ctx->stream));  // error word, counters, queue heads
    // pageable sources above: the copies complete before the call returns
    int32_t* ctrl = (int32_t*)ctx->d_ctrl.p;
    b.masks = (const rz::MaskDev*)ctx->d_masks.p;
    b.err = ctrl;           // [0] error word
    b.counters = ctrl + 4;  // [4] unused, [5] fallbacks
    return RZ_OK;
}

// Persistent grid: resident CTAs per SM from the occupancy, or the tuned count.
int batch_grid(rz_ctx* ctx, int n_items, bool lines = false) {
    const int occ = std::max(1, lines ? rz::mask_lines_occupancy() : rz::mask_bands_occupancy());
    const int per_sm = ctx->tune_ctas > 0 ? std::min(ctx->tune_ctas, occ) : occ;
    return std::max(1, std::min(n_items, ctx->num_sms * per_sm));
}

// ---------------------------------------------------------------------------
// Batches through the line pipeline (k_mask_lines): one fill per path, every
// segment flattened once, the lines of a path contiguous.
// ---------------------------------------------------------------------------
// The band kernel (tree walks per band, overlapped with coverage in one
// persistent launch) is the default for batches of small paths; the lines
// kernel (flatten once, then bands) is selected with RZ_BATCH_KERNEL=lines.
bool use_lines_kernel() {
    const char* e = std::getenv("RZ_BATCH_KERNEL");
    return e && std::strcmp(e, "lines") == 0;
}

// The glyph pipeline (rz_glyph.cu: records, walk, emit, cover) is the default
// for batch plans; RZ_BATCH_KERNEL=bands selects the band kernel instead.
bool use_glyph_pipeline() {
    const char* e = std::getenv("RZ_BATCH_KERNEL");
    return !(e && (std::strcmp(e, "bands") == 0 || std::strcmp(e, "lines") == 0));
}

// Subpath offsets non-decreasing within the segments, path offsets
// non-decreasing within the subpaths: every slot belongs to one path.
bool offsets_monotone(const uint32_t* sub, uint32_t n_sub, uint32_t n_seg, const uint32_t* psub, uint32_t n_paths) {
    for (uint32_t i = 0; i < n_sub; ++i)
        if (sub[i] > sub[i + 1]) return false;
    if (sub[n_sub] > n_seg) return false;
    for (uint32_t p = 0; p < n_paths; ++p)
        if (psub[p] > psub[p + 1]) return false;
    return psub[n_paths] <= n_sub;
}

int glyph_grid(rz_ctx* ctx, int n_items) {
    const int occ = std::max(1, rz::glyph_cover_occupancy());
    const int per_sm = ctx->tune_ctas > 0 ? std::min(ctx->tune_ctas, occ) : occ;
    return std::max(1, std::min(n_items, ctx->num_sms * per_sm));
}

// Records, walks, chain offsets and vertices of a batch on `st` (the path
// flags cleared first).
cudaError_t glyph_enqueue_flatten(const rz::GlyphDev& g, uint32_t* scan_tmp, uint32_t n_paths, cudaStream_t st) {
    const uint64_t n = (uint64_t)g.b.n_segments + g.b.n_subpaths;
    cudaError_t e = cudaSuccess;
    if (n_paths) e = cudaMemsetAsync(g.path_flags, 0, (size_t)n_paths * 4, st);
    if (e == cudaSuccess) e = rz::launch_glyph_walk(g, st);
    if (e == cudaSuccess) e = rz::scan_u32(g.chain, n + 1, scan_tmp, st);
    if (e == cudaSuccess) e = rz::launch_glyph_emit(g, st);
    return e;
}

// Buffers of the glyph pipeline for batch `b` (device memory), sized by one
// walk + scan on `st`; the vertex buffer gets an eighth of slack for inputs
// rewritten between launches (more is reported as ERR_CAPACITY).
cudaError_t glyph_setup(const rz::BatchDev& b, rz::GlyphDev& g, DevBuf& recs, DevBuf& coefs, DevBuf& chain,
                        DevBuf& code, DevBuf& pflags, DevBuf& vtx, DevBuf& scan, DevBuf& paths, cudaStream_t st) {
    const uint64_t n = (uint64_t)b.n_segments + b.n_subpaths;
    cudaError_t e = recs.ensure(std::max<uint64_t>(n, 1) * sizeof(rz::GlyphRec));
    if (e == cudaSuccess) e = paths.ensure(std::max<uint64_t>(b.n_paths, 1) * rz::glyph_path_bytes());
    if (e == cudaSuccess) e = coefs.ensure(std::max<uint64_t>(n, 1) * sizeof(rz::GlyphCoef));
    if (e == cudaSuccess) e = chain.ensure((n + 1) * 4);
    if (e == cudaSuccess) e = code.ensure(std::max<uint64_t>(n, 1) * 8);
    if (e == cudaSuccess) e = pflags.ensure(std::max<uint64_t>(b.n_paths, 1) * 4);
    if (e == cudaSuccess) e = scan.ensure(rz::scan_temp_words(n + 1) * 4 + 64);
    if (e == cudaSuccess) e = cudaMemsetAsync(chain.p, 0, (n + 1) * 4, st);
    if (e != cudaSuccess) return e;
    g = rz::GlyphDev{};
    g.b = b;
    g.walk_slots = rz::kWalkSlotsDefault;
    g.recs = (rz::GlyphRec*)recs.p;
    g.coefs = (rz::GlyphCoef*)coefs.p;
    g.chain = (uint32_t*)chain.p;
    g.code = (unsigned long long*)code.p;
    g.path_flags = (uint32_t*)pflags.p;
    g.paths = paths.p;
    g.vtx = nullptr;
    g.vtx_cap = 0;  // the sizing pass emits nothing
    if (b.n_paths) e = cudaMemsetAsync(g.path_flags, 0, (size_t)b.n_paths * 4, st);
    if (e == cudaSuccess) e = rz::launch_glyph_walk(g, st);
    if (e == cudaSuccess) e = rz::scan_u32(g.chain, n + 1, (uint32_t*)scan.p, st);
    uint32_t total = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&total, g.chain + n, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    const uint64_t want = std::min<uint64_t>((uint64_t)total + total / 8 + 1024, 0xffffffffull);
    e = vtx.ensure(want * sizeof(int4));
    if (e != cudaSuccess) return e;
    g.vtx = (int4*)vtx.p;
    g.vtx_cap = (uint32_t)std::min<uint64_t>(vtx.cap / sizeof(int4), 0xffffffffull);
    // the sizing pass may have recorded errors (NaN, depth) and re-decisions: the first launch counts them again
    return cudaMemsetAsync(b.err, 0, 32, st);
}



// Fills of a batch from host copies of its offsets, rules and transforms.
uint32_t lines_fills(const std::vector<rz::MaskDev>& masks, const uint32_t* sub_off, const uint32_t* path_sub,
                     const uint8_t* rules, const double* trs, std::vector<rz::FillDev>& fills) {
    const size_t P = masks.size();
    fills.assign(P, rz::FillDev{});
    uint32_t slot = 0;
    for (size_t p = 0; p < P; ++p) {
        rz::FillDev& f = fills[p];
        f.sub0 = path_sub[p];
        f.sub1 = path_sub[p + 1];
        f.seg0 = sub_off[f.sub0];
        f.seg1 = sub_off[f.sub1];
        f.slot0 = slot;
        slot += (f.seg1 - f.seg0) + (f.sub1 - f.sub0);
        f.width = masks[p].width;
        f.height = masks[p].height;
        f.clip_width = masks[p].clip_width;
        f.rule = rules ? rules[p] : 0;
        f.paint = -1;
        const double id[6] = {1, 0, 0, 0, 1, 0};
        std::memcpy(f.tr, trs ? trs + 6 * p : id, sizeof(f.tr));
    }
    return slot;
}

rz::SceneDev lines_scene(const rz::BatchDev& b, const rz::FillDev* fills, uint32_t n_fills, uint32_t n_slots,
                         uint32_t* slot_count) {
    rz::SceneDev S{};
    S.kind = b.kind;
    S.pts = b.pts;
    S.sub_off = b.sub_off;
    S.fills = fills;
    S.n_fills = n_fills;
    S.n_slots = n_slots;
    S.n_segments = b.n_segments;
    S.n_subpaths = b.n_subpaths;
    S.thr64 = b.thr64;
    S.thr32 = b.thr32;
    S.slot_count = slot_count;
    S.err = b.err;
    S.counters = b.counters;
    return S;
}

// Count + scan (lines per slot, then their offsets) on `st`.
rz_status lines_count(rz_ctx* ctx, rz::SceneDev& S, uint32_t* scan_tmp, cudaStream_t st) {
    const uint64_t nt = rz::slot_tasks(S.n_slots, S.task_depth) + 1;
    RZ_CUDA(cudaMemsetAsync(S.slot_count, 0, nt * 4, st));
    RZ_CUDA(rz::launch_flatten_count(S, st));
    RZ_CUDA(rz::scan_u32(S.slot_count, nt, scan_tmp, st));
    return RZ_OK;
}

// One batch render through the lines kernel (masks and items already staged in b / ctx->d_items).
rz_status run_lines(rz_ctx* ctx, const rz::BatchDev& b, const std::vector<rz::FillDev>& fills, uint32_t n_slots,
                    const Items& items, Trace& tr) {
    const int n = (int)items.items.size();
    if (n == 0 || fills.empty()) return RZ_OK;
    RZ_CUDA(ctx->p_fills.ensure(fills.size() * sizeof(rz::FillDev)));
    RZ_CUDA(cudaMemcpyAsync(ctx->p_fills.p, fills.data(), fills.size() * sizeof(rz::FillDev), cudaMemcpyHostToDevice,
                            ctx->stream));
    RZ_CUDA(ctx->p_slots.ensure((rz::slot_tasks(n_slots, 0) + 1) * 4));
    RZ_CUDA(ctx->p_scan.ensure(rz::scan_temp_words(rz::slot_tasks(n_slots, 0) + 1) * 4 + 64));
    rz::SceneDev S = lines_scene(b, (const rz::FillDev*)ctx->p_fills.p, (uint32_t)fills.size(), n_slots,
                                 (uint32_t*)ctx->p_slots.p);
    rz_status st = lines_count(ctx, S, (uint32_t*)ctx->p_scan.p, ctx->stream);
    if (st) return st;
    uint32_t n_lines = 0;
    RZ_CUDA(cudaMemcpyAsync(&n_lines, S.slot_count + rz::slot_tasks(n_slots, 0), 4, cudaMemcpyDeviceToHost,
                            ctx->stream));
    RZ_CUDA(cudaStreamSynchronize(ctx->stream));
    tr.mark("flatten_count");
    RZ_CUDA(ctx->p_lines.ensure((uint64_t)std::max(n_lines, 1u) * 2 * sizeof(int4)));
    S.lines = (int4*)ctx->p_lines.p;
    S.n_lines = n_lines;
    S.line_cap = n_lines;
    RZ_CUDA(rz::launch_flatten_emit(S, ctx->stream));
    int32_t* queue = (int32_t*)ctx->d_ctrl.p + 8;
    RZ_CUDA(cudaMemsetAsync(queue, 0, 4, ctx->stream));
    RZ_CUDA(rz::launch_mask_lines(S, b.masks, (const rz::WorkItem*)ctx->d_items.p, n, queue, b.out,
                                  batch_grid(ctx, n, true), ctx->stream));
    return RZ_OK;
}

// Slot records of a batch (k_band_records) in `buf`, when the batch has any
// and the buffer can hold them; otherwise the band kernel builds them per band.
rz::BatchDev with_records(const rz::BatchDev& b, uint32_t n_paths, DevBuf& buf) {
    rz::BatchDev r = b;
    r.n_paths = n_paths;
    r.recs = nullptr;
    const uint64_t n = (uint64_t)b.n_segments + b.n_subpaths;
    if (n == 0 || n_paths >= (1u << 30)) return r;
    if (buf.ensure(n * rz::band_record_bytes()) != cudaSuccess) {
        (void)cudaGetLastError();  // out of memory: per-band records
        return r;
    }
    r.recs = (const rz::SlotRec*)buf.p;
    return r;
}

rz_status run_bands(rz_ctx* ctx, const rz::BatchDev& b_in, const Items& items, bool per_path) {
    int32_t* queue = (int32_t*)ctx->d_ctrl.p + 8;
    const rz::WorkItem* d_items = (const rz::WorkItem*)ctx->d_items.p;
    if (items.items.empty()) return RZ_OK;
    const rz::BatchDev b = with_records(b_in, (uint32_t)(items.path_first.size() - 1), ctx->p_recs);
    RZ_CUDA(rz::launch_band_records(b, ctx->stream));
    if (!per_path) {
        const int n = (int)items.items.size();
        if (n == 0) return RZ_OK;
        const int grid = batch_grid(ctx, n);
        RZ_CUDA(cudaMemsetAsync(queue, 0, 4, ctx->stream));
        RZ_CUDA(rz::launch_mask_bands(b, d_items, n, queue, grid, ctx->stream));
    } else {
        for (size_t p = 0; p + 1 < items.path_first.size(); ++p) {
            const int f = items.path_first[p], n = items.path_first[p + 1] - f;
            if (n == 0) continue;
            RZ_CUDA(rz::launch_mask_bands(b, d_items + f, n, nullptr, n, ctx->stream));
        }
    }
    return RZ_OK;
}

// ---------------------------------------------------------------------------
// Host batches with page-locked output, in chunks of paths.  Three streams
// carry a chunk each: its segments up (s_in), its records and band kernel
// (the context stream), its masks down (s_out), so the host link moves one
// chunk's inputs and another's masks while the SMs render a third.  The masks
// are rendered into device memory and leave in one copy per chunk: the span
// from the chunk's first mask element to its last, padding included.
// ---------------------------------------------------------------------------
struct PipeChunk {
    uint32_t p_lo, p_hi;          // paths
    size_t item_lo, item_hi;      // work items (LPT order within the chunk)
    uint64_t out_lo, out_hi;      // output elements copied back
};

constexpr uint64_t kPipeChunkBytes = 32ull << 20;  // output bytes per chunk
constexpr int kPipeMaxChunks = 16;                 // queue heads in the control words

// Chunks of about equal pixel counts, the first and the last of half that
// size (the first download waits for the first chunk's render, the last
// render's download ends the call); none when the batch is too small to gain
// from overlap or its masks are laid out so that the chunks' spans overlap.
std::vector<PipeChunk> pipe_chunks(const std::vector<rz::MaskDev>& masks, uint64_t out_len) {
    std::vector<PipeChunk> chunks;
    const uint64_t bytes = out_len * 4;
    if (masks.size() < 2 || bytes < 2 * kPipeChunkBytes) return chunks;
    const int K = (int)std::min<uint64_t>(kPipeMaxChunks - 1, bytes / kPipeChunkBytes);
    uint64_t total = 0;
    for (const rz::MaskDev& m : masks)
        if (m.width > 0 && m.height > 0) total += (uint64_t)m.width * m.height;
    if (total == 0) return chunks;
    uint64_t acc = 0, spans = 0;
    uint32_t p_lo = 0;
    for (uint32_t p = 0; p < masks.size(); ++p) {
        const rz::MaskDev& m = masks[p];
        if (m.width > 0 && m.height > 0) acc += (uint64_t)m.width * m.height;
        const bool last = p + 1 == masks.size();
        if (!last && acc * 2 * K < total * (2 * chunks.size() + 1)) continue;
        PipeChunk c{p_lo, p + 1, 0, 0, ~0ull, 0};
        for (uint32_t q = p_lo; q <= p; ++q) {
            const rz::MaskDev& n = masks[q];
            if (n.width <= 0 || n.height <= 0) continue;
            c.out_lo = std::min<uint64_t>(c.out_lo, n.offset);
            c.out_hi = std::max<uint64_t>(c.out_hi, n.offset + (uint64_t)(n.height - 1) * n.row_stride + n.width);
        }
        if (c.out_hi > c.out_lo) {
            spans += c.out_hi - c.out_lo;
            chunks.push_back(c);
        } else if (!chunks.empty()) {
            chunks.back().p_hi = p + 1;  // no pixels: joins the chunk before
        } else {
            continue;  // leading paths without pixels join the first chunk
        }
        p_lo = p + 1;
    }
    if (chunks.size() < 2 || spans > out_len + out_len / 8) chunks.clear();  // interleaved layouts: one launch
    if (!chunks.empty()) chunks.front().p_lo = 0;
    return chunks;
}

rz_status pipe_streams(rz_ctx* ctx, size_t n_events) {
    if (!ctx->s_in) RZ_CUDA(cudaStreamCreateWithFlags(&ctx->s_in, cudaStreamNonBlocking));
    if (!ctx->s_out) RZ_CUDA(cudaStreamCreateWithFlags(&ctx->s_out, cudaStreamNonBlocking));
    // a call that failed half-way may have left copies queued: none may touch the buffers of this one
    RZ_CUDA(cudaStreamSynchronize(ctx->s_in));
    RZ_CUDA(cudaStreamSynchronize(ctx->s_out));
    while (ctx->pipe_ev.size() < n_events) {
        cudaEvent_t e;
        RZ_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ctx->pipe_ev.push_back(e);
    }
    return RZ_OK;
}

// Uploads the segments of each chunk (host sources hk / hp), renders it and
// copies its masks into the page-locked `out`.  b: the small arrays staged,
// the segment buffers allocated; hsub / hpsub: host copies of the offsets.
// A chunk's work list is built, sorted and uploaded just before its launch,
// so the first chunk renders while the host prepares the others.
rz_status run_pipelined(rz_ctx* ctx, rz::BatchDev b, const std::vector<rz::MaskDev>& masks,
                        std::vector<PipeChunk>& chunks, const uint32_t* hsub, const uint32_t* hpsub,
                        const char* hk, const char* hp, float* out, uint64_t out_len, Trace& tr) {
    const size_t K = chunks.size(), P = masks.size();
    rz_status st = pipe_streams(ctx, 2 * K + 1);
    if (st) return st;
    cudaEvent_t* ev_in = ctx->pipe_ev.data();
    cudaEvent_t* ev_done = ev_in + K;
    cudaEvent_t ev_out = ev_in[2 * K];
    // band heights and the first item of every path
    std::vector<int> rows(P, 0);
    std::vector<size_t> first(P + 1, 0);
    for (size_t p = 0; p < P; ++p) {
        const rz::MaskDev& m = masks[p];
        size_t n = 0;
        if (m.width > 0 && m.height > 0) {
            rows[p] = band_rows(m.clip_width, m.height, ctx->tune_rows_cap);
            n = (size_t)((m.height + rows[p] - 1) / rows[p]);
        }
        first[p + 1] = first[p] + n;
    }
    const size_t n_items = first[P];
    const size_t sz_m = P * sizeof(rz::MaskDev), sz_i = std::max<size_t>(n_items, 1) * sizeof(rz::WorkItem);
    RZ_CUDA(ctx->d_masks.ensure(sz_m + 16));
    RZ_CUDA(ctx->d_items.ensure(sz_i));
    RZ_CUDA(ctx->d_ctrl.ensure(256));
    RZ_CUDA(ctx->d_out.ensure(out_len * 4 + 16));
    RZ_CUDA(ctx->h_plan.ensure(sz_m + sz_i + 64));
    b.out = (float*)ctx->d_out.p;
    b.masks = (const rz::MaskDev*)ctx->d_masks.p;
    int32_t* ctrl = (int32_t*)ctx->d_ctrl.p;
    b.err = ctrl;
    b.counters = ctrl + 4;
    const rz::BatchDev br = with_records(b, (uint32_t)P, ctx->p_recs);
    char* hplan = (char*)ctx->h_plan.p;
    std::memcpy(hplan, masks.data(), sz_m);
    rz::WorkItem* h_items = (rz::WorkItem*)(hplan + ((sz_m + 15) & ~(size_t)15));
    RZ_CUDA(cudaMemsetAsync(ctrl, 0, 256, ctx->stream));  // error word, counters, queue heads
    RZ_CUDA(cudaEventRecord(ev_out, ctx->stream));
    RZ_CUDA(cudaStreamWaitEvent(ctx->s_in, ev_out, 0));  // the small arrays, then everything on s_in
    RZ_CUDA(cudaMemcpyAsync(ctx->d_masks.p, hplan, sz_m, cudaMemcpyHostToDevice, ctx->s_in));
    tr.mark("prepare");
    rz::WorkItem* d_items = (rz::WorkItem*)ctx->d_items.p;
    int32_t* queues = ctrl + 16;
    for (size_t k = 0; k < K; ++k) {
        PipeChunk& c = chunks[k];
        c.item_lo = first[c.p_lo];
        c.item_hi = first[c.p_hi];
        rz::WorkItem* it = h_items + c.item_lo;
        for (uint32_t p = c.p_lo; p < c.p_hi; ++p) {
            const rz::MaskDev& m = masks[p];
            for (int y = 0, i = 0; y < m.height && rows[p] > 0; y += rows[p], ++i) {
                rz::WorkItem& w = h_items[first[p] + i];
                w.path = p;
                w.y0 = (uint16_t)y;
                w.rows = (uint16_t)std::min(rows[p], m.height - y);
            }
        }
        const size_t n = c.item_hi - c.item_lo;
        lpt_sort(it, n, masks);
        // one upload queue in chunk order: the chunk's work list, then its segments
        if (n) RZ_CUDA(cudaMemcpyAsync(d_items + c.item_lo, it, n * sizeof(rz::WorkItem), cudaMemcpyHostToDevice,
                                       ctx->s_in));
        const uint32_t s0 = hsub[hpsub[c.p_lo]], s1 = hsub[hpsub[c.p_hi]];
        if (s1 > s0) {
            RZ_CUDA(cudaMemcpyAsync((uint8_t*)ctx->d_kind.p + s0, hk + s0, s1 - s0, cudaMemcpyHostToDevice, ctx->s_in));
            RZ_CUDA(cudaMemcpyAsync((char*)ctx->d_pts.p + 64ull * s0, hp + 64ull * s0, 64ull * (s1 - s0),
                                    cudaMemcpyHostToDevice, ctx->s_in));
        }
        RZ_CUDA(cudaEventRecord(ev_in[k], ctx->s_in));
        RZ_CUDA(cudaStreamWaitEvent(ctx->stream, ev_in[k], 0));
        RZ_CUDA(rz::launch_band_records(br, hsub[hpsub[c.p_lo]], hsub[hpsub[c.p_hi]], hpsub[c.p_lo], hpsub[c.p_hi],
                                        ctx->stream));
        if (n) RZ_CUDA(rz::launch_mask_bands(br, d_items + c.item_lo, (int)n, queues + k, batch_grid(ctx, (int)n),
                                             ctx->stream));
        RZ_CUDA(cudaEventRecord(ev_done[k], ctx->stream));
        RZ_CUDA(cudaStreamWaitEvent(ctx->s_out, ev_done[k], 0));
        RZ_CUDA(cudaMemcpyAsync(out + c.out_lo, b.out + c.out_lo, (c.out_hi - c.out_lo) * 4, cudaMemcpyDeviceToHost,
                                ctx->s_out));
    }
    RZ_CUDA(cudaEventRecord(ev_out, ctx->s_out));
    RZ_CUDA(cudaStreamWaitEvent(ctx->stream, ev_out, 0));  // the call's stream covers every copy
    return RZ_OK;
}

rz_status read_error(rz_ctx* ctx) {
    int32_t code = 0;
    RZ_CUDA(cudaMemcpyAsync(&code, ctx->d_ctrl.p, 4, cudaMemcpyDeviceToHost, ctx->stream));
    RZ_CUDA(cudaStreamSynchronize(ctx->stream));
    return status_from_device(ctx, code);
}

rz_status check_path(rz_ctx* ctx, const rz_path* path) {
    if (!path) return fail(ctx, RZ_ERR_INVALID, "path is null");
    if (path->n_segments && (!path->seg_kind || !path->seg_pts)) return fail(ctx, RZ_ERR_INVALID, "null segments");
    if (!path->subpath_off) return fail(ctx, RZ_ERR_INVALID, "null subpath_off");
    if (path->subpath_off[path->n_subpaths] > path->n_segments)
        return fail(ctx, RZ_ERR_INVALID, "subpath_off exceeds n_segments");
    for (uint32_t i = 0; i < path->n_subpaths; ++i)
        if (path->subpath_off[i] > path->subpath_off[i + 1]) return fail(ctx, RZ_ERR_INVALID, "subpath_off decreasing");
    for (uint32_t i = 0; i < path->n_segments; ++i)
        if (path->seg_kind[i] > RZ_SEG_ARC) return fail(ctx, RZ_ERR_INVALID, "bad segment kind");
    return RZ_OK;
}

void set_thresholds(rz::BatchDev& b, double flatness) {
    b.thr64 = 16.0 * flatness * flatness;  // PathFlattenIter::new src/path.rs:745-755
    b.thr32 = (float)b.thr64;
    // thr32 must not exceed the binary64 threshold (strict comparison at the boundary is re-decided in f64)
}

// Renders one path into a dense f32 (height x width) device buffer.
rz_status render_single(rz_ctx* ctx, const rz_path* path, const double tr[6], int32_t rule, double flatness,
                        uint64_t width, uint64_t height, bool iter_semantics) {
    rz_status st = check_path(ctx, path);
    if (st) return st;
    if (!valid_flatness(flatness)) return fail(ctx, RZ_ERR_INVALID, "flatness must be > 0 and finite");
    if (rule != RZ_FILL_NONZERO && rule != RZ_FILL_EVENODD) return fail(ctx, RZ_ERR_INVALID, "bad fill rule");
    if (width > 16383 || height > 16383) return fail(ctx, RZ_ERR_INVALID, "image too large (max 16383 x 16383)");
    RZ_CUDA(cudaSetDevice(ctx->device));
    Trace trc("render_single");
    rz::BatchDev b{};
    const uint32_t path_sub[2] = {0, path->n_subpaths};
    const uint8_t r8 = (uint8_t)rule;
    st = stage_host(ctx, path->seg_kind, path->seg_pts, path->n_segments, path->subpath_off, path->n_subpaths,
                    path_sub, 1, tr, &r8, b, nullptr, nullptr, &trc);
    if (st) return st;
    std::vector<rz::MaskDev> masks(1);
    masks[0].offset = 0;
    masks[0].width = (int32_t)width;
    masks[0].height = (int32_t)height;
    masks[0].row_stride = (int32_t)width;
    masks[0].clip_width = (int32_t)(iter_semantics ? width : width - 1);
    Items items;
    build_items(masks, false, items);
    st = stage_plan(ctx, masks, items, b);
    if (st) return st;
    trc.mark("plan");
    RZ_CUDA(ctx->d_out.ensure(width * height * 4 + 16));
    b.out = (float*)ctx->d_out.p;
    set_thresholds(b, flatness);
    st = run_bands(ctx, b, items, false);
    if (st) return st;
    trc.gpu_mark(ctx->stream, "bands");
    return RZ_OK;
}

}  // namespace

// Segment x band products above this take the line pipeline: a 200-cubic
// path over a 512^2 mask (31 bands, 6,231) renders in 0.19 ms there against
// 0.30 ms of band kernel (31 CTAs re-walking every tree).
#ifndef RZ_PIPELINE_MIN
#define RZ_PIPELINE_MIN 4000
#endif
namespace {
rz_status mask_pipeline(rz_ctx* ctx, const rz_path* path, const double tr[6], int32_t rule, double flatness,
                        uint64_t width, uint64_t height);

// The band kernel re-walks every segment for each band of rows; paths whose
// segments x bands product is large go through the line pipeline instead,
// which flattens every segment once and bins the lines by band.
bool use_pipeline(const rz_path* path, uint64_t width, uint64_t height) {
    if (!path) return false;
    const int rows = band_rows((int)width - 1, (int)height);
    const uint64_t bands = (height + rows - 1) / rows;
    return bands * ((uint64_t)path->n_segments + path->n_subpaths) > (uint64_t)RZ_PIPELINE_MIN;
}
}  // namespace

extern "C" {

rz_status rz_mask(rz_ctx* ctx, const rz_path* path, const double tr[6], int32_t fill_rule, double flatness,
                  double* img, rz_shape shape) {
    if (!ctx) return RZ_ERR_INVALID;
    std::lock_guard<std::mutex> lock(ctx->mu);
    if (!tr || !img) return fail(ctx, RZ_ERR_INVALID, "null argument");
    if (shape.width == 0 || shape.height == 0) return RZ_OK;
    rz_status st;
    Trace trc("rz_mask");
    if (use_pipeline(path, shape.width, shape.height)) {
        st = check_path(ctx, path);
        if (st) return st;
        if (!valid_flatness(flatness)) return fail(ctx, RZ_ERR_INVALID, "flatness must be > 0 and finite");
        if (fill_rule != RZ_FILL_NONZERO && fill_rule != RZ_FILL_EVENODD) return fail(ctx, RZ_ERR_INVALID, "bad fill rule");
        if (shape.width > 16383 || shape.height > 16383) return fail(ctx, RZ_ERR_INVALID, "image too large");
        RZ_CUDA(cudaSetDevice(ctx->device));
        st = mask_pipeline(ctx, path, tr, fill_rule, flatness, shape.width, shape.height);
    } else {
        st = render_single(ctx, path, tr, fill_rule, flatness, shape.width, shape.height, false);
    }
    if (st) return st;
    trc.gpu_mark(ctx->stream, "render");
    const size_t n = shape.width * shape.height;
    RZ_CUDA(ctx->h_out.ensure(n * 4));
    RZ_CUDA(cudaMemcpyAsync(ctx->h_out.p, ctx->d_out.p, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    st = read_error(ctx);
    if (st) return st;
    trc.mark("download");
    const float* src = (const float*)ctx->h_out.p;
    parallel_for((int64_t)shape.height, 32, [&](int64_t y0, int64_t y1) {
        for (int64_t y = y0; y < y1; ++y) {
            const float* s = src + (uint64_t)y * shape.width;
            double* d = img + shape.start + (uint64_t)y * shape.row_stride;
            if (shape.col_stride == 1) {
                for (uint64_t x = 0; x < shape.width; ++x) d[x] = (double)s[x];
            } else {
                for (uint64_t x = 0; x < shape.width; ++x) d[x * shape.col_stride] = (double)s[x];
            }
        }
    });
    trc.mark("to_f64");
    return RZ_OK;
}

rz_status rz_mask_iter(rz_ctx* ctx, const rz_path* path, const double tr[6], int32_t fill_rule, double flatness,
                       uint64_t width, uint64_t height, rz_pixel* pixels, uint64_t cap, uint64_t* n_pixels) {
    if (!ctx) return RZ_ERR_INVALID;
    std::lock_guard<std::mutex> lock(ctx->mu);
    if (!tr || !n_pixels) return fail(ctx, RZ_ERR_INVALID, "null argument");
    *n_pixels = 0;
    if (width == 0 || height == 0) return RZ_OK;  // src/rasterize.rs:320-322
    rz_status st = render_single(ctx, path, tr, fill_rule, flatness, width, height, true);
    if (st) return st;
    const size_t n = width * height;
    RZ_CUDA(ctx->h_out.ensure(n * 4));
    RZ_CUDA(cudaMemcpyAsync(ctx->h_out.p, ctx->d_out.p, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    st = read_error(ctx);
    if (st) return st;
    const float* src = (const float*)ctx->h_out.p;
    uint64_t k = 0;
    for (uint64_t y = 0; y < height; ++y)
        for (uint64_t x = 0; x < width; ++x) {
            const float a = src[y * width + x];
            if (std::fabs(a) < 1e-6f) continue;
            if (k < cap && pixels) {
                pixels[k].x = x;
                pixels[k].y = y;
                pixels[k].alpha = (double)a;
            }
            ++k;
        }
    *n_pixels = k;
    return RZ_OK;
}

static rz_status mask_batch_impl(rz_ctx* ctx, const rz_path_batch* batch, double flatness, float* out,
                                 uint64_t out_len, bool per_path) {
    if (!ctx) return RZ_ERR_INVALID;
    std::lock_guard<std::mutex> lock(ctx->mu);
    if (!batch || !out || !batch->masks) return fail(ctx, RZ_ERR_INVALID, "null argument");
    if (!valid_flatness(flatness)) return fail(ctx, RZ_ERR_INVALID, "flatness must be > 0 and finite");
    RZ_CUDA(cudaSetDevice(ctx->device));
    Trace tr("rz_mask_batch");
    const uint32_t P = batch->n_paths;
    std::vector<rz::MaskDev> masks(P);
    for (uint32_t p = 0; p < P; ++p) {
        const rz_mask_desc& d = batch->masks[p];
        if (d.width > 16383 || d.height > 16383 || (d.height > 0 && d.row_stride < d.width))
            return fail(ctx, RZ_ERR_INVALID, "bad mask descriptor");
        if (d.width && d.height && d.offset + (uint64_t)(d.height - 1) * d.row_stride + d.width > out_len)
            return fail(ctx, RZ_ERR_INVALID, "mask exceeds output buffer");
        masks[p].offset = d.offset;
        masks[p].width = (int32_t)d.width;
        masks[p].height = (int32_t)d.height;
        masks[p].row_stride = (int32_t)d.row_stride;
        masks[p].clip_width = (int32_t)d.width - 1;
    }
    rz::BatchDev b{};
    rz_status st;
    if (batch->memory == RZ_MEM_HOST) {
        for (uint32_t p = 0; p < P; ++p)
            if (batch->path_subpath_off[p] > batch->path_subpath_off[p + 1])
                return fail(ctx, RZ_ERR_INVALID, "path_subpath_off decreasing");
        if (batch->path_subpath_off[P] > batch->n_subpaths) return fail(ctx, RZ_ERR_INVALID, "bad path_subpath_off");
        for (uint32_t i = 0; i < batch->n_subpaths; ++i)
            if (batch->subpath_off[i] > batch->subpath_off[i + 1])
                return fail(ctx, RZ_ERR_INVALID, "subpath_off decreasing");
        if (batch->subpath_off[batch->n_subpaths] > batch->n_segments)
            return fail(ctx, RZ_ERR_INVALID, "subpath_off exceeds n_segments");
        tr.mark("validate");
        // page-locked output of a large batch: chunks of paths, uploads and downloads overlapped with rendering
        std::vector<PipeChunk> chunks;
        if (!per_path && !use_lines_kernel() && mapped_host(out)) chunks = pipe_chunks(masks, out_len);
        const char *hk = nullptr, *hp = nullptr;
        tr.mark("chunks");
        st = stage_host(ctx, batch->seg_kind, batch->seg_pts, batch->n_segments, batch->subpath_off,
                        batch->n_subpaths, batch->path_subpath_off, P, batch->transforms, batch->fill_rules, b,
                        chunks.empty() ? nullptr : &hk, chunks.empty() ? nullptr : &hp, &tr);
        if (st) return st;
        tr.mark("stage_inputs");
        if (!chunks.empty()) {
            set_thresholds(b, flatness);
            const uint32_t* hsub = ctx->expanded ? ctx->x_sub.data() : batch->subpath_off;
            const uint32_t* hpsub = ctx->expanded ? ctx->x_psub.data() : batch->path_subpath_off;
            st = run_pipelined(ctx, b, masks, chunks, hsub, hpsub, hk, hp, out, out_len, tr);
            if (st) return st;
            tr.mark("enqueue");
            st = read_error(ctx);
            tr.mark("sync");
            return st;
        }
    } else {
        b.kind = batch->seg_kind;
        b.pts = batch->seg_pts;
        b.sub_off = batch->subpath_off;
        b.path_sub = batch->path_subpath_off;
        b.tr = batch->transforms;
        b.rule = batch->fill_rules;
        b.n_segments = batch->n_segments;
        b.n_subpaths = batch->n_subpaths;
    }
    const bool lines = !per_path && batch->memory == RZ_MEM_HOST && use_lines_kernel();
    Items items;
    build_items(masks, per_path, items, ctx->tune_rows_cap, lines ? rz::lines_band_floats() : 0);
    tr.mark("items");
    st = stage_plan(ctx, masks, items, b);
    if (st) return st;
    set_thresholds(b, flatness);
    // page-locked host output: the kernel writes the masks straight into it
    // (over NVLink-C2C on Grace), so no device copy and no copy back
    void* direct_out = batch->memory == RZ_MEM_HOST ? mapped_host(out) : nullptr;
    if (batch->memory == RZ_MEM_HOST && !direct_out) {
        RZ_CUDA(ctx->d_out.ensure(out_len * 4 + 16));
        b.out = (float*)ctx->d_out.p;
    } else {
        b.out = direct_out ? (float*)direct_out : out;
    }
    b.flat_out = direct_out ? 1 : 0;
    tr.mark("stage_plan");
    if (lines) {
        std::vector<rz::FillDev> fills;
        const uint32_t n_slots = lines_fills(masks, ctx->expanded ? ctx->x_sub.data() : batch->subpath_off,
                                             ctx->expanded ? ctx->x_psub.data() : batch->path_subpath_off,
                                             batch->fill_rules, batch->transforms, fills);
        st = run_lines(ctx, b, fills, n_slots, items, tr);
    } else {
        st = run_bands(ctx, b, items, per_path);
    }
    if (st) return st;
    if (batch->memory == RZ_MEM_HOST && !direct_out)
        RZ_CUDA(cudaMemcpyAsync(out, b.out, out_len * 4, cudaMemcpyDeviceToHost, ctx->stream));
    tr.mark("enqueue");
    st = read_error(ctx);
    tr.mark("sync");
    return st;
}

rz_status rz_mask_batch(rz_ctx* ctx, const rz_path_batch* batch, double flatness, float* out, uint64_t out_len) {
    return mask_batch_impl(ctx, batch, flatness, out, out_len, false);
}

rz_status rz_mask_batch_per_path(rz_ctx* ctx, const rz_path_batch* batch, double flatness, float* out,
                                 uint64_t out_len) {
    return mask_batch_impl(ctx, batch, flatness, out, out_len, true);
}

rz_status rz_flatten_counts(rz_ctx* ctx, const rz_path* path, const double tr[6], double flatness,
                            uint32_t* counts, uint64_t cap, uint64_t* n_counts) {
    if (!ctx) return RZ_ERR_INVALID;
    std::lock_guard<std::mutex> lock(ctx->mu);
    rz_status st = check_path(ctx, path);
    if (st) return st;
    if (!tr || !n_counts) return fail(ctx, RZ_ERR_INVALID, "null argument");
    if (!valid_flatness(flatness)) return fail(ctx, RZ_ERR_INVALID, "flatness must be > 0 and finite");
    RZ_CUDA(cudaSetDevice(ctx->device));
    rz::BatchDev b{};
    const uint32_t path_sub[2] = {0, path->n_subpaths};
    st = stage_host(ctx, path->seg_kind, path->seg_pts, path->n_segments, path->subpath_off, path->n_subpaths,
                    path_sub, 1, tr, nullptr, b);
    if (st) return st;
    std::vector<rz::MaskDev> none;
    Items items;
    st = stage_plan(ctx, none, items, b);
    if (st) return st;
    set_thresholds(b, flatness);
    const uint64_t n = (uint64_t)path->n_segments + path->n_subpaths;
    *n_counts = n;
    const uint64_t ne = (uint64_t)b.n_segments + b.n_subpaths;  // after host arc expansion
    RZ_CUDA(ctx->d_counts.ensure(ne * 4 + 4));
    RZ_CUDA(rz::launch_flatten_counts(b, b.n_segments, b.n_subpaths, (uint32_t*)ctx->d_counts.p, ctx->stream));
    std::vector<uint32_t> dev_counts(ne);
    if (ne) RZ_CUDA(cudaMemcpyAsync(dev_counts.data(), ctx->d_counts.p, ne * 4, cudaMemcpyDeviceToHost, ctx->stream));
    st = read_error(ctx);
    if (st) return st;
    std::vector<uint32_t> agg(n, 0);
    if (ctx->expanded) {
        for (uint32_t j = 0; j < b.n_segments; ++j) agg[ctx->x_segmap[j]] += dev_counts[j];
        for (uint32_t t = 0; t < b.n_subpaths; ++t) agg[path->n_segments + ctx->x_submap[t]] = dev_counts[b.n_segments + t];
    } else {
        agg = dev_counts;
    }
    if (counts) std::memcpy(counts, agg.data(), std::min(cap, n) * 4);
    return RZ_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batch plans
// ---------------------------------------------------------------------------
struct rz_batch_plan {
    rz_ctx* ctx = nullptr;
    rz::BatchDev b{};
    Items items;
    DevBuf d_masks, d_items, d_ctrl, d_recs;
    // lines kernel: fills, line offsets, scan scratch, lines
    bool lines = false;
    DevBuf d_fills, d_slots, d_scan, d_lines;
    // glyph pipeline: records, coefficients, chain lengths / offsets, tree codes, path flags, vertices
    bool glyph = false;
    rz::GlyphDev g{};
    DevBuf d_grecs, d_gcoef, d_chain, d_code, d_pflags, d_vtx, d_gpaths;
    int grid = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t capture_stream = nullptr;
};

extern "C" {

rz_batch_plan* rz_batch_plan_create(rz_ctx* ctx, const rz_path_batch* batch, double flatness, float* out,
                                    uint64_t out_len, rz_status* status) {
    auto bail = [&](rz_status st) {
        if (status) *status = st;
        return (rz_batch_plan*)nullptr;
    };
    if (!ctx) return bail(RZ_ERR_INVALID);
    std::lock_guard<std::mutex> lock(ctx->mu);
    if (!batch || !out || !batch->masks || batch->memory != RZ_MEM_DEVICE)
        return bail(fail(ctx, RZ_ERR_INVALID, "a plan needs a device-memory batch and output"));
    if (!valid_flatness(flatness)) return bail(fail(ctx, RZ_ERR_INVALID, "flatness must be > 0 and finite"));
    if (cudaSetDevice(ctx->device) != cudaSuccess) return bail(fail(ctx, RZ_ERR_CUDA, "cudaSetDevice"));
    const uint32_t P = batch->n_paths;
    std::vector<rz::MaskDev> masks(P);
    for (uint32_t p = 0; p < P; ++p) {
        const rz_mask_desc& d = batch->masks[p];
        if (d.width > 16383 || d.height > 16383 || (d.height > 0 && d.row_stride < d.width))
            return bail(fail(ctx, RZ_ERR_INVALID, "bad mask descriptor"));
        if (d.width && d.height && d.offset + (uint64_t)(d.height - 1) * d.row_stride + d.width > out_len)
            return bail(fail(ctx, RZ_ERR_INVALID, "mask exceeds output buffer"));
        masks[p].offset = d.offset;
        masks[p].width = (int32_t)d.width;
        masks[p].height = (int32_t)d.height;
        masks[p].row_stride = (int32_t)d.row_stride;
        masks[p].clip_width = (int32_t)d.width - 1;
    }
    rz_batch_plan* plan = new rz_batch_plan();
    plan->ctx = ctx;
    // the lines kernel needs the offsets on the host and no raw arcs (those are expanded by the band kernel)
    std::vector<uint8_t> h_kind;
    std::vector<uint32_t> h_sub, h_psub;
    std::vector<uint8_t> h_rule;
    std::vector<double> h_tr;
    if (use_lines_kernel() && P > 0) {
        h_kind.resize(batch->n_segments);
        h_sub.resize((size_t)batch->n_subpaths + 1);
        h_psub.resize((size_t)P + 1);
        cudaError_t ce = cudaSuccess;
        if (batch->n_segments)
            ce = cudaMemcpy(h_kind.data(), batch->seg_kind, batch->n_segments, cudaMemcpyDeviceToHost);
        if (ce == cudaSuccess)
            ce = cudaMemcpy(h_sub.data(), batch->subpath_off, h_sub.size() * 4, cudaMemcpyDeviceToHost);
        if (ce == cudaSuccess)
            ce = cudaMemcpy(h_psub.data(), batch->path_subpath_off, h_psub.size() * 4, cudaMemcpyDeviceToHost);
        if (ce == cudaSuccess && batch->fill_rules) {
            h_rule.resize(P);
            ce = cudaMemcpy(h_rule.data(), batch->fill_rules, P, cudaMemcpyDeviceToHost);
        }
        if (ce == cudaSuccess && batch->transforms) {
            h_tr.resize((size_t)P * 6);
            ce = cudaMemcpy(h_tr.data(), batch->transforms, h_tr.size() * 8, cudaMemcpyDeviceToHost);
        }
        if (ce != cudaSuccess) {
            delete plan;
            return bail(cuda_fail(ctx, ce, "plan: reading the batch offsets"));
        }
        bool ok = !(batch->n_segments && std::memchr(h_kind.data(), RZ_SEG_ARC, batch->n_segments));
        for (uint32_t p = 0; ok && p < P; ++p) ok = h_psub[p] <= h_psub[p + 1] && h_psub[p + 1] <= batch->n_subpaths;
        for (uint32_t i = 0; ok && i < batch->n_subpaths; ++i) ok = h_sub[i] <= h_sub[i + 1];
        ok = ok && h_sub[batch->n_subpaths] <= batch->n_segments;
        plan->lines = ok;
    }
    if (!plan->lines && P > 0 && use_glyph_pipeline()) {
        // the glyph pipeline needs non-decreasing subpath and path offsets (every slot in one path)
        h_sub.resize((size_t)batch->n_subpaths + 1);
        h_psub.resize((size_t)P + 1);
        cudaError_t ce = cudaMemcpy(h_sub.data(), batch->subpath_off, h_sub.size() * 4, cudaMemcpyDeviceToHost);
        if (ce == cudaSuccess)
            ce = cudaMemcpy(h_psub.data(), batch->path_subpath_off, h_psub.size() * 4, cudaMemcpyDeviceToHost);
        if (ce != cudaSuccess) {
            delete plan;
            return bail(cuda_fail(ctx, ce, "plan: reading the batch offsets"));
        }
        plan->glyph = offsets_monotone(h_sub.data(), batch->n_subpaths, batch->n_segments, h_psub.data(), P);
    }
    build_items(masks, false, plan->items, ctx->tune_rows_cap,
                plan->lines ? rz::lines_band_floats() : (plan->glyph ? rz::kGlyphBandFloats : 0));
    const size_t sz_m = std::max<size_t>(masks.size(), 1) * sizeof(rz::MaskDev);
    const size_t sz_i = std::max<size_t>(plan->items.items.size(), 1) * sizeof(rz::WorkItem);
    cudaError_t e = plan->d_masks.ensure(sz_m);
    if (e == cudaSuccess) e = plan->d_items.ensure(sz_i);
    if (e == cudaSuccess) e = plan->d_ctrl.ensure(64);
    if (e == cudaSuccess && !masks.empty())
        e = cudaMemcpy(plan->d_masks.p, masks.data(), masks.size() * sizeof(rz::MaskDev), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !plan->items.items.empty())
        e = cudaMemcpy(plan->d_items.p, plan->items.items.data(), plan->items.items.size() * sizeof(rz::WorkItem),
                       cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(plan->d_ctrl.p, 0, 64);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&plan->capture_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        rz_batch_plan_destroy(plan);
        return bail(cuda_fail(ctx, e, "plan setup"));
    }
    rz::BatchDev& b = plan->b;
    b.kind = batch->seg_kind;
    b.pts = batch->seg_pts;
    b.sub_off = batch->subpath_off;
    b.path_sub = batch->path_subpath_off;
    b.tr = batch->transforms;
    b.rule = batch->fill_rules;
    b.n_segments = batch->n_segments;
    b.n_subpaths = batch->n_subpaths;
    b.masks = (const rz::MaskDev*)plan->d_masks.p;
    b.out = out;
    b.flat_out = mapped_host(out) ? 1 : 0;  // page-locked host output: whole-line spans
    int32_t* ctrl = (int32_t*)plan->d_ctrl.p;
    b.err = ctrl;
    b.counters = ctrl + 4;
    set_thresholds(b, flatness);
    const int n = (int)plan->items.items.size();
    plan->grid = plan->glyph ? glyph_grid(ctx, n) : batch_grid(ctx, n, plan->lines);
    if (!plan->lines && !plan->glyph && n > 0) b = with_records(b, P, plan->d_recs);
    if (plan->glyph) {
        b.n_paths = P;
        e = glyph_setup(b, plan->g, plan->d_grecs, plan->d_gcoef, plan->d_chain, plan->d_code, plan->d_pflags,
                        plan->d_vtx, plan->d_scan, plan->d_gpaths, plan->capture_stream);
        if (e != cudaSuccess) {
            rz_batch_plan_destroy(plan);
            return bail(cuda_fail(ctx, e, "plan: glyph pipeline buffers"));
        }
        if (ctx->tune_walk > 0) plan->g.walk_slots = ctx->tune_walk;
    }
    int32_t* queue = ctrl + 8;
    rz::SceneDev S{};
    if (plan->lines) {
        // fills, offsets and a first count + scan (outside the graph) to size the line buffer
        std::vector<rz::FillDev> fills;
        const uint32_t n_slots = lines_fills(masks, h_sub.data(), h_psub.data(), batch->fill_rules ? h_rule.data() : nullptr,
                                             batch->transforms ? h_tr.data() : nullptr, fills);
        e = plan->d_fills.ensure(std::max<size_t>(fills.size(), 1) * sizeof(rz::FillDev));
        if (e == cudaSuccess && !fills.empty())
            e = cudaMemcpy(plan->d_fills.p, fills.data(), fills.size() * sizeof(rz::FillDev), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = plan->d_slots.ensure((rz::slot_tasks(n_slots, 0) + 1) * 4);
        if (e == cudaSuccess) e = plan->d_scan.ensure(rz::scan_temp_words(rz::slot_tasks(n_slots, 0) + 1) * 4 + 64);
        S = lines_scene(b, (const rz::FillDev*)plan->d_fills.p, (uint32_t)fills.size(), n_slots,
                        (uint32_t*)plan->d_slots.p);
        uint32_t n_lines = 0;
        if (e == cudaSuccess && lines_count(ctx, S, (uint32_t*)plan->d_scan.p, plan->capture_stream) != RZ_OK)
            e = cudaErrorUnknown;
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(&n_lines, S.slot_count + rz::slot_tasks(n_slots, 0), 4, cudaMemcpyDeviceToHost,
                                plan->capture_stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(plan->capture_stream);
        if (e == cudaSuccess) e = plan->d_lines.ensure((uint64_t)std::max(n_lines, 1u) * 2 * sizeof(int4));
        S.lines = (int4*)plan->d_lines.p;
        S.n_lines = n_lines;
        // replays of changed geometry get the buffer's slack, then an RZ_ERR_CAPACITY status, never an overrun
        S.line_cap = (uint32_t)std::min<uint64_t>(plan->d_lines.cap / (2 * sizeof(int4)), 0xffffffffull);
        if (e != cudaSuccess) {
            rz_batch_plan_destroy(plan);
            return bail(cuda_fail(ctx, e, "plan: line buffer"));
        }
    }
    // capture: (lines: count, scan, emit,) reset the queue head, one persistent launch
    e = cudaStreamBeginCapture(plan->capture_stream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        if (plan->lines) {
            lines_count(ctx, S, (uint32_t*)plan->d_scan.p, plan->capture_stream);
            rz::launch_flatten_emit(S, plan->capture_stream);
        }
        if (plan->glyph) glyph_enqueue_flatten(plan->g, (uint32_t*)plan->d_scan.p, P, plan->capture_stream);
        cudaMemsetAsync(queue, 0, 4, plan->capture_stream);
        if (n > 0) {
            if (plan->glyph)
                rz::launch_glyph_cover(plan->g, (const rz::WorkItem*)plan->d_items.p, n, queue, plan->grid,
                                       plan->capture_stream);
            else if (plan->lines)
                rz::launch_mask_lines(S, (const rz::MaskDev*)plan->d_masks.p, (const rz::WorkItem*)plan->d_items.p, n,
                                      queue, out, plan->grid, plan->capture_stream);
            else {
                rz::launch_band_records(b, plan->capture_stream);
                rz::launch_mask_bands(b, (const rz::WorkItem*)plan->d_items.p, n, queue, plan->grid,
                                      plan->capture_stream);
            }
        }
        e = cudaStreamEndCapture(plan->capture_stream, &plan->graph);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&plan->exec, plan->graph, 0);
    if (e != cudaSuccess) {
        rz_batch_plan_destroy(plan);
        return bail(cuda_fail(ctx, e, "graph capture"));
    }
    if (status) *status = RZ_OK;
    return plan;
}

rz_status rz_batch_plan_launch(rz_batch_plan* plan) {
    if (!plan) return RZ_ERR_INVALID;
    rz_ctx* ctx = plan->ctx;
    RZ_CUDA(cudaGraphLaunch(plan->exec, ctx->stream));
    return RZ_OK;
}

rz_status rz_batch_plan_status(rz_batch_plan* plan) {
    if (!plan) return RZ_ERR_INVALID;
    rz_ctx* ctx = plan->ctx;
    int32_t code = 0;
    RZ_CUDA(cudaMemcpyAsync(&code, plan->d_ctrl.p, 4, cudaMemcpyDeviceToHost, ctx->stream));
    RZ_CUDA(cudaStreamSynchronize(ctx->stream));
    if (code) RZ_CUDA(cudaMemsetAsync(plan->d_ctrl.p, 0, 4, ctx->stream));
    return status_from_device(ctx, code);
}

rz_status rz_batch_plan_info(rz_batch_plan* plan, uint64_t* n_items, uint64_t* fallbacks) {
    if (!plan) return RZ_ERR_INVALID;
    rz_ctx* ctx = plan->ctx;
    if (n_items) *n_items = plan->items.items.size();
    if (fallbacks) {
        int32_t f = 0;
        RZ_CUDA(cudaMemcpyAsync(&f, (int32_t*)plan->d_ctrl.p + 5, 4, cudaMemcpyDeviceToHost, ctx->stream));
        RZ_CUDA(cudaStreamSynchronize(ctx->stream));
        *fallbacks = (uint64_t)f;
    }
    return RZ_OK;
}

void rz_batch_plan_destroy(rz_batch_plan* plan) {
    if (!plan) return;
    if (plan->ctx) cudaStreamSynchronize(plan->ctx->stream);
    if (plan->exec) cudaGraphExecDestroy(plan->exec);
    if (plan->graph) cudaGraphDestroy(plan->graph);
    if (plan->capture_stream) cudaStreamDestroy(plan->capture_stream);
    plan->d_masks.release();
    plan->d_items.release();
    plan->d_ctrl.release();
    plan->d_recs.release();
    plan->d_fills.release();
    plan->d_slots.release();
    plan->d_scan.release();
    plan->d_lines.release();
    plan->d_grecs.release();
    plan->d_gcoef.release();
    plan->d_chain.release();
    plan->d_code.release();
    plan->d_pflags.release();
    plan->d_vtx.release();
    plan->d_gpaths.release();
    delete plan;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Line pipeline: large paths and painted scenes
// ---------------------------------------------------------------------------
namespace {

// Rasterizer::fill's paint set-up (src/rasterize.rs:78-97) for a fill drawn
// with transform `tr` (binary64): units transform, its inverse, stops.
void prepare_paint(const rz_paint& in, const rzhost::Xf& tr, bool have_bbox, const rzhost::Box& bbox0,
                   rz::PaintDev& out) {
    std::memset(&out, 0, sizeof(out));
    out.kind = in.kind;
    out.spread = in.spread;
    out.linear_colors = in.linear_colors ? 1 : 0;
    if (in.kind == RZ_PAINT_SOLID) {
        for (int i = 0; i < 4; ++i) out.color[i] = in.color[i];
        return;
    }
    rzhost::Xf ptr;
    std::memcpy(ptr.m, in.tr, sizeof(ptr.m));
    rzhost::Xf units;
    if (in.units == RZ_UNITS_USER_SPACE) {
        units = rzhost::xf_mul(tr, ptr);
    } else {
        if (!have_bbox) {
            out.kind = -1;  // empty path: nothing drawn
            return;
        }
        // BBox::unit_transform: translate(x, y) * scale(width, height) (src/geometry.rs:662-664)
        const rzhost::Xf t{{1.0, 0.0, bbox0.x0, 0.0, 1.0, bbox0.y0}};
        const rzhost::Xf sc{{bbox0.x1 - bbox0.x0, 0.0, 0.0, 0.0, bbox0.y1 - bbox0.y0, 0.0}};
        units = rzhost::xf_mul(rzhost::xf_mul(tr, rzhost::xf_mul(t, sc)), ptr);
    }
    rzhost::Xf pix;
    if (!rzhost::xf_invert(units, pix)) {
        out.kind = -1;  // not invertible: nothing drawn (src/rasterize.rs:92)
        return;
    }
    // GradStops::new: stable sort by position, a black stop when empty; sRGB stops when !linear_colors
    struct St {
        double pos;
        float c[4];
    };
    std::vector<St> stops;
    for (uint32_t i = 0; i < std::min<uint32_t>(in.n_stops, rz::kMaxStops); ++i) {
        St t;
        t.pos = in.stops[i].position;
        std::memcpy(t.c, in.stops[i].color, sizeof(t.c));
        stops.push_back(t);
    }
    std::stable_sort(stops.begin(), stops.end(), [](const St& a, const St& b) { return a.pos < b.pos; });
    if (stops.empty()) stops.push_back(St{0.0, {0.f, 0.f, 0.f, 1.f}});
    out.nstops = (int)stops.size();
    for (int i = 0; i < out.nstops; ++i) {
        if (!in.linear_colors) rzhost::into_srgb(stops[i].c);
        out.pos[i] = (float)stops[i].pos;
        for (int c = 0; c < 4; ++c) out.col[i][c] = stops[i].c[c];
    }
    if (in.kind == RZ_PAINT_LINEAR) {
        const double dx = in.end[0] - in.start[0], dy = in.end[1] - in.start[1];
        const double dd = dx * dx + dy * dy;
        const double ux = dx / dd, uy = dy / dd;
        // t of a local pixel centre (x, y) = g0 x + g1 y + g2 (GradLinear::at, src/grad.rs:202-211)
        const double g[3] = {pix.m[0] * ux + pix.m[3] * uy, pix.m[1] * ux + pix.m[4] * uy,
                             (pix.m[2] - in.start[0]) * ux + (pix.m[5] - in.start[1]) * uy};
        for (int i = 0; i < 3; ++i) {
            out.gh[i] = (float)g[i];
            out.gl[i] = (float)(g[i] - (double)out.gh[i]);
        }
    } else {
        // p - focal centre of a local pixel centre, composed in binary64
        const double q[6] = {pix.m[0], pix.m[1], pix.m[2] - in.end[0], pix.m[3], pix.m[4], pix.m[5] - in.end[1]};
        for (int i = 0; i < 6; ++i) {
            out.q[i] = (float)q[i];
            out.qd[i] = q[i];
        }
        out.cdxd = in.start[0] - in.end[0];
        out.cdyd = in.start[1] - in.end[1];
        out.rdd = in.radius - in.fradius;
        out.frd = in.fradius;
        out.cdx = (float)out.cdxd;
        out.cdy = (float)out.cdyd;
        out.rd = (float)out.rdd;
        out.fr = (float)out.frd;
        out.a64 = (out.cdxd * out.cdxd + out.cdyd * out.cdyd) - out.rdd * out.rdd;
        out.radial_linear = std::fabs(out.a64) < rzhost::kEps ? 1 : 0;
    }
}

struct HostScene {
    std::vector<rz::FillDev> fills;
    // or the fills already built on the device (ctx->p_fills, n_dev_fills of them): nothing to upload
    uint32_t n_dev_fills = 0;
    std::vector<rz::PaintDev> paints;
    const uint8_t* kind = nullptr;
    const double* pts = nullptr;
    const uint32_t* sub_off = nullptr;
    uint32_t n_seg = 0, n_sub = 0;
    uint32_t n_slots = 0, n_entries = 0;
    int band_rows = 1, n_bands = 0, max_clip = 1;
    int task_depth = 0;  // flatten tasks per slot = 2^task_depth (2 for large segments)
    std::vector<uint32_t> task_off;  // or per slot: first task (2^k tasks each), then the total
};

// Flatten tasks per slot from each segment's root flatness (the reference's
// formula on the transformed control points): a curve whose tree is about D
// levels deep gets 2^(D - leaf_shift) subtree tasks (at most 1024), so every
// task walks about 2^leaf_shift leaves however long the curve (8 by default;
// small scenes, whose few tasks leave most SMs idle, take shorter ones).
// Closing lines and lines get one.
void adaptive_tasks(HostScene& hs, double flatness, int leaf_shift = 3) {
    const double thr = 16.0 * flatness * flatness;
    hs.task_off.assign((size_t)hs.n_slots + 1, 0);
    for (const rz::FillDev& f : hs.fills) {
        const uint32_t nseg = f.seg1 - f.seg0, nslot = nseg + (f.sub1 - f.sub0);
        // per slot: the log2 of its task count (slots of different fills never overlap)
        parallel_for((int64_t)nslot, 2048, [&](int64_t i0, int64_t i1) {
            for (int64_t i = i0; i < i1; ++i) {
                int depth = 0;
                if (i < (int64_t)nseg) {
                    const uint32_t g = f.seg0 + (uint32_t)i;
                    const int kind = hs.kind[g];
                    if (kind == RZ_SEG_QUAD || kind == RZ_SEG_CUBIC) {
                        const double* p = hs.pts + 8ull * g;
                        double x[4], y[4];
                        for (int q = 0; q < 4; ++q) {
                            x[q] = f.tr[0] * p[2 * q] + f.tr[1] * p[2 * q + 1] + f.tr[2];
                            y[q] = f.tr[3] * p[2 * q] + f.tr[4] * p[2 * q + 1] + f.tr[5];
                        }
                        double fl;
                        if (kind == RZ_SEG_QUAD) {
                            const double ux = 2 * x[1] - x[0] - x[2], uy = 2 * y[1] - y[0] - y[2];
                            fl = ux * ux + uy * uy;
                        } else {
                            const double ux = 3 * x[1] - 2 * x[0] - x[3], uy = 3 * y[1] - 2 * y[0] - y[3];
                            const double vx = 3 * x[2] - x[0] - 2 * x[3], vy = 3 * y[2] - y[0] - 2 * y[3];
                            fl = std::max(ux * ux, vx * vx) + std::max(uy * uy, vy * vy);
                        }
                        int d = 0;
                        while (d < 22 && std::isfinite(fl) && fl >= thr) {
                            fl /= 16.0;
                            ++d;
                        }
                        depth = std::min(10, std::max(0, d - leaf_shift));
                    }
                }
                hs.task_off[f.slot0 + i] = (uint32_t)depth;
            }
        });
    }
    uint32_t acc = 0;  // depths -> first task of each slot
    for (uint32_t s = 0; s < hs.n_slots; ++s) {
        const uint32_t depth = hs.task_off[s];
        hs.task_off[s] = acc;
        acc += 1u << depth;
    }
    hs.task_off[hs.n_slots] = acc;
}

// CTAs per SM of the paint composite: its blends wait on L2 round trips, so
// more resident warps hide them (at the cost of shorter bands).
#ifndef RZ_PAINT_CTAS
#define RZ_PAINT_CTAS 3
#endif

int choose_band_rows(int canvas_w, int canvas_h, bool paint_mode, int num_sms) {
    const int stride = rz::band_stride(canvas_w);
    const int per_row = 4 * stride;  // the coverage band (colours stay in the canvas)
    // coverage only: tall bands (one CTA per SM) amortise a line's per-band set-up; with paint, RZ_PAINT_CTAS
    // CTAs per SM
    const int budget = paint_mode ? 200 * 1024 / RZ_PAINT_CTAS : 208 * 1024;
    const int rmax = std::max(1, std::min(std::min(budget / per_row, 64), std::max(canvas_h, 1)));
    const int64_t slots = (int64_t)std::max(num_sms, 1) * (paint_mode ? RZ_PAINT_CTAS : 1);
    // the band kernel runs in waves of `slots` bands: the height whose waves cost least, counting each band's
    // rows plus a fixed share for the lines that cross its edges
    int best = rmax;
    int64_t best_cost = INT64_MAX;
    for (int r = rmax; r >= 1; --r) {
        const int64_t bands = (canvas_h + r - 1) / r;
        const int64_t cost = (bands + slots - 1) / slots * (r + 4);
        if (cost < best_cost) {
            best_cost = cost;
            best = r;
        }
    }
    return best;
}

// Adds one fill (its view, transform, paint, slots and bands) to `hs`.
void add_fill(HostScene& hs, uint32_t sub0, uint32_t sub1, int col0, int row0, int width, int height, int clip_width,
              const rzhost::Xf& tr, int rule, int paint) {
    if (width <= 0 || height <= 0) return;
    rz::FillDev f{};
    f.sub0 = sub0;
    f.sub1 = sub1;
    f.seg0 = hs.sub_off[sub0];
    f.seg1 = hs.sub_off[sub1];
    f.slot0 = hs.n_slots;
    f.col0 = col0;
    f.row0 = row0;
    f.width = width;
    f.height = height;
    f.clip_width = clip_width;
    f.rule = rule;
    f.paint = paint;
    std::memcpy(f.tr, tr.m, sizeof(f.tr));
    f.band0 = row0 / hs.band_rows;
    f.nbands = (row0 + height - 1) / hs.band_rows - f.band0 + 1;
    f.entry0 = hs.n_entries;
    hs.n_slots += (f.seg1 - f.seg0) + (sub1 - sub0);
    hs.n_entries += (uint32_t)f.nbands;
    hs.max_clip = std::max(hs.max_clip, clip_width);
    hs.fills.push_back(f);
}

// Flatten + bin on the device (pipeline steps 1-5): every fill's lines, the
// per-(fill, band) counts and starts, and the band lists.  `leaf` (device,
// may be null) receives each line's segment and tree node.
// speculative: the lines and lists go into the buffers as they are and the
// counts stay on the device (no host round trip between the passes); a
// buffer too small shows as RZ_ERR_CAPACITY once the composite has run, and
// the caller then sizes the buffers from the device counts and runs again.
rz_status build_lines(rz_ctx* ctx, HostScene& hs, rz::SceneDev& S, Trace& tr, DevBuf* leaf,
                      bool speculative = false) {
    if (!hs.n_dev_fills) {
        RZ_CUDA(ctx->p_fills.ensure(hs.fills.size() * sizeof(rz::FillDev)));
        RZ_CUDA(cudaMemcpyAsync(ctx->p_fills.p, hs.fills.data(), hs.fills.size() * sizeof(rz::FillDev),
                                cudaMemcpyHostToDevice, ctx->stream));
    }
    S.fills = (const rz::FillDev*)ctx->p_fills.p;
    // 1) lines per slot, 2) offsets (one extra element receives the total)
    if (!hs.task_off.empty()) {
        RZ_CUDA(ctx->p_tasks.ensure(hs.task_off.size() * 4));
        RZ_CUDA(cudaMemcpyAsync(ctx->p_tasks.p, hs.task_off.data(), hs.task_off.size() * 4, cudaMemcpyHostToDevice,
                                ctx->stream));
        S.task_off = (const uint32_t*)ctx->p_tasks.p;
        S.n_tasks = hs.task_off.back();
    }
    const uint64_t ns = rz::scene_tasks(S) + 1;
    RZ_CUDA(ctx->p_slots.ensure(ns * 4));
    S.slot_count = (uint32_t*)ctx->p_slots.p;
    RZ_CUDA(cudaMemsetAsync(S.slot_count, 0, ns * 4, ctx->stream));
    tr.gpu_mark(ctx->stream, "upload");
    RZ_CUDA(rz::launch_flatten_count(S, ctx->stream));
    tr.gpu_mark(ctx->stream, "flatten_count");
    const uint64_t ne = (uint64_t)hs.n_entries + 1;
    RZ_CUDA(ctx->p_scan.ensure(rz::scan_temp_words(std::max(ns, ne)) * 4 + 64));
    RZ_CUDA(rz::scan_u32(S.slot_count, ns, (uint32_t*)ctx->p_scan.p, ctx->stream));
    if (speculative) {
        constexpr size_t kMinLines = 1u << 16;
        RZ_CUDA(ctx->p_lines.ensure(kMinLines * 2 * sizeof(int4)));
        const uint64_t cap = std::min<uint64_t>(ctx->p_lines.cap / (2 * sizeof(int4)), 0xffffffffull);
        S.line_cap = (uint32_t)cap;
        S.n_lines = (uint32_t)cap;  // launch bound; the count is read on the device
        S.n_lines_dev = S.slot_count + (ns - 1);
    } else {
        uint32_t n_lines = 0;
        RZ_CUDA(cudaMemcpyAsync(&n_lines, S.slot_count + (ns - 1), 4, cudaMemcpyDeviceToHost, ctx->stream));
        RZ_CUDA(cudaStreamSynchronize(ctx->stream));
        rz_status st = read_error(ctx);
        if (st) return st;
        if (leaf) {
            RZ_CUDA(leaf->ensure((uint64_t)std::max(n_lines, 1u) * sizeof(uint2)));
            S.leaf = (uint2*)leaf->p;
        }
        S.n_lines = n_lines;
        S.line_cap = n_lines;
        RZ_CUDA(ctx->p_lines.ensure((uint64_t)std::max(n_lines, 1u) * 2 * sizeof(int4)));
    }
    // 3) lines + per-(fill, band) counts
    S.lines = (int4*)ctx->p_lines.p;
    RZ_CUDA(ctx->p_ecount.ensure(ne * 4));
    RZ_CUDA(ctx->p_estart.ensure(ne * 4));
    RZ_CUDA(ctx->p_ecursor.ensure(ne * 4));
    S.entry_count = (uint32_t*)ctx->p_ecount.p;
    S.entry_start = (uint32_t*)ctx->p_estart.p;
    S.entry_cursor = (uint32_t*)ctx->p_ecursor.p;
    RZ_CUDA(cudaMemsetAsync(S.entry_count, 0, ne * 4, ctx->stream));
    RZ_CUDA(cudaMemsetAsync(S.entry_cursor, 0, ne * 4, ctx->stream));
    RZ_CUDA(rz::launch_flatten_emit(S, ctx->stream));
    tr.gpu_mark(ctx->stream, "flatten_emit");
    // 4) list starts per (fill, band)
    RZ_CUDA(cudaMemcpyAsync(S.entry_start, S.entry_count, ne * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    RZ_CUDA(rz::scan_u32(S.entry_start, ne, (uint32_t*)ctx->p_scan.p, ctx->stream));
    if (speculative) {
        constexpr size_t kMinPairs = 1u << 18;
        RZ_CUDA(ctx->p_pairs.ensure(kMinPairs * 4));
    } else {
        uint32_t n_pairs = 0;
        RZ_CUDA(cudaMemcpyAsync(&n_pairs, S.entry_start + hs.n_entries, 4, cudaMemcpyDeviceToHost, ctx->stream));
        RZ_CUDA(cudaStreamSynchronize(ctx->stream));
        RZ_CUDA(ctx->p_pairs.ensure((uint64_t)std::max(n_pairs, 1u) * 4));
    }
    // 5) line lists
    S.pairs = (uint32_t*)ctx->p_pairs.p;
    S.pair_cap = (uint32_t)std::min<uint64_t>(ctx->p_pairs.cap / 4, 0xffffffffull);
    tr.gpu_mark(ctx->stream, "entry_scan");
    RZ_CUDA(rz::launch_bin_scatter(S, ctx->stream));
    tr.gpu_mark(ctx->stream, "bin_scatter");
    return RZ_OK;
}

// After a speculative pass that ran out of room: the buffers sized from the
// device's counts (the lines' total and the lists' total).
rz_status grow_line_buffers(rz_ctx* ctx, const rz::SceneDev& S, uint32_t n_entries) {
    uint32_t n_lines = 0, n_pairs = 0;
    RZ_CUDA(cudaMemcpyAsync(&n_lines, S.n_lines_dev, 4, cudaMemcpyDeviceToHost, ctx->stream));
    RZ_CUDA(cudaMemcpyAsync(&n_pairs, S.entry_start + n_entries, 4, cudaMemcpyDeviceToHost, ctx->stream));
    RZ_CUDA(cudaStreamSynchronize(ctx->stream));
    RZ_CUDA(ctx->p_lines.ensure((uint64_t)std::max(n_lines, 1u) * 2 * sizeof(int4)));
    RZ_CUDA(ctx->p_pairs.ensure((uint64_t)std::max(n_pairs, 1u) * 4));
    return RZ_OK;
}

// Flatten + bin + composite on the device.  canvas: device buffer (RGBA
// pixels when paints are given, else an f32 mask), stride in pixels.
#ifndef RZ_SMALL_LEAF_SHIFT
#define RZ_SMALL_LEAF_SHIFT 1
#endif

// A mask of one small fill (at most ~64 K lines expected, times its bands at most ~8 M): every band
// reading every line costs less than the offsets scan, the per-band counts and lists and their launches.
bool small_scene(const HostScene& hs, const rz::SceneDev& S) {
    if (hs.fills.size() != 1) return false;
    const uint64_t tasks = hs.task_off.empty() ? ((uint64_t)hs.n_slots << hs.task_depth) : hs.task_off.back();
    const uint64_t est_lines = 8 * tasks;  // subtree tasks are sized to about 8 leaves each
    if (est_lines > (1u << 16) || est_lines * (uint64_t)S.n_bands > (1u << 23)) return false;
    // a slot at the task cap (1024) may have a tree far deeper than the estimate
    for (size_t s = 0; s + 1 < hs.task_off.size(); ++s)
        if (hs.task_off[s + 1] - hs.task_off[s] >= 1024u) return false;
    return true;
}

// The small-scene route: one pass flattens every task into lines it reserves on a device counter, then the
// composite gives every band every line.  RZ_ERR_CAPACITY: the trees were deeper than the estimate and there
// were more lines than the route takes (the composite then returns at once); the caller takes the binned
// pipeline instead (every band reading every line of a large scene would cost lines x bands).
rz_status run_small(rz_ctx* ctx, HostScene& hs, rz::SceneDev& S, int cov_stride, int smem, Trace& tr) {
    RZ_CUDA(ctx->p_fills.ensure(hs.fills.size() * sizeof(rz::FillDev)));
    RZ_CUDA(cudaMemcpyAsync(ctx->p_fills.p, hs.fills.data(), hs.fills.size() * sizeof(rz::FillDev),
                            cudaMemcpyHostToDevice, ctx->stream));
    S.fills = (const rz::FillDev*)ctx->p_fills.p;
    if (!hs.task_off.empty()) {
        RZ_CUDA(ctx->p_tasks.ensure(hs.task_off.size() * 4));
        RZ_CUDA(cudaMemcpyAsync(ctx->p_tasks.p, hs.task_off.data(), hs.task_off.size() * 4, cudaMemcpyHostToDevice,
                                ctx->stream));
        S.task_off = (const uint32_t*)ctx->p_tasks.p;
        S.n_tasks = hs.task_off.back();
    }
    uint32_t* counter = (uint32_t*)ctx->d_ctrl.p + 15;  // zeroed with the control words
    // at most this many lines: beyond it every band reading every line costs more than the binned pipeline
    constexpr size_t kSmallLines = 1u << 16;
    RZ_CUDA(ctx->p_lines.ensure(kSmallLines * 2 * sizeof(int4)));
    const uint64_t cap = kSmallLines;
    S.lines = (int4*)ctx->p_lines.p;
    S.line_cap = (uint32_t)cap;
    S.n_lines = (uint32_t)cap;
    S.n_lines_dev = counter;
    S.pairs = nullptr;  // every band takes every line
    tr.gpu_mark(ctx->stream, "upload");
    RZ_CUDA(rz::launch_flatten_emit_alloc(S, counter, ctx->stream));
    tr.gpu_mark(ctx->stream, "flatten_emit_alloc");
    RZ_CUDA(rz::launch_composite(S, cov_stride, smem, ctx->stream));
    tr.gpu_mark(ctx->stream, "composite");
    return read_error(ctx);
}

rz_status run_pipeline(rz_ctx* ctx, HostScene& hs, double flatness, float* canvas, int64_t canvas_stride, int canvas_w,
                       int canvas_h, const float* bg_dev, bool load_canvas, uint32_t* rgba8 = nullptr) {
    Trace tr("pipeline");
    const bool paint_mode = !hs.paints.empty();
    rz::SceneDev S{};
    S.kind = (const uint8_t*)ctx->d_kind.p;
    S.pts = (const double*)ctx->d_pts.p;
    S.sub_off = (const uint32_t*)ctx->d_sub.p;
    S.n_fills = (uint32_t)hs.fills.size();
    S.n_slots = hs.n_slots;
    S.n_segments = hs.n_seg;
    S.n_subpaths = hs.n_sub;
    S.task_depth = hs.task_depth;
    S.thr64 = 16.0 * flatness * flatness;
    S.thr32 = (float)S.thr64;
    S.canvas_w = canvas_w;
    S.canvas_h = canvas_h;
    S.band_rows = hs.band_rows;
    S.n_bands = (canvas_h + hs.band_rows - 1) / hs.band_rows;
    S.canvas = canvas;
    S.canvas_stride = canvas_stride;
    S.bg = bg_dev;
    S.load_canvas = load_canvas ? 1 : 0;
    S.rgba8 = rgba8;
    RZ_CUDA(ctx->d_ctrl.ensure(64));
    RZ_CUDA(cudaMemsetAsync(ctx->d_ctrl.p, 0, 64, ctx->stream));
    S.err = (int32_t*)ctx->d_ctrl.p;
    S.counters = (int32_t*)ctx->d_ctrl.p + 4;
    if (S.n_bands == 0) return read_error(ctx);
    int cov_stride = 0;
    const int smem = rz::composite_smem_bytes(canvas_w, hs.band_rows, hs.max_clip, paint_mode, &cov_stride);
    if (S.n_fills == 0) {
        // nothing to draw: the composite still writes the background
        if (paint_mode) {
            RZ_CUDA(ctx->p_paints.ensure(sizeof(rz::PaintDev)));
            S.paints = (const rz::PaintDev*)ctx->p_paints.p;
            RZ_CUDA(rz::launch_composite(S, cov_stride, smem, ctx->stream));
        }
        return read_error(ctx);
    }
    if (paint_mode) {
        RZ_CUDA(ctx->p_paints.ensure(hs.paints.size() * sizeof(rz::PaintDev)));
        RZ_CUDA(cudaMemcpyAsync(ctx->p_paints.p, hs.paints.data(), hs.paints.size() * sizeof(rz::PaintDev),
                                cudaMemcpyHostToDevice, ctx->stream));
        S.paints = (const rz::PaintDev*)ctx->p_paints.p;
    }
    if (!paint_mode && !load_canvas && small_scene(hs, S)) {
        // a few thousand tasks fill a fraction of the SMs: shorter tasks, more of them, cut the longest walk
        if (!hs.task_off.empty()) adaptive_tasks(hs, flatness, RZ_SMALL_LEAF_SHIFT);
        rz::SceneDev S1 = S;
        rz_status st = run_small(ctx, hs, S1, cov_stride, smem, tr);
        if (st != RZ_ERR_CAPACITY) return st;
        // more lines than the estimate: the binned pipeline below, over a cleared mask (its composite leaves
        // bands without lines untouched)
        RZ_CUDA(cudaMemset2DAsync(canvas, (size_t)canvas_stride * 4, 0, (size_t)canvas_w * 4, (size_t)canvas_h,
                                  ctx->stream));
        RZ_CUDA(cudaMemsetAsync(ctx->d_ctrl.p, 0, 64, ctx->stream));
        ctx->last_error.clear();
    }
    // the composite writes every pixel from bg (or leaves untouched mask bands zero): a pass
    // that ran out of list room can run again; over a loaded canvas the buffers are sized first
    const bool speculative = !load_canvas;
    rz::SceneDev S0 = S;
    rz_status st = build_lines(ctx, hs, S, tr, nullptr, speculative);
    if (st) return st;
    // 6) composite
    RZ_CUDA(rz::launch_composite(S, cov_stride, smem, ctx->stream));
    tr.gpu_mark(ctx->stream, "composite");
    st = read_error(ctx);
    if (st == RZ_ERR_CAPACITY && speculative) {
        st = grow_line_buffers(ctx, S, hs.n_entries);
        if (st) return st;
        S = S0;
        RZ_CUDA(cudaMemsetAsync(ctx->d_ctrl.p, 0, 64, ctx->stream));
        ctx->last_error.clear();
        st = build_lines(ctx, hs, S, tr, nullptr, false);
        if (st) return st;
        RZ_CUDA(rz::launch_composite(S, cov_stride, smem, ctx->stream));
        st = read_error(ctx);
    }
    return st;
}

// Segments of `hs` staged into the context's device buffers (arcs expanded).
rz_status stage_scene_segments(rz_ctx* ctx, const uint8_t* kind, const double* pts, uint32_t n_seg,
                               const uint32_t* sub_off, uint32_t n_sub, const uint32_t* fill_sub, uint32_t n_fills,
                               HostScene& hs, std::vector<uint32_t>& fill_sub_out, Trace* trace = nullptr) {
    rz::BatchDev b{};
    rz_status st =
        stage_host(ctx, kind, pts, n_seg, sub_off, n_sub, fill_sub, n_fills, nullptr, nullptr, b, nullptr, nullptr, trace);
    if (st) return st;
    if (ctx->expanded) {
        hs.kind = ctx->x_kind.data();
        hs.pts = ctx->x_pts.data();
        hs.sub_off = ctx->x_sub.data();
        hs.n_seg = (uint32_t)ctx->x_kind.size();
        hs.n_sub = (uint32_t)ctx->x_sub.size() - 1;
        fill_sub_out = ctx->x_psub;
    } else {
        hs.kind = kind;
        hs.pts = pts;
        hs.sub_off = sub_off;
        hs.n_seg = n_seg;
        hs.n_sub = n_sub;
        fill_sub_out.assign(fill_sub, fill_sub + n_fills + 1);
    }
    return RZ_OK;
}

// Device bytes to host memory: directly when `dst` is page-locked, else through
// the page-locked staging buffer and a parallel host copy.  Synchronises.
rz_status copy_out_bytes(rz_ctx* ctx, void* dst, const void* src_dev, uint64_t bytes) {
    if (mapped_host(dst)) {
        RZ_CUDA(cudaMemcpyAsync(dst, src_dev, bytes, cudaMemcpyDeviceToHost, ctx->stream));
        RZ_CUDA(cudaStreamSynchronize(ctx->stream));
        return RZ_OK;
    }
    RZ_CUDA(ctx->h_out.ensure(bytes));
    RZ_CUDA(cudaMemcpyAsync(ctx->h_out.p, src_dev, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    RZ_CUDA(cudaStreamSynchronize(ctx->stream));
    const char* src = (const char*)ctx->h_out.p;
    const int64_t chunks = (int64_t)((bytes + (1u << 20) - 1) >> 20);
    parallel_for(chunks, 4, [&](int64_t c0, int64_t c1) {
        const uint64_t b0 = (uint64_t)c0 << 20, b1 = std::min<uint64_t>((uint64_t)c1 << 20, bytes);
        std::memcpy((char*)dst + b0, src + b0, b1 - b0);
    });
    return RZ_OK;
}

// Renders one large path as a mask with the line pipeline (mask semantics).
rz_status mask_pipeline(rz_ctx* ctx, const rz_path* path, const double tr[6], int32_t rule, double flatness,
                        uint64_t width, uint64_t height) {
    Trace trc("mask_pipeline host");
    HostScene hs;
    std::vector<uint32_t> fsub;
    const uint32_t psub[2] = {0, path->n_subpaths};
    rz_status st = stage_scene_segments(ctx, path->seg_kind, path->seg_pts, path->n_segments, path->subpath_off,
                                        path->n_subpaths, psub, 1, hs, fsub, &trc);
    if (st) return st;
    hs.band_rows = choose_band_rows((int)width, (int)height, false, ctx->num_sms);
    rzhost::Xf t;
    std::memcpy(t.m, tr, sizeof(t.m));
    add_fill(hs, fsub[0], fsub[1], 0, 0, (int)width, (int)height, (int)width - 1, t, rule, -1);
    adaptive_tasks(hs, flatness);  // a path this large has long segments: subtree tasks by their depth
    trc.mark("tasks");
    RZ_CUDA(ctx->d_out.ensure(width * height * 4 + 16));
    RZ_CUDA(cudaMemsetAsync(ctx->d_out.p, 0, width * height * 4, ctx->stream));
    return run_pipeline(ctx, hs, flatness, (float*)ctx->d_out.p, (int64_t)width, (int)width, (int)height, nullptr,
                        false);
}

// Path::stroke of subpaths [sub0, sub1) of a host path that may hold arcs
// (expanded first, as PathBuilder::arc_to would have).  Appends the outline
// (segments and subpath ends relative to what it appends).
rz_status stroke_subpaths(const uint8_t* kind, const double* pts, const uint32_t* sub_off, const uint8_t* closed,
                          uint32_t sub0, uint32_t sub1, const rz_stroke_style& style, std::vector<uint8_t>& okind,
                          std::vector<double>& opts, std::vector<uint32_t>& oends) {
    if (!(style.width >= 0.0) || !std::isfinite(style.width) || std::isnan(style.miter_limit) ||
        style.line_join < RZ_JOIN_MITER || style.line_join > RZ_JOIN_ROUND || style.line_cap < RZ_CAP_BUTT ||
        style.line_cap > RZ_CAP_ROUND)
        return RZ_ERR_INVALID;
    const rzhost::Style st{style.width, style.line_join, style.line_cap, style.miter_limit};
    std::vector<uint8_t> k;
    std::vector<double> p;
    std::vector<uint32_t> so{0};
    std::vector<uint8_t> cl;
    for (uint32_t sp = sub0; sp < sub1; ++sp) {
        for (uint32_t i = sub_off[sp]; i < sub_off[sp + 1]; ++i) {
            if (kind[i] == RZ_SEG_ARC) {
                if (!rzhost::expand_arc(pts + 8ull * i, k, p)) return RZ_ERR_ARC;
            } else if (kind[i] <= RZ_SEG_CUBIC) {
                k.push_back(kind[i]);
                p.insert(p.end(), pts + 8ull * i, pts + 8ull * i + 8);
            } else {
                return RZ_ERR_INVALID;
            }
        }
        so.push_back((uint32_t)k.size());
        cl.push_back(closed ? closed[sp] : 0);
    }
    rzhost::stroke_path(k.data(), p.data(), so.data(), cl.data(), 0, (uint32_t)cl.size(), st, okind, opts, oends);
    return RZ_OK;
}

#include "rz_scene_tree.cpp.inc"

}  // namespace

extern "C" {

rz_status rz_fill(rz_ctx* ctx, const rz_path* path, const double tr[6], int32_t fill_rule, double flatness,
                  const rz_paint* paint, float* img, rz_shape shape) {
    if (!ctx) return RZ_ERR_INVALID;
    std::lock_guard<std::mutex> lock(ctx->mu);
    rz_status st = check_path(ctx, path);
    if (st) return st;
    if (!tr || !paint || !img) return fail(ctx, RZ_ERR_INVALID, "null argument");
    if (!valid_flatness(flatness)) return fail(ctx, RZ_ERR_INVALID, "flatness must be > 0 and finite");
    if (shape.width == 0 || shape.height == 0) return RZ_OK;
    if (shape.width > 16383 || shape.height > 16383) return fail(ctx, RZ_ERR_INVALID, "image too large");
    if (paint->n_stops > (uint32_t)rz::kMaxStops) return fail(ctx, RZ_ERR_INVALID, "more than 16 stops");
    RZ_CUDA(cudaSetDevice(ctx->device));
    HostScene hs;
    std::vector<uint32_t> fsub;
    const uint32_t psub[2] = {0, path->n_subpaths};
    st = stage_scene_segments(ctx, path->seg_kind, path->seg_pts, path->n_segments, path->subpath_off,
                              path->n_subpaths, psub, 1, hs, fsub);
    if (st) return st;
    const int W = (int)shape.width, H = (int)shape.height;
    hs.band_rows = choose_band_rows(W, H, true, ctx->num_sms);
    rzhost::Xf t;
    std::memcpy(t.m, tr, sizeof(t.m));
    rzhost::Box bb0{};
    const rzhost::Xf id{{1, 0, 0, 0, 1, 0}};
    const bool have = rzhost::path_bbox(hs.kind, hs.pts, hs.sub_off, fsub[0], fsub[1], id, bb0);
    hs.paints.resize(1);
    prepare_paint(*paint, t, have, bb0, hs.paints[0]);
    if (hs.paints[0].kind < 0) return RZ_OK;
    // mask_iter semantics: the view is the image, clip at its width
    add_fill(hs, fsub[0], fsub[1], 0, 0, W, H, W, t, fill_rule, 0);
    // dense device copy of the view, blended in place, copied back
    const size_t n = (size_t)W * H;
    RZ_CUDA(ctx->h_out.ensure(n * 16));
    float* h = (float*)ctx->h_out.p;
    parallel_for(H, 64, [&](int64_t y0, int64_t y1) {
        for (int64_t y = y0; y < y1; ++y)
            for (int x = 0; x < W; ++x)
                std::memcpy(h + 4 * ((size_t)y * W + x),
                            img + 4 * (shape.start + y * shape.row_stride + x * shape.col_stride), 16);
    });
    RZ_CUDA(ctx->p_canvas.ensure(n * 16));
    RZ_CUDA(cudaMemcpyAsync(ctx->p_canvas.p, h, n * 16, cudaMemcpyHostToDevice, ctx->stream));
    st = run_pipeline(ctx, hs, flatness, (float*)ctx->p_canvas.p, W, W, H, nullptr, true);
    if (st) return st;
    RZ_CUDA(cudaMemcpyAsync(h, ctx->p_canvas.p, n * 16, cudaMemcpyDeviceToHost, ctx->stream));
    RZ_CUDA(cudaStreamSynchronize(ctx->stream));
    parallel_for(H, 64, [&](int64_t y0, int64_t y1) {
        for (int64_t y = y0; y < y1; ++y)
            for (int x = 0; x < W; ++x)
                std::memcpy(img + 4 * (shape.start + y * shape.row_stride + x * shape.col_stride),
                            h + 4 * ((size_t)y * W + x), 16);
    });
    return RZ_OK;
}

// Scene::render into an RGBA f32 canvas, or (rgba8 non-null) straight into
// sRGB8 RGBA bytes with the encode fused into the composite's epilogue.
static rz_status render_scene_impl(rz_ctx* ctx, const rz_scene* scene, double flatness, const float bg[4],
                                   float* canvas, uint8_t* rgba8, uint32_t width, uint32_t height) {
    if (!ctx) return RZ_ERR_INVALID;
    std::lock_guard<std::mutex> lock(ctx->mu);
    if (!canvas && !rgba8) return fail(ctx, RZ_ERR_INVALID, "null argument");
    rz_status st0 = check_scene(ctx, scene, flatness, width, height);
    if (st0) return st0;
    const uint32_t F = scene->n_fills;
    RZ_CUDA(cudaSetDevice(ctx->device));
    Trace tr("rz_render_scene");
    HostScene hs;
    std::vector<uint32_t> fsub;
    rz_status st = stage_scene_segments(ctx, scene->seg_kind, scene->seg_pts, scene->n_segments, scene->subpath_off,
                                        scene->n_subpaths, scene->fill_subpath_off, F, hs, fsub);
    if (st) return st;
    tr.mark("stage_segments");
    const int W = (int)width, H = (int)height;
    hs.band_rows = choose_band_rows(W, H, true, ctx->num_sms);
    const rzhost::Xf id{{1, 0, 0, 0, 1, 0}};
    // tight bounding boxes of every fill (transformed; untransformed only for
    // BoundingBox paint units), computed in parallel
    std::vector<rzhost::Box> pbox(F), ubox(F);
    std::vector<uint8_t> have_p(F, 0), have_u(F, 0);
    parallel_for((int64_t)F, 8, [&](int64_t f0, int64_t f1) {
        for (int64_t f = f0; f < f1; ++f) {
            rzhost::Xf t = id;
            if (scene->transforms) std::memcpy(t.m, scene->transforms + 6ull * f, sizeof(t.m));
            have_p[f] = rzhost::path_bbox(hs.kind, hs.pts, hs.sub_off, fsub[f], fsub[f + 1], t, pbox[f]);
            if (have_p[f] && scene->paints[scene->fill_paint[f]].units == RZ_UNITS_BOUNDING_BOX)
                have_u[f] = rzhost::path_bbox(hs.kind, hs.pts, hs.sub_off, fsub[f], fsub[f + 1], id, ubox[f]);
        }
    });
    tr.mark("bbox");
    for (uint32_t f = 0; f < F; ++f) {
        rzhost::Xf t = id;
        if (scene->transforms) std::memcpy(t.m, scene->transforms + 6ull * f, sizeof(t.m));
        // Pipeline::build_rec Fill: bbox of the path, intersected with the view (src/scene.rs:288-298)
        if (!have_p[f]) continue;
        const rzhost::Box pb = pbox[f];
        const double vx1 = (double)W, vy1 = (double)H;
        if (0.0 > pb.x1 || pb.x0 > vx1 || 0.0 > pb.y1 || pb.y0 > vy1) continue;
        const rzhost::Box nb{std::fmax(0.0, pb.x0), std::fmax(0.0, pb.y0), std::fmin(vx1, pb.x1), std::fmin(vy1, pb.y1)};
        // render_rec Fill: the view of the layer and the align transform (src/scene.rs:407-430)
        long col_min = (long)std::floor(nb.x0), col_max = (long)std::ceil(nb.x1) + 1;
        long row_min = (long)std::floor(nb.y0), row_max = (long)std::ceil(nb.y1) + 1;
        if (col_min < 0) col_min = W;  // `as usize` wraps; view_shape clamps (src/image.rs:588-605)
        if (row_min < 0) row_min = H;
        if (col_max < 0) col_max = W;
        if (row_max < 0) row_max = H;
        row_min = std::min<long>(row_min, H);
        row_max = std::max(std::min<long>(row_max, H), row_min);
        col_min = std::min<long>(col_min, W);
        col_max = std::max(std::min<long>(col_max, W), col_min);
        const rzhost::Xf align{{1.0, 0.0, -std::floor(nb.x0), 0.0, 1.0, -std::floor(nb.y0)}};
        const rzhost::Xf tr_fill = rzhost::xf_mul(align, t);
        const int vw = (int)(col_max - col_min), vh = (int)(row_max - row_min);
        if (vw <= 0 || vh <= 0) continue;
        rz::PaintDev pd;
        prepare_paint(scene->paints[scene->fill_paint[f]], tr_fill, have_u[f] != 0, ubox[f], pd);
        if (pd.kind < 0) continue;
        hs.paints.push_back(pd);
        const int rule = scene->fill_rules ? scene->fill_rules[f] : 0;
        add_fill(hs, fsub[f], fsub[f + 1], (int)col_min, (int)row_min, vw, vh, vw, tr_fill, rule,
                 (int)hs.paints.size() - 1);
    }
    if (hs.paints.empty()) hs.paints.resize(1);  // paint mode even with nothing to draw
    tr.mark("fills");
    const size_t n = (size_t)W * H;
    RZ_CUDA(ctx->p_canvas.ensure(n * 16 + 16));
    RZ_CUDA(ctx->d_counts.ensure(64));
    float bgv[4] = {0.f, 0.f, 0.f, 0.f};
    if (bg) std::memcpy(bgv, bg, sizeof(bgv));
    RZ_CUDA(cudaMemcpyAsync(ctx->d_counts.p, bgv, 16, cudaMemcpyHostToDevice, ctx->stream));
    if (rgba8) {
        RZ_CUDA(ctx->p_rgba8.ensure(n * 4 + 16));
        st = run_pipeline(ctx, hs, flatness, (float*)ctx->p_canvas.p, W, W, H, (const float*)ctx->d_counts.p, false,
                          (uint32_t*)ctx->p_rgba8.p);
        if (st) return st;
        tr.mark("pipeline");
        st = copy_out_bytes(ctx, rgba8, ctx->p_rgba8.p, n * 4);
        tr.mark("copy_out");
        return st;
    }
    st = run_pipeline(ctx, hs, flatness, (float*)ctx->p_canvas.p, W, W, H, (const float*)ctx->d_counts.p, false);
    if (st) return st;
    tr.mark("pipeline");
    if (mapped_host(canvas)) {
        RZ_CUDA(cudaMemcpyAsync(canvas, ctx->p_canvas.p, n * 16, cudaMemcpyDeviceToHost, ctx->stream));
        RZ_CUDA(cudaStreamSynchronize(ctx->stream));
    } else {
        // pageable canvas: page-locked staging, then a parallel host copy
        RZ_CUDA(ctx->h_out.ensure(n * 16));
        RZ_CUDA(cudaMemcpyAsync(ctx->h_out.p, ctx->p_canvas.p, n * 16, cudaMemcpyDeviceToHost, ctx->stream));
        RZ_CUDA(cudaStreamSynchronize(ctx->stream));
        const char* src = (const char*)ctx->h_out.p;
        parallel_for((int64_t)H, 16, [&](int64_t y0, int64_t y1) {
            std::memcpy((char*)canvas + (size_t)y0 * W * 16, src + (size_t)y0 * W * 16, (size_t)(y1 - y0) * W * 16);
        });
    }
    tr.mark("copy_out");
    return RZ_OK;
}

rz_status rz_render_scene(rz_ctx* ctx, const rz_scene* scene, double flatness, const float bg[4], float* canvas,
                          uint32_t width, uint32_t height) {
    if (ctx && !canvas) return fail(ctx, RZ_ERR_INVALID, "null argument");
    return render_scene_impl(ctx, scene, flatness, bg, canvas, nullptr, width, height);
}

rz_status rz_render_scene_rgba8(rz_ctx* ctx, const rz_scene* scene, double flatness, const float bg[4],
                                uint8_t* rgba8, uint32_t width, uint32_t height) {
    if (ctx && !rgba8) return fail(ctx, RZ_ERR_INVALID, "null argument");
    return render_scene_impl(ctx, scene, flatness, bg, nullptr, rgba8, width, height);
}

rz_status rz_stroke_path(const rz_path* path, const rz_stroke_style* style, uint8_t* seg_kind, double* seg_pts,
                         uint32_t seg_cap, uint32_t* subpath_off, uint32_t sub_cap, uint32_t* n_segments,
                         uint32_t* n_subpaths) {
    if (!path || !style || !n_segments || !n_subpaths) return RZ_ERR_INVALID;
    if (path->n_segments && (!path->seg_kind || !path->seg_pts)) return RZ_ERR_INVALID;
    if (!path->subpath_off || path->subpath_off[path->n_subpaths] > path->n_segments) return RZ_ERR_INVALID;
    for (uint32_t i = 0; i < path->n_subpaths; ++i)
        if (path->subpath_off[i] > path->subpath_off[i + 1]) return RZ_ERR_INVALID;
    std::vector<uint8_t> okind;
    std::vector<double> opts;
    std::vector<uint32_t> oends;
    const rz_status st = stroke_subpaths(path->seg_kind, path->seg_pts, path->subpath_off, path->closed, 0,
                                         path->n_subpaths, *style, okind, opts, oends);
    if (st) return st;
    *n_segments = (uint32_t)okind.size();
    *n_subpaths = (uint32_t)oends.size();
    if (!seg_kind && !seg_pts && !subpath_off) return RZ_OK;
    if (seg_cap < okind.size() || sub_cap < oends.size() + 1 || !seg_kind || !seg_pts || !subpath_off)
        return RZ_ERR_CAPACITY;
    std::memcpy(seg_kind, okind.data(), okind.size());
    std::memcpy(seg_pts, opts.data(), opts.size() * sizeof(double));
    subpath_off[0] = 0;
    for (size_t i = 0; i < oends.size(); ++i) subpath_off[i + 1] = oends[i];
    return RZ_OK;
}

rz_status rz_write_image(const uint8_t* rgba8, uint32_t width, uint32_t height, int32_t format, uint8_t* out,
                         uint64_t cap, uint64_t* len) {
    if (!len || (!rgba8 && (uint64_t)width * height)) return RZ_ERR_INVALID;
    const uint64_t npx = (uint64_t)width * height;
    char ppm_head[64];
    int ppm_len = 0;
    uint64_t need = 0;
    switch (format) {
        case RZ_IMAGE_BMP:
            if (npx * 4 + 122 > 0xffffffffull) return RZ_ERR_INVALID;  // sizes are u32 in the header
            need = 122 + npx * 4;
            break;
        case RZ_IMAGE_RGBA: need = 8 + npx * 4; break;
        case RZ_IMAGE_PPM:
            ppm_len = std::snprintf(ppm_head, sizeof(ppm_head), "P6 %u %u 255 ", width, height);
            need = (uint64_t)ppm_len + npx * 3;
            break;
        default: return RZ_ERR_INVALID;
    }
    *len = need;
    if (!out) return RZ_OK;
    if (cap < need) return RZ_ERR_CAPACITY;
    uint8_t* o = out;
    auto u32 = [&o](uint32_t v) {
        for (int i = 0; i < 4; ++i) *o++ = (uint8_t)(v >> (8 * i));
    };
    if (format == RZ_IMAGE_BMP) {
        // Image::write_bmp (src/image.rs:165-212): file header, BITMAPV4HEADER with
        // bit fields and the sRGB colour space, rows bottom-up, 4 bytes a pixel
        const uint32_t data = (uint32_t)(npx * 4), off = 14 + 108;
        *o++ = 'B';
        *o++ = 'M';
        u32(data + off);
        u32(0);
        u32(off);
        u32(108);
        u32(width);
        u32(height);
        u32(0x00200001u);  // 1 plane, 32 bits per pixel
        u32(3);            // BI_BITFIELDS
        u32(data);
        u32(2835);  // 72 dpi, both directions
        u32(2835);
        u32(0);
        u32(0);
        u32(0x000000ffu);  // the four channel masks, in the reference's order
        u32(0x0000ff00u);
        u32(0x00ff0000u);
        u32(0xff000000u);
        u32(0x73524742u);  // 'sRGB'
        std::memset(o, 0, 48);
        o += 48;
        for (uint32_t r = height; r-- > 0;) {
            std::memcpy(o, rgba8 + (uint64_t)r * width * 4, (size_t)width * 4);
            o += (size_t)width * 4;
        }
    } else if (format == RZ_IMAGE_RGBA) {
        // Image::write_rgba (src/image.rs:136-149): height, width, pixels
        u32(height);
        u32(width);
        std::memcpy(o, rgba8, npx * 4);
    } else {
        // Image::write_ppm (src/image.rs:151-163): the alpha byte is dropped
        std::memcpy(o, ppm_head, (size_t)ppm_len);
        o += ppm_len;
        for (uint64_t i = 0; i < npx; ++i) {
            *o++ = rgba8[4 * i];
            *o++ = rgba8[4 * i + 1];
            *o++ = rgba8[4 * i + 2];
        }
    }
    return RZ_OK;
}

rz_status rz_render_scene_tree(rz_ctx* ctx, const rz_scene* scene, const rz_scene_node* nodes, uint32_t n_nodes,
                               double flatness, const float bg[4], float* canvas, uint8_t* rgba8, uint32_t width,
                               uint32_t height) {
    if (!ctx) return RZ_ERR_INVALID;
    std::lock_guard<std::mutex> lock(ctx->mu);
    rz_status st = check_scene(ctx, scene, flatness, width, height);
    if (st) return st;
    if ((!nodes && n_nodes) || (!canvas && !rgba8)) return fail(ctx, RZ_ERR_INVALID, "null argument");
    RZ_CUDA(cudaSetDevice(ctx->device));
    Trace tr("rz_render_scene_tree");
    SceneTree T;
    T.sc = scene;
    T.nodes = nodes;
    T.n = n_nodes;
    T.end.assign(n_nodes, 0);
    if (n_nodes) {
        uint32_t e = 0;
        st = parse_tree(ctx, T, 0, 0, e);
        if (st) return st;
        if (e != n_nodes) return fail(ctx, RZ_ERR_INVALID, "scene tree: nodes after the root's subtree");
    }
    // the entry table; every Stroke node's outline becomes one more entry,
    // appended after the fills' subpaths
    const uint32_t F = scene->n_fills;
    T.E.resize(F);
    for (uint32_t f = 0; f < F; ++f) {
        T.E[f].own = kIdentity;
        if (scene->transforms) std::memcpy(T.E[f].own.m, scene->transforms + 6ull * f, sizeof(T.E[f].own.m));
        T.E[f].rule = scene->fill_rules ? scene->fill_rules[f] : 0;
        T.E[f].paint = scene->fill_paint[f];
    }
    T.stroke_of.assign(n_nodes, 0);
    st = stage_scene_segments(ctx, scene->seg_kind, scene->seg_pts, scene->n_segments, scene->subpath_off,
                              scene->n_subpaths, scene->fill_subpath_off, F, T.base, T.fsub);
    if (st) return st;
    bool strokes = false;
    for (uint32_t i = 0; i < n_nodes; ++i) strokes = strokes || nodes[i].kind == RZ_NODE_STROKE;
    if (strokes) st = stroke_on_device(ctx, T, scene, nodes, n_nodes);
    if (st) return st;
    tr.mark("stage_segments");
    // Pipeline::build with view = the canvas, tr = identity (src/scene.rs:186-199)
    const int W = (int)width, H = (int)height;
    int root = -1;
    if (n_nodes) {
        precompute_bboxes(T);
        tr.mark("bboxes");
        root = build_rec(T, 0, OptBox{true, rzhost::Box{0.0, 0.0, (double)W, (double)H}}, kIdentity);
    }
    tr.mark("build");
    // the root layer is the view: Layer::new(view, bg)
    const uint64_t n = (uint64_t)W * (uint64_t)H;
    if (n == 0) return RZ_OK;
    RZ_CUDA(ctx->p_canvas.ensure(n * 16 + 16));
    TreePlan P;
    P.hs.kind = T.base.kind;
    P.hs.pts = T.base.pts;
    P.hs.sub_off = T.base.sub_off;
    P.hs.n_seg = T.base.n_seg;
    P.hs.n_sub = T.base.n_sub;
    P.hs.band_rows = choose_band_rows(W, H, true, ctx->num_sms);
    PlanLayer R;
    R.w = W;
    R.h = H;
    TreeOp init{};
    init.kind = TreeOp::kFillColor;
    init.w = W;
    init.h = H;
    if (bg) std::memcpy(init.color, bg, sizeof(init.color));
    P.ops.push_back(init);
    if (root >= 0) {
        plan_rec(T, P, root, R);
        plan_flush(P, R);
    }
    tr.mark("plan");
    float* const canvas_dev = (float*)ctx->p_canvas.p;
    st = run_plan(ctx, P, flatness, canvas_dev, W, H);
    if (st) return st;
    tr.mark("render");
    if (canvas) {
        st = copy_out_bytes(ctx, canvas, canvas_dev, n * 16);
        if (st) return st;
    }
    if (rgba8) {
        RZ_CUDA(ctx->p_rgba8.ensure(n * 4 + 16));
        RZ_CUDA(rz::launch_encode_rgba8(canvas_dev, (uint8_t*)ctx->p_rgba8.p, n, ctx->stream));
        st = copy_out_bytes(ctx, rgba8, ctx->p_rgba8.p, n * 4);
        if (st) return st;
    }
    tr.mark("copy_out");
    return read_error(ctx);
}

rz_status rz_encode_rgba8(rz_ctx* ctx, const float* canvas, uint64_t n_pixels, uint8_t* rgba8, int32_t memory) {
    if (!ctx) return RZ_ERR_INVALID;
    std::lock_guard<std::mutex> lock(ctx->mu);
    if (n_pixels == 0) return RZ_OK;
    if (!canvas || !rgba8) return fail(ctx, RZ_ERR_INVALID, "null argument");
    if (memory != RZ_MEM_HOST && memory != RZ_MEM_DEVICE) return fail(ctx, RZ_ERR_INVALID, "bad memory kind");
    if (n_pixels > (1ull << 36)) return fail(ctx, RZ_ERR_INVALID, "too many pixels");
    RZ_CUDA(cudaSetDevice(ctx->device));
    if (memory == RZ_MEM_DEVICE) {
        if (((uintptr_t)canvas & 15) || ((uintptr_t)rgba8 & 3))
            return fail(ctx, RZ_ERR_INVALID, "misaligned device buffer (canvas 16 bytes, rgba8 4 bytes)");
        RZ_CUDA(rz::launch_encode_rgba8(canvas, rgba8, n_pixels, ctx->stream));
        return RZ_OK;
    }
    RZ_CUDA(ctx->p_encode_in.ensure(n_pixels * 16 + 16));
    RZ_CUDA(ctx->p_rgba8.ensure(n_pixels * 4 + 16));
    RZ_CUDA(cudaMemcpyAsync(ctx->p_encode_in.p, canvas, n_pixels * 16, cudaMemcpyHostToDevice, ctx->stream));
    RZ_CUDA(rz::launch_encode_rgba8((const float*)ctx->p_encode_in.p, (uint8_t*)ctx->p_rgba8.p, n_pixels, ctx->stream));
    return copy_out_bytes(ctx, rgba8, ctx->p_rgba8.p, n_pixels * 4);
}

rz_status rz_encode_mask_rgba8(rz_ctx* ctx, const void* mask, int32_t elem_size, uint64_t n_pixels, uint8_t* rgba8,
                               int32_t memory) {
    if (!ctx) return RZ_ERR_INVALID;
    std::lock_guard<std::mutex> lock(ctx->mu);
    if (n_pixels == 0) return RZ_OK;
    if (!mask || !rgba8) return fail(ctx, RZ_ERR_INVALID, "null argument");
    if (elem_size != 4 && elem_size != 8) return fail(ctx, RZ_ERR_INVALID, "elem_size must be 4 or 8");
    if (memory != RZ_MEM_HOST && memory != RZ_MEM_DEVICE) return fail(ctx, RZ_ERR_INVALID, "bad memory kind");
    if (n_pixels > (1ull << 36)) return fail(ctx, RZ_ERR_INVALID, "too many pixels");
    RZ_CUDA(cudaSetDevice(ctx->device));
    if (memory == RZ_MEM_DEVICE) {
        if (((uintptr_t)mask & (uintptr_t)(elem_size - 1)) || ((uintptr_t)rgba8 & 3))
            return fail(ctx, RZ_ERR_INVALID, "misaligned device buffer");
        RZ_CUDA(rz::launch_encode_mask_rgba8(mask, elem_size, rgba8, n_pixels, ctx->stream));
        return RZ_OK;
    }
    RZ_CUDA(ctx->p_encode_in.ensure(n_pixels * (uint64_t)elem_size + 16));
    RZ_CUDA(ctx->p_rgba8.ensure(n_pixels * 4 + 16));
    RZ_CUDA(cudaMemcpyAsync(ctx->p_encode_in.p, mask, n_pixels * (uint64_t)elem_size, cudaMemcpyHostToDevice,
                            ctx->stream));
    RZ_CUDA(rz::launch_encode_mask_rgba8(ctx->p_encode_in.p, elem_size, (uint8_t*)ctx->p_rgba8.p, n_pixels,
                                         ctx->stream));
    return copy_out_bytes(ctx, rgba8, ctx->p_rgba8.p, n_pixels * 4);
}

}  // extern "C"

#include "rz_diff_api.cpp.inc"

// ---------------------------------------------------------------------------
// Batch autotuner
// ---------------------------------------------------------------------------
namespace {

// The tuner's candidates for the glyph pipeline: band-height cap (the work
// item's shape) x resident cover CTAs per SM, each timed as one full pass
// (records, walk, scan, emit, cover) on the caller's batch; median of 3
// after a warm-up.
rz_status tune_glyph(rz_ctx* ctx, const std::vector<rz::MaskDev>& masks, rz::BatchDev b, rz_tune_result* result) {
    const uint32_t P = (uint32_t)masks.size();
    const int occ = std::max(1, rz::glyph_cover_occupancy());
    const int caps[5] = {16, 32, 64, 128, 256};
    const int saved_cap = ctx->tune_rows_cap, saved_ctas = ctx->tune_ctas;
    std::memset(result, 0, sizeof(*result));
    result->ms = 1e30f;
    Items items;
    build_items(masks, false, items, 256, rz::kGlyphBandFloats);
    rz_status st = stage_plan(ctx, masks, items, b);
    if (st) return st;
    b.n_paths = P;
    rz::GlyphDev g{};
    RZ_CUDA(glyph_setup(b, g, ctx->g_recs, ctx->g_coef, ctx->g_chain, ctx->g_code, ctx->g_pflags, ctx->g_vtx,
                        ctx->g_scan, ctx->g_paths, ctx->stream));
    cudaEvent_t e0, e1;
    RZ_CUDA(cudaEventCreate(&e0));
    RZ_CUDA(cudaEventCreate(&e1));
    int32_t* queue = (int32_t*)ctx->d_ctrl.p + 8;
    for (int ci = 0; ci < 5 && st == RZ_OK; ++ci) {
        build_items(masks, false, items, caps[ci], rz::kGlyphBandFloats);
        const int n = (int)items.items.size();
        if (ctx->d_items.ensure(std::max(n, 1) * sizeof(rz::WorkItem)) != cudaSuccess ||
            cudaMemcpyAsync(ctx->d_items.p, items.items.data(), n * sizeof(rz::WorkItem), cudaMemcpyHostToDevice,
                            ctx->stream) != cudaSuccess) {
            st = RZ_ERR_CUDA;
            break;
        }
        for (int per_sm = occ; per_sm >= std::max(1, occ - 2) && st == RZ_OK; --per_sm) {
            const int grid = std::max(1, std::min(n, ctx->num_sms * per_sm));
            float t[3] = {0.f, 0.f, 0.f};
            for (int rep = 0; rep < 4 && st == RZ_OK; ++rep) {
                cudaError_t e = cudaEventRecord(e0, ctx->stream);
                if (e == cudaSuccess) e = glyph_enqueue_flatten(g, (uint32_t*)ctx->g_scan.p, P, ctx->stream);
                if (e == cudaSuccess) e = cudaMemsetAsync(queue, 0, 4, ctx->stream);
                if (e == cudaSuccess)
                    e = rz::launch_glyph_cover(g, (const rz::WorkItem*)ctx->d_items.p, n, queue, grid, ctx->stream);
                if (e == cudaSuccess) e = cudaEventRecord(e1, ctx->stream);
                if (e == cudaSuccess) e = cudaEventSynchronize(e1);
                if (e != cudaSuccess) {
                    st = RZ_ERR_CUDA;
                    break;
                }
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (rep > 0) t[rep - 1] = ms;  // the first launch warms up
            }
            if (st) break;
            st = read_error(ctx);
            if (st) break;
            std::sort(t, t + 3);
            if (result->n_entries < 24)
                result->entries[result->n_entries++] = rz_tune_entry{caps[ci], per_sm, t[1], rz::kWalkSlotsDefault};
            if (t[1] < result->ms) {
                result->ms = t[1];
                result->band_rows_cap = caps[ci];
                result->ctas_per_sm = per_sm;
            }
        }
    }
    // slots per lane of the tree walk (32 times that per warp), at the chosen band shape
    result->walk_slots = rz::kWalkSlotsDefault;
    if (st == RZ_OK) {
        build_items(masks, false, items, result->band_rows_cap, rz::kGlyphBandFloats);
        const int n = (int)items.items.size();
        if (ctx->d_items.ensure(std::max(n, 1) * sizeof(rz::WorkItem)) != cudaSuccess ||
            cudaMemcpyAsync(ctx->d_items.p, items.items.data(), n * sizeof(rz::WorkItem), cudaMemcpyHostToDevice,
                            ctx->stream) != cudaSuccess)
            st = RZ_ERR_CUDA;
        const int grid = std::max(1, std::min(n, ctx->num_sms * result->ctas_per_sm));
        const int slots[3] = {1, 2, 8};  // 4, the default, was timed above
        for (int si = 0; si < 3 && st == RZ_OK; ++si) {
            g.walk_slots = slots[si];
            float t[3] = {0.f, 0.f, 0.f};
            for (int rep = 0; rep < 4 && st == RZ_OK; ++rep) {
                cudaError_t e = cudaEventRecord(e0, ctx->stream);
                if (e == cudaSuccess) e = glyph_enqueue_flatten(g, (uint32_t*)ctx->g_scan.p, P, ctx->stream);
                if (e == cudaSuccess) e = cudaMemsetAsync(queue, 0, 4, ctx->stream);
                if (e == cudaSuccess)
                    e = rz::launch_glyph_cover(g, (const rz::WorkItem*)ctx->d_items.p, n, queue, grid, ctx->stream);
                if (e == cudaSuccess) e = cudaEventRecord(e1, ctx->stream);
                if (e == cudaSuccess) e = cudaEventSynchronize(e1);
                if (e != cudaSuccess) {
                    st = RZ_ERR_CUDA;
                    break;
                }
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (rep > 0) t[rep - 1] = ms;  // the first launch warms up
            }
            if (st) break;
            st = read_error(ctx);
            if (st) break;
            std::sort(t, t + 3);
            if (result->n_entries < 24)
                result->entries[result->n_entries++] =
                    rz_tune_entry{result->band_rows_cap, result->ctas_per_sm, t[1], slots[si]};
            if (t[1] < result->ms) {
                result->ms = t[1];
                result->walk_slots = slots[si];
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st) {
        ctx->tune_rows_cap = saved_cap;
        ctx->tune_ctas = saved_ctas;
        return st == RZ_ERR_CUDA ? fail(ctx, st, "tuning launch failed") : st;
    }
    ctx->tune_rows_cap = result->band_rows_cap;
    ctx->tune_ctas = result->ctas_per_sm;
    ctx->tune_walk = result->walk_slots;
    return RZ_OK;
}

}  // namespace

extern "C" {

const char* rz_device_name(rz_ctx* ctx) {
    if (!ctx) return "";
    std::lock_guard<std::mutex> lock(ctx->mu);
    if (ctx->device_name.empty()) {
        cudaDeviceProp prop;
        if (cudaGetDeviceProperties(&prop, ctx->device) == cudaSuccess) ctx->device_name = prop.name;
        else cudaGetLastError();
    }
    return ctx->device_name.c_str();
}

rz_status rz_set_tuning(rz_ctx* ctx, int32_t band_rows_cap, int32_t ctas_per_sm, int32_t walk_slots) {
    if (!ctx) return RZ_ERR_INVALID;
    std::lock_guard<std::mutex> lock(ctx->mu);
    if (band_rows_cap < 0 || band_rows_cap > 256 || ctas_per_sm < 0 || ctas_per_sm > 32 || walk_slots < 0 ||
        walk_slots > 16)
        return fail(ctx, RZ_ERR_INVALID, "band_rows_cap must be 0..256, ctas_per_sm 0..32 and walk_slots 0..16");
    ctx->tune_rows_cap = band_rows_cap ? band_rows_cap : 256;
    ctx->tune_ctas = ctas_per_sm;
    ctx->tune_walk = walk_slots;
    return RZ_OK;
}

rz_status rz_tune_batch(rz_ctx* ctx, const rz_path_batch* batch, double flatness, float* out, uint64_t out_len,
                        rz_tune_result* result) {
    if (!ctx) return RZ_ERR_INVALID;
    std::lock_guard<std::mutex> lock(ctx->mu);
    if (!batch || !out || !batch->masks || !result || batch->memory != RZ_MEM_DEVICE)
        return fail(ctx, RZ_ERR_INVALID, "the tuner needs a device-memory batch and output");
    if (!valid_flatness(flatness)) return fail(ctx, RZ_ERR_INVALID, "flatness must be > 0 and finite");
    RZ_CUDA(cudaSetDevice(ctx->device));
    const uint32_t P = batch->n_paths;
    std::vector<rz::MaskDev> masks(P);
    for (uint32_t p = 0; p < P; ++p) {
        const rz_mask_desc& d = batch->masks[p];
        if (d.width > 16383 || d.height > 16383 || (d.height > 0 && d.row_stride < d.width))
            return fail(ctx, RZ_ERR_INVALID, "bad mask descriptor");
        if (d.width && d.height && d.offset + (uint64_t)(d.height - 1) * d.row_stride + d.width > out_len)
            return fail(ctx, RZ_ERR_INVALID, "mask exceeds output buffer");
        masks[p].offset = d.offset;
        masks[p].width = (int32_t)d.width;
        masks[p].height = (int32_t)d.height;
        masks[p].row_stride = (int32_t)d.row_stride;
        masks[p].clip_width = (int32_t)d.width - 1;
    }
    rz::BatchDev b{};
    b.kind = batch->seg_kind;
    b.pts = batch->seg_pts;
    b.sub_off = batch->subpath_off;
    b.path_sub = batch->path_subpath_off;
    b.tr = batch->transforms;
    b.rule = batch->fill_rules;
    b.n_segments = batch->n_segments;
    b.n_subpaths = batch->n_subpaths;
    b.out = out;
    set_thresholds(b, flatness);
    // the kernel batch plans of this batch will use: the glyph pipeline when its offsets allow it
    bool glyph = false;
    if (P > 0 && use_glyph_pipeline()) {
        std::vector<uint32_t> h_sub((size_t)batch->n_subpaths + 1), h_psub((size_t)P + 1);
        RZ_CUDA(cudaMemcpy(h_sub.data(), batch->subpath_off, h_sub.size() * 4, cudaMemcpyDeviceToHost));
        RZ_CUDA(cudaMemcpy(h_psub.data(), batch->path_subpath_off, h_psub.size() * 4, cudaMemcpyDeviceToHost));
        glyph = offsets_monotone(h_sub.data(), batch->n_subpaths, batch->n_segments, h_psub.data(), P);
    }
    if (glyph) return tune_glyph(ctx, masks, b, result);
    const int occ = std::max(1, rz::mask_bands_occupancy());
    const int caps[5] = {16, 32, 64, 128, 256};
    const int saved_cap = ctx->tune_rows_cap, saved_ctas = ctx->tune_ctas;
    std::memset(result, 0, sizeof(*result));
    result->ms = 1e30f;
    cudaEvent_t e0, e1;
    RZ_CUDA(cudaEventCreate(&e0));
    RZ_CUDA(cudaEventCreate(&e1));
    rz_status st = RZ_OK;
    for (int ci = 0; ci < 5 && st == RZ_OK; ++ci) {
        for (int per_sm = occ; per_sm >= std::max(1, occ - 1) && st == RZ_OK; --per_sm) {
            ctx->tune_rows_cap = caps[ci];
            ctx->tune_ctas = per_sm;
            Items items;
            build_items(masks, false, items, caps[ci]);
            rz::BatchDev bb = b;
            st = stage_plan(ctx, masks, items, bb);
            if (st) break;
            float t[3] = {0.f, 0.f, 0.f};
            for (int rep = 0; rep < 4 && st == RZ_OK; ++rep) {
                if (cudaEventRecord(e0, ctx->stream) != cudaSuccess) { st = RZ_ERR_CUDA; break; }
                st = run_bands(ctx, bb, items, false);
                if (st) break;
                if (cudaEventRecord(e1, ctx->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) {
                    st = RZ_ERR_CUDA;
                    break;
                }
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (rep > 0) t[rep - 1] = ms;  // the first launch warms up
            }
            if (st) break;
            st = read_error(ctx);
            if (st) break;
            std::sort(t, t + 3);
            if (result->n_entries < 24) result->entries[result->n_entries++] = rz_tune_entry{caps[ci], per_sm, t[1], 0};
            if (t[1] < result->ms) {
                result->ms = t[1];
                result->band_rows_cap = caps[ci];
                result->ctas_per_sm = per_sm;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st) {
        ctx->tune_rows_cap = saved_cap;
        ctx->tune_ctas = saved_ctas;
        return st == RZ_ERR_CUDA ? fail(ctx, st, "tuning launch failed") : st;
    }
    ctx->tune_rows_cap = result->band_rows_cap;
    ctx->tune_ctas = result->ctas_per_sm;
    return RZ_OK;
}

}  // extern "C"
