// rz_api.cu -- host runtime behind the C ABI (include/rasterize_gb300.h).
//
// A context owns a stream and growable device buffers.  Host-memory calls
// stage inputs through pinned memory, launch the band kernel and copy the
// masks back; device-memory batches are launched in place.  A batch plan
// keeps the work list and mask descriptors resident on the device and
// replays the launch from a captured CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/rasterize_gb300.h"
#include "rz_host_arc.cpp.inc"
#include "rz_kernels.cuh"

namespace rz {
cudaError_t init_kernels();
cudaError_t launch_mask_bands(const BatchDev& b, const WorkItem* items, int n_items, int32_t* queue, int grid,
                              cudaStream_t stream);
int mask_bands_occupancy();
int band_floats();
cudaError_t launch_flatten_counts(const BatchDev& b, uint32_t n_segments, uint32_t n_subpaths, uint32_t* counts,
                                  cudaStream_t stream);
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
    HostBuf h_stage, h_out;
    // host-side arc expansion scratch
    std::vector<uint8_t> x_kind;
    std::vector<double> x_pts;
    std::vector<uint32_t> x_sub, x_psub, x_segmap, x_submap;
    bool expanded = false;  // the last stage_host expanded arcs
};

namespace {

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

// Band height for a mask: as many rows as fit in the shared band.
int band_rows(int clip_width, int height) {
    const int stride = rz::band_stride(clip_width);
    int rows = std::max(1, rz::band_floats() / stride);
    return std::min(rows, std::max(1, height));
}

struct Items {
    std::vector<rz::WorkItem> items;
    std::vector<int> path_first;  // first item of each path (items grouped by path)
};

// Work items sorted by decreasing band area so the persistent CTAs pick the
// longest items first (LPT order); `grouped` keeps path order instead.
void build_items(const std::vector<rz::MaskDev>& masks, bool grouped, Items& out) {
    out.items.clear();
    out.path_first.assign(masks.size() + 1, 0);
    for (size_t p = 0; p < masks.size(); ++p) {
        out.path_first[p] = (int)out.items.size();
        const rz::MaskDev& m = masks[p];
        if (m.width <= 0 || m.height <= 0) continue;
        const int rows = band_rows(m.clip_width, m.height);
        for (int y = 0; y < m.height; y += rows) {
            rz::WorkItem w;
            w.path = (uint32_t)p;
            w.y0 = (uint16_t)y;
            w.rows = (uint16_t)std::min(rows, m.height - y);
            out.items.push_back(w);
        }
    }
    out.path_first[masks.size()] = (int)out.items.size();
    if (!grouped) {
        std::stable_sort(out.items.begin(), out.items.end(), [&](const rz::WorkItem& a, const rz::WorkItem& b) {
            const long ca = (long)a.rows * masks[a.path].width;
            const long cb = (long)b.rows * masks[b.path].width;
            return ca > cb;
        });
    }
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
        rz::init_kernels() != cudaSuccess) {
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
    DevBuf* bufs[] = {&c->d_kind, &c->d_pts, &c->d_sub, &c->d_psub, &c->d_tr, &c->d_rule,
                      &c->d_masks, &c->d_items, &c->d_out, &c->d_ctrl, &c->d_counts};
    for (DevBuf* b : bufs) b->release();
    c->h_stage.release();
    c->h_out.release();
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
                     const uint8_t* rule, rz::BatchDev& b) {
    // arcs are converted to cubics on the host, as PathBuilder::arc_to does
    bool has_arc = false;
    for (uint32_t i = 0; i < n_seg && !has_arc; ++i) has_arc = kind[i] == RZ_SEG_ARC;
    ctx->expanded = has_arc;
    if (has_arc) {
        if (!rzhost::expand_batch(kind, pts, sub_off, path_sub, n_paths, ctx->x_kind, ctx->x_pts, ctx->x_sub,
                                  ctx->x_psub, ctx->x_segmap, ctx->x_submap))
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
    const bool direct = pinned(kind) && pinned(pts);
    const size_t total = (direct ? 0 : al(sz_kind) + al(sz_pts)) + al(sz_sub) + al(sz_psub) + al(sz_tr) + al(sz_rule);
    RZ_CUDA(ctx->h_stage.ensure(total));
    // wait for earlier copies out of the staging buffer before overwriting it
    RZ_CUDA(cudaStreamSynchronize(ctx->stream));
    char* h = (char*)ctx->h_stage.p;
    size_t o = 0;
    auto put = [&](const void* src, size_t n) {
        char* dst = h + o;
        if (n) std::memcpy(dst, src, n);
        o += al(n);
        return dst;
    };
    const char* hk = direct ? (const char*)kind : put(kind, sz_kind);
    const char* hp = direct ? (const char*)pts : put(pts, sz_pts);
    char* hs = put(sub_off, sz_sub);
    char* hq = put(path_sub, sz_psub);
    char* ht = tr ? put(tr, sz_tr) : nullptr;
    char* hr = rule ? put(rule, sz_rule) : nullptr;
    RZ_CUDA(ctx->d_kind.ensure(sz_kind + 1));
    RZ_CUDA(ctx->d_pts.ensure(sz_pts + 8));
    RZ_CUDA(ctx->d_sub.ensure(sz_sub));
    RZ_CUDA(ctx->d_psub.ensure(sz_psub));
    if (sz_kind) RZ_CUDA(cudaMemcpyAsync(ctx->d_kind.p, hk, sz_kind, cudaMemcpyHostToDevice, ctx->stream));
    if (sz_pts) RZ_CUDA(cudaMemcpyAsync(ctx->d_pts.p, hp, sz_pts, cudaMemcpyHostToDevice, ctx->stream));
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
    RZ_CUDA(ctx->d_ctrl.ensure(64));
    if (sz_m) RZ_CUDA(cudaMemcpyAsync(ctx->d_masks.p, masks.data(), sz_m, cudaMemcpyHostToDevice, ctx->stream));
    if (!items.items.empty())
        RZ_CUDA(cudaMemcpyAsync(ctx->d_items.p, items.items.data(), items.items.size() * sizeof(rz::WorkItem),
                                cudaMemcpyHostToDevice, ctx->stream));
    RZ_CUDA(cudaMemsetAsync(ctx->d_ctrl.p, 0, 64, ctx->stream));
    // pageable sources above: the copies complete before the call returns
    int32_t* ctrl = (int32_t*)ctx->d_ctrl.p;
    b.masks = (const rz::MaskDev*)ctx->d_masks.p;
    b.err = ctrl;           // [0] error word
    b.counters = ctrl + 4;  // [4] unused, [5] fallbacks
    return RZ_OK;
}

rz_status run_bands(rz_ctx* ctx, const rz::BatchDev& b, const Items& items, bool per_path) {
    int32_t* queue = (int32_t*)ctx->d_ctrl.p + 8;
    const rz::WorkItem* d_items = (const rz::WorkItem*)ctx->d_items.p;
    if (!per_path) {
        const int n = (int)items.items.size();
        if (n == 0) return RZ_OK;
        const int occ = std::max(1, rz::mask_bands_occupancy());
        const int grid = std::min(n, ctx->num_sms * occ);
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
    rz::BatchDev b{};
    const uint32_t path_sub[2] = {0, path->n_subpaths};
    const uint8_t r8 = (uint8_t)rule;
    st = stage_host(ctx, path->seg_kind, path->seg_pts, path->n_segments, path->subpath_off, path->n_subpaths,
                    path_sub, 1, tr, &r8, b);
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
    RZ_CUDA(ctx->d_out.ensure(width * height * 4 + 16));
    b.out = (float*)ctx->d_out.p;
    set_thresholds(b, flatness);
    st = run_bands(ctx, b, items, false);
    if (st) return st;
    return RZ_OK;
}

}  // namespace

extern "C" {

rz_status rz_mask(rz_ctx* ctx, const rz_path* path, const double tr[6], int32_t fill_rule, double flatness,
                  double* img, rz_shape shape) {
    if (!ctx) return RZ_ERR_INVALID;
    std::lock_guard<std::mutex> lock(ctx->mu);
    if (!tr || !img) return fail(ctx, RZ_ERR_INVALID, "null argument");
    if (shape.width == 0 || shape.height == 0) return RZ_OK;
    rz_status st = render_single(ctx, path, tr, fill_rule, flatness, shape.width, shape.height, false);
    if (st) return st;
    const size_t n = shape.width * shape.height;
    RZ_CUDA(ctx->h_out.ensure(n * 4));
    RZ_CUDA(cudaMemcpyAsync(ctx->h_out.p, ctx->d_out.p, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    st = read_error(ctx);
    if (st) return st;
    const float* src = (const float*)ctx->h_out.p;
    for (uint64_t y = 0; y < shape.height; ++y)
        for (uint64_t x = 0; x < shape.width; ++x)
            img[shape.start + y * shape.row_stride + x * shape.col_stride] = (double)src[y * shape.width + x];
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
        st = stage_host(ctx, batch->seg_kind, batch->seg_pts, batch->n_segments, batch->subpath_off,
                        batch->n_subpaths, batch->path_subpath_off, P, batch->transforms, batch->fill_rules, b);
        if (st) return st;
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
    Items items;
    build_items(masks, per_path, items);
    st = stage_plan(ctx, masks, items, b);
    if (st) return st;
    set_thresholds(b, flatness);
    if (batch->memory == RZ_MEM_HOST) {
        RZ_CUDA(ctx->d_out.ensure(out_len * 4 + 16));
        b.out = (float*)ctx->d_out.p;
    } else {
        b.out = out;
    }
    st = run_bands(ctx, b, items, per_path);
    if (st) return st;
    if (batch->memory == RZ_MEM_HOST)
        RZ_CUDA(cudaMemcpyAsync(out, b.out, out_len * 4, cudaMemcpyDeviceToHost, ctx->stream));
    return read_error(ctx);
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
    DevBuf d_masks, d_items, d_ctrl;
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
    build_items(masks, false, plan->items);
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
    int32_t* ctrl = (int32_t*)plan->d_ctrl.p;
    b.err = ctrl;
    b.counters = ctrl + 4;
    set_thresholds(b, flatness);
    const int n = (int)plan->items.items.size();
    const int occ = std::max(1, rz::mask_bands_occupancy());
    plan->grid = std::max(1, std::min(n, ctx->num_sms * occ));
    // capture: reset the queue head, one persistent launch
    int32_t* queue = ctrl + 8;
    e = cudaStreamBeginCapture(plan->capture_stream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaMemsetAsync(queue, 0, 4, plan->capture_stream);
        if (n > 0)
            rz::launch_mask_bands(b, (const rz::WorkItem*)plan->d_items.p, n, queue, plan->grid,
                                  plan->capture_stream);
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
    delete plan;
}

}  // extern "C"
