// rz_noalloc.cu -- batch rendering without any memory allocation.
//
// rz_mask_batch_noalloc renders a device-memory batch exactly like
// rz_mask_batch, but it allocates nothing: no cudaMalloc / cudaFree, no
// pinned host buffers, no heap memory, and it needs no rz_ctx.  It is meant
// for callers that must not allocate while they render: code running inside
// another framework's memory pool or arena, real-time loops that cannot
// afford an allocator call, and hosts whose device memory is fully reserved
// up front.
//
// The band kernel's scratch (mask descriptors, the work list of row bands,
// the queue head, the error word and a counter) lives in the file-scope
// device array `g_scratch` below, kScratchBytes large; every GPU that loads
// this library holds it until the process exits.  Host-side staging uses
// file-scope host arrays of the same capacity.  Batches beyond the limits
// (kMaxPaths paths or kMaxItems row bands) are rejected with
// RZ_ERR_CAPACITY.
//
// All calls share the one array, which keeps the last call's contents: the
// queue head, error word and counters are cleared at the start of every call,
// and calls whose work overlaps on the GPU race on the array.  Inside one
// process the calls are serialised: each holds a process-wide lock on the
// host staging arrays until its work has finished, so a call on a second GPU
// waits for a call on the first.  The first call on a device performs a one-time set-up
// with that device current (the array's device address and the kernel's
// shared-memory attribute); make that first call before any stream capture.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>

#include "../../include/rasterize_gb300.h"
#include "rz_kernels.cuh"

namespace rz {
cudaError_t init_kernels();
cudaError_t launch_mask_bands(const BatchDev& b, const WorkItem* items, int n_items, int32_t* queue, int grid,
                              cudaStream_t stream);
int mask_bands_occupancy();
int band_floats();
}  // namespace rz

namespace {

constexpr int kMaxPaths = 16384;
constexpr int kMaxItems = 65536;
constexpr size_t kCtrlBytes = 256;
constexpr size_t kMasksBytes = (size_t)kMaxPaths * sizeof(rz::MaskDev);
constexpr size_t kItemsBytes = (size_t)kMaxItems * sizeof(rz::WorkItem);
constexpr size_t kScratchBytes = kCtrlBytes + kMasksBytes + kItemsBytes;  // 896 KiB + 256 B

// The scratch of rz_mask_batch_noalloc: [ctrl words | mask descriptors | work items].
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// Host staging of the same layout (file scope: no heap allocation).
static rz::MaskDev h_masks[kMaxPaths];
static rz::WorkItem h_items[kMaxItems];
static std::mutex g_host_mu;  // the host arrays are shared by all calls

constexpr int kMaxDevices = 64;
struct DeviceSetup {
    bool done = false;
    unsigned char* scratch = nullptr;  // device address of g_scratch on this device
    int num_sms = 0;
    int occupancy = 0;
};
static DeviceSetup g_setup[kMaxDevices];
static std::mutex g_setup_mu;

// One-time set-up per device, with that device current.
rz_status device_setup(int device, DeviceSetup*& out) {
    if (device < 0 || device >= kMaxDevices) return RZ_ERR_INVALID;
    std::lock_guard<std::mutex> lock(g_setup_mu);
    DeviceSetup& s = g_setup[device];
    if (!s.done) {
        void* ptr = nullptr;
        if (cudaGetSymbolAddress(&ptr, g_scratch) != cudaSuccess) return RZ_ERR_CUDA;
        if (rz::init_kernels() != cudaSuccess) return RZ_ERR_CUDA;
        if (cudaDeviceGetAttribute(&s.num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
            return RZ_ERR_CUDA;
        s.occupancy = std::max(1, rz::mask_bands_occupancy());
        s.scratch = static_cast<unsigned char*>(ptr);
        s.done = true;
    }
    out = &s;
    return RZ_OK;
}

}  // namespace

extern "C" {

RZ_API rz_status rz_mask_batch_noalloc(const rz_path_batch* batch, double flatness, float* out, uint64_t out_len,
                                       void* stream) {
    if (!batch || !out || !batch->masks || batch->memory != RZ_MEM_DEVICE) return RZ_ERR_INVALID;
    if (!std::isfinite(flatness) || !(16.0 * flatness * flatness > 0.0)) return RZ_ERR_INVALID;  // as rz_mask_batch
    const uint32_t P = batch->n_paths;
    if (P > (uint32_t)kMaxPaths) return RZ_ERR_CAPACITY;
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) return RZ_ERR_NO_DEVICE;
    DeviceSetup* setup = nullptr;
    rz_status st = device_setup(device, setup);
    if (st != RZ_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;

    std::lock_guard<std::mutex> lock(g_host_mu);
    // mask descriptors and the work list (row bands, longest first)
    int n_items = 0;
    for (uint32_t p = 0; p < P; ++p) {
        const rz_mask_desc& d = batch->masks[p];
        if (d.width > 16383 || d.height > 16383 || (d.height > 0 && d.row_stride < d.width)) return RZ_ERR_INVALID;
        if (d.width && d.height && d.offset + (uint64_t)(d.height - 1) * d.row_stride + d.width > out_len)
            return RZ_ERR_INVALID;
        rz::MaskDev& m = h_masks[p];
        m.offset = d.offset;
        m.width = (int32_t)d.width;
        m.height = (int32_t)d.height;
        m.row_stride = (int32_t)d.row_stride;
        m.clip_width = (int32_t)d.width - 1;
        if (m.width <= 0 || m.height <= 0) continue;
        const int stride = rz::band_stride(m.clip_width);
        const int rows = std::min(std::min(256, std::max(1, rz::band_floats() / stride)), m.height);
        for (int y = 0; y < m.height; y += rows) {
            if (n_items >= kMaxItems) return RZ_ERR_CAPACITY;
            h_items[n_items].path = p;
            h_items[n_items].y0 = (uint16_t)y;
            h_items[n_items].rows = (uint16_t)std::min(rows, m.height - y);
            ++n_items;
        }
    }
    std::sort(h_items, h_items + n_items, [](const rz::WorkItem& a, const rz::WorkItem& b) {
        const long ca = (long)a.rows * h_masks[a.path].width, cb = (long)b.rows * h_masks[b.path].width;
        if (ca != cb) return ca > cb;
        return a.path != b.path ? a.path < b.path : a.y0 < b.y0;
    });

    unsigned char* base = setup->scratch;
    int32_t* ctrl = reinterpret_cast<int32_t*>(base);
    rz::MaskDev* d_masks = reinterpret_cast<rz::MaskDev*>(base + kCtrlBytes);
    rz::WorkItem* d_items = reinterpret_cast<rz::WorkItem*>(base + kCtrlBytes + kMasksBytes);
    // the array keeps the last call's contents: clear the words that must start at zero
    if (cudaMemsetAsync(ctrl, 0, kCtrlBytes, s) != cudaSuccess) return RZ_ERR_CUDA;
    if (P && cudaMemcpyAsync(d_masks, h_masks, P * sizeof(rz::MaskDev), cudaMemcpyHostToDevice, s) != cudaSuccess)
        return RZ_ERR_CUDA;
    if (n_items &&
        cudaMemcpyAsync(d_items, h_items, n_items * sizeof(rz::WorkItem), cudaMemcpyHostToDevice, s) != cudaSuccess)
        return RZ_ERR_CUDA;

    rz::BatchDev b{};
    b.kind = batch->seg_kind;
    b.pts = batch->seg_pts;
    b.sub_off = batch->subpath_off;
    b.path_sub = batch->path_subpath_off;
    b.tr = batch->transforms;
    b.rule = batch->fill_rules;
    b.masks = d_masks;
    b.out = out;
    b.err = ctrl;            // [0] error word
    b.counters = ctrl + 4;   // [5] binary64 re-decisions
    b.thr64 = 16.0 * flatness * flatness;
    b.thr32 = (float)b.thr64;
    b.n_segments = batch->n_segments;
    b.n_subpaths = batch->n_subpaths;
    if (n_items) {
        const int grid = std::min(n_items, setup->num_sms * setup->occupancy);
        if (rz::launch_mask_bands(b, d_items, n_items, ctrl + 8, grid, s) != cudaSuccess) return RZ_ERR_CUDA;
    }
    // the staging arrays are reused by the next call: wait for the copies, read the error word
    int32_t code = 0;
    if (cudaMemcpyAsync(&code, ctrl, sizeof(code), cudaMemcpyDeviceToHost, s) != cudaSuccess) return RZ_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return RZ_ERR_CUDA;
    // the kernel writes RZ_ERR_NAN, RZ_ERR_DEPTH or RZ_ERR_ARC; any other word is reported as a capacity error,
    // the way the context entry points map it
    if (code == RZ_OK || code == RZ_ERR_NAN || code == RZ_ERR_DEPTH || code == RZ_ERR_ARC) return code;
    return RZ_ERR_CAPACITY;
}

}  // extern "C"
