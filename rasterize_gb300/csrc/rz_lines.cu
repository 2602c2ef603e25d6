// rz_lines.cu -- batched masks from flattened lines.
//
// The batch path of many independent masks: every segment slot of every path
// is flattened once by the pipeline's count / scan / emit kernels (subtree
// tasks, the reference's exact bisection tree), so the lines of path p are
// contiguous in the line buffer.  k_mask_lines then renders the masks:
// persistent CTAs pull (path, band of rows) work items in decreasing-area
// order from a device queue, accumulate the path's lines that reach the band
// into a shared-memory band (exact fixed point), scan the rows, apply the
// fill rule and stream the band to the mask.  Three barriers per item, no
// tree walk inside the band loop.
#include "rz_device.cuh"
#include "rz_kernels.cuh"
#include "rz_pipeline.cuh"

namespace rz {

constexpr int kLinesThreads = 256;
constexpr int kLinesBandBytes = 48 * 1024;  // 4 CTAs per SM
constexpr int kLinesBandFloats = kLinesBandBytes / 4;

__global__ void __launch_bounds__(kLinesThreads, 4) k_mask_lines(SceneDev S, const MaskDev* __restrict__ masks,
                                                                 const WorkItem* __restrict__ items, int n_items,
                                                                 int32_t* queue, float* out) {
    extern __shared__ float4 sm4[];
    float* acc = reinterpret_cast<float*>(sm4);
    __shared__ int s_item;
    const int tid = threadIdx.x;
    for (;;) {
        if (tid == 0) s_item = atomicAdd(queue, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= n_items) break;
        const WorkItem wi = items[it];
        const MaskDev m = masks[wi.path];
        const FillDev& f = S.fills[wi.path];
        Band B;
        B.acc = acc;
        B.stride = band_stride(m.clip_width);
        B.bh = wi.rows;
        B.y0 = wi.y0;
        B.img_h = m.height;
        B.width_f = (float)m.clip_width;
        B.width_i = m.clip_width;
        const int n4 = (B.bh * B.stride) >> 2;
        for (int i = tid; i < n4; i += kLinesThreads) sm4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        __syncthreads();
        // the path's lines: its slots are contiguous, slot_count holds their line offsets
        const uint32_t nslot = (f.seg1 - f.seg0) + (f.sub1 - f.sub0);
        const uint32_t l0 = S.slot_count[task_first(S, f.slot0)];
        const uint32_t l1 = min(S.slot_count[task_first(S, f.slot0 + nslot)], S.line_cap);
        // anchors are within a few px of the exact ends: a margin of 8 rows keeps every line that reaches the band
        const int32_t ylo = (B.y0 - 8) * 65536, yhi = (B.y0 + B.bh + 8) * 65536;
        for (uint32_t l = l0 + tid; l < l1; l += kLinesThreads) {
            const int4 a = S.lines[2ull * l], b = S.lines[2ull * l + 1];
            if (max(a.y, b.y) < ylo || min(a.y, b.y) > yhi) continue;
            accumulate_vtx(B, line_vtx(a, B.y0), line_vtx(b, B.y0));
        }
        __syncthreads();
        MaskStore st{out, m.offset, (int64_t)m.row_stride, B.y0, m.width};
        band_scan<kLinesThreads>(B, m.width, f.rule, st);
        __syncthreads();
    }
}

int lines_band_floats() { return kLinesBandFloats; }

cudaError_t init_lines_kernel() {
    return cudaFuncSetAttribute(k_mask_lines, cudaFuncAttributeMaxDynamicSharedMemorySize, kLinesBandBytes);
}

int mask_lines_occupancy() {
    int blocks = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_mask_lines, kLinesThreads, kLinesBandBytes);
    return blocks;
}

cudaError_t launch_mask_lines(const SceneDev& S, const MaskDev* masks, const WorkItem* items, int n_items,
                              int32_t* queue, float* out, int grid, cudaStream_t st) {
    if (n_items <= 0) return cudaSuccess;
    k_mask_lines<<<grid, kLinesThreads, kLinesBandBytes, st>>>(S, masks, items, n_items, queue, out);
    return cudaGetLastError();
}

}  // namespace rz
