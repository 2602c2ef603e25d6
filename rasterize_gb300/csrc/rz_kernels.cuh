// rz_kernels.cuh -- kernel-side data layout shared by the kernels and the host runtime.
#pragma once
#include <stdint.h>

namespace rz {

// One path of a batch as the kernels see it (device memory).
struct MaskDev {
    uint64_t offset;     // element offset of pixel (0,0) in the output
    int32_t width;       // mask width (pixels written)
    int32_t height;
    int32_t row_stride;  // elements between output rows
    int32_t clip_width;  // the reference's `width`: width-1 (mask) or width (mask_iter)
};

struct SlotRec;  // per-slot segment record of the band kernel (rz_band.cu)

struct BatchDev {
    const uint8_t* kind;        // [n_segments]
    const double* pts;          // [n_segments * 8]
    const uint32_t* sub_off;    // [n_subpaths + 1] global segment offsets
    const uint32_t* path_sub;   // [n_paths + 1] subpath ranges
    const double* tr;           // [n_paths * 6] or null (identity)
    const uint8_t* rule;        // [n_paths] or null (NonZero)
    const MaskDev* masks;       // [n_paths]
    float* out;
    int32_t* err;               // device error word (first error wins)
    int32_t* counters;          // [0] work-queue head, [1] binary64 fallbacks
    double thr64;               // 16 f^2 as the reference computes it
    float thr32;
    uint32_t n_segments;        // array extents: offsets are clamped to them
    uint32_t n_subpaths;
    uint32_t n_paths;           // extent of path_sub / tr (record pass)
    int32_t flat_out;           // packed masks are written as one span per band (page-locked host output)
    const SlotRec* recs;        // [n_segments + n_subpaths] built by k_band_records, or null (built per band)
};

// A band of rows of one path's mask: the unit of work of the band kernel.
struct WorkItem {
    uint32_t path;
    uint16_t y0;
    uint16_t rows;
};

// Band geometry shared by host and device: row stride in shared memory.  At
// least clip_width + 3 columns (two spill columns of the reference's writes
// past `width`), rounded up to whole 16-pixel scan chunks.
__host__ __device__ inline int band_stride(int clip_width) { return ((clip_width + 3) + 15) & ~15; }

}  // namespace rz
