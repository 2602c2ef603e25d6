// rz_pipeline.cuh -- data layout of the line pipeline (large paths, scenes).
//
// Kernels, in launch order:
//   k_flatten_count  one thread per segment slot: lines its bisection tree emits
//   scan             exclusive prefix of the counts (line offsets)
//   k_flatten_emit   walks again, writes 16.16 lines, counts lines per (fill, band)
//   scan             exclusive prefix of the (fill, band) counts
//   k_bin_scatter    line indices into their (fill, band) lists
//   k_composite      one CTA per row band of the canvas: fills in order, signed
//                    area in shared memory, row prefix, fill rule, paint, source-over
#pragma once
#include <stdint.h>

namespace rz {

constexpr int kMaxStops = 16;

// Flattening work is split into 2^task_depth subtree tasks per segment slot
// (task t = slot * 2^task_depth + j walks the subtree at depth task_depth,
// index j), so large segments spread over several threads and a warp's
// threads do similar amounts of work.  Lines stay in tree order.  Small
// segments use depth 0 (every task loads its segment).
__host__ __device__ inline uint64_t slot_tasks(uint64_t n_slots, int task_depth) { return n_slots << task_depth; }

// One fill of a scene (or the single path of a large mask), device memory.
struct FillDev {
    uint32_t sub0, sub1;     // subpath range (global)
    uint32_t seg0, seg1;     // segment range (global)
    uint32_t slot0;          // first flatten slot (segments, then one closing line per subpath)
    uint32_t entry0;         // first (fill, band) entry
    int32_t col0, row0;      // canvas position of the fill's local (0, 0)
    int32_t width, height;   // view: local columns [0, width), rows [0, height)
    int32_t clip_width;      // the reference's `width` for this view
    int32_t band0, nbands;   // canvas bands the view touches
    int32_t rule, paint;     // fill rule, paint index (-1: coverage only)
    double tr[6];            // transform into local coordinates (binary64)
};

struct PaintDev {
    int32_t kind;           // 0 solid, 1 linear, 2 radial, -1 draws nothing
    int32_t spread;         // 0 pad, 1 repeat, 2 reflect
    int32_t linear_colors;  // 0: stops are sRGB, results converted back to linear
    int32_t nstops;
    int32_t radial_linear;  // radial with |A| < EPSILON: the equation is linear in t
    int32_t pad;
    // linear: t of a local pixel centre (x, y) = g0 x + g1 y + g2, each
    // coefficient a double-float pair gh + gl composed in binary64
    float gh[3], gl[3];
    // radial: pd = p - focal centre of a local pixel centre (x, y):
    // (q0 x + q1 y + q2, q3 x + q4 y + q5), FP32 and binary64
    float q[6];
    double qd[6];
    float cdx, cdy, rd, fr;       // c - fc, r - fr, focal radius
    double cdxd, cdyd, rdd, frd;  // same in binary64
    double a64;                   // A = |cd|^2 - rd^2
    float color[4];               // solid colour
    float pos[kMaxStops];
    float col[kMaxStops][4];
};

struct SceneDev;

struct SceneDev {
    const uint8_t* kind;
    const double* pts;
    const uint32_t* sub_off;
    const FillDev* fills;
    const PaintDev* paints;
    uint32_t n_fills;
    uint32_t n_slots;
    uint32_t n_segments;
    uint32_t n_subpaths;
    int32_t task_depth;      // flatten tasks per slot = 2^task_depth (when task_off is null)
    const uint32_t* task_off;  // [n_slots + 1] first task of each slot (2^k tasks each), or null
    uint32_t n_tasks;        // tasks in total when task_off is set
    double thr64;
    float thr32;
    int32_t canvas_w, canvas_h;
    int32_t band_rows;       // canvas rows per band
    int32_t n_bands;
    // pipeline buffers
    uint32_t* slot_count;    // [tasks + 1] lines per flatten task, then its exclusive prefix (line offsets)
    int4* lines;             // [2 * n_lines] per end point: exact 16.16 anchor (x, y), FP32 remainder (dx, dy)
    uint32_t n_lines;        // lines, or (n_lines_dev set) an upper bound for launch sizes
    const uint32_t* n_lines_dev;  // non-null: the line count in device memory (sized without a host round trip)
    uint32_t line_cap;       // lines the buffer holds (the emit pass reports more as ERR_CAPACITY)
    uint32_t pair_cap;       // (line, band) pairs the list buffer holds (the scatter reports more)
    uint32_t* entry_count;   // [n_entries]
    uint32_t* entry_start;   // [n_entries] exclusive prefix of entry_count
    uint32_t* entry_cursor;  // [n_entries]
    uint32_t* pairs;         // [n_pairs] line indices grouped by (fill, band)
    uint2* leaf;             // [n_lines] (input segment or ~0, depth << 27 | index) per line, or null
    // output
    float* canvas;           // RGBA f32 (scenes) or f32 mask (coverage only)
    int64_t canvas_stride;   // elements between rows (pixels for RGBA: 4 floats each)
    const float* bg;         // background colour or null (canvas already initialised)
    int32_t load_canvas;     // 1: blend over the canvas content instead of bg
    uint32_t* rgba8;         // non-null: the band is written as sRGB8 RGBA (canvas_w words a row) instead of f32
    int32_t* err;
    int32_t* counters;
};

// Differentiable batch (rz_diff.cu): images stacked in one canvas, one fill per path.
struct DiffDev {
    SceneDev S;          // lines binned per row (S.band_rows = 1)
    int32_t cta_rows;    // rows of a CTA (one warp each); divides the image height
    int32_t paths;       // per image
    int32_t segs;        // per path
    int32_t width, height;
    int32_t rule;
    float alpha;         // paint alpha
    const float* ctrl;   // control points (FP32)
    const float* image;  // forward image (backward input)
    const float* dl_dimage;
    float* out;          // forward: images; backward: d loss / d ctrl
};

}  // namespace rz

namespace rz {

// First flatten task of slot `slot`, and the number of tasks of a scene.
__device__ __forceinline__ uint64_t task_first(const SceneDev& S, uint32_t slot) {
    return S.task_off ? (uint64_t)S.task_off[slot] : ((uint64_t)slot << S.task_depth);
}
__host__ __device__ inline uint64_t scene_tasks(const SceneDev& S) {
    return S.task_off ? (uint64_t)S.n_tasks : slot_tasks(S.n_slots, S.task_depth);
}

}  // namespace rz
