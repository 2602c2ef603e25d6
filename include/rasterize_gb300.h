/*
 * rasterize_gb300.h -- C ABI of the GB300 (sm_103a) rasterizer library.
 *
 * Drop-in boundary for the `Rasterizer` trait of aslpavel/rasterize v0.6.7
 * (src/rasterize.rs:44-101): a Rust `GpuRasterizer` shim (an `extern "C"`
 * block over these declarations plus a `Rasterizer` impl) packs its `Path`
 * (src/path.rs:228-233) into `rz_path`, calls these entry points and keeps
 * the crate's `Path` / `Transform` / `FillRule` / `ImageMut` API unchanged.  Every entry point returns a status; nothing traps or
 * panics.  All functions are callable from any host thread; calls on one
 * context are serialised on the context's stream.
 */
#ifndef RASTERIZE_GB300_H
#define RASTERIZE_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define RZ_API __attribute__((visibility("default")))
#else
#define RZ_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
typedef int32_t rz_status;
#define RZ_OK 0
#define RZ_ERR_NAN 1          /* a segment holds NaN: the reference panics (src/path.rs:765-767) */
#define RZ_ERR_INVALID 2      /* bad argument (sizes, pointers, flatness <= 0, ...) */
#define RZ_ERR_CUDA 3         /* CUDA runtime error; rz_last_error() has the text */
#define RZ_ERR_NO_DEVICE 4    /* no CUDA device / the library cannot run here */
#define RZ_ERR_DEPTH 5        /* a curve needs more than 22 bisection levels */
#define RZ_ERR_ARC 6          /* an arc has no finite cubic count (the reference never terminates) */
#define RZ_ERR_CAPACITY 7     /* an internal buffer limit was exceeded */

/* ---- enums mirroring the reference ------------------------------------- */
#define RZ_SEG_LINE 0  /* Segment::Line  src/curve.rs:905-909 */
#define RZ_SEG_QUAD 1  /* Segment::Quad */
#define RZ_SEG_CUBIC 2 /* Segment::Cubic */
#define RZ_SEG_ARC 3   /* PathBuilder::arc_to arguments, expanded on the device (src/path.rs:945-972) */

#define RZ_FILL_NONZERO 0 /* FillRule::NonZero src/path.rs:21-47 */
#define RZ_FILL_EVENODD 1 /* FillRule::EvenOdd */

#define RZ_MEM_HOST 0   /* pointers in a descriptor are host memory */
#define RZ_MEM_DEVICE 1 /* pointers in a descriptor are device memory of the context's GPU */

/* ---- paths -------------------------------------------------------------- */
/* One path in the reference's structure-of-arrays form (src/path.rs:228-233).
 * seg_pts holds 8 doubles per segment: up to four control points
 * x0 y0 x1 y1 x2 y2 x3 y3; an ARC holds sx sy dx dy rx ry x_axis_rot_deg flags
 * (flags bit0 = large_arc, bit1 = sweep).  subpath_off has n_subpaths + 1
 * segment offsets.  closed is informational: rasterizers always close
 * (src/rasterize.rs:307).  Host memory. */
typedef struct rz_path {
    const uint8_t* seg_kind;
    const double* seg_pts;
    const uint32_t* subpath_off;
    const uint8_t* closed;
    uint32_t n_segments;
    uint32_t n_subpaths;
} rz_path;

/* Strided image view, element units (image.rs:6-35 Shape). */
typedef struct rz_shape {
    uint64_t start;
    uint64_t width;
    uint64_t height;
    uint64_t row_stride;
    uint64_t col_stride;
} rz_shape;

/* Sparse pixel yielded by Rasterizer::mask_iter (src/rasterize.rs:664-672). */
typedef struct rz_pixel {
    uint64_t x;
    uint64_t y;
    double alpha;
} rz_pixel;

/* Many independent paths, each rendered into its own mask.  Segments of all
 * paths are concatenated; subpath_off holds global segment offsets
 * (n_subpaths + 1); path_subpath_off (n_paths + 1) gives each path's subpath
 * range.  transforms: n_paths * 6 doubles or NULL (identity).  fill_rules:
 * n_paths bytes or NULL (NonZero).  `memory` says where seg_kind, seg_pts,
 * subpath_off, path_subpath_off, transforms and fill_rules live; masks
 * (descriptors) are always host memory. */
typedef struct rz_mask_desc {
    uint64_t offset;     /* element offset of pixel (0,0) in the output buffer */
    uint32_t width;
    uint32_t height;
    uint32_t row_stride; /* elements between rows (>= width) */
    uint32_t reserved;
} rz_mask_desc;

typedef struct rz_path_batch {
    uint32_t n_paths;
    uint32_t n_segments;
    uint32_t n_subpaths;
    int32_t memory;
    const uint8_t* seg_kind;
    const double* seg_pts;
    const uint32_t* subpath_off;
    const uint32_t* path_subpath_off;
    const double* transforms;
    const uint8_t* fill_rules;
    const rz_mask_desc* masks;
} rz_path_batch;

typedef struct rz_ctx rz_ctx;

/* ---- context ------------------------------------------------------------ */
/* Creates a context on `device` with its own non-blocking stream.  Replaces
 * the constructor `SignedDifferenceRasterizer::new(flatness)`
 * (src/rasterize.rs:284-296); flatness is passed per call instead. */
RZ_API rz_ctx* rz_create(int device, rz_status* status);
RZ_API void rz_destroy(rz_ctx* ctx);
/* Text of the last error on this context ("" when none). */
RZ_API const char* rz_last_error(const rz_ctx* ctx);
/* Runs the context's work on `stream` (a cudaStream_t; NULL = the legacy
 * default stream) instead of the context's own stream. */
RZ_API rz_status rz_set_stream(rz_ctx* ctx, void* stream);
RZ_API void* rz_get_stream(const rz_ctx* ctx);
RZ_API rz_status rz_synchronize(rz_ctx* ctx);
/* Library version string. */
RZ_API const char* rz_version(void);

/* ---- Rasterizer::mask -------------------------------------------------- */
/* SignedDifferenceRasterizer::mask (src/rasterize.rs:299-311) followed by the
 * fill rule (src/rasterize.rs:473-507): rasterises `path` transformed by
 * `tr` (6 doubles, src/geometry.rs:317) into the host f64 view `img`/`shape`.
 * The view's pixels are overwritten with the mask the reference produces on a
 * zeroed image (the reference's contract, src/path.rs:509-512). */
RZ_API rz_status rz_mask(rz_ctx* ctx, const rz_path* path, const double tr[6], int32_t fill_rule,
                  double flatness, double* img, rz_shape shape);

/* SignedDifferenceRasterizer::mask_iter (src/rasterize.rs:313-355): writes up
 * to `cap` pixels with |alpha| >= 1e-6 in row-major order into `pixels` and
 * their total count into *n_pixels (which may exceed cap). */
RZ_API rz_status rz_mask_iter(rz_ctx* ctx, const rz_path* path, const double tr[6], int32_t fill_rule,
                       double flatness, uint64_t width, uint64_t height, rz_pixel* pixels,
                       uint64_t cap, uint64_t* n_pixels);

/* Renders every path of `batch` into its own f32 mask in `out` (mask
 * semantics as rz_mask; out has out_len elements, host or device memory per
 * batch->memory).  One persistent-kernel launch for the whole batch; a large
 * host batch with page-locked `out` is rendered in chunks of paths whose
 * uploads and downloads overlap the rendering.  Elements of a host `out` that
 * no mask covers (row padding, gaps between masks) may be overwritten. */
RZ_API rz_status rz_mask_batch(rz_ctx* ctx, const rz_path_batch* batch, double flatness, float* out,
                        uint64_t out_len);

/* Same batch rendered the plain way: one rasterisation launch per path, in
 * path order (the per-path GPU baseline the batched kernel is measured against). */
RZ_API rz_status rz_mask_batch_per_path(rz_ctx* ctx, const rz_path_batch* batch, double flatness,
                                 float* out, uint64_t out_len);

/* ---- paints and scenes --------------------------------------------------- */
#define RZ_PAINT_SOLID 0  /* LinColor (src/color.rs:357-374) */
#define RZ_PAINT_LINEAR 1 /* GradLinear (src/grad.rs:150-226) */
#define RZ_PAINT_RADIAL 2 /* GradRadial (src/grad.rs:300-426) */
#define RZ_UNITS_USER_SPACE 0 /* Units::UserSpaceOnUse (src/rasterize.rs:170-177) */
#define RZ_UNITS_BOUNDING_BOX 1
#define RZ_SPREAD_PAD 0 /* GradSpread (src/grad.rs:7-31) */
#define RZ_SPREAD_REPEAT 1
#define RZ_SPREAD_REFLECT 2

/* GradStop (src/grad.rs:41-52): position and premultiplied linear RGBA. */
typedef struct rz_stop {
    double position;
    float color[4];
} rz_stop;

/* A Paint.  Solid: `color` (premultiplied linear RGBA).  Linear: start, end.
 * Radial: start = center, end = focal center, radius, fradius.  Gradients
 * take stops (sorted like GradStops::new), units, spread, linear_colors and
 * their own transform `tr`.  At most 16 stops.  Host memory. */
typedef struct rz_paint {
    int32_t kind;
    int32_t units;
    int32_t spread;
    int32_t linear_colors;
    double tr[6];
    double start[2];
    double end[2];
    double radius;
    double fradius;
    float color[4];
    const rz_stop* stops;
    uint32_t n_stops;
    uint32_t reserved;
} rz_paint;

/* A Scene that is a Group of Fill nodes in drawing order (src/scene.rs:69-200),
 * rendered with Scene::render(tr = identity, view = the canvas, bg).  Paths of
 * all fills are concatenated: subpath_off holds global segment offsets
 * (n_subpaths + 1), fill_subpath_off (n_fills + 1) gives each fill's subpath
 * range.  transforms: n_fills * 6 (NULL = identity), fill_rules: n_fills (NULL
 * = NonZero), fill_paint: paint index per fill.  Host memory. */
typedef struct rz_scene {
    uint32_t n_fills;
    uint32_t n_segments;
    uint32_t n_subpaths;
    uint32_t n_paints;
    const uint8_t* seg_kind;
    const double* seg_pts;
    const uint32_t* subpath_off;
    const uint32_t* fill_subpath_off;
    const double* transforms;
    const uint8_t* fill_rules;
    const uint32_t* fill_paint;
    const rz_paint* paints;
    const uint8_t* subpath_closed; /* n_subpaths flags or NULL (all open): only strokes read them */
} rz_scene;

/* Rasterizer::fill (src/rasterize.rs:69-115): paints `path` (transformed by
 * tr) with `paint` and composites it source-over into the host RGBA f32 view
 * `img` (4 floats per pixel; shape in pixels), exactly where and how the
 * reference's signed-difference rasterizer would. */
RZ_API rz_status rz_fill(rz_ctx* ctx, const rz_path* path, const double tr[6], int32_t fill_rule, double flatness,
                         const rz_paint* paint, float* img, rz_shape shape);

/* Scene::render (src/scene.rs:186-199, Pipeline::render_rec Fill :407-435)
 * of a Group of fills over a width x height RGBA f32 canvas (host memory, row
 * major, 4 floats per pixel) initialised to bg (NULL: transparent).  The
 * fills are flattened and binned by (fill, row band) once, then one CTA per
 * row band composites every fill in order. */
RZ_API rz_status rz_render_scene(rz_ctx* ctx, const rz_scene* scene, double flatness, const float bg[4],
                                 float* canvas, uint32_t width, uint32_t height);

/* ---- stroking ------------------------------------------------------------ */
#define RZ_JOIN_MITER 0 /* LineJoin::Miter(miter_limit) (src/path.rs:78-95; default, limit 4) */
#define RZ_JOIN_BEVEL 1
#define RZ_JOIN_ROUND 2
#define RZ_CAP_BUTT 0 /* LineCap (src/path.rs:103-117; default Butt) */
#define RZ_CAP_SQUARE 1
#define RZ_CAP_ROUND 2
/* StrokeStyle (src/path.rs:121-137). */
typedef struct rz_stroke_style {
    double width;
    double miter_limit; /* LineJoin::Miter's limit */
    int32_t line_join;
    int32_t line_cap;
} rz_stroke_style;

/* Host-only: Path::stroke (src/path.rs:374-415), the outline path of `path`
 * stroked with `style` (path->closed says which subpaths are closed; NULL:
 * all open).  Every outline subpath is closed.  Call once with NULL arrays
 * for *n_segments / *n_subpaths, then with arrays of those sizes
 * (subpath_off: n_subpaths + 1); smaller caps return RZ_ERR_CAPACITY.  Arcs
 * are expanded first.  Needs no context or GPU. */
RZ_API rz_status rz_stroke_path(const rz_path* path, const rz_stroke_style* style, uint8_t* seg_kind,
                                double* seg_pts, uint32_t seg_cap, uint32_t* subpath_off, uint32_t sub_cap,
                                uint32_t* n_segments, uint32_t* n_subpaths);

/* ---- scene trees: groups, transforms, opacity and clip layers ----------- */
/* One node of a scene tree (SceneInner, src/scene.rs:19-62), in pre-order: a
 * node, then the subtrees of its children.  Fill entries are those of the
 * rz_scene the nodes come with; an entry's own transform (scene->transforms,
 * NULL = identity) applies first, under the transforms of its ancestors. */
#define RZ_NODE_FILL 0      /* Fill: arg = fill entry (path, rule, paint) */
#define RZ_NODE_GROUP 1     /* Group: arg = number of child subtrees that follow */
#define RZ_NODE_TRANSFORM 2 /* Transform: tr, then one child subtree */
#define RZ_NODE_OPACITY 3   /* Opacity: opacity (clamped to [0, 1] as Scene::opacity does), one child */
#define RZ_NODE_CLIP 4      /* Clip: arg = fill entry of the clip path (its rule; paint unused), units, one child */
#define RZ_NODE_STROKE 5    /* Stroke: arg = fill entry (path, paint; rule unused), stroke style; filled NonZero */
typedef struct rz_scene_node {
    int32_t kind;
    uint32_t arg;
    int32_t units;        /* RZ_UNITS_USER_SPACE or RZ_UNITS_BOUNDING_BOX (Clip) */
    int32_t line_join;    /* Stroke: RZ_JOIN_* */
    int32_t line_cap;     /* Stroke: RZ_CAP_* */
    int32_t reserved;
    double opacity;       /* Opacity */
    double width;         /* Stroke */
    double miter_limit;   /* Stroke, RZ_JOIN_MITER */
    double tr[6];         /* Transform */
} rz_scene_node;

/* Scene::render (src/scene.rs:186-199) of the tree nodes[0 .. n_nodes) with
 * view = the width x height canvas and tr = identity: Pipeline::build_rec
 * (:268-357) on the host, then render_rec (:397-458).  Fills queued for one
 * layer go through the line pipeline together; an Opacity or Clip node renders
 * its child into a layer of its own (device memory, per nesting depth), a Clip
 * renders its path's mask with the same pipeline, and one compose kernel
 * blends the child onto its parent layer (Layer::compose, :532-565).  Output:
 * the RGBA f32 canvas (host), the sRGB8 RGBA bytes (host), or both (either
 * may be NULL).  With nothing in view the canvas is the background. */
RZ_API rz_status rz_render_scene_tree(rz_ctx* ctx, const rz_scene* scene, const rz_scene_node* nodes,
                                      uint32_t n_nodes, double flatness, const float bg[4], float* canvas,
                                      uint8_t* rgba8, uint32_t width, uint32_t height);

/* ---- output encode: premultiplied linear RGBA f32 -> sRGB8 RGBA ---------- */
/* Scene::render followed by `to_rgba` of every pixel (From<LinColor> for RGBA,
 * src/color.rs:164-175), what Image::write_bmp / write_png / write_rgba store
 * (src/image.rs:136-229).  The encode runs in the composite's epilogue, so only
 * 4 bytes a pixel leave the GPU.  rgba8: width * height * 4 bytes, host memory. */
RZ_API rz_status rz_render_scene_rgba8(rz_ctx* ctx, const rz_scene* scene, double flatness, const float bg[4],
                                       uint8_t* rgba8, uint32_t width, uint32_t height);
/* `to_rgba` of n premultiplied linear RGBA f32 pixels: unmultiply (alpha <= 1e-6
 * gives 0), the x86 l2s fit (src/simd/x86.rs:197-214), (c * 255 + 0.5) as u8;
 * alpha is not unmultiplied.  memory: RZ_MEM_HOST or RZ_MEM_DEVICE for both
 * arrays (a device canvas 16-byte aligned, rgba8 4-byte aligned; the call is
 * then asynchronous on the context's stream). */
RZ_API rz_status rz_encode_rgba8(rz_ctx* ctx, const float* canvas, uint64_t n_pixels, uint8_t* rgba8,
                                 int32_t memory);
/* `to_rgba` of a mask (Scalar, src/color.rs:429-432): grey linear_to_srgb(1 - m),
 * alpha 255.  elem_size 8: f64 masks (converted to f32 first, as the reference
 * does), 4: f32. */
RZ_API rz_status rz_encode_mask_rgba8(rz_ctx* ctx, const void* mask, int32_t elem_size, uint64_t n_pixels,
                                      uint8_t* rgba8, int32_t memory);

#define RZ_IMAGE_BMP 0  /* Image::write_bmp (src/image.rs:165-212) */
#define RZ_IMAGE_RGBA 1 /* Image::write_rgba (src/image.rs:136-149) */
#define RZ_IMAGE_PPM 2  /* Image::write_ppm (src/image.rs:151-163) */
/* Host-only: the file bytes of an sRGB8 RGBA image (row major, 4 bytes a pixel)
 * in `format`.  *len receives the size; out NULL asks for the size only, a
 * smaller cap returns RZ_ERR_CAPACITY.  Needs no context or GPU. */
RZ_API rz_status rz_write_image(const uint8_t* rgba8, uint32_t width, uint32_t height, int32_t format,
                                uint8_t* out, uint64_t cap, uint64_t* len);

/* ---- batch plans: resident work list + CUDA graph replay ---------------- */
/* A plan fixes one device-memory batch (batch->memory == RZ_MEM_DEVICE), its
 * output buffer and flatness.  Creating it sizes the plan's buffers (one pass
 * over the trees and a host round trip), uploads the work list (bands of rows,
 * longest first) and mask descriptors once and captures a CUDA graph; each
 * launch replays the graph (queue reset, record pass, tree walk, vertex offsets,
 * vertex emission, persistent cover kernel; with RZ_BATCH_KERNEL=bands the
 * record pass and the band kernel) on the context's stream without any host
 * synchronisation.  The input arrays may be rewritten between launches (same
 * sizes); geometry that outgrows the sized buffers is reported as
 * RZ_ERR_CAPACITY by rz_batch_plan_status, never written past them. */
typedef struct rz_batch_plan rz_batch_plan;
RZ_API rz_batch_plan* rz_batch_plan_create(rz_ctx* ctx, const rz_path_batch* batch, double flatness, float* out,
                                           uint64_t out_len, rz_status* status);
RZ_API rz_status rz_batch_plan_launch(rz_batch_plan* plan);
/* Waits for the plan's launches and returns the first device error since the
 * last call (RZ_ERR_NAN, RZ_ERR_DEPTH, ...), then clears it. */
RZ_API rz_status rz_batch_plan_status(rz_batch_plan* plan);
/* Number of work items (bands) and binary64 flatness re-decisions so far. */
RZ_API rz_status rz_batch_plan_info(rz_batch_plan* plan, uint64_t* n_items, uint64_t* fallbacks);
RZ_API void rz_batch_plan_destroy(rz_batch_plan* plan);

/* Allocation-free variant of rz_mask_batch (no counterpart in the reference).
 * For callers that cannot allocate device memory while rendering: code that
 * runs inside another framework's memory pool, real-time loops, hosts whose
 * device memory is reserved up front.  Renders a device-memory batch
 * (batch->memory == RZ_MEM_DEVICE) into the device buffer `out` on `stream`
 * (NULL = legacy default stream) of the current device, with no cudaMalloc,
 * no pinned or heap allocation and no rz_ctx.  The kernel's scratch is one
 * static 896 KiB device array per GPU (held until the process exits): at most
 * 16384 paths and 65536 row bands per call, larger batches return
 * RZ_ERR_CAPACITY.  The first call on a device does a one-time set-up.  Calls
 * share the array and must not overlap on the GPU; within one process they are
 * serialised by a process-wide lock, across devices too.  The call is
 * synchronous: it returns after its work has finished (it reads the error
 * word), so it cannot be captured into a CUDA graph. */
RZ_API rz_status rz_mask_batch_noalloc(const rz_path_batch* batch, double flatness, float* out, uint64_t out_len,
                                       void* stream);

/* Counts the flattened lines of every segment exactly as
 * PathFlattenIter (src/path.rs:734-796) emits them: counts[i] for segment i
 * after arc expansion, then one entry per subpath for the closing line.
 * n_counts receives the number of entries (may exceed cap). */
RZ_API rz_status rz_flatten_counts(rz_ctx* ctx, const rz_path* path, const double tr[6], double flatness,
                            uint32_t* counts, uint64_t cap, uint64_t* n_counts);

/* ------------------------------------------------------------------------
 * Batch autotuner.  Times the batch kernels on the caller's device-memory
 * batch (rendering into `out`) for every candidate band-height cap (16, 32,
 * 64, 128, 256 rows: the work-item shape) and resident CTAs per SM (the
 * occupancy limit and one or two less), then, for the glyph pipeline, the
 * slots each lane of the tree walk takes (1, 2, 4, 8: 32 to 256 segments per
 * warp) at the fastest shape; keeps the fastest in the context for later
 * rz_mask_batch / rz_batch_plan_create calls, and reports every entry.
 * rz_set_tuning applies a stored choice (0, 0, 0 restores the defaults).
 * ------------------------------------------------------------------------ */
typedef struct rz_tune_entry {
    int32_t band_rows_cap;
    int32_t ctas_per_sm;
    float ms;            /* median of 3 launches, CUDA events */
    int32_t walk_slots;  /* slots per lane of the glyph pipeline's tree walk (32 per warp times that); 0: n/a */
} rz_tune_entry;

typedef struct rz_tune_result {
    int32_t band_rows_cap;  /* the fastest */
    int32_t ctas_per_sm;
    float ms;
    uint32_t n_entries;
    rz_tune_entry entries[24];
    int32_t walk_slots;
} rz_tune_result;

RZ_API rz_status rz_tune_batch(rz_ctx* ctx, const rz_path_batch* batch, double flatness, float* out, uint64_t out_len,
                               rz_tune_result* result);
/* walk_slots 0 keeps the default (4). */
RZ_API rz_status rz_set_tuning(rz_ctx* ctx, int32_t band_rows_cap, int32_t ctas_per_sm, int32_t walk_slots);
/* Name of the context's GPU (for keying stored tunings). */
RZ_API const char* rz_device_name(rz_ctx* ctx);

/* ------------------------------------------------------------------------
 * Differentiable batch.  The reference has no adjoint; the forward composes
 * Rasterizer::fill (src/rasterize.rs:69-115: mask_iter with the image size,
 * then source-over) for closed cubic paths drawn in order with one solid paint
 * of alpha `paint_alpha`, and keeps the alpha channel of each image.
 *
 * Control points are FP32 in device memory: image i, path p, point j at
 * ctrl[2 * ((i * paths_per_image + p) * 3 * segs_per_path + j)] (x, y).
 * Segment s of a path is the cubic (V_s, C1_s, C2_s, V_{(s+1) mod segs}) with
 * V_s = point 3s, C1_s = point 3s + 1, C2_s = point 3s + 2, so every path is
 * closed.  Images are width x height f32, row-major, image i at offset
 * i * width * height.
 * ------------------------------------------------------------------------ */
typedef struct rz_diff_batch {
    uint32_t n_images;
    uint32_t paths_per_image;
    uint32_t segs_per_path;
    uint32_t width, height;
    int32_t fill_rule;   /* RZ_FILL_NONZERO or RZ_FILL_EVENODD */
    float paint_alpha;   /* 0 < alpha < 1 */
    const float* ctrl;   /* device memory */
} rz_diff_batch;

/* Forward: every image (device memory, overwritten). */
RZ_API rz_status rz_diff_forward(rz_ctx* ctx, const rz_diff_batch* batch, double flatness, float* image);

/* sum over n of (image - target)^2 into *loss (host, binary64 accumulation);
 * dl_dimage (device, may be null) receives 2 (image - target). */
RZ_API rz_status rz_l2_loss(rz_ctx* ctx, const float* image, const float* target, uint64_t n, double* loss,
                            float* dl_dimage);

/* Adjoint: d loss / d control points (device memory, same layout as ctrl,
 * overwritten) from d loss / d image (device), given the forward `image`.
 * The bisection tree is held fixed and every flattened line is recomputed
 * (nothing is stored between the passes). */
RZ_API rz_status rasterize_backward(rz_ctx* ctx, const rz_diff_batch* batch, double flatness, const float* image,
                                    const float* dl_dimage, float* dl_dctrl);

#ifdef __cplusplus
}
#endif
#endif /* RASTERIZE_GB300_H */
