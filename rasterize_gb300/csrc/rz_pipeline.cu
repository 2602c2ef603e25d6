// rz_pipeline.cu -- line pipeline for large paths and painted scenes.
//
// k_flatten_count / k_flatten_emit flatten every segment slot (segments, then
// one closing line per subpath) with the reference's exact bisection tree
// (FP32 decisions, binary64 replays) into 16.16 lines in the fill's local
// frame; the emit pass also counts lines per (fill, band).  k_bin_scatter
// lists each band's lines per fill (a counting sort keyed by (fill, band)),
// and k_composite renders one canvas row band per CTA: for every fill in
// order it accumulates the fill's lines in shared memory, scans the rows,
// applies the fill rule and blends the fill's paint source-over into an RGBA
// band kept in shared memory (Rasterizer::fill + Pipeline::render_rec,
// src/rasterize.rs:69-115, src/scene.rs:407-435).
#include <atomic>

#include "rz_color.cuh"
#include "rz_device.cuh"
#include "rz_kernels.cuh"
#include "rz_pipeline.cuh"

namespace rz {

__device__ __forceinline__ void pset_err(int32_t* err, int code) { atomicCAS(err, 0, code); }

// Fill owning flatten slot s (fills are in slot order).
__device__ __forceinline__ uint32_t fill_of_slot(const SceneDev& S, uint32_t s) {
    uint32_t lo = 0, hi = S.n_fills;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (S.fills[mid].slot0 <= s) lo = mid; else hi = mid;
    }
    return lo;
}

// Loads the binary64 segment of slot s (untransformed); false for an empty
// closing line (empty subpath).  Closing line: Line(subpath.end(), subpath.start()).
__device__ bool slot_segment(const SceneDev& S, const FillDev& f, uint32_t s, Seg64& g, uint32_t& src) {
    const uint32_t i = s - f.slot0;
    const uint32_t nseg = f.seg1 - f.seg0;
    if (i < nseg) {
        src = f.seg0 + i;
        g.kind = S.kind[src];
        const double2* p2 = reinterpret_cast<const double2*>(S.pts + 8ull * src);
        #pragma unroll
        for (int j = 0; j < 4; ++j) {
            const double2 q = __ldg(p2 + j);
            g.x[j] = q.x;
            g.y[j] = q.y;
        }
        return g.kind != SEG_ARC;  // scenes arrive with arcs expanded
    }
    const uint32_t sp = f.sub0 + (i - nseg);
    const uint32_t s0 = S.sub_off[sp], s1 = min(S.sub_off[sp + 1], S.n_segments);
    if (s1 <= s0) return false;
    src = 0xffffffffu;
    const int kl = S.kind[s1 - 1];
    const int nl = kl == SEG_LINE ? 1 : (kl == SEG_QUAD ? 2 : 3);
    g.kind = SEG_LINE;
    g.x[0] = S.pts[8ull * (s1 - 1) + 2 * nl];
    g.y[0] = S.pts[8ull * (s1 - 1) + 2 * nl + 1];
    g.x[1] = S.pts[8ull * s0];
    g.y[1] = S.pts[8ull * s0 + 1];
    g.x[2] = g.y[2] = g.x[3] = g.y[3] = 0.0;
    return true;
}

struct SlotState {
    bool ok = false;    // a segment to flatten
    bool fits = false;  // inside the 16.16 range
    uint32_t src = 0xffffffffu;  // input segment (~0: a closing line)
    Seg64 g;            // binary64, transformed
    FixSeg F;
    SegRec r;
    FlatCoef c;
    float qerr = 0.f;
};

__device__ void load_slot(const SceneDev& S, const FillDev& f, uint32_t s, SlotState& st) {
    uint32_t src = 0;
    st.ok = slot_segment(S, f, s, st.g, src);
    if (!st.ok) return;
    st.src = src;
    const int n = seg_npts(st.g.kind);
    bool nan = false, fits = true;
    #pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (j < n) {
            tr_apply64(f.tr, st.g.x[j], st.g.y[j], st.g.x[j], st.g.y[j]);
            nan |= is_nan_bits(st.g.x[j]) || is_nan_bits(st.g.y[j]);
            fits &= d2fix(st.g.x[j], st.F.x[j]) & d2fix(st.g.y[j], st.F.y[j]);
        } else {
            st.F.x[j] = st.F.y[j] = 0;
        }
    }
    if (nan) {  // the reference panics on NaN (src/path.rs:765-767)
        pset_err(S.err, ERR_NAN);
        st.ok = false;
        return;
    }
    st.F.kind = st.g.kind;
    st.fits = fits;
    if (fits) {
        make_record(st.F, st.g.x, st.g.y, st.r);
        st.r.src = src;
        st.c = rec_flat(st.r, st.qerr);
    }
}

// FITS: the slot is inside the 16.16 range (a fixed-point record), known at
// compile time so a walk over records keeps nothing of the binary64 segment live.
template <int FITS>  // 1 record, 0 binary64 segment, -1 either (st.fits)
__device__ __forceinline__ int slot_decide(const SceneDev& S, const FillDev& f, const SlotState& st, int d, uint32_t k,
                                           int& fallbacks) {
    if (FITS == 1 || (FITS < 0 && st.fits))
        return decide_node(st.r, st.c, st.qerr, d, k, S.thr32, S.thr64, S.pts, f.tr, fallbacks);
    const FlatCoef c = flat_coef(st.g);
    return node_is_leaf(st.g, c, d, k, S.thr64, S.thr32, fallbacks);
}

// Leaves of task j of the slot's tree, in order; `emit(d, k)` per leaf.  A
// leaf above the task depth belongs to the first task under it.  Returns
// false on a tree deeper than MAX_DEPTH.
template <int FITS = -1, class Emit>
__device__ bool walk_task(const SceneDev& S, const FillDev& f, const SlotState& st, uint32_t j, int td,
                          int& fallbacks, Emit& emit) {
    for (int d = 0; d < td; ++d) {
        const int up = td - d;
        if (slot_decide<FITS>(S, f, st, d, j >> up, fallbacks)) {
            if ((j & ((1u << up) - 1u)) == 0u) emit(d, j >> up);
            return true;
        }
    }
    int d = td;
    uint32_t k = j;
    for (;;) {
        if (!slot_decide<FITS>(S, f, st, d, k, fallbacks)) {
            if (d >= MAX_DEPTH) return false;
            ++d;
            k <<= 1;
            continue;
        }
        emit(d, k);
        while (d > td && (k & 1u)) {
            k >>= 1;
            --d;
        }
        if (d == td) return true;
        k += 1u;
    }
}

struct CountLeaves {
    uint32_t n = 0;
    __device__ void operator()(int, uint32_t) { ++n; }
};

// A leaf is one line, or two (the reference's x rules split it) when the
// slot's coordinates are beyond the 16.16 range.
// Slot s, subtree index j and subtree depth td of flatten task t.
__device__ __forceinline__ void task_slot(const SceneDev& S, uint64_t t, uint32_t& s, uint32_t& j, int& td) {
    if (S.task_off) {
        uint32_t lo = 0, hi = S.n_slots;  // largest s with task_off[s] <= t (every slot has a task)
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (S.task_off[mid] <= t) lo = mid; else hi = mid;
        }
        s = lo;
        j = (uint32_t)(t - S.task_off[lo]);
        td = __ffs(S.task_off[lo + 1] - S.task_off[lo]) - 1;
    } else {
        s = (uint32_t)(t >> S.task_depth);
        j = (uint32_t)(t & ((1u << S.task_depth) - 1u));
        td = S.task_depth;
    }
}

__global__ void k_flatten_count(SceneDev S) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= scene_tasks(S)) return;
    uint32_t s, j;
    int td;
    task_slot(S, t, s, j, td);
    const FillDev& f = S.fills[fill_of_slot(S, s)];
    SlotState st;
    load_slot(S, f, s, st);
    uint32_t n = 0;
    int fallbacks = 0;
    if (st.ok) {
        CountLeaves c;
        if (!walk_task(S, f, st, j, td, fallbacks, c)) pset_err(S.err, ERR_DEPTH);
        n = st.fits ? c.n : 2u * c.n;
    }
    S.slot_count[t] = n;
    if (fallbacks) atomicAdd(&S.counters[1], fallbacks);
}

// Rows [r0, r1) of the fill's view a line with 16.16 end heights ya, yb
// reaches; false when none.  The range is widened by one 16.16 unit so a line
// whose rounded height sits on a row boundary still reaches the row its exact
// height enters.  Zero-height lines add no coverage and are skipped, except
// for the adjoint (leaf codes requested): moving an end vertically still
// changes the loss.
__device__ __forceinline__ bool line_rows(const SceneDev& S, const FillDev& f, int32_t ya, int32_t yb, int& r0,
                                          int& r1) {
    const int32_t ylo = min(ya, yb), yhi = max(ya, yb);
    if (ylo == yhi && !S.leaf) return false;  // no signed coverage
    r0 = max((ylo - 1) >> 16, 0);             // floor
    r1 = min((yhi + 1 + 65535) >> 16, f.height);  // ceil (exclusive)
    return r0 < r1;
}

__device__ __forceinline__ int32_t fix_add(int32_t a, float d) { return a + __float2int_rn(d * 65536.0f); }

// A line end point: exact 16.16 anchor plus FP32 remainder (px).
__device__ __forceinline__ int4 end_point(int32_t ax, int32_t ay, float dx, float dy) {
    return make_int4(ax, ay, __float_as_int(dx), __float_as_int(dy));
}

// A leaf of a segment beyond the 16.16 range: the reference's x rules
// (src/rasterize.rs:372-393) and a pure y clip in binary64, then anchors +
// remainders.  Up to two lines (e[0], e[1]) and (e[2], e[3]); returns how many
// slots the leaf takes (2), unused ones hold a degenerate line (never binned).
static __device__ __noinline__ int emit_big_leaf(const Seg64 g, int d, uint32_t k, int clip_width, int height,
                                                  int4 (&e)[4]) {
    const VertexCoef v = vertex_coef(g);
    double x0, y0, x1, y1;
    vertex_big(v, k, d, 0.0, x0, y0);
    vertex_big(v, k + 1u, d, 0.0, x1, y1);
    double px[2][2], py[2][2];
    const int np = clip_line_x64((double)clip_width, x0, y0, x1, y1, px, py);
    #pragma unroll
    for (int i = 0; i < 2; ++i) {
        e[2 * i] = e[2 * i + 1] = make_int4(0, 0, 0, 0);
        if (i < np && clip_y64(-1.0, (double)height + 1.0, px[i], py[i])) {
            int32_t a, b2, c, f;
            if (d2fix(px[i][0], a) & d2fix(py[i][0], b2) & d2fix(px[i][1], c) & d2fix(py[i][1], f)) {
                const double u = 1.0 / 65536.0;
                e[2 * i] = end_point(a, b2, (float)(px[i][0] - a * u), (float)(py[i][0] - b2 * u));
                e[2 * i + 1] = end_point(c, f, (float)(px[i][1] - c * u), (float)(py[i][1] - f * u));
            }
        }
    }
    return np;
}

// The lines of a walk, written from line offset `out` on, with their
// per-(fill, band) counts.  Holds copies of what it needs, so nothing of the
// kernel's parameters or the slot state has to live in local memory.
template <bool FITS>
struct EmitLines {
    int4* lines;
    uint2* leaf;
    uint32_t* entry_count;
    int32_t* err;
    uint32_t line_cap;
    int band_rows, row0, height, clip_width, band0, nbands;
    uint32_t entry0;
    uint32_t out;
    uint32_t src;
    const SlotState& st;
    uint32_t* hist = nullptr;  // the block's counts of entries [hist_e0, hist_e0 + n) in shared memory, or null
    uint32_t hist_e0 = 0;
    uint32_t pend_e = 0xffffffffu, pend_n = 0;  // a run of lines counted in one (fill, band) entry

    __device__ __forceinline__ EmitLines(const SceneDev& S, const FillDev& f, const SlotState& st, uint32_t first)
        : lines(S.lines), leaf(S.leaf), entry_count(S.entry_count), err(S.err), line_cap(S.line_cap),
          band_rows(S.band_rows), row0(f.row0), height(f.height), clip_width(f.clip_width), band0(f.band0),
          nbands(f.nbands), entry0(f.entry0), out(first), src(st.src), st(st) {}

    __device__ __forceinline__ void flush() {
        if (pend_n) atomicAdd(&entry_count[pend_e], pend_n);
        pend_n = 0;
    }
    __device__ __forceinline__ void count(int4 a, int4 b) {
        const int32_t ya = fix_add(a.y, __int_as_float(a.w)), yb = fix_add(b.y, __int_as_float(b.w));
        const int32_t ylo = min(ya, yb), yhi = max(ya, yb);
        if (ylo == yhi && !leaf) return;  // line_rows: no signed coverage
        const int r0 = max((ylo - 1) >> 16, 0);
        const int r1 = min((yhi + 1 + 65535) >> 16, height);
        if (r0 >= r1) return;
        const int b0 = max((r0 + row0) / band_rows, band0);
        const int b1 = min((r1 - 1 + row0) / band_rows, band0 + nbands - 1);
        if (b0 > b1) return;
        if (hist) {
            // difference-coded: +1 at the first band, -1 after the last (prefix-summed once per block)
            const uint32_t i0 = entry0 + (b0 - band0) - hist_e0;
            atomicAdd(&hist[i0], 1u);
            atomicAdd(&hist[i0 + (uint32_t)(b1 - b0) + 1u], 0xffffffffu);
            return;
        }
        if (b0 == b1) {
            // consecutive lines of a walk mostly fall in one band: their counts are added once per run
            const uint32_t e = entry0 + (b0 - band0);
            if (e != pend_e) {
                flush();
                pend_e = e;
            }
            ++pend_n;
        } else {
            for (int bb = b0; bb <= b1; ++bb) atomicAdd(&entry_count[entry0 + (bb - band0)], 1u);
        }
    }
    __device__ __forceinline__ void write(int4 a, int4 b, bool binned) {
        if (out >= line_cap) {  // the geometry changed since the buffer was sized: report, never overrun
            if (binned) atomicCAS(err, 0, ERR_CAPACITY);
            ++out;
            return;
        }
        lines[2ull * out] = a;
        lines[2ull * out + 1] = b;
        ++out;
        if (binned && entry_count) count(a, b);
    }
    __device__ __forceinline__ void operator()(int d, uint32_t k) {
        const uint32_t first = out;
        if (FITS) {
            // integer pixel of the vertex as the 16.16 anchor, its fraction as the remainder
            const uint32_t t0 = k << (MAX_DEPTH - d), t1 = (k + 1u) << (MAX_DEPTH - d);
            const VtxQ a = t0 == prev_t ? prev : rec_vtx(st.r, k, d, 0);
            const VtxQ b = rec_vtx(st.r, k + 1u, d, 0);
            prev_t = t1;
            prev = b;
            write(end_point(a.col << 16, a.row << 16, a.fx, a.fy), end_point(b.col << 16, b.row << 16, b.fx, b.fy),
                  true);
        } else {
            int4 e[4];
            const int np = emit_big_leaf(st.g, d, k, clip_width, height, e);
            write(e[0], e[1], np > 0);
            write(e[2], e[3], np > 1);
        }
        if (leaf) {
            const uint2 code = make_uint2(src, ((uint32_t)d << 27) | k);
            for (uint32_t i = first; i < out && i < line_cap; ++i) leaf[i] = code;
        }
    }
    // the last leaf's end vertex, as t * 2^MAX_DEPTH: the next leaf of the walk starts there
    uint32_t prev_t = 0xffffffffu;
    VtxQ prev;
};

// A flatten task of a slot beyond the 16.16 range, out of line so the record
// walk keeps no binary64 state (the scene by value: the copy is made on this
// rare path only).
static __device__ __noinline__ void emit_task_big(const SceneDev S, uint32_t fill, uint32_t s, uint32_t j, int td,
                                                  uint32_t first) {
    const FillDev& f = S.fills[fill];
    SlotState st;
    load_slot(S, f, s, st);
    int fallbacks = 0;
    EmitLines<false> e(S, f, st, first);
    walk_task<0>(S, f, st, j, td, fallbacks, e);
    e.flush();
}

// Entries (fill, band) a block of flatten tasks or of lines can reach when
// its fills' entries span at most kHistEntries: counted in shared memory and
// added to the global counters once per block.  Every line of a walk lands in
// a few neighbouring bands, and one global atomic per line and band would
// serialise on the few cache lines that hold a fill's counters.  A line's
// bands are consecutive entries, so the emit counts it as a difference (two
// shared atomics however many bands it crosses) and the block prefix-sums
// the window before adding it.
constexpr int kHistEntries = 2048;
constexpr int kEmitThreads = 128;

// In-place inclusive prefix of h[0, n) (n <= kHistEntries) by the THREADS
// threads of the block, each over its own run of consecutive entries.
// Starts and ends with a block barrier.
template <int THREADS>
__device__ void block_prefix_hist(uint32_t* h, uint32_t n) {
    constexpr int PER = kHistEntries / THREADS;
    __shared__ uint32_t s_warp[THREADS / 32];
    __syncthreads();
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const uint32_t base = (uint32_t)t * PER;
    uint32_t v[PER], sum = 0;
    #pragma unroll
    for (int i = 0; i < PER; ++i) {
        v[i] = base + i < n ? h[base + i] : 0u;
        sum += v[i];
    }
    uint32_t incl = sum;
    #pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t o = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += o;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    uint32_t run = incl - sum;
    for (int w = 0; w < warp; ++w) run += s_warp[w];
    #pragma unroll
    for (int i = 0; i < PER; ++i) {
        run += v[i];
        if (base + i < n) h[base + i] = run;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(kEmitThreads) k_flatten_emit(SceneDev S) {
    __shared__ uint32_t s_hist[kHistEntries + 1];  // one past the window: a difference's end
    __shared__ uint32_t s_e0, s_n;
    const uint64_t nt = scene_tasks(S);
    const uint64_t t0 = (uint64_t)blockIdx.x * kEmitThreads;
    const uint64_t t = t0 + threadIdx.x;
    if (threadIdx.x == 0) {
        uint32_t sa, sb, j;
        int td;
        task_slot(S, t0, sa, j, td);
        task_slot(S, min(t0 + kEmitThreads, nt) - 1, sb, j, td);
        const FillDev& fa = S.fills[fill_of_slot(S, sa)];
        const FillDev& fb = S.fills[fill_of_slot(S, sb)];
        const uint32_t e1 = fb.entry0 + (uint32_t)fb.nbands;
        s_e0 = fa.entry0;
        s_n = S.entry_count && e1 - fa.entry0 <= (uint32_t)kHistEntries ? e1 - fa.entry0 : 0u;
    }
    __syncthreads();
    const uint32_t hn = s_n, he0 = s_e0;
    for (uint32_t i = threadIdx.x; i <= hn; i += kEmitThreads) s_hist[i] = 0u;
    __syncthreads();
    if (t < nt) {
        uint32_t s, j;
        int td;
        task_slot(S, t, s, j, td);
        const uint32_t fill = fill_of_slot(S, s);
        const FillDev& f = S.fills[fill];
        SlotState st;
        load_slot(S, f, s, st);
        if (st.ok && !st.fits) {
            emit_task_big(S, fill, s, j, td, S.slot_count[t]);
        } else if (st.ok) {
            int fallbacks = 0;
            EmitLines<true> e(S, f, st, S.slot_count[t]);
            if (hn) {
                e.hist = s_hist;
                e.hist_e0 = he0;
            }
            walk_task<1>(S, f, st, j, td, fallbacks, e);
            e.flush();
        }
    }
    if (hn == 0) return;  // (uniform over the block)
    block_prefix_hist<kEmitThreads>(s_hist, hn);
    for (uint32_t i = threadIdx.x; i < hn; i += kEmitThreads)
        if (s_hist[i]) atomicAdd(&S.entry_count[he0 + i], s_hist[i]);
}

// Small scenes in one pass: every flatten task counts its leaves, reserves
// its lines with one atomic on *n_lines and emits them there.  No offsets
// scan and no per-band counts: the composite then gives every band every
// line (lines of different tasks interleave; the integer coverage does not
// depend on their order).
__global__ void __launch_bounds__(kEmitThreads) k_flatten_emit_alloc(SceneDev S, uint32_t* n_lines) {
    const uint64_t t = (uint64_t)blockIdx.x * kEmitThreads + threadIdx.x;
    if (t >= scene_tasks(S)) return;
    uint32_t s, j;
    int td;
    task_slot(S, t, s, j, td);
    const uint32_t fill = fill_of_slot(S, s);
    const FillDev& f = S.fills[fill];
    SlotState st;
    load_slot(S, f, s, st);
    if (!st.ok) return;
    CountLeaves c;
    int fallbacks = 0;
    if (!walk_task(S, f, st, j, td, fallbacks, c)) {
        pset_err(S.err, ERR_DEPTH);
        return;
    }
    if (fallbacks) atomicAdd(&S.counters[1], fallbacks);
    const uint32_t n = st.fits ? c.n : 2u * c.n;
    if (n == 0) return;
    const uint32_t first = atomicAdd(n_lines, n);
    if (!st.fits) {
        emit_task_big(S, fill, s, j, td, first);
    } else {
        EmitLines<true> e(S, f, st, first);
        walk_task<1>(S, f, st, j, td, fallbacks, e);
    }
}

// Lines of the scene (at most the buffer's capacity when counted on the device).
__device__ __forceinline__ uint32_t scene_lines(const SceneDev& S) {
    return S.n_lines_dev ? min(*S.n_lines_dev, S.line_cap) : S.n_lines;
}

// Fill owning line l among fills [lo, hi) (slot_count holds the line offsets
// of the flatten tasks).
__device__ __forceinline__ uint32_t fill_of_line(const SceneDev& S, uint32_t l, uint32_t lo = 0, uint32_t hi = 0) {
    if (hi == 0) hi = S.n_fills;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        const uint32_t first =
            S.fills[mid].slot0 < S.n_slots ? S.slot_count[task_first(S, S.fills[mid].slot0)] : scene_lines(S);
        if (first <= l) lo = mid; else hi = mid;
    }
    return lo;
}

// Bands [b0, b1] of the fill's bands that line l reaches (b0 > b1: none).
__device__ __forceinline__ void line_bands(const SceneDev& S, const FillDev& f, uint32_t l, int& b0, int& b1) {
    b0 = 0;
    b1 = -1;
    const int4 a = S.lines[2ull * l], b = S.lines[2ull * l + 1];
    const int32_t ya = fix_add(a.y, __int_as_float(a.w)), yb = fix_add(b.y, __int_as_float(b.w));
    int r0, r1;
    if (line_rows(S, f, ya, yb, r0, r1)) {
        b0 = max((r0 + f.row0) / S.band_rows, f.band0);
        b1 = min((r1 - 1 + f.row0) / S.band_rows, f.band0 + f.nbands - 1);
    }
}

// Line l into its (fill, band) lists with global atomics; called by all 32
// lanes of a warp (l >= n_lines: no line).  Consecutive lines mostly fall in
// one entry: the lanes with the same single entry take their slots with one
// atomic.
// A list slot beyond the buffer (sized before the lines were counted) is
// reported as ERR_CAPACITY and not written.
__device__ __forceinline__ void put_pair(const SceneDev& S, uint32_t i, uint32_t l) {
    if (i < S.pair_cap) S.pairs[i] = l;
    else pset_err(S.err, ERR_CAPACITY);
}

__device__ void bin_line_global(const SceneDev& S, uint32_t l, uint32_t n_lines) {
    const int lane = threadIdx.x & 31;
    int b0 = 0, b1 = -1;
    const FillDev* f = nullptr;
    if (l < n_lines) {
        f = &S.fills[fill_of_line(S, l)];
        line_bands(S, *f, l, b0, b1);
    }
    // one entry: aggregated per warp; none: a key no other lane has; several: one atomic per entry below
    const long long key = b0 == b1 ? (long long)(f->entry0 + (b0 - f->band0)) : -1 - (long long)threadIdx.x;
    const unsigned same = __match_any_sync(0xffffffffu, key);
    if (b0 == b1) {
        const uint32_t e = (uint32_t)key;
        const int leader = __ffs(same) - 1;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(&S.entry_cursor[e], (uint32_t)__popc(same));
        base = __shfl_sync(same, base, leader);
        put_pair(S, S.entry_start[e] + base + __popc(same & ((1u << lane) - 1u)), l);
    } else {
        for (int bb = b0; bb <= b1; ++bb) {
            const uint32_t e = f->entry0 + (bb - f->band0);
            put_pair(S, S.entry_start[e] + atomicAdd(&S.entry_cursor[e], 1u), l);
        }
    }
}

// A block takes kBinLines consecutive lines.  When their fills' entries fit
// the shared histogram: count per entry in shared memory, reserve each
// entry's slots with one global atomic, then place the lines with shared
// atomics (the order inside a list is free: coverage sums are exact).
constexpr int kBinThreads = 256;
constexpr int kBinLines = 4 * kBinThreads;

__global__ void __launch_bounds__(kBinThreads) k_bin_scatter(SceneDev S) {
    __shared__ uint32_t s_cnt[kHistEntries];
    __shared__ uint32_t s_base[kHistEntries];
    __shared__ uint32_t s_e0, s_n, s_fa, s_fb;
    const uint32_t n_lines = scene_lines(S);
    const uint32_t l0 = blockIdx.x * kBinLines;
    if (l0 >= n_lines) return;  // the grid covers the buffer's capacity
    const uint32_t l1 = min(l0 + kBinLines, n_lines);
    if (threadIdx.x == 0) {
        const uint32_t fa = fill_of_line(S, l0), fb = fill_of_line(S, l1 - 1);
        const uint32_t e0 = S.fills[fa].entry0, e1 = S.fills[fb].entry0 + (uint32_t)S.fills[fb].nbands;
        s_e0 = e0;
        s_n = e1 - e0 <= (uint32_t)kHistEntries ? e1 - e0 : 0u;
        s_fa = fa;
        s_fb = fb + 1;
    }
    __syncthreads();
    const uint32_t n = s_n, e0 = s_e0, fa = s_fa, fb = s_fb;
    if (n == 0) {
        for (uint32_t l = l0 + threadIdx.x; l < l0 + kBinLines; l += kBinThreads) bin_line_global(S, l < l1 ? l : n_lines, n_lines);
        return;
    }
    for (uint32_t i = threadIdx.x; i < n; i += kBinThreads) s_cnt[i] = 0u;
    __syncthreads();
    // each thread's lines l0 + threadIdx.x + k kBinThreads: their first entry (relative to e0) and band count,
    // kept in registers from the count to the placement
    constexpr int kPer = kBinLines / kBinThreads;
    uint32_t e_lo[kPer];
    int nb[kPer];
    #pragma unroll
    for (int k = 0; k < kPer; ++k) {
        const uint32_t l = l0 + threadIdx.x + (uint32_t)k * kBinThreads;
        e_lo[k] = 0u;
        nb[k] = 0;
        if (l < l1) {
            const FillDev& f = S.fills[fill_of_line(S, l, fa, fb)];
            int b0, b1;
            line_bands(S, f, l, b0, b1);
            if (b0 <= b1) {
                e_lo[k] = f.entry0 + (uint32_t)(b0 - f.band0) - e0;
                nb[k] = b1 - b0 + 1;
            }
        }
        // (the placement below takes one shared atomic per line and band anyway: a difference-coded count
        // here measured no faster)
        for (int i = 0; i < nb[k]; ++i) atomicAdd(&s_cnt[e_lo[k] + i], 1u);
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < n; i += kBinThreads) {
        const uint32_t c = s_cnt[i];
        if (c) s_base[i] = S.entry_start[e0 + i] + atomicAdd(&S.entry_cursor[e0 + i], c);
        s_cnt[i] = 0u;
    }
    __syncthreads();
    #pragma unroll
    for (int k = 0; k < kPer; ++k) {
        const uint32_t l = l0 + threadIdx.x + (uint32_t)k * kBinThreads;
        for (int i = 0; i < nb[k]; ++i) {
            const uint32_t e = e_lo[k] + (uint32_t)i;
            put_pair(S, s_base[e] + atomicAdd(&s_cnt[e], 1u), l);
        }
    }
}

// ---------------------------------------------------------------------------
// Paint (grad.rs, color.rs) in FP32
// ---------------------------------------------------------------------------
// GradSpread::at (src/grad.rs:24-30) on an FP32 offset
__device__ __forceinline__ float spread_at(int spread, float t) {
    if (spread == 1) {  // Repeat: rem_euclid(t, 1)
        float r = fmodf(t, 1.f);
        return r < 0.f ? r + 1.f : r;
    }
    if (spread == 2) {  // Reflect: |rem_euclid(t + 1, 2) - 1|
        float r = fmodf(t + 1.f, 2.f);
        if (r < 0.f) r += 2.f;
        return fabsf(r - 1.f);
    }
    return t;
}

// GradSpread::at on a binary64 offset
__device__ __forceinline__ float spread_at64(int spread, double t) {
    if (spread == 1) {
        const double r = fmod(t, 1.0);
        return (float)(r < 0.0 ? r + 1.0 : r);
    }
    if (spread == 2) {
        double r = fmod(t + 1.0, 2.0);
        if (r < 0.0) r += 2.0;
        return (float)fabs(r - 1.0);
    }
    return (float)t;
}

// GradSpread::at on a double-float offset th + tl (|tl| <= ulp(th)).  The
// period is removed from th exactly (x - k * period is exact for the k
// nearest below), so the fraction keeps the low word: repeat and reflect stay
// accurate however many periods away the pixel is.
__device__ __forceinline__ float spread_at_df(int spread, float th, float tl) {
    if (spread == 0) return th + tl;
    const float period = spread == 1 ? 1.f : 2.f;
    const float k = floorf(th * (1.f / period)) * period;
    float r = __fadd_rn(th, -k) + tl;
    if (r < 0.f) r += period;
    else if (r >= period) r -= period;
    if (spread == 1) return r;
    return r < 1.f ? r : 2.f - r;  // |((t + 1) rem 2) - 1| with r = t rem 2
}

// Offset of a linear gradient: g0 x + g1 y + g2 in double-float arithmetic
// (x, y are pixel centres, exact in FP32; products split with an FMA).
__device__ __forceinline__ float linear_offset(const PaintDev& p, float x, float y) {
    const float p0 = __fmul_rn(p.gh[0], x), e0 = fmaf(p.gh[0], x, -p0);
    const float p1 = __fmul_rn(p.gh[1], y), e1 = fmaf(p.gh[1], y, -p1);
    float s, es, t, et;
    two_sum(p0, p1, s, es);
    two_sum(s, p.gh[2], t, et);
    const float lo = ((e0 + e1) + (es + et)) + fmaf(p.gl[0], x, fmaf(p.gl[1], y, p.gl[2]));
    const float th = __fadd_rn(t, lo);
    const float tl = lo - __fadd_rn(th, -t);
    return spread_at_df(p.spread, th, tl);
}

// GradRadial::offset (src/grad.rs:361-396) with quadratic_solve
// (src/utils.rs:205-231) in binary64; false when there is no root.
static __device__ __noinline__ bool radial_offset64(const PaintDev& p, float px, float py, double& t) {
    const double pdx = (double)px * p.qd[0] + (double)py * p.qd[1] + p.qd[2];
    const double pdy = (double)px * p.qd[3] + (double)py * p.qd[4] + p.qd[5];
    const double a = p.a64;
    const double b = -2.0 * ((p.cdxd * pdx + p.cdyd * pdy) + p.frd * p.rdd);
    const double c = (pdx * pdx + pdy * pdy) - p.frd * p.frd;
    const double eps = 2.220446049250313e-16;
    if (fabs(a) < eps) {
        if (fabs(b) > eps) {
            t = -c / b;
            return true;
        }
        return false;
    }
    const double disc = b * b - 4.0 * a * c;
    if (fabs(disc) < eps) {
        t = -b / (2.0 * a);
        return true;
    }
    if (disc < 0.0) return false;
    const double sq = sqrt(disc);
    double r0, r1;
    if (b >= 0.0) {
        const double mul = -b - sq;
        r0 = mul / (2.0 * a);
        r1 = 2.0 * c / mul;
    } else {
        const double mul = -b + sq;
        r0 = 2.0 * c / mul;
        r1 = mul / (2.0 * a);
    }
    t = fmax(r0, r1);
    return true;
}

// simd/x86.rs:217-244 s2l on all four lanes (the reference's default build)
__device__ __forceinline__ float s2l(float v) {
    const float x1 = 2.0843103538116825f * v - 1.0843103538116827f;
    const float x2 = x1 * x1, x3 = x2 * x1;
    const float hi = 0.23361048543711943f + 0.4665843122387033f * x1 + 0.26901741378006355f * x2 +
                     0.031661580753065945f * x3;
    return v <= 0.04045f ? v * 0.07739938080495357f : hi;
}

__device__ float4 paint_at(const PaintDev& p, float px, float py) {
    if (p.kind == 0) return make_float4(p.color[0], p.color[1], p.color[2], p.color[3]);
    float t;
    if (p.kind == 1) {
        t = linear_offset(p, px, py);
    } else {
        // FP32 first; binary64 near the cone's edge (root count undecided),
        // for the degenerate linear case, and where a repeated or reflected
        // spread needs the fraction of a large offset
        bool wide = p.radial_linear != 0;
        if (!wide) {
            const float pdx = fmaf(px, p.q[0], fmaf(py, p.q[1], p.q[2]));
            const float pdy = fmaf(px, p.q[3], fmaf(py, p.q[4], p.q[5]));
            const float b = -2.f * ((p.cdx * pdx + p.cdy * pdy) + p.fr * p.rd);
            const float c = (pdx * pdx + pdy * pdy) - p.fr * p.fr;
            const float a = (float)p.a64;
            const float disc = b * b - 4.f * a * c;
            if (fabsf(disc) <= 1e-4f * (b * b + fabsf(4.f * a * c))) {
                wide = true;
            } else {
                if (disc < 0.f) return make_float4(0.f, 0.f, 0.f, 0.f);
                const float sq = sqrtf(disc);
                float r0, r1;
                if (b >= 0.f) {
                    const float mul = -b - sq;
                    r0 = mul / (2.f * a);
                    r1 = 2.f * c / mul;
                } else {
                    const float mul = -b + sq;
                    r0 = 2.f * c / mul;
                    r1 = mul / (2.f * a);
                }
                t = fmaxf(r0, r1);
                if (p.spread != 0 && !(fabsf(t) <= 1.f)) wide = true;
                else t = spread_at(p.spread, t);
            }
        }
        if (wide) {
            double t64;
            if (!radial_offset64(p, px, py, t64)) return make_float4(0.f, 0.f, 0.f, 0.f);
            t = spread_at64(p.spread, t64);
        }
    }
    // GradStops::at (src/grad.rs:116-139): first stop with position >= t
    int lo = 0, hi = p.nstops;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (p.pos[mid] < t) lo = mid + 1; else hi = mid;
    }
    float4 col;
    if (lo == 0) {
        col = make_float4(p.col[0][0], p.col[0][1], p.col[0][2], p.col[0][3]);
    } else if (lo == p.nstops) {
        const int i = p.nstops - 1;
        col = make_float4(p.col[i][0], p.col[i][1], p.col[i][2], p.col[i][3]);
    } else {
        const float ratio = (t - p.pos[lo - 1]) / (p.pos[lo] - p.pos[lo - 1]);
        const float* c0 = p.col[lo - 1];
        const float* c1 = p.col[lo];
        col = make_float4(c1[0] * ratio + c0[0] * (1.f - ratio), c1[1] * ratio + c0[1] * (1.f - ratio),
                          c1[2] * ratio + c0[2] * (1.f - ratio), c1[3] * ratio + c0[3] * (1.f - ratio));
    }
    if (!p.linear_colors) {
        // LinColor::into_linear (src/color.rs:326-333): s2l of the unmultiplied colour, times alpha
        const float a = col.w;
        if (a <= 1e-6f) return make_float4(0.f, 0.f, 0.f, 0.f);
        col = make_float4(s2l(col.x / a) * a, s2l(col.y / a) * a, s2l(col.z / a) * a, s2l(col.w / a) * a);
    }
    return col;
}

// ---------------------------------------------------------------------------
// Composite
// ---------------------------------------------------------------------------


struct BlendEpi {
    float4* rgba;        // the canvas at the band's first row and the view's first column
    int64_t stride;      // pixels between canvas rows
    int col0;            // canvas column of local x = 0 (already in rgba)
    int y0_local;        // local row of band row 0
    int width;           // view width
    const PaintDev* paint;
    __device__ __forceinline__ void operator()(int r, int x0, const float (&a)[kScanChunk]) const {
        #pragma unroll
        for (int i = 0; i < kScanChunk; ++i) {
            const int x = x0 + i;
            if (x >= width) break;
            const float al = a[i];
            if (fabsf(al) < 1e-6f) continue;  // mask_iter skips these pixels (src/rasterize.rs:347-349)
            const float4 c = paint_at(*paint, (float)x + 0.5f, (float)(y0_local + r) + 0.5f);
            float4& d = rgba[r * stride + x];
            // dst.blend_over(color.with_alpha(alpha)) = src + dst * (1 - src.a) (src/color.rs:342-349)
            const float4 s = make_float4(c.x * al, c.y * al, c.z * al, c.w * al);
            const float inv = 1.f - s.w;
            d = make_float4(s.x + d.x * inv, s.y + d.y * inv, s.z + d.z * inv, s.w + d.w * inv);
        }
    }
};

struct AlphaEpi {  // coverage-only fills write the mask
    float* out;
    int64_t stride;
    int row_base;  // canvas row of band row 0
    int col0, width;
    __device__ __forceinline__ void operator()(int r, int x0, const float (&a)[kScanChunk]) const {
        float* o = out + (int64_t)(row_base + r) * stride + col0 + x0;
        #pragma unroll
        for (int i = 0; i < kScanChunk; ++i)
            if (x0 + i < width) o[i] = a[i];
    }
};

// smem: the coverage band (band_rows x cov_stride words)
// The binary64 route of accumulate_vtx for line l.
static __device__ __noinline__ void composite_slow_line(const SceneDev& S, const Band& B, uint32_t l) {
    const VtxQ a = line_vtx(S.lines[2ull * l], B.y0), b = line_vtx(S.lines[2ull * l + 1], B.y0);
    accumulate_line64(B, (double)a.col + (double)a.fx, (double)a.row + (double)a.fy, (double)b.col + (double)b.fx,
                      (double)b.row + (double)b.fy);
}

// THREADS: 512 for masks (one CTA per SM), 256 with paint (three CTAs per SM:
// while one CTA's blends wait on L2, the others accumulate or blend).  With paint the band's
// colours stay in the canvas itself (L2-resident while the band is worked
// on): only the coverage band takes shared memory, so bands are tall and the
// per-fill work of a band covers many rows.
// Masks: one 512-thread CTA per SM (the band takes the shared memory), so up
// to 128 registers; paint: three 256-thread CTAs per SM.
template <int THREADS>
__global__ void __launch_bounds__(THREADS, THREADS == 512 ? 1 : 3) k_composite(SceneDev S, int cov_stride) {
    extern __shared__ float4 sm4[];
    __shared__ PaintDev s_paint;
    __shared__ uint32_t s_slow[THREADS / 32][64];  // per warp: at most 31 queued + 32 new
    const int lane = threadIdx.x & 31;
    float* cov = reinterpret_cast<float*>(sm4);
    const bool paint_mode = S.paints != nullptr;
    const int band = blockIdx.x;
    const int row_base = band * S.band_rows;
    const int rows = min(S.band_rows, S.canvas_h - row_base);
    if (rows <= 0) return;
    // no lists (small scenes): a flatten pass that failed (too many lines) leaves nothing to do here
    if (S.pairs == nullptr && S.err != nullptr && *(volatile const int32_t*)S.err != 0) return;
    float4* canvas4 = reinterpret_cast<float4*>(S.canvas) + (int64_t)row_base * S.canvas_stride;
    if (paint_mode && !S.load_canvas) {
        const float4 v = S.bg ? make_float4(S.bg[0], S.bg[1], S.bg[2], S.bg[3]) : make_float4(0.f, 0.f, 0.f, 0.f);
        for (int i = threadIdx.x; i < rows * S.canvas_w; i += THREADS) {
            const int r = i / S.canvas_w, x = i - r * S.canvas_w;
            canvas4[(int64_t)r * S.canvas_stride + x] = v;
        }
    }
    for (uint32_t fi = 0; fi < S.n_fills; ++fi) {
        const FillDev& f = S.fills[fi];
        if (band < f.band0 || band >= f.band0 + f.nbands) continue;
        // no lists (small scenes): every band takes every line, dropping those whose rows miss it
        const bool all = S.pairs == nullptr;
        const uint32_t e = f.entry0 + (band - f.band0);
        const uint32_t n = all ? scene_lines(S) : S.entry_count[e];
        if (n == 0) continue;  // full-width bands: no line, no coverage
        Band B;
        B.acc = cov;
        B.stride = band_stride(f.clip_width);
        B.bh = rows;
        B.y0 = row_base - f.row0;  // local row of band row 0
        B.img_h = f.height;
        B.width_f = (float)f.clip_width;
        B.width_i = f.clip_width;
        __syncthreads();  // previous fill done with the band (and its paint record)
        if (paint_mode) {
            // the fill's paint record in shared memory: read by every covered pixel
            const uint32_t* src = reinterpret_cast<const uint32_t*>(S.paints + f.paint);
            uint32_t* dst = reinterpret_cast<uint32_t*>(&s_paint);
            for (int i = threadIdx.x; i < (int)(sizeof(PaintDev) / 4); i += THREADS) dst[i] = src[i];
        }
        const int n4 = (rows * B.stride) >> 2;
        for (int i = threadIdx.x; i < n4; i += THREADS) sm4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        __syncthreads();
        const uint32_t start = all ? 0u : S.entry_start[e];
        // Lines that need the binary64 route (long, or at the x rules) are queued per warp and taken 32 at a
        // time, so the slow route runs with full warps instead of a few lanes of every step.
        uint32_t* q = s_slow[threadIdx.x >> 5];
        int nq = 0;
        auto queue_slow = [&](bool slow, uint32_t l) {  // (warp-uniform call)
            const unsigned m = __ballot_sync(0xffffffffu, slow);
            if (slow) q[nq + __popc(m & ((1u << lane) - 1u))] = l;
            nq += __popc(m);
            if (nq >= 32) {
                __syncwarp();
                nq -= 32;
                composite_slow_line(S, B, q[nq + lane]);
                __syncwarp();
            }
        };
        if (all) {
            // every line of the scene (n is at most the line capacity): most miss the band, so only the two
            // row words are read first, four lines a thread at once, and the rest of a line only if it is near
            constexpr int kU = 4;
            for (uint32_t j0 = threadIdx.x & ~31u; j0 < n; j0 += kU * THREADS) {
                int32_t ya[kU], yb[kU];
                #pragma unroll
                for (int u = 0; u < kU; ++u) {
                    const uint32_t j = j0 + (uint32_t)u * THREADS + lane;
                    ya[u] = yb[u] = INT32_MIN;
                    if (j < n) {
                        ya[u] = S.lines[2ull * j].y;
                        yb[u] = S.lines[2ull * j + 1].y;
                    }
                }
                #pragma unroll
                for (int u = 0; u < kU; ++u) {
                    const uint32_t j = j0 + (uint32_t)u * THREADS + lane;
                    const int ra = (ya[u] >> 16) - B.y0, rb = (yb[u] >> 16) - B.y0;
                    bool slow = false;
                    if (j < n && min(ra, rb) <= rows + 1 && max(ra, rb) >= -2)
                        slow = !accumulate_vtx_short(B, line_vtx(S.lines[2ull * j], B.y0),
                                                     line_vtx(S.lines[2ull * j + 1], B.y0));
                    queue_slow(slow, j);
                }
            }
        } else {
            for (uint32_t j0 = threadIdx.x & ~31u; j0 < n; j0 += THREADS) {
                const uint32_t j = j0 + lane;
                uint32_t l = 0;
                bool slow = false;
                // slots and lines beyond the buffers (reported by the earlier passes) are skipped
                if (j < n && start + j < S.pair_cap) l = S.pairs[start + j];
                if (j < n && start + j < S.pair_cap && l < S.line_cap) {
                    const int4 a = S.lines[2ull * l], b = S.lines[2ull * l + 1];
                    slow = !accumulate_vtx_short(B, line_vtx(a, B.y0), line_vtx(b, B.y0));
                }
                queue_slow(slow, l);
            }
        }
        __syncwarp();
        if (lane < nq) composite_slow_line(S, B, q[lane]);
        __syncthreads();
        if (paint_mode) {
            BlendEpi epi{canvas4 + f.col0, S.canvas_stride, f.col0, B.y0, f.width, &s_paint};
            band_scan<THREADS>(B, f.width, f.rule, epi);
        } else {
            AlphaEpi epi{S.canvas, S.canvas_stride, row_base, f.col0, f.width};
            band_scan<THREADS>(B, f.width, f.rule, epi);
        }
    }
    if (paint_mode && S.rgba8) {
        __syncthreads();  // the block's blends are visible to the block
        // fused output encode: From<LinColor> for RGBA per pixel, 4 bytes out instead of 16
        uint32_t* o = S.rgba8 + (int64_t)row_base * S.canvas_w;
        for (int i = threadIdx.x; i < rows * S.canvas_w; i += THREADS) {
            const int r = i / S.canvas_w, x = i - r * S.canvas_w;
            __stcs(o + i, encode_lin_rgba8(canvas4[(int64_t)r * S.canvas_stride + x]));
        }
    }
}

// ---------------------------------------------------------------------------
// launchers (declared in rz_api.cu)
// ---------------------------------------------------------------------------
cudaError_t launch_flatten_count(const SceneDev& S, cudaStream_t st) {
    const uint64_t n = scene_tasks(S);
    if (n == 0) return cudaSuccess;
    k_flatten_count<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(S);
    return cudaGetLastError();
}

cudaError_t launch_flatten_emit(const SceneDev& S, cudaStream_t st) {
    const uint64_t n = scene_tasks(S);
    if (n == 0) return cudaSuccess;
    k_flatten_emit<<<(unsigned)((n + kEmitThreads - 1) / kEmitThreads), kEmitThreads, 0, st>>>(S);
    return cudaGetLastError();
}

cudaError_t launch_flatten_emit_alloc(const SceneDev& S, uint32_t* n_lines, cudaStream_t st) {
    const uint64_t n = scene_tasks(S);
    if (n == 0) return cudaSuccess;
    k_flatten_emit_alloc<<<(unsigned)((n + kEmitThreads - 1) / kEmitThreads), kEmitThreads, 0, st>>>(S, n_lines);
    return cudaGetLastError();
}

cudaError_t launch_bin_scatter(const SceneDev& S, cudaStream_t st) {
    if (S.n_lines == 0) return cudaSuccess;
    k_bin_scatter<<<(S.n_lines + kBinLines - 1) / kBinLines, kBinThreads, 0, st>>>(S);
    return cudaGetLastError();
}

// Shared memory of the composite for a canvas width / band height / max view clip width.
int composite_smem_bytes(int canvas_w, int band_rows, int max_clip_width, bool paint_mode, int* cov_stride) {
    const int stride = band_stride(max_clip_width);
    *cov_stride = stride;
    (void)canvas_w;
    (void)paint_mode;
    return 4 * band_rows * stride;
}

// The shared-memory attribute is per device and kernel: the largest size set
// so far on each device (contexts on several GPUs, host threads calling at once).
constexpr int kMaxAttrDevices = 64;
static std::atomic<int> g_composite_smem[2][kMaxAttrDevices];

template <int THREADS>
static cudaError_t launch_composite_t(const SceneDev& S, int cov_stride, int smem, cudaStream_t st,
                                      std::atomic<int>* attr) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::atomic<int>* configured = dev >= 0 && dev < kMaxAttrDevices ? &attr[dev] : nullptr;
    if (!configured || smem > configured->load()) {
        e = cudaFuncSetAttribute(k_composite<THREADS>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        if (configured) {
            int cur = configured->load();
            while (smem > cur && !configured->compare_exchange_weak(cur, smem)) {
            }
        }
    }
    k_composite<THREADS><<<S.n_bands, THREADS, smem, st>>>(S, cov_stride);
    return cudaGetLastError();
}

cudaError_t launch_composite(const SceneDev& S, int cov_stride, int smem, cudaStream_t st) {
    if (S.paints) return launch_composite_t<256>(S, cov_stride, smem, st, g_composite_smem[0]);
    return launch_composite_t<512>(S, cov_stride, smem, st, g_composite_smem[1]);
}

}  // namespace rz
