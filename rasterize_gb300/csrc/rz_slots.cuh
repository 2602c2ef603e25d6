// rz_slots.cuh -- segment slots of a path batch as the batch kernels see them.
//
// A batch's flatten slots are its segments, then one closing line per subpath
// (src/path.rs:776-786).  This header holds what the band kernel (rz_band.cu)
// and the glyph pipeline (rz_glyph.cu) share: loading and transforming a slot,
// its fixed-point record (SlotRec, built once per launch), and the binary64
// walks of the rare slots the fixed-point route cannot take (raw arcs of
// device-memory batches, coordinates beyond 16.16).
#pragma once
#include "rz_arc.cuh"
#include "rz_device.cuh"
#include "rz_kernels.cuh"

namespace rz {

__device__ __forceinline__ void set_err(int32_t* err, int code) { atomicCAS(err, 0, code); }

// Flattens one reference segment (already transformed) into the band by a
// thread-serial walk (arcs of device-memory inputs, segments beyond the
// fixed-point range).  Kept out of line: it is the rare path.
static __device__ __noinline__ void band_segment(const BatchDev& b, const Band& B, const Seg64& s, int& fallbacks) {
    const int n = seg_npts(s.kind);
    double ymin = s.y[0], ymax = s.y[0];
    bool nan = false;
    for (int i = 0; i < n; ++i) {
        nan |= isnan(s.x[i]) || isnan(s.y[i]);
        ymin = fmin(ymin, s.y[i]);
        ymax = fmax(ymax, s.y[i]);
    }
    if (nan) {  // the reference panics on NaN (src/path.rs:765-767)
        set_err(b.err, ERR_NAN);
        return;
    }
    const double oy = (double)B.y0;
    if (ymax < oy - 1.0 || ymin > oy + (double)B.bh + 1.0) return;  // the curve stays in its hull
    const FlatCoef c = flat_coef(s);
    const VertexCoef v = vertex_coef(s);
    TreeWalk w;
    w.start();
    double px = v.p0x, py = v.p0y - oy;
    while (!w.done) {
        if (!node_is_leaf(s, c, w.d, w.k, b.thr64, b.thr32, fallbacks)) {
            if (w.d >= MAX_DEPTH) { set_err(b.err, ERR_DEPTH); return; }
            ++w.d;
            w.k <<= 1;
            continue;
        }
        double qx, qy;
        vertex_big(v, w.k + 1u, w.d, oy, qx, qy);
        accumulate_line64(B, px, py, qx, qy);
        px = qx;
        py = qy;
        w.next_after_leaf();
    }
}

__device__ inline void transform_seg(Seg64& s, const double* m) {
    if (!m) return;
    for (int i = 0; i < seg_npts(s.kind); ++i) tr_apply64(m, s.x[i], s.y[i], s.x[i], s.y[i]);
}

// Start (first=true) or end point of a subpath as PathFlattenIter sees it:
// the first / last reference segment after arc expansion.
static __device__ bool subpath_point(const BatchDev& b, uint32_t s0, uint32_t s1, bool first, double& x, double& y) {
    Seg64 tmp[4];
    if (first) {
        for (uint32_t i = s0; i < s1; ++i) {
            const int n = expand_segment(b.kind[i], b.pts + 8ull * i, tmp);
            if (n > 0) { x = tmp[0].x[0]; y = tmp[0].y[0]; return true; }
        }
    } else {
        for (uint32_t i = s1; i > s0; --i) {
            const int n = expand_segment(b.kind[i - 1], b.pts + 8ull * (i - 1), tmp);
            if (n > 0) {
                const Seg64& l = tmp[n - 1];
                const int k = seg_npts(l.kind) - 1;
                x = l.x[k];
                y = l.y[k];
                return true;
            }
        }
    }
    return false;
}

// An input ARC (device-memory batches): expand in binary64 and walk serially.
static __device__ __noinline__ void band_arc(const BatchDev& b, const Band& B, uint32_t g, const double* trm,
                                      int& fallbacks) {
    Seg64 parts[4];
    const int np = expand_segment(SEG_ARC, b.pts + 8ull * g, parts);
    if (np < 0) set_err(b.err, ERR_ARC);
    for (int j = 0; j < np; ++j) {
        transform_seg(parts[j], trm);
        band_segment(b, B, parts[j], fallbacks);
    }
}

struct SlotCoef {
    FlatCoef c;
    float qerr;
};

// Band-kernel decision: coefficients cached per segment slot.
__device__ __forceinline__ int decide_slot(const BatchDev& b, const SegRec& r, const SlotCoef& sc, int d, uint32_t k,
                                           const double* trm, int& fallbacks) {
    return decide_node(r, sc.c, sc.qerr, d, k, b.thr32, b.thr64, b.pts, trm, fallbacks);
}

// Kinds of an input slot after the transform (slot_points).
enum : int { SLOT_EMPTY = 0, SLOT_FIX = 1, SLOT_ARC = 2, SLOT_BIG = 3, SLOT_NAN = 4 };

// Input slot `idx`: segment idx (closing == false) or the closing line of
// subpath idx, Line(subpath.end(), subpath.start()) (src/path.rs:776-786),
// transformed by trm.  SLOT_FIX: F is the 16.16 copy of the binary64 points
// sx, sy; SLOT_BIG: a point lies beyond the 16.16 range; SLOT_ARC: a raw arc
// (device-memory input); SLOT_EMPTY: a subpath without segments.
__device__ __forceinline__ int slot_points(const BatchDev& b, uint32_t idx, bool closing, const double* trm,
                                           FixSeg& F, double (&sx)[4], double (&sy)[4], uint32_t& src) {
    F.kind = SEG_LINE;
    src = 0xffffffffu;  // input segment (binary64 re-decisions); none for closing lines
    int npts = 0;
    if (!closing) {
        const int kind = b.kind[idx];
        if (kind == SEG_ARC) return SLOT_ARC;
        F.kind = kind;
        npts = seg_npts(kind);
        const double2* p2 = reinterpret_cast<const double2*>(b.pts + 8ull * idx);
        #pragma unroll
        for (int j = 0; j < 4; ++j) {
            const double2 q = __ldg(p2 + j);
            sx[j] = q.x;
            sy[j] = q.y;
        }
        src = idx;
    } else {
        const uint32_t s1 = min(b.sub_off[idx + 1], b.n_segments);
        const uint32_t s0 = b.sub_off[idx];
        if (s1 > s0 && subpath_point(b, s0, s1, false, sx[0], sy[0]) && subpath_point(b, s0, s1, true, sx[1], sy[1]))
            npts = 2;
    }
    if (!npts) return SLOT_EMPTY;
    bool nan = false, fits = true;
    #pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (j < npts) {
            if (trm) tr_apply64(trm, sx[j], sy[j], sx[j], sy[j]);
            nan |= is_nan_bits(sx[j]) || is_nan_bits(sy[j]);
            fits &= d2fix(sx[j], F.x[j]) & d2fix(sy[j], F.y[j]);
        } else {
            F.x[j] = F.y[j] = 0;
            sx[j] = sy[j] = 0.0;
        }
    }
    if (nan) return SLOT_NAN;
    return fits ? SLOT_FIX : SLOT_BIG;
}

// Loads input segment slot i of a work item (segments, then one closing line
// per subpath), transforms it and, when it lies in the fixed-point range and
// its hull meets the band's rows, writes its record and decision
// coefficients.  Arcs and segments beyond the range are flattened here by the
// binary64 walk.  Kept out of line: its binary64 temporaries would otherwise
// compete for registers with the tree walk.
static __device__ __noinline__ bool band_load(const BatchDev& b, const Band& B, uint32_t seg0, uint32_t n_seg,
                                              uint32_t sub0, uint32_t i, const double* trm, SegRec& rec,
                                              SlotCoef& coef, int& fallbacks) {
    const bool closing = i >= n_seg;
    const uint32_t idx = closing ? sub0 + (i - n_seg) : seg0 + i;
    FixSeg F;
    double sx[4], sy[4];
    uint32_t src;
    const int kind = slot_points(b, idx, closing, trm, F, sx, sy, src);
    if (kind == SLOT_ARC) {
        band_arc(b, B, idx, trm, fallbacks);  // device-memory input with raw arcs
    } else if (kind == SLOT_NAN) {
        set_err(b.err, ERR_NAN);  // the reference panics on NaN (src/path.rs:765-767)
    } else if (kind == SLOT_BIG) {
        Seg64 S;  // beyond the fixed-point range: binary64 walk
        S.kind = F.kind;
        #pragma unroll
        for (int j = 0; j < 4; ++j) { S.x[j] = sx[j]; S.y[j] = sy[j]; }
        band_segment(b, B, S, fallbacks);
    } else if (kind == SLOT_FIX && hull_meets_rows(F, B.y0, B.bh)) {
        make_record(F, sx, sy, rec);
        rec.src = src;
        coef.c = rec_flat(rec, coef.qerr);
        return true;
    }
    return false;
}

// ---------------------------------------------------------------------------
// Slot records
//
// A path's segments are the same for every band of its mask, so their
// records are built once per launch by k_band_records (one thread per slot,
// no barriers) instead of once per band.  Record j < n_segments is segment
// j, record n_segments + s the closing line of subpath s.  A band copies the
// 96-byte records of its path into shared memory and keeps those whose hull
// meets its rows.  Slots the fixed-point route cannot take (arcs, segments
// beyond 16.16, NaN) are marked slow and go through band_load as before;
// so are records built with another path's transform (offsets that put a
// segment into two paths).
// ---------------------------------------------------------------------------
struct __align__(16) SlotRec {
    SegRec rec;          // bytes 0-59
    uint32_t tag;        // state << 30 | owning path (kAnyPath: no transforms)
    SlotCoef coef;       // bytes 64-87
    int32_t ymin, ymax;  // control hull rows, 16.16
};
static_assert(sizeof(SegRec) == 60 && sizeof(SlotCoef) == 24 && sizeof(SlotRec) == 96, "record layout");

constexpr uint32_t kAnyPath = 0x3fffffffu;
enum : uint32_t { REC_FIX = 0, REC_EMPTY = 1, REC_SLOW = 2 };

// Largest k < n with a[k] <= v (0 when there is none): the range of a
// non-decreasing offset array that holds v.
__device__ __forceinline__ uint32_t last_le(const uint32_t* a, uint32_t n, uint32_t v) {
    uint32_t lo = 0, hi = n;  // answer in [lo, hi)
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (a[mid] <= v) lo = mid; else hi = mid;
    }
    return lo;
}

// The record of slot j (j < n_segments: segment j; else the closing line of
// subpath j - n_segments), built with the transform of its owning path.
// Returns the slot's kind (SLOT_*).
__device__ __forceinline__ int build_slot_record(const BatchDev& b, uint32_t j, SlotRec& r) {
    const bool closing = j >= b.n_segments;
    const uint32_t idx = closing ? j - b.n_segments : j;
    uint32_t owner = kAnyPath;
    const double* trm = nullptr;
    if (b.tr && b.n_paths) {
        const uint32_t sub = closing ? idx : last_le(b.sub_off, b.n_subpaths + 1, idx);
        owner = min(last_le(b.path_sub, b.n_paths + 1, sub), b.n_paths - 1);
        trm = b.tr + 6ull * owner;
    }
    FixSeg F;
    double sx[4], sy[4];
    uint32_t src;
    const int kind = slot_points(b, idx, closing, trm, F, sx, sy, src);
    uint32_t state = REC_SLOW;
    int32_t ymin = 0, ymax = 0;
    if (kind == SLOT_EMPTY) {
        state = REC_EMPTY;
    } else if (kind == SLOT_FIX) {
        state = REC_FIX;
        make_record(F, sx, sy, r.rec);
        r.rec.src = src;
        r.coef.c = rec_flat(r.rec, r.coef.qerr);
        ymin = ymax = F.y[0];
        #pragma unroll
        for (int i = 1; i < 4; ++i) {
            if (i < seg_npts(F.kind)) {
                ymin = min(ymin, F.y[i]);
                ymax = max(ymax, F.y[i]);
            }
        }
    }
    if (state != REC_FIX) {
        r.rec = SegRec{};
        r.coef = SlotCoef{};
    }
    r.tag = state << 30 | owner;
    r.ymin = ymin;
    r.ymax = ymax;
    return kind;
}

}  // namespace rz
