// rz_band.cu -- the persistent band kernel: flatten + signed-area coverage +
// row prefix + fill rule for many independent paths in one launch.
//
// Work items are (path, band of rows); a CTA pulls items from a device queue
// (an atomic head counter), so thousands of uneven paths balance across the
// 152 SMs.  Per item the CTA clears a shared-memory accumulation band
// (rows x (clip_width + 3) floats), every thread walks the bisection trees of
// a strided subset of the path's segments (skipping segments whose control
// hull misses the band), accumulates signed area differences with shared
// atomics, and finally one warp per row runs a two-sum compensated prefix
// scan, applies the fill rule and streams the row to HBM with float4 stores.
// Nothing but the masks themselves is written to global memory.
#include "rz_arc.cuh"
#include "rz_device.cuh"
#include "rz_kernels.cuh"

namespace rz {

__device__ __forceinline__ void set_err(int32_t* err, int code) { atomicCAS(err, 0, code); }

// Flattens one reference segment (already transformed) into the band by a
// thread-serial walk (arcs of device-memory inputs, segments beyond the
// fixed-point range).  Kept out of line: it is the rare path.
__device__ __noinline__ void band_segment(const BatchDev& b, const Band& B, const Seg64& s, int& fallbacks) {
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
    if (v.small) {
        const double ox = floor(v.p0x);
        const int oxi = (int)ox;
        const float p0rx = (float)(v.p0x - ox), p0ry = (float)(v.p0y - oy);
        float px = p0rx, py = p0ry;
        while (!w.done) {
            if (!node_is_leaf(s, c, w.d, w.k, b.thr64, b.thr32, fallbacks)) {
                if (w.d >= MAX_DEPTH) { set_err(b.err, ERR_DEPTH); return; }
                ++w.d;
                w.k <<= 1;
                continue;
            }
            float qx, qy;
            vertex_small(v, w.k + 1u, w.d, ox, oy, p0rx, p0ry, qx, qy);
            accumulate_line(B, oxi, px, py, qx, qy);
            px = qx;
            py = qy;
            w.next_after_leaf();
        }
    } else {
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
}

__device__ inline void transform_seg(Seg64& s, const double* m) {
    if (!m) return;
    for (int i = 0; i < seg_npts(s.kind); ++i) tr_apply64(m, s.x[i], s.y[i], s.x[i], s.y[i]);
}

// Start (first=true) or end point of a subpath as PathFlattenIter sees it:
// the first / last reference segment after arc expansion.
__device__ bool subpath_point(const BatchDev& b, uint32_t s0, uint32_t s1, bool first, double& x, double& y) {
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
__device__ __noinline__ void band_arc(const BatchDev& b, const Band& B, uint32_t g, const double* trm,
                                      int& fallbacks) {
    Seg64 parts[4];
    const int np = expand_segment(SEG_ARC, b.pts + 8ull * g, parts);
    if (np < 0) set_err(b.err, ERR_ARC);
    for (int j = 0; j < np; ++j) {
        transform_seg(parts[j], trm);
        band_segment(b, B, parts[j], fallbacks);
    }
}

// Warp scan of one band row: two-sum compensated prefix of the signed
// differences, fill rule, coalesced store (src/rasterize.rs:473-507).
__device__ void scan_row_store(const float* row, int width, int rule, float* out_row, bool vec_ok) {
    const int lane = threadIdx.x & 31;
    float cs = 0.f, ce = 0.f;  // running (sum, error) carried across chunks
    for (int c0 = 0; c0 < width; c0 += 128) {
        const int c = c0 + 4 * lane;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (c + 3 < width) {
            v = *reinterpret_cast<const float4*>(row + c);
        } else {
            if (c < width) v.x = row[c];
            if (c + 1 < width) v.y = row[c + 1];
            if (c + 2 < width) v.z = row[c + 2];
        }
        // local inclusive prefix (two-sum)
        float s1, e1, s2, e2, s3, e3;
        two_sum(v.x, v.y, s1, e1);
        two_sum(s1, v.z, s2, e2);
        e2 += e1;
        two_sum(s2, v.w, s3, e3);
        e3 += e2;
        // warp inclusive scan of lane totals
        float ts = s3, te = e3;
        #pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const float os = __shfl_up_sync(0xffffffffu, ts, off);
            const float oe = __shfl_up_sync(0xffffffffu, te, off);
            if (lane >= off) {
                float ns, ne;
                two_sum(os, ts, ns, ne);
                ts = ns;
                te = oe + te + ne;
            }
        }
        float xs = __shfl_up_sync(0xffffffffu, ts, 1);
        float xe = __shfl_up_sync(0xffffffffu, te, 1);
        if (lane == 0) { xs = 0.f; xe = 0.f; }
        // base = carry + exclusive lane prefix
        float bs, be;
        two_sum(cs, xs, bs, be);
        be += ce + xe;
        float w0s, w0e, w1s, w1e, w2s, w2e, w3s, w3e;
        two_sum(bs, v.x, w0s, w0e);
        two_sum(bs, s1, w1s, w1e);
        two_sum(bs, s2, w2s, w2e);
        two_sum(bs, s3, w3s, w3e);
        float4 a;
        a.x = alpha_from_winding(rule, w0s + (w0e + be));
        a.y = alpha_from_winding(rule, w1s + (w1e + be + e1));
        a.z = alpha_from_winding(rule, w2s + (w2e + be + e2));
        a.w = alpha_from_winding(rule, w3s + (w3e + be + e3));
        if (vec_ok && c + 3 < width) {
            __stcs(reinterpret_cast<float4*>(out_row + c), a);
        } else {
            if (c < width) out_row[c] = a.x;
            if (c + 1 < width) out_row[c + 1] = a.y;
            if (c + 2 < width) out_row[c + 2] = a.z;
            if (c + 3 < width) out_row[c + 3] = a.w;
        }
        // carry += warp total
        const float tot_s = __shfl_sync(0xffffffffu, ts, 31);
        const float tot_e = __shfl_sync(0xffffffffu, te, 31);
        float ns, ne;
        two_sum(cs, tot_s, ns, ne);
        cs = ns;
        ce = ce + tot_e + ne;
    }
}

// ---------------------------------------------------------------------------
// Leaf-parallel flattening
//
// Per work item the CTA takes the path's segments 256 at a time.  Every thread
// turns its segment into a record in shared memory and walks the bisection
// tree with FP32 decisions; each leaf it finds is appended (one shared atomic)
// to a leaf buffer as (segment slot, depth, index).  When the buffer is full,
// or every walk has ended, all threads drain it together: a leaf's two end
// vertices are evaluated from the record (FP32 relative to the record's
// integer origin for small segments, binary64 otherwise) and the line's signed
// area is accumulated into the band.  Shared vertices of neighbouring leaves
// are evaluated by the same expression on the same dyadic t, so they agree
// bit for bit and windings telescope.
// ---------------------------------------------------------------------------
struct SegRec {
    int32_t xb;      // integer column origin (floor of P0.x)
    int16_t anchor;  // anchor level a: vertices are B(m / 2^a) exactly plus an FP32 remainder
    int16_t kind;
    int32_t p0x, p0y, pnx, pny;           // 16.16, relative to (xb, band row y0)
    int32_t d1x, d1y, d2x, d2y, d3x, d3y;  // control point differences, 16.16
    float mag;                            // max |absolute coordinate|, px (binary64 chain error term)
    uint32_t src;                         // input segment, for binary64 re-decisions (~0: a line)
};

struct LeafCode {
    uint32_t k;
    uint16_t slot;
    uint16_t d;
};

constexpr int kThreads = 256;
constexpr int kLeafCap = 1024;  // >= the widest breadth-first level that can end in leaves
constexpr int kSpreadDepth = 2;                      // levels expanded breadth-first by the whole CTA
constexpr int kLevelCap = kThreads << kSpreadDepth;  // nodes per breadth-first level
constexpr int kBandBytes = 36 * 1024;
constexpr int kBandFloats = kBandBytes / 4;
constexpr int kChunk = 16;  // pixels per thread in the row scan
struct SlotCoef {
    FlatCoef c;
    float qerr;
};
constexpr int kSmemBytes = kBandBytes + kThreads * (int)sizeof(SegRec) + kThreads * (int)sizeof(SlotCoef) +
                           kLeafCap * (int)sizeof(LeafCode) + 2 * kLevelCap * (int)sizeof(uint32_t);
static_assert(kLeafCap * (int)sizeof(LeafCode) >= (kBandFloats / kChunk) * (int)sizeof(float),
              "the leaf buffer doubles as the chunk-total array of the scan");

// Power-basis coefficients in px: B(t) - P0 = t (c1 + t (c2 + t c3)).  For a
// cubic c2 and c3 are also the flatness coefficients a2 and a3; for a quad c2
// is P0 - 2 P1 + P2.
__device__ __forceinline__ void rec_coefs(const SegRec& r, int kind, float& c1x, float& c1y, float& c2x, float& c2y,
                                          float& c3x, float& c3y) {
    const float d1x = (float)r.d1x * FIX_ONE_INV, d1y = (float)r.d1y * FIX_ONE_INV;
    const float d2x = (float)r.d2x * FIX_ONE_INV, d2y = (float)r.d2y * FIX_ONE_INV;
    const float d3x = (float)r.d3x * FIX_ONE_INV, d3y = (float)r.d3y * FIX_ONE_INV;
    if (kind == SEG_CUBIC) {
        c1x = 3.f * d1x; c1y = 3.f * d1y;
        c2x = 3.f * (d2x - d1x); c2y = 3.f * (d2y - d1y);
        c3x = (d1x - 2.f * d2x) + d3x; c3y = (d1y - 2.f * d2y) + d3y;
    } else if (kind == SEG_QUAD) {
        c1x = 2.f * d1x; c1y = 2.f * d1y;
        c2x = d2x - d1x; c2y = d2y - d1y;
        c3x = c3y = 0.f;
    } else {
        c1x = d1x; c1y = d1y;
        c2x = c2y = c3x = c3y = 0.f;
    }
}

// Decision coefficients of a record and the bound of their error against the
// binary64 control points (16.16 quantisation, 2^-17 px per coordinate, plus
// FP32 rounding).
__device__ __forceinline__ FlatCoef rec_flat(const SegRec& r, float& qerr) {
    float c1x, c1y, c2x, c2y, c3x, c3y;
    rec_coefs(r, r.kind, c1x, c1y, c2x, c2y, c3x, c3y);
    FlatCoef c;
    c.a2x = c2x; c.a2y = c2y; c.a3x = c3x; c.a3y = c3y;
    c.mag = r.mag;
    const float sx = fabsf((float)r.d1x) + fabsf((float)r.d2x) + fabsf((float)r.d3x);
    const float sy = fabsf((float)r.d1y) + fabsf((float)r.d2y) + fabsf((float)r.d3y);
    qerr = ldexpf(fmaxf(sx, sy) * FIX_ONE_INV, -19) + 12.f * ldexpf(1.f, -17);
    return c;
}

// Builds the leaf-drain record of fixed-point segment `s` for the band; false
// when its control hull misses the band rows.
__device__ inline bool make_record(const Band& B, const FixSeg& s, SegRec& r) {
    int32_t ymin = s.y[0], ymax = s.y[0];
    #pragma unroll
    for (int i = 1; i < 4; ++i) {
        if (i < seg_npts(s.kind)) {
            ymin = min(ymin, s.y[i]);
            ymax = max(ymax, s.y[i]);
        }
    }
    const int32_t oy = B.y0 << 16;  // heights are limited to 16383 rows
    if (ymax < oy - 65536 || ymin > oy + ((B.bh + 1) << 16)) return false;
    const int n = seg_npts(s.kind);
    const int32_t xb = s.x[0] >> 16;  // floor
    const int32_t ox = xb << 16;
    r.xb = xb;
    r.p0x = s.x[0] - ox;
    r.p0y = s.y[0] - oy;
    r.pnx = s.x[n - 1] - ox;
    r.pny = s.y[n - 1] - oy;
    r.d1x = s.x[1] - s.x[0];
    r.d1y = s.y[1] - s.y[0];
    r.d2x = n > 2 ? s.x[2] - s.x[1] : 0;
    r.d2y = n > 2 ? s.y[2] - s.y[1] : 0;
    r.d3x = n > 3 ? s.x[3] - s.x[2] : 0;
    r.d3y = n > 3 ? s.y[3] - s.y[2] : 0;
    float c1x, c1y, c2x, c2y, c3x, c3y;
    rec_coefs(r, s.kind, c1x, c1y, c2x, c2y, c3x, c3y);
    // Anchor level: sub-curves over 2^-a of the parameter span stay below ~32 px,
    // so the FP32 remainder keeps ~1e-5 px.  Lines need no anchors (t is 0 or 1).
    const float ext = fmaxf(fabsf(c1x) + fabsf(c2x) + fabsf(c3x), fabsf(c1y) + fabsf(c2y) + fabsf(c3y));
    int a = 0;
    if (s.kind != SEG_LINE) {
        while (a < 9 && ldexpf(ext, -a) > 32.f) ++a;
    }
    int32_t mx = 0;
    #pragma unroll
    for (int i = 0; i < 4; ++i) mx = max(mx, max(abs(s.x[i]), abs(s.y[i])));  // unused points are 0
    r.mag = (float)mx * FIX_ONE_INV;
    r.anchor = (int16_t)a;
    r.kind = (int16_t)s.kind;
    return true;
}

// Vertex at t = j / 2^d as an exact 16.16 point A (relative to the record's
// origin) plus an FP32 remainder D in px.  The anchor depends on t only, so
// two leaves sharing a vertex compute it identically.
__device__ __forceinline__ void rec_vertex(const SegRec& r, uint32_t j, int d, int32_t& ax, int32_t& ay, float& dx,
                                           float& dy) {
    if (j == 0) {
        ax = r.p0x; ay = r.p0y; dx = dy = 0.f;
        return;
    }
    if ((j >> d) != 0u) {
        ax = r.pnx; ay = r.pny; dx = dy = 0.f;
        return;
    }
    const int a = r.anchor;
    float c1x, c1y, c2x, c2y, c3x, c3y;
    rec_coefs(r, r.kind, c1x, c1y, c2x, c2y, c3x, c3y);
    if (a == 0) {
        const float t = ldexpf((float)j, -d);
        ax = r.p0x; ay = r.p0y;
        dx = t * fmaf(t, fmaf(t, c3x, c2x), c1x);
        dy = t * fmaf(t, fmaf(t, c3y, c2y), c1y);
        return;
    }
    // anchor m / 2^a <= t, exact B(m / 2^a) from integer power-basis coefficients
    const uint32_t m = d >= a ? (j >> (d - a)) : (j << (a - d));
    const uint32_t jm = d >= a ? (m << (d - a)) : j;
    const long long mm = (long long)m;
    // integer power basis: B(t) - P0 = t (k1 + t (k2 + t k3)) in 16.16 units
    long long k1x, k1y, k2x, k2y, k3x, k3y;
    if (r.kind == SEG_CUBIC) {
        k1x = 3ll * r.d1x; k1y = 3ll * r.d1y;
        k2x = 3ll * ((long long)r.d2x - r.d1x); k2y = 3ll * ((long long)r.d2y - r.d1y);
        k3x = (long long)r.d1x - 2ll * r.d2x + r.d3x; k3y = (long long)r.d1y - 2ll * r.d2y + r.d3y;
    } else {  // quad (lines never reach here: their vertices are end points)
        k1x = 2ll * r.d1x; k1y = 2ll * r.d1y;
        k2x = (long long)r.d2x - r.d1x; k2y = (long long)r.d2y - r.d1y;
        k3x = k3y = 0;
    }
    const long long s1 = 1ll << a, s2 = 1ll << (2 * a);
    const long long nx = ((k3x * mm + k2x * s1) * mm + k1x * s2) * mm;
    const long long ny = ((k3y * mm + k2y * s1) * mm + k1y * s2) * mm;
    const int sh = 3 * a;
    const long long half = 1ll << (sh - 1);
    ax = r.p0x + (int32_t)((nx + half) >> sh);
    ay = r.p0y + (int32_t)((ny + half) >> sh);
    if (jm == j) {
        dx = dy = 0.f;
        return;
    }
    // remainder over dt = t - m / 2^a with the local power basis at tA
    const float tA = ldexpf((float)m, -a);
    const float dt = ldexpf((float)(j - jm), -d);
    const float b1x = fmaf(tA, fmaf(3.f * tA, c3x, 2.f * c2x), c1x);
    const float b1y = fmaf(tA, fmaf(3.f * tA, c3y, 2.f * c2y), c1y);
    const float b2x = fmaf(3.f * tA, c3x, c2x), b2y = fmaf(3.f * tA, c3y, c2y);
    dx = dt * fmaf(dt, fmaf(dt, c3x, b2x), b1x);
    dy = dt * fmaf(dt, fmaf(dt, c3y, b2y), b1y);
}

// Row prefix of the band (signed differences -> winding), fill rule and
// store (src/rasterize.rs:473-507).  Every thread owns 16-pixel chunks:
// 1) in-place inclusive prefix of each chunk, chunk totals to `tot`;
// 2) per row, an exclusive scan of the chunk totals (two-sum compensated
//    carry, so long rows keep ~1e-7 accuracy);
// 3) base + chunk prefix -> alpha, written to HBM with 16-byte stores.
__device__ void band_scan_store(const Band& B, const MaskDev& m, int rule, float* out, float* tot) {
    const int W = m.width;
    const int cr = (W + kChunk - 1) / kChunk;  // chunks per row
    const int nc = cr * B.bh;
    for (int c = threadIdx.x; c < nc; c += kThreads) {
        const int r = c / cr, x0 = (c - r * cr) * kChunk;
        float4* row4 = reinterpret_cast<float4*>(B.acc + r * B.stride + x0);
        float run = 0.f;
        #pragma unroll
        for (int q = 0; q < kChunk / 4; ++q) {
            float4 v = row4[q];  // stride >= width + 2 rounded to 4: in bounds; columns >= W are ignored
            const int x = x0 + 4 * q;
            if (x >= W) v.x = 0.f;
            if (x + 1 >= W) v.y = 0.f;
            if (x + 2 >= W) v.z = 0.f;
            if (x + 3 >= W) v.w = 0.f;
            v.x += run;
            v.y += v.x;
            v.z += v.y;
            v.w += v.z;
            run = v.w;
            row4[q] = v;
        }
        tot[c] = run;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    for (int r = threadIdx.x >> 5; r < B.bh; r += kThreads / 32) {
        float cs = 0.f, ce = 0.f;  // compensated carry across 32-chunk groups
        for (int q0 = 0; q0 < cr; q0 += 32) {
            const int q = q0 + lane;
            const float v = q < cr ? tot[r * cr + q] : 0.f;
            float incl = v;
            #pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const float o = __shfl_up_sync(0xffffffffu, incl, off);
                if (lane >= off) incl += o;
            }
            if (q < cr) tot[r * cr + q] = cs + (incl - v) + ce;  // exclusive base of the chunk
            const float group = __shfl_sync(0xffffffffu, incl, 31);
            float ns, ne;
            two_sum(cs, group, ns, ne);
            cs = ns;
            ce += ne;
        }
    }
    __syncthreads();
    for (int c = threadIdx.x; c < nc; c += kThreads) {
        const int r = c / cr, x0 = (c - r * cr) * kChunk;
        const float base = tot[c];
        const float4* row4 = reinterpret_cast<const float4*>(B.acc + r * B.stride + x0);
        float* o = out + m.offset + (uint64_t)(B.y0 + r) * (uint64_t)m.row_stride + x0;
        const bool vec = ((reinterpret_cast<uintptr_t>(o) & 15u) == 0) && (x0 + kChunk <= W);
        #pragma unroll
        for (int q = 0; q < kChunk / 4; ++q) {
            const float4 v = row4[q];
            float4 a;
            a.x = alpha_from_winding(rule, base + v.x);
            a.y = alpha_from_winding(rule, base + v.y);
            a.z = alpha_from_winding(rule, base + v.z);
            a.w = alpha_from_winding(rule, base + v.w);
            const int x = x0 + 4 * q;
            if (vec) {
                __stcs(reinterpret_cast<float4*>(o) + q, a);
            } else {
                if (x < W) o[4 * q] = a.x;
                if (x + 1 < W) o[4 * q + 1] = a.y;
                if (x + 2 < W) o[4 * q + 2] = a.z;
                if (x + 3 < W) o[4 * q + 3] = a.w;
            }
        }
    }
}

// Reference decision for node (d, k) of a record: FP32 with a rigorous bound,
// binary64 replay of the split chain when too close to call.
__device__ __forceinline__ int decide_node(const BatchDev& b, const SegRec& r, const SlotCoef& sc, int d, uint32_t k,
                                           const double* trm, int& fallbacks) {
    if (r.kind == SEG_LINE) return 1;
    const int v = decide_fp32(r.kind, sc.c, d, k, b.thr32, sc.qerr);
    if (v >= 0) return v;
    Seg64 S;
    S.kind = r.kind;
    const double* p = b.pts + 8ull * r.src;
    #pragma unroll
    for (int j = 0; j < 4; ++j) { S.x[j] = p[2 * j]; S.y[j] = p[2 * j + 1]; }
    transform_seg(S, trm);
    ++fallbacks;
    return flatness_chain64(S, d, k) < b.thr64 ? 1 : 0;
}

__device__ inline void drain_leaf(const Band& B, const SegRec* recs, const LeafCode c) {
    const SegRec& r = recs[c.slot];
    int32_t a0x, a0y, a1x, a1y;
    float d0x, d0y, d1x, d1y;
    rec_vertex(r, c.k, c.d, a0x, a0y, d0x, d0y);
    rec_vertex(r, c.k + 1u, c.d, a1x, a1y, d1x, d1y);
    if (abs(a1x - a0x) > (128 << 16) || abs(a1y - a0y) > (128 << 16)) {
        // long line (straight segments, closing lines): exact binary64 route
        const double u = 1.0 / 65536.0;
        accumulate_line64(B, (double)r.xb + (double)a0x * u + (double)d0x, (double)a0y * u + (double)d0y,
                          (double)r.xb + (double)a1x * u + (double)d1x, (double)a1y * u + (double)d1y);
        return;
    }
    // both ends relative to the integer column of the first anchor
    const int32_t cb = a0x >> 16;
    const int32_t base = cb << 16;
    const float x0 = (float)(a0x - base) * FIX_ONE_INV + d0x;
    const float x1 = (float)(a1x - base) * FIX_ONE_INV + d1x;
    const float y0 = (float)a0y * FIX_ONE_INV + d0y;
    const float y1 = (float)a1y * FIX_ONE_INV + d1y;
    accumulate_line(B, r.xb + cb, x0, y0, x1, y1);
}

// queue != nullptr: persistent CTAs pull items from the queue head;
// queue == nullptr: one item per CTA (item = blockIdx.x), the plain launch.
__global__ void __launch_bounds__(kThreads, 3) k_mask_bands(BatchDev b, const WorkItem* __restrict__ items, int n_items,
                                                        int32_t* queue) {
    extern __shared__ float4 smem4[];
    float* acc = reinterpret_cast<float*>(smem4);
    SegRec* recs = reinterpret_cast<SegRec*>(reinterpret_cast<char*>(smem4) + kBandBytes);
    SlotCoef* coefs = reinterpret_cast<SlotCoef*>(reinterpret_cast<char*>(recs) + kThreads * sizeof(SegRec));
    LeafCode* leaves = reinterpret_cast<LeafCode*>(reinterpret_cast<char*>(coefs) + kThreads * sizeof(SlotCoef));
    uint32_t* level[2];
    level[0] = reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(leaves) + kLeafCap * sizeof(LeafCode));
    level[1] = level[0] + kLevelCap;
    __shared__ int s_item;
    __shared__ int s_nleaf;
    __shared__ int s_nlevel[2];
    int fallbacks = 0;
    const int tid = threadIdx.x;
    for (int round = 0;; ++round) {
        if (tid == 0) {
            s_item = queue ? atomicAdd(queue, 1) : (round == 0 ? (int)blockIdx.x : n_items);
            s_nleaf = 0;
        }
        __syncthreads();
        const int it = s_item;
        if (it >= n_items) break;
        const WorkItem wi = items[it];
        const MaskDev m = b.masks[wi.path];
        Band B;
        B.acc = acc;
        B.stride = band_stride(m.clip_width);
        B.bh = wi.rows;
        B.y0 = wi.y0;
        B.img_h = m.height;
        B.width_f = (float)m.clip_width;
        B.width_i = m.clip_width;
        const int n4 = (B.bh * B.stride) >> 2;
        for (int i = tid; i < n4; i += kThreads) smem4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        __syncthreads();

        // ranges are clamped to the arrays so malformed offsets cannot read out of bounds
        const uint32_t sub1 = min(b.path_sub[wi.path + 1], b.n_subpaths);
        const uint32_t sub0 = min(b.path_sub[wi.path], sub1);
        const uint32_t seg1 = min(b.sub_off[sub1], b.n_segments);
        const uint32_t seg0 = min(b.sub_off[sub0], seg1);
        const uint32_t n_seg = seg1 - seg0, n_close = sub1 - sub0;
        const double* trm = b.tr ? b.tr + 6ull * wi.path : nullptr;
        for (uint32_t base = 0; base < n_seg + n_close; base += kThreads) {
            const uint32_t i = base + tid;
            bool active = false;
            FixSeg F;
            F.kind = SEG_LINE;
            uint32_t src = 0xffffffffu;  // input segment (binary64 re-decisions); none for closing lines
            double sx[4], sy[4];
            int npts = 0;
            if (i < n_seg) {
                const uint32_t g = seg0 + i;
                const int kind = b.kind[g];
                const double2* p2 = reinterpret_cast<const double2*>(b.pts + 8ull * g);
                if (kind == SEG_ARC) {
                    band_arc(b, B, g, trm, fallbacks);  // device-memory input with raw arcs
                } else {
                    F.kind = kind;
                    npts = seg_npts(kind);
                    #pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const double2 q = __ldg(p2 + j);
                        sx[j] = q.x;
                        sy[j] = q.y;
                    }
                    src = g;
                }
            } else if (i < n_seg + n_close) {
                // closing line Line(subpath.end(), subpath.start()).transform(tr) (src/path.rs:776-786)
                const uint32_t sp = sub0 + (i - n_seg);
                const uint32_t s1 = min(b.sub_off[sp + 1], b.n_segments);
                const uint32_t s0 = b.sub_off[sp];
                if (s1 > s0 && subpath_point(b, s0, s1, false, sx[0], sy[0]) &&
                    subpath_point(b, s0, s1, true, sx[1], sy[1])) {
                    F.kind = SEG_LINE;
                    npts = 2;
                }
            }
            if (npts) {
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
                if (nan) {  // the reference panics on NaN (src/path.rs:765-767)
                    set_err(b.err, ERR_NAN);
                } else if (!fits) {
                    // beyond the fixed-point range: binary64 walk
                    Seg64 S;
                    S.kind = F.kind;
                    #pragma unroll
                    for (int j = 0; j < 4; ++j) { S.x[j] = sx[j]; S.y[j] = sy[j]; }
                    band_segment(b, B, S, fallbacks);
                } else {
                    active = make_record(B, F, recs[tid]);
                    recs[tid].src = src;
                    if (active) coefs[tid].c = rec_flat(recs[tid], coefs[tid].qerr);
                }
            }
            // ---- breadth-first over the top levels of every tree, all threads together
            if (tid == 0) { s_nlevel[0] = 0; s_nlevel[1] = 0; }
            __syncthreads();
            if (active) level[0][atomicAdd(&s_nlevel[0], 1)] = (uint32_t)tid << 24;
            int cur = 0;
            for (int d = 0; d < kSpreadDepth; ++d) {
                __syncthreads();
                const int n = s_nlevel[cur];
                for (int j = tid; j < n; j += kThreads) {
                    const uint32_t node = level[cur][j];
                    const int slot = (int)(node >> 24);
                    const uint32_t k = node & 0xffffffu;
                    if (decide_node(b, recs[slot], coefs[slot], d, k, trm, fallbacks)) {
                        LeafCode lc;
                        lc.k = k;
                        lc.slot = (uint16_t)slot;
                        lc.d = (uint16_t)d;
                        leaves[atomicAdd(&s_nleaf, 1)] = lc;
                    } else {
                        const int q = atomicAdd(&s_nlevel[cur ^ 1], 2);
                        level[cur ^ 1][q] = node + k;          // (slot, 2k)
                        level[cur ^ 1][q + 1] = node + k + 1u;  // (slot, 2k + 1)
                    }
                }
                __syncthreads();
                // drain the leaves of this level
                const int nl = s_nleaf;
                for (int j = tid; j < nl; j += kThreads) drain_leaf(B, recs, leaves[j]);
                __syncthreads();
                if (tid == 0) {
                    s_nleaf = 0;
                    s_nlevel[cur] = 0;
                }
                cur ^= 1;
            }
            __syncthreads();
            // ---- the remaining subtrees (roots at depth kSpreadDepth) walked serially, spread over threads
            const int n_sub = s_nlevel[cur];
            int task = tid;
            TreeWalk W;
            W.d = kSpreadDepth;
            W.k = 0;
            W.done = task >= n_sub;
            int slot = 0;
            if (!W.done) {
                slot = (int)(level[cur][task] >> 24);
                W.k = level[cur][task] & 0xffffffu;
            }
            for (;;) {
                while (!W.done) {
                    const int leaf = decide_node(b, recs[slot], coefs[slot], W.d, W.k, trm, fallbacks);
                    if (!leaf) {
                        if (W.d >= MAX_DEPTH) {
                            set_err(b.err, ERR_DEPTH);
                            W.done = true;
                            break;
                        }
                        ++W.d;
                        W.k <<= 1;
                        continue;
                    }
                    const int idx = atomicAdd(&s_nleaf, 1);
                    if (idx >= kLeafCap) break;  // buffer full: this leaf is retried after the drain
                    LeafCode lc;
                    lc.k = W.k;
                    lc.slot = (uint16_t)slot;
                    lc.d = (uint16_t)W.d;
                    leaves[idx] = lc;
                    // next leaf of this subtree, or the next subtree of this thread
                    while (W.d > kSpreadDepth && (W.k & 1u)) {
                        W.k >>= 1;
                        --W.d;
                    }
                    if (W.d == kSpreadDepth) {
                        task += kThreads;
                        if (task < n_sub) {
                            slot = (int)(level[cur][task] >> 24);
                            W.k = level[cur][task] & 0xffffffu;
                        } else {
                            W.done = true;
                        }
                    } else {
                        W.k += 1;
                    }
                }
                __syncthreads();
                const int n = min(s_nleaf, kLeafCap);
                for (int j = tid; j < n; j += kThreads) drain_leaf(B, recs, leaves[j]);
                const int more = __syncthreads_or(!W.done);
                if (tid == 0) s_nleaf = 0;
                __syncthreads();
                if (!more) break;
            }
        }
        __syncthreads();

        const int rule = b.rule ? b.rule[wi.path] : 0;
        band_scan_store(B, m, rule, b.out, reinterpret_cast<float*>(leaves));
        __syncthreads();
    }
    if (fallbacks) atomicAdd(&b.counters[1], fallbacks);
}

// Host-callable launchers (declared in rz_api.cu).  init_kernels() runs once
// per context creation, outside any stream capture.
cudaError_t init_kernels() {
    return cudaFuncSetAttribute(k_mask_bands, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
}

int band_floats() { return kBandFloats; }
int band_smem_bytes() { return kSmemBytes; }

cudaError_t launch_mask_bands(const BatchDev& b, const WorkItem* items, int n_items, int32_t* queue, int grid,
                              cudaStream_t stream) {
    k_mask_bands<<<grid, kThreads, kSmemBytes, stream>>>(b, items, n_items, queue);
    return cudaGetLastError();
}

int mask_bands_occupancy() {
    int blocks = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_mask_bands, kThreads, kSmemBytes);
    return blocks;
}

}  // namespace rz

namespace rz {

// Per input segment: number of lines PathFlattenIter emits for it (arcs:
// summed over their cubics); then one entry per subpath for its closing line.
__global__ void k_flatten_counts(BatchDev b, uint32_t n_segments, uint32_t n_subpaths, uint32_t* counts) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_segments) {
        Seg64 parts[4];
        const int np = expand_segment(b.kind[i], b.pts + 8ull * i, parts);
        if (np < 0) { set_err(b.err, ERR_ARC); counts[i] = 0; return; }
        uint32_t total = 0;
        int fallbacks = 0;
        for (int j = 0; j < np; ++j) {
            Seg64& s = parts[j];
            transform_seg(s, b.tr);
            bool nan = false;
            for (int q = 0; q < seg_npts(s.kind); ++q) nan |= isnan(s.x[q]) || isnan(s.y[q]);
            if (nan) { set_err(b.err, ERR_NAN); continue; }
            const FlatCoef c = flat_coef(s);
            TreeWalk w;
            w.start();
            while (!w.done) {
                if (!node_is_leaf(s, c, w.d, w.k, b.thr64, b.thr32, fallbacks)) {
                    if (w.d >= MAX_DEPTH) { set_err(b.err, ERR_DEPTH); w.done = true; break; }
                    ++w.d;
                    w.k <<= 1;
                    continue;
                }
                ++total;
                w.next_after_leaf();
            }
        }
        counts[i] = total;
        if (fallbacks) atomicAdd(&b.counters[1], fallbacks);
    } else if (i < n_segments + n_subpaths) {
        const uint32_t sp = i - n_segments;
        const uint32_t s1 = min(b.sub_off[sp + 1], n_segments), s0 = b.sub_off[sp];
        double x, y;
        counts[i] = (s1 > s0 && subpath_point(b, s0, s1, true, x, y)) ? 1u : 0u;
    }
}

cudaError_t launch_flatten_counts(const BatchDev& b, uint32_t n_segments, uint32_t n_subpaths, uint32_t* counts,
                                  cudaStream_t stream) {
    const uint32_t n = n_segments + n_subpaths;
    if (n == 0) return cudaSuccess;
    k_flatten_counts<<<(n + 127) / 128, 128, 0, stream>>>(b, n_segments, n_subpaths, counts);
    return cudaGetLastError();
}

}  // namespace rz
