// rz_device.cuh -- device building blocks of the GB300 rasterizer.
//
// Flattening (src/path.rs:734-796, src/curve.rs:413-456, 692-747): the
// reference bisects every curve at t = 1/2 until `flatness() < 16 f^2`.  The
// leaf set of that tree depends on strict f64 comparisons, so it is
// reproduced exactly: each node's flatness is evaluated in FP32 from the
// curve's power-basis coefficients (no control points are materialised) with
// a rigorous error bound, and only a node whose value lies inside the bound
// is re-decided in binary64 by replaying the reference's own split chain
// (`flatness_chain64`).  Vertices are evaluated relative to the segment start
// so FP32 keeps ~1e-6 px; shared vertices are computed once and reused by both
// lines, so windings telescope exactly.
//
// Coverage (src/rasterize.rs:365-507): lines are clipped with the reference's
// own x rules (drop x > width, fully-right lines become vertical at
// width - 0.001, x < 0 parts become vertical at x = 0), then their signed
// area differences are accumulated in shared memory per row band; a warp
// scan with two-sum compensation turns differences into winding numbers and
// the fill rule into alpha.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace rz {

enum : int { SEG_LINE = 0, SEG_QUAD = 1, SEG_CUBIC = 2, SEG_ARC = 3 };
enum : int { ERR_NAN = 1, ERR_DEPTH = 5, ERR_ARC = 6, ERR_CAPACITY = 7 };
constexpr int MAX_DEPTH = 22;  // 3k+2 < 2^24 keeps the node parameter exact in FP32

// binary64 without contraction: the reference's Rust code never fuses a*b+c
__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }

struct Seg64 {
    int kind;
    double x[4], y[4];
};

// Transform::apply src/geometry.rs:363-367
__device__ __forceinline__ void tr_apply64(const double* m, double x, double y, double& ox, double& oy) {
    ox = da(da(dm(x, m[0]), dm(y, m[1])), m[2]);
    oy = da(da(dm(x, m[3]), dm(y, m[4])), m[5]);
}

__device__ __forceinline__ int seg_npts(int kind) { return kind == SEG_LINE ? 2 : (kind == SEG_QUAD ? 3 : 4); }

// Quad::split src/curve.rs:449-456, Cubic::split :731-747 (one half)
__device__ inline void split_half64(Seg64& s, bool right) {
    if (s.kind == SEG_CUBIC) {
        double mx = da(da(da(dm(0.125, s.x[0]), dm(0.375, s.x[1])), dm(0.375, s.x[2])), dm(0.125, s.x[3]));
        double my = da(da(da(dm(0.125, s.y[0]), dm(0.375, s.y[1])), dm(0.375, s.y[2])), dm(0.125, s.y[3]));
        if (!right) {
            double x1 = da(dm(0.5, s.x[0]), dm(0.5, s.x[1])), y1 = da(dm(0.5, s.y[0]), dm(0.5, s.y[1]));
            double x2 = da(da(dm(0.25, s.x[0]), dm(0.5, s.x[1])), dm(0.25, s.x[2]));
            double y2 = da(da(dm(0.25, s.y[0]), dm(0.5, s.y[1])), dm(0.25, s.y[2]));
            s.x[1] = x1; s.y[1] = y1; s.x[2] = x2; s.y[2] = y2; s.x[3] = mx; s.y[3] = my;
        } else {
            double x1 = da(da(dm(0.25, s.x[1]), dm(0.5, s.x[2])), dm(0.25, s.x[3]));
            double y1 = da(da(dm(0.25, s.y[1]), dm(0.5, s.y[2])), dm(0.25, s.y[3]));
            double x2 = da(dm(0.5, s.x[2]), dm(0.5, s.x[3])), y2 = da(dm(0.5, s.y[2]), dm(0.5, s.y[3]));
            s.x[0] = mx; s.y[0] = my; s.x[1] = x1; s.y[1] = y1; s.x[2] = x2; s.y[2] = y2;
        }
    } else if (s.kind == SEG_QUAD) {
        double mx = dm(0.25, da(da(s.x[0], dm(2.0, s.x[1])), s.x[2]));
        double my = dm(0.25, da(da(s.y[0], dm(2.0, s.y[1])), s.y[2]));
        if (!right) {
            s.x[1] = dm(0.5, da(s.x[0], s.x[1])); s.y[1] = dm(0.5, da(s.y[0], s.y[1]));
            s.x[2] = mx; s.y[2] = my;
        } else {
            s.x[1] = dm(0.5, da(s.x[1], s.x[2])); s.y[1] = dm(0.5, da(s.y[1], s.y[2]));
            s.x[0] = mx; s.y[0] = my;
        }
    }
}

// Quad::flatness src/curve.rs:413-417, Cubic::flatness :692-697
__device__ inline double flatness64(const Seg64& s) {
    if (s.kind == SEG_QUAD) {
        double x = ds(ds(dm(2.0, s.x[1]), s.x[0]), s.x[2]);
        double y = ds(ds(dm(2.0, s.y[1]), s.y[0]), s.y[2]);
        return da(dm(x, x), dm(y, y));
    }
    if (s.kind == SEG_CUBIC) {
        double ux = ds(ds(dm(3.0, s.x[1]), dm(2.0, s.x[0])), s.x[3]);
        double uy = ds(ds(dm(3.0, s.y[1]), dm(2.0, s.y[0])), s.y[3]);
        double vx = ds(ds(dm(3.0, s.x[2]), s.x[0]), dm(2.0, s.x[3]));
        double vy = ds(ds(dm(3.0, s.y[2]), s.y[0]), dm(2.0, s.y[3]));
        return da(fmax(dm(ux, ux), dm(vx, vx)), fmax(dm(uy, uy), dm(vy, vy)));
    }
    return 0.0;
}

// The reference's flatness of node (d, k): replay the split chain in binary64.
__device__ __noinline__ double flatness_chain64(Seg64 s, int d, uint32_t k) {
    for (int i = d - 1; i >= 0; --i) split_half64(s, (k >> i) & 1u);
    return flatness64(s);
}

struct FlatCoef {
    float a2x, a2y, a3x, a3y;
    float mag;  // max |coordinate| of the control points (f64 error term)
};

// ---------------------------------------------------------------------------
// Fixed point 16.16 from binary64 with integer instructions only (GB300's
// FP64 pipe is ~1/64 of FP32).  Deterministic round-half-even of x * 2^16;
// returns false for |x| >= 16384 px, infinities and NaN.
// ---------------------------------------------------------------------------
constexpr double FIX_RANGE = 16384.0;

__device__ __forceinline__ bool d2fix(double x, int32_t& out) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((bits >> 52) & 0x7ffull);
    if (e == 0) {  // zero or subnormal: below the fixed-point resolution
        out = 0;
        return true;
    }
    if (e >= 1023 + 14) return false;  // |x| >= 16384, inf, NaN
    const unsigned long long mant = (bits & 0xfffffffffffffull) | (1ull << 52);
    const int sh = 1059 - e;  // value * 2^16 = mant * 2^(e - 1059)
    unsigned long long q;
    if (sh >= 64) {
        q = 0;
    } else {
        q = mant >> sh;
        const unsigned long long rem = mant - (q << sh);
        const unsigned long long half = 1ull << (sh - 1);
        if (rem > half || (rem == half && (q & 1ull))) ++q;
    }
    const int32_t v = (int32_t)q;
    out = (bits >> 63) ? -v : v;
    return true;
}

__device__ __forceinline__ bool is_nan_bits(double x) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    return ((bits >> 52) & 0x7ffull) == 0x7ffull && (bits & 0xfffffffffffffull) != 0ull;
}

constexpr float FIX_ONE_INV = 1.0f / 65536.0f;

// A reference segment in fixed point (after the path transform).
struct FixSeg {
    int kind;
    int32_t x[4], y[4];
};

// Flatness coefficients from fixed-point control points, in px, and the
// bound of their error against the binary64 values (quantisation 2^-17 px per
// coordinate plus FP32 rounding).
__device__ inline FlatCoef flat_coef_fix(const FixSeg& s, float& qerr) {
    FlatCoef c;
    int32_t mx = 0;
    #pragma unroll
    for (int i = 0; i < 4; ++i) mx = max(mx, max(abs(s.x[i]), abs(s.y[i])));  // unused points are 0
    c.mag = (float)mx * FIX_ONE_INV;
    const float dx1 = (float)(s.x[1] - s.x[0]) * FIX_ONE_INV, dy1 = (float)(s.y[1] - s.y[0]) * FIX_ONE_INV;
    if (s.kind == SEG_CUBIC) {
        const float dx2 = (float)(s.x[2] - s.x[1]) * FIX_ONE_INV, dy2 = (float)(s.y[2] - s.y[1]) * FIX_ONE_INV;
        const float dx3 = (float)(s.x[3] - s.x[2]) * FIX_ONE_INV, dy3 = (float)(s.y[3] - s.y[2]) * FIX_ONE_INV;
        c.a2x = 3.f * (dx2 - dx1);
        c.a2y = 3.f * (dy2 - dy1);
        c.a3x = (dx1 - 2.f * dx2) + dx3;
        c.a3y = (dy1 - 2.f * dy2) + dy3;
        qerr = ldexpf(fmaxf(fabsf(dx1) + fabsf(dx2) + fabsf(dx3), fabsf(dy1) + fabsf(dy2) + fabsf(dy3)), -19) +
               12.f * ldexpf(1.f, -17);
    } else if (s.kind == SEG_QUAD) {
        const float dx2 = (float)(s.x[2] - s.x[1]) * FIX_ONE_INV, dy2 = (float)(s.y[2] - s.y[1]) * FIX_ONE_INV;
        c.a2x = dx2 - dx1;
        c.a2y = dy2 - dy1;
        c.a3x = c.a3y = 0.f;
        qerr = ldexpf(fmaxf(fabsf(dx1) + fabsf(dx2), fabsf(dy1) + fabsf(dy2)), -21) + 4.f * ldexpf(1.f, -17);
    } else {
        c.a2x = c.a2y = c.a3x = c.a3y = 0.f;
        qerr = 0.f;
    }
    return c;
}

// Per-segment data for exact FP32 flatness decisions.
//   cubic: sub-curve over [kh, (k+1)h] has u = -h^2 (a2 + a3 h(3k+1)),
//          v = -h^2 (a2 + a3 h(3k+2)) with a2 = 3(P0 - 2P1 + P2),
//          a3 = P3 - P0 + 3(P1 - P2); flatness = h^4 G.
//   quad:  2c1 - c0 - c2 = -h^2 (P0 - 2P1 + P2); flatness = h^4 |a2|^2.

__device__ inline FlatCoef flat_coef(const Seg64& s) {
    FlatCoef c;
    double mag = 0.0;
    for (int i = 0; i < seg_npts(s.kind); ++i) mag = fmax(mag, fmax(fabs(s.x[i]), fabs(s.y[i])));
    c.mag = (float)mag;
    if (s.kind == SEG_CUBIC) {
        c.a2x = (float)(3.0 * ((s.x[0] - 2.0 * s.x[1]) + s.x[2]));
        c.a2y = (float)(3.0 * ((s.y[0] - 2.0 * s.y[1]) + s.y[2]));
        c.a3x = (float)((s.x[3] - s.x[0]) + 3.0 * (s.x[1] - s.x[2]));
        c.a3y = (float)((s.y[3] - s.y[0]) + 3.0 * (s.y[1] - s.y[2]));
    } else if (s.kind == SEG_QUAD) {
        c.a2x = (float)((s.x[0] - 2.0 * s.x[1]) + s.x[2]);
        c.a2y = (float)((s.y[0] - 2.0 * s.y[1]) + s.y[2]);
        c.a3x = 0.f;
        c.a3y = 0.f;
    } else {
        c.a2x = c.a2y = c.a3x = c.a3y = 0.f;
    }
    return c;
}

// FP32 decision of `flatness(node) < thr` with a rigorous error bound:
// 1 = leaf, 0 = split, -1 = too close to call (re-decide in binary64).
// qerr bounds |a2 - a2_true| and |a3 - a3_true| (px) when the coefficients
// come from rounded inputs.
__device__ inline int decide_fp32(int kind, const FlatCoef& c, int d, uint32_t k, float thr32, float qerr) {
    const float h = ldexpf(1.0f, -d);
    const float td = ldexpf(thr32, 4 * d);  // thr * 16^d, exact power-of-two scaling
    const float scale = ldexpf(1.0f, 2 * d);  // chain error grows like 4^d in w units
    float G, E;
    if (kind == SEG_CUBIC) {
        const float tu = h * (float)(3u * k + 1u);
        const float tv = h * (float)(3u * k + 2u);
        const float wux = fmaf(c.a3x, tu, c.a2x), wvx = fmaf(c.a3x, tv, c.a2x);
        const float wuy = fmaf(c.a3y, tu, c.a2y), wvy = fmaf(c.a3y, tv, c.a2y);
        const float gx = fmaxf(wux * wux, wvx * wvx), gy = fmaxf(wuy * wuy, wvy * wvy);
        G = gx + gy;
        const float q = qerr * (1.f + tv);
        const float bx = ldexpf(fabsf(c.a2x) + fabsf(c.a3x) * tv, -21) + ldexpf(c.mag * scale, -40) + q;
        const float by = ldexpf(fabsf(c.a2y) + fabsf(c.a3y) * tv, -21) + ldexpf(c.mag * scale, -40) + q;
        const float wx = sqrtf(gx), wy = sqrtf(gy);
        E = (2.f * wx + bx) * bx + (2.f * wy + by) * by + ldexpf(G, -19);
    } else {
        G = c.a2x * c.a2x + c.a2y * c.a2y;
        const float bx = ldexpf(fabsf(c.a2x), -21) + ldexpf(c.mag * scale, -40) + qerr;
        const float by = ldexpf(fabsf(c.a2y), -21) + ldexpf(c.mag * scale, -40) + qerr;
        E = (2.f * fabsf(c.a2x) + bx) * bx + (2.f * fabsf(c.a2y) + by) * by + ldexpf(G, -19);
    }
    if (isfinite(G) && isfinite(E) && isfinite(td)) {
        if (G + E < td) return 1;
        if (G - E >= td) return 0;
    }
    return -1;
}

// Decides `flatness(node) < thr` exactly as the reference.  thr64 = 16 f f.
// Returns 1 = leaf, 0 = split; `fallbacks` counts binary64 replays.
__device__ inline int node_is_leaf(const Seg64& root, const FlatCoef& c, int d, uint32_t k, double thr64,
                                   float thr32, int& fallbacks, float qerr = 0.f) {
    if (root.kind == SEG_LINE) return thr64 > 0.0;  // Line::flatness == 0 (src/curve.rs:233-235)
    const int r = decide_fp32(root.kind, c, d, k, thr32, qerr);
    if (r >= 0) return r;
    ++fallbacks;
    return flatness_chain64(root, d, k) < thr64 ? 1 : 0;
}

// In-order leaf walk over the bisection tree: the reference's stack DFS
// (push right, push left, pop) visits leaves left to right.
struct TreeWalk {
    int d;
    uint32_t k;
    bool done;
    __device__ void start() { d = 0; k = 0; done = false; }
    // Advance from leaf (d, k) to the next node to examine.
    __device__ void next_after_leaf() {
        while (d > 0 && (k & 1u)) { k >>= 1; --d; }
        if (d == 0) { done = true; return; }
        k += 1;
    }
};

// Power-basis coefficients relative to P0 (B(t) = P0 + t(c1 + t(c2 + t c3))).
struct VertexCoef {
    double p0x, p0y, pnx, pny;   // first and last control point
    double c1x, c1y, c2x, c2y, c3x, c3y;
    float f1x, f1y, f2x, f2y, f3x, f3y;  // FP32 copies for small segments
    bool small;                          // FP32 evaluation error below ~1e-6 px
};

__device__ inline VertexCoef vertex_coef(const Seg64& s) {
    VertexCoef v;
    int n = seg_npts(s.kind);
    v.p0x = s.x[0]; v.p0y = s.y[0];
    v.pnx = s.x[n - 1]; v.pny = s.y[n - 1];
    if (s.kind == SEG_CUBIC) {
        v.c1x = 3.0 * (s.x[1] - s.x[0]); v.c1y = 3.0 * (s.y[1] - s.y[0]);
        v.c2x = 3.0 * ((s.x[0] - 2.0 * s.x[1]) + s.x[2]); v.c2y = 3.0 * ((s.y[0] - 2.0 * s.y[1]) + s.y[2]);
        v.c3x = (s.x[3] - s.x[0]) + 3.0 * (s.x[1] - s.x[2]); v.c3y = (s.y[3] - s.y[0]) + 3.0 * (s.y[1] - s.y[2]);
    } else if (s.kind == SEG_QUAD) {
        v.c1x = 2.0 * (s.x[1] - s.x[0]); v.c1y = 2.0 * (s.y[1] - s.y[0]);
        v.c2x = (s.x[0] - 2.0 * s.x[1]) + s.x[2]; v.c2y = (s.y[0] - 2.0 * s.y[1]) + s.y[2];
        v.c3x = v.c3y = 0.0;
    } else {
        v.c1x = s.x[1] - s.x[0]; v.c1y = s.y[1] - s.y[0];
        v.c2x = v.c2y = v.c3x = v.c3y = 0.0;
    }
    // FP32 Horner error is about 3 * 2^-24 * ext: ext < 48 keeps vertices within ~1e-5 px
    const double ext = fmax(fabs(v.c1x) + fabs(v.c2x) + fabs(v.c3x), fabs(v.c1y) + fabs(v.c2y) + fabs(v.c3y));
    v.small = ext < 48.0;
    v.f1x = (float)v.c1x; v.f1y = (float)v.c1y;
    v.f2x = (float)v.c2x; v.f2y = (float)v.c2y;
    v.f3x = (float)v.c3x; v.f3y = (float)v.c3y;
    return v;
}

// Vertex at t = j / 2^d.  Small segments: FP32 relative to (ox, oy) with the
// exact end point at t = 1.  Otherwise binary64 absolute x, band-relative y.
__device__ inline void vertex_small(const VertexCoef& v, uint32_t j, int d, double ox, double oy, float p0rx,
                                    float p0ry, float& rx, float& ry) {
    if (j == 0) { rx = p0rx; ry = p0ry; return; }
    if ((j >> d) != 0u) {
        rx = (float)(v.pnx - ox);
        ry = (float)(v.pny - oy);
        return;
    }
    const float t = ldexpf((float)j, -d);
    rx = p0rx + t * fmaf(t, fmaf(t, v.f3x, v.f2x), v.f1x);
    ry = p0ry + t * fmaf(t, fmaf(t, v.f3y, v.f2y), v.f1y);
}

__device__ inline void vertex_big(const VertexCoef& v, uint32_t j, int d, double oy, double& x, double& y) {
    if (j == 0) { x = v.p0x; y = v.p0y - oy; return; }
    if ((j >> d) != 0u) { x = v.pnx; y = v.pny - oy; return; }
    const double t = ldexp((double)j, -d);
    x = v.p0x + t * fma(t, fma(t, v.c3x, v.c2x), v.c1x);
    y = (v.p0y + t * fma(t, fma(t, v.c3y, v.c2y), v.c1y)) - oy;
}

// ---------------------------------------------------------------------------
// Coverage accumulation into a shared-memory row band
// ---------------------------------------------------------------------------
struct Band {
    float* acc;     // bh rows x stride floats
    int stride;     // >= width_i + 2
    int bh;         // rows in this band
    int y0;         // first image row of the band
    int img_h;      // image height (rows >= img_h are never written)
    float width_f;  // the reference's `width` = image_width - 1 (clip column)
    int width_i;
};

__device__ __forceinline__ void sadd(float* p, float v) { atomicAdd(p, v); }

// One line (band-relative coordinates, x relative to integer column `xb`)
// already clipped by the x rules; distributes its signed differences row by
// row exactly like signed_difference_line (src/rasterize.rs:405-469).
__device__ inline void accumulate_piece(const Band& B, int xb, float x0, float y0, float x1, float y1) {
    if (y0 == y1) return;  // no signed coverage (the reference skips |dy| < EPSILON)
    float dir = 1.f;
    if (y0 > y1) {
        float t = x0; x0 = x1; x1 = t;
        t = y0; y0 = y1; y1 = t;
        dir = -1.f;
    }
    const float ylim = (float)min(B.bh, B.img_h - B.y0);
    const float ya_all = fmaxf(y0, fmaxf(0.f, -(float)B.y0));
    const float yb_all = fminf(y1, ylim);
    if (!(ya_all < yb_all)) return;
    const float dxdy = (x1 - x0) / (y1 - y0);
    const float xmax_rel = B.width_f - (float)xb;  // the reference's `width`, relative
    const int r0 = (int)floorf(ya_all);
    const int r1 = (int)ceilf(yb_all);
    for (int r = max(r0, 0); r < min(r1, B.bh); ++r) {
        const float ya = fmaxf(ya_all, (float)r);
        const float yb = fminf(yb_all, (float)(r + 1));
        if (!(ya < yb)) continue;
        const float dy = yb - ya;
        const float d = dir * dy;
        const float xa = fmaf(ya - y0, dxdy, x0);
        const float xn = fmaf(yb - y0, dxdy, x0);
        // in the reference x walks from the lower y end: mean is symmetric
        const float xlo = fminf(xa, xn), xhi = fmaxf(xa, xn);
        const float x0_floor = fmaxf(floorf(xlo), -(float)xb);
        int x0i = (int)x0_floor;
        const float x1_ceil = fminf(ceilf(xhi), xmax_rel);
        int x1i = (int)x1_ceil;
        float* row = B.acc + r * B.stride + xb;
        x0i = min(x0i, B.width_i + 1 - xb);
        if (x1i <= x0i + 1) {
            const float xmf = 0.5f * (xa + xn) - x0_floor;
            sadd(row + x0i, d * (1.f - xmf));
            sadd(row + x0i + 1, d * xmf);
        } else {
            const float s = 1.f / (xhi - xlo);
            const float x0f = xlo - x0_floor;
            const float x1f = xhi - x1_ceil + 1.f;
            const float a0 = 0.5f * s * (1.f - x0f) * (1.f - x0f);
            const float am = 0.5f * s * x1f * x1f;
            sadd(row + x0i, d * a0);
            if (x1i == x0i + 2) {
                sadd(row + x0i + 1, d * (1.f - a0 - am));
            } else {
                const float a1 = s * (1.5f - x0f);
                sadd(row + x0i + 1, d * (a1 - a0));
                const float ds_ = d * s;
                for (int xi = x0i + 2; xi < x1i - 1; ++xi) sadd(row + xi, ds_);
                const float a2 = a1 + (float)(x1i - x0i - 3) * s;
                sadd(row + x1i - 1, d * (1.f - a2 - am));
            }
            sadd(row + x1i, d * am);
        }
    }
}

// Piece of a line after the x rules, in binary64 (x absolute, y relative to
// the band).  Clips it to the band's rows (a pure geometric clip, so the area
// inside is unchanged) and hands a short FP32 copy to accumulate_piece with x
// relative to an integer column near the piece.
__device__ inline void accumulate_piece64(const Band& B, double x0, double y0, double x1, double y1) {
    if (y0 == y1) return;
    const double lo = fmax(-1.0, -(double)B.y0 - 1.0);
    const double hi = (double)min(B.bh, B.img_h - B.y0) + 1.0;
    const double ymin = fmin(y0, y1), ymax = fmax(y0, y1);
    if (ymax <= lo || ymin >= hi) return;
    if (ymin < lo || ymax > hi) {
        const double dxdy = (x1 - x0) / (y1 - y0);
        if (y0 < lo) { x0 = x0 + (lo - y0) * dxdy; y0 = lo; }
        else if (y0 > hi) { x0 = x0 + (hi - y0) * dxdy; y0 = hi; }
        if (y1 < lo) { x1 = x0 + (lo - y0) * dxdy; y1 = lo; }
        else if (y1 > hi) { x1 = x0 + (hi - y0) * dxdy; y1 = hi; }
    }
    const int xb = (int)floor(fmin(x0, x1));
    accumulate_piece(B, xb, (float)(x0 - xb), (float)y0, (float)(x1 - xb), (float)y1);
}

// A flattened line in binary64 (x absolute, y relative to the band): applies
// the reference's right-edge rule (src/rasterize.rs:372-387) and
// split_at_zero_x (:923-937), then accumulates the pieces.
__device__ __noinline__ void accumulate_line64(const Band& B, double ax, double ay, double bx, double by) {
    const double width = (double)B.width_i;
    if (ax > width || bx > width) {
        if (ax > width && bx > width) {
            ax = width - 0.001;
            bx = width - 0.001;
        } else {
            const double t = (ax - width) / (ax - bx);
            const double my = (1.0 - t) * ay + t * by;
            if (ax < width) { bx = width; by = my; }
            else { ax = width; ay = my; }
        }
    }
    if (ax >= 0.0 && bx >= 0.0) {
        accumulate_piece64(B, ax, ay, bx, by);
    } else if (ax <= 0.0 && bx <= 0.0) {
        accumulate_piece64(B, 0.0, ay, 0.0, by);
    } else {
        const double t = ax / (ax - bx);
        const double mx = (1.0 - t) * ax + t * bx, my = (1.0 - t) * ay + t * by;
        if (ax < 0.0) {
            accumulate_piece64(B, mx, my, bx, by);
            accumulate_piece64(B, 0.0, ay, mx, my);
        } else {
            accumulate_piece64(B, ax, ay, mx, my);
            accumulate_piece64(B, mx, my, 0.0, by);
        }
    }
}

// A short line given relative to integer column xb (y relative to the band):
// stays in FP32 unless an x rule applies or it is long, then takes the
// binary64 route.
__device__ __forceinline__ void accumulate_line(const Band& B, int xb, float x0, float y0, float x1, float y1) {
    const float xlo = (float)xb + fminf(x0, x1), xhi = (float)xb + fmaxf(x0, x1);
    if (xlo > 0.01f && xhi < B.width_f - 0.01f && fabsf(x1 - x0) <= 64.f && fabsf(y1 - y0) <= 64.f) {
        accumulate_piece(B, xb, x0, y0, x1, y1);
    } else {
        accumulate_line64(B, (double)xb + (double)x0, (double)y0, (double)xb + (double)x1, (double)y1);
    }
}

// ---------------------------------------------------------------------------
// Row prefix sum (two-sum compensated warp scan) + fill rule
// ---------------------------------------------------------------------------
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bp = s - a;
    e = (a - (s - bp)) + (b - bp);
}

// FillRule::alpha_from_winding src/path.rs:32-46 (NonZero clamps, EvenOdd folds)
__device__ __forceinline__ float alpha_from_winding(int rule, float w) {
    if (rule == 1) {
        float r = fmodf(w + 1.f, 2.f);
        if (r < 0.f) r += 2.f;
        return fabsf(r - 1.f);
    }
    const float v = fabsf(w);
    return v >= 1.f ? 1.f : (v < 1e-6f ? 0.f : v);
}

}  // namespace rz
