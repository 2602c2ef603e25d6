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
// area differences are accumulated as int32 fixed point in shared memory per
// row band; an exact integer warp scan turns differences into winding numbers
// and the fill rule into alpha.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace rz {

enum : int { SEG_LINE = 0, SEG_QUAD = 1, SEG_CUBIC = 2, SEG_ARC = 3 };
enum : int { ERR_NAN = 1, ERR_DEPTH = 5, ERR_ARC = 6, ERR_CAPACITY = 7 };
constexpr int MAX_DEPTH = 22;
#ifndef RZ_ANCHOR_PX
#define RZ_ANCHOR_PX 2
#endif  // 3k+2 < 2^24 keeps the node parameter exact in FP32

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
static __device__ __noinline__ double flatness_chain64(Seg64 s, int d, uint32_t k) {
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

// 2^e for -126 <= e <= 127, exact, without a libm call.
__device__ __forceinline__ float pow2f(int e) { return __int_as_float((127 + e) << 23); }

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
// FINITE: the coefficients are known to be finite and bounded (fixed-point
// records: |a2|, |a3| < 2^18 px, so G and E stay finite; an infinite td only
// says what the exact comparison says), and the checks are left out.
template <bool FINITE = false>
__device__ inline int decide_fp32(int kind, const FlatCoef& c, int d, uint32_t k, float thr32, float qerr) {
    const float h = pow2f(-d);
    const float td = thr32 * pow2f(4 * d);     // thr * 16^d, exact power-of-two scaling
    const float ms = c.mag * pow2f(2 * d - 40);  // chain error grows like 4^d in w units
    const float e21 = pow2f(-21), e19 = pow2f(-19);
    // One formula for cubics and quads (a quad's a3 is 0: u = v and G = |a2|^2, the reference's quad
    // flatness), so a warp that mixes the two kinds does not diverge here.
    (void)kind;
    const float tu = h * (float)(3u * k + 1u);
    const float tv = h * (float)(3u * k + 2u);
    const float wux = fmaf(c.a3x, tu, c.a2x), wvx = fmaf(c.a3x, tv, c.a2x);
    const float wuy = fmaf(c.a3y, tu, c.a2y), wvy = fmaf(c.a3y, tv, c.a2y);
    const float gx = fmaxf(wux * wux, wvx * wvx), gy = fmaxf(wuy * wuy, wvy * wvy);
    const float G = gx + gy;
    const float q = qerr * (1.f + tv);
    const float bx = (fabsf(c.a2x) + fabsf(c.a3x) * tv) * e21 + ms + q;
    const float by = (fabsf(c.a2y) + fabsf(c.a3y) * tv) * e21 + ms + q;
    // sqrt(gx) without a square root: gx is the larger square, so its root is the larger |w| (widened by
    // 2^-22 to cover the rounding of the square and of a correctly rounded root)
    const float wx = fmaxf(fabsf(wux), fabsf(wvx)) * 1.00000024f, wy = fmaxf(fabsf(wuy), fabsf(wvy)) * 1.00000024f;
    const float E = (2.f * wx + bx) * bx + (2.f * wy + by) * by + G * e19;
    if (FINITE || (isfinite(G) && isfinite(E) && isfinite(td))) {
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
    return v;
}

// Vertex at t = j / 2^d in binary64: absolute x, y relative to row oy.
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
// Signed areas are accumulated in 32-bit fixed point, COV_ONE per unit of
// winding: shared-memory integer atomics are order independent and the row
// prefix is exact, so long rows with large windings lose nothing (EvenOdd
// maps winding error 1:1 into coverage).  Windings wrap modulo 1024 (int32
// holds +-512 units), which keeps EvenOdd parity and keeps NonZero's |w| >= 1
// for every winding that is not within one unit of a multiple of 1024.
// Band-relative y must stay below 511 rows (band heights are capped at 256).
constexpr int COV_SHIFT = 22;
constexpr int COV_ONE = 1 << COV_SHIFT;
constexpr float COV_ONE_F = 4194304.0f;

struct Band {
    float* acc;     // bh rows x stride accumulation words (int32 fixed point, COV_ONE per unit)
    int stride;     // >= width_i + 2
    int bh;         // rows in this band
    int y0;         // first image row of the band
    int img_h;      // image height (rows >= img_h are never written)
    float width_f;  // the reference's `width` = image_width - 1 (clip column)
    int width_i;
};

// Adds v to an accumulation word.  Bands always live in shared memory: a
// reduction on the shared window (no return value, no generic-address check).
__device__ __forceinline__ void sadd(float* p, int v) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("red.shared.add.s32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}

// Signed height `d` (fixed point) of one row, spread over the pixels the line
// covers between xa and xn (FP32, relative to integer column xb) as in
// signed_difference_line (src/rasterize.rs:433-466).  Each pixel receives the
// difference of the rounded cumulative shares, so every pixel is within one
// fixed-point unit of the exact share however long the span, and the row
// receives exactly `d` (the row prefix telescopes).
// INSIDE: the caller has checked that the line stays more than 0.01 px inside
// (0, width), so the clamps to the image's columns cannot change anything and
// are left out.
template <bool INSIDE = false>
__device__ __forceinline__ void accumulate_row(const Band& B, int r, int xb, float xa, float xn, int d) {
    const float df = (float)d;
    const float xlo = fminf(xa, xn), xhi = fmaxf(xa, xn);
    const float x0_floor = INSIDE ? floorf(xlo) : fmaxf(floorf(xlo), -(float)xb);
    int x0i = (int)x0_floor;
    const float x1_ceil = INSIDE ? ceilf(xhi) : fminf(ceilf(xhi), B.width_f - (float)xb);  // the reference's `width`
    const int x1i = (int)x1_ceil;
    float* row = B.acc + r * B.stride + xb;
    if (!INSIDE) x0i = min(x0i, B.width_i + 1 - xb);
    if (x1i <= x0i + 1) {
        const float xmf = 0.5f * (xa + xn) - x0_floor;
        const int c0 = __float2int_rn(df * (1.f - xmf));
        sadd(row + x0i, c0);
        sadd(row + x0i + 1, d - c0);
        return;
    }
    const float s = __fdividef(1.f, xhi - xlo);  // xhi - xlo > 1: the hardware reciprocal, within 2 ulp
    const float x0f = xlo - x0_floor;
    const float x1f = xhi - x1_ceil + 1.f;
    const float a0 = 0.5f * s * (1.f - x0f) * (1.f - x0f);  // share of the first pixel
    const float am = 0.5f * s * x1f * x1f;                  // share of the last pixel
    const int c0 = __float2int_rn(df * a0);
    const int c_end = __float2int_rn(df * (1.f - am));  // cumulative through pixel x1i - 1
    sadd(row + x0i, c0);
    if (x1i == x0i + 2) {
        sadd(row + x0i + 1, c_end - c0);
    } else {
        const float a1 = s * (1.5f - x0f);  // cumulative through pixel x0i + 1
        int prev = __float2int_rn(df * a1);
        sadd(row + x0i + 1, prev - c0);
        for (int xi = x0i + 2; xi < x1i - 1; ++xi) {
            const int cur = __float2int_rn(df * fmaf((float)(xi - x0i - 1), s, a1));
            sadd(row + xi, cur - prev);
            prev = cur;
        }
        sadd(row + x1i - 1, c_end - prev);
    }
    sadd(row + x1i, d - c_end);
}

constexpr int kShortLine = 32;

// A short line piece (at most kShortLine px each way) already clipped by the
// x rules: x in FP32 relative to column xb, y band-relative in fixed point.
// Walks its rows like signed_difference_line (src/rasterize.rs:405-469); the
// row crossings are interpolated from the exact fixed-point heights, so their
// x error stays below ~kShortLine * 2^-23 px.
template <bool INSIDE = false>
__device__ __forceinline__ void accumulate_piece(const Band& B, int xb, float x0, int32_t q0, float x1, int32_t q1) {
    if (q0 == q1) return;  // no signed coverage (the reference skips |dy| < EPSILON)
    int dir = 1;
    if (q0 > q1) {
        const float t = x0; x0 = x1; x1 = t;
        const int32_t u = q0; q0 = q1; q1 = u;
        dir = -1;
    }
    const int row_lo = max(0, -B.y0);
    const int row_hi = min(B.bh, B.img_h - B.y0);
    const int32_t qa_all = max(q0, row_lo << COV_SHIFT);
    const int32_t qb_all = min(q1, row_hi << COV_SHIFT);
    if (!(qa_all < qb_all)) return;
    const int r0 = qa_all >> COV_SHIFT;
    const int r1 = (qb_all + COV_ONE - 1) >> COV_SHIFT;
    if (r1 == r0 + 1 && qa_all == q0 && qb_all == q1) {  // one row, unclipped: the ends are the crossings
        accumulate_row<INSIDE>(B, r0, xb, x0, x1, dir * (q1 - q0));
        return;
    }
    const float dxq = __fdividef(x1 - x0, (float)(q1 - q0));  // px per fixed-point unit of height (within 2 ulp)
    for (int r = r0; r < r1; ++r) {
        const int32_t qa = max(qa_all, r << COV_SHIFT);
        const int32_t qb = min(qb_all, (r + 1) << COV_SHIFT);
        if (!(qa < qb)) continue;
        const float xa = qa == q0 ? x0 : fmaf((float)(qa - q0), dxq, x0);
        const float xn = qb == q1 ? x1 : fmaf((float)(qb - q0), dxq, x0);
        accumulate_row<INSIDE>(B, r, xb, xa, xn, dir * (qb - qa));
    }
}

// A long piece: x absolute in binary64, y band-relative in fixed point
// (already clipped to the band's rows, so q fits in 32 bits), with its slope
// dxdy in px per row.  The x of the row boundaries is stepped in 64-bit fixed
// point (2^-40 px: after 16384 rows the accumulated step error is below
// 1e-8 px), so the rows cost integer instructions.  Every row is handed to the
// FP32 distribution relative to its own integer column.
constexpr int kLongFrac = 40;
static __device__ __noinline__ void accumulate_piece_long(const Band& B, double x0, int32_t q0, double x1,
                                                          int32_t q1, double dxdy) {
    if (q0 == q1) return;
    int dir = 1;
    if (q0 > q1) {
        const double t = x0; x0 = x1; x1 = t;
        const int32_t u = q0; q0 = q1; q1 = u;
        dir = -1;
    }
    const int row_lo = max(0, -B.y0);
    const int row_hi = min(B.bh, B.img_h - B.y0);
    const int32_t qa_all = max(q0, row_lo << COV_SHIFT);
    const int32_t qb_all = min(q1, row_hi << COV_SHIFT);
    if (!(qa_all < qb_all)) return;
    const double dxq = dxdy * (1.0 / 4194304.0);  // px per fixed-point unit of height (exact scaling)
    const int r0 = qa_all >> COV_SHIFT;
    const int r1 = (qb_all + COV_ONE - 1) >> COV_SHIFT;
    const double one = 1099511627776.0;  // 2^40
    // x at the top of row r0 + 1 and the step per row, in units of 2^-40 px
    long long xb_fix = __double2ll_rn((x0 + (double)(((r0 + 1) << COV_SHIFT) - q0) * dxq) * one);
    const long long step = __double2ll_rn(dxdy * one);
    const long long x1_fix = __double2ll_rn(x1 * one);
    long long xa_fix = qa_all == q0 ? __double2ll_rn(x0 * one) : __double2ll_rn((x0 + (double)(qa_all - q0) * dxq) * one);
    for (int r = r0; r < r1; ++r) {
        const int32_t qa = max(qa_all, r << COV_SHIFT);
        const int32_t qb = min(qb_all, (r + 1) << COV_SHIFT);
        const long long xn_fix = qb == q1 ? x1_fix
                                          : (qb == qb_all ? __double2ll_rn((x0 + (double)(qb - q0) * dxq) * one) : xb_fix);
        if (qa < qb) {
            const long long lo = min(xa_fix, xn_fix);
            const long long col = lo >> kLongFrac;  // floor
            const long long base = col << kLongFrac;
            const float fa = (float)(xa_fix - base) * (1.0f / 1099511627776.0f);
            const float fn = (float)(xn_fix - base) * (1.0f / 1099511627776.0f);
            accumulate_row(B, r, (int)col, fa, fn, dir * (qb - qa));
        }
        xa_fix = xn_fix;
        xb_fix += step;
    }
}

// Piece of a line after the x rules, in binary64 (x absolute, y relative to
// the band).  Clips it to the band's rows (a pure geometric clip, so the area
// inside is unchanged; one binary64 division for the slope, which the long
// route reuses), quantises y (COV_ONE per row) and dispatches it: short pieces
// to the FP32 distribution, long ones to the fixed-point row stepping.
__device__ inline void accumulate_piece64(const Band& B, double x0, double y0, double x1, double y1) {
    if (y0 == y1) return;
    const double lo = fmax(-1.0, -(double)B.y0 - 1.0);
    const double hi = (double)min(B.bh, B.img_h - B.y0) + 1.0;
    const double ymin = fmin(y0, y1), ymax = fmax(y0, y1);
    if (ymax <= lo || ymin >= hi) return;
    const double dxdy = (x1 - x0) / (y1 - y0);
    if (ymin < lo || ymax > hi) {
        if (y0 < lo) { x0 = x0 + (lo - y0) * dxdy; y0 = lo; }
        else if (y0 > hi) { x0 = x0 + (hi - y0) * dxdy; y0 = hi; }
        if (y1 < lo) { x1 = x0 + (lo - y0) * dxdy; y1 = lo; }
        else if (y1 > hi) { x1 = x0 + (hi - y0) * dxdy; y1 = hi; }
    }
    const int32_t q0 = __double2int_rn(y0 * 4194304.0), q1 = __double2int_rn(y1 * 4194304.0);
    if (fabs(x1 - x0) <= (double)kShortLine && abs(q1 - q0) <= (kShortLine << COV_SHIFT)) {
        const int xb = (int)floor(fmin(x0, x1));
        accumulate_piece(B, xb, (float)(x0 - xb), q0, (float)(x1 - xb), q1);
    } else {
        accumulate_piece_long(B, x0, q0, x1, q1, dxdy);
    }
}

// A flattened line in binary64 (x absolute, y relative to the band): applies
// the reference's right-edge rule (src/rasterize.rs:372-387) and
// split_at_zero_x (:923-937), then accumulates the pieces.
static __device__ __noinline__ void accumulate_line64(const Band& B, double ax, double ay, double bx, double by) {
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

// A flattened line vertex: integer column and band-relative row plus FP32
// fractions (a few px at most).  Both ends of every line go through the same
// quantisation, so a vertex shared by two lines gets one fixed-point height.
struct VtxQ {
    int32_t col, row;
    float fx, fy;
};

// Line between two vertices.  Short lines away from the x rules stay in FP32
// with exact fixed-point heights; the rest take the binary64 route, which
// quantises the same vertex to the same height.
// The FP32 route of accumulate_vtx alone: false when the line needs the
// binary64 route (long, or near the x rules' columns), which the caller then
// takes outside its hot loop.
__device__ __forceinline__ bool accumulate_vtx_short(const Band& B, const VtxQ& a, const VtxQ& b) {
    const int dc = b.col - a.col, dr = b.row - a.row;
    if (abs(dc) >= kShortLine || abs(dr) >= kShortLine) return false;
    if (a.row < -kShortLine - 4 || a.row > B.bh + kShortLine + 4) return true;  // wholly above or below
    const float x0 = a.fx, x1 = (float)dc + b.fx;
    const float xlo = (float)a.col + fminf(x0, x1), xhi = (float)a.col + fmaxf(x0, x1);
    if (!(xlo > 0.01f && xhi < B.width_f - 0.01f)) return false;
    const int32_t q0 = a.row * COV_ONE + __float2int_rn(a.fy * COV_ONE_F);
    const int32_t q1 = b.row * COV_ONE + __float2int_rn(b.fy * COV_ONE_F);
    accumulate_piece<true>(B, a.col, x0, q0, x1, q1);
    return true;
}

__device__ __forceinline__ void accumulate_vtx(const Band& B, const VtxQ& a, const VtxQ& b) {
    const int dc = b.col - a.col, dr = b.row - a.row;
    if (abs(dc) < kShortLine && abs(dr) < kShortLine) {
        // wholly above or below the band's rows (this also keeps the heights in int32)
        if (a.row < -kShortLine - 4 || a.row > B.bh + kShortLine + 4) return;
        const float x0 = a.fx, x1 = (float)dc + b.fx;
        const float xlo = (float)a.col + fminf(x0, x1), xhi = (float)a.col + fmaxf(x0, x1);
        if (xlo > 0.01f && xhi < B.width_f - 0.01f) {
            const int32_t q0 = a.row * COV_ONE + __float2int_rn(a.fy * COV_ONE_F);
            const int32_t q1 = b.row * COV_ONE + __float2int_rn(b.fy * COV_ONE_F);
            accumulate_piece<true>(B, a.col, x0, q0, x1, q1);
            return;
        }
    }
    accumulate_line64(B, (double)a.col + (double)a.fx, (double)a.row + (double)a.fy, (double)b.col + (double)b.fx,
                      (double)b.row + (double)b.fy);
}

// A stored line end (exact 16.16 anchor + FP32 remainder, frame of its view)
// as a vertex with its row relative to band row `row0`.
__device__ __forceinline__ VtxQ line_vtx(int4 e, int row0) {
    VtxQ v;
    v.col = e.x >> 16;
    v.row = (e.y >> 16) - row0;
    v.fx = fmaf((float)(e.x & 0xffff), 1.0f / 65536.0f, __int_as_float(e.z));
    v.fy = fmaf((float)(e.y & 0xffff), 1.0f / 65536.0f, __int_as_float(e.w));
    return v;
}

// ---------------------------------------------------------------------------
// Row prefix sum (exact integer) + fill rule
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

// FillRule::alpha_from_winding on a fixed-point winding (COV_ONE per unit):
// EvenOdd's |((w + 1) rem_euclid 2) - 1| is exact with a mask.
__device__ __forceinline__ float alpha_from_winding_fix(int rule, int32_t w) {
    if (rule == 1) {
        const int32_t r = (int32_t)(((uint32_t)w + (1u << 22)) & ((1u << 23) - 1u));
        return (float)abs(r - (1 << 22)) * (1.0f / 4194304.0f);
    }
    const float v = fabsf((float)w * (1.0f / 4194304.0f));
    return v >= 1.f ? 1.f : (v < 1e-6f ? 0.f : v);
}

// alpha_from_winding_fix with a rule known at compile time, in integer
// instructions and one FP32 add: for 0 <= m <= 2^22 the bits 0x3f800000 +
// 2m are the float 1 + m 2^-22 exactly, so subtracting 1 gives m 2^-22
// exactly (the same value the conversion route rounds to).  NonZero keeps
// the 1e-6 cut-off: m 2^-22 < 1e-6 exactly when m <= 4.
template <int RULE>
__device__ __forceinline__ float alpha_fix(uint32_t w) {
    uint32_t m;
    if (RULE == 1) {
        const int32_t r = (int32_t)((w + (1u << 22)) & ((1u << 23) - 1u));
        m = (uint32_t)abs(r - (1 << 22));
    } else {
        const uint32_t a = (int32_t)w < 0 ? 0u - w : w;
        m = min(a, 1u << 22);
        m = m <= 4u ? 0u : m;
    }
    return __int_as_float((int32_t)(0x3f800000u + (m << 1))) - 1.0f;
}

// The x rules of signed_difference_line (src/rasterize.rs:372-393) on a
// binary64 line: the part beyond `width` is dropped (a line entirely beyond
// becomes vertical at width - 0.001), then split_at_zero_x
// (src/rasterize.rs:923-937) turns the x < 0 part into a vertical line at 0.
// Returns the number of pieces (0..2); piece i is (px[i][0], py[i][0]) ->
// (px[i][1], py[i][1]).
__device__ inline int clip_line_x64(double width, double ax, double ay, double bx, double by, double (&px)[2][2],
                                    double (&py)[2][2]) {
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
        px[0][0] = ax; py[0][0] = ay; px[0][1] = bx; py[0][1] = by;
        return 1;
    }
    if (ax <= 0.0 && bx <= 0.0) {
        px[0][0] = 0.0; py[0][0] = ay; px[0][1] = 0.0; py[0][1] = by;
        return 1;
    }
    const double t = ax / (ax - bx);
    const double mx = (1.0 - t) * ax + t * bx, my = (1.0 - t) * ay + t * by;
    if (ax < 0.0) {
        px[0][0] = mx; py[0][0] = my; px[0][1] = bx; py[0][1] = by;
        px[1][0] = 0.0; py[1][0] = ay; px[1][1] = mx; py[1][1] = my;
    } else {
        px[0][0] = ax; py[0][0] = ay; px[0][1] = mx; py[0][1] = my;
        px[1][0] = mx; py[1][0] = my; px[1][1] = 0.0; py[1][1] = by;
    }
    return 2;
}

// Pure geometric clip of a piece to rows [lo, hi] (the area inside is
// unchanged); false when nothing is left.
__device__ inline bool clip_y64(double lo, double hi, double (&x)[2], double (&y)[2]) {
    const double ymin = fmin(y[0], y[1]), ymax = fmax(y[0], y[1]);
    if (ymax <= lo || ymin >= hi || y[0] == y[1]) return false;
    if (ymin < lo || ymax > hi) {
        const double dxdy = (x[1] - x[0]) / (y[1] - y[0]);
        const double x0 = x[0], y0 = y[0];
        for (int i = 0; i < 2; ++i) {
            if (y[i] < lo) { x[i] = x0 + (lo - y0) * dxdy; y[i] = lo; }
            else if (y[i] > hi) { x[i] = x0 + (hi - y0) * dxdy; y[i] = hi; }
        }
    }
    return true;
}

// ---------------------------------------------------------------------------
// Row prefix of a band (signed differences -> winding) and fill rule
// (src/rasterize.rs:473-507), in exact fixed-point integer arithmetic.  One
// warp per row, kScanChunk = 4 pixels per lane: a 16-byte load, the lane's
// inclusive prefix, a warp shuffle scan of the lane totals and the carry of
// the previous 128 columns; then epi(row, x0, alpha[4]) per lane.
// ---------------------------------------------------------------------------
constexpr int kScanChunk = 4;

// CLEAR: every word the band's writes can reach (columns [0, width + 2),
// the reference's two spill columns included) is zeroed as it is read, so the
// band is clear for the next work item without a separate pass.
template <int THREADS, class Epi, bool CLEAR = false>
__device__ void band_scan(const Band& B, int width, int rule, const Epi& epi) {
    const int lane = threadIdx.x & 31;
    const int span = CLEAR ? width + 2 : width;  // stride >= width + 2, a multiple of 16
    for (int r = threadIdx.x >> 5; r < B.bh; r += THREADS / 32) {
        int4* row4 = reinterpret_cast<int4*>(B.acc + r * B.stride);
        uint32_t carry = 0;  // unsigned: the winding wraps by design
        for (int x0 = 0; x0 < span; x0 += 32 * kScanChunk) {
            const int x = x0 + kScanChunk * lane;
            int4 v = make_int4(0, 0, 0, 0);
            if (x < span) {
                v = row4[x >> 2];
                if (CLEAR) row4[x >> 2] = make_int4(0, 0, 0, 0);
            }
            const uint32_t a0 = x < width ? (uint32_t)v.x : 0u;
            const uint32_t a1 = a0 + (x + 1 < width ? (uint32_t)v.y : 0u);
            const uint32_t a2 = a1 + (x + 2 < width ? (uint32_t)v.z : 0u);
            const uint32_t a3 = a2 + (x + 3 < width ? (uint32_t)v.w : 0u);
            uint32_t incl = a3;
            #pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const uint32_t o = __shfl_up_sync(0xffffffffu, incl, off);
                if (lane >= off) incl += o;
            }
            const uint32_t base = carry + incl - a3;
            carry += __shfl_sync(0xffffffffu, incl, 31);
            if (x < width) {
                const float a[kScanChunk] = {alpha_from_winding_fix(rule, (int32_t)(base + a0)),
                                             alpha_from_winding_fix(rule, (int32_t)(base + a1)),
                                             alpha_from_winding_fix(rule, (int32_t)(base + a2)),
                                             alpha_from_winding_fix(rule, (int32_t)(base + a3))};
                epi(r, x, a);
            }
        }
    }
}

// The row scan of a mask band with 8 pixels a lane (two 16-byte loads, 256
// columns per warp step) for a fill rule known at compile time (RULE: 0
// NonZero, 1 EvenOdd), clearing the words it reads (columns [0, width + 2))
// and streaming the alphas to mask rows `out + (y0 + r) * row_stride`.
// Bit-identical to band_scan with MaskStore.
// Rows of at most 128 columns are scanned several to a warp: L lanes (a power
// of two, 8 columns each) per row, the warp scan segmented to L lanes.  The
// sums are the same integers in the same wrap-around arithmetic.
template <int THREADS, int RULE>
__device__ void band_scan8_narrow(const Band& B, int width, float* out, int64_t row_stride, int y0) {
    const int lane = threadIdx.x & 31;
    const int span = width + 2;  // <= 128
    const int lg = span <= 8 ? 0 : 32 - __clz((span + 7) / 8 - 1);  // log2 L
    const int L = 1 << lg;
    const int sl = lane & (L - 1);
    const int per_warp = 32 >> lg;
    const int x = 8 * sl;
    for (int r0 = (threadIdx.x >> 5) * per_warp; r0 < B.bh; r0 += (THREADS / 32) * per_warp) {
        const int r = r0 + (lane >> lg);
        const bool live = r < B.bh;
        int4 v = make_int4(0, 0, 0, 0), u = make_int4(0, 0, 0, 0);
        if (live && x < span) {
            int4* row4 = reinterpret_cast<int4*>(B.acc + r * B.stride);
            v = row4[x >> 2];
            u = row4[(x >> 2) + 1];  // x + 8 <= stride
            row4[x >> 2] = make_int4(0, 0, 0, 0);
            row4[(x >> 2) + 1] = make_int4(0, 0, 0, 0);
        }
        // the spill columns only reach prefixes at or past width, which are not stored
        uint32_t a[8];
        a[0] = (uint32_t)v.x;
        a[1] = a[0] + (uint32_t)v.y;
        a[2] = a[1] + (uint32_t)v.z;
        a[3] = a[2] + (uint32_t)v.w;
        a[4] = a[3] + (uint32_t)u.x;
        a[5] = a[4] + (uint32_t)u.y;
        a[6] = a[5] + (uint32_t)u.z;
        a[7] = a[6] + (uint32_t)u.w;
        uint32_t incl = a[7];
        for (int off = 1; off < L; off <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, incl, off, L);
            if (sl >= off) incl += t;
        }
        const uint32_t base = incl - a[7];
        if (live && x < width) {
            float* o = out + (int64_t)(y0 + r) * row_stride;
            float al[8];
            #pragma unroll
            for (int i = 0; i < 8; ++i) al[i] = alpha_fix<RULE>(base + a[i]);
            if ((reinterpret_cast<uintptr_t>(o) & 15u) == 0 && x + 8 <= width) {
                __stcs(reinterpret_cast<float4*>(o + x), make_float4(al[0], al[1], al[2], al[3]));
                __stcs(reinterpret_cast<float4*>(o + x + 4), make_float4(al[4], al[5], al[6], al[7]));
            } else {
                #pragma unroll
                for (int i = 0; i < 8; ++i)
                    if (x + i < width) o[x + i] = al[i];
            }
        }
    }
}

template <int THREADS, int RULE>
__device__ void band_scan8(const Band& B, int width, float* out, int64_t row_stride, int y0) {
    const int lane = threadIdx.x & 31;
    const int span = width + 2;  // stride >= width + 2, a multiple of 16
    if (span <= 128) {
        band_scan8_narrow<THREADS, RULE>(B, width, out, row_stride, y0);
        return;
    }
    for (int r = threadIdx.x >> 5; r < B.bh; r += THREADS / 32) {
        int4* row4 = reinterpret_cast<int4*>(B.acc + r * B.stride);
        float* o = out + (int64_t)(y0 + r) * row_stride;
        const bool aligned = (reinterpret_cast<uintptr_t>(o) & 15u) == 0;
        uint32_t carry = 0;  // unsigned: the winding wraps by design
        for (int x0 = 0; x0 < span; x0 += 256) {
            const int x = x0 + 8 * lane;
            int4 v = make_int4(0, 0, 0, 0), u = make_int4(0, 0, 0, 0);
            if (x < span) {
                v = row4[x >> 2];
                u = row4[(x >> 2) + 1];  // x + 8 <= stride
                row4[x >> 2] = make_int4(0, 0, 0, 0);
                row4[(x >> 2) + 1] = make_int4(0, 0, 0, 0);
            }
            // the spill columns (width, width + 1) only reach prefixes at or past width, which are not stored
            uint32_t a[8];
            a[0] = (uint32_t)v.x;
            a[1] = a[0] + (uint32_t)v.y;
            a[2] = a[1] + (uint32_t)v.z;
            a[3] = a[2] + (uint32_t)v.w;
            a[4] = a[3] + (uint32_t)u.x;
            a[5] = a[4] + (uint32_t)u.y;
            a[6] = a[5] + (uint32_t)u.z;
            a[7] = a[6] + (uint32_t)u.w;
            uint32_t incl = a[7];
            #pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const uint32_t t = __shfl_up_sync(0xffffffffu, incl, off);
                if (lane >= off) incl += t;
            }
            const uint32_t base = carry + incl - a[7];
            carry += __shfl_sync(0xffffffffu, incl, 31);
            float al[8];
            #pragma unroll
            for (int i = 0; i < 8; ++i) al[i] = alpha_fix<RULE>(base + a[i]);
            if (aligned && x + 8 <= width) {
                __stcs(reinterpret_cast<float4*>(o + x), make_float4(al[0], al[1], al[2], al[3]));
                __stcs(reinterpret_cast<float4*>(o + x + 4), make_float4(al[4], al[5], al[6], al[7]));
            } else if (x < width) {
                #pragma unroll
                for (int i = 0; i < 8; ++i)
                    if (x + i < width) o[x + i] = al[i];
            }
        }
    }
}

// Mask epilogue of the row scan: a 16-byte streaming store of 4 alphas.
struct MaskStore {
    float* out;
    uint64_t offset;
    int64_t row_stride;
    int y0, width;
    __device__ __forceinline__ void operator()(int r, int x0, const float (&a)[kScanChunk]) const {
        float* o = out + offset + (uint64_t)(y0 + r) * (uint64_t)row_stride + x0;
        if (((reinterpret_cast<uintptr_t>(o) & 15u) == 0) && (x0 + kScanChunk <= width)) {
            __stcs(reinterpret_cast<float4*>(o), make_float4(a[0], a[1], a[2], a[3]));
        } else {
            #pragma unroll
            for (int i = 0; i < kScanChunk; ++i)
                if (x0 + i < width) o[i] = a[i];
        }
    }
};

// Staging epilogue of the row scan: the alphas replace the row's accumulation
// words in shared memory (each lane reads its 4 words before it writes them).
struct SmemStore {
    float* acc;
    int stride;
    __device__ __forceinline__ void operator()(int r, int x0, const float (&a)[kScanChunk]) const {
        *reinterpret_cast<float4*>(acc + r * stride + x0) = make_float4(a[0], a[1], a[2], a[3]);
    }
};

// Streams a staged band (rows x width alphas at `stride` in shared memory) to
// a mask whose rows are packed (row stride == width): one contiguous span of
// rows * width floats, written with aligned 16-byte stores, so every 128-byte
// line inside the span is written whole by one warp instruction.  Over a
// host link (page-locked output) partial lines cost a transaction each.
template <int THREADS>
__device__ void band_flush(const float* acc, int stride, int rows, int width, float* dst) {
    const uint32_t n = (uint32_t)rows * (uint32_t)width;
    const uint32_t head = min((uint32_t)(((16u - ((uint32_t)reinterpret_cast<uintptr_t>(dst) & 15u)) & 15u) >> 2), n);
    const uint32_t n4 = (n - head) >> 2;
    const uint32_t tid = threadIdx.x;
    if (tid < head) {
        const uint32_t r = tid / (uint32_t)width;
        dst[tid] = acc[r * stride + (tid - r * width)];
    }
    float4* d4 = reinterpret_cast<float4*>(dst + head);
    for (uint32_t j = tid; j < n4; j += THREADS) {
        const uint32_t i = head + 4u * j;
        uint32_t r = i / (uint32_t)width, c = i - r * (uint32_t)width;
        float v[4];
        #pragma unroll
        for (int k = 0; k < 4; ++k) {
            v[k] = acc[r * stride + c];
            if (++c == (uint32_t)width) {
                c = 0;
                ++r;
            }
        }
        __stcs(d4 + j, make_float4(v[0], v[1], v[2], v[3]));
    }
    for (uint32_t i = head + 4u * n4 + tid; i < n; i += THREADS) {
        const uint32_t r = i / (uint32_t)width;
        dst[i] = acc[r * stride + (i - r * width)];
    }
}

// ---------------------------------------------------------------------------
// Segment records shared by the band kernel and the line pipeline
// ---------------------------------------------------------------------------
struct SegRec {
    int32_t xb, yb;  // record origin: integer column and row of P0 (image frame)
    int8_t anchor;   // anchor level a: vertices are B(m / 2^a) exactly plus an FP32 remainder
    int8_t scale;    // k: coordinates are integers in units of 2^-k px (16..24)
    int16_t kind;
    int32_t p0x, p0y, pnx, pny;           // end points relative to (xb, yb)
    int32_t d1x, d1y, d2x, d2y, d3x, d3y;  // control point differences
    float mag;                            // max |absolute coordinate|, px (binary64 chain error term)
    uint32_t src;                         // input segment, for binary64 re-decisions (~0: a line)
};

// Power-basis coefficients in px: B(t) - P0 = t (c1 + t (c2 + t c3)).  For a
// cubic c2 and c3 are also the flatness coefficients a2 and a3; for a quad c2
// is P0 - 2 P1 + P2.
__device__ __forceinline__ void rec_coefs(const SegRec& r, int kind, float& c1x, float& c1y, float& c2x, float& c2y,
                                          float& c3x, float& c3y) {
    const float u = pow2f(-r.scale);
    const float d1x = (float)r.d1x * u, d1y = (float)r.d1y * u;
    const float d2x = (float)r.d2x * u, d2y = (float)r.d2y * u;
    const float d3x = (float)r.d3x * u, d3y = (float)r.d3y * u;
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
// binary64 control points (quantisation 2^-(k+1) px per coordinate, plus FP32
// rounding).
__device__ __forceinline__ FlatCoef rec_flat(const SegRec& r, float& qerr) {
    float c1x, c1y, c2x, c2y, c3x, c3y;
    rec_coefs(r, r.kind, c1x, c1y, c2x, c2y, c3x, c3y);
    FlatCoef c;
    c.a2x = c2x; c.a2y = c2y; c.a3x = c3x; c.a3y = c3y;
    c.mag = r.mag;
    const float u = pow2f(-r.scale);
    const float sx = fabsf((float)r.d1x) + fabsf((float)r.d2x) + fabsf((float)r.d3x);
    const float sy = fabsf((float)r.d1y) + fabsf((float)r.d2y) + fabsf((float)r.d3y);
    qerr = fmaxf(sx, sy) * u * pow2f(-19) + 6.f * u;
    return c;
}

// Control hull of a fixed-point segment against rows [y0 - 1, y0 + rows + 1).
__device__ __forceinline__ bool hull_meets_rows(const FixSeg& s, int y0, int rows) {
    int32_t ymin = s.y[0], ymax = s.y[0];
    #pragma unroll
    for (int i = 1; i < 4; ++i) {
        if (i < seg_npts(s.kind)) {
            ymin = min(ymin, s.y[i]);
            ymax = max(ymax, s.y[i]);
        }
    }
    const int32_t oy = y0 << 16;  // image heights are limited to 16383 rows
    return !(ymax < oy - 65536 || ymin > oy + ((rows + 1) << 16));
}

// x * 2^k rounded half-even, integer instructions only; |x| < 16384 (checked
// by d2fix), k <= 24.
__device__ __forceinline__ long long d2fix_k(double x, int k) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((bits >> 52) & 0x7ffull);
    if (e == 0) return 0;
    const unsigned long long mant = (bits & 0xfffffffffffffull) | (1ull << 52);
    const int sh = 1075 - k - e;  // x * 2^k = mant * 2^-sh
    unsigned long long q;
    if (sh >= 64) {
        q = 0;
    } else if (sh <= 0) {
        q = mant << (-sh);
    } else {
        q = mant >> sh;
        const unsigned long long rem = mant - (q << sh);
        const unsigned long long half = 1ull << (sh - 1);
        if (rem > half || (rem == half && (q & 1ull))) ++q;
    }
    return (bits >> 63) ? -(long long)q : (long long)q;
}

// Record of a segment inside the 16.16 range: binary64 control points `sx`,
// `sy` (after the transform) and their 16.16 copy `s`.  Coordinates are
// re-quantised relative to the integer origin at P0 with the finest scale
// 2^-k that keeps every difference in int32 (2^-24 px for segments up to
// ~60 px), so the vertices stay within ~1e-7 px of the binary64 curve.
__device__ inline void make_record(const FixSeg& s, const double (&sx)[4], const double (&sy)[4], SegRec& r) {
    const int n = seg_npts(s.kind);
    const int32_t xb = s.x[0] >> 16, yb = s.y[0] >> 16;  // floor
    int32_t ext16 = 0, mx = 0;
    #pragma unroll
    for (int i = 0; i < 4; ++i) {
        if (i < n) {
            ext16 = max(ext16, max(abs(s.x[i] - (xb << 16)), abs(s.y[i] - (yb << 16))));
            mx = max(mx, max(abs(s.x[i]), abs(s.y[i])));
        }
    }
    // 2 * extent * 2^k < 2^31
    const int bits = 32 - __clz(ext16 + 65536);
    const int k = min(24, max(16, 46 - bits));
    long long X[4], Y[4];
    #pragma unroll
    for (int i = 0; i < 4; ++i) {
        X[i] = i < n ? d2fix_k(sx[i], k) : 0;
        Y[i] = i < n ? d2fix_k(sy[i], k) : 0;
    }
    const long long ox = (long long)xb << k, oy = (long long)yb << k;
    const long long xn = n == 2 ? X[1] : (n == 3 ? X[2] : X[3]);
    const long long yn = n == 2 ? Y[1] : (n == 3 ? Y[2] : Y[3]);
    r.xb = xb;
    r.yb = yb;
    r.scale = (int8_t)k;
    r.p0x = (int32_t)(X[0] - ox);
    r.p0y = (int32_t)(Y[0] - oy);
    r.pnx = (int32_t)(xn - ox);
    r.pny = (int32_t)(yn - oy);
    r.d1x = (int32_t)(X[1] - X[0]);
    r.d1y = (int32_t)(Y[1] - Y[0]);
    r.d2x = n > 2 ? (int32_t)(X[2] - X[1]) : 0;
    r.d2y = n > 2 ? (int32_t)(Y[2] - Y[1]) : 0;
    r.d3x = n > 3 ? (int32_t)(X[3] - X[2]) : 0;
    r.d3y = n > 3 ? (int32_t)(Y[3] - Y[2]) : 0;
    r.kind = (int16_t)s.kind;
    float c1x, c1y, c2x, c2y, c3x, c3y;
    rec_coefs(r, s.kind, c1x, c1y, c2x, c2y, c3x, c3y);
    // Anchor level: sub-curves over 2^-a of the parameter span stay below
    // RZ_ANCHOR_PX px, so the FP32 remainder keeps ~RZ_ANCHOR_PX x 1e-7 px.
    // Lines need no anchors (t is 0 or 1).  a <= 9 keeps the integer
    // evaluation below 2^62.
    const float ext = fmaxf(fabsf(c1x) + fabsf(c2x) + fabsf(c3x), fabsf(c1y) + fabsf(c2y) + fabsf(c3y));
    int a = 0;
    if (s.kind != SEG_LINE) {
        while (a < 9 && ext * pow2f(-a) > (float)RZ_ANCHOR_PX) ++a;
    }
    r.mag = (float)mx * FIX_ONE_INV;
    r.anchor = (int8_t)a;
}

// Vertex at t = j / 2^d as an exact integer point I (units 2^-k, relative to
// the record's origin) plus an FP32 remainder R in px.  The anchor depends on
// t only, so two leaves sharing a vertex compute it identically.
__device__ __forceinline__ void rec_vertex(const SegRec& r, uint32_t j, int d, int32_t& ix, int32_t& iy, float& rx,
                                           float& ry) {
    if (j == 0) {
        ix = r.p0x; iy = r.p0y; rx = ry = 0.f;
        return;
    }
    if ((j >> d) != 0u) {
        ix = r.pnx; iy = r.pny; rx = ry = 0.f;
        return;
    }
    const int a = r.anchor;
    float c1x, c1y, c2x, c2y, c3x, c3y;
    rec_coefs(r, r.kind, c1x, c1y, c2x, c2y, c3x, c3y);
    if (a == 0) {
        const float t = (float)j * pow2f(-d);
        ix = r.p0x; iy = r.p0y;
        rx = t * fmaf(t, fmaf(t, c3x, c2x), c1x);
        ry = t * fmaf(t, fmaf(t, c3y, c2y), c1y);
        return;
    }
    // anchor m / 2^a <= t, exact B(m / 2^a) from integer power-basis coefficients
    const uint32_t m = d >= a ? (j >> (d - a)) : (j << (a - d));
    const uint32_t jm = d >= a ? (m << (d - a)) : j;
    const long long mm = (long long)m;
    // integer power basis: B(t) - P0 = t (k1 + t (k2 + t k3)) in units of 2^-k
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
    const long long qx = (nx + half) >> sh, qy = (ny + half) >> sh;
    ix = r.p0x + (int32_t)qx;
    iy = r.p0y + (int32_t)qy;
    // the rounding of the anchor (|.| <= 2^(sh-1), an int32), carried in the remainder
    const float ru = pow2f(-(r.scale + sh));
    rx = (float)(int32_t)(nx - qx * (1ll << sh)) * ru;
    ry = (float)(int32_t)(ny - qy * (1ll << sh)) * ru;
    if (jm == j) return;
    // remainder over dt = t - m / 2^a with the local power basis at tA
    const float tA = (float)m * pow2f(-a);
    const float dt = (float)(j - jm) * pow2f(-d);
    const float b1x = fmaf(tA, fmaf(3.f * tA, c3x, 2.f * c2x), c1x);
    const float b1y = fmaf(tA, fmaf(3.f * tA, c3y, 2.f * c2y), c1y);
    const float b2x = fmaf(3.f * tA, c3x, c2x), b2y = fmaf(3.f * tA, c3y, c2y);
    rx += dt * fmaf(dt, fmaf(dt, c3x, b2x), b1x);
    ry += dt * fmaf(dt, fmaf(dt, c3y, b2y), b1y);
}

// Vertex of a record as an integer column / row (row relative to `row0`)
// plus FP32 fractions.
__device__ __forceinline__ VtxQ rec_vtx(const SegRec& r, uint32_t j, int d, int row0) {
    int32_t ix, iy;
    float rx, ry;
    rec_vertex(r, j, d, ix, iy, rx, ry);
    const int k = r.scale;
    const int32_t mask = (1 << k) - 1;
    const float u = pow2f(-k);
    VtxQ v;
    v.col = r.xb + (ix >> k);
    v.row = r.yb + (iy >> k) - row0;
    v.fx = fmaf((float)(ix & mask), u, rx);
    v.fy = fmaf((float)(iy & mask), u, ry);
    return v;
}

// Reference decision for node (d, k) of a record: FP32 with a rigorous bound,
// binary64 replay of the split chain when too close to call.  `pts` and
// `trm` give the record's binary64 source segment.
__device__ __forceinline__ int decide_node(const SegRec& r, const FlatCoef& c, float qerr, int d, uint32_t k,
                                           float thr32, double thr64, const double* pts, const double* trm,
                                           int& fallbacks) {
    if (r.kind == SEG_LINE) return 1;
    const int v = decide_fp32<true>(r.kind, c, d, k, thr32, qerr);
    if (v >= 0) return v;
    Seg64 S;
    S.kind = r.kind;
    const double* p = pts + 8ull * r.src;
    #pragma unroll
    for (int j = 0; j < 4; ++j) { S.x[j] = p[2 * j]; S.y[j] = p[2 * j + 1]; }
    if (trm) {
        #pragma unroll
        for (int j = 0; j < 4; ++j) tr_apply64(trm, S.x[j], S.y[j], S.x[j], S.y[j]);
    }
    ++fallbacks;
    return flatness_chain64(S, d, k) < thr64 ? 1 : 0;
}

}  // namespace rz
