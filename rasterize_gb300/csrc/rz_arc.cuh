// rz_arc.cuh -- SVG elliptic arc -> cubics on the device, in binary64.
//
// Restates EllipArc::new_param (src/ellipse.rs:40-96) and
// EllipArcCubicIter (src/ellipse.rs:159-214) as PathBuilder::arc_to
// (src/path.rs:945-972) applies them: the endpoint-to-centre
// parametrisation (SVG implementation notes eqs. 5.1-5.6) followed by at most
// four cubic pieces of <= pi/2 each with
// alpha = sin(d) (sqrt(4 + 3 tan^2(d/2)) - 1) / 3.
// Arithmetic follows the reference's operation order without contraction;
// the transcendental functions are CUDA's binary64 ones.
#pragma once
#include "rz_device.cuh"

namespace rz {

constexpr double PI64 = 3.141592653589793;
constexpr double EPS64 = 2.220446049250313e-16;

__device__ inline double rem_euclid64(double a, double b) {
    double r = fmod(a, b);
    return r < 0.0 ? da(r, fabs(b)) : r;
}

// Point::angle_between src/geometry.rs:186-203 (false for None)
__device__ inline bool angle_between64(double ax, double ay, double bx, double by, double& out) {
    const double lengths = dm(hypot(ax, ay), hypot(bx, by));
    if (lengths < EPS64) return false;
    double c = da(dm(ax, bx), dm(ay, by)) / lengths;
    c = c < -1.0 ? -1.0 : (c > 1.0 ? 1.0 : c);
    const double ang = acos(c);
    const double cross = ds(dm(ax, by), dm(ay, bx));
    out = cross < 0.0 ? -ang : ang;
    return true;
}

// Returns the number of cubics (0..4), -1 when new_param yields None (the
// builder falls back to line_to), -2 when the cubic count is not finite.
__device__ inline int arc_to_cubics64(const double* a, Seg64* out) {
    const double sx = a[0], sy = a[1], dx = a[2], dy = a[3];
    double rx = fabs(a[4]), ry = fabs(a[5]);
    const int flags = (int)a[7];
    const bool large = flags & 1, sweep = (flags & 2) != 0;
    const double phi = dm(a[6], PI64) / 180.0;
    // Eq 5.1: rotate(-phi) applied to 0.5 (src - dst)
    const double hx = dm(0.5, ds(sx, dx)), hy = dm(0.5, ds(sy, dy));
    const double sn = sin(-phi), cs = cos(-phi);
    const double x1 = da(da(dm(hx, cs), dm(hy, -sn)), 0.0);
    const double y1 = da(da(dm(hx, sn), dm(hy, cs)), 0.0);
    const double qx = x1 / rx, qy = y1 / ry;
    const double s = da(dm(qx, qx), dm(qy, qy));
    if (s > 1.0) {
        const double ss = sqrt(s);
        rx = dm(rx, ss);
        ry = dm(ry, ss);
    }
    // Eq 5.2
    const double rxry = dm(rx, ry), rxy1 = dm(rx, y1), ryx1 = dm(ry, x1);
    double sq = sqrt(fmax(ds(dm(rxry, rxry) / da(dm(rxy1, rxy1), dm(ryx1, ryx1)), 1.0), 0.0));
    if (large == sweep) sq = -sq;
    const double cx = dm(sq, dm(rx, y1) / ry);
    const double cy = dm(sq, dm(-ry, x1) / rx);
    // Eq 5.3
    const double sp = sin(phi), cp = cos(phi);
    const double ccx = da(da(da(dm(cx, cp), dm(cy, -sp)), 0.0), dm(0.5, da(dx, sx)));
    const double ccy = da(da(da(dm(cx, sp), dm(cy, cp)), 0.0), dm(0.5, da(dy, sy)));
    // Eq 5.5-6
    const double v1x = ds(x1, cx) / rx, v1y = ds(y1, cy) / ry;
    const double v2x = ds(-x1, cx) / rx, v2y = ds(-y1, cy) / ry;
    double eta, eta_delta;
    if (!angle_between64(1.0, 0.0, v1x, v1y, eta)) return -1;
    if (!angle_between64(v1x, v1y, v2x, v2y, eta_delta)) return -1;
    eta_delta = rem_euclid64(eta_delta, dm(2.0, PI64));
    if (!sweep && eta_delta > 0.0) eta_delta = ds(eta_delta, dm(2.0, PI64));
    else if (sweep && eta_delta < 0.0) eta_delta = da(eta_delta, dm(2.0, PI64));
    // EllipArcCubicIter::new / next
    const double count = ceil(fabs(eta_delta) / (PI64 / 2.0));
    if (!isfinite(count)) return -2;
    const double delta = eta_delta / count;
    const double last = ds(count, 1.0);
    int n = 0;
    for (double idx = 0.0; !(idx > last); idx = da(idx, 1.0)) {
        if (n >= 4) return -2;
        const double e1 = da(eta, dm(delta, idx));
        const double e2 = da(e1, delta);
        const double tn = tan(ds(e2, e1) / 2.0);
        const double sqv = sqrt(da(4.0, dm(3.0, dm(tn, tn))));
        const double alpha = dm(sin(ds(e2, e1)), ds(sqv, 1.0)) / 3.0;
        const double s1 = sin(e1), c1 = cos(e1), s2 = sin(e2), c2 = cos(e2);
        // at = rotate(phi)[rx cos, ry sin] + center; deriv = rotate(phi)[-rx sin, ry cos]
        const double ax0 = dm(rx, c1), ay0 = dm(ry, s1);
        const double p0x = da(da(da(dm(ax0, cp), dm(ay0, -sp)), 0.0), ccx);
        const double p0y = da(da(da(dm(ax0, sp), dm(ay0, cp)), 0.0), ccy);
        const double bx0 = dm(-rx, s1), by0 = dm(ry, c1);
        const double d0x = da(da(dm(bx0, cp), dm(by0, -sp)), 0.0);
        const double d0y = da(da(dm(bx0, sp), dm(by0, cp)), 0.0);
        const double ax3 = dm(rx, c2), ay3 = dm(ry, s2);
        const double p3x = da(da(da(dm(ax3, cp), dm(ay3, -sp)), 0.0), ccx);
        const double p3y = da(da(da(dm(ax3, sp), dm(ay3, cp)), 0.0), ccy);
        const double bx3 = dm(-rx, s2), by3 = dm(ry, c2);
        const double d3x = da(da(dm(bx3, cp), dm(by3, -sp)), 0.0);
        const double d3y = da(da(dm(bx3, sp), dm(by3, cp)), 0.0);
        Seg64& o = out[n++];
        o.kind = SEG_CUBIC;
        o.x[0] = p0x; o.y[0] = p0y;
        o.x[1] = da(p0x, dm(alpha, d0x)); o.y[1] = da(p0y, dm(alpha, d0y));
        o.x[2] = ds(p3x, dm(alpha, d3x)); o.y[2] = ds(p3y, dm(alpha, d3y));
        o.x[3] = p3x; o.y[3] = p3y;
    }
    return n;
}

// Expands input segment i into at most four reference segments (untransformed).
// Returns the count, or -2 when an arc has no finite cubic count.
__device__ inline int expand_segment(int kind, const double* p, Seg64* out) {
    if (kind != SEG_ARC) {
        Seg64& o = out[0];
        o.kind = kind;
        for (int j = 0; j < 4; ++j) { o.x[j] = p[2 * j]; o.y[j] = p[2 * j + 1]; }
        return 1;
    }
    const int n = arc_to_cubics64(p, out);
    if (n == -1) {
        // PathBuilder::line_to skips a point that is_close_to the position
        if (fabs(p[0] - p[2]) < EPS64 && fabs(p[1] - p[3]) < EPS64) return 0;
        Seg64& o = out[0];
        o.kind = SEG_LINE;
        o.x[0] = p[0]; o.y[0] = p[1]; o.x[1] = p[2]; o.y[1] = p[3];
        o.x[2] = o.y[2] = o.x[3] = o.y[3] = 0.0;
        return 1;
    }
    return n;
}

}  // namespace rz
