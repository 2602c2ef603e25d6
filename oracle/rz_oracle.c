/*
 * rz_oracle.c -- CPU f64 restatement of aslpavel/rasterize v0.6.7's hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: pytest, the smoke test
 * and the CPU baseline leg of bench.py load it.  The product library
 * (rasterize_gb300/) never links, loads or calls anything in oracle/.
 *
 * Every function follows the cited reference lines operation by operation, in
 * the same IEEE-754 binary64 order, so results match the Rust crate bit for bit
 * on the same inputs (Rust never contracts a*b+c into an FMA; this file must be
 * compiled with -ffp-contract=off for the same reason).
 *
 * Parity is pinned by the reference's own known-answer tests, restated in
 * tests/test_oracle_kat.py with the reference's expected numbers.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define RZO_EPSILON 2.220446049250313e-16      /* geometry.rs:14 f64::EPSILON */
#define RZO_EPSILON_SQRT 1.4901161193847656e-08 /* geometry.rs:16 */
#define RZO_PI 3.141592653589793

enum { SEG_LINE = 0, SEG_QUAD = 1, SEG_CUBIC = 2, SEG_ARC = 3 };
enum { RULE_NONZERO = 0, RULE_EVENODD = 1 };

typedef struct { double x, y; } pt;
typedef struct { double m[6]; } xform; /* [m00, m01, m02, m10, m11, m12] geometry.rs:317 */
typedef struct { int kind; pt p[4]; } seg;
typedef struct { pt a, b; } line_t;

/* ------------------------------------------------------------------------ */
/* geometry.rs                                                              */
/* ------------------------------------------------------------------------ */

/* Transform::apply geometry.rs:363-367 */
static inline pt tr_apply(const xform* t, pt p) {
    pt r;
    r.x = p.x * t->m[0] + p.y * t->m[1] + t->m[2];
    r.y = p.x * t->m[3] + p.y * t->m[4] + t->m[5];
    return r;
}

/* Transform * Transform geometry.rs:519-539 */
static xform tr_mul(xform s, xform o) {
    xform r;
    r.m[0] = s.m[0] * o.m[0] + s.m[1] * o.m[3];
    r.m[1] = s.m[0] * o.m[1] + s.m[1] * o.m[4];
    r.m[2] = s.m[0] * o.m[2] + s.m[1] * o.m[5] + s.m[2];
    r.m[3] = s.m[3] * o.m[0] + s.m[4] * o.m[3];
    r.m[4] = s.m[3] * o.m[1] + s.m[4] * o.m[4];
    r.m[5] = s.m[3] * o.m[2] + s.m[4] * o.m[5] + s.m[5];
    return r;
}

/* Transform::invert geometry.rs:370-384; returns 0 when not invertible */
static int tr_invert(xform t, xform* out) {
    double m00 = t.m[0], m01 = t.m[1], m02 = t.m[2], m10 = t.m[3], m11 = t.m[4], m12 = t.m[5];
    double det = m00 * m11 - m10 * m01;
    if (fabs(det) <= RZO_EPSILON) return 0;
    double o00 = m11 / det;
    double o01 = -m01 / det;
    double o10 = -m10 / det;
    double o11 = m00 / det;
    double o02 = -o00 * m02 - o01 * m12;
    double o12 = -o10 * m02 - o11 * m12;
    out->m[0] = o00; out->m[1] = o01; out->m[2] = o02;
    out->m[3] = o10; out->m[4] = o11; out->m[5] = o12;
    return 1;
}

static xform tr_identity(void) { xform t = {{1, 0, 0, 0, 1, 0}}; return t; }
static xform tr_translate(double tx, double ty) { xform t = {{1, 0, tx, 0, 1, ty}}; return t; }
static xform tr_scale(double sx, double sy) { xform t = {{sx, 0, 0, 0, sy, 0}}; return t; }
/* Transform::new_rotate geometry.rs:409-412 */
static xform tr_rotate(double a) { xform t = {{cos(a), -sin(a), 0, sin(a), cos(a), 0}}; return t; }

static double rust_fmax(double a, double b) { return fmax(a, b); }
static double rust_fmin(double a, double b) { return fmin(a, b); }
/* f64::rem_euclid */
static double rem_euclid(double a, double b) {
    double r = fmod(a, b);
    return r < 0.0 ? r + fabs(b) : r;
}
/* utils.rs:7-17 clamp */
static double clampd(double v, double lo, double hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* Point::cos_between / angle_between geometry.rs:186-203; returns 0 for None */
static int angle_between(pt a, pt b, double* out) {
    double lengths = hypot(a.x, a.y) * hypot(b.x, b.y);
    if (lengths < RZO_EPSILON) return 0;
    double cosv = (a.x * b.x + a.y * b.y) / lengths;
    double ang = acos(clampd(cosv, -1.0, 1.0));
    double cross = a.x * b.y - a.y * b.x;
    *out = cross < 0.0 ? -ang : ang;
    return 1;
}

/* ------------------------------------------------------------------------ */
/* curve.rs                                                                 */
/* ------------------------------------------------------------------------ */

static int seg_npts(int kind) { return kind == SEG_LINE ? 2 : (kind == SEG_QUAD ? 3 : 4); }

static seg seg_transform(const seg* s, const xform* t) {
    seg r; r.kind = s->kind;
    int n = seg_npts(s->kind);
    for (int i = 0; i < n; i++) r.p[i] = tr_apply(t, s->p[i]);
    for (int i = n; i < 4; i++) r.p[i] = s->p[i];
    return r;
}

static pt seg_start(const seg* s) { return s->p[0]; }
static pt seg_end(const seg* s) { return s->p[seg_npts(s->kind) - 1]; }

/* Line::flatness curve.rs:233-235, Quad::flatness :413-417, Cubic::flatness :692-697 */
static double seg_flatness(const seg* s) {
    if (s->kind == SEG_LINE) return 0.0;
    if (s->kind == SEG_QUAD) {
        const pt* p = s->p;
        double x = 2.0 * p[1].x - p[0].x - p[2].x;
        double y = 2.0 * p[1].y - p[0].y - p[2].y;
        return x * x + y * y;
    }
    const pt* p = s->p;
    double ux = 3.0 * p[1].x - 2.0 * p[0].x - p[3].x;
    double uy = 3.0 * p[1].y - 2.0 * p[0].y - p[3].y;
    double vx = 3.0 * p[2].x - p[0].x - 2.0 * p[3].x;
    double vy = 3.0 * p[2].y - p[0].y - 2.0 * p[3].y;
    return rust_fmax(ux * ux, vx * vx) + rust_fmax(uy * uy, vy * vy);
}

/* Line::split via split_at(0.5) curve.rs:258-262 (only reachable with flatness <= 0),
 * Quad::split :449-456, Cubic::split :731-747 */
static void seg_split(const seg* s, seg* a, seg* b) {
    a->kind = b->kind = s->kind;
    const pt* p = s->p;
    if (s->kind == SEG_LINE) {
        /* Line::at curve.rs:249-252: (1 - t) * p0 + t * p1 */
        pt mid = { 0.5 * p[0].x + 0.5 * p[1].x, 0.5 * p[0].y + 0.5 * p[1].y };
        a->p[0] = p[0]; a->p[1] = mid;
        b->p[0] = mid; b->p[1] = p[1];
    } else if (s->kind == SEG_QUAD) {
        pt mid = { 0.25 * (p[0].x + 2.0 * p[1].x + p[2].x), 0.25 * (p[0].y + 2.0 * p[1].y + p[2].y) };
        a->p[0] = p[0];
        a->p[1].x = 0.5 * (p[0].x + p[1].x); a->p[1].y = 0.5 * (p[0].y + p[1].y);
        a->p[2] = mid;
        b->p[0] = mid;
        b->p[1].x = 0.5 * (p[1].x + p[2].x); b->p[1].y = 0.5 * (p[1].y + p[2].y);
        b->p[2] = p[2];
    } else {
        pt mid = { 0.125 * p[0].x + 0.375 * p[1].x + 0.375 * p[2].x + 0.125 * p[3].x,
                   0.125 * p[0].y + 0.375 * p[1].y + 0.375 * p[2].y + 0.125 * p[3].y };
        a->p[0] = p[0];
        a->p[1].x = 0.5 * p[0].x + 0.5 * p[1].x; a->p[1].y = 0.5 * p[0].y + 0.5 * p[1].y;
        a->p[2].x = 0.25 * p[0].x + 0.5 * p[1].x + 0.25 * p[2].x;
        a->p[2].y = 0.25 * p[0].y + 0.5 * p[1].y + 0.25 * p[2].y;
        a->p[3] = mid;
        b->p[0] = mid;
        b->p[1].x = 0.25 * p[1].x + 0.5 * p[2].x + 0.25 * p[3].x;
        b->p[1].y = 0.25 * p[1].y + 0.5 * p[2].y + 0.25 * p[3].y;
        b->p[2].x = 0.5 * p[2].x + 0.5 * p[3].x; b->p[2].y = 0.5 * p[2].y + 0.5 * p[3].y;
        b->p[3] = p[3];
    }
}

/* Segment::has_nans curve.rs:1081-1089 */
static int seg_has_nans(const seg* s) {
    int n = seg_npts(s->kind);
    for (int i = 0; i < n; i++)
        if (isnan(s->p[i].x) || isnan(s->p[i].y)) return 1;
    return 0;
}

/* Quad::at curve.rs:432-440, Cubic::at :712-722 */
static pt seg_at(const seg* s, double t) {
    const pt* p = s->p;
    pt r;
    if (s->kind == SEG_LINE) {
        r.x = (1.0 - t) * p[0].x + t * p[1].x;
        r.y = (1.0 - t) * p[0].y + t * p[1].y;
    } else if (s->kind == SEG_QUAD) {
        double t1 = t, t_1 = 1.0 - t;
        double t2 = t1 * t1, t_2 = t_1 * t_1;
        r.x = t_2 * p[0].x + 2.0 * t1 * t_1 * p[1].x + t2 * p[2].x;
        r.y = t_2 * p[0].y + 2.0 * t1 * t_1 * p[1].y + t2 * p[2].y;
    } else {
        double t1 = t, t_1 = 1.0 - t;
        double t2 = t1 * t1, t_2 = t_1 * t_1;
        double t3 = t2 * t1, t_3 = t_2 * t_1;
        r.x = t_3 * p[0].x + 3.0 * t1 * t_2 * p[1].x + 3.0 * t2 * t_1 * p[2].x + t3 * p[3].x;
        r.y = t_3 * p[0].y + 3.0 * t1 * t_2 * p[1].y + 3.0 * t2 * t_1 * p[2].y + t3 * p[3].y;
    }
    return r;
}

/* ------------------------------------------------------------------------ */
/* utils.rs:205-231 quadratic_solve; returns number of roots, in push order  */
/* ------------------------------------------------------------------------ */
static int quadratic_solve(double a, double b, double c, double* r) {
    if (fabs(a) < RZO_EPSILON) {
        if (fabs(b) > RZO_EPSILON) { r[0] = -c / b; return 1; }
        return 0;
    }
    double disc = b * b - 4.0 * a * c;
    if (fabs(disc) < RZO_EPSILON) {
        r[0] = -b / (2.0 * a);
        return 1;
    } else if (disc > 0.0) {
        double sq = sqrt(disc);
        if (b >= 0.0) {
            double mul = -b - sq;
            r[0] = mul / (2.0 * a);
            r[1] = 2.0 * c / mul;
        } else {
            double mul = -b + sq;
            r[0] = 2.0 * c / mul;
            r[1] = mul / (2.0 * a);
        }
        return 2;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* BBox geometry.rs:543-674 and Curve::bbox curve.rs:270-273, :505-513, :810-818 */
/* ------------------------------------------------------------------------ */
typedef struct { pt min, max; } bbox_t;

static bbox_t bbox_new(pt p0, pt p1) {
    bbox_t b;
    if (p0.x <= p1.x) { b.min.x = p0.x; b.max.x = p1.x; } else { b.min.x = p1.x; b.max.x = p0.x; }
    if (p0.y <= p1.y) { b.min.y = p0.y; b.max.y = p1.y; } else { b.min.y = p1.y; b.max.y = p0.y; }
    return b;
}
static bbox_t bbox_extend(bbox_t b, pt p) {
    if (p.x < b.min.x) b.min.x = p.x; else if (p.x > b.max.x) b.max.x = p.x;
    if (p.y < b.min.y) b.min.y = p.y; else if (p.y > b.max.y) b.max.y = p.y;
    return b;
}
static bbox_t bbox_union_opt(bbox_t b, const bbox_t* init) {
    if (!init) return b;
    return bbox_extend(bbox_extend(b, init->min), init->max);
}
static int bbox_contains(bbox_t b, pt p) {
    return b.min.x <= p.x && p.x <= b.max.x && b.min.y <= p.y && p.y <= b.max.y;
}

static bbox_t seg_bbox(const seg* s, const bbox_t* init) {
    const pt* p = s->p;
    if (s->kind == SEG_LINE) return bbox_union_opt(bbox_new(p[0], p[1]), init);
    if (s->kind == SEG_QUAD) {
        bbox_t b = bbox_union_opt(bbox_new(p[0], p[2]), init);
        if (bbox_contains(b, p[1])) return b;
        /* Quad::extremities curve.rs:535-555 */
        double a0 = p[2].x - 2.0 * p[1].x + p[0].x, a1 = p[2].y - 2.0 * p[1].y + p[0].y;
        double b0 = p[1].x - p[0].x, b1 = p[1].y - p[0].y;
        if (fabs(a0) > RZO_EPSILON) {
            double t0 = -b0 / a0;
            if (t0 >= 0.0 && t0 <= 1.0) b = bbox_extend(b, seg_at(s, t0));
        }
        if (fabs(a1) > RZO_EPSILON) {
            double t1 = -b1 / a1;
            if (t1 >= 0.0 && t1 <= 1.0) b = bbox_extend(b, seg_at(s, t1));
        }
        return b;
    }
    bbox_t b = bbox_union_opt(bbox_new(p[0], p[3]), init);
    if (bbox_contains(b, p[1]) && bbox_contains(b, p[2])) return b;
    /* Cubic::extremities curve.rs:853-864 */
    double a0 = -1.0 * p[0].x + 3.0 * p[1].x - 3.0 * p[2].x + 1.0 * p[3].x;
    double a1 = -1.0 * p[0].y + 3.0 * p[1].y - 3.0 * p[2].y + 1.0 * p[3].y;
    double b0 = 2.0 * p[0].x - 4.0 * p[1].x + 2.0 * p[2].x;
    double b1 = 2.0 * p[0].y - 4.0 * p[1].y + 2.0 * p[2].y;
    double c0 = -1.0 * p[0].x + p[1].x;
    double c1 = -1.0 * p[0].y + p[1].y;
    double r[4];
    int n = quadratic_solve(a0, b0, c0, r);
    n += quadratic_solve(a1, b1, c1, r + n);
    for (int i = 0; i < n; i++)
        if (r[i] >= 0.0 && r[i] <= 1.0) b = bbox_extend(b, seg_at(s, r[i]));
    return b;
}

/* ------------------------------------------------------------------------ */
/* ellipse.rs -- EllipArc::new_param :40-96 and EllipArcCubicIter :159-214   */
/* ------------------------------------------------------------------------ */

/* Converts an SVG arc into cubics exactly like PathBuilder::arc_to
 * (path.rs:945-972).  Returns the number of cubics written to out (8 doubles
 * each), -1 when new_param returns None (the builder falls back to line_to),
 * -2 when the cubic count is not finite (the reference iterator never ends). */
int rzo_arc_to_cubics(double sx, double sy, double dx, double dy, double rx, double ry,
                      double x_axis_rot, int large_flag, int sweep_flag, double* out, int cap) {
    pt src = {sx, sy}, dst = {dx, dy};
    rx = fabs(rx);
    ry = fabs(ry);
    double phi = x_axis_rot * RZO_PI / 180.0;
    xform rot_m = tr_rotate(-phi);
    pt half = { 0.5 * (src.x - dst.x), 0.5 * (src.y - dst.y) };
    pt p1 = tr_apply(&rot_m, half);
    double x1 = p1.x, y1 = p1.y;
    double sx1 = x1 / rx, sy1 = y1 / ry;
    double s = sx1 * sx1 + sy1 * sy1;
    if (s > 1.0) {
        double ss = sqrt(s);
        rx = rx * ss;
        ry = ry * ss;
    }
    double rxry = rx * ry, rxy1 = rx * y1, ryx1 = ry * x1;
    double sq = sqrt(rust_fmax(rxry * rxry / (rxy1 * rxy1 + ryx1 * ryx1) - 1.0, 0.0));
    if (large_flag == sweep_flag) sq = -sq;
    pt center = { sq * (rx * y1 / ry), sq * (-ry * x1 / rx) };
    double cx = center.x, cy = center.y;
    xform rot_p = tr_rotate(phi);
    pt cr = tr_apply(&rot_p, center);
    pt c = { cr.x + 0.5 * (dst.x + src.x), cr.y + 0.5 * (dst.y + src.y) };
    pt v0 = {1.0, 0.0};
    pt v1 = { (x1 - cx) / rx, (y1 - cy) / ry };
    pt v2 = { (-x1 - cx) / rx, (-y1 - cy) / ry };
    double eta, eta_delta;
    if (!angle_between(v0, v1, &eta)) return -1;
    if (!angle_between(v1, v2, &eta_delta)) return -1;
    eta_delta = rem_euclid(eta_delta, 2.0 * RZO_PI);
    if (!sweep_flag && eta_delta > 0.0) eta_delta = eta_delta - 2.0 * RZO_PI;
    else if (sweep_flag && eta_delta < 0.0) eta_delta = eta_delta + 2.0 * RZO_PI;

    /* EllipArcCubicIter::new :168-181 */
    double segment_max_angle = RZO_PI / 2.0;
    double segment_count = ceil(fabs(eta_delta) / segment_max_angle);
    if (!isfinite(segment_count)) return -2;
    double segment_delta = eta_delta / segment_count;
    double last_index = segment_count - 1.0;
    int n = 0;
    for (double idx = 0.0; !(idx > last_index); idx += 1.0) {
        if (n >= cap) return -3;
        double eta_1 = eta + segment_delta * idx;
        double eta_2 = eta_1 + segment_delta;
        double tn = tan((eta_2 - eta_1) / 2.0);
        double sqv = sqrt(4.0 + 3.0 * (tn * tn));
        double alpha = sin(eta_2 - eta_1) * (sqv - 1.0) / 3.0;
        /* EllipArcCubicIter::at :183-193 */
        double s1 = sin(eta_1), c1 = cos(eta_1), s2 = sin(eta_2), c2 = cos(eta_2);
        pt a0 = tr_apply(&rot_p, (pt){rx * c1, ry * s1});
        pt p0 = { a0.x + c.x, a0.y + c.y };
        pt d0 = tr_apply(&rot_p, (pt){-rx * s1, ry * c1});
        pt a3 = tr_apply(&rot_p, (pt){rx * c2, ry * s2});
        pt p3 = { a3.x + c.x, a3.y + c.y };
        pt d3 = tr_apply(&rot_p, (pt){-rx * s2, ry * c2});
        pt q1 = { p0.x + alpha * d0.x, p0.y + alpha * d0.y };
        pt q2 = { p3.x - alpha * d3.x, p3.y - alpha * d3.y };
        double* o = out + 8 * n;
        o[0] = p0.x; o[1] = p0.y; o[2] = q1.x; o[3] = q1.y;
        o[4] = q2.x; o[5] = q2.y; o[6] = p3.x; o[7] = p3.y;
        n++;
    }
    return n;
}

/* ------------------------------------------------------------------------ */
/* path.rs -- PathFlattenIter :734-796                                      */
/* ------------------------------------------------------------------------ */

static seg load_seg(const uint8_t* kind, const double* pts, long i) {
    seg s;
    s.kind = kind[i];
    for (int k = 0; k < 4; k++) { s.p[k].x = pts[8 * i + 2 * k]; s.p[k].y = pts[8 * i + 2 * k + 1]; }
    return s;
}

typedef void (*line_sink)(void* ctx, line_t l);

/* Flattens every subpath; close=true (what every rasterizer passes,
 * rasterize.rs:307,330,552,568).  counts (optional) receives the number of
 * lines emitted per segment, followed by one entry per subpath for the closing
 * line.  Returns 0, or -1 where the reference panics on NaN (path.rs:765-767). */
static int flatten_path(const uint8_t* kind, const double* pts, const uint32_t* sub_off, long nsub,
                        const xform* tr, double flatness, line_sink sink, void* ctx, long* counts) {
    double thr = 16.0 * flatness * flatness;
    long cap = 256;
    seg* stack = (seg*)malloc(sizeof(seg) * cap);
    long nseg_total = nsub > 0 ? (long)sub_off[nsub] : 0;
    for (long s = 0; s < nsub; s++) {
        long b = sub_off[s], e = sub_off[s + 1];
        if (e <= b) continue; /* Path::get never yields an empty SubPath */
        for (long i = b; i < e; i++) {
            seg root = load_seg(kind, pts, i);
            long top = 0, emitted = 0;
            stack[top++] = seg_transform(&root, tr);
            while (top > 0) {
                seg cur = stack[--top];
                if (seg_has_nans(&cur)) { free(stack); return -1; }
                if (seg_flatness(&cur) < thr) {
                    line_t l = { seg_start(&cur), seg_end(&cur) };
                    sink(ctx, l);
                    emitted++;
                    continue;
                }
                seg a, bb;
                seg_split(&cur, &a, &bb);
                if (top + 2 > cap) { cap *= 2; stack = (seg*)realloc(stack, sizeof(seg) * cap); }
                stack[top++] = bb;
                stack[top++] = a;
            }
            if (counts) counts[i] = emitted;
        }
        /* closing line: Line::new(subpath.end(), subpath.start()).transform(tr) :776-786 */
        seg first = load_seg(kind, pts, b), last = load_seg(kind, pts, e - 1);
        line_t cl = { tr_apply(tr, seg_end(&last)), tr_apply(tr, seg_start(&first)) };
        sink(ctx, cl);
        if (counts) counts[nseg_total + s] = 1;
    }
    free(stack);
    return 0;
}

typedef struct { double* out; long n, cap; } line_buf;
static void sink_buf(void* ctx, line_t l) {
    line_buf* b = (line_buf*)ctx;
    if (b->n < b->cap && b->out) {
        double* o = b->out + 4 * b->n;
        o[0] = l.a.x; o[1] = l.a.y; o[2] = l.b.x; o[3] = l.b.y;
    }
    b->n++;
}

/* Returns the number of lines (may exceed cap; only cap are written), or -1 on NaN. */
long rzo_flatten(const uint8_t* kind, const double* pts, const uint32_t* sub_off, long nsub,
                 const double* trm, double flatness, double* out, long cap, long* counts) {
    xform tr; memcpy(tr.m, trm, sizeof(tr.m));
    line_buf b = { out, 0, cap };
    if (flatten_path(kind, pts, sub_off, nsub, &tr, flatness, sink_buf, &b, counts) < 0) return -1;
    return b.n;
}

/* ------------------------------------------------------------------------ */
/* rasterize.rs -- SignedDifferenceRasterizer                               */
/* ------------------------------------------------------------------------ */

typedef struct {
    double* data; long data_len;
    long start, width, height, row_stride, col_stride; /* image.rs:6-35 Shape */
} img_t;

static inline long shape_offset(const img_t* im, long row, long col) {
    return im->start + row * im->row_stride + col * im->col_stride;
}

/* split_at_zero_x rasterize.rs:923-937; returns number of lines (1 or 2): out[0]=line, out[1]=rest */
static int split_at_zero_x(line_t l, line_t* out) {
    pt p0 = l.a, p1 = l.b;
    if (p0.x >= 0.0 && p1.x >= 0.0) { out[0] = l; return 1; }
    if (p0.x <= 0.0 && p1.x <= 0.0) {
        out[0].a = (pt){0.0, p0.y}; out[0].b = (pt){0.0, p1.y};
        return 1;
    }
    double t = p0.x / (p0.x - p1.x);
    pt mid = { (1.0 - t) * p0.x + t * p1.x, (1.0 - t) * p0.y + t * p1.y }; /* Line::at */
    if (p0.x < 0.0) {
        out[0].a = mid; out[0].b = p1;
        out[1].a = (pt){0.0, p0.y}; out[1].b = mid;
    } else {
        out[0].a = p0; out[0].b = mid;
        out[1].a = mid; out[1].b = (pt){0.0, p1.y};
    }
    return 2;
}

/* signed_difference_line rasterize.rs:365-470 */
static void signed_difference_line(img_t* im, line_t line) {
    pt p0 = line.a, p1 = line.b;
    double width = (double)im->width - 1.0;
    line_t ln = line;
    if (p0.x > width || p1.x > width) {
        if (p0.x > width && p1.x > width) {
            ln.a = (pt){width - 0.001, p0.y};
            ln.b = (pt){width - 0.001, p1.y};
        } else {
            double t = (p0.x - width) / (p0.x - p1.x);
            pt mid = { width, (1.0 - t) * p0.y + t * p1.y };
            if (p0.x < width) { ln.a = p0; ln.b = mid; }
            else { ln.a = mid; ln.b = p1; }
        }
    }
    line_t parts[2];
    int np = split_at_zero_x(ln, parts);
    if (np == 2) signed_difference_line(im, parts[1]);
    p0 = parts[0].a;
    p1 = parts[0].b;
    double* data = im->data;
    long stride = im->col_stride;
    if (fabs(p0.y - p1.y) < RZO_EPSILON) return;
    double dir;
    if (p0.y < p1.y) { dir = 1.0; }
    else { dir = -1.0; pt t = p0; p0 = p1; p1 = t; }
    double dxdy = (p1.x - p0.x) / (p1.y - p0.y);
    double ystart = rust_fmax(p0.y, 0.0);
    long y = (long)ystart; /* `as usize` of a non-negative value truncates */
    double x = p0.y < 0.0 ? p0.x - p0.y * dxdy : p0.x;
    double x_next = x;
    double yend_f = rust_fmax(ceil(p1.y), 0.0);
    long yend = (long)yend_f;
    if (yend > im->height) yend = im->height;
    for (; y < yend; y++) {
        x = x_next;
        long row_offset = shape_offset(im, y, 0);
        double dy = rust_fmin((double)(y + 1), p1.y) - rust_fmax((double)y, p0.y);
        double d = dir * dy;
        x_next = x + dxdy * dy;
        double x0 = x < x_next ? x : x_next;
        double x1 = x < x_next ? x_next : x;
        double x0_floor = rust_fmax(floor(x0), 0.0);
        int x0i = (int)x0_floor;
        double x1_ceil = rust_fmin(ceil(x1), width);
        int x1i = (int)x1_ceil;
        if (x1i <= x0i + 1) {
            double xmf = 0.5 * (x + x_next) - x0_floor;
            data[row_offset + (long)x0i * stride] += d * (1.0 - xmf);
            long offset = row_offset + (long)(x0i + 1) * stride;
            if (offset < im->data_len) data[offset] += d * xmf;
        } else {
            double s = 1.0 / (x1 - x0);
            double x0f = x0 - x0_floor;
            double x1f = x1 - x1_ceil + 1.0;
            double a0 = 0.5 * s * (1.0 - x0f) * (1.0 - x0f);
            double am = 0.5 * s * x1f * x1f;
            data[row_offset + (long)x0i * stride] += d * a0;
            if (x1i == x0i + 2) {
                data[row_offset + (long)(x0i + 1) * stride] += d * (1.0 - a0 - am);
            } else {
                double a1 = s * (1.5 - x0f);
                data[row_offset + (long)(x0i + 1) * stride] += d * (a1 - a0);
                for (int xi = x0i + 2; xi < x1i - 1; xi++)
                    data[row_offset + (long)xi * stride] += d * s;
                double a2 = a1 + (double)(x1i - x0i - 3) * s;
                data[row_offset + (long)(x1i - 1) * stride] += d * (1.0 - a2 - am);
            }
            data[row_offset + (long)x1i * stride] += d * am;
        }
    }
}

/* signed_difference_to_mask rasterize.rs:473-507 */
static void signed_difference_to_mask(img_t* im, int rule) {
    double* data = im->data;
    for (long y = 0; y < im->height; y++) {
        double acc = 0.0;
        for (long x = 0; x < im->width; x++) {
            long off = shape_offset(im, y, x);
            acc += data[off];
            if (rule == RULE_NONZERO) {
                double v = fabs(acc);
                data[off] = v > 1.0 ? 1.0 : (v < 1e-6 ? 0.0 : v);
            } else {
                data[off] = fabs(rem_euclid(acc + 1.0, 2.0) - 1.0);
            }
        }
    }
}

/* FillRule::alpha_from_winding path.rs:32-46 */
double rzo_alpha_from_winding(int rule, double w) {
    if (rule == RULE_EVENODD) return fabs(rem_euclid(w + 1.0, 2.0) - 1.0);
    double v = fabs(w);
    return v >= 1.0 ? 1.0 : (v < 1e-6 ? 0.0 : v);
}

static void sink_sd(void* ctx, line_t l) { signed_difference_line((img_t*)ctx, l); }

/* Public: signed_difference_line on an image (used by the KAT restating
 * test_signed_difference_line rasterize.rs:945-1003). */
void rzo_signed_difference_line(double* data, long data_len, long start, long width, long height,
                                long row_stride, long col_stride, double x0, double y0, double x1, double y1) {
    img_t im = { data, data_len, start, width, height, row_stride, col_stride };
    line_t l = { {x0, y0}, {x1, y1} };
    signed_difference_line(&im, l);
}

/* SignedDifferenceRasterizer::mask rasterize.rs:299-311 (image assumed zeroed, path.rs:509-512) */
int rzo_mask(const uint8_t* kind, const double* pts, const uint32_t* sub_off, long nsub,
             const double* trm, int rule, double flatness,
             double* data, long data_len, long start, long width, long height, long row_stride, long col_stride) {
    xform tr; memcpy(tr.m, trm, sizeof(tr.m));
    img_t im = { data, data_len, start, width, height, row_stride, col_stride };
    if (flatten_path(kind, pts, sub_off, nsub, &tr, flatness, sink_sd, &im, NULL) < 0) return -1;
    signed_difference_to_mask(&im, rule);
    return 0;
}

/* SignedDifferenceRasterizer::mask_iter rasterize.rs:313-355, materialised: out
 * (height x width, row-major, zero-initialised by the caller) receives alpha at
 * every pixel the iterator yields.  Returns the number of yielded pixels. */
long rzo_mask_iter(const uint8_t* kind, const double* pts, const uint32_t* sub_off, long nsub,
                   const double* trm, int rule, double flatness, long width, long height, double* out) {
    if (width == 0 || height == 0) return 0;
    xform tr; memcpy(tr.m, trm, sizeof(tr.m));
    long w1 = width + 1;
    double* buf = (double*)calloc((size_t)(w1 * height), sizeof(double));
    img_t im = { buf, w1 * height, 0, w1, height, w1, 1 };
    if (flatten_path(kind, pts, sub_off, nsub, &tr, flatness, sink_sd, &im, NULL) < 0) { free(buf); return -1; }
    long n = 0;
    double winding = 0.0;
    for (long index = 0; index < w1 * height; index++) {
        long y = index / w1, x = index - y * w1;
        if (x == 0) winding = 0.0;
        else if (x >= width) continue;
        winding += buf[index];
        double alpha = rzo_alpha_from_winding(rule, winding);
        if (fabs(alpha) < 1e-6) continue;
        out[y * width + x] = alpha;
        n++;
    }
    free(buf);
    return n;
}

/* ------------------------------------------------------------------------ */
/* rasterize.rs -- ActiveEdgeRasterizer :517-920 (independent cross-check)  */
/* ------------------------------------------------------------------------ */

typedef struct { line_t line; double dxdy; double dydx; int has_dydx; double dir; long row; } edge_t;
typedef struct { line_t line; int has_line; double reminder; int has_rem; double dydx; int has_dydx; long column; double dir; } rowit_t;

static double next_ceil(double v) { return floor(v) + 1.0; }

/* Edge::new :765-798 */
static int edge_new(line_t l, edge_t* e) {
    pt p0 = l.a, p1 = l.b;
    if (fabs(p0.y - p1.y) < RZO_EPSILON) return 0;
    double dir;
    if (p0.y <= p1.y) dir = 1.0; else { dir = -1.0; pt t = p0; p0 = p1; p1 = t; }
    double dx = p1.x - p0.x, dy = p1.y - p0.y;
    double dxdy = dx / dy;
    e->has_dydx = fabs(dxdy) > RZO_EPSILON_SQRT;
    e->dydx = e->has_dydx ? dy / dx : 0.0;
    if (p0.y < 0.0) p0 = (pt){ p0.x - p0.y * dxdy, 0.0 };
    e->line.a = p0; e->line.b = p1;
    e->dxdy = dxdy; e->dir = dir;
    double fr = floor(p0.y);
    e->row = fr < 0 ? 0 : (long)fr;
    return 1;
}

/* EdgeRowIter::new :836-869 */
static int rowit_new(edge_t* e, rowit_t* it) {
    pt p0 = e->line.a, p1 = e->line.b;
    if (p1.y - p0.y < RZO_EPSILON) return 0;
    double y_split = rust_fmin(next_ceil(p0.y), p1.y);
    double x_split = p0.x + e->dxdy * (y_split - p0.y);
    pt ps = { x_split, y_split };
    e->line.a = ps; e->line.b = p1;
    double dir; line_t ln;
    if (p0.x <= ps.x) { dir = e->dir; ln.a = p0; ln.b = ps; }
    else { dir = -e->dir; ln.a = ps; ln.b = p0; }
    it->line = ln; it->has_line = 1; it->has_rem = 0; it->reminder = 0;
    it->dydx = e->dydx; it->has_dydx = e->has_dydx;
    double sx = ln.a.x;
    it->column = sx < 0 ? 0 : (long)sx;
    it->dir = dir;
    return 1;
}

/* EdgeRowIter::next :872-893; returns 0 when exhausted */
static int rowit_next(rowit_t* it, double* out) {
    if (it->has_line) {
        pt p0 = it->line.a, p1 = it->line.b;
        it->has_line = 0;
        double x_ceil = next_ceil(p0.x);
        double x = rust_fmin(x_ceil, p1.x);
        double h = it->has_dydx ? it->dydx * (x - p0.x) : rust_fmin(next_ceil(p0.y), p1.y) - p0.y;
        double y = p0.y + h;
        double s0 = (2.0 * x_ceil - x - p0.x) * h / 2.0;
        double s1 = h - s0;
        if (p1.x > x) { it->line.a = (pt){x, y}; it->line.b = p1; it->has_line = 1; }
        double s_prev = it->has_rem ? it->reminder : 0.0;
        it->reminder = it->dir * s1; it->has_rem = 1;
        *out = it->dir * s0 + s_prev;
        return 1;
    }
    if (it->has_rem) { it->has_rem = 0; *out = it->reminder; return 1; }
    return 0;
}

typedef struct { edge_t* e; long n, cap; } edge_vec;
static void sink_edges(void* ctx, line_t l) {
    edge_vec* v = (edge_vec*)ctx;
    line_t parts[2];
    int np = split_at_zero_x(l, parts);
    for (int k = 0; k < np; k++) {
        edge_t e;
        if (!edge_new(parts[k], &e)) continue;
        if (v->n == v->cap) { v->cap = v->cap ? v->cap * 2 : 256; v->e = (edge_t*)realloc(v->e, sizeof(edge_t) * v->cap); }
        v->e[v->n++] = e;
    }
}

static int cmp_edge_row_desc(const void* a, const void* b) {
    long ra = ((const edge_t*)a)->row, rb = ((const edge_t*)b)->row;
    return ra < rb ? 1 : (ra > rb ? -1 : 0);
}
static int cmp_rowit_col_desc(const void* a, const void* b) {
    long ca = ((const rowit_t*)a)->column, cb = ((const rowit_t*)b)->column;
    return ca < cb ? 1 : (ca > cb ? -1 : 0);
}

/* ActiveEdgeRasterizer::mask :537-556 via ActiveEdgeIter :578-732.  The
 * result does not depend on the unstable sort order up to fp rounding. */
int rzo_mask_ae(const uint8_t* kind, const double* pts, const uint32_t* sub_off, long nsub,
                const double* trm, int rule, double flatness,
                double* data, long width, long height) {
    xform tr; memcpy(tr.m, trm, sizeof(tr.m));
    edge_vec ev = {0, 0, 0};
    if (flatten_path(kind, pts, sub_off, nsub, &tr, flatness, sink_edges, &ev, NULL) < 0) { free(ev.e); return -1; }
    /* filter edge.row < height */
    long m = 0;
    for (long i = 0; i < ev.n; i++) if (ev.e[i].row < height) ev.e[m++] = ev.e[i];
    ev.n = m;
    qsort(ev.e, ev.n, sizeof(edge_t), cmp_edge_row_desc);
    edge_t* active = (edge_t*)malloc(sizeof(edge_t) * (ev.n + 1));
    long nactive = 0;
    rowit_t* inact = (rowit_t*)malloc(sizeof(rowit_t) * (ev.n + 1));
    long ninact = 0;
    rowit_t* acts = (rowit_t*)malloc(sizeof(rowit_t) * (ev.n + 1));
    long nacts = 0;
    long nedges = ev.n; /* edge_inactive = ev.e[0..nedges), sorted by row desc */
    long row = 0, column = 0;
    double winding = 0.0;
#define NEXT_ROW() do { \
        ninact = 0; nacts = 0; \
        long w_ = 0; \
        for (long i_ = 0; i_ < nactive; i_++) { \
            rowit_t it_; \
            if (rowit_new(&active[i_], &it_)) { inact[ninact++] = it_; active[w_++] = active[i_]; } \
        } \
        nactive = w_; \
        long pp_ = nedges; \
        while (pp_ > 0 && !(ev.e[pp_ - 1].row > row)) pp_--; \
        for (long i_ = pp_; i_ < nedges; i_++) { \
            edge_t e_ = ev.e[i_]; rowit_t it_; \
            if (rowit_new(&e_, &it_)) { inact[ninact++] = it_; active[nactive++] = e_; } \
        } \
        nedges = pp_; \
        qsort(inact, ninact, sizeof(rowit_t), cmp_rowit_col_desc); \
    } while (0)
    NEXT_ROW();
    for (;;) {
        if (row >= height) break;
        while (ninact > 0) {
            rowit_t it = inact[ninact - 1];
            if (it.column <= column) { acts[nacts++] = it; ninact--; }
            else break;
        }
        /* EdgeAccIter::next :908-920 */
        int have = 0; double acc = 0.0;
        if (nacts > 0) {
            have = 1;
            long w = 0;
            for (long i = 0; i < nacts; i++) {
                double v;
                if (rowit_next(&acts[i], &v)) { acc += v; acts[w++] = acts[i]; }
            }
            nacts = w;
        }
        if (have) winding += acc;
        else if (fabs(winding) < RZO_EPSILON_SQRT) {
            if (ninact > 0 && inact[ninact - 1].column < width) {
                column = inact[ninact - 1].column;
            } else {
                column = 0; row += 1; winding = 0.0; NEXT_ROW();
            }
            continue;
        }
        data[row * width + column] = rzo_alpha_from_winding(rule, winding);
        column += 1;
        if (column >= width) { column = 0; row += 1; winding = 0.0; NEXT_ROW(); }
    }
#undef NEXT_ROW
    free(active); free(inact); free(acts); free(ev.e);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* path.rs:374-415, 692-732 Path::stroke; curve.rs:977-1076 line_join /     */
/* line_cap; curve.rs:1290-1433 offsets (Tiller-Hanson)                     */
/* ------------------------------------------------------------------------ */
typedef struct { seg* v; long n, cap; } segvec;
static void sv_push(segvec* s, seg x) {
    if (s->n == s->cap) { s->cap = s->cap ? 2 * s->cap : 16; s->v = (seg*)realloc(s->v, (size_t)s->cap * sizeof(seg)); }
    s->v[s->n++] = x;
}
/* inserts b (all of it) at position at of a */
static void sv_insert(segvec* a, long at, const segvec* b) {
    for (long i = 0; i < b->n; i++) sv_push(a, b->v[0]);
    memmove(a->v + at + b->n, a->v + at, (size_t)(a->n - b->n - at) * sizeof(seg));
    memcpy(a->v + at, b->v, (size_t)b->n * sizeof(seg));
}
static pt p_sub(pt a, pt b) { pt r = { a.x - b.x, a.y - b.y }; return r; }
static pt p_add(pt a, pt b) { pt r = { a.x + b.x, a.y + b.y }; return r; }
static pt p_scale(double s, pt a) { pt r = { s * a.x, s * a.y }; return r; }
static double p_dot(pt a, pt b) { return a.x * b.x + a.y * b.y; }           /* geometry.rs:155-159 */
static double p_cross(pt a, pt b) { return a.x * b.y - a.y * b.x; }         /* geometry.rs:162-166 */
static double p_length(pt a) { return hypot(a.x, a.y); }                     /* geometry.rs:144-147 */
static int p_close(pt a, pt b) { return fabs(a.x - b.x) < RZO_EPSILON && fabs(a.y - b.y) < RZO_EPSILON; }
static int p_normalize(pt a, pt* out) {                                      /* geometry.rs:175-183 */
    double l = p_length(a);
    if (l < RZO_EPSILON) return 0;
    out->x = a.x / l; out->y = a.y / l;
    return 1;
}
static seg mk_line(pt a, pt b) { seg s; memset(&s, 0, sizeof(s)); s.kind = SEG_LINE; s.p[0] = a; s.p[1] = b; return s; }
static pt l_at(line_t l, double t) { pt r = { (1.0 - t) * l.a.x + t * l.b.x, (1.0 - t) * l.a.y + t * l.b.y }; return r; }
/* Line::intersect curve.rs:204-215 */
static int l_intersect(line_t s, line_t o, double* t0, double* t1) {
    double x1 = s.a.x, y1 = s.a.y, x2 = s.b.x, y2 = s.b.y, x3 = o.a.x, y3 = o.a.y, x4 = o.b.x, y4 = o.b.y;
    double det = (x4 - x3) * (y1 - y2) - (x1 - x2) * (y4 - y3);
    if (fabs(det) < RZO_EPSILON) return 0;
    *t0 = ((y3 - y4) * (x1 - x3) + (x4 - x3) * (y1 - y3)) / det;
    *t1 = ((y1 - y2) * (x1 - x3) + (x2 - x1) * (y1 - y3)) / det;
    return 1;
}
static int unit01(double t) { return t >= 0.0 && t <= 1.0; }
/* Segment::ends curve.rs:195-197 (line), 377-388 (quad), 647-666 (cubic) */
static void s_ends(const seg* s, line_t* start, line_t* end) {
    const pt* p = s->p;
    if (s->kind == SEG_LINE) { start->a = end->a = p[0]; start->b = end->b = p[1]; return; }
    if (s->kind == SEG_QUAD) {
        line_t a = { p[0], p[1] }, b = { p[1], p[2] };
        if (p_close(p[0], p[1])) { *start = b; *end = b; }
        else if (p_close(p[1], p[2])) { *start = a; *end = a; }
        else { *start = a; *end = b; }
        return;
    }
    int st = 0, en = 0;
    for (int i = 0; i < 3; i++) if (!p_close(p[i], p[i + 1])) { st = i; break; }
    for (int i = 3; i >= 1; i--) if (!p_close(p[i], p[i - 1])) { en = i; break; }
    if (en == 0) en = 1;
    start->a = p[st]; start->b = p[st + 1];
    end->a = p[en - 1]; end->b = p[en];
}
/* line_offset curve.rs:1290-1295 */
static int l_offset(line_t l, double dist, line_t* out) {
    pt d = p_sub(l.b, l.a), nrm = { d.y, -d.x }, u;
    if (!p_normalize(nrm, &u)) return 0;
    pt off = p_scale(dist, u);
    out->a = p_add(l.a, off); out->b = p_add(l.b, off);
    return 1;
}
/* polyline_offset curve.rs:1302-1352 */
static int polyline_offset(pt* ps, int n, double dist) {
    if (n == 0) return 1;
    int have = 0, index = 0;
    line_t prev = { {0, 0}, {0, 0} };
    for (;;) {
        int repeats = 1;
        for (int i = index; i < n - 1; i++) { if (!p_close(ps[i], ps[i + 1])) break; repeats++; }
        if (index + repeats >= n) break;
        index += repeats;
        line_t src = { ps[index - 1], ps[index] }, next;
        l_offset(src, dist, &next);
        pt point = next.a;
        double t0, t1;
        if (have && l_intersect(prev, next, &t0, &t1)) point = l_at(prev, t0);
        for (int i = index - repeats; i < index; i++) ps[i] = point;
        prev = next;
        have = 1;
    }
    if (!have) return 0;
    for (int i = index; i < n; i++) ps[i] = prev.b;
    return 1;
}
static double diag_length(const seg* s) {  /* bbox(None).diag().length() */
    bbox_t b = seg_bbox(s, NULL);
    return p_length(p_sub(b.min, b.max));
}
/* quad_offset_should_split curve.rs:1355-1368 */
static int quad_split_needed(const seg* q) {
    pt p0 = q->p[0], p1 = q->p[1], p2 = q->p[2];
    if (p_dot(p_sub(p0, p1), p_sub(p2, p1)) > 0.0) return 1;
    pt mass = { (p0.x + p1.x + p2.x) / 3.0, (p0.y + p1.y + p2.y) / 3.0 };
    double dist = p_length(p_sub(mass, seg_at(q, 0.5)));
    return diag_length(q) * 0.1 < dist;
}
/* cubic_offset_should_split curve.rs:1412-1431 */
static int cubic_split_needed(const seg* c) {
    pt p0 = c->p[0], p1 = c->p[1], p2 = c->p[2], p3 = c->p[3];
    if (p_dot(p_sub(p3, p0), p_sub(p2, p1)) < 0.0) return 1;
    double a0 = p_cross(p_sub(p3, p0), p_sub(p1, p0)), a1 = p_cross(p_sub(p3, p0), p_sub(p2, p0));
    if (a0 * a1 < 0.0) return 1;
    pt mass = { (p0.x + p1.x + p2.x + p3.x) / 4.0, (p0.y + p1.y + p2.y + p3.y) / 4.0 };
    double dist = p_length(p_sub(mass, seg_at(c, 0.5)));
    return diag_length(c) * 0.1 < dist;
}
typedef struct { double width, miter; int join, cap; } stroke_t;
enum { J_MITER = 0, J_BEVEL = 1, J_ROUND = 2 };
enum { C_BUTT = 0, C_SQUARE = 1, C_ROUND = 2 };
/* Segment::line_join curve.rs:977-1047 */
static void line_join(const seg* self, const seg* other, const stroke_t* st, segvec* out) {
    pt e = seg_end(self), s = seg_start(other);
    if (p_close(e, s)) return;
    seg bevel = mk_line(e, s);
    line_t t0l, start, end, t1l;
    s_ends(self, &t0l, &start);
    s_ends(other, &end, &t1l);
    double t0, t1;
    if (st->join == J_BEVEL) { sv_push(out, bevel); return; }
    if (st->join == J_MITER) {
        if (!l_intersect(start, end, &t0, &t1) || (unit01(t0) && unit01(t1))) { sv_push(out, bevel); return; }
        pt p0 = p_sub(start.b, start.a), p1 = p_sub(end.a, end.b);
        double lengths = p_length(p0) * p_length(p1);             /* cos_between geometry.rs:196-203 */
        if (lengths < RZO_EPSILON) { sv_push(out, bevel); return; }
        double c = p_dot(p0, p1) / lengths;
        double miter_length = st->width / sqrt((1.0 - c) / 2.0);
        if (miter_length < st->miter) {
            pt p = l_at(start, t0);
            sv_push(out, mk_line(start.b, p));
            sv_push(out, mk_line(p, end.a));
        } else {
            sv_push(out, bevel);
        }
        return;
    }
    if (l_intersect(start, end, &t0, &t1) && unit01(t0) && unit01(t1)) { sv_push(out, bevel); return; }
    int sweep = p_cross(p_sub(start.b, start.a), p_sub(s, e)) >= 0.0;
    double r = st->width / 2.0, cub[64];
    int n = rzo_arc_to_cubics(start.b.x, start.b.y, end.a.x, end.a.y, r, r, 0.0, 0, sweep, cub, 8);
    if (n < 0) { sv_push(out, bevel); return; }
    for (int i = 0; i < n; i++) {
        seg c; c.kind = SEG_CUBIC;
        for (int j = 0; j < 4; j++) { c.p[j].x = cub[8 * i + 2 * j]; c.p[j].y = cub[8 * i + 2 * j + 1]; }
        sv_push(out, c);
    }
}
/* Segment::line_cap curve.rs:1050-1076 */
static void line_cap(const seg* self, const seg* other, const stroke_t* st, segvec* out) {
    pt e = seg_end(self), s = seg_start(other);
    if (p_close(e, s)) return;
    if (st->cap == C_BUTT) { sv_push(out, mk_line(e, s)); return; }
    if (st->cap == C_SQUARE) {
        line_t t0l, from;
        s_ends(self, &t0l, &from);
        pt tang;
        if (p_normalize(p_sub(from.b, from.a), &tang)) {
            seg l0 = mk_line(e, p_add(e, p_scale(st->width / 2.0, tang)));
            seg l1 = mk_line(l0.p[1], p_add(l0.p[1], p_sub(s, e)));
            sv_push(out, l0);
            sv_push(out, l1);
            sv_push(out, mk_line(l1.p[1], s));
        }
        return;
    }
    stroke_t r = *st;
    r.join = J_ROUND;
    line_join(self, other, &r, out);
}
/* quad_offset_rec curve.rs:1371-1383 (split_at(0.5)) */
static void quad_offset_rec(seg q, double dist, segvec* out, int depth) {
    if (quad_split_needed(&q) && depth < 3) {
        const pt* p = q.p;
        double t = 0.5, t1 = t, t_1 = 1.0 - t, t2 = t1 * t1, t_2 = t_1 * t_1;
        pt mid = { t_2 * p[0].x + 2.0 * t1 * t_1 * p[1].x + t2 * p[2].x,
                   t_2 * p[0].y + 2.0 * t1 * t_1 * p[1].y + t2 * p[2].y };
        seg a = q, b = q;
        a.p[1].x = t_1 * p[0].x + t * p[1].x; a.p[1].y = t_1 * p[0].y + t * p[1].y; a.p[2] = mid;
        b.p[0] = mid; b.p[1].x = t_1 * p[1].x + t * p[2].x; b.p[1].y = t_1 * p[1].y + t * p[2].y;
        quad_offset_rec(a, dist, out, depth + 1);
        quad_offset_rec(b, dist, out, depth + 1);
        return;
    }
    if (polyline_offset(q.p, 3, dist)) sv_push(out, q);
}
/* cubic_offset_rec curve.rs:1386-1409 (Cubic::split) */
static int cubic_offset_rec(seg c, int have_last, seg last, double dist, segvec* out, int depth, seg* res) {
    if (cubic_split_needed(&c) && depth < 3) {
        seg a, b, l;
        seg_split(&c, &a, &b);
        int h = cubic_offset_rec(a, have_last, last, dist, out, depth + 1, &l);
        return cubic_offset_rec(b, h, l, dist, out, depth + 1, res);
    }
    seg r = c;
    if (polyline_offset(r.p, 4, dist)) {
        if (have_last && !p_close(seg_end(&last), seg_start(&r))) {
            stroke_t st = { dist * 2.0, 0.0, J_ROUND, C_ROUND };
            line_join(&last, &r, &st, out);
        }
        sv_push(out, r);
        *res = r;
        return 1;
    }
    *res = last;
    return have_last;
}
static void seg_offset(const seg* s, double dist, segvec* out) {
    if (s->kind == SEG_LINE) {
        line_t l = { s->p[0], s->p[1] }, o;
        if (l_offset(l, dist, &o)) sv_push(out, mk_line(o.a, o.b));
    } else if (s->kind == SEG_QUAD) {
        quad_offset_rec(*s, dist, out, 0);
    } else {
        seg last, res;
        memset(&last, 0, sizeof(last));
        cubic_offset_rec(*s, 0, last, dist, out, 0, &res);
    }
}
/* stroke_segment path.rs:692-705 */
static void stroke_segment(segvec* segs, const seg* s, const stroke_t* st, int cap) {
    long offset = segs->n;
    seg_offset(s, st->width / 2.0, segs);
    if (offset != 0 && segs->n > offset) {
        segvec j = { NULL, 0, 0 };
        seg src = segs->v[offset - 1], dst = segs->v[offset];
        if (cap) line_cap(&src, &dst, st, &j); else line_join(&src, &dst, st, &j);
        if (j.n) sv_insert(segs, offset, &j);
        free(j.v);
    }
}
/* stroke_close path.rs:708-732 */
static void stroke_close(pt sp_start, pt sp_end, segvec* segs, const stroke_t* st, int forward) {
    if (segs->n == 0) return;
    seg first = segs->v[0], last = segs->v[segs->n - 1];
    line_t close = forward ? (line_t){ sp_end, sp_start } : (line_t){ sp_start, sp_end }, off;
    if (l_offset(close, st->width / 2.0, &off) && p_length(p_sub(off.a, off.b)) * 100.0 > st->width) {
        seg c = mk_line(off.a, off.b);
        line_join(&last, &c, st, segs);
        sv_push(segs, c);
        line_join(&c, &first, st, segs);
    } else {
        line_join(&last, &first, st, segs);
    }
}
static seg reversed(const seg* s) {
    seg r = *s;
    int n = seg_npts(s->kind);
    for (int i = 0; i < n; i++) r.p[i] = s->p[n - 1 - i];
    return r;
}
/* Path::stroke path.rs:374-415 of an arc-free path.  Writes up to seg_cap
 * segments (kind, 8 doubles) and the subpath offsets (n_sub + 1); returns
 * the segment count (and *n_sub), or -1 when a cap is too small. */
long rzo_stroke(const uint8_t* kind, const double* pts, const uint32_t* sub_off, long nsub, const uint8_t* closed,
                double width, int join, double miter, int cap, uint8_t* okind, double* opts, long seg_cap,
                uint32_t* osub, long sub_cap, long* n_sub) {
    stroke_t st = { width, miter, join, cap };
    segvec segs = { NULL, 0, 0 }, fwd = { NULL, 0, 0 };
    long nseg = 0, ns = 0;
    if (sub_cap < 1) return -1;
    osub[0] = 0;
    for (long sp = 0; sp < nsub; sp++) {
        fwd.n = 0;
        for (uint32_t i = sub_off[sp]; i < sub_off[sp + 1]; i++) sv_push(&fwd, load_seg(kind, pts, i));
        if (fwd.n == 0) continue;
        int is_closed = closed && closed[sp];
        pt sp_start = seg_start(&fwd.v[0]), sp_end = seg_end(&fwd.v[fwd.n - 1]);
        for (long i = 0; i < fwd.n; i++) stroke_segment(&segs, &fwd.v[i], &st, 0);
        long back = fwd.n;
        for (int pass = 0; pass < 2; pass++) {
            if (pass == 1) {
                while (back > 0) { back--; seg r = reversed(&fwd.v[back]); stroke_segment(&segs, &r, &st, 0); }
            }
            if (is_closed) {
                stroke_close(sp_start, sp_end, &segs, &st, pass == 0);
            } else if (pass == 0) {
                back--;
                seg r = reversed(&fwd.v[back]);
                stroke_segment(&segs, &r, &st, 1);
                continue;
            } else if (segs.n) {
                seg last = segs.v[segs.n - 1], first = segs.v[0];
                line_cap(&last, &first, &st, &segs);
            }
            if (segs.n) {  /* Path::push(&segments, true) */
                if (nseg + segs.n > seg_cap || ns + 2 > sub_cap) { free(segs.v); free(fwd.v); return -1; }
                for (long i = 0; i < segs.n; i++) {
                    okind[nseg] = (uint8_t)segs.v[i].kind;
                    double* o = opts + 8 * nseg;
                    memset(o, 0, 8 * sizeof(double));
                    for (int j = 0; j < seg_npts(segs.v[i].kind); j++) { o[2 * j] = segs.v[i].p[j].x; o[2 * j + 1] = segs.v[i].p[j].y; }
                    nseg++;
                }
                osub[++ns] = (uint32_t)nseg;
                segs.n = 0;
            }
        }
    }
    free(segs.v);
    free(fwd.v);
    *n_sub = ns;
    return nseg;
}

/* ------------------------------------------------------------------------ */
/* color.rs / simd -- premultiplied linear colors                           */
/* ------------------------------------------------------------------------ */

typedef struct { float v[4]; } col4;

/* simd/x86.rs:197-214 l2s (polynomial fit, applied to all four lanes) */
static col4 l2s_x86(col4 x0) {
    col4 r;
    for (int i = 0; i < 4; i++) {
        float a = x0.v[i];
        float x1 = sqrtf(a), x2 = sqrtf(x1), x3 = sqrtf(x2);
        float high = (-0.01848558f * a) + (0.6445592f * x1) + (0.70994765f * x2) - (0.33605254f * x3);
        r.v[i] = a <= 0.0031308f ? a * 12.92f : high;
    }
    return r;
}
/* simd/x86.rs:217-244 s2l */
static col4 s2l_x86(col4 vs) {
    col4 r;
    for (int i = 0; i < 4; i++) {
        float v = vs.v[i];
        float x1 = 2.0843103538116825f * v - 1.0843103538116827f;
        float x2 = x1 * x1;
        float x3 = x2 * x1;
        float high = 0.23361048543711943f + 0.4665843122387033f * x1 + 0.26901741378006355f * x2 +
                     0.031661580753065945f * x3;
        r.v[i] = v <= 0.04045f ? v * 0.07739938080495357f : high;
    }
    return r;
}
/* Scalar conversions color.rs:465-486 (linear_to_srgb uses the same fit as l2s) */
float rzo_linear_to_srgb(float x0) {
    if (x0 <= 0.0031308f) return x0 * 12.92f;
    float x1 = sqrtf(x0), x2 = sqrtf(x1), x3 = sqrtf(x2);
    return -0.01848558f * x0 + 0.6445592f * x1 + 0.70994765f * x2 - 0.33605254f * x3;
}
float rzo_srgb_to_linear(float v) {
    if (v <= 0.04045f) return v / 12.92f;
    return powf((v + 0.055f) / 1.055f, 2.4f);
}
/* LinColor::unmultiply color.rs:300-309 */
static col4 unmultiply(col4 c) {
    float a = c.v[3];
    col4 r = {{0, 0, 0, 0}};
    if (a <= 1e-6f) return r;
    for (int i = 0; i < 4; i++) r.v[i] = c.v[i] / a;
    return r;
}
/* into_srgb / into_linear color.rs:314-333 */
static col4 into_srgb(col4 c) {
    col4 u = l2s_x86(unmultiply(c));
    for (int i = 0; i < 4; i++) u.v[i] = u.v[i] * c.v[3];
    return u;
}
static col4 into_linear(col4 c) {
    col4 u = s2l_x86(unmultiply(c));
    for (int i = 0; i < 4; i++) u.v[i] = u.v[i] * c.v[3];
    return u;
}
void rzo_into_srgb(const float* in, float* out) { col4 c; memcpy(c.v, in, 16); c = into_srgb(c); memcpy(out, c.v, 16); }
void rzo_into_linear(const float* in, float* out) { col4 c; memcpy(c.v, in, 16); c = into_linear(c); memcpy(out, c.v, 16); }
void rzo_l2s(const float* in, float* out) { col4 c; memcpy(c.v, in, 16); c = l2s_x86(c); memcpy(out, c.v, 16); }
void rzo_s2l(const float* in, float* out) { col4 c; memcpy(c.v, in, 16); c = s2l_x86(c); memcpy(out, c.v, 16); }

/* Rust `(v * 255.0 + 0.5) as u8`: saturating, truncating, NaN -> 0 (color.rs:169-172) */
static uint8_t u8_sat(float v) {
    float t = v * 255.0f;
    float s = t + 0.5f;
    if (!(s > 0.0f)) return 0;
    if (s >= 255.0f) return 255;
    return (uint8_t)s;
}
/* From<LinColor> for RGBA color.rs:164-175: l2s of the unmultiplied colour, alpha as is */
void rzo_encode_rgba8(const float* canvas, long n, uint8_t* out) {
    for (long i = 0; i < n; i++) {
        col4 c;
        memcpy(c.v, canvas + 4 * i, 16);
        col4 u = l2s_x86(unmultiply(c));
        out[4 * i + 0] = u8_sat(u.v[0]);
        out[4 * i + 1] = u8_sat(u.v[1]);
        out[4 * i + 2] = u8_sat(u.v[2]);
        out[4 * i + 3] = u8_sat(c.v[3]);
    }
}
/* Scalar::to_rgba color.rs:429-432 (f64 mask, cast to f32 first) */
void rzo_encode_mask_rgba8(const double* mask, long n, uint8_t* out) {
    for (long i = 0; i < n; i++) {
        uint8_t v = u8_sat(rzo_linear_to_srgb(1.0f - (float)mask[i]));
        out[4 * i + 0] = out[4 * i + 1] = out[4 * i + 2] = v;
        out[4 * i + 3] = 255;
    }
}
/* The l2s byte thresholds: T[k] = the smallest f32 u in [0, 1] whose byte
   u8_sat(linear_to_srgb(u)) is >= k (k = 1..255; T[0] = 0), by a scan of
   every f32 in [0, 1].  Returns 1 when the byte never decreases on [0, 1]
   (then byte(u) = k exactly when T[k] <= u < T[k + 1]). */
int rzo_l2s_byte_thresholds(float* T) {
    int prev = 0, mono = 1;
    T[0] = 0.0f;
    for (int k = 1; k < 256; k++) T[k] = INFINITY;
    for (uint32_t b = 0; b <= 0x3F800000u; b++) {
        float u;
        memcpy(&u, &b, 4);
        int v = u8_sat(rzo_linear_to_srgb(u));
        if (v < prev) mono = 0;
        for (int k = prev + 1; k <= v; k++) T[k] = u;
        if (v > prev) prev = v;
    }
    return mono;
}
/* From<RGBA> for LinColor color.rs:394-406 */
void rzo_lin_from_rgba8(const uint8_t* rgba, float* out) {
    float a = (float)rgba[3] / 255.0f;
    out[0] = rzo_srgb_to_linear((float)rgba[0] / 255.0f) * a;
    out[1] = rzo_srgb_to_linear((float)rgba[1] / 255.0f) * a;
    out[2] = rzo_srgb_to_linear((float)rgba[2] / 255.0f) * a;
    out[3] = a;
}

/* ------------------------------------------------------------------------ */
/* grad.rs -- spread, stops, linear and radial gradients                    */
/* ------------------------------------------------------------------------ */

enum { PAINT_SOLID = 0, PAINT_LINEAR = 1, PAINT_RADIAL = 2 };
enum { UNITS_USER = 0, UNITS_BBOX = 1 };
enum { SPREAD_PAD = 0, SPREAD_REPEAT = 1, SPREAD_REFLECT = 2 };

#define RZO_MAX_STOPS 32
/* Flat paint record shared with the Python side (oracle.py mirrors it). */
typedef struct {
    int32_t kind, units, spread, linear_colors;
    double tr[6];
    double p0[2], p1[2]; /* linear: start, end; radial: center, fcenter */
    double r0, r1;       /* radial: radius, fradius */
    int32_t nstops, pad;
    double stop_pos[RZO_MAX_STOPS];
    float stop_col[RZO_MAX_STOPS][4];
    float solid[4];
} rzo_paint;

/* GradSpread::at grad.rs:24-30 */
static double spread_at(int spread, double t) {
    if (spread == SPREAD_REPEAT) return rem_euclid(t, 1.0);
    if (spread == SPREAD_REFLECT) return fabs(rem_euclid(t + 1.0, 2.0) - 1.0);
    return t;
}

/* A paint prepared like GradLinear::new / GradRadial::new (stops sorted by
 * GradStops::new grad.rs:86-99, converted to sRGB when !linear_colors). */
typedef struct {
    rzo_paint p;
    int nstops;
    double pos[RZO_MAX_STOPS];
    col4 col[RZO_MAX_STOPS];
    pt dir; /* linear: (end - start) / |end - start|^2 */
} prepared_paint;

static void prepare_paint(const rzo_paint* in, prepared_paint* out) {
    memset(out, 0, sizeof(*out));
    out->p = *in;
    int n = in->nstops;
    if (n > RZO_MAX_STOPS) n = RZO_MAX_STOPS;
    /* stable insertion sort with partial_cmp(...).unwrap_or(Greater) */
    int idx[RZO_MAX_STOPS];
    for (int i = 0; i < n; i++) idx[i] = i;
    for (int i = 1; i < n; i++) {
        int k = idx[i], j = i - 1;
        /* element k moves before idx[j] while cmp(k, idx[j]) == Less */
        while (j >= 0) {
            double a = in->stop_pos[k], b = in->stop_pos[idx[j]];
            int less = (a < b); /* NaN compares Greater -> never Less */
            if (!less) break;
            idx[j + 1] = idx[j];
            j--;
        }
        idx[j + 1] = k;
    }
    if (n == 0) {
        out->nstops = 1;
        out->pos[0] = 0.0;
        col4 black = {{0, 0, 0, 1}};
        out->col[0] = black;
    } else {
        out->nstops = n;
        for (int i = 0; i < n; i++) {
            out->pos[i] = in->stop_pos[idx[i]];
            memcpy(out->col[i].v, in->stop_col[idx[i]], 16);
        }
    }
    if (in->kind != PAINT_SOLID && !in->linear_colors)
        for (int i = 0; i < out->nstops; i++) out->col[i] = into_srgb(out->col[i]);
    if (in->kind == PAINT_LINEAR) {
        pt d = { in->p1[0] - in->p0[0], in->p1[1] - in->p0[1] };
        double dd = d.x * d.x + d.y * d.y;
        out->dir.x = d.x / dd;
        out->dir.y = d.y / dd;
    }
}

/* LinColor::lerp color.rs:352-354: other * t + self * (1 - t) */
static col4 col_lerp(col4 a, col4 b, float t) {
    col4 r;
    for (int i = 0; i < 4; i++) r.v[i] = b.v[i] * t + a.v[i] * (1.0f - t);
    return r;
}

/* GradStops::at grad.rs:116-139 (binary search for the first stop with position >= t) */
static col4 stops_at(const prepared_paint* pp, double t) {
    int size = pp->nstops;
    int lo = 0, hi = size;
    while (lo < hi) { /* partition point of `position < t` */
        int mid = (lo + hi) / 2;
        if (pp->pos[mid] < t) lo = mid + 1; else hi = mid;
    }
    int index = lo;
    if (index == 0) return pp->col[0];
    if (index == size) return pp->col[size - 1];
    double p0 = pp->pos[index - 1], p1 = pp->pos[index];
    double ratio = (t - p0) / (p1 - p0);
    return col_lerp(pp->col[index - 1], pp->col[index], (float)ratio);
}

/* Paint::at for LinColor (color.rs:357-360), GradLinear (grad.rs:202-211), GradRadial (:361-411) */
static col4 paint_at(const prepared_paint* pp, pt p) {
    const rzo_paint* in = &pp->p;
    col4 c;
    if (in->kind == PAINT_SOLID) { memcpy(c.v, in->solid, 16); return c; }
    double t;
    if (in->kind == PAINT_LINEAR) {
        pt d = { p.x - in->p0[0], p.y - in->p0[1] };
        t = d.x * pp->dir.x + d.y * pp->dir.y;
    } else {
        pt cd = { in->p0[0] - in->p1[0], in->p0[1] - in->p1[1] };
        pt pd = { p.x - in->p1[0], p.y - in->p1[1] };
        double rd = in->r0 - in->r1;
        double a = (cd.x * cd.x + cd.y * cd.y) - rd * rd;
        double b = -2.0 * ((cd.x * pd.x + cd.y * pd.y) + in->r1 * rd);
        double cc = (pd.x * pd.x + pd.y * pd.y) - in->r1 * in->r1;
        double r[2];
        int n = quadratic_solve(a, b, cc, r);
        if (n == 0) { col4 z = {{0, 0, 0, 0}}; return z; }
        t = n == 2 ? rust_fmax(r[0], r[1]) : r[0];
    }
    c = stops_at(pp, spread_at(in->spread, t));
    return in->linear_colors ? c : into_linear(c);
}

/* Public: evaluate a paint at a point (used by gradient KATs). */
void rzo_paint_at(const rzo_paint* paint, double x, double y, float* out) {
    prepared_paint pp;
    prepare_paint(paint, &pp);
    pt p = {x, y};
    col4 c = paint_at(&pp, p);
    memcpy(out, c.v, 16);
}
/* Public: GradRadial::offset (grad.rs:361-396); returns 0 for None. */
int rzo_radial_offset(const rzo_paint* in, double x, double y, double* out) {
    pt cd = { in->p0[0] - in->p1[0], in->p0[1] - in->p1[1] };
    pt pd = { x - in->p1[0], y - in->p1[1] };
    double rd = in->r0 - in->r1;
    double a = (cd.x * cd.x + cd.y * cd.y) - rd * rd;
    double b = -2.0 * ((cd.x * pd.x + cd.y * pd.y) + in->r1 * rd);
    double cc = (pd.x * pd.x + pd.y * pd.y) - in->r1 * in->r1;
    double r[2];
    int n = quadratic_solve(a, b, cc, r);
    if (n == 0) return 0;
    *out = n == 2 ? rust_fmax(r[0], r[1]) : r[0];
    return 1;
}
double rzo_spread_at(int spread, double t) { return spread_at(spread, t); }

/* Path::bbox path.rs:428-432 (tight, via Curve::bbox).  Returns 0 for an empty path. */
static int path_bbox(const uint8_t* kind, const double* pts, const uint32_t* sub_off, long nsub,
                     const xform* tr, bbox_t* out) {
    int have = 0;
    bbox_t b;
    for (long s = 0; s < nsub; s++) {
        long beg = sub_off[s], end = sub_off[s + 1];
        if (end <= beg) continue;
        for (long i = beg; i < end; i++) {
            seg sg = load_seg(kind, pts, i);
            seg st = seg_transform(&sg, tr);
            b = seg_bbox(&st, have ? &b : NULL);
            have = 1;
        }
    }
    if (have) *out = b;
    return have;
}

int rzo_path_bbox(const uint8_t* kind, const double* pts, const uint32_t* sub_off, long nsub,
                  const double* trm, double* out) {
    xform tr; memcpy(tr.m, trm, sizeof(tr.m));
    bbox_t b;
    if (!path_bbox(kind, pts, sub_off, nsub, &tr, &b)) return 0;
    out[0] = b.min.x; out[1] = b.min.y; out[2] = b.max.x; out[3] = b.max.y;
    return 1;
}

/* ------------------------------------------------------------------------ */
/* Rasterizer::fill rasterize.rs:69-115 (SD mask_iter + fill_impl)          */
/* ------------------------------------------------------------------------ */

/* img: LinColor (4 floats per pixel) view with Shape in pixel units. */
int rzo_fill(const uint8_t* kind, const double* pts, const uint32_t* sub_off, long nsub,
             const double* trm, int rule, double flatness, const rzo_paint* paint,
             float* data, long start, long width, long height, long row_stride, long col_stride) {
    if (width == 0 || height == 0) return 0;
    xform tr; memcpy(tr.m, trm, sizeof(tr.m));
    prepared_paint pp;
    prepare_paint(paint, &pp);
    int solid = paint->kind == PAINT_SOLID;
    xform pixel_tr = tr_identity();
    if (!solid) {
        xform paint_tr; memcpy(paint_tr.m, paint->tr, sizeof(paint_tr.m));
        xform units_tr;
        if (paint->units == UNITS_USER) {
            units_tr = tr_mul(tr, paint_tr);
        } else {
            xform id = tr_identity();
            bbox_t b;
            if (!path_bbox(kind, pts, sub_off, nsub, &id, &b)) return 0;
            /* BBox::unit_transform geometry.rs:662-664 */
            xform unit = tr_mul(tr_translate(b.min.x, b.min.y),
                                tr_scale(b.max.x - b.min.x, b.max.y - b.min.y));
            units_tr = tr_mul(tr_mul(tr, unit), paint_tr);
        }
        if (!tr_invert(units_tr, &pixel_tr)) return 0;
    }
    /* mask_iter with W+1 columns */
    long w1 = width + 1;
    double* buf = (double*)calloc((size_t)(w1 * height), sizeof(double));
    img_t im = { buf, w1 * height, 0, w1, height, w1, 1 };
    if (flatten_path(kind, pts, sub_off, nsub, &tr, flatness, sink_sd, &im, NULL) < 0) { free(buf); return -1; }
    col4 solid_col = {{0, 0, 0, 0}};
    if (solid) solid_col = paint_at(&pp, (pt){0.0, 0.0});
    double winding = 0.0;
    for (long index = 0; index < w1 * height; index++) {
        long y = index / w1, x = index - y * w1;
        if (x == 0) winding = 0.0;
        else if (x >= width) continue;
        winding += buf[index];
        double alpha = rzo_alpha_from_winding(rule, winding);
        if (fabs(alpha) < 1e-6) continue;
        col4 color;
        if (solid) color = solid_col;
        else {
            pt point = { (double)x + 0.5, (double)y + 0.5 };
            color = paint_at(&pp, tr_apply(&pixel_tr, point));
        }
        float* dst = data + 4 * (start + y * row_stride + x * col_stride);
        float af = (float)alpha;
        float src[4];
        for (int i = 0; i < 4; i++) src[i] = color.v[i] * af;
        float inv = 1.0f - src[3];
        for (int i = 0; i < 4; i++) dst[i] = src[i] + dst[i] * inv;
    }
    free(buf);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* scene.rs -- Scene::render for a Group of Fill nodes in path order        */
/* (Pipeline::build_rec :268-357, render :384-395, render_rec Fill :407-430) */
/* ------------------------------------------------------------------------ */

/* fills: n entries; fill f has nsubs[f] subpaths whose nsubs[f] + 1 absolute
 * segment offsets (into the shared kind/pts arrays) start at
 * sub_tab[sub_start[f]].  view = (0,0,canvas_w,canvas_h), tr = identity,
 * bg = background (Layer::new with a color). */
int rzo_scene_render(const uint8_t* kind, const double* pts, const uint32_t* sub_tab,
                     const int64_t* sub_start, const int64_t* nsubs, long n, const double* trs,
                     const int32_t* rules, const rzo_paint* paints, double flatness, long canvas_w,
                     long canvas_h, const float* bg, float* canvas) {
    /* Layer::new(view bbox, bg): x0 = floor(0), width = ceil(w) - floor(0) */
    for (long i = 0; i < canvas_w * canvas_h; i++) memcpy(canvas + 4 * i, bg, 16);
    bbox_t view = { {0.0, 0.0}, {(double)canvas_w, (double)canvas_h} };
    for (long f = 0; f < n; f++) {
        xform tr; memcpy(tr.m, trs + 6 * f, sizeof(tr.m));
        const uint32_t* so = sub_tab + sub_start[f];
        long nsub = (long)nsubs[f];
        bbox_t pb;
        if (!path_bbox(kind, pts, so, nsub, &tr, &pb)) continue;
        /* view_apply: view.intersect(bbox) geometry.rs:648-657, range_intersect :677-688 */
        if (view.min.x > pb.max.x || pb.min.x > view.max.x) continue;
        if (view.min.y > pb.max.y || pb.min.y > view.max.y) continue;
        bbox_t nb = bbox_new((pt){ rust_fmax(view.min.x, pb.min.x), rust_fmax(view.min.y, pb.min.y) },
                             (pt){ rust_fmin(view.max.x, pb.max.x), rust_fmin(view.max.y, pb.max.y) });
        long layer_x = 0, layer_y = 0; /* floor(view.min) */
        long col_min = (long)floor(nb.min.x) - layer_x;
        long col_max = (long)ceil(nb.max.x) - layer_x + 1;
        long row_min = (long)floor(nb.min.y) - layer_y;
        long row_max = (long)ceil(nb.max.y) - layer_y + 1;
        /* `i32 as usize` wraps a negative value to a huge one, which
         * view_shape then clamps to the image size (image.rs:588-605) */
        if (col_min < 0) col_min = canvas_w;
        if (row_min < 0) row_min = canvas_h;
        if (col_max < 0) col_max = canvas_w;
        if (row_max < 0) row_max = canvas_h;
        if (row_min > canvas_h) row_min = canvas_h;
        if (row_max > canvas_h) row_max = canvas_h;
        if (row_max < row_min) row_max = row_min;
        if (col_min > canvas_w) col_min = canvas_w;
        if (col_max > canvas_w) col_max = canvas_w;
        if (col_max < col_min) col_max = col_min;
        xform align = tr_translate(-floor(nb.min.x), -floor(nb.min.y));
        xform ptr = tr_mul(align, tr);
        int rc = rzo_fill(kind, pts, so, nsub, ptr.m, rules[f], flatness, &paints[f], canvas,
                          row_min * canvas_w + col_min, col_max - col_min, row_max - row_min, canvas_w, 1);
        if (rc < 0) return rc;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Differentiable batch.  The reference has no adjoint: this composes its   */
/* Rasterizer::fill (rasterize.rs:69-115, i.e. mask_iter with the image     */
/* size :313-355, then source-over) for closed cubic paths drawn in order   */
/* with a solid paint of alpha `a` (the alpha channel of the image), and    */
/* adds the adjoint of that image with respect to every control point, the  */
/* bisection tree held fixed.                                               */
/*                                                                          */
/* Control points of one image: point j of path p at ctrl[2 * (p * 3 * segs */
/* + j)]; segment s is the cubic (V_s, C1_s, C2_s, V_{(s+1) mod segs}) with  */
/* V_s = point 3s, C1_s = 3s + 1, C2_s = 3s + 2.  The closing line of every  */
/* path starts and ends at V_0 and adds nothing.                            */
/* ------------------------------------------------------------------------ */

typedef struct { pt a, b; int seg; double t0, t1; } tline_t;
typedef struct { tline_t* v; long n, cap; } tline_vec;

static void tline_push(tline_vec* lv, tline_t l) {
    if (lv->n == lv->cap) {
        lv->cap = lv->cap ? 2 * lv->cap : 1024;
        lv->v = (tline_t*)realloc(lv->v, sizeof(tline_t) * lv->cap);
    }
    lv->v[lv->n++] = l;
}

static void diff_indices(int s, int segs, int idx[4]) {
    idx[0] = 3 * s; idx[1] = 3 * s + 1; idx[2] = 3 * s + 2; idx[3] = 3 * ((s + 1) % segs);
}

static seg diff_segment(const double* ctrl, long p, int segs, int s) {
    seg c;
    c.kind = SEG_CUBIC;
    const double* b = ctrl + 2L * p * 3 * segs;
    int idx[4];
    diff_indices(s, segs, idx);
    for (int k = 0; k < 4; k++) c.p[k] = (pt){b[2 * idx[k]], b[2 * idx[k] + 1]};
    return c;
}

static void bernstein3(double t, double b[4]) {
    double mt = 1.0 - t;
    b[0] = mt * mt * mt; b[1] = 3.0 * t * mt * mt; b[2] = 3.0 * t * t * mt; b[3] = t * t * t;
}

static pt bez3(const seg* c, double t) {
    double b[4];
    bernstein3(t, b);
    pt r = {0.0, 0.0};
    for (int k = 0; k < 4; k++) { r.x += b[k] * c->p[k].x; r.y += b[k] * c->p[k].y; }
    return r;
}

/* PathFlattenIter on path p (path.rs:734-796) with every line's segment and
 * parameter range.  With `frozen`, the tree of the `frozen` control points
 * is used and the vertices are evaluated on `ctrl` at the same parameters
 * (finite differences with the tree held fixed). */
static int diff_flatten(const double* ctrl, const double* frozen, long p, int segs, double flatness, tline_vec* out) {
    double thr = 16.0 * flatness * flatness;
    typedef struct { seg s; double t0, t1; } node_t;
    long cap = 256, top = 0;
    node_t* stack = (node_t*)malloc(sizeof(node_t) * cap);
    for (int s = 0; s < segs; s++) {
        seg root = diff_segment(frozen ? frozen : ctrl, p, segs, s);
        seg real = diff_segment(ctrl, p, segs, s);
        top = 0;
        stack[top++] = (node_t){root, 0.0, 1.0};
        while (top > 0) {
            node_t cur = stack[--top];
            if (seg_has_nans(&cur.s)) { free(stack); return -1; }
            if (seg_flatness(&cur.s) < thr) {
                tline_t l;
                l.seg = s; l.t0 = cur.t0; l.t1 = cur.t1;
                if (frozen) { l.a = bez3(&real, cur.t0); l.b = bez3(&real, cur.t1); }
                else { l.a = seg_start(&cur.s); l.b = seg_end(&cur.s); }
                tline_push(out, l);
                continue;
            }
            seg a, b;
            seg_split(&cur.s, &a, &b);
            double tm = 0.5 * (cur.t0 + cur.t1);
            if (top + 2 > cap) { cap *= 2; stack = (node_t*)realloc(stack, sizeof(node_t) * cap); }
            stack[top++] = (node_t){b, tm, cur.t1};
            stack[top++] = (node_t){a, cur.t0, tm};
        }
    }
    free(stack);
    return 0;
}

/* Winding of every pixel of a W x H image from the lines of one path
 * (mask_iter's (W+1)-column buffer and row prefix, rasterize.rs:325-352). */
static void diff_winding(const tline_vec* lv, long W, long H, double* buf, double* wind) {
    memset(buf, 0, sizeof(double) * (size_t)((W + 1) * H));
    img_t im = {buf, (W + 1) * H, 0, W + 1, H, W + 1, 1};
    for (long i = 0; i < lv->n; i++) {
        line_t l = {lv->v[i].a, lv->v[i].b};
        signed_difference_line(&im, l);
    }
    for (long y = 0; y < H; y++) {
        double acc = 0.0;
        for (long x = 0; x < W; x++) {
            acc += buf[y * (W + 1) + x];
            wind[y * W + x] = acc;
        }
    }
}

/* alpha as Rasterizer::fill uses it: pixels with |alpha| < 1e-6 are skipped */
static double diff_alpha(int rule, double w) {
    double a = rzo_alpha_from_winding(rule, w);
    return fabs(a) < 1e-6 ? 0.0 : a;
}

static double diff_dalpha(int rule, double w) {
    if (rule == RULE_EVENODD) {
        double r = rem_euclid(w + 1.0, 2.0) - 1.0;
        if (fabs(r) < 1e-6) return 0.0;
        return r > 0.0 ? 1.0 : -1.0;
    }
    double v = fabs(w);
    if (v >= 1.0 || v < 1e-6) return 0.0;
    return w > 0.0 ? 1.0 : -1.0;
}

/* Image (alpha channel) of `n_paths` paths drawn in order; image: W x H, written. */
int rzo_diff_forward(const double* ctrl, const double* frozen, long n_paths, long segs, long W, long H, double a,
                     int rule, double flatness, double* image) {
    memset(image, 0, sizeof(double) * (size_t)(W * H));
    double* buf = (double*)malloc(sizeof(double) * (size_t)((W + 1) * H));
    double* wind = (double*)malloc(sizeof(double) * (size_t)(W * H));
    tline_vec lv = {0, 0, 0};
    int rc = 0;
    for (long p = 0; p < n_paths && rc == 0; p++) {
        lv.n = 0;
        if (diff_flatten(ctrl, frozen, p, (int)segs, flatness, &lv) < 0) { rc = -1; break; }
        diff_winding(&lv, W, H, buf, wind);
        for (long i = 0; i < W * H; i++) {
            double al = diff_alpha(rule, wind[i]);
            if (al == 0.0) continue;
            image[i] = a * al + image[i] * (1.0 - a * al);
        }
    }
    free(lv.v); free(buf); free(wind);
    return rc;
}

typedef struct { double v, d[4]; } dual4;

static dual4 dv_const(double v) { dual4 r = {v, {0, 0, 0, 0}}; return r; }
static dual4 dv_add(dual4 a, dual4 b) { for (int k = 0; k < 4; k++) a.d[k] += b.d[k]; a.v += b.v; return a; }
static dual4 dv_sub(dual4 a, dual4 b) { for (int k = 0; k < 4; k++) a.d[k] -= b.d[k]; a.v -= b.v; return a; }
static dual4 dv_mul(dual4 a, dual4 b) {
    dual4 r; r.v = a.v * b.v;
    for (int k = 0; k < 4; k++) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
    return r;
}
static dual4 dv_div(dual4 a, dual4 b) {
    dual4 r; r.v = a.v / b.v;
    for (int k = 0; k < 4; k++) r.d[k] = (a.d[k] - r.v * b.d[k]) / b.v;
    return r;
}
static dual4 dv_lerp(dual4 a, dual4 b, dual4 t) {  /* (1 - t) a + t b */
    return dv_add(dv_mul(dv_sub(dv_const(1.0), t), a), dv_mul(t, b));
}

/* Mean of W_row over [lo, hi] and its derivatives; W_row(X) = G[k+1] + (k+1-X) g[k]
 * on [k, k+1) is the loss change per unit of signed height at X (G: suffix
 * sums of g, G[W] = 0). */
static void diff_row_mean(const double* G, const double* g, long W, double lo, double hi, double* I, double* dlo,
                          double* dhi) {
    if (lo < 0.0) lo = 0.0;
    if (hi > (double)W) hi = (double)W;
    if (hi < lo) hi = lo;
    double D = hi - lo;
    if (D < 1e-12) {
        long k = (long)floor(lo);
        if (k > W - 1) k = W - 1;
        if (k < 0) k = 0;
        *I = G[k + 1] + ((double)(k + 1) - lo) * g[k];
        *dlo = *dhi = -0.5 * g[k];
        return;
    }
    long k0 = (long)floor(lo), k1 = (long)floor(hi);
    if (k1 > W - 1) k1 = W - 1;
    double sI = 0.0, slo = 0.0, shi = 0.0;
    for (long k = k0; k <= k1; k++) {
        double a = fmax(lo, (double)k), b = fmin(hi, (double)(k + 1));
        if (b <= a) continue;
        double ka = (double)(k + 1) - a, kb = (double)(k + 1) - b;
        sI += G[k + 1] * (b - a) + g[k] * 0.5 * (ka * ka - kb * kb);
        shi += -g[k] * 0.5 * ((b - lo) * (b - lo) - (a - lo) * (a - lo));
        slo += -g[k] * 0.5 * ((hi - a) * (hi - a) - (hi - b) * (hi - b));
    }
    *I = sI / D;
    *dhi = shi / (D * D);
    *dlo = slo / (D * D);
}

/* d(sum over pixels of g * winding contribution of the piece p -> q)/d(line ends) */
static void diff_piece(dual4 px, dual4 py, dual4 qx, dual4 qy, long W, long H, const double* G, const double* g,
                       double out[4]) {
    if (fabs(py.v - qy.v) < 1e-300) {
        /* horizontal: no coverage, but its height derivative moves coverage in */
        long r = (long)floor(py.v);
        if (r < 0 || r >= H) return;
        double I, dlo, dhi;
        diff_row_mean(G + r * (W + 1), g + r * W, W, fmin(px.v, qx.v), fmax(px.v, qx.v), &I, &dlo, &dhi);
        for (int k = 0; k < 4; k++) out[k] += I * (qy.d[k] - py.d[k]);
        return;
    }
    double dir = 1.0;
    if (py.v > qy.v) { dual4 t = px; px = qx; qx = t; t = py; py = qy; qy = t; dir = -1.0; }
    dual4 k_ = dv_div(dv_sub(qx, px), dv_sub(qy, py));  /* dx/dy */
    long r0 = (long)floor(py.v), r1 = (long)ceil(qy.v);
    if (r0 < 0) r0 = 0;
    if (r1 > H) r1 = H;
    for (long r = r0; r < r1; r++) {
        int start_in = py.v >= (double)r, end_in = qy.v <= (double)(r + 1);
        dual4 sa = start_in ? py : dv_const((double)r);
        dual4 sb = end_in ? qy : dv_const((double)(r + 1));
        if (sb.v <= sa.v) continue;
        dual4 xa = start_in ? px : dv_add(px, dv_mul(dv_sub(sa, py), k_));
        dual4 xn = end_in ? qx : dv_add(px, dv_mul(dv_sub(sb, py), k_));
        dual4 h = dv_sub(sb, sa);
        dual4 lo = xa.v <= xn.v ? xa : xn, hi = xa.v <= xn.v ? xn : xa;
        double I, dlo, dhi;
        diff_row_mean(G + r * (W + 1), g + r * W, W, lo.v, hi.v, &I, &dlo, &dhi);
        for (int k = 0; k < 4; k++)
            out[k] += dir * (I * h.d[k] + h.v * (dlo * lo.d[k] + dhi * hi.d[k]));
    }
}

/* The x rules of signed_difference_line (rasterize.rs:372-393, 923-937) on
 * dual numbers, then the pieces. */
static void diff_line(pt a, pt b, long W, long H, const double* G, const double* g, double out[4]) {
    dual4 x0 = {a.x, {1, 0, 0, 0}}, y0 = {a.y, {0, 1, 0, 0}}, x1 = {b.x, {0, 0, 1, 0}}, y1 = {b.y, {0, 0, 0, 1}};
    double width = (double)W;
    if (x0.v > width || x1.v > width) {
        if (x0.v > width && x1.v > width) {
            x0 = dv_const(width - 0.001);
            x1 = dv_const(width - 0.001);
        } else {
            dual4 t = dv_div(dv_sub(x0, dv_const(width)), dv_sub(x0, x1));
            dual4 my = dv_lerp(y0, y1, t);
            if (x0.v < width) { x1 = dv_const(width); y1 = my; }
            else { x0 = dv_const(width); y0 = my; }
        }
    }
    if (x0.v >= 0.0 && x1.v >= 0.0) {
        diff_piece(x0, y0, x1, y1, W, H, G, g, out);
    } else if (x0.v <= 0.0 && x1.v <= 0.0) {
        diff_piece(dv_const(0.0), y0, dv_const(0.0), y1, W, H, G, g, out);
    } else {
        dual4 t = dv_div(x0, dv_sub(x0, x1));
        dual4 mx = dv_lerp(x0, x1, t), my = dv_lerp(y0, y1, t);
        if (x0.v < 0.0) {
            diff_piece(mx, my, x1, y1, W, H, G, g, out);
            diff_piece(dv_const(0.0), y0, mx, my, W, H, G, g, out);
        } else {
            diff_piece(x0, y0, mx, my, W, H, G, g, out);
            diff_piece(mx, my, dv_const(0.0), y1, W, H, G, g, out);
        }
    }
}

/* Adjoint: dl_dctrl (same layout as ctrl, overwritten) from dl_dimage, given
 * the forward image.  d image / d alpha_p = a (1 - image) / (1 - a alpha_p)
 * for source-over, so every path is independent once the image is known. */
int rzo_diff_backward(const double* ctrl, long n_paths, long segs, long W, long H, double a, int rule,
                      double flatness, const double* image, const double* dl_dimage, double* dl_dctrl) {
    memset(dl_dctrl, 0, sizeof(double) * (size_t)(n_paths * 3 * segs * 2));
    double* buf = (double*)malloc(sizeof(double) * (size_t)((W + 1) * H));
    double* wind = (double*)malloc(sizeof(double) * (size_t)(W * H));
    double* g = (double*)malloc(sizeof(double) * (size_t)(W * H));
    double* G = (double*)malloc(sizeof(double) * (size_t)((W + 1) * H));
    tline_vec lv = {0, 0, 0};
    int rc = 0;
    for (long p = 0; p < n_paths; p++) {
        lv.n = 0;
        if (diff_flatten(ctrl, NULL, p, (int)segs, flatness, &lv) < 0) { rc = -1; break; }
        diff_winding(&lv, W, H, buf, wind);
        for (long i = 0; i < W * H; i++) {
            double al = diff_alpha(rule, wind[i]);
            double da = al == 0.0 ? 0.0 : diff_dalpha(rule, wind[i]);
            g[i] = da == 0.0 ? 0.0 : dl_dimage[i] * a * (1.0 - image[i]) / (1.0 - a * al) * da;
        }
        for (long y = 0; y < H; y++) {
            G[y * (W + 1) + W] = 0.0;
            for (long x = W - 1; x >= 0; x--) G[y * (W + 1) + x] = G[y * (W + 1) + x + 1] + g[y * W + x];
        }
        double* out = dl_dctrl + 2L * p * 3 * segs;
        for (long i = 0; i < lv.n; i++) {
            const tline_t* l = &lv.v[i];
            double d4[4] = {0, 0, 0, 0};
            diff_line(l->a, l->b, W, H, G, g, d4);
            int idx[4];
            diff_indices(l->seg, (int)segs, idx);
            double b0[4], b1[4];
            bernstein3(l->t0, b0);
            bernstein3(l->t1, b1);
            for (int j = 0; j < 4; j++) {
                out[2 * idx[j]] += d4[0] * b0[j] + d4[2] * b1[j];
                out[2 * idx[j] + 1] += d4[1] * b0[j] + d4[3] * b1[j];
            }
        }
    }
    free(lv.v); free(buf); free(wind); free(g); free(G);
    return rc;
}
