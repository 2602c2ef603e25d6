// rz_stroke.cu -- Path::stroke on the GPU (src/path.rs:374-415, 692-732;
// src/curve.rs:977-1076, 1290-1433), binary64 with every product and sum
// rounded on its own (dm / da / ds), as the reference computes.
//
// The outline of a subpath is a sequence of units, laid out by the host:
//   OFFSET   the offset pieces of one input segment (forward, or reversed
//            for the way back): Tiller-Hanson with splits up to depth 3 and
//            Round joins between pieces of a cubic that do not meet;
//   JOIN     the join (or, once per open subpath, the cap) from the last
//            piece of the nearest earlier non-empty OFFSET of the same list
//            to the first piece of the OFFSET that follows it;
//   CLOSE    stroke_close of a closed subpath's list (forward or back);
//   CAPEND   the cap from the last piece of an open subpath's list to its
//            first piece.
// Every unit's pieces depend only on its own segment and its neighbours'
// end pieces.  OFFSET units come first: the curves' split trees level by level
// and their leaves one thread each, then one thread per unit assembles its
// pieces (into kStrokeOffsetMax slots each, or counted and then packed when
// those slots would be too large); then one thread per other unit, reading
// the neighbours' pieces, counts its own; the host turns the counts into the
// outline's layout, and the other units' pieces and the OFFSET pieces land in
// place.  hypot and the arc's transcendental functions are CUDA's binary64 ones.
#include <cuda_runtime.h>
#include <stdint.h>

#include "rz_arc.cuh"
#include "rz_stroke.cuh"

namespace rz {

struct SP {
    double x, y;
};
struct SSeg {
    int kind;  // 0 line, 1 quad, 2 cubic
    SP p[4];
};
struct SLn {
    SP a, b;
};

__device__ __forceinline__ SP padd(SP a, SP b) { return SP{da(a.x, b.x), da(a.y, b.y)}; }
__device__ __forceinline__ SP psub(SP a, SP b) { return SP{ds(a.x, b.x), ds(a.y, b.y)}; }
__device__ __forceinline__ SP pmul(double s, SP a) { return SP{dm(s, a.x), dm(s, a.y)}; }
__device__ __forceinline__ double pdot(SP a, SP b) { return da(dm(a.x, b.x), dm(a.y, b.y)); }
__device__ __forceinline__ double pcross(SP a, SP b) { return ds(dm(a.x, b.y), dm(a.y, b.x)); }
__device__ __forceinline__ double plen(SP a) { return hypot(a.x, a.y); }
__device__ __forceinline__ bool pclose(SP a, SP b) { return fabs(ds(a.x, b.x)) < EPS64 && fabs(ds(a.y, b.y)) < EPS64; }
__device__ __forceinline__ bool pnormalize(SP a, SP& out) {
    const double l = plen(a);
    if (l < EPS64) return false;
    out = SP{a.x / l, a.y / l};
    return true;
}
__device__ __forceinline__ int slast(int kind) { return kind == 0 ? 1 : (kind == 1 ? 2 : 3); }
__device__ __forceinline__ SP sstart(const SSeg& s) { return s.p[0]; }
__device__ __forceinline__ SP send(const SSeg& s) { return s.p[slast(s.kind)]; }
__device__ __forceinline__ SSeg sline(SP a, SP b) {
    SSeg s;
    s.kind = 0;
    s.p[0] = a;
    s.p[1] = b;
    s.p[2] = s.p[3] = SP{0.0, 0.0};
    return s;
}

// Line::at, Line::intersect (src/curve.rs:204-215, 250-253)
__device__ __forceinline__ SP lat(const SLn& l, double t) {
    const double u = ds(1.0, t);
    return SP{da(dm(u, l.a.x), dm(t, l.b.x)), da(dm(u, l.a.y), dm(t, l.b.y))};
}
__device__ __forceinline__ bool lintersect(const SLn& s, const SLn& o, double& t0, double& t1) {
    const double x1 = s.a.x, y1 = s.a.y, x2 = s.b.x, y2 = s.b.y, x3 = o.a.x, y3 = o.a.y, x4 = o.b.x, y4 = o.b.y;
    const double det = ds(dm(ds(x4, x3), ds(y1, y2)), dm(ds(x1, x2), ds(y4, y3)));
    if (fabs(det) < EPS64) return false;
    t0 = da(dm(ds(y3, y4), ds(x1, x3)), dm(ds(x4, x3), ds(y1, y3))) / det;
    t1 = da(dm(ds(y1, y2), ds(x1, x3)), dm(ds(x2, x1), ds(y1, y3))) / det;
    return true;
}
__device__ __forceinline__ bool in01(double t) { return t >= 0.0 && t <= 1.0; }

// Segment::ends (src/curve.rs:195-197, 377-388, 647-666)
__device__ void sends(const SSeg& s, SLn& start, SLn& end) {
    if (s.kind == 0) {
        start = end = SLn{s.p[0], s.p[1]};
    } else if (s.kind == 1) {
        const SLn a{s.p[0], s.p[1]}, b{s.p[1], s.p[2]};
        if (pclose(s.p[0], s.p[1])) start = end = b;
        else if (pclose(s.p[1], s.p[2])) start = end = a;
        else { start = a; end = b; }
    } else {
        int i0 = 0, i1 = 0;
        for (int i = 0; i < 3; ++i)
            if (!pclose(s.p[i], s.p[i + 1])) { i0 = i; break; }
        for (int i = 3; i >= 1; --i)
            if (!pclose(s.p[i], s.p[i - 1])) { i1 = i; break; }
        if (i1 < 1) i1 = 1;
        start = SLn{s.p[i0], s.p[i0 + 1]};
        end = SLn{s.p[i1 - 1], s.p[i1]};
    }
}

// Quad::at, Cubic::at (src/curve.rs:432-441, 712-723)
__device__ SP sat(const SSeg& s, double t) {
    const double t1 = t, t_1 = ds(1.0, t), t2 = dm(t1, t1), t_2 = dm(t_1, t_1);
    const SP* p = s.p;
    if (s.kind == 1) {
        const double w1 = dm(dm(2.0, t1), t_1);
        return SP{da(da(dm(t_2, p[0].x), dm(w1, p[1].x)), dm(t2, p[2].x)),
                  da(da(dm(t_2, p[0].y), dm(w1, p[1].y)), dm(t2, p[2].y))};
    }
    const double t3 = dm(t2, t1), t_3 = dm(t_2, t_1);
    const double w1 = dm(dm(3.0, t1), t_2), w2 = dm(dm(3.0, t2), t_1);
    return SP{da(da(da(dm(t_3, p[0].x), dm(w1, p[1].x)), dm(w2, p[2].x)), dm(t3, p[3].x)),
              da(da(da(dm(t_3, p[0].y), dm(w1, p[1].y)), dm(w2, p[2].y)), dm(t3, p[3].y))};
}

// quadratic_solve (src/utils.rs:205-231)
__device__ int qsolve(double a, double b, double c, double* r) {
    if (fabs(a) < EPS64) {
        if (fabs(b) > EPS64) {
            r[0] = -c / b;
            return 1;
        }
        return 0;
    }
    const double disc = ds(dm(b, b), dm(dm(4.0, a), c));
    if (fabs(disc) < EPS64) {
        r[0] = -b / dm(2.0, a);
        return 1;
    }
    if (disc > 0.0) {
        const double sq = sqrt(disc);
        if (b >= 0.0) {
            const double mul = ds(-b, sq);
            r[0] = mul / dm(2.0, a);
            r[1] = dm(2.0, c) / mul;
        } else {
            const double mul = da(-b, sq);
            r[0] = dm(2.0, c) / mul;
            r[1] = mul / dm(2.0, a);
        }
        return 2;
    }
    return 0;
}

struct SBox {
    double x0, y0, x1, y1;
};
__device__ __forceinline__ SBox bnew(SP a, SP b) {
    SBox r;
    if (a.x <= b.x) { r.x0 = a.x; r.x1 = b.x; } else { r.x0 = b.x; r.x1 = a.x; }
    if (a.y <= b.y) { r.y0 = a.y; r.y1 = b.y; } else { r.y0 = b.y; r.y1 = a.y; }
    return r;
}
__device__ __forceinline__ SBox bext(SBox b, SP p) {
    if (p.x < b.x0) b.x0 = p.x; else if (p.x > b.x1) b.x1 = p.x;
    if (p.y < b.y0) b.y0 = p.y; else if (p.y > b.y1) b.y1 = p.y;
    return b;
}
__device__ __forceinline__ bool bcontains(SBox b, SP p) { return b.x0 <= p.x && p.x <= b.x1 && b.y0 <= p.y && p.y <= b.y1; }

// Curve::bbox(None) of a quad or cubic (src/curve.rs:505-513, 815-824)
__device__ SBox sbbox(const SSeg& s) {
    const SP* p = s.p;
    if (s.kind == 1) {
        SBox b = bnew(p[0], p[2]);
        if (bcontains(b, p[1])) return b;
        const double a0 = da(ds(p[2].x, dm(2.0, p[1].x)), p[0].x), a1 = da(ds(p[2].y, dm(2.0, p[1].y)), p[0].y);
        const double b0 = ds(p[1].x, p[0].x), b1 = ds(p[1].y, p[0].y);
        if (fabs(a0) > EPS64) {
            const double t0 = -b0 / a0;
            if (in01(t0)) b = bext(b, sat(s, t0));
        }
        if (fabs(a1) > EPS64) {
            const double t1 = -b1 / a1;
            if (in01(t1)) b = bext(b, sat(s, t1));
        }
        return b;
    }
    SBox b = bnew(p[0], p[3]);
    if (bcontains(b, p[1]) && bcontains(b, p[2])) return b;
    const double a0 = da(ds(da(dm(-1.0, p[0].x), dm(3.0, p[1].x)), dm(3.0, p[2].x)), dm(1.0, p[3].x));
    const double a1 = da(ds(da(dm(-1.0, p[0].y), dm(3.0, p[1].y)), dm(3.0, p[2].y)), dm(1.0, p[3].y));
    const double b0 = da(ds(dm(2.0, p[0].x), dm(4.0, p[1].x)), dm(2.0, p[2].x));
    const double b1 = da(ds(dm(2.0, p[0].y), dm(4.0, p[1].y)), dm(2.0, p[2].y));
    const double c0 = da(dm(-1.0, p[0].x), p[1].x), c1 = da(dm(-1.0, p[0].y), p[1].y);
    double r[4];
    int n = qsolve(a0, b0, c0, r);
    n += qsolve(a1, b1, c1, r + n);
    for (int i = 0; i < n; ++i)
        if (in01(r[i])) b = bext(b, sat(s, r[i]));
    return b;
}

// line_offset (src/curve.rs:1290-1295)
__device__ bool loffset(const SLn& l, double dist, SLn& out) {
    const SP d = psub(l.b, l.a);
    SP n;
    if (!pnormalize(SP{d.y, -d.x}, n)) return false;
    const SP off = pmul(dist, n);
    out = SLn{padd(l.a, off), padd(l.b, off)};
    return true;
}

// polyline_offset (src/curve.rs:1302-1352)
__device__ bool polyoffset(SP* ps, int n, double dist) {
    bool have = false;
    SLn prev{};
    int index = 0;
    for (;;) {
        int repeats = 1;
        for (int i = index; i < n - 1; ++i) {
            if (!pclose(ps[i], ps[i + 1])) break;
            repeats += 1;
        }
        if (index + repeats >= n) break;
        index += repeats;
        SLn next;
        loffset(SLn{ps[index - 1], ps[index]}, dist, next);
        SP point = next.a;
        double t0, t1;
        if (have && lintersect(prev, next, t0, t1)) point = lat(prev, t0);
        for (int i = index - repeats; i < index; ++i) ps[i] = point;
        prev = next;
        have = true;
    }
    if (!have) return false;
    for (int i = index; i < n; ++i) ps[i] = prev.b;
    return true;
}

__device__ double sdiag(const SSeg& s) {
    const SBox b = sbbox(s);
    return hypot(ds(b.x0, b.x1), ds(b.y0, b.y1));
}

// quad_offset_should_split (src/curve.rs:1355-1368)
__device__ bool qsplit_needed(const SSeg& q) {
    const SP p0 = q.p[0], p1 = q.p[1], p2 = q.p[2];
    if (pdot(psub(p0, p1), psub(p2, p1)) > 0.0) return true;
    const SP mass{da(da(p0.x, p1.x), p2.x) / 3.0, da(da(p0.y, p1.y), p2.y) / 3.0};
    return dm(sdiag(q), 0.1) < plen(psub(mass, sat(q, 0.5)));
}

// cubic_offset_should_split (src/curve.rs:1412-1431)
__device__ bool csplit_needed(const SSeg& c) {
    const SP p0 = c.p[0], p1 = c.p[1], p2 = c.p[2], p3 = c.p[3];
    if (pdot(psub(p3, p0), psub(p2, p1)) < 0.0) return true;
    const double a0 = pcross(psub(p3, p0), psub(p1, p0)), a1 = pcross(psub(p3, p0), psub(p2, p0));
    if (dm(a0, a1) < 0.0) return true;
    const SP mass{da(da(da(p0.x, p1.x), p2.x), p3.x) / 4.0, da(da(da(p0.y, p1.y), p2.y), p3.y) / 4.0};
    return dm(sdiag(c), 0.1) < plen(psub(mass, sat(c, 0.5)));
}

// Pieces go to `out` (up to `cap`, then only counted).
// Pieces go to `out` (up to `cap`, then only counted), or, with gkind set,
// straight to pieces gbase, gbase + 1, ... of a global piece array (no
// thread-local buffer: a large one lives in local memory).
struct Sink {
    SSeg* out;
    int cap;
    int n;
    uint8_t* gkind = nullptr;
    double* gpts = nullptr;
    uint64_t gbase = 0;
    __device__ void push(const SSeg& s) {
        if (n < cap) {
            if (gkind) {
                const uint64_t i = gbase + (uint64_t)n;
                gkind[i] = (uint8_t)s.kind;
                const int last = s.kind == 0 ? 1 : (s.kind == 1 ? 2 : 3);
                for (int j = 0; j < 4; ++j) {
                    gpts[8 * i + 2 * j] = j <= last ? s.p[j].x : 0.0;
                    gpts[8 * i + 2 * j + 1] = j <= last ? s.p[j].y : 0.0;
                }
            } else if (out) {
                out[n] = s;
            }
        }
        ++n;
    }
};

// The Round join's arc (EllipArc::new_param + to_cubics), or the bevel when
// new_param gives None.
__device__ void sround(SP from, SP to, double r, bool sweep, const SSeg& bevel, Sink& out) {
    const double a[8] = {from.x, from.y, to.x, to.y, r, r, 0.0, sweep ? 2.0 : 0.0};
    Seg64 cub[4];
    const int n = arc_to_cubics64(a, cub);
    if (n < 0) {
        out.push(bevel);
        return;
    }
    for (int i = 0; i < n; ++i) {
        SSeg c;
        c.kind = 2;
        for (int j = 0; j < 4; ++j) c.p[j] = SP{cub[i].x[j], cub[i].y[j]};
        out.push(c);
    }
}

// Segment::line_join (src/curve.rs:977-1047)
__device__ void sjoin(const SSeg& self, const SSeg& other, double width, int join, double miter, Sink& out) {
    const SP e = send(self), s = sstart(other);
    if (pclose(e, s)) return;
    const SSeg bevel = sline(e, s);
    SLn tmp, start, end;
    sends(self, tmp, start);
    sends(other, end, tmp);
    double t0, t1;
    if (join == STROKE_JOIN_BEVEL) {
        out.push(bevel);
    } else if (join == STROKE_JOIN_MITER) {
        if (!lintersect(start, end, t0, t1) || (in01(t0) && in01(t1))) {
            out.push(bevel);
            return;
        }
        const SP p0 = psub(start.b, start.a), p1 = psub(end.a, end.b);
        const double lengths = dm(plen(p0), plen(p1));
        if (lengths < EPS64) {
            out.push(bevel);
            return;
        }
        const double c = pdot(p0, p1) / lengths;
        const double ml = width / sqrt(ds(1.0, c) / 2.0);
        if (ml < miter) {
            const SP p = lat(start, t0);
            out.push(sline(start.b, p));
            out.push(sline(p, end.a));
        } else {
            out.push(bevel);
        }
    } else {
        if (lintersect(start, end, t0, t1) && in01(t0) && in01(t1)) {
            out.push(bevel);
            return;
        }
        const bool sweep = pcross(psub(start.b, start.a), psub(s, e)) >= 0.0;
        sround(start.b, end.a, width / 2.0, sweep, bevel, out);
    }
}

// Segment::line_cap (src/curve.rs:1050-1076)
__device__ void scap(const SSeg& self, const SSeg& other, double width, int cap, Sink& out) {
    const SP e = send(self), s = sstart(other);
    if (pclose(e, s)) return;
    if (cap == STROKE_CAP_BUTT) {
        out.push(sline(e, s));
    } else if (cap == STROKE_CAP_SQUARE) {
        SLn tmp, from;
        sends(self, tmp, from);
        SP tang;
        if (pnormalize(psub(from.b, from.a), tang)) {
            const SSeg l0 = sline(e, padd(e, pmul(width / 2.0, tang)));
            const SSeg l1 = sline(l0.p[1], padd(l0.p[1], psub(s, e)));
            out.push(l0);
            out.push(l1);
            out.push(sline(l1.p[1], s));
        }
    } else {
        sjoin(self, other, width, STROKE_JOIN_ROUND, 0.0, out);
    }
}

__device__ SSeg load_sseg(const uint8_t* kind, const double* pts, uint32_t g, bool reversed) {
    SSeg s;
    const int k = kind[g];
    s.kind = k == SEG_LINE ? 0 : (k == SEG_QUAD ? 1 : 2);
    const int n = slast(s.kind);
    for (int j = 0; j < 4; ++j) s.p[j] = SP{pts[8ull * g + 2 * j], pts[8ull * g + 2 * j + 1]};
    if (reversed)
        for (int j = 0; j <= n / 2; ++j) {
            const SP t = s.p[j];
            s.p[j] = s.p[n - j];
            s.p[n - j] = t;
        }
    return s;
}

__device__ __forceinline__ SSeg read_piece(const uint8_t* kind, const double* pts, uint64_t i) {
    SSeg s;
    s.kind = kind[i];
    for (int j = 0; j < 4; ++j) s.p[j] = SP{pts[8 * i + 2 * j], pts[8 * i + 2 * j + 1]};
    return s;
}

__device__ __forceinline__ void write_piece(uint8_t* kind, double* pts, uint64_t i, const SSeg& s) {
    kind[i] = (uint8_t)s.kind;
    const int n = slast(s.kind);
    for (int j = 0; j < 4; ++j) {
        pts[8 * i + 2 * j] = j <= n ? s.p[j].x : 0.0;
        pts[8 * i + 2 * j + 1] = j <= n ? s.p[j].y : 0.0;
    }
}

// ---------------------------------------------------------------------------
// Segment::offset (src/curve.rs:275-277, 515-517, 825-827), node-parallel.
// The reference splits a quad (split_at(0.5)) or a cubic (Cubic::split) while
// quad/cubic_offset_should_split says so, up to depth 3, depth first, offsets
// each leaf's control polygon and puts a Round join between consecutive pieces
// of a cubic that do not meet.  GB300's FP64 pipe is paid per warp
// instruction, so a thread per segment walking its own tree (lanes at
// different nodes doing different work) wastes most of it.  Here every kernel
// gives its threads the same work: the split decision of one node (levels 0,
// 1, 2; a node at depth 3 is always a leaf), the offset of one leaf, then the
// assembly of one unit's pieces in depth-first order (position k << (3 - d))
// with the joins between them.  Each node's operations and their order are
// the reference's, so the pieces are the same.
// ---------------------------------------------------------------------------
__device__ __forceinline__ SSeg node_seg(const StrokeNode& n) {
    SSeg s;
    s.kind = n.kind;
    for (int j = 0; j < 4; ++j) s.p[j] = SP{n.p[2 * j], n.p[2 * j + 1]};
    return s;
}
__device__ __forceinline__ void put_node(StrokeNode* list, uint32_t* counter, uint32_t t, uint32_t k, int d,
                                         const SSeg& s) {
    StrokeNode& n = list[atomicAdd(counter, 1u)];
    n.t = t;
    n.k = k;
    n.d = d;
    n.kind = s.kind;
    for (int j = 0; j < 4; ++j) {
        n.p[2 * j] = s.p[j].x;
        n.p[2 * j + 1] = s.p[j].y;
    }
}

// Split decision of one node: two children into `out` (depth 3 children go to
// the leaves), or the node itself into the leaves.
__device__ void node_step(const StrokeNodes& N, const StrokeNode& n, StrokeNode* out, uint32_t* out_count) {
    const SSeg c = node_seg(n);
    const bool split = c.kind == 1 ? qsplit_needed(c) : csplit_needed(c);
    if (!split) {
        put_node(N.leaves, N.counters + 2, n.t, n.k, n.d, c);
        return;
    }
    SSeg a = c, b = c;
    const SP* p = c.p;
    if (c.kind == 1) {
        const double t = 0.5, t1 = t, t_1 = ds(1.0, t), t2 = dm(t1, t1), t_2 = dm(t_1, t_1);
        const double w1 = dm(dm(2.0, t1), t_1);
        const SP mid{da(da(dm(t_2, p[0].x), dm(w1, p[1].x)), dm(t2, p[2].x)),
                     da(da(dm(t_2, p[0].y), dm(w1, p[1].y)), dm(t2, p[2].y))};
        a.p[1] = SP{da(dm(t_1, p[0].x), dm(t, p[1].x)), da(dm(t_1, p[0].y), dm(t, p[1].y))};
        a.p[2] = mid;
        b.p[0] = mid;
        b.p[1] = SP{da(dm(t_1, p[1].x), dm(t, p[2].x)), da(dm(t_1, p[1].y), dm(t, p[2].y))};
    } else {
        const SP mid{da(da(da(dm(0.125, p[0].x), dm(0.375, p[1].x)), dm(0.375, p[2].x)), dm(0.125, p[3].x)),
                     da(da(da(dm(0.125, p[0].y), dm(0.375, p[1].y)), dm(0.375, p[2].y)), dm(0.125, p[3].y))};
        a.p[1] = SP{da(dm(0.5, p[0].x), dm(0.5, p[1].x)), da(dm(0.5, p[0].y), dm(0.5, p[1].y))};
        a.p[2] = SP{da(da(dm(0.25, p[0].x), dm(0.5, p[1].x)), dm(0.25, p[2].x)),
                    da(da(dm(0.25, p[0].y), dm(0.5, p[1].y)), dm(0.25, p[2].y))};
        a.p[3] = mid;
        b.p[0] = mid;
        b.p[1] = SP{da(da(dm(0.25, p[1].x), dm(0.5, p[2].x)), dm(0.25, p[3].x)),
                    da(da(dm(0.25, p[1].y), dm(0.5, p[2].y)), dm(0.25, p[3].y))};
        b.p[2] = SP{da(dm(0.5, p[2].x), dm(0.5, p[3].x)), da(dm(0.5, p[2].y), dm(0.5, p[3].y))};
    }
    StrokeNode* dst = n.d + 1 == 3 ? N.leaves : out;
    uint32_t* cnt = n.d + 1 == 3 ? N.counters + 2 : out_count;
    put_node(dst, cnt, n.t, 2 * n.k, n.d + 1, a);
    put_node(dst, cnt, n.t, 2 * n.k + 1, n.d + 1, b);
}

__global__ void k_stroke_roots(StrokeArgs A, StrokeNodes N) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N.n_curves) return;
    const StrokeUnit un = A.units[A.order[t]];
    const SSeg s = load_sseg(A.kind, A.pts, un.seg, un.aux != 0);
    StrokeNode n;
    n.t = t;
    n.k = 0;
    n.d = 0;
    n.kind = s.kind;
    for (int j = 0; j < 4; ++j) {
        n.p[2 * j] = s.p[j].x;
        n.p[2 * j + 1] = s.p[j].y;
    }
    node_step(N, n, N.list[0], N.counters + 0);
}

__global__ void k_stroke_level(StrokeNodes N, int in) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N.counters[in]) return;
    node_step(N, N.list[in][i], N.list[in ^ 1], N.counters + (in ^ 1));
}

// One leaf: polyline_offset of its control polygon (src/curve.rs:1302-1352).
__global__ void k_stroke_leaves(StrokeArgs A, StrokeNodes N) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N.counters[2]) return;
    const StrokeNode& n = N.leaves[i];
    const StrokeUnit un = A.units[A.order[n.t]];
    const double dist = A.styles[un.style].width / 2.0;
    SSeg r = node_seg(n);
    if (!polyoffset(r.p, slast(r.kind) + 1, dist)) return;
    const uint64_t slot = 8ull * n.t + (n.k << (3 - n.d));
    write_piece(N.piece_kind, N.piece_pts, slot, r);
    atomicOr(N.valid + n.t, 1u << (n.k << (3 - n.d)));
}

// One OFFSET unit of the order list: a line's offset, or a curve's pieces in
// order with a Round join between consecutive pieces that do not meet.
__global__ void k_stroke_assemble(StrokeArgs A, StrokeNodes N, bool emit) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A.n_order) return;
    const uint32_t u = A.order[t];
    const StrokeUnit un = A.units[u];
    const double dist = A.styles[un.style].width / 2.0;
    Sink sink{nullptr, emit ? kStrokeOffsetMax : 0, 0};
    if (emit) {
        sink.gkind = A.tmp_kind;
        sink.gpts = A.tmp_pts;
        sink.gbase = A.off_start[u];
    }
    if (t >= N.n_curves) {
        const SSeg s = load_sseg(A.kind, A.pts, un.seg, un.aux != 0);
        SLn l;
        if (loffset(SLn{s.p[0], s.p[1]}, dist, l)) sink.push(sline(l.a, l.b));
    } else {
        bool have_last = false;
        SSeg last{};
        for (uint32_t m = N.valid[t]; m; m &= m - 1u) {
            const SSeg r = read_piece(N.piece_kind, N.piece_pts, 8ull * t + (__ffs(m) - 1));
            if (r.kind == 2 && have_last && !pclose(send(last), sstart(r)))
                sjoin(last, r, dm(dist, 2.0), STROKE_JOIN_ROUND, 0.0, sink);
            sink.push(r);
            have_last = true;
            last = r;
        }
    }
    if (!emit || A.strided) A.counts[u] = (uint32_t)sink.n;
}

// The nearest non-empty OFFSET unit in [lo, hi) from the end (last) or from the start.
__device__ int find_offset(const StrokeArgs& A, uint32_t lo, uint32_t hi, bool last) {
    if (last) {
        for (uint32_t v = hi; v-- > lo;)
            if (A.units[v].type == STROKE_OFFSET && A.counts[v]) return (int)v;
    } else {
        for (uint32_t v = lo; v < hi; ++v)
            if (A.units[v].type == STROKE_OFFSET && A.counts[v]) return (int)v;
    }
    return -1;
}

// JOIN / CAP / CLOSE / CAPEND units (the odd units): counts, or pieces at
// fin_start[u] of the output.  With a join buffer the counting pass keeps the
// pieces and the emitting pass only copies them.
__global__ void k_stroke_joins(StrokeArgs A, bool emit) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t u = 2 * t + 1;
    if (u >= A.n_units) return;
    const StrokeUnit un = A.units[u];
    if (un.type == STROKE_OFFSET) return;
    if (emit && A.join_kind) {
        const uint64_t o = A.fin_start[u];
        for (uint32_t i = 0; i < A.counts[u] && i < 9; ++i) {
            A.out_kind[o + i] = A.join_kind[9ull * t + i];
            for (int j = 0; j < 8; ++j) A.out_pts[8 * (o + i) + j] = A.join_pts[8 * (9ull * t + i) + j];
        }
        return;
    }
    const StrokeStyleDev st = A.styles[un.style];
    // counting: into the join buffer when there is one; emitting: into the outline
    Sink sink{nullptr, 9, 0};
    if (!emit && A.join_kind) {
        sink.gkind = A.join_kind;
        sink.gpts = A.join_pts;
        sink.gbase = 9ull * t;
    } else if (emit) {
        sink.gkind = A.out_kind;
        sink.gpts = A.out_pts;
        sink.gbase = A.fin_start[u];
    } else {
        sink.cap = 0;
    }
    if (un.type == STROKE_JOIN || un.type == STROKE_JOIN_CAP) {
        // joins the last piece before it to the first piece of the OFFSET unit after it
        if (A.counts[u + 1]) {
            const int v = find_offset(A, un.list0, u, true);
            if (v >= 0) {
                const SSeg prev = read_piece(A.tmp_kind, A.tmp_pts, A.off_start[v] + A.counts[v] - 1);
                const SSeg next = read_piece(A.tmp_kind, A.tmp_pts, A.off_start[u + 1]);
                if (un.type == STROKE_JOIN_CAP) scap(prev, next, st.width, st.cap, sink);
                else sjoin(prev, next, st.width, st.join, st.miter, sink);
            }
        }
    } else {
        const int vf = find_offset(A, un.list0, u, false), vl = find_offset(A, un.list0, u, true);
        if (vf >= 0) {
            const SSeg first = read_piece(A.tmp_kind, A.tmp_pts, A.off_start[vf]);
            const SSeg last = read_piece(A.tmp_kind, A.tmp_pts, A.off_start[vl] + A.counts[vl] - 1);
            if (un.type == STROKE_CAPEND) {
                scap(last, first, st.width, st.cap, sink);
            } else {
                // stroke_close (src/path.rs:708-732): the subpath's closing line, offset
                const SP s0 = sstart(load_sseg(A.kind, A.pts, un.seg, false));
                const SP s1 = send(load_sseg(A.kind, A.pts, un.aux, false));
                const SLn close = un.type == STROKE_CLOSE_FWD ? SLn{s1, s0} : SLn{s0, s1};
                SLn off;
                if (loffset(close, st.width / 2.0, off) && dm(plen(psub(off.a, off.b)), 100.0) > st.width) {
                    const SSeg c = sline(off.a, off.b);
                    sjoin(last, c, st.width, st.join, st.miter, sink);
                    sink.push(c);
                    sjoin(c, first, st.width, st.join, st.miter, sink);
                } else {
                    sjoin(last, first, st.width, st.join, st.miter, sink);
                }
            }
        }
    }
    if (!emit) A.counts[u] = (uint32_t)sink.n;
}

// OFFSET units' pieces from the compact buffer to their place in the output.
__global__ void k_stroke_gather(StrokeArgs A) {
    const uint32_t u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= A.n_units || A.units[u].type != STROKE_OFFSET) return;
    const uint64_t src = A.off_start[u], dst = A.fin_start[u];
    for (uint32_t i = 0; i < A.counts[u]; ++i) {
        A.out_kind[dst + i] = A.tmp_kind[src + i];
        for (int j = 0; j < 8; ++j) A.out_pts[8 * (dst + i) + j] = A.tmp_pts[8 * (src + i) + j];
    }
}

// The units of Path::stroke's loop over one subpath of m segments (base b):
// the way out, OFFSET of segment k at b + 2k with a JOIN before it (k > 0);
// then at b + 2m - 1 the turn (CLOSE_FWD of a closed subpath, else the cap
// JOIN); the way back, OFFSET of reversed segment m - 1 - k at b + 2m + 2k
// with a JOIN before it (k > 0); at b + 4m - 1 the end (CLOSE_BWD or CAPEND).
// A closed subpath's way back is a list of its own (it starts at b + 2m).
__global__ void k_stroke_units(const StrokeSub* __restrict__ subs, uint32_t n_subs, StrokeUnit* __restrict__ units,
                               uint64_t n_units) {
    const uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= n_units) return;
    uint32_t lo = 0, hi = n_subs - 1;  // the last subpath whose base is <= u
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (subs[mid].base <= u) lo = mid; else hi = mid - 1;
    }
    const StrokeSub sb = subs[lo];
    const uint64_t b = sb.base;
    const uint32_t m = sb.m, i = (uint32_t)(u - b);
    StrokeUnit un;
    un.style = sb.style;
    un.seg = un.aux = 0;
    if (i < 2 * m - 1) {  // the way out
        un.list0 = (uint32_t)b;
        if (i & 1u) {
            un.type = STROKE_JOIN;
        } else {
            un.type = STROKE_OFFSET;
            un.seg = sb.s0 + i / 2;
        }
    } else if (i == 2 * m - 1) {
        un.list0 = (uint32_t)b;
        if (sb.closed) {
            un.type = STROKE_CLOSE_FWD;
            un.seg = sb.s0;
            un.aux = sb.s0 + m - 1;
        } else {
            un.type = STROKE_JOIN_CAP;
        }
    } else if (i < 4 * m - 1) {  // the way back
        un.list0 = (uint32_t)(sb.closed ? b + 2 * m : b);
        const uint32_t k = i - 2 * m;
        if (k & 1u) {
            un.type = STROKE_JOIN;
        } else {
            un.type = STROKE_OFFSET;
            un.seg = sb.s0 + m - 1 - k / 2;
            un.aux = 1;
        }
    } else {
        un.list0 = (uint32_t)(sb.closed ? b + 2 * m : b);
        if (sb.closed) {
            un.type = STROKE_CLOSE_BWD;
            un.seg = sb.s0;
            un.aux = sb.s0 + m - 1;
        } else {
            un.type = STROKE_CAPEND;
        }
    }
    units[u] = un;
}

cudaError_t launch_stroke_units(const StrokeSub* subs, uint32_t n_subs, StrokeUnit* units, uint64_t n_units,
                                cudaStream_t st) {
    if (n_units == 0 || n_subs == 0) return cudaSuccess;
    k_stroke_units<<<(unsigned)((n_units + 255) / 256), 256, 0, st>>>(subs, n_subs, units, n_units);
    return cudaGetLastError();
}

cudaError_t launch_stroke_nodes(const StrokeArgs& A, const StrokeNodes& N, cudaStream_t st) {
    const uint32_t n = N.n_curves;
    if (n == 0) return cudaSuccess;
    k_stroke_roots<<<(n + 127) / 128, 128, 0, st>>>(A, N);
    k_stroke_level<<<(2 * n + 127) / 128, 128, 0, st>>>(N, 0);  // depth 1 -> depth 2 nodes in list[1]
    k_stroke_level<<<(4 * n + 127) / 128, 128, 0, st>>>(N, 1);  // depth 2 -> depth 3, all leaves
    k_stroke_leaves<<<(8 * n + 127) / 128, 128, 0, st>>>(A, N);
    return cudaGetLastError();
}

cudaError_t launch_stroke_assemble(const StrokeArgs& A, const StrokeNodes& N, bool emit, cudaStream_t st) {
    if (A.n_order == 0) return cudaSuccess;
    k_stroke_assemble<<<(A.n_order + 127) / 128, 128, 0, st>>>(A, N, emit);
    return cudaGetLastError();
}

cudaError_t launch_stroke(const StrokeArgs& A, int phase, cudaStream_t st) {
    if (A.n_units == 0) return cudaSuccess;
    const unsigned grid = (A.n_units + 127) / 128;
    const unsigned grid_odd = (A.n_units / 2 + 127) / 128;  // the non-OFFSET units are the odd ones
    switch (phase) {
        case 2: if (grid_odd) k_stroke_joins<<<grid_odd, 128, 0, st>>>(A, false); break;
        case 3: if (grid_odd) k_stroke_joins<<<grid_odd, 128, 0, st>>>(A, true); break;
        case 4: k_stroke_gather<<<grid, 128, 0, st>>>(A); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace rz
