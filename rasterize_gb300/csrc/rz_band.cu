// rz_band.cu -- the persistent band kernel: flatten + signed-area coverage +
// row prefix + fill rule for many independent paths in one launch.
//
// Work items are (path, band of rows); a CTA pulls items from a device queue
// (an atomic head counter), so thousands of uneven paths balance across the
// 152 SMs.  Per item the CTA clears a shared-memory accumulation band
// (rows x (clip_width + 3) words), every thread walks the bisection trees of
// a strided subset of the path's segments (skipping segments whose control
// hull misses the band), accumulates signed area differences with shared
// int32 fixed-point atomics, and finally one warp per row runs an exact
// integer prefix scan, applies the fill rule and streams the row to HBM with
// float4 stores.
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
struct SlotCoef {
    FlatCoef c;
    float qerr;
};

// Band-kernel decision: coefficients cached per segment slot.
__device__ __forceinline__ int decide_slot(const BatchDev& b, const SegRec& r, const SlotCoef& sc, int d, uint32_t k,
                                           const double* trm, int& fallbacks) {
    return decide_node(r, sc.c, sc.qerr, d, k, b.thr32, b.thr64, b.pts, trm, fallbacks);
}

constexpr int kSmemBytes = kBandBytes + kThreads * (int)sizeof(SegRec) + kThreads * (int)sizeof(SlotCoef) +
                           kLeafCap * (int)sizeof(LeafCode) + 2 * kLevelCap * (int)sizeof(uint32_t);



__device__ inline void drain_leaf(const Band& B, const SegRec* recs, const LeafCode c) {
    const SegRec& r = recs[c.slot];
    accumulate_vtx(B, rec_vtx(r, c.k, c.d, B.y0), rec_vtx(r, c.k + 1u, c.d, B.y0));
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

// Records of segments [seg_lo, seg_lo + n_seg) and of the closing lines of
// subpaths [sub_lo, sub_lo + n_sub).
__global__ void __launch_bounds__(256) k_band_records(BatchDev b, SlotRec* __restrict__ out, uint32_t seg_lo,
                                                      uint32_t n_seg, uint32_t sub_lo, uint32_t n_sub) {
    const uint32_t t = blockIdx.x * 256u + threadIdx.x;
    if ((uint64_t)t >= (uint64_t)n_seg + n_sub) return;
    const bool closing = t >= n_seg;
    const uint32_t idx = closing ? sub_lo + (t - n_seg) : seg_lo + t;
    const uint32_t j = closing ? b.n_segments + idx : idx;
    uint32_t owner = kAnyPath;
    const double* trm = nullptr;
    if (b.tr && b.n_paths) {
        const uint32_t sub = closing ? idx : last_le(b.sub_off, b.n_subpaths + 1, idx);
        owner = min(last_le(b.path_sub, b.n_paths + 1, sub), b.n_paths - 1);
        trm = b.tr + 6ull * owner;
    }
    SlotRec r;
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
    out[j] = r;
}

// Slot i of a work item from its record: 1 when the record is taken (its hull
// meets the band), 0 when the slot adds nothing to the band, -1 when the slot
// must go through band_load.
__device__ __forceinline__ int band_take(const BatchDev& b, const Band& B, uint32_t path, uint32_t seg0,
                                         uint32_t n_seg, uint32_t sub0, uint32_t i, SegRec& rec, SlotCoef& coef) {
    const uint32_t ri = i < n_seg ? seg0 + i : b.n_segments + sub0 + (i - n_seg);
    const int4* q = reinterpret_cast<const int4*>(b.recs + ri);
    const int4 c0 = __ldg(q), c1 = __ldg(q + 1), c2 = __ldg(q + 2), c3 = __ldg(q + 3), c4 = __ldg(q + 4),
               c5 = __ldg(q + 5);
    const uint32_t tag = (uint32_t)c3.w, owner = tag & kAnyPath, state = tag >> 30;
    if ((owner != kAnyPath && owner != path) || state == REC_SLOW) return -1;
    if (state != REC_FIX) return 0;
    const int32_t oy = B.y0 << 16;  // the test of hull_meets_rows
    if (c5.w < oy - 65536 || c5.z > oy + ((B.bh + 1) << 16)) return 0;
    int* r = reinterpret_cast<int*>(&rec);
    r[0] = c0.x; r[1] = c0.y; r[2] = c0.z; r[3] = c0.w;
    r[4] = c1.x; r[5] = c1.y; r[6] = c1.z; r[7] = c1.w;
    r[8] = c2.x; r[9] = c2.y; r[10] = c2.z; r[11] = c2.w;
    r[12] = c3.x; r[13] = c3.y; r[14] = c3.z;
    int* c = reinterpret_cast<int*>(&coef);
    c[0] = c4.x; c[1] = c4.y; c[2] = c4.z; c[3] = c4.w;
    c[4] = c5.x; c[5] = c5.y;
    return 1;
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
    __shared__ int s_task;  // next subtree to walk (threads that finish early take the next one)
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
            if (i < n_seg + n_close) {
                const int t = b.recs ? band_take(b, B, wi.path, seg0, n_seg, sub0, i, recs[tid], coefs[tid]) : -1;
                active = t > 0 || (t < 0 && band_load(b, B, seg0, n_seg, sub0, i, trm, recs[tid], coefs[tid],
                                                      fallbacks));
            }
            // ---- breadth-first over the top levels of every tree, all threads together
            if (tid == 0) { s_nlevel[0] = 0; s_nlevel[1] = 0; s_task = kThreads; }
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
                    if (decide_slot(b, recs[slot], coefs[slot], d, k, trm, fallbacks)) {
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
            // ---- the remaining subtrees (roots at depth kSpreadDepth) walked serially, handed out to threads
            //      as they finish (subtree sizes vary widely)
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
                    const int leaf = decide_slot(b, recs[slot], coefs[slot], W.d, W.k, trm, fallbacks);
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
                        task = atomicAdd(&s_task, 1);
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
        if (b.flat_out && m.row_stride == m.width) {
            // staged in shared memory, then one contiguous span per band
            band_scan<kThreads>(B, m.width, rule, SmemStore{acc, B.stride});
            __syncthreads();
            band_flush<kThreads>(acc, B.stride, B.bh, m.width, b.out + m.offset + (uint64_t)B.y0 * (uint64_t)m.width);
        } else {
            MaskStore st{b.out, m.offset, (int64_t)m.row_stride, B.y0, m.width};
            band_scan<kThreads>(B, m.width, rule, st);
        }
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
uint64_t band_record_bytes() { return sizeof(SlotRec); }

// Records of segments [seg_lo, seg_hi) and closing lines of subpaths [sub_lo, sub_hi).
cudaError_t launch_band_records(const BatchDev& b, uint32_t seg_lo, uint32_t seg_hi, uint32_t sub_lo, uint32_t sub_hi,
                                cudaStream_t stream) {
    seg_hi = min(seg_hi, b.n_segments);
    sub_hi = min(sub_hi, b.n_subpaths);
    const uint32_t n_seg = seg_hi > seg_lo ? seg_hi - seg_lo : 0, n_sub = sub_hi > sub_lo ? sub_hi - sub_lo : 0;
    const uint64_t n = (uint64_t)n_seg + n_sub;
    if (n == 0 || !b.recs) return cudaSuccess;
    k_band_records<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(b, const_cast<SlotRec*>(b.recs), seg_lo, n_seg,
                                                                     sub_lo, n_sub);
    return cudaGetLastError();
}

cudaError_t launch_band_records(const BatchDev& b, cudaStream_t stream) {
    return launch_band_records(b, 0, b.n_segments, 0, b.n_subpaths, stream);
}
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
