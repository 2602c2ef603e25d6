// rz_glyph.cu -- the glyph pipeline: many small paths, each into its own mask.
//
// Separate kernels for the separate kinds of work of a batch, so that each
// runs at full occupancy without block barriers between unlike phases:
//
//   k_glyph_records  one thread per flatten slot (segments, then one closing
//                    line per subpath, src/path.rs:776-786): the slot's
//                    fixed-point record and decision coefficients.
//   k_glyph_walk     the reference's exact bisection tree of every slot
//                    (src/path.rs:734-796), FP32 decisions with binary64
//                    replays; each lane walks several slots in one flat loop.
//                    Writes the number of vertices of the slot's line chain
//                    (leaves + 1) and the tree's shape as a pre-order bit code.
//   (scan)           exclusive prefix of the chain lengths: vertex offsets.
//   k_glyph_emit     a block of slots expands its tree codes into shared
//                    memory, then evaluates one vertex per thread (an integer
//                    pixel plus FP32 fractions) and stores the block's chains
//                    contiguously.
//   k_glyph_cover    persistent CTAs pull (path, band of rows) items from a
//                    queue: every line of the path that reaches the band adds
//                    its exact signed area to an int32 band in shared memory
//                    (src/rasterize.rs:365-470), then one warp per row scans,
//                    applies the fill rule (src/rasterize.rs:473-507), streams
//                    the row out and clears the band behind it.  Two barriers
//                    per item.
//
// Vertices are a function of their parameter t only (rec_vtx), so a vertex
// shared by two lines is one value and windings telescope exactly; the
// coverage arithmetic is the band kernel's (rz_band.cu), so both kernels
// render the same masks.  Slots the fixed-point route cannot take (raw arcs
// of device-memory batches, coordinates beyond 16.16) have empty chains;
// their paths are flagged and k_glyph_cover walks those slots per band in
// binary64, as the band kernel does.
#include "rz_glyph.cuh"
#include "rz_slots.cuh"

namespace rz {

// Bit i of a tree code: node i of the pre-order walk splits (1) or is a leaf
// (0).  A tree of more than 64 nodes (33 leaves or more) is marked long and
// walked again with its decisions by the emit pass.
constexpr unsigned long long kCodeLong = ~0ull;  // never a valid code: the last node of a walk is a leaf

// The end flag of a chain's last vertex lives in the row word: rows are
// within +-16384, so row + 2^30 cannot be mistaken for a row.
constexpr int32_t kChainEnd = 1 << 30;

__device__ __forceinline__ int4 pack_vtx(const VtxQ& v, bool end) {
    return make_int4(v.col, v.row + (end ? kChainEnd : 0), __float_as_int(v.fx), __float_as_int(v.fy));
}

__device__ __forceinline__ bool vtx_end(const int4& w) { return w.y >= (kChainEnd >> 1); }

// The vertex of a packed word with its row relative to band row y0.
__device__ __forceinline__ VtxQ unpack_vtx(const int4& w, int y0) {
    VtxQ v;
    v.col = w.x;
    v.row = (w.y >= (kChainEnd >> 1) ? w.y - kChainEnd : w.y) - y0;
    v.fx = __int_as_float(w.z);
    v.fy = __int_as_float(w.w);
    return v;
}

// Owning path of slot j (non-decreasing offsets: every slot in one path).
__device__ __forceinline__ uint32_t slot_path(const BatchDev& b, uint32_t j) {
    const uint32_t sub = j >= b.n_segments ? j - b.n_segments : last_le(b.sub_off, b.n_subpaths + 1, j);
    return min(last_le(b.path_sub, b.n_paths + 1, sub), b.n_paths - 1);
}

__device__ __forceinline__ FlatCoef flat_of(const GlyphCoef& c) {
    FlatCoef f;
    f.a2x = c.a2x;
    f.a2y = c.a2y;
    f.a3x = c.a3x;
    f.a3y = c.a3y;
    f.mag = c.mag;
    return f;
}

__global__ void __launch_bounds__(256) k_glyph_records(GlyphDev g) {
    const uint32_t j = blockIdx.x * 256u + threadIdx.x;
    const BatchDev& b = g.b;
    const uint32_t n = b.n_segments + b.n_subpaths;
    if (j >= n) return;
    SlotRec r;
    const int kind = build_slot_record(b, j, r);
    GlyphRec out;
    out.rec = r.rec;
    out.tag = r.tag;
    g.recs[j] = out;
    GlyphCoef c;
    c.a2x = r.coef.c.a2x;
    c.a2y = r.coef.c.a2y;
    c.a3x = r.coef.c.a3x;
    c.a3y = r.coef.c.a3y;
    c.mag = r.coef.c.mag;
    c.qerr = r.coef.qerr;
    g.coefs[j] = c;
    if ((r.tag >> 30) == REC_SLOW) {
        if (kind == SLOT_NAN) set_err(b.err, ERR_NAN);  // the reference panics on NaN (src/path.rs:765-767)
        if (b.n_paths) atomicOr(&g.path_flags[slot_path(b, j)], 1u);
    }
}

// Each lane walks the trees of g.walk_slots slots one after the other in one
// flat loop (a lane that finishes a tree starts its next slot while the other
// lanes keep deciding), so the warp's lanes stay busy however uneven the
// trees.  The next slot's record is loaded while the current tree is walked.
// The number of slots per lane (segments per warp / 32) is tuned per batch.

__global__ void __launch_bounds__(256) k_glyph_walk(GlyphDev g) {
    const BatchDev& b = g.b;
    const uint32_t n = b.n_segments + b.n_subpaths;
    const uint32_t warp = (blockIdx.x * 256u + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    const int per_lane = g.walk_slots;
    const uint32_t first = warp * 32u * (uint32_t)per_lane + lane;
    int fallbacks = 0;
    int s = 0;            // index in the lane's list of the slot held in `next`
    uint32_t j = 0;       // slot being walked
    bool walking = false;
    SegRec rec, nrec;
    GlyphCoef nc{};
    uint32_t ntag = REC_EMPTY << 30;
    FlatCoef fc;
    float qerr = 0.f;
    const double* trm = nullptr;
    int d = 0, pos = 0;
    uint32_t k = 0, leaves = 0;
    unsigned long long code = 0;
    if (first < n) {
        const GlyphRec gr = g.recs[first];
        nrec = gr.rec;
        ntag = gr.tag;
        nc = g.coefs[first];
    }
    for (;;) {
        if (!walking) {
            // take the prefetched slot and prefetch the one after it; slots that are not fixed-point
            // records have empty chains
            for (;;) {
                if (s >= per_lane) break;
                j = first + 32u * (uint32_t)s;
                if (j >= n) {
                    s = per_lane;
                    break;
                }
                const uint32_t tag = ntag;
                rec = nrec;
                const GlyphCoef c = nc;
                ++s;
                const uint32_t jn = first + 32u * (uint32_t)s;
                if (s < per_lane && jn < n) {
                    const GlyphRec gr = g.recs[jn];
                    nrec = gr.rec;
                    ntag = gr.tag;
                    nc = g.coefs[jn];
                }
                if ((tag >> 30) == REC_FIX) {
                    fc = flat_of(c);
                    qerr = c.qerr;
                    const uint32_t owner = tag & kAnyPath;
                    trm = (b.tr && owner != kAnyPath) ? b.tr + 6ull * owner : nullptr;
                    walking = true;
                    d = 0;
                    k = 0;
                    pos = 0;
                    leaves = 0;
                    code = 0;
                    break;
                }
                g.chain[j] = 0;
                g.code[j] = 0;
            }
            if (!walking) break;
        }
        const int leaf = decide_node(rec, fc, qerr, d, k, b.thr32, b.thr64, b.pts, trm, fallbacks);
        if (pos < 64) code |= (unsigned long long)(leaf ^ 1) << pos;
        ++pos;
        bool done = false;
        if (!leaf) {
            if (d >= MAX_DEPTH) {
                set_err(b.err, ERR_DEPTH);
                leaves = 0;
                done = true;
            } else {
                ++d;
                k <<= 1;
            }
        } else {
            ++leaves;
            // next node after a leaf: climb over the trailing right children, then the right sibling
            const int up = min(__ffs(~k) - 1, d);
            k >>= up;
            d -= up;
            if (d == 0) done = true;
            else k += 1u;
        }
        if (done) {
            g.chain[j] = leaves ? leaves + 1 : 0;
            g.code[j] = pos > 64 ? kCodeLong : code;
            walking = false;
        }
    }
    if (fallbacks) atomicAdd(&b.counters[1], fallbacks);
}

// Chain vertices of a block of 256 slots: vertex parameters are expanded
// from the tree codes into shared memory (one thread per slot), then
// evaluated one vertex per thread and stored contiguously (the block's chains
// are one range of the vertex buffer).  Vertices beyond the staging capacity
// are evaluated by their slot's thread.
constexpr int kEmitStage = 3584;

struct EmitCode {
    uint32_t slot_end;  // local slot | end flag << 8 | depth << 9
    uint32_t j;         // vertex parameter t = j / 2^depth
};

__device__ __forceinline__ void emit_vertex(const GlyphDev& g, const SegRec& r, uint32_t v, uint32_t j, int d,
                                            bool end) {
    if (v < g.vtx_cap) g.vtx[v] = pack_vtx(rec_vtx(r, j, d, 0), end);
}

// Vertex parameters of one slot's chain in order: (0, 0), then the right end
// of every leaf; `put(j, d)` per vertex until `v1 - v0` vertices.
template <class Put>
__device__ __forceinline__ void chain_params(const GlyphDev& g, uint32_t slot, const SegRec& r, uint32_t tag,
                                             unsigned long long code, uint32_t count, Put& put) {
    uint32_t done = 1;
    put(0u, 0);
    if (code != kCodeLong) {
        int d = 0, pos = 0;
        uint32_t k = 0;
        while (done < count) {
            if ((code >> pos) & 1ull) {  // split: the left child is next
                ++pos;
                ++d;
                k <<= 1;
                continue;
            }
            ++pos;
            put(k + 1u, d);
            ++done;
            const int up = min(__ffs(~k) - 1, d);
            k >>= up;
            d -= up;
            if (d == 0) break;
            k += 1u;
        }
    } else {
        // more than 64 nodes: the walk again, with its decisions
        const BatchDev& b = g.b;
        const GlyphCoef c = g.coefs[slot];
        const FlatCoef fc = flat_of(c);
        const uint32_t owner = tag & kAnyPath;
        const double* trm = (b.tr && owner != kAnyPath) ? b.tr + 6ull * owner : nullptr;
        int fallbacks = 0;
        TreeWalk w;
        w.start();
        while (!w.done && done < count) {
            if (!decide_node(r, fc, c.qerr, w.d, w.k, b.thr32, b.thr64, b.pts, trm, fallbacks)) {
                if (w.d >= MAX_DEPTH) break;  // the walk pass reported it
                ++w.d;
                w.k <<= 1;
                continue;
            }
            put(w.k + 1u, w.d);
            ++done;
            w.next_after_leaf();
        }
    }
}

__global__ void __launch_bounds__(256) k_glyph_emit(GlyphDev g) {
    __shared__ GlyphRec s_rec[256];
    __shared__ EmitCode s_code[kEmitStage];
    const BatchDev& b = g.b;
    const uint32_t n = b.n_segments + b.n_subpaths;
    const uint32_t j0 = blockIdx.x * 256u;
    const uint32_t j = j0 + threadIdx.x;
    const uint32_t base = g.chain[j0];
    const uint32_t top = g.chain[min(j0 + 256u, n)];
    uint32_t v0 = 0, v1 = 0;
    unsigned long long code = 0;
    if (j < n) {
        v0 = g.chain[j];
        v1 = g.chain[j + 1];
        if (v1 > v0) {
            if (v1 > g.vtx_cap) {
                set_err(b.err, ERR_CAPACITY);  // the geometry grew since the buffer was sized
                v1 = v0;
            } else {
                s_rec[threadIdx.x] = g.recs[j];
                code = g.code[j];
            }
        }
    }
    const SegRec& r = s_rec[threadIdx.x].rec;
    // 1) vertex parameters in chain order, staged
    if (v1 > v0) {
        uint32_t v = v0;
        auto put = [&](uint32_t jj, int dd) {
            const uint32_t at = v - base;
            if (at < (uint32_t)kEmitStage)
                s_code[at] = EmitCode{threadIdx.x | (v + 1 == v1 ? 256u : 0u) | ((uint32_t)dd << 9), jj};
            ++v;
        };
        chain_params(g, j, r, s_rec[threadIdx.x].tag, code, v1 - v0, put);
    }
    __syncthreads();
    // 2) one vertex per thread, stored contiguously
    const uint32_t staged = min(top > base ? top - base : 0u, (uint32_t)kEmitStage);
    for (uint32_t i = threadIdx.x; i < staged; i += 256u) {
        const EmitCode e = s_code[i];
        emit_vertex(g, s_rec[e.slot_end & 255u].rec, base + i, e.j, (int)(e.slot_end >> 9), (e.slot_end & 256u) != 0);
    }
    // 3) the rest of a block with more vertices than the stage holds, by the slots' own threads
    if (v1 > v0 && v1 - base > (uint32_t)kEmitStage) {
        const uint32_t from = max(v0, base + (uint32_t)kEmitStage);
        uint32_t v = v0;
        auto put = [&](uint32_t jj, int dd) {
            if (v >= from) emit_vertex(g, r, v, jj, dd, v + 1 == v1);
            ++v;
        };
        chain_params(g, j, r, s_rec[threadIdx.x].tag, code, v1 - v0, put);
    }
}

constexpr int kCoverThreads = 256;

// What a cover work item needs of its path, gathered once per launch by
// k_glyph_paths so an item starts with two loads instead of a chain of five.
struct __align__(16) GlyphPath {
    uint32_t vs0, vs1;    // vertex range of the segments' chains
    uint32_t vc0, vc1;    // vertex range of the closing lines' chains
    uint32_t seg0, seg1;  // segment range (the binary64 slow path)
    uint32_t sub0, sub1;  // subpath range
    uint32_t flags;       // bit 0: slots the fixed-point route cannot take; bits 8-15: fill rule
    uint32_t pad[3];
};

__global__ void __launch_bounds__(256) k_glyph_paths(GlyphDev g, GlyphPath* __restrict__ out) {
    const uint32_t p = blockIdx.x * 256u + threadIdx.x;
    const BatchDev& b = g.b;
    if (p >= b.n_paths) return;
    // ranges are clamped to the arrays so malformed offsets cannot read out of bounds
    const uint32_t sub1 = min(b.path_sub[p + 1], b.n_subpaths);
    const uint32_t sub0 = min(b.path_sub[p], sub1);
    const uint32_t seg1 = min(b.sub_off[sub1], b.n_segments);
    const uint32_t seg0 = min(b.sub_off[sub0], seg1);
    GlyphPath q;
    q.vs0 = min(g.chain[seg0], g.vtx_cap);
    q.vs1 = min(g.chain[seg1], g.vtx_cap);
    q.vc0 = min(g.chain[b.n_segments + sub0], g.vtx_cap);
    q.vc1 = min(g.chain[b.n_segments + sub1], g.vtx_cap);
    q.seg0 = seg0;
    q.seg1 = seg1;
    q.sub0 = sub0;
    q.sub1 = sub1;
    q.flags = (g.path_flags[p] & 1u) | ((uint32_t)(b.rule ? b.rule[p] : 0) << 8);
    q.pad[0] = q.pad[1] = q.pad[2] = 0;
    out[p] = q;
}

template <bool FLAT, int RULE>
__device__ __forceinline__ void cover_finish(const Band& B, const MaskDev& m, float* out, float* acc) {
    if (!FLAT) {
        band_scan8<kCoverThreads, RULE>(B, m.width, out + m.offset, (int64_t)m.row_stride, B.y0);
    } else {
        // page-locked host output: staged in shared memory, then one contiguous span per band
        band_scan<kCoverThreads>(B, m.width, RULE, SmemStore{acc, B.stride});
        __syncthreads();
        band_flush<kCoverThreads>(acc, B.stride, B.bh, m.width, out + m.offset + (uint64_t)B.y0 * (uint64_t)m.width);
        __syncthreads();
        const int n4 = (B.bh * B.stride) >> 2;
        for (int i = threadIdx.x; i < n4; i += kCoverThreads)
            reinterpret_cast<float4*>(acc)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

// Lines of vertex range [v0, v1) that reach the band.  A vertex's row word
// is the row of its anchor; the FP32 fraction can reach several rows beyond
// it, so the test uses floor(row + fy).  Each thread takes kLineBatch lines
// a step and issues all their loads before it uses any.
#ifndef RZ_COVER_BATCH
#define RZ_COVER_BATCH 1
#endif
#ifndef RZ_COVER_MIN_BLOCKS
#define RZ_COVER_MIN_BLOCKS 4
#endif
constexpr int kLineBatch = RZ_COVER_BATCH;

// Line from packed vertices a -> c: false when it needs the binary64 route.
__device__ __forceinline__ bool cover_line(const Band& B, const int4& a, const int4& c) {
    if (vtx_end(a)) return true;
    const VtxQ va = unpack_vtx(a, 0), vc = unpack_vtx(c, 0);
    const int ra = va.row + __float2int_rd(va.fy), rc = vc.row + __float2int_rd(vc.fy);
    if (max(ra, rc) < B.y0 - 1 || min(ra, rc) > B.y0 + B.bh) return true;
    return accumulate_vtx_short(B, unpack_vtx(a, B.y0), unpack_vtx(c, B.y0));
}

// The lines of vertex range [v0, v1); those that need the binary64 route are
// taken after the loop, so the loop holds no call and its loads can batch.
__device__ __forceinline__ void cover_range(const GlyphDev& g, const Band& B, uint32_t v0, uint32_t v1) {
    if (v1 <= v0 + 1) return;
    const uint32_t n = v1 - 1 - v0;  // line i runs from vertex v0 + i to v0 + i + 1
    uint32_t slow = 0;               // bit q: line i0 + q * kCoverThreads of the current step
    for (uint32_t i0 = threadIdx.x; i0 < n; i0 += kCoverThreads * kLineBatch) {
        int4 a[kLineBatch], c[kLineBatch];
        #pragma unroll
        for (int q = 0; q < kLineBatch; ++q) {
            const uint32_t i = i0 + q * kCoverThreads;
            if (i < n) {
                a[q] = g.vtx[v0 + i];
                c[q] = g.vtx[v0 + i + 1];
            }
        }
        #pragma unroll
        for (int q = 0; q < kLineBatch; ++q)
            if (i0 + q * kCoverThreads < n && !cover_line(B, a[q], c[q])) slow |= 1u << q;
        if (slow) {
            for (int q = 0; q < kLineBatch; ++q) {
                if (!((slow >> q) & 1u)) continue;
                const uint32_t i = i0 + q * kCoverThreads;
                accumulate_vtx(B, unpack_vtx(g.vtx[v0 + i], B.y0), unpack_vtx(g.vtx[v0 + i + 1], B.y0));
            }
            slow = 0;
        }
    }
}

// The item a CTA works on, staged in shared memory: the next one is fetched
// by thread 0 while the block works on the current one.
struct CoverItem {
    WorkItem wi;
    int32_t valid;
    int32_t pad;
    MaskDev m;
    GlyphPath p;
};

__device__ __forceinline__ void fetch_item(const GlyphDev& g, const WorkItem* items, int n_items, int32_t* queue,
                                           const GlyphPath* paths, CoverItem& dst) {
    const int it = atomicAdd(queue, 1);
    if (it >= n_items) {
        dst.valid = 0;
        return;
    }
    const WorkItem wi = items[it];
    dst.wi = wi;
    dst.m = g.b.masks[wi.path];
    dst.p = paths[wi.path];
    dst.valid = 1;
}

template <bool FLAT>
__global__ void __launch_bounds__(kCoverThreads, RZ_COVER_MIN_BLOCKS) k_glyph_cover(GlyphDev g, const GlyphPath* __restrict__ paths,
                                                                 const WorkItem* __restrict__ items, int n_items,
                                                                 int32_t* queue) {
    extern __shared__ float4 smg4[];
    float* acc = reinterpret_cast<float*>(smg4);
    __shared__ CoverItem s_it[2];
    const BatchDev& b = g.b;
    for (int i = threadIdx.x; i < kGlyphBandFloats / 4; i += kCoverThreads) smg4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (threadIdx.x == 0) fetch_item(g, items, n_items, queue, paths, s_it[0]);
    __syncthreads();
    int fallbacks = 0;
    for (int cur = 0;; cur ^= 1) {
        const CoverItem& ci = s_it[cur];
        if (!ci.valid) break;
        const WorkItem wi = ci.wi;
        const MaskDev m = ci.m;
        const GlyphPath q = ci.p;
        // the next item's loads overlap this item's work
        if (threadIdx.x == 0) fetch_item(g, items, n_items, queue, paths, s_it[cur ^ 1]);
        Band B;
        B.acc = acc;
        B.stride = band_stride(m.clip_width);
        B.bh = wi.rows;
        B.y0 = wi.y0;
        B.img_h = m.height;
        B.width_f = (float)m.clip_width;
        B.width_i = m.clip_width;
        cover_range(g, B, q.vs0, q.vs1);
        cover_range(g, B, q.vc0, q.vc1);
        if (q.flags & 1u) {
            // slots of this path the fixed-point route cannot take: binary64 per band
            const uint32_t n_seg = q.seg1 - q.seg0, n_close = q.sub1 - q.sub0;
            const double* trm = b.tr ? b.tr + 6ull * wi.path : nullptr;
            for (uint32_t i = threadIdx.x; i < n_seg + n_close; i += kCoverThreads) {
                const uint32_t j = i < n_seg ? q.seg0 + i : b.n_segments + q.sub0 + (i - n_seg);
                if ((g.recs[j].tag >> 30) != REC_SLOW) continue;
                SegRec rec;
                SlotCoef coef;
                band_load(b, B, q.seg0, n_seg, q.sub0, i, trm, rec, coef, fallbacks);  // never a fixed-point slot here
            }
        }
        __syncthreads();
        if ((q.flags >> 8) & 1u) cover_finish<FLAT, 1>(B, m, b.out, acc);
        else cover_finish<FLAT, 0>(B, m, b.out, acc);
        __syncthreads();  // the band is clear and the next item is staged
    }
    if (fallbacks) atomicAdd(&b.counters[1], fallbacks);
}

// ---------------------------------------------------------------------------
// Host-callable launchers
// ---------------------------------------------------------------------------
cudaError_t init_glyph_kernels() {
    cudaError_t e = cudaFuncSetAttribute(k_glyph_cover<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         kGlyphBandBytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_glyph_cover<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGlyphBandBytes);
    return e;
}

int glyph_cover_occupancy() {
    int blocks = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_glyph_cover<false>, kCoverThreads, kGlyphBandBytes);
    return blocks;
}

uint64_t glyph_path_bytes() { return sizeof(GlyphPath); }

// Records and tree walks of every slot.
cudaError_t launch_glyph_walk(const GlyphDev& g, cudaStream_t st) {
    const uint64_t n = (uint64_t)g.b.n_segments + g.b.n_subpaths;
    if (n == 0) return cudaSuccess;
    k_glyph_records<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(g);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const uint64_t per_block = 256ull * (uint64_t)g.walk_slots;
    k_glyph_walk<<<(unsigned)((n + per_block - 1) / per_block), 256, 0, st>>>(g);
    return cudaGetLastError();
}

// Chain vertices, then the per-path descriptors of the cover items.
cudaError_t launch_glyph_emit(const GlyphDev& g, cudaStream_t st) {
    const uint64_t n = (uint64_t)g.b.n_segments + g.b.n_subpaths;
    if (n) {
        k_glyph_emit<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(g);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (g.b.n_paths && g.paths) {
        k_glyph_paths<<<(g.b.n_paths + 255) / 256, 256, 0, st>>>(g, reinterpret_cast<GlyphPath*>(g.paths));
        return cudaGetLastError();
    }
    return cudaSuccess;
}

cudaError_t launch_glyph_cover(const GlyphDev& g, const WorkItem* items, int n_items, int32_t* queue, int grid,
                               cudaStream_t st) {
    if (n_items <= 0) return cudaSuccess;
    const GlyphPath* paths = reinterpret_cast<const GlyphPath*>(g.paths);
    if (g.b.flat_out)
        k_glyph_cover<true><<<grid, kCoverThreads, kGlyphBandBytes, st>>>(g, paths, items, n_items, queue);
    else
        k_glyph_cover<false><<<grid, kCoverThreads, kGlyphBandBytes, st>>>(g, paths, items, n_items, queue);
    return cudaGetLastError();
}

}  // namespace rz
