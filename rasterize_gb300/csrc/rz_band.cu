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
#include "rz_slots.cuh"

namespace rz {


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


constexpr int kSmemBytes = kBandBytes + kThreads * (int)sizeof(SegRec) + kThreads * (int)sizeof(SlotCoef) +
                           kLeafCap * (int)sizeof(LeafCode) + 2 * kLevelCap * (int)sizeof(uint32_t);



__device__ inline void drain_leaf(const Band& B, const SegRec* recs, const LeafCode c) {
    const SegRec& r = recs[c.slot];
    accumulate_vtx(B, rec_vtx(r, c.k, c.d, B.y0), rec_vtx(r, c.k + 1u, c.d, B.y0));
}

// Records of segments [seg_lo, seg_lo + n_seg) and of the closing lines of
// subpaths [sub_lo, sub_lo + n_sub).
__global__ void __launch_bounds__(256) k_band_records(BatchDev b, SlotRec* __restrict__ out, uint32_t seg_lo,
                                                      uint32_t n_seg, uint32_t sub_lo, uint32_t n_sub) {
    const uint32_t t = blockIdx.x * 256u + threadIdx.x;
    if ((uint64_t)t >= (uint64_t)n_seg + n_sub) return;
    const bool closing = t >= n_seg;
    const uint32_t j = closing ? b.n_segments + sub_lo + (t - n_seg) : seg_lo + t;
    SlotRec r;
    build_slot_record(b, j, r);
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
