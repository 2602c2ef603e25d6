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

// Flattens one reference segment (already transformed) into the band.
__device__ void band_segment(const BatchDev& b, const Band& B, const Seg64& s, int& fallbacks) {
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

// queue != nullptr: persistent CTAs pull items from the queue head;
// queue == nullptr: one item per CTA (item = blockIdx.x), the plain launch.
template <int THREADS>
__global__ void __launch_bounds__(THREADS) k_mask_bands(BatchDev b, const WorkItem* __restrict__ items,
                                                        int n_items, int32_t* queue) {
    extern __shared__ float4 smem4[];
    float* acc = reinterpret_cast<float*>(smem4);
    __shared__ int s_item;
    int fallbacks = 0;
    for (int round = 0;; ++round) {
        if (queue) {
            if (threadIdx.x == 0) s_item = atomicAdd(queue, 1);
            __syncthreads();
        } else if (threadIdx.x == 0) {
            s_item = round == 0 ? (int)blockIdx.x : n_items;
        }
        if (!queue) __syncthreads();
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
        for (int i = threadIdx.x; i < n4; i += THREADS) smem4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        __syncthreads();

        // ranges are clamped to the arrays so malformed offsets cannot read out of bounds
        const uint32_t sub1 = min(b.path_sub[wi.path + 1], b.n_subpaths);
        const uint32_t sub0 = min(b.path_sub[wi.path], sub1);
        const uint32_t seg1 = min(b.sub_off[sub1], b.n_segments);
        const uint32_t seg0 = min(b.sub_off[sub0], seg1);
        const uint32_t n_seg = seg1 - seg0, n_close = sub1 - sub0;
        const double* trm = b.tr ? b.tr + 6ull * wi.path : nullptr;
        for (uint32_t i = threadIdx.x; i < n_seg + n_close; i += THREADS) {
            if (i < n_seg) {
                const uint32_t g = seg0 + i;
                Seg64 parts[4];
                const int np = expand_segment(b.kind[g], b.pts + 8ull * g, parts);
                if (np < 0) { set_err(b.err, ERR_ARC); continue; }
                for (int j = 0; j < np; ++j) {
                    transform_seg(parts[j], trm);
                    band_segment(b, B, parts[j], fallbacks);
                }
            } else {
                // closing line Line(subpath.end(), subpath.start()).transform(tr) (src/path.rs:776-786)
                const uint32_t sp = sub0 + (i - n_seg);
                const uint32_t s1 = min(b.sub_off[sp + 1], b.n_segments);
                const uint32_t s0 = b.sub_off[sp];
                if (s1 <= s0) continue;
                Seg64 l;
                l.kind = SEG_LINE;
                if (!subpath_point(b, s0, s1, false, l.x[0], l.y[0])) continue;
                if (!subpath_point(b, s0, s1, true, l.x[1], l.y[1])) continue;
                l.x[2] = l.y[2] = l.x[3] = l.y[3] = 0.0;
                transform_seg(l, trm);
                band_segment(b, B, l, fallbacks);
            }
        }
        __syncthreads();

        const int rule = b.rule ? b.rule[wi.path] : 0;
        const int lane_warps = THREADS / 32;
        const int warp = threadIdx.x >> 5;
        for (int r = warp; r < B.bh; r += lane_warps) {
            float* out_row = b.out + m.offset + (uint64_t)(B.y0 + r) * (uint64_t)m.row_stride;
            const bool vec_ok = ((reinterpret_cast<uintptr_t>(out_row) & 15u) == 0);
            scan_row_store(acc + r * B.stride, m.width, rule, out_row, vec_ok);
        }
        __syncthreads();
    }
    if (fallbacks) atomicAdd(&b.counters[1], fallbacks);
}

// Host-callable launchers (declared in rz_api.cu).  init_kernels() runs once
// per context creation, outside any stream capture.
cudaError_t init_kernels() {
    return cudaFuncSetAttribute(k_mask_bands<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}

cudaError_t launch_mask_bands(const BatchDev& b, const WorkItem* items, int n_items, int32_t* queue, int grid,
                              int smem_bytes, cudaStream_t stream) {
    k_mask_bands<256><<<grid, 256, smem_bytes, stream>>>(b, items, n_items, queue);
    return cudaGetLastError();
}

int mask_bands_occupancy(int smem_bytes) {
    int blocks = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_mask_bands<256>, 256, smem_bytes);
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
