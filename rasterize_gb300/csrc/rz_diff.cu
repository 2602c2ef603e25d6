// rz_diff.cu -- differentiable batch: forward composite and hand-written adjoint.
//
// The images are stacked into one tall canvas (image i owns canvas rows
// [i H, (i + 1) H)) so the line pipeline flattens every path once and bins
// its lines by (path, row).  One CTA per band of R rows (R divides H, so a
// band belongs to one image; one warp per row, which reads only its row's
// lists) then:
//
//   forward   for the paths of its image in order: signed area of the path's
//             lines in shared memory (exact fixed point), row prefix, fill
//             rule, A += a alpha (1 - A)  (Rasterizer::fill + source-over,
//             src/rasterize.rs:69-115, alpha channel of a solid paint);
//   backward  for every path of its image: the same coverage, then per pixel
//             g = dL/dA * dA/dalpha * dalpha/dw with dA/dalpha =
//             a (1 - A) / (1 - a alpha) (so paths are independent once the
//             forward image is known), the row suffix sums G of g, and for
//             every line of the path in the band the derivative of
//             sum_pixels g * (the line's winding contribution) with respect
//             to the line's end points, restricted to the band's rows.
//
// Line derivative.  A line adds to the winding of pixel x in row r the area
// of the pixel to the right of it, so its loss term over row r is
// h * mean_{X in [xa, xn]} W_r(X) with h the signed height of its piece in
// the row and W_r(X) = G[k+1] + (k + 1 - X) g[k] on [k, k+1) (piecewise
// linear, continuous).  The mean and its derivatives in xa, xn are exact
// integrals over the pixels the piece spans; xa, xn, h carry forward-mode
// derivatives (dual numbers) through the reference's x rules
// (src/rasterize.rs:372-393, 923-937) and the row clipping.  The end points
// are B(t) at the dyadic parameters of the frozen bisection tree, so the
// chain to the control points is the cubic Bernstein weights.
#include "rz_device.cuh"
#include "rz_kernels.cuh"
#include "rz_pipeline.cuh"

namespace rz {

// ---------------------------------------------------------------------------
// FP32 control points -> the pipeline's binary64 cubic segments, and the
// scene around them: path p is subpath p (segments p segs .. (p + 1) segs - 1)
// and fill p, whose view is its image (W x H at canvas row (p / P) H, clip
// column W), one (fill, row) entry per image row.
// ---------------------------------------------------------------------------
__global__ void k_diff_segments(const float* __restrict__ ctrl, uint32_t n_paths, uint32_t paths_per_image, int segs,
                                int width, int height, int rule, uint8_t* kind, double* pts, uint32_t* sub_off,
                                FillDev* fills) {
    const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g <= n_paths) sub_off[g] = (uint32_t)g * (uint32_t)segs;
    if (g < n_paths) {
        const uint32_t p = (uint32_t)g;
        FillDev f{};
        f.sub0 = p;
        f.sub1 = p + 1u;
        f.seg0 = p * (uint32_t)segs;
        f.seg1 = f.seg0 + (uint32_t)segs;
        f.slot0 = p * (uint32_t)(segs + 1);  // the segments, then the closing line
        f.entry0 = p * (uint32_t)height;
        f.col0 = 0;
        f.row0 = (int32_t)(p / paths_per_image) * height;
        f.width = width;
        f.height = height;
        f.clip_width = width;
        f.band0 = f.row0;  // one-row bands
        f.nbands = height;
        f.rule = rule;
        f.paint = 0;
        f.tr[0] = 1.0;
        f.tr[4] = 1.0;
        fills[p] = f;
    }
    if (g >= (uint64_t)n_paths * segs) return;
    const uint64_t p = g / segs;
    const int s = (int)(g - p * segs);
    const float2* c = reinterpret_cast<const float2*>(ctrl) + p * 3ull * segs;
    const int idx[4] = {3 * s, 3 * s + 1, 3 * s + 2, 3 * ((s + 1) % segs)};
    #pragma unroll
    for (int j = 0; j < 4; ++j) {
        const float2 q = c[idx[j]];
        pts[8 * g + 2 * j] = (double)q.x;
        pts[8 * g + 2 * j + 1] = (double)q.y;
    }
    kind[g] = SEG_CUBIC;
}

// ---------------------------------------------------------------------------
// Shared per-band setup
// ---------------------------------------------------------------------------
constexpr int kDiffThreads = 256;




// Marks a superset of the accumulation words that accumulate_vtx writes for
// the line a -> b: in every band row the line reaches (rows widened by 0.01),
// its x range there clamped to [0, width] like the x rules, one word more on
// each side and the carry word after it.  Widens [lo, hi] to the marked
// columns.
__device__ void diff_mark(const Band& B, const VtxQ& a, const VtxQ& b, uint32_t* bits, int wpr, int& lo, int& hi) {
    const float ax = (float)a.col + a.fx, bx = (float)b.col + b.fx;
    const float ay = (float)a.row + a.fy, by = (float)b.row + b.fy;
    if (ay == by) return;  // no signed height
    const float ylo = fminf(ay, by), yhi = fmaxf(ay, by);
    const int r0 = max((int)floorf(ylo - 0.01f), 0), r1 = min((int)floorf(yhi + 0.01f), B.bh - 1);
    const float inv = __fdividef(1.f, by - ay), dx = bx - ax;  // |by - ay| > 0: the marks are widened anyway
    const int cmax = B.width_i + 2;
    for (int r = r0; r <= r1; ++r) {
        const float t0 = fminf(fmaxf(((float)r - 0.01f - ay) * inv, 0.f), 1.f);
        const float t1 = fminf(fmaxf(((float)r + 1.01f - ay) * inv, 0.f), 1.f);
        const float x0 = fmaf(t0, dx, ax), x1 = fmaf(t1, dx, ax);
        const float xl = fminf(fmaxf(fminf(x0, x1), 0.f), B.width_f);
        const float xh = fminf(fmaxf(fmaxf(x0, x1), 0.f), B.width_f);
        const int c0 = max((int)floorf(xl) - 1, 0), c1 = min((int)floorf(xh) + 2, cmax);
        lo = min(lo, c0);
        hi = max(hi, c1);
        uint32_t* row = bits + r * wpr;
        for (int w = c0 >> 5; w <= (c1 >> 5); ++w) {
            const int lo = max(c0 - (w << 5), 0), hi = min(c1 - (w << 5), 31);
            const uint32_t upto = hi == 31 ? 0xffffffffu : ((1u << (hi + 1)) - 1u);
            atomicOr(&row[w], upto & ~((1u << lo) - 1u));
        }
    }
}

// ---------------------------------------------------------------------------
// Forward
// ---------------------------------------------------------------------------
// Widens [lo, hi] to the columns the accumulation of the line a -> b can
// write in its band row: the line's x range clamped to [0, width] like the x
// rules, one column more on the left and two on the right (the pixel after
// the last covered one takes the rest of the row's height; FP32 rounding of
// the ends stays far below a column).
__device__ __forceinline__ void line_cols(const Band& B, const VtxQ& a, const VtxQ& b, int& lo, int& hi) {
    const float ax = (float)a.col + a.fx, bx = (float)b.col + b.fx;
    const float xl = fminf(fmaxf(fminf(ax, bx), 0.f), B.width_f);
    const float xh = fminf(fmaxf(fmaxf(ax, bx), 0.f), B.width_f);
    lo = min(lo, max((int)floorf(xl) - 1, 0));
    hi = max(hi, min((int)floorf(xh) + 2, B.width_i + 2));
}

// A += a alpha (1 - A) for the pixels the fill does not skip (|alpha| < 1e-6,
// src/rasterize.rs:347-349): the lane's 4 pixels at x, windings w[0..3].
template <int RULE>
__device__ __forceinline__ void diff_blend4(float* Arow, int x, int width, bool vec, float alpha, const uint32_t (&w)[4]) {
    if (vec && x < width) {
        // four pixels at once; a skipped pixel takes fma(0, 1 - A, A) = A exactly
        float4 dv = *reinterpret_cast<const float4*>(Arow + x);
        float* d = reinterpret_cast<float*>(&dv);
        #pragma unroll
        for (int i = 0; i < 4; ++i) {
            const float al = alpha_fix<RULE>(w[i]);  // NonZero: 0 below 1e-6 already
            d[i] = fmaf(RULE == 1 && al < 1e-6f ? 0.f : alpha * al, 1.f - d[i], d[i]);
        }
        *reinterpret_cast<float4*>(Arow + x) = dv;
        return;
    }
    #pragma unroll
    for (int i = 0; i < 4; ++i) {
        if (x + i >= width) break;
        const float al = alpha_fix<RULE>(w[i]);
        if (al < 1e-6f) continue;
        float& d = Arow[x + i];
        d = fmaf(alpha * al, 1.f - d, d);
    }
}

// STEPS 128-pixel steps of the row prefix from column x0 (clearing the words
// it reads below x_end), the fill rule and the blend.  The steps' warp scans
// are independent, so their shuffles interleave instead of forming one
// dependent chain per step; the carry then runs over the steps in order.
// Columns at or past `width` (lines write up to width + 2) are cleared but
// take no part in the prefix.
template <int RULE, int STEPS>
__device__ __forceinline__ void diff_scan_steps(int4* row4, int x0, int x_end, int width, bool vec, float alpha,
                                                float* Arow, uint32_t& carry, int lane) {
    uint32_t a[STEPS][4], incl[STEPS];
    #pragma unroll
    for (int g = 0; g < STEPS; ++g) {
        const int x = x0 + 128 * g + 4 * lane;
        int4 v = make_int4(0, 0, 0, 0);
        if (x < x_end) {
            v = row4[x >> 2];
            row4[x >> 2] = make_int4(0, 0, 0, 0);
        }
        a[g][0] = x < width ? (uint32_t)v.x : 0u;
        a[g][1] = a[g][0] + (x + 1 < width ? (uint32_t)v.y : 0u);
        a[g][2] = a[g][1] + (x + 2 < width ? (uint32_t)v.z : 0u);
        a[g][3] = a[g][2] + (x + 3 < width ? (uint32_t)v.w : 0u);
        incl[g] = a[g][3];
    }
    #pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        #pragma unroll
        for (int g = 0; g < STEPS; ++g) {
            const uint32_t o = __shfl_up_sync(0xffffffffu, incl[g], off);
            if (lane >= off) incl[g] += o;
        }
    }
    #pragma unroll
    for (int g = 0; g < STEPS; ++g) {
        const uint32_t base = carry + incl[g] - a[g][3];
        carry += __shfl_sync(0xffffffffu, incl[g], 31);
        const uint32_t w[4] = {base + a[g][0], base + a[g][1], base + a[g][2], base + a[g][3]};
        diff_blend4<RULE>(Arow, x0 + 128 * g + 4 * lane, width, vec, alpha, w);
    }
}

// Row prefix of one band row over the columns [lo, hi] that the path's lines
// wrote (clearing them as it reads), fill rule and blend.  The winding is 0
// before lo (nothing to blend) and constant after hi: the rest of the row
// takes one alpha, blended only if the fill keeps it.  One warp, 4 pixels per
// lane per step.
template <int RULE>
__device__ void diff_scan_blend_span(float* crow, int width, float alpha, float* Arow, int lo, int hi, int lane) {
    int4* row4 = reinterpret_cast<int4*>(crow);
    uint32_t carry = 0;
    const bool vec = (width & 3) == 0;  // rows of A are 16-byte aligned: whole float4 chunks
    const int x_end = hi + 1;           // < the row stride (width + 3 at least)
    int x0 = lo & ~3;
    while (x_end - x0 > 384) {
        diff_scan_steps<RULE, 4>(row4, x0, x_end, width, vec, alpha, Arow, carry, lane);
        x0 += 512;
    }
    if (x_end - x0 > 128) {
        diff_scan_steps<RULE, 2>(row4, x0, x_end, width, vec, alpha, Arow, carry, lane);
        x0 += 256;
    }
    if (x_end - x0 > 0) {
        diff_scan_steps<RULE, 1>(row4, x0, x_end, width, vec, alpha, Arow, carry, lane);
        x0 += 128;
    }
    if (x0 >= width) return;
    const float al = alpha_fix<RULE>(carry);
    if (al < 1e-6f) return;
    for (int x = x0 + lane; x < width; x += 32) Arow[x] = fmaf(alpha * al, 1.f - Arow[x], Arow[x]);
}

// The line lists of canvas row `band` (lists are binned per row) of paths
// p0 + lane (one per lane, 32 at a time): every lane loads its path's
// (fill, row) entry at once instead of one path after the other.  n = 0 for
// paths past the image's last.
__device__ __forceinline__ void path_entries(const DiffDev& D, int img, int band, int p0, int lane, uint32_t& n,
                                             uint32_t& start) {
    n = 0;
    start = 0;
    const int p = p0 + lane;
    if (p < D.paths) {
        const FillDev& f = D.S.fills[img * D.paths + p];
        const uint32_t e = f.entry0 + (band - f.band0);
        n = D.S.entry_count[e];
        start = D.S.entry_start[e];
    }
}

// The one-row band of image row `row` for the differentiable batch: every
// path's fill is the whole image (view W x H at canvas row img * H, clip W).
__device__ __forceinline__ Band diff_row_band(const DiffDev& D, float* crow, int row, int img) {
    Band B;
    B.acc = crow;
    B.stride = band_stride(D.width);
    B.bh = 1;
    B.y0 = row - img * D.height;
    B.img_h = D.height;
    B.width_f = (float)D.width;
    B.width_i = D.width;
    return B;
}

// Whether the line a -> b (rows relative to a one-row band) can write the
// row: it has a signed height and reaches [-0.01, 1.01].
__device__ __forceinline__ bool line_reaches_row(const VtxQ& a, const VtxQ& b) {
    const float ay = (float)a.row + a.fy, by = (float)b.row + b.fy;
    return ay != by && fminf(ay, by) < 1.01f && fmaxf(ay, by) > -0.01f;
}

// One warp per band row, with no block barrier after the start: rows are
// independent (a line writes only its own rows' words), so each warp takes
// every path's lines that reach its row, accumulates them into its row
// (int32 shared atomics), then scans and blends the columns they wrote.
template <int RULE>
__global__ void __launch_bounds__(kDiffThreads, 3) k_diff_forward(DiffDev D, int cov_stride) {
    extern __shared__ float4 sm4[];
    float* cov = reinterpret_cast<float*>(sm4);
    const SceneDev& S = D.S;
    const int rows = D.cta_rows;
    float* A = cov + rows * cov_stride;
    const int row_base = blockIdx.x * rows;
    const int img = row_base / D.height;
    for (int i = threadIdx.x; i < rows * D.width; i += kDiffThreads) A[i] = 0.f;
    for (int i = threadIdx.x; i < (rows * cov_stride) >> 2; i += kDiffThreads) sm4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp >= rows) return;
    float* crow = cov + warp * cov_stride;
    float* Arow = A + warp * D.width;
    const int row = row_base + warp;
    const Band B = diff_row_band(D, crow, row, img);
    for (int p0 = 0; p0 < D.paths; p0 += 32) {
        uint32_t my_n, my_start;
        path_entries(D, img, row, p0, lane, my_n, my_start);  // lists are binned per row
        uint32_t todo = __ballot_sync(0xffffffffu, my_n != 0);  // paths with no line in the row add nothing
      while (todo) {
        const int q = __ffs(todo) - 1;
        todo &= todo - 1u;
        const uint32_t n = __shfl_sync(0xffffffffu, my_n, q), start = __shfl_sync(0xffffffffu, my_start, q);
        int lo = D.width + 2, hi = -1;  // the columns written
        for (uint32_t j = lane; j < n; j += 32) {
            const uint32_t l = S.pairs[start + j];
            const VtxQ a = line_vtx(S.lines[2ull * l], B.y0), b = line_vtx(S.lines[2ull * l + 1], B.y0);
            if (!line_reaches_row(a, b)) continue;
            line_cols(B, a, b, lo, hi);
            accumulate_vtx(B, a, b);
        }
        hi = __reduce_max_sync(0xffffffffu, hi);
        if (hi < 0) continue;  // no crossing in this row: the winding is 0 along it
        lo = __reduce_min_sync(0xffffffffu, lo);
        __syncwarp();
        diff_scan_blend_span<RULE>(crow, D.width, D.alpha, Arow, lo, hi, lane);
        __syncwarp();
      }
    }
    float* out = D.out + (uint64_t)row * D.width;  // canvas rows are image rows
    for (int i = lane; i < D.width; i += 32) out[i] = Arow[i];
}

// ---------------------------------------------------------------------------
// Backward
// ---------------------------------------------------------------------------
struct Dual {
    float v, d[4];
};
__device__ __forceinline__ Dual dconst(float v) { return Dual{v, {0.f, 0.f, 0.f, 0.f}}; }
__device__ __forceinline__ Dual dadd(const Dual& a, const Dual& b) {
    return Dual{a.v + b.v, {a.d[0] + b.d[0], a.d[1] + b.d[1], a.d[2] + b.d[2], a.d[3] + b.d[3]}};
}
__device__ __forceinline__ Dual dsub(const Dual& a, const Dual& b) {
    return Dual{a.v - b.v, {a.d[0] - b.d[0], a.d[1] - b.d[1], a.d[2] - b.d[2], a.d[3] - b.d[3]}};
}
__device__ __forceinline__ Dual dmul(const Dual& a, const Dual& b) {
    Dual r;
    r.v = a.v * b.v;
    #pragma unroll
    for (int k = 0; k < 4; ++k) r.d[k] = fmaf(a.d[k], b.v, a.v * b.d[k]);
    return r;
}
// One hardware reciprocal (within 2 ulp) per quotient: the derivatives do not
// need the correctly rounded division.
__device__ __forceinline__ Dual ddiv(const Dual& a, const Dual& b) {
    Dual r;
    const float inv = __fdividef(1.f, b.v);
    r.v = a.v * inv;
    #pragma unroll
    for (int k = 0; k < 4; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * inv;
    return r;
}
__device__ __forceinline__ Dual dlerp(const Dual& a, const Dual& b, const Dual& t) {  // (1 - t) a + t b
    return dadd(a, dmul(t, dsub(b, a)));
}

// The adjoint's per-row data is sparse.  A pixel's winding is fractional only
// where a line of the path crosses it, and those pixels are among the
// accumulation words the lines write.  Every other pixel has an integer
// winding, so its dalpha/dw is 0.  `bits` marks a superset of the written
// words.  After diff_sparse_row, each marked word of the row holds g there
// (as float bits) and P the inclusive prefix of g along the row; tot[r] is the
// row's sum.
struct CellView {
    const uint32_t* bits;  // rows x wpr
    const float* g;        // rows x stride (the band)
    const float* P;        // rows x stride
    const float* tot;      // rows
    int wpr, stride, W;
    // g[k] and G[k+1] = sum of g over the pixels after k, row r
    __device__ __forceinline__ void at(int r, int k, float& gk, float& Gk1) const {
        const uint32_t* brow = bits + r * wpr;
        const int o = r * stride;
        if ((brow[k >> 5] >> (k & 31)) & 1u) {
            gk = g[o + k];
            Gk1 = tot[r] - P[o + k];
            return;
        }
        gk = 0.f;  // an unmarked pixel: integer winding, no slope; G from the next marked one
        Gk1 = 0.f;
        int w = (k + 1) >> 5;
        uint32_t word = w < wpr ? brow[w] & (0xffffffffu << ((k + 1) & 31)) : 0u;
        while (!word && ++w < wpr) word = brow[w];
        if (word) {
            const int m = (w << 5) + __ffs(word) - 1;
            if (m < W) Gk1 = tot[r] - P[o + m] + g[o + m];
        }
    }
};

// Mean of W_r over [lo, hi] (x relative to column c0) and its derivatives,
// W_r(X) = G[k+1] + (k + 1 - X) g[k] on [k, k+1).
__device__ void diff_row_mean(const CellView& V, int r, int c0, float lo, float hi, float& I, float& dlo,
                              float& dhi) {
    const int W = V.W;
    const float wmax = (float)(W - c0), wmin = (float)(-c0);
    lo = fminf(fmaxf(lo, wmin), wmax);
    hi = fminf(fmaxf(hi, lo), wmax);
    const float D = hi - lo;
    if (D < 1e-6f) {
        int k = (int)floorf(lo);
        k = min(max(k + c0, 0), W - 1);
        const float kr = (float)(k - c0);
        float gk, Gk1;
        V.at(r, k, gk, Gk1);
        I = Gk1 + (kr + 1.f - lo) * gk;
        dlo = dhi = -0.5f * gk;
        return;
    }
    const int k0 = (int)floorf(lo), k1 = min((int)floorf(hi), W - 1 - c0);
    if (k1 == k0 || hi <= (float)(k0 + 1)) {  // one pixel: the mean in closed form
        float gk, Gk1;
        V.at(r, k0 + c0, gk, Gk1);
        I = Gk1 + ((float)(k0 + 1) - 0.5f * (lo + hi)) * gk;
        dlo = dhi = -0.5f * gk;
        return;
    }
    float sI = 0.f, slo = 0.f, shi = 0.f;
    for (int k = k0; k <= k1; ++k) {
        const float a = fmaxf(lo, (float)k), b = fminf(hi, (float)(k + 1));
        if (b <= a) continue;
        float gk, Gk1;
        V.at(r, k + c0, gk, Gk1);
        const float ka = (float)(k + 1) - a, kb = (float)(k + 1) - b;
        sI += Gk1 * (b - a) + gk * 0.5f * (ka * ka - kb * kb);
        shi -= gk * 0.5f * ((b - lo) * (b - lo) - (a - lo) * (a - lo));
        slo -= gk * 0.5f * ((hi - a) * (hi - a) - (hi - b) * (hi - b));
    }
    const float inv = __fdividef(1.f, D);  // D >= 1e-6
    I = sI * inv;
    dhi = shi * inv * inv;
    dlo = slo * inv * inv;
}

// d(sum over the row's pixels of g * winding contribution of the piece p -> q)/d(line ends);
// x relative to column c0, y relative to the row (which is y in [0, 1)).
__device__ void diff_piece(Dual px, Dual py, Dual qx, Dual qy, int c0, const CellView& V, float (&out)[4]) {
    if (py.v == qy.v) {
        // horizontal: no coverage, but moving an end vertically brings coverage in
        if (!(py.v >= 0.f && py.v < 1.f)) return;
        float I, dlo, dhi;
        diff_row_mean(V, 0, c0, fminf(px.v, qx.v), fmaxf(px.v, qx.v), I, dlo, dhi);
        #pragma unroll
        for (int k = 0; k < 4; ++k) out[k] += I * (qy.d[k] - py.d[k]);
        return;
    }
    float dir = 1.f;
    if (py.v > qy.v) {
        Dual t = px; px = qx; qx = t;
        t = py; py = qy; qy = t;
        dir = -1.f;
    }
    if (!(py.v < 1.f && qy.v > 0.f)) return;  // the piece misses the row
    const bool start_in = py.v >= 0.f, end_in = qy.v <= 1.f;
    const Dual sa = start_in ? py : dconst(0.f);
    const Dual sb = end_in ? qy : dconst(1.f);
    if (!(sb.v > sa.v)) return;
    Dual xa = px, xn = qx;  // x where the piece enters and leaves the row
    if (!start_in || !end_in) {
        const Dual kx = ddiv(dsub(qx, px), dsub(qy, py));  // dx/dy
        if (!start_in) xa = dadd(px, dmul(dsub(sa, py), kx));
        if (!end_in) xn = dadd(px, dmul(dsub(sb, py), kx));
    }
    const Dual h = dsub(sb, sa);
    const bool ord = xa.v <= xn.v;
    const Dual& lo = ord ? xa : xn;
    const Dual& hi = ord ? xn : xa;
    float I, dlo, dhi;
    diff_row_mean(V, 0, c0, lo.v, hi.v, I, dlo, dhi);
    #pragma unroll
    for (int k = 0; k < 4; ++k) out[k] += dir * (I * h.d[k] + h.v * (dlo * lo.d[k] + dhi * hi.d[k]));
}

// diff_piece for a line that no x rule changes (both ends in [0, width]),
// with the gradient of F = dir h I(lo, hi) taken in reverse mode through
// the row clip: the same quantities as the dual numbers in a few scalar
// operations.  (ax, ay) -> (bx, by), x relative to column c0, y relative to
// the row.
__device__ __forceinline__ void diff_piece_inside(float ax, float ay, float bx, float by, int c0, const CellView& V,
                                                  float (&out)[4]) {
    float I, dlo, dhi;
    if (ay == by) {
        // horizontal: no coverage, but moving an end vertically brings coverage in
        if (!(ay >= 0.f && ay < 1.f)) return;
        diff_row_mean(V, 0, c0, fminf(ax, bx), fmaxf(ax, bx), I, dlo, dhi);
        out[1] -= I;
        out[3] += I;
        return;
    }
    const bool down = ay < by;  // p -> q runs down the rows
    const float px = down ? ax : bx, py = down ? ay : by, qx = down ? bx : ax, qy = down ? by : ay;
    if (!(py < 1.f && qy > 0.f)) return;  // the piece misses the row
    const bool start_in = py >= 0.f, end_in = qy <= 1.f;
    const float sa = start_in ? py : 0.f, sb = end_in ? qy : 1.f;
    if (!(sb > sa)) return;
    float xa = px, xn = qx, inv = 0.f, kx = 0.f;  // x where the piece enters and leaves the row
    if (!start_in || !end_in) {
        inv = __fdividef(1.f, qy - py);
        kx = (qx - px) * inv;  // dx/dy
        if (!start_in) xa = px + (sa - py) * kx;
        if (!end_in) xn = px + (sb - py) * kx;
    }
    const float h = sb - sa;
    const bool ord = xa <= xn;
    diff_row_mean(V, 0, c0, ord ? xa : xn, ord ? xn : xa, I, dlo, dhi);
    const float dir = down ? 1.f : -1.f;
    const float gh = dir * I;                           // dF/dh
    const float gxa = dir * h * (ord ? dlo : dhi);      // dF/dxa
    const float gxn = dir * h * (ord ? dhi : dlo);      // dF/dxn
    float gpx = 0.f, gpy = 0.f, gqx = 0.f, gqy = 0.f;
    if (start_in) {  // xa = px, h = sb - py
        gpx += gxa;
        gpy -= gh;
    } else {  // xa = px + u kx, u = sa - py, kx = (qx - px) / (qy - py)
        const float u = (sa - py) * inv, t = gxa * u;
        gpx += gxa - t;
        gpy += t * kx - gxa * kx;
        gqx += t;
        gqy -= t * kx;
    }
    if (end_in) {  // xn = qx, h = qy - sa
        gqx += gxn;
        gqy += gh;
    } else {  // xn = px + v kx, v = sb - py
        const float v = (sb - py) * inv, t = gxn * v;
        gpx += gxn - t;
        gpy += t * kx - gxn * kx;
        gqx += t;
        gqy -= t * kx;
    }
    out[0] += down ? gpx : gqx;
    out[1] += down ? gpy : gqy;
    out[2] += down ? gqx : gpx;
    out[3] += down ? gqy : gpy;
}

// The reference's x rules on dual numbers (width = W, relative to column c0), then the pieces.
__device__ void diff_line(float ax, float ay, float bx, float by, int c0, const CellView& V, float (&out)[4]) {
    Dual x0{ax, {1.f, 0.f, 0.f, 0.f}}, y0{ay, {0.f, 1.f, 0.f, 0.f}};
    Dual x1{bx, {0.f, 0.f, 1.f, 0.f}}, y1{by, {0.f, 0.f, 0.f, 1.f}};
    const float width = (float)(V.W - c0), zero = (float)(-c0);
    if (ax <= width && bx <= width && ax >= zero && bx >= zero) {  // no x rule applies: most lines
        diff_piece_inside(ax, ay, bx, by, c0, V, out);
        return;
    }
    if (x0.v > width || x1.v > width) {
        if (x0.v > width && x1.v > width) {
            x0 = dconst(width - 0.001f);
            x1 = dconst(width - 0.001f);
        } else {
            const Dual t = ddiv(dsub(x0, dconst(width)), dsub(x0, x1));
            const Dual my = dlerp(y0, y1, t);
            if (x0.v < width) { x1 = dconst(width); y1 = my; }
            else { x0 = dconst(width); y0 = my; }
        }
    }
    if (x0.v >= zero && x1.v >= zero) {
        diff_piece(x0, y0, x1, y1, c0, V, out);
    } else if (x0.v <= zero && x1.v <= zero) {
        diff_piece(dconst(zero), y0, dconst(zero), y1, c0, V, out);
    } else {
        const Dual t = ddiv(dsub(x0, dconst(zero)), dsub(x0, x1));
        const Dual mx = dlerp(x0, x1, t), my = dlerp(y0, y1, t);
        if (x0.v < zero) {
            diff_piece(mx, my, x1, y1, c0, V, out);
            diff_piece(dconst(zero), y0, mx, my, c0, V, out);
        } else {
            diff_piece(x0, y0, mx, my, c0, V, out);
            diff_piece(mx, my, dconst(zero), y1, c0, V, out);
        }
    }
}

// g = dL/dA * a (1 - A) / (1 - a alpha) * dalpha/dw at pixel x of the row,
// winding wn (0 where the forward skips the pixel or the fill has no slope).
template <int RULE>
__device__ __forceinline__ float diff_g(const DiffDev& D, uint32_t wn, int x, int W, const float* dlrow,
                                        const float* Arow) {
    if (x >= W) return 0.f;
    const float al = alpha_fix<RULE>(wn);
    if (al < 1e-6f) return 0.f;  // pixels the forward skips have no slope
    float da = 0.f;
    if (RULE == 1) {
        const int32_t fo = (int32_t)((wn + (1u << 22)) & ((1u << 23) - 1u)) - (1 << 22);
        da = fo > 0 ? 1.f : -1.f;
    } else if (al < 1.f) {
        da = (int32_t)wn > 0 ? 1.f : -1.f;
    }
    if (da == 0.f) return 0.f;
    // 1 - a alpha lies in [1 - a, 1]: the hardware quotient (within 2 ulp) is enough
    return __fdividef(dlrow[x] * D.alpha * (1.f - Arow[x]), 1.f - D.alpha * al) * da;
}

// Sparse pass over the words wlo..whi of one row (one warp; no other word
// holds a mark): the marked pixels in increasing order, 64 at a time, two
// per lane (lane i takes the marked pixels of ranks c + 2i and c + 2i + 1:
// the first's 32-word block by a search over the words' prefix counts and its
// bit by a select within the word, the second the next mark after it).  Warp scans give the exact integer windings there
// (the prefix of the marked words; the others are 0),
// g = dL/dA * a (1 - A) / (1 - a alpha) * dalpha/dw, and the inclusive prefix
// P of g.  g overwrites the coverage word, P goes to its own row; *tot gets
// the row's sum.
template <int RULE>
__device__ void diff_sparse_row(const DiffDev& D, int wlo, int whi, int row, const uint32_t* brow, float* cov_row,
                                float* prow, float* tot, int lane) {
    const int W = D.width;
    int32_t* crow = reinterpret_cast<int32_t*>(cov_row);
    const float* Arow = D.image + (uint64_t)row * W;
    const float* dlrow = D.dl_dimage + (uint64_t)row * W;
    uint32_t wcarry = 0;
    float gcarry = 0.f;
    for (int w0 = wlo; w0 <= whi; w0 += 32) {
        const uint32_t mine = w0 + lane <= whi ? brow[w0 + lane] : 0u;
        const int cnt = __popc(mine);
        int incl = cnt;  // marked pixels in words w0 .. w0 + lane
        #pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int o = __shfl_up_sync(0xffffffffu, incl, off);
            if (lane >= off) incl += o;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        const int excl = incl - cnt;
        const uint32_t nonempty = __ballot_sync(0xffffffffu, mine != 0u);
        for (int c = 0; c < total; c += 64) {
            const int r = c + 2 * lane;  // this lane's ranks: r and r + 1
            // the word holding rank r: the number of words whose inclusive count is <= r
            int j = 0;
            #pragma unroll
            for (int step = 16; step >= 1; step >>= 1) {
                const int v = __shfl_sync(0xffffffffu, incl, j + step - 1);
                if (v <= r) j += step;
            }
            j = min(j, 31);
            const uint32_t wbits = __shfl_sync(0xffffffffu, mine, j);
            int k = r - __shfl_sync(0xffffffffu, excl, j);  // rank within the word
            int pos = 0;
            #pragma unroll
            for (int w = 16; w >= 1; w >>= 1) {
                const int in = __popc((wbits >> pos) & ((1u << w) - 1u));
                if (k >= in) {
                    k -= in;
                    pos += w;
                }
            }
            // rank r + 1: the next mark of the same word, else the first mark of the next marked word
            const uint32_t above = pos == 31 ? 0u : wbits & (0xfffffffeu << pos);
            const uint32_t later = j == 31 ? 0u : nonempty & (0xfffffffeu << j);
            const int j2 = later ? __ffs(later) - 1 : j;
            const uint32_t wbits2 = __shfl_sync(0xffffffffu, mine, j2);
            const bool live0 = r < total, live1 = r + 1 < total;
            const int x0 = ((w0 + j) << 5) + pos;
            const int x1 = above ? ((w0 + j) << 5) + __ffs(above) - 1 : ((w0 + j2) << 5) + __ffs(wbits2) - 1;
            const uint32_t d0 = live0 ? (uint32_t)crow[x0] : 0u, d1 = live1 ? (uint32_t)crow[x1] : 0u;
            uint32_t wi = d0 + d1;
            #pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const uint32_t o = __shfl_up_sync(0xffffffffu, wi, off);
                if (lane >= off) wi += o;
            }
            // windings at x0 and x1 (exact: integer prefix)
            const uint32_t wn1 = wcarry + wi, wn0 = wn1 - d1;
            wcarry += __shfl_sync(0xffffffffu, wi, 31);
            const float g0 = live0 ? diff_g<RULE>(D, wn0, x0, W, dlrow, Arow) : 0.f;
            const float g1 = live1 ? diff_g<RULE>(D, wn1, x1, W, dlrow, Arow) : 0.f;
            float gi = g0 + g1;
            #pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const float o = __shfl_up_sync(0xffffffffu, gi, off);
                if (lane >= off) gi += o;
            }
            const float gex = __shfl_up_sync(0xffffffffu, gi, 1);
            const float p0 = gcarry + (lane ? gex : 0.f) + g0;
            if (live0) {
                crow[x0] = __float_as_int(g0);
                prow[x0] = p0;
            }
            if (live1) {
                crow[x1] = __float_as_int(g1);
                prow[x1] = p0 + g1;
            }
            gcarry += __shfl_sync(0xffffffffu, gi, 31);
        }
    }
    if (lane == 0) *tot = gcarry;
}

// 3 CTAs per SM (<= 85 registers).  One warp per band row with no block
// barrier after the start (rows are independent, and so are paths given the
// forward image): for each path the warp accumulates the lines that reach its
// row, marking the words they write, runs the sparse row pass, differentiates
// its row's share of every line and chains it to the control points, then
// clears the marked words.
template <int RULE>
__global__ void __launch_bounds__(kDiffThreads, 3) k_diff_backward(DiffDev D, int cov_stride) {
    extern __shared__ float4 sm4[];
    const SceneDev& S = D.S;
    const int rows = D.cta_rows;
    const int wpr = (cov_stride + 31) >> 5;
    float* cov = reinterpret_cast<float*>(sm4);  // coverage words, then g
    float* P = cov + rows * cov_stride;
    float* tot = P + rows * cov_stride;
    uint32_t* bits = reinterpret_cast<uint32_t*>(tot + 8);
    const int row_base = blockIdx.x * rows;
    const int img = row_base / D.height;
    float2* out = reinterpret_cast<float2*>(D.out);
    for (int i = threadIdx.x; i < rows * cov_stride; i += kDiffThreads) cov[i] = 0.f;
    for (int i = threadIdx.x; i < rows * wpr; i += kDiffThreads) bits[i] = 0u;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp >= rows) return;
    float* crow = cov + warp * cov_stride;
    float* prow = P + warp * cov_stride;
    uint32_t* brow = bits + warp * wpr;
    const int row = row_base + warp;
    const Band B = diff_row_band(D, crow, row, img);
    for (int p0 = 0; p0 < D.paths; p0 += 32) {
        uint32_t my_n, my_start;
        path_entries(D, img, row, p0, lane, my_n, my_start);  // lists are binned per row
        uint32_t todo = __ballot_sync(0xffffffffu, my_n != 0);  // no line in the row: nothing to move
      while (todo) {
        const int q = __ffs(todo) - 1;
        todo &= todo - 1u;
        const uint32_t n = __shfl_sync(0xffffffffu, my_n, q), start = __shfl_sync(0xffffffffu, my_start, q);
        int lo = D.width + 2, hi = -1;  // the marked columns
        for (uint32_t j = lane; j < n; j += 32) {
            const uint32_t l = S.pairs[start + j];
            const VtxQ a = line_vtx(S.lines[2ull * l], B.y0), b = line_vtx(S.lines[2ull * l + 1], B.y0);
            if (!line_reaches_row(a, b)) continue;
            accumulate_vtx(B, a, b);
            diff_mark(B, a, b, brow, wpr, lo, hi);
        }
        // nothing marked: nothing written in this row, g is 0 along it and no line moves the loss
        hi = __reduce_max_sync(0xffffffffu, hi);
        if (hi < 0) continue;
        lo = __reduce_min_sync(0xffffffffu, lo);
        const int wlo = lo >> 5, whi = hi >> 5;
        __syncwarp();
        diff_sparse_row<RULE>(D, wlo, whi, row, brow, crow, prow, tot + warp, lane);
        __syncwarp();
        const CellView V{brow, crow, prow, tot + warp, wpr, cov_stride, D.width};
        // the lists hold the lines of path p0 + q of the image: segments path_seg0 .. path_seg1 - 1
        const uint32_t path_seg0 = ((uint32_t)img * (uint32_t)D.paths + (uint32_t)(p0 + q)) * (uint32_t)D.segs;
        const uint32_t path_seg1 = path_seg0 + (uint32_t)D.segs;
        for (uint32_t j = lane; j < n; j += 32) {
            const uint32_t l = S.pairs[start + j];
            const uint2 code = S.leaf[l];
            if (code.x == 0xffffffffu) continue;  // a closing line (zero length here)
            const VtxQ a = line_vtx(S.lines[2ull * l], B.y0), b = line_vtx(S.lines[2ull * l + 1], B.y0);
            const float ay = (float)a.row + a.fy, by = (float)b.row + b.fy;
            if (!(fminf(ay, by) < 1.0f && fmaxf(ay, by) >= 0.0f)) continue;  // no share of this row
            const int c0 = a.col;
            float d4[4] = {0.f, 0.f, 0.f, 0.f};
            diff_line(a.fx, ay, (float)(b.col - c0) + b.fx, by, c0, V, d4);
            if (d4[0] == 0.f && d4[1] == 0.f && d4[2] == 0.f && d4[3] == 0.f) continue;
            // chain to the control points: Bernstein weights at the frozen tree's parameters
            // (segment seg of the path: control points 3 seg .. 3 seg + 2, then the next segment's first)
            const uint32_t seg = code.x;
            const int d = (int)(code.y >> 27);
            const uint32_t k = code.y & ((1u << 27) - 1u);
            const float t0 = (float)k * pow2f(-d), t1 = (float)(k + 1u) * pow2f(-d);
            const bool last = seg + 1u == path_seg1;
            const float u0 = 1.f - t0, u1 = 1.f - t1;
            const float b0[4] = {u0 * u0 * u0, 3.f * t0 * u0 * u0, 3.f * t0 * t0 * u0, t0 * t0 * t0};
            const float b1[4] = {u1 * u1 * u1, 3.f * t1 * u1 * u1, 3.f * t1 * t1 * u1, t1 * t1 * t1};
            float2* o = out + 3ull * seg;
            float2* o3 = last ? out + 3ull * path_seg0 : o + 3;
            #pragma unroll
            for (int q = 0; q < 4; ++q)
                atomicAdd(q < 3 ? o + q : o3, make_float2(d4[0] * b0[q] + d4[2] * b1[q], d4[1] * b0[q] + d4[3] * b1[q]));
        }
        __syncwarp();
        // clear the words wlo..whi (every marked pixel, so every written one) and their bitmask words
        float4* c4 = reinterpret_cast<float4*>(crow);
        const int e4 = min((whi + 1) << 3, cov_stride >> 2);
        for (int i = (wlo << 3) + lane; i < e4; i += 32) c4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int w = wlo + lane; w <= whi; w += 32) brow[w] = 0u;
        __syncwarp();
      }
    }
}

// ---------------------------------------------------------------------------
// L2 loss: sum (A - T)^2 in binary64, dL/dA = 2 (A - T)
// ---------------------------------------------------------------------------
__global__ void k_l2_loss(const float* __restrict__ A, const float* __restrict__ T, uint64_t n, double* loss,
                          float* dl) {
    double acc = 0.0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const float d = A[i] - T[i];
        acc += (double)d * (double)d;
        if (dl) dl[i] = 2.f * d;
    }
    #pragma unroll
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
    __shared__ double wsum[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) wsum[warp] = acc;
    __syncthreads();
    if (warp == 0) {
        acc = lane < (int)(blockDim.x >> 5) ? wsum[lane] : 0.0;
        #pragma unroll
        for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
        if (lane == 0) atomicAdd(loss, acc);
    }
}

// ---------------------------------------------------------------------------
// launchers (declared in rz_api.cu)
// ---------------------------------------------------------------------------
int diff_smem_bytes(int width, int band_rows, bool backward, int* cov_stride) {
    const int stride = band_stride(width);
    *cov_stride = stride;
    if (!backward) return 4 * band_rows * stride + 4 * band_rows * width;  // coverage + A
    // coverage words (then g), the prefix of g, row sums, the bitmask of marked words
    return 8 * band_rows * stride + 32 + 4 * band_rows * ((stride + 31) >> 5);
}

cudaError_t launch_diff_segments(const float* ctrl, uint32_t n_paths, uint32_t paths_per_image, int segs, int width,
                                 int height, int rule, uint8_t* kind, double* pts, uint32_t* sub_off, FillDev* fills,
                                 cudaStream_t st) {
    const uint64_t n = std::max<uint64_t>((uint64_t)n_paths * segs, (uint64_t)n_paths + 1);
    k_diff_segments<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(ctrl, n_paths, paths_per_image, segs, width, height,
                                                                   rule, kind, pts, sub_off, fills);
    return cudaGetLastError();
}

cudaError_t launch_diff(const DiffDev& D, bool backward, int cov_stride, int smem, cudaStream_t st) {
    if (backward) {
        auto kern = D.rule == 1 ? k_diff_backward<1> : k_diff_backward<0>;
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        kern<<<D.S.canvas_h / D.cta_rows, kDiffThreads, smem, st>>>(D, cov_stride);
    } else {
        auto kern = D.rule == 1 ? k_diff_forward<1> : k_diff_forward<0>;
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        kern<<<D.S.canvas_h / D.cta_rows, kDiffThreads, smem, st>>>(D, cov_stride);
    }
    return cudaGetLastError();
}

cudaError_t launch_l2_loss(const float* A, const float* T, uint64_t n, double* loss, float* dl, int num_sms,
                           cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    const uint64_t blocks = std::min<uint64_t>((n + 255) / 256, (uint64_t)num_sms * 8);
    k_l2_loss<<<(unsigned)blocks, 256, 0, st>>>(A, T, n, loss, dl);
    return cudaGetLastError();
}

}  // namespace rz
