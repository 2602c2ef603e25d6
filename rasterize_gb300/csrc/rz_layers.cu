// rz_layers.cu -- the layers of a scene tree (src/scene.rs:436-565): a
// layer's initial colour, and Layer::compose of a child layer onto its parent
// for Opacity (src = src * opacity, then dst.blend_over(src), :436-443) and
// Clip (child * mask, then dst.blend_over(child), :444-456).  Layers are
// premultiplied linear RGBA f32 rectangles of the canvas grid; a clip mask is
// f32.  Every product and sum is rounded on its own, like the reference's SSE
// arithmetic, so compose adds no error of its own.
#include <cuda_runtime.h>
#include <stdint.h>

namespace rz {

constexpr int kLayerThreads = 256;

__global__ void __launch_bounds__(kLayerThreads) k_layer_fill(float4* __restrict__ buf, uint64_t n, float4 v) {
    for (uint64_t i = (uint64_t)blockIdx.x * kLayerThreads + threadIdx.x; i < n; i += (uint64_t)gridDim.x * kLayerThreads)
        buf[i] = v;
}

// One rectangle of the canvas grid and where it lives: pixel (x, y) of the
// canvas is element (y - y0) * w + (x - x0).
struct LayerRect {
    int32_t x0, y0, w, h;
};

// dst = dst.blend_over(s) over the canvas rectangle [x0, x1) x [y0, y1) (the
// intersection of dst and src), with s = src * mask where the mask layer
// covers the pixel and s = s * opacity when scale_opacity is set.
__global__ void __launch_bounds__(kLayerThreads)
    k_layer_compose(float4* __restrict__ dst, LayerRect d, const float4* __restrict__ src, LayerRect s,
                    const float* __restrict__ mask, LayerRect m, float opacity, int scale_opacity, int x0, int y0,
                    int x1, int y1) {
    const int w = x1 - x0;
    const uint64_t n = (uint64_t)w * (uint64_t)(y1 - y0);
    for (uint64_t i = (uint64_t)blockIdx.x * kLayerThreads + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * kLayerThreads) {
        const int x = x0 + (int)(i % (uint64_t)w), y = y0 + (int)(i / (uint64_t)w);
        float4 c = src[(uint64_t)(y - s.y0) * s.w + (x - s.x0)];
        if (mask && x >= m.x0 && x < m.x0 + m.w && y >= m.y0 && y < m.y0 + m.h) {
            // child_layer.compose(&mask, |dst, src| dst * (src as f32))
            const float a = mask[(uint64_t)(y - m.y0) * m.w + (x - m.x0)];
            c = make_float4(__fmul_rn(c.x, a), __fmul_rn(c.y, a), __fmul_rn(c.z, a), __fmul_rn(c.w, a));
        }
        if (scale_opacity)
            c = make_float4(__fmul_rn(c.x, opacity), __fmul_rn(c.y, opacity), __fmul_rn(c.z, opacity),
                            __fmul_rn(c.w, opacity));
        // LinColor::blend_over (src/color.rs:342-344): src + dst * (1 - src.alpha)
        float4& o = dst[(uint64_t)(y - d.y0) * d.w + (x - d.x0)];
        const float4 v = o;
        const float t = __fsub_rn(1.0f, c.w);
        o = make_float4(__fadd_rn(c.x, __fmul_rn(v.x, t)), __fadd_rn(c.y, __fmul_rn(v.y, t)),
                        __fadd_rn(c.z, __fmul_rn(v.z, t)), __fadd_rn(c.w, __fmul_rn(v.w, t)));
    }
}

static unsigned layer_grid(uint64_t n) {
    const uint64_t b = (n + kLayerThreads - 1) / kLayerThreads;
    return (unsigned)(b < 1 ? 1 : (b > 4096 ? 4096 : b));
}

cudaError_t launch_layer_fill(float* buf, uint64_t n_pixels, const float v[4], cudaStream_t st) {
    if (n_pixels == 0) return cudaSuccess;
    k_layer_fill<<<layer_grid(n_pixels), kLayerThreads, 0, st>>>(reinterpret_cast<float4*>(buf), n_pixels,
                                                                  make_float4(v[0], v[1], v[2], v[3]));
    return cudaGetLastError();
}

// rects as {x0, y0, w, h}; mask may be null (then m is ignored).
cudaError_t launch_layer_compose(float* dst, const int32_t d[4], const float* src, const int32_t s[4],
                                 const float* mask, const int32_t m[4], float opacity, bool scale_opacity, int x0,
                                 int y0, int x1, int y1, cudaStream_t st) {
    if (x1 <= x0 || y1 <= y0) return cudaSuccess;
    const LayerRect D{d[0], d[1], d[2], d[3]}, S{s[0], s[1], s[2], s[3]};
    const LayerRect M = mask ? LayerRect{m[0], m[1], m[2], m[3]} : LayerRect{0, 0, 0, 0};
    const uint64_t n = (uint64_t)(x1 - x0) * (uint64_t)(y1 - y0);
    k_layer_compose<<<layer_grid(n), kLayerThreads, 0, st>>>(reinterpret_cast<float4*>(dst), D,
                                                              reinterpret_cast<const float4*>(src), S, mask, M,
                                                              opacity, scale_opacity ? 1 : 0, x0, y0, x1, y1);
    return cudaGetLastError();
}

}  // namespace rz
