// rz_color.cuh -- sRGB8 encoding of premultiplied linear colours and masks,
// operation for operation as the reference rounds them: no FMA contraction
// (every product and sum is rounded on its own, like the SSE code), IEEE
// division and square root, and Rust's saturating `as u8`.
#pragma once
#include <stdint.h>

namespace rz {

// `(v * 255.0 + 0.5) as u8`: truncation toward zero, saturating at 0 and 255, NaN -> 0.
__device__ __forceinline__ uint32_t srgb_u8(float v) {
    const float s = __fadd_rn(__fmul_rn(v, 255.0f), 0.5f);
    if (!(s > 0.0f)) return 0u;
    return s >= 255.0f ? 255u : (uint32_t)s;
}

// linear_to_srgb (src/color.rs:465-477) and the x86 l2s lane (src/simd/x86.rs:197-214):
// the same fit, x * 12.92 at or below 0.0031308.
__device__ __forceinline__ float l2s_lane(float x0) {
    const float x1 = __fsqrt_rn(x0), x2 = __fsqrt_rn(x1), x3 = __fsqrt_rn(x2);
    const float high = __fsub_rn(__fadd_rn(__fadd_rn(__fmul_rn(-0.01848558f, x0), __fmul_rn(0.6445592f, x1)),
                                           __fmul_rn(0.70994765f, x2)),
                                 __fmul_rn(0.33605254f, x3));
    return x0 <= 0.0031308f ? __fmul_rn(x0, 12.92f) : high;
}

// From<LinColor> for RGBA (src/color.rs:164-175): unmultiply (alpha <= 1e-6 -> 0,
// src/color.rs:308-316), l2s, then bytes r, g, b, a little-endian in one word.
__device__ __forceinline__ uint32_t encode_lin_rgba8(float4 c) {
    float r = 0.f, g = 0.f, b = 0.f;
    if (!(c.w <= 1e-6f)) {
        r = __fdiv_rn(c.x, c.w);
        g = __fdiv_rn(c.y, c.w);
        b = __fdiv_rn(c.z, c.w);
    }
    return srgb_u8(l2s_lane(r)) | (srgb_u8(l2s_lane(g)) << 8) | (srgb_u8(l2s_lane(b)) << 16) | (srgb_u8(c.w) << 24);
}

// Scalar::to_rgba (src/color.rs:429-432): grey linear_to_srgb(1 - m), opaque.
__device__ __forceinline__ uint32_t encode_mask_rgba8(float m) {
    const uint32_t v = srgb_u8(l2s_lane(__fsub_rn(1.0f, m)));
    return v | (v << 8) | (v << 16) | 0xff000000u;
}

}  // namespace rz
