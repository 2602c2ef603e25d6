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

// The byte of the fit's branch (u above 0.0031308) from one hardware power:
// with t = u^(1/8) taken as ex2.approx(lg2.approx(u) / 8), the fit is the
// polynomial -0.01848558 t^8 + 0.6445592 t^4 + 0.70994765 t^2 - 0.33605254 t,
// whose t f'(t) is at most 6.2 for u up to 4.  With u itself known to a
// relative 4e-7 (an approximate quotient) t is within a relative 2.5e-7, the
// fit within 1.6e-6 of the IEEE route's (both routes' roundings included) and
// the byte position b = fit * 255 + 0.5 within 4.5e-4.  So where b lies more
// than kByteGuard from an integer (or above 255 + kByteGuard: saturated) both
// routes give the same byte.  Returns false otherwise (0.2 % of values) or
// outside (0.00313082, 4]: the caller then takes the IEEE route.
constexpr float kByteGuard = 1e-3f;

__device__ __forceinline__ float ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float lg2_approx(float x) {
    float y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ bool fit_byte(float u, uint32_t& byte) {
    if (!(u > 0.00313082f && u <= 4.0f)) return false;
    const float t = ex2_approx(0.125f * lg2_approx(u));
    const float t2 = t * t, t4 = t2 * t2, t8 = t4 * t4;
    const float fit = fmaf(-0.01848558f, t8, fmaf(0.6445592f, t4, fmaf(0.70994765f, t2, -0.33605254f * t)));
    const float b = fmaf(fit, 255.0f, 0.5f);
    if (b >= 255.0f + kByteGuard) {
        byte = 255u;
        return true;
    }
    const float f = b - truncf(b);
    byte = (uint32_t)b;
    return f > kByteGuard && f < 1.0f - kByteGuard;
}

// srgb_u8(l2s_lane(u)) of an exact u: the linear branch directly, the fit's
// branch through fit_byte, the rest (and NaN, infinities) the IEEE route.
__device__ __forceinline__ uint32_t l2s_byte(float u) {
    if (u <= 0.0031308f) return srgb_u8(__fmul_rn(u, 12.92f));
    uint32_t byte;
    if (fit_byte(u, byte)) return byte;
    return srgb_u8(l2s_lane(u));
}

// One colour channel of From<LinColor> for RGBA: l2s of unmultiply's c / a
// (src/color.rs:308-316: 0 when a <= 1e-6).  ra is an approximate 1 / a: the
// quotient c * ra is within a relative 4e-7 of the IEEE c / a, which only the
// IEEE route recomputes.
__device__ __forceinline__ uint32_t channel_byte(float c, float a, float ra) {
    if (a == 1.0f) return l2s_byte(c);  // c / 1 == c
    if (a <= 1e-6f || c == 0.0f) return 0u;
    uint32_t byte;
    if (fit_byte(c * ra, byte)) return byte;
    return srgb_u8(l2s_lane(__fdiv_rn(c, a)));
}

// From<LinColor> for RGBA (src/color.rs:164-175): bytes r, g, b, a (alpha as
// is) little-endian in one word.
__device__ __forceinline__ uint32_t encode_lin_rgba8(float4 c) {
    const float ra = rcp_approx(c.w);
    return channel_byte(c.x, c.w, ra) | (channel_byte(c.y, c.w, ra) << 8) | (channel_byte(c.z, c.w, ra) << 16) |
           (srgb_u8(c.w) << 24);
}

// Scalar::to_rgba (src/color.rs:429-432): grey linear_to_srgb(1 - m), opaque.
__device__ __forceinline__ uint32_t encode_mask_rgba8(float m) {
    const uint32_t v = l2s_byte(__fsub_rn(1.0f, m));
    return v | (v << 8) | (v << 16) | 0xff000000u;
}

}  // namespace rz
