// rz_encode.cu -- output encode: premultiplied linear RGBA f32 (or a mask) to
// sRGB8 RGBA bytes, the per-pixel `Color::to_rgba` that the reference's image
// writers call (src/image.rs:136-229).  Pure streaming work: 16 (or 4 / 8)
// bytes read and 4 written per pixel, so the kernels are HBM-bound; each
// thread converts 4 pixels per step (one 16-byte store) in a grid-stride loop
// sized to the SM count.
#include <cuda_runtime.h>

#include "rz_color.cuh"

namespace rz {

constexpr int kEncThreads = 256;

__global__ void __launch_bounds__(kEncThreads) k_encode_rgba8(const float4* __restrict__ in, uint32_t* __restrict__ out,
                                                              uint64_t n) {
    const uint64_t n4 = n >> 2;
    const uint64_t step = (uint64_t)gridDim.x * kEncThreads;
    for (uint64_t q = (uint64_t)blockIdx.x * kEncThreads + threadIdx.x; q < n4; q += step) {
        const float4 a = __ldcs(in + 4 * q), b = __ldcs(in + 4 * q + 1);
        const float4 c = __ldcs(in + 4 * q + 2), d = __ldcs(in + 4 * q + 3);
        const uint4 v = make_uint4(encode_lin_rgba8(a), encode_lin_rgba8(b), encode_lin_rgba8(c), encode_lin_rgba8(d));
        __stcs(reinterpret_cast<uint4*>(out) + q, v);
    }
    // the last n % 4 pixels
    const uint64_t t = (uint64_t)blockIdx.x * kEncThreads + threadIdx.x;
    if (t < (n & 3)) out[4 * n4 + t] = encode_lin_rgba8(in[4 * n4 + t]);
}

template <typename T>
__global__ void __launch_bounds__(kEncThreads) k_encode_mask_rgba8(const T* __restrict__ in, uint32_t* __restrict__ out,
                                                                   uint64_t n) {
    const uint64_t n4 = n >> 2;
    const uint64_t step = (uint64_t)gridDim.x * kEncThreads;
    for (uint64_t q = (uint64_t)blockIdx.x * kEncThreads + threadIdx.x; q < n4; q += step) {
        // `self as f32` first (src/color.rs:430), then the f32 arithmetic
        const uint4 v = make_uint4(encode_mask_rgba8((float)in[4 * q]), encode_mask_rgba8((float)in[4 * q + 1]),
                                   encode_mask_rgba8((float)in[4 * q + 2]), encode_mask_rgba8((float)in[4 * q + 3]));
        __stcs(reinterpret_cast<uint4*>(out) + q, v);
    }
    const uint64_t t = (uint64_t)blockIdx.x * kEncThreads + threadIdx.x;
    if (t < (n & 3)) out[4 * n4 + t] = encode_mask_rgba8((float)in[4 * n4 + t]);
}

// Grid: 4 CTAs of 256 threads per SM (enough bytes in flight to saturate HBM),
// fewer when the image is small.
static unsigned encode_grid(uint64_t n) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    const uint64_t need = ((n >> 2) + kEncThreads - 1) / kEncThreads;
    const uint64_t cap = 4ull * (uint64_t)sms;
    return (unsigned)(need < 1 ? 1 : (need < cap ? need : cap));
}

// `in` and `out` must be 16-byte aligned (the host checks).
cudaError_t launch_encode_rgba8(const float* in, uint8_t* out, uint64_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_encode_rgba8<<<encode_grid(n), kEncThreads, 0, st>>>(reinterpret_cast<const float4*>(in),
                                                            reinterpret_cast<uint32_t*>(out), n);
    return cudaGetLastError();
}

cudaError_t launch_encode_mask_rgba8(const void* in, int elem_size, uint8_t* out, uint64_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    if (elem_size == 8)
        k_encode_mask_rgba8<double><<<encode_grid(n), kEncThreads, 0, st>>>(static_cast<const double*>(in),
                                                                             reinterpret_cast<uint32_t*>(out), n);
    else
        k_encode_mask_rgba8<float><<<encode_grid(n), kEncThreads, 0, st>>>(static_cast<const float*>(in),
                                                                            reinterpret_cast<uint32_t*>(out), n);
    return cudaGetLastError();
}

}  // namespace rz
