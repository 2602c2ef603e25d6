// rz_encode.cu -- output encode: premultiplied linear RGBA f32 (or a mask) to
// sRGB8 RGBA bytes, the per-pixel `Color::to_rgba` that the reference's image
// writers call (src/image.rs:136-229).  Streaming work: 16 (or 4 / 8) bytes
// read and 4 written per pixel.  A warp reads 32 consecutive pixels per load
// (512 bytes for RGBA f32) and writes 32 consecutive words; each thread keeps
// 4 loads in flight, in a grid-stride loop sized to the SM count.
#include <cuda_runtime.h>

#include "rz_color.cuh"

namespace rz {

constexpr int kEncThreads = 256;
constexpr int kEncPerThread = 4;

__global__ void __launch_bounds__(kEncThreads) k_encode_rgba8(const float4* __restrict__ in, uint32_t* __restrict__ out,
                                                              uint64_t n) {
    const uint64_t step = (uint64_t)gridDim.x * kEncThreads * kEncPerThread;
    for (uint64_t base = (uint64_t)blockIdx.x * kEncThreads * kEncPerThread + threadIdx.x; base < n; base += step) {
        float4 v[kEncPerThread];
        #pragma unroll
        for (int j = 0; j < kEncPerThread; ++j) {
            const uint64_t i = base + (uint64_t)j * kEncThreads;
            if (i < n) v[j] = __ldcs(in + i);
        }
        #pragma unroll
        for (int j = 0; j < kEncPerThread; ++j) {
            const uint64_t i = base + (uint64_t)j * kEncThreads;
            if (i < n) __stcs(out + i, encode_lin_rgba8(v[j]));
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(kEncThreads) k_encode_mask_rgba8(const T* __restrict__ in, uint32_t* __restrict__ out,
                                                                   uint64_t n) {
    const uint64_t step = (uint64_t)gridDim.x * kEncThreads * kEncPerThread;
    for (uint64_t base = (uint64_t)blockIdx.x * kEncThreads * kEncPerThread + threadIdx.x; base < n; base += step) {
        T v[kEncPerThread];
        #pragma unroll
        for (int j = 0; j < kEncPerThread; ++j) {
            const uint64_t i = base + (uint64_t)j * kEncThreads;
            if (i < n) v[j] = __ldcs(in + i);
        }
        #pragma unroll
        for (int j = 0; j < kEncPerThread; ++j) {
            const uint64_t i = base + (uint64_t)j * kEncThreads;
            // `self as f32` first (src/color.rs:430), then the f32 arithmetic
            if (i < n) __stcs(out + i, encode_mask_rgba8((float)v[j]));
        }
    }
}

// Grid: 8 CTAs of 256 threads per SM (as many as the registers allow resident,
// the rest queue), fewer when the image is small.
static unsigned encode_grid(uint64_t n) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    const uint64_t per_cta = (uint64_t)kEncThreads * kEncPerThread;
    const uint64_t need = (n + per_cta - 1) / per_cta;
    const uint64_t cap = 8ull * (uint64_t)sms;
    return (unsigned)(need < 1 ? 1 : (need < cap ? need : cap));
}

// `in` is 16-byte aligned and `out` 4-byte aligned (the host checks).
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
