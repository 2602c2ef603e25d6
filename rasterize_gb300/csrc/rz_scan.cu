// rz_scan.cu -- device-wide exclusive prefix sum of uint32 counts.
//
// Used by the line pipeline to turn per-slot line counts into line offsets
// (the "warp-level exclusive scan" that allocates output slots) and
// per-(fill, band) counts into list starts.  Blocks of 1024 elements: each
// block scans its elements with warp shuffles and writes its total; the
// totals are scanned the same way (recursively) and added back.
#include <cuda_runtime.h>
#include <stdint.h>

namespace rz {

constexpr int kScanBlock = 1024;

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
    const int lane = threadIdx.x & 31;
    #pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t o = __shfl_up_sync(0xffffffffu, v, off);
        if (lane >= off) v += o;
    }
    return v;
}

// In-place exclusive scan of each 1024-element block; block totals to `sums`.
__global__ void __launch_bounds__(kScanBlock) k_scan_blocks(uint32_t* data, uint64_t n, uint32_t* sums) {
    __shared__ uint32_t warp_tot[32];
    const uint64_t i = (uint64_t)blockIdx.x * kScanBlock + threadIdx.x;
    const uint32_t v = i < n ? data[i] : 0u;
    const uint32_t incl = warp_incl_scan(v);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const uint32_t t = warp_tot[lane];
        const uint32_t ti = warp_incl_scan(t);
        warp_tot[lane] = ti - t;  // exclusive warp offsets
        if (lane == 31 && sums) sums[blockIdx.x] = ti;
    }
    __syncthreads();
    if (i < n) data[i] = warp_tot[warp] + incl - v;
}

__global__ void k_scan_add(uint32_t* data, uint64_t n, const uint32_t* offsets) {
    const uint64_t i = (uint64_t)blockIdx.x * kScanBlock + threadIdx.x;
    if (i < n && blockIdx.x > 0) data[i] += offsets[blockIdx.x];
}

// Temporary words needed by scan_u32 for n elements.
uint64_t scan_temp_words(uint64_t n) {
    uint64_t words = 0;
    while (n > (uint64_t)kScanBlock) {
        n = (n + kScanBlock - 1) / kScanBlock;
        words += n;
    }
    return words + 1;
}

// Exclusive scan of data[0, n) in place.  temp holds scan_temp_words(n) words.
cudaError_t scan_u32(uint32_t* data, uint64_t n, uint32_t* temp, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    const uint64_t blocks = (n + kScanBlock - 1) / kScanBlock;
    if (blocks == 1) {
        k_scan_blocks<<<1, kScanBlock, 0, stream>>>(data, n, nullptr);
        return cudaGetLastError();
    }
    uint32_t* sums = temp;
    k_scan_blocks<<<(unsigned)blocks, kScanBlock, 0, stream>>>(data, n, sums);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = scan_u32(sums, blocks, temp + blocks, stream);
    if (e != cudaSuccess) return e;
    k_scan_add<<<(unsigned)blocks, kScanBlock, 0, stream>>>(data, n, sums);
    return cudaGetLastError();
}

}  // namespace rz
