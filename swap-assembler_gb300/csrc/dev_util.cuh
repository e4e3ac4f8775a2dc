// Device helpers shared by the .cu files of the library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace swg {

// Block-wide exclusive scan of one uint64 per thread (blockDim = NT).
template <int NT>
__device__ __forceinline__ uint64_t block_exclusive_scan(uint64_t v, uint64_t *warp_buf,
                                                         uint64_t *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint64_t y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) warp_buf[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint64_t w = lane < NT / 32 ? warp_buf[lane] : 0;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint64_t y = __shfl_up_sync(0xffffffffu, w, d);
            if (lane >= d) w += y;
        }
        if (lane < NT / 32) warp_buf[lane] = w;
    }
    __syncthreads();
    const uint64_t warp_prefix = warp ? warp_buf[warp - 1] : 0;
    if (total) *total = warp_buf[NT / 32 - 1];
    __syncthreads();
    return warp_prefix + x - v;
}


}  // namespace swg
