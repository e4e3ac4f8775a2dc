// FASTA framing and 2-bit packing on the device.
//
// Same framing as the host path (and the reference, kmerGraph.cpp:113-114,
// 160-233): from the first '>', lines alternate header / ONE sequence line;
// acgt upper-cased, any other byte read as 'A'; sequences shorter than k
// dropped. Steps: newlines per 4 KiB chunk -> scan -> every newline's
// position -> record r = (line 2r, line 2r+1) -> keep sequences of length >= k
// -> scan of kept reads and of their 16-base words -> pack. Every read starts
// on a word boundary of the packed stream (read_off is a multiple of 16), so
// each packed word belongs to one read and is written by one thread.
#include <cuda_runtime.h>

#include "dev_util.cuh"
#include "swg_internal.h"

namespace swg {
namespace {

constexpr int kFBlock = 256;
constexpr int kFBytes = 16;
constexpr uint64_t kFChunk = (uint64_t)kFBlock * kFBytes;  // bytes per block
constexpr int kGItems = 8;
constexpr uint64_t kGChunk = (uint64_t)kFBlock * kGItems;  // items per scan block

__device__ __forceinline__ void load16(const unsigned char *__restrict__ t, uint64_t n, uint64_t i,
                                       unsigned char b[kFBytes]) {
    if (i + kFBytes <= n) {
        const uint4 v = *reinterpret_cast<const uint4 *>(t + i);  // i is a multiple of 16
        const unsigned w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int j = 0; j < kFBytes; ++j) b[j] = (unsigned char)(w[j >> 2] >> (8 * (j & 3)));
    } else {
#pragma unroll
        for (int j = 0; j < kFBytes; ++j) b[j] = i + j < n ? t[i + j] : (unsigned char)1;
    }
}

// Newlines per chunk; any NUL byte raises flag.
__global__ void __launch_bounds__(kFBlock) k_nl_count(const unsigned char *__restrict__ t, uint64_t n,
                                                      uint64_t *__restrict__ counts,
                                                      unsigned *__restrict__ flag) {
    __shared__ uint64_t wb[kFBlock / 32];
    unsigned char b[kFBytes];
    load16(t, n, (uint64_t)blockIdx.x * kFChunk + (uint64_t)threadIdx.x * kFBytes, b);
    unsigned c = 0, z = 0;
#pragma unroll
    for (int j = 0; j < kFBytes; ++j) {
        c += b[j] == '\n';
        z |= b[j] == 0;
    }
    uint64_t total;
    block_exclusive_scan<kFBlock>(c, wb, &total);
    if (threadIdx.x == 0) counts[blockIdx.x] = total;
    if (z) atomicOr(flag, 1u);
}

// Position of every newline, in order.
__global__ void __launch_bounds__(kFBlock) k_nl_pos(const unsigned char *__restrict__ t, uint64_t n,
                                                    const uint64_t *__restrict__ chunk_base,
                                                    uint64_t *__restrict__ nl) {
    __shared__ uint64_t wb[kFBlock / 32];
    const uint64_t base = (uint64_t)blockIdx.x * kFChunk + (uint64_t)threadIdx.x * kFBytes;
    unsigned char b[kFBytes];
    load16(t, n, base, b);
    unsigned c = 0;
#pragma unroll
    for (int j = 0; j < kFBytes; ++j) c += b[j] == '\n';
    uint64_t pos = chunk_base[blockIdx.x] + block_exclusive_scan<kFBlock>(c, wb, nullptr);
#pragma unroll
    for (int j = 0; j < kFBytes; ++j)
        if (b[j] == '\n') nl[pos++] = base + j;
}

// Generic exclusive scan of uint64 (in place allowed).
__global__ void __launch_bounds__(kFBlock) k_gscan_reduce(const uint64_t *__restrict__ in, uint64_t n,
                                                          uint64_t *__restrict__ sums) {
    __shared__ uint64_t wb[kFBlock / 32];
    const uint64_t base = (uint64_t)blockIdx.x * kGChunk;
    uint64_t s = 0;
    for (int it = 0; it < kGItems; ++it) {
        const uint64_t i = base + (uint64_t)it * kFBlock + threadIdx.x;
        if (i < n) s += in[i];
    }
    uint64_t total;
    block_exclusive_scan<kFBlock>(s, wb, &total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024) k_gscan_blocks(uint64_t *sums, uint64_t nb, uint64_t *total) {
    __shared__ uint64_t wb[32];
    __shared__ uint64_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint64_t base = 0; base < nb; base += 1024) {
        const uint64_t i = base + threadIdx.x;
        const uint64_t v = i < nb ? sums[i] : 0;
        uint64_t t;
        const uint64_t ex = block_exclusive_scan<1024>(v, wb, &t);
        const uint64_t c = carry;
        if (i < nb) sums[i] = c + ex;
        __syncthreads();
        if (threadIdx.x == 0) carry = c + t;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void __launch_bounds__(kFBlock) k_gscan_write(const uint64_t *in, uint64_t n,
                                                         const uint64_t *__restrict__ sums,
                                                         uint64_t *out) {
    __shared__ uint64_t wb[kFBlock / 32];
    const uint64_t base = (uint64_t)blockIdx.x * kGChunk + (uint64_t)threadIdx.x * kGItems;
    uint64_t v[kGItems];
    uint64_t s = 0;
#pragma unroll
    for (int it = 0; it < kGItems; ++it) {
        v[it] = base + it < n ? in[base + it] : 0;
        s += v[it];
    }
    uint64_t run = sums[blockIdx.x] + block_exclusive_scan<kFBlock>(s, wb, nullptr);
#pragma unroll
    for (int it = 0; it < kGItems; ++it) {
        if (base + it < n) out[base + it] = run;
        run += v[it];
    }
}

// Record r: header line 2r, sequence line 2r+1 (line 0 starts at byte 0).
__global__ void k_rec_len(const uint64_t *__restrict__ nl, uint64_t n_rec, int k,
                          uint64_t *__restrict__ keep, uint64_t *__restrict__ words) {
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_rec) return;
    const uint64_t start = nl[2 * r] + 1, end = nl[2 * r + 1];
    const uint64_t L = end - start;
    const bool ok = L >= (uint64_t)k;
    keep[r] = ok ? 1 : 0;
    words[r] = ok ? (L + 15) / 16 : 0;
}

__device__ __forceinline__ uint32_t code_of(unsigned char ch) {
    switch (ch) {
        case 'C': case 'c': return 1u;
        case 'G': case 'g': return 2u;
        case 'T': case 't': return 3u;
        default: return 0u;
    }
}

// One warp per record: kept reads get their offset/length and packed words.
__global__ void k_rec_pack(const unsigned char *__restrict__ t, const uint64_t *__restrict__ nl,
                           uint64_t n_rec, int k, const uint64_t *__restrict__ read_idx,
                           const uint64_t *__restrict__ word_off, uint64_t *__restrict__ off,
                           uint32_t *__restrict__ len, uint32_t *__restrict__ packed) {
    const uint64_t r = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (r >= n_rec) return;
    const uint64_t start = nl[2 * r] + 1, end = nl[2 * r + 1];
    const uint64_t L = end - start;
    if (L < (uint64_t)k) return;
    const uint64_t w0 = word_off[r];
    if (lane == 0) {
        const uint64_t ri = read_idx[r];
        off[ri] = w0 * 16;
        len[ri] = (uint32_t)L;
    }
    const uint64_t nw = (L + 15) / 16;
    for (uint64_t w = lane; w < nw; w += 32) {
        uint32_t word = 0;
        const uint64_t p = start + w * 16;
#pragma unroll
        for (int j = 0; j < 16; ++j)
            if (p + j < end) word |= code_of(t[p + j]) << (30 - 2 * j);
        packed[w0 + w] = word;
    }
}

}  // namespace

uint64_t framing_chunks(uint64_t n) { return (n + kFChunk - 1) / kFChunk; }

uint64_t gscan_scratch(uint64_t n) { return (n + kGChunk - 1) / kGChunk + 1; }

int launch_gscan(const uint64_t *in, uint64_t *out, uint64_t n, uint64_t *scratch, uint64_t *total,
                 cudaStream_t s) {
    const uint64_t nb = (n + kGChunk - 1) / kGChunk;
    if (nb == 0) {
        cudaMemsetAsync(total, 0, sizeof(uint64_t), s);
        return 0;
    }
    k_gscan_reduce<<<(unsigned)nb, kFBlock, 0, s>>>(in, n, scratch);
    k_gscan_blocks<<<1, 1024, 0, s>>>(scratch, nb, total);
    k_gscan_write<<<(unsigned)nb, kFBlock, 0, s>>>(in, n, scratch, out);
    return 3;
}

int launch_nl_count(const unsigned char *t, uint64_t n, uint64_t *counts, unsigned *flag,
                    cudaStream_t s) {
    const uint64_t nc = framing_chunks(n);
    if (!nc) return 0;
    k_nl_count<<<(unsigned)nc, kFBlock, 0, s>>>(t, n, counts, flag);
    return 1;
}

int launch_nl_pos(const unsigned char *t, uint64_t n, const uint64_t *chunk_base, uint64_t *nl,
                  cudaStream_t s) {
    const uint64_t nc = framing_chunks(n);
    if (!nc) return 0;
    k_nl_pos<<<(unsigned)nc, kFBlock, 0, s>>>(t, n, chunk_base, nl);
    return 1;
}

int launch_rec_len(const uint64_t *nl, uint64_t n_rec, int k, uint64_t *keep, uint64_t *words,
                   cudaStream_t s) {
    if (!n_rec) return 0;
    k_rec_len<<<(unsigned)((n_rec + 255) / 256), 256, 0, s>>>(nl, n_rec, k, keep, words);
    return 1;
}

int launch_rec_pack(const unsigned char *t, const uint64_t *nl, uint64_t n_rec, int k,
                    const uint64_t *read_idx, const uint64_t *word_off, uint64_t *off,
                    uint32_t *len, uint32_t *packed, cudaStream_t s) {
    if (!n_rec) return 0;
    const uint64_t threads = n_rec * 32;
    k_rec_pack<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(t, nl, n_rec, k, read_idx,
                                                                 word_off, off, len, packed);
    return 1;
}

}  // namespace swg
