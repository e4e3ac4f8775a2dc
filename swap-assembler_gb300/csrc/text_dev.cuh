// Device helpers shared by the text writers (emit.cu, merge.cu): decimal
// formatting, reverse complement, stream-ordered scratch.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "swg_internal.h"

namespace swg {

static __constant__ unsigned long long kPow10[20] = {
    1ull, 10ull, 100ull, 1000ull, 10000ull,
    100000ull, 1000000ull, 10000000ull, 100000000ull, 1000000000ull,
    10000000000ull, 100000000000ull, 1000000000000ull, 10000000000000ull, 100000000000000ull,
    1000000000000000ull, 10000000000000000ull, 100000000000000000ull, 1000000000000000000ull, 10000000000000000000ull};

// Decimal digits of v ("%llu").
__device__ __forceinline__ int ndig(uint64_t v) {
    int d = 1;
#pragma unroll
    for (int i = 1; i < 20; ++i) d += v >= kPow10[i];
    return d;
}

__device__ __forceinline__ char *put_u64(char *p, uint64_t v) {
    const int d = ndig(v);
    for (int j = d - 1; j >= 0; --j) {
        p[j] = (char)('0' + (int)(v % 10));
        v /= 10;
    }
    return p + d;
}

// Reverse complement of a k-mer in the low 2k bits (kmerGraph.cpp:5-14):
// complement = bitwise NOT, reverse the 2-bit groups (bit reverse + swap of
// the bits inside each group).
__device__ __forceinline__ uint64_t rc_dev(uint64_t a, int k) {
    const uint64_t r = __brevll(~a);
    const uint64_t s = ((r >> 1) & 0x5555555555555555ull) | ((r & 0x5555555555555555ull) << 1);
    return s >> (64 - 2 * k);
}

// Neighbour id printed for slot s of key K (the host kmer_graph_neighbour):
// descriptor K (s < 4) or rc(K) (s >= 4), base s%4 appended, last k bases N;
// N if canonical, else complement(N) with base s flipped back (k odd) — the
// reference's nReverseStr[i] indexing (graph.cpp:3393,3423).
__device__ __forceinline__ uint64_t neighbour_dev(uint64_t key, int slot, int k) {
    const uint64_t kmask = (1ull << (2 * k)) - 1;
    const uint64_t d = slot < 4 ? key : rc_dev(key, k);
    const uint64_t nn = ((d << 2) | (uint64_t)(slot & 3)) & kmask;
    if (nn >= rc_dev(nn, k)) return nn;
    uint64_t out = nn ^ kmask;
    if (k & 1) out ^= 3ull << (2 * (k - 1 - slot));
    return out;
}

// Stream-ordered device scratch, freed on every return path.
// With a pool, from that pool (one that keeps its memory for reuse).
struct Scratch {
    cudaStream_t s;
    cudaMemPool_t pool;
    void *p[48] = {};
    int n = 0;
    explicit Scratch(cudaStream_t st, cudaMemPool_t mp = nullptr) : s(st), pool(mp) {}
    template <typename T>
    bool get(T **out, uint64_t count) {
        *out = nullptr;
        if (n == 48) return false;
        const size_t bytes = std::max<uint64_t>(count, 1) * sizeof(T);
        const cudaError_t e = pool ? cudaMallocFromPoolAsync((void **)out, bytes, pool, s)
                                   : cudaMallocAsync((void **)out, bytes, s);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        p[n++] = *out;
        return true;
    }
    ~Scratch() {
        for (int i = 0; i < n; ++i) cudaFreeAsync(p[i], s);
    }
};

#define EMIT_CUDA(call, what)                           \
    do {                                                \
        const cudaError_t e_ = (call);                  \
        if (e_ != cudaSuccess) return cuda_err(e_, what); \
    } while (0)

// Error status for a failed CUDA call (message kept for swg_last_error).
swg_status cuda_err(cudaError_t e, const char *what);
// Exclusive prefix of len[0..n) into off[0..n], off[n] = total.
swg_status scan_lengths(const uint64_t *len, uint64_t *off, uint64_t n, Scratch &scr, cudaStream_t s);

}  // namespace swg
