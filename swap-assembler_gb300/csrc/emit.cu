// On-device emission of the two text outputs of a built graph: the node
// lines with their 8 multiplicities (printLocalNodeGraph, graph.cpp:569) and
// the -s adjacency file kmerGraph.txt (printKmerGraph, graph.cpp:3352-3440,
// with node::getNodeID's neighbour ids, graph.cpp:164-196). The lines are
// ordered by their first token on the device (CUB radix sort), every line's
// length is computed, scanned, and each thread formats its line into one
// device text buffer, which is streamed to the file through two pinned host
// buffers (copy of chunk i+1 overlaps the fwrite of chunk i). Byte-identical
// with the host writers in writers.cpp.
#include <cuda_runtime.h>

#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <cstdio>
#include <string>

#include "swg_internal.h"
#include "text_dev.cuh"

namespace swg {
namespace {

// ---- node lines: "K A# # ... # m0 .. m7\n" (arc string "ACGT"[s%4] iff m_s != 0)
__global__ void k_node_len(const unsigned long long *__restrict__ mult, const unsigned long long *__restrict__ keys,
                           uint64_t n, uint64_t *__restrict__ len) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t m = mult[i];
    uint64_t l = (uint64_t)ndig(keys[i]) + 1;  // key and the newline
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        const unsigned v = (unsigned)(m >> (8 * s)) & 0xffu;
        l += 2 + (v != 0) + 1 + (uint64_t)ndig(v);  // " A#" or " #", then " m"
    }
    len[i] = l;
}

__global__ void k_node_write(const unsigned long long *__restrict__ mult, const unsigned long long *__restrict__ keys,
                             uint64_t n, const uint64_t *__restrict__ off, char *__restrict__ text) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t m = mult[i];
    char *p = put_u64(text + off[i], keys[i]);
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        *p++ = ' ';
        if ((m >> (8 * s)) & 0xffu) *p++ = "ACGT"[s & 3];
        *p++ = '#';
    }
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        *p++ = ' ';
        p = put_u64(p, (m >> (8 * s)) & 0xffu);
    }
    *p = '\n';
}

// ---- kmerGraph.txt: per node a line "K n.." for the set slots 0-3 and a
// line "rc(K) n.." for the set slots 4-7; lines ordered by first token.
__global__ void k_kg_count(const unsigned long long *__restrict__ mult, uint64_t n, uint64_t *__restrict__ cnt) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t m = mult[i];
    cnt[i] = (uint64_t)((m & 0xffffffffull) != 0) + (uint64_t)((m >> 32) != 0);
}

__global__ void k_kg_entries(const unsigned long long *__restrict__ keys, const unsigned long long *__restrict__ mult,
                             uint64_t n, int k, const uint64_t *__restrict__ pos,
                             unsigned long long *__restrict__ tok, unsigned long long *__restrict__ idx) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t m = mult[i];
    uint64_t p = pos[i];
    if (m & 0xffffffffull) {
        tok[p] = keys[i];
        idx[p++] = 2 * i;
    }
    if (m >> 32) {
        tok[p] = rc_dev(keys[i], k);
        idx[p] = 2 * i + 1;
    }
}

__global__ void k_kg_len(const unsigned long long *__restrict__ tok, const unsigned long long *__restrict__ idx,
                         uint64_t lines, const unsigned long long *__restrict__ keys,
                         const unsigned long long *__restrict__ mult, int k, uint64_t *__restrict__ len) {
    const uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= lines) return;
    const uint64_t i = idx[q] >> 1;
    const int half = (int)(idx[q] & 1);
    const uint64_t m = mult[i], key = keys[i];
    uint64_t l = (uint64_t)ndig(tok[q]) + 1;
    for (int s = 4 * half; s < 4 * half + 4; ++s)
        if ((m >> (8 * s)) & 0xffu) l += 1 + (uint64_t)ndig(neighbour_dev(key, s, k));
    len[q] = l;
}

__global__ void k_kg_write(const unsigned long long *__restrict__ tok, const unsigned long long *__restrict__ idx,
                           uint64_t lines, const unsigned long long *__restrict__ keys,
                           const unsigned long long *__restrict__ mult, int k, const uint64_t *__restrict__ off,
                           char *__restrict__ text) {
    const uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= lines) return;
    const uint64_t i = idx[q] >> 1;
    const int half = (int)(idx[q] & 1);
    const uint64_t m = mult[i], key = keys[i];
    char *p = put_u64(text + off[q], tok[q]);
    for (int s = 4 * half; s < 4 * half + 4; ++s) {
        if (!((m >> (8 * s)) & 0xffu)) continue;
        *p++ = ' ';
        p = put_u64(p, neighbour_dev(key, s, k));
    }
    *p = '\n';
}

inline unsigned blocks_for(uint64_t n) { return (unsigned)((n + 255) / 256); }

}  // namespace

swg_status cuda_err(cudaError_t e, const char *what) {
    cudaGetLastError();
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? SWG_ERR_OOM : SWG_ERR_CUDA;
}


// Exclusive prefix of len[0..n) into off[0..n], off[n] = total (bytes).
swg_status scan_lengths(const uint64_t *len, uint64_t *off, uint64_t n, Scratch &scr, cudaStream_t s) {
    uint64_t *tmp = nullptr;
    if (!scr.get(&tmp, gscan_scratch(n))) return cuda_err(cudaErrorMemoryAllocation, "scan scratch");
    launch_gscan(len, off, n, tmp, off + n, s);
    return SWG_OK;
}

// Writes text[0..bytes) to path: 64 MiB chunks copied into two pinned
// buffers in turn; the copy of one chunk overlaps the fwrite of the other.
swg_status stream_to_file(const char *d_text, uint64_t bytes, const char *path, cudaStream_t s) {
    FILE *fp = std::fopen(path, "wb");
    if (!fp) {
        set_error(std::string("cannot open ") + path);
        return SWG_ERR_IO;
    }
    constexpr uint64_t kChunk = 64ull << 20;
    char *h[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    swg_status st = SWG_OK;
    cudaError_t e = cudaSuccess;
    for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
        e = cudaHostAlloc((void **)&h[b], std::min(kChunk, std::max<uint64_t>(bytes, 1)), cudaHostAllocDefault);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[b], cudaEventDisableTiming);
    }
    const uint64_t chunks = (bytes + kChunk - 1) / kChunk;
    if (e == cudaSuccess && chunks) {
        e = cudaMemcpyAsync(h[0], d_text, std::min(kChunk, bytes), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaEventRecord(ev[0], s);
    }
    for (uint64_t c = 0; c < chunks && e == cudaSuccess && st == SWG_OK; ++c) {
        const int b = (int)(c & 1);
        if (c + 1 < chunks) {  // the next chunk's copy goes out before this one is written
            const uint64_t o = (c + 1) * kChunk;
            e = cudaMemcpyAsync(h[b ^ 1], d_text + o, std::min(kChunk, bytes - o), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaEventRecord(ev[b ^ 1], s);
            if (e != cudaSuccess) break;
        }
        e = cudaEventSynchronize(ev[b]);
        if (e != cudaSuccess) break;
        const uint64_t nb = std::min(kChunk, bytes - c * kChunk);
        if (std::fwrite(h[b], 1, nb, fp) != nb) st = SWG_ERR_IO;
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    for (int b = 0; b < 2; ++b) {
        if (ev[b]) cudaEventDestroy(ev[b]);
        if (h[b]) cudaFreeHost(h[b]);
    }
    const bool closed = std::fclose(fp) == 0;
    if (e != cudaSuccess) return cuda_err(e, "streaming the text to the file");
    if (st != SWG_OK || !closed) {
        set_error(std::string("write failed: ") + path);
        return SWG_ERR_IO;
    }
    return SWG_OK;
}

swg_status emit_node_lines(const unsigned long long *d_keys, const unsigned long long *d_mult, uint64_t n,
                           int k, const char *path, cudaStream_t s) {
    Scratch scr(s);
    unsigned long long *keys = nullptr, *mult = nullptr;
    uint64_t *len = nullptr, *off = nullptr;
    if (!scr.get(&keys, n) || !scr.get(&mult, n) || !scr.get(&len, n) || !scr.get(&off, n + 1))
        return cuda_err(cudaErrorMemoryAllocation, "node-line scratch");
    if (n) {  // order by key
        size_t tb = 0;
        EMIT_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb, d_keys, keys, d_mult, mult, (int64_t)n, 0, 2 * k, s),
                  "sort size");
        unsigned char *tmp = nullptr;
        if (!scr.get(&tmp, tb)) return cuda_err(cudaErrorMemoryAllocation, "sort scratch");
        EMIT_CUDA(cub::DeviceRadixSort::SortPairs(tmp, tb, d_keys, keys, d_mult, mult, (int64_t)n, 0, 2 * k, s),
                  "sort");
        k_node_len<<<blocks_for(n), 256, 0, s>>>(mult, keys, n, len);
    }
    swg_status st = scan_lengths(len, off, n, scr, s);
    if (st) return st;
    uint64_t bytes = 0;
    EMIT_CUDA(cudaMemcpyAsync(&bytes, off + n, 8, cudaMemcpyDeviceToHost, s), "text size");
    EMIT_CUDA(cudaStreamSynchronize(s), "text size");
    char *text = nullptr;
    if (!scr.get(&text, bytes)) return cuda_err(cudaErrorMemoryAllocation, "node-line text");
    if (n) k_node_write<<<blocks_for(n), 256, 0, s>>>(mult, keys, n, off, text);
    EMIT_CUDA(cudaGetLastError(), "node-line kernels");
    return stream_to_file(text, bytes, path, s);
}

swg_status emit_kmer_graph(const unsigned long long *d_keys, const unsigned long long *d_mult, uint64_t n, int k,
                           const char *path, cudaStream_t s) {
    if (k < 8 || k > 31) {
        set_error("kmerGraph.txt needs 8 <= k <= 31 (the reference indexes the slot as a base position)");
        return SWG_ERR_BAD_INPUT;
    }
    Scratch scr(s);
    uint64_t *cnt = nullptr, *pos = nullptr;
    if (!scr.get(&cnt, n) || !scr.get(&pos, n + 1)) return cuda_err(cudaErrorMemoryAllocation, "line scratch");
    if (n) k_kg_count<<<blocks_for(n), 256, 0, s>>>(d_mult, n, cnt);
    swg_status st = scan_lengths(cnt, pos, n, scr, s);
    if (st) return st;
    uint64_t lines = 0;
    EMIT_CUDA(cudaMemcpyAsync(&lines, pos + n, 8, cudaMemcpyDeviceToHost, s), "line count");
    EMIT_CUDA(cudaStreamSynchronize(s), "line count");
    unsigned long long *tok = nullptr, *idx = nullptr, *tok2 = nullptr, *idx2 = nullptr;
    uint64_t *len = nullptr, *off = nullptr;
    if (!scr.get(&tok, lines) || !scr.get(&idx, lines) || !scr.get(&tok2, lines) || !scr.get(&idx2, lines) ||
        !scr.get(&len, lines) || !scr.get(&off, lines + 1))
        return cuda_err(cudaErrorMemoryAllocation, "line scratch");
    if (lines) {
        k_kg_entries<<<blocks_for(n), 256, 0, s>>>(d_keys, d_mult, n, k, pos, tok, idx);
        size_t tb = 0;
        EMIT_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb, tok, tok2, idx, idx2, (int64_t)lines, 0, 2 * k, s),
                  "sort size");
        unsigned char *tmp = nullptr;
        if (!scr.get(&tmp, tb)) return cuda_err(cudaErrorMemoryAllocation, "sort scratch");
        EMIT_CUDA(cub::DeviceRadixSort::SortPairs(tmp, tb, tok, tok2, idx, idx2, (int64_t)lines, 0, 2 * k, s),
                  "sort");
        k_kg_len<<<blocks_for(lines), 256, 0, s>>>(tok2, idx2, lines, d_keys, d_mult, k, len);
    }
    st = scan_lengths(len, off, lines, scr, s);
    if (st) return st;
    uint64_t bytes = 0;
    EMIT_CUDA(cudaMemcpyAsync(&bytes, off + lines, 8, cudaMemcpyDeviceToHost, s), "text size");
    EMIT_CUDA(cudaStreamSynchronize(s), "text size");
    char *text = nullptr;
    if (!scr.get(&text, bytes)) return cuda_err(cudaErrorMemoryAllocation, "kmerGraph text");
    if (lines) k_kg_write<<<blocks_for(lines), 256, 0, s>>>(tok2, idx2, lines, d_keys, d_mult, k, off, text);
    EMIT_CUDA(cudaGetLastError(), "kmerGraph kernels");
    return stream_to_file(text, bytes, path, s);
}

}  // namespace swg
