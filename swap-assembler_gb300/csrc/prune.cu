// Two of the reference's rank-0 passes over the merged graph, on the device:
// masterTipsRemoval (graph.cpp:2194-2265) and masterLowCoverageEdgeRemoval
// (graph.cpp:2267-2300). They work on the merged graph's lines (node key, per
// arc slot its length, multiplicity, string offset and the far end's arc
// back) and then rewrite its text (gathered node lines in key order, deleted
// and arc-less nodes left out as gatherDistNodeGraph does, graph.cpp:587-596).
//
// Tips: a node with exactly one arc, shorter than k, loses that arc, so does
// the far node's arc back, and the node is deleted. The reference visits the
// nodes in its node map's order, removing tips as it meets them; here every
// node that is a tip when the pass starts is judged on that state — the same
// as visiting all other nodes first and then the tips in key order. Of two
// tips whose arcs join them to each other, the one with the smaller key is
// deleted and the other keeps no arc. An arc that leads back to its own node
// is left alone (graph.cpp:2244).
//
// Low coverage: avg = sum(len * m) / sum(len) over the arcs of the nodes left
// (integer division); every arc shorter than 2k with m < avg / 4 is cut (both
// ends' arcs meet the test alike, having the same length and multiplicity).
// The reference divides by zero when no arc is left; here nothing is cut.
#include <cuda_runtime.h>

#include <cooperative_groups.h>
#include <cooperative_groups/reduce.h>

#include <algorithm>
#include <cstdint>

#include "swg_internal.h"
#include "text_dev.cuh"

namespace swg {
namespace {

namespace cg = cooperative_groups;

constexpr unsigned char kNoTip = 8;

__device__ __forceinline__ void agg_add(unsigned long long *ctr, unsigned long long v) {
    cg::coalesced_group g = cg::coalesced_threads();
    const unsigned long long sum = cg::reduce(g, v, cg::plus<unsigned long long>());
    if (g.thread_rank() == 0) atomicAdd(ctr, sum);
}

// The slot of a node's one arc when the node is a tip, else kNoTip.
__global__ void k_pr_tipslot(MergedGraph m, unsigned char *__restrict__ tip) {
    const uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= m.lines) return;
    unsigned char t = kNoTip;
    if (!m.del[q]) {
        int num = 0, slot = 0;
        for (int s = 0; s < 8; ++s)
            if (m.len[8 * q + s]) ++num, slot = s;
        if (num == 1 && m.len[8 * q + slot] < (unsigned)m.k) t = (unsigned char)slot;
    }
    tip[q] = t;
}

__global__ void k_pr_tips(MergedGraph m, const unsigned char *__restrict__ tip, unsigned long long *count) {
    const uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= m.lines || tip[q] == kNoTip) return;
    const unsigned s = tip[q];
    const unsigned b = m.back[8 * q + s];
    const uint64_t far = b >> 3, fs = b & 7;
    if (far == q) return;  // the arc leads back to this node
    m.len[8 * q + s] = 0;
    m.mult[8 * q + s] = 0;
    // a tip at the far end joined only to this one: the smaller key goes first,
    // removes both arcs, and the other is left without arcs (lines are in key order)
    if (tip[far] != kNoTip && far < q) return;
    m.len[8 * far + fs] = 0;
    m.mult[8 * far + fs] = 0;
    m.del[q] = 1;
    agg_add(count, 1);
}

// sums[0] = sum(len * m), sums[1] = sum(len) over the arcs of nodes left.
__global__ void k_pr_cov(MergedGraph m, unsigned long long *sums) {
    const uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= m.lines || m.del[q]) return;
    unsigned long long cov = 0, nuc = 0;
    for (int s = 0; s < 8; ++s) {
        const unsigned l = m.len[8 * q + s];
        nuc += l;
        cov += (unsigned long long)l * m.mult[8 * q + s];
    }
    agg_add(&sums[0], cov);
    agg_add(&sums[1], nuc);
}

__global__ void k_pr_low(MergedGraph m, const unsigned long long *sums, unsigned long long *count) {
    const uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= m.lines || m.del[q]) return;
    const unsigned long long avg = sums[1] ? sums[0] / sums[1] : 0;
    unsigned cut = 0;
    for (int s = 0; s < 8; ++s) {
        const unsigned l = m.len[8 * q + s];
        // multiplicity < 0.25 * avgCoverage (graph.cpp:2294), exactly: 4 * m < avg
        if (l < 2u * (unsigned)m.k && 4ull * m.mult[8 * q + s] < avg) {
            cut += l != 0;
            m.len[8 * q + s] = 0;
            m.mult[8 * q + s] = 0;
        }
    }
    if (cut) agg_add(count, cut);
}

// ---- rewrite of the text
__global__ void k_pr_len(MergedGraph m, uint64_t *__restrict__ out, unsigned long long *printed) {
    const uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= m.lines) return;
    uint64_t sum = 0;
    if (!m.del[q])
        for (int s = 0; s < 8; ++s) sum += m.len[8 * q + s];
    out[q] = sum ? 69 + sum : 0;
    if (sum) agg_add(printed, 1);
}

__global__ void k_pr_write(MergedGraph m, const uint64_t *__restrict__ off, char *__restrict__ text) {
    const uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= m.lines || off[q + 1] == off[q]) return;
    char *const start = text + off[q];
    char *p = put_u64(start, m.key[q]);
    uint64_t vlen = 69;
    for (int s = 0; s < 8; ++s) {
        *p++ = ' ';
        const unsigned l = m.len[8 * q + s];
        m.src2[8 * q + s] = (unsigned long long)(p - text);
        p += l;
        vlen += l;
        *p++ = '#';
    }
    for (int s = 0; s < 8; ++s) {
        *p++ = ' ';
        p = put_u64(p, m.mult[8 * q + s]);
    }
    while ((uint64_t)(p - start) < vlen - 1) *p++ = ' ';
    *p = '\n';
}

// The arc strings move from the old text to the new one in 4 KiB chunks, a
// block per chunk, so that a few very long arcs (whole chains) spread over
// the GPU too: chunk counts per arc slot, their prefix, then each block finds
// its arc by binary search in the prefix.
constexpr unsigned kChunk = 4096;

__global__ void k_pr_chunks(MergedGraph m, uint64_t *__restrict__ chunks) {
    const uint64_t a = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a < 8 * m.lines) chunks[a] = (m.len[a] + kChunk - 1) / kChunk;
}

__global__ void k_pr_copy(MergedGraph m, const uint64_t *__restrict__ first, uint64_t n_chunks,
                          const char *__restrict__ from, char *__restrict__ to) {
    const uint64_t arcs = 8 * m.lines;
    for (uint64_t c = blockIdx.x; c < n_chunks; c += gridDim.x) {
        uint64_t lo = 0, hi = arcs;  // the last arc whose first chunk is <= c
        while (hi - lo > 1) {
            const uint64_t mid = (lo + hi) / 2;
            if (first[mid] <= c) lo = mid;
            else hi = mid;
        }
        const uint64_t at = (c - first[lo]) * kChunk;
        const uint64_t rest = m.len[lo] - at;
        const unsigned l = rest < kChunk ? (unsigned)rest : kChunk;
        const char *src = from + m.src[lo] + at;
        char *dst = to + m.src2[lo] + at;
        for (unsigned i = threadIdx.x; i < l; i += blockDim.x) dst[i] = src[i];
    }
}

inline unsigned blocks(uint64_t n) { return (unsigned)std::max<uint64_t>((n + 255) / 256, 1); }

// Writes the lines into the spare text, then swaps it in.
swg_status rewrite(MergedGraph *m, cudaStream_t s, Scratch &scr) {
    uint64_t *len = nullptr, *off = nullptr;
    unsigned long long *printed = nullptr;
    if (!scr.get(&len, m->lines) || !scr.get(&off, m->lines + 1) || !scr.get(&printed, 1))
        return cuda_err(cudaErrorMemoryAllocation, "rewrite workspace");
    EMIT_CUDA(cudaMemsetAsync(printed, 0, 8, s), "rewrite");
    if (m->lines) k_pr_len<<<blocks(m->lines), 256, 0, s>>>(*m, len, printed);
    swg_status st = scan_lengths(len, off, m->lines, scr, s);
    if (st) return st;
    uint64_t h[2] = {0, 0};
    EMIT_CUDA(cudaMemcpyAsync(&h[0], off + m->lines, 8, cudaMemcpyDeviceToHost, s), "text size");
    EMIT_CUDA(cudaMemcpyAsync(&h[1], printed, 8, cudaMemcpyDeviceToHost, s), "text size");
    EMIT_CUDA(cudaStreamSynchronize(s), "text size");
    const uint64_t bytes = h[0] + 1;
    if (bytes > m->text2_cap) {
        cudaFree(m->text2);
        m->text2 = nullptr;
        m->text2_cap = 0;
        EMIT_CUDA(cudaMalloc((void **)&m->text2, bytes), "merged text");
        m->text2_cap = bytes;
    }
    if (m->lines) {
        uint64_t *chunks = nullptr, *first = nullptr;
        if (!scr.get(&chunks, 8 * m->lines) || !scr.get(&first, 8 * m->lines + 1))
            return cuda_err(cudaErrorMemoryAllocation, "rewrite workspace");
        k_pr_write<<<blocks(m->lines), 256, 0, s>>>(*m, off, m->text2);
        k_pr_chunks<<<blocks(8 * m->lines), 256, 0, s>>>(*m, chunks);
        st = scan_lengths(chunks, first, 8 * m->lines, scr, s);
        if (st) return st;
        uint64_t n_chunks = 0;
        EMIT_CUDA(cudaMemcpyAsync(&n_chunks, first + 8 * m->lines, 8, cudaMemcpyDeviceToHost, s), "chunks");
        EMIT_CUDA(cudaStreamSynchronize(s), "chunks");
        if (n_chunks)
            k_pr_copy<<<(unsigned)std::min<uint64_t>(n_chunks, 1u << 20), 256, 0, s>>>(*m, first, n_chunks,
                                                                                      m->text, m->text2);
    }
    EMIT_CUDA(cudaMemsetAsync(m->text2 + h[0], '\n', 1, s), "merged text");
    EMIT_CUDA(cudaGetLastError(), "rewrite kernels");
    EMIT_CUDA(cudaStreamSynchronize(s), "rewrite");
    std::swap(m->text, m->text2);
    std::swap(m->text_cap, m->text2_cap);
    std::swap(m->src, m->src2);
    m->text_bytes = bytes;
    m->nodes = h[1];
    return SWG_OK;
}

}  // namespace

swg_status prune_tips(MergedGraph *m, cudaStream_t s, uint64_t *count) {
    Scratch scr(s);
    unsigned char *tip = nullptr;
    unsigned long long *ctr = nullptr;
    if (!scr.get(&tip, m->lines) || !scr.get(&ctr, 1)) return cuda_err(cudaErrorMemoryAllocation, "tips workspace");
    EMIT_CUDA(cudaMemsetAsync(ctr, 0, 8, s), "tips");
    if (m->lines) {
        k_pr_tipslot<<<blocks(m->lines), 256, 0, s>>>(*m, tip);
        k_pr_tips<<<blocks(m->lines), 256, 0, s>>>(*m, tip, ctr);
    }
    EMIT_CUDA(cudaMemcpyAsync(count, ctr, 8, cudaMemcpyDeviceToHost, s), "tips");
    return rewrite(m, s, scr);
}

swg_status prune_low_coverage(MergedGraph *m, cudaStream_t s, uint64_t *count) {
    Scratch scr(s);
    unsigned long long *ctr = nullptr;
    if (!scr.get(&ctr, 3)) return cuda_err(cudaErrorMemoryAllocation, "low-coverage workspace");
    EMIT_CUDA(cudaMemsetAsync(ctr, 0, 24, s), "low coverage");
    if (m->lines) {
        k_pr_cov<<<blocks(m->lines), 256, 0, s>>>(*m, ctr);
        k_pr_low<<<blocks(m->lines), 256, 0, s>>>(*m, ctr, ctr + 2);
    }
    EMIT_CUDA(cudaMemcpyAsync(count, ctr + 2, 8, cudaMemcpyDeviceToHost, s), "low coverage");
    return rewrite(m, s, scr);
}

}  // namespace swg
