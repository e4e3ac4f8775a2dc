// The reference's rank-0 passes over the merged graph that follow the merge,
// on the device: masterTipsRemoval (graph.cpp:2194-2265),
// masterLowCoverageEdgeRemoval (graph.cpp:2267-2300) and the re-merge the
// reference runs after each, masterSimplifyNodeGraph (graph.cpp:2089-2192,
// described with its kernels below). They work on the merged graph's lines (node key, per
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
#include <cstring>

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
// the GPU too: chunk counts per piece, their prefix, then each block finds
// its piece by binary search in the prefix. A piece is an arc's own string
// (its first `own` bytes, the whole arc unless a merge lengthened it) or,
// after a merge, a merged node's arc string placed inside an end's new arc.
constexpr unsigned kChunk = 4096;

struct Pieces {
    const unsigned *own;                    // per arc slot: bytes of its old string (nullptr: len)
    uint64_t n;                             // extra pieces
    const unsigned long long *src;          // old-text offset
    const unsigned *len;
    const unsigned *arc;                    // the arc slot whose new string receives it
    const unsigned long long *at;           // offset inside that string
};

__device__ __forceinline__ unsigned own_len(const MergedGraph &m, const Pieces &x, uint64_t a) {
    if (m.del[a >> 3]) return 0;
    return x.own ? x.own[a] : m.len[a];
}

__global__ void k_pr_chunks(MergedGraph m, Pieces x, uint64_t *__restrict__ chunks) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t arcs = 8 * m.lines;
    if (i < arcs) chunks[i] = (own_len(m, x, i) + kChunk - 1) / kChunk;
    else if (i < arcs + x.n) chunks[i] = (x.len[i - arcs] + kChunk - 1) / kChunk;
}

__global__ void k_pr_copy(MergedGraph m, Pieces x, const uint64_t *__restrict__ first, uint64_t n_chunks,
                          const char *__restrict__ from, char *__restrict__ to) {
    const uint64_t arcs = 8 * m.lines, pieces = arcs + x.n;
    for (uint64_t c = blockIdx.x; c < n_chunks; c += gridDim.x) {
        uint64_t lo = 0, hi = pieces;  // the last piece whose first chunk is <= c
        while (hi - lo > 1) {
            const uint64_t mid = (lo + hi) / 2;
            if (first[mid] <= c) lo = mid;
            else hi = mid;
        }
        const uint64_t at = (c - first[lo]) * kChunk;
        uint64_t src, dst, len;
        if (lo < arcs) {
            src = m.src[lo];
            dst = m.src2[lo];
            len = own_len(m, x, lo);
        } else {
            const uint64_t j = lo - arcs;
            src = x.src[j];
            dst = m.src2[x.arc[j]] + x.at[j];
            len = x.len[j];
        }
        const uint64_t rest = len - at;
        const unsigned l = rest < kChunk ? (unsigned)rest : kChunk;
        const char *a = from + src + at;
        char *b = to + dst + at;
        for (unsigned i = threadIdx.x; i < l; i += blockDim.x) b[i] = a[i];
    }
}

inline unsigned blocks(uint64_t n) { return (unsigned)std::max<uint64_t>((n + 255) / 256, 1); }

// Writes the lines into the spare text, then swaps it in.
swg_status rewrite(MergedGraph *m, cudaStream_t s, Scratch &scr, const Pieces &x = Pieces{}) {
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
        const uint64_t pieces = 8 * m->lines + x.n;
        uint64_t *chunks = nullptr, *first = nullptr;
        if (!scr.get(&chunks, pieces) || !scr.get(&first, pieces + 1))
            return cuda_err(cudaErrorMemoryAllocation, "rewrite workspace");
        k_pr_write<<<blocks(m->lines), 256, 0, s>>>(*m, off, m->text2);
        k_pr_chunks<<<blocks(pieces), 256, 0, s>>>(*m, x, chunks);
        st = scan_lengths(chunks, first, pieces, scr, s);
        if (st) return st;
        uint64_t n_chunks = 0;
        EMIT_CUDA(cudaMemcpyAsync(&n_chunks, first + pieces, 8, cudaMemcpyDeviceToHost, s), "chunks");
        EMIT_CUDA(cudaStreamSynchronize(s), "chunks");
        if (n_chunks)
            k_pr_copy<<<(unsigned)std::min<uint64_t>(n_chunks, 1u << 20), 256, 0, s>>>(*m, x, first, n_chunks,
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


// ---- masterSimplifyNodeGraph (graph.cpp:2089-2192) over the lines: a node
// left with exactly one arc on each side (the last nonempty slot of each
// half) whose arcs do not lead back to itself is merged away; each chain of
// such nodes between two other nodes collapses into the two end arcs, whose
// strings are the concatenation of the chain's arcs. The multiplicity is the
// reference's weighted average in size_t arithmetic (graph.cpp:2157-2163),
// taken in the merge's visiting order — chain numbered from its smaller end
// arc (key, slot), node p at level ctz(p) — so a pairwise reduction of the
// chain's arcs weighted by their lengths. A cycle of such nodes is cut at its
// largest key. Chains are found by pointer jumping over two walk states per
// node (the line graph is small next to the k-molecule graph).
constexpr unsigned long long kTerm = 1ull << 63;
constexpr unsigned kNone = 0xffffffffu;

struct SimplifyArgs {
    MergedGraph m;
    unsigned char *fl;  // bit0 merged away, bits1-2 right slot, bits3-4 left slot - 4
    unsigned long long *nx[2], *ws[2], *mx[2];
    unsigned *cn[2];
    unsigned *chain_of;  // per arc slot of an end: chain id (at its start arc)
    unsigned long long *ch_eoff;
    unsigned *ch_m;
    unsigned char *ent_m;
    unsigned long long *ent_l;
    unsigned *ent_chain;
    unsigned long long *cls_count, *cls_cursor;
    unsigned long long *ctr;  // [0] mergeable nodes [1] cycles cut [2] chains [3] states left in cycles
    unsigned *own;
    unsigned long long *xsrc, *xat;
    unsigned *xlen, *xarc;
};

__device__ __forceinline__ bool sm_m(const SimplifyArgs &a, uint64_t q) { return a.fl[q] & 1u; }
__device__ __forceinline__ int sm_rs(unsigned char f) { return (f >> 1) & 3; }
__device__ __forceinline__ int sm_ls(unsigned char f) { return 4 + ((f >> 3) & 3); }

__device__ __forceinline__ unsigned long long agg_inc(unsigned long long *ctr) {
    cg::coalesced_group g = cg::coalesced_threads();
    unsigned long long base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(ctr, (unsigned long long)g.size());
    return g.shfl(base, 0) + g.thread_rank();
}

__device__ __forceinline__ unsigned long long agg_add_labeled(unsigned long long *ctr, int label,
                                                              unsigned long long step) {
    cg::coalesced_group g = cg::labeled_partition(cg::coalesced_threads(), label);
    unsigned long long base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(ctr + label, step * g.size());
    return g.shfl(base, 0) + step * g.thread_rank();
}

__global__ void k_sm_classify(SimplifyArgs a) {
    const uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= a.m.lines) return;
    int rc = 0, lc = 0, rs = 0, ls = 4;
    if (!a.m.del[q])
        for (int s = 0; s < 8; ++s)
            if (a.m.len[8 * q + s]) {
                if (s < 4) ++rc, rs = s;
                else ++lc, ls = s;
            }
    const bool merged = rc == 1 && lc == 1 && (a.m.back[8 * q + rs] >> 3) != q && (a.m.back[8 * q + ls] >> 3) != q;
    a.fl[q] = (unsigned char)((merged ? 1 : 0) | (rs << 1) | ((ls - 4) << 3));
    if (merged) agg_inc(&a.ctr[0]);
}

// Walk state 2q+d leaves line q by its right (d = 0) or left (d = 1) arc; the
// next line is entered by the slot the back link names: entered from the
// left (slot >= 4), it is traversed leaving by its right arc.
__global__ void k_sm_init(SimplifyArgs a) {
    const uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= a.m.lines || !sm_m(a, q)) return;
    const unsigned char f = a.fl[q];
    for (int d = 0; d < 2; ++d) {
        const int slot = d ? sm_ls(f) : sm_rs(f);
        const unsigned b = a.m.back[8 * q + slot];
        const uint64_t far = b >> 3;
        const uint64_t st = 2 * q + d;
        a.nx[0][st] = sm_m(a, far) ? 2 * far + ((b & 7) >= 4 ? 0 : 1) : (kTerm | b);
        a.cn[0][st] = 1;
        a.ws[0][st] = a.m.len[8 * q + slot];
        a.mx[0][st] = a.m.key[q];
    }
}

__global__ void k_sm_jump(SimplifyArgs a, int in) {
    const uint64_t st = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (st >= 2 * a.m.lines || !sm_m(a, st >> 1)) return;
    const int out = in ^ 1;
    const unsigned long long nx = a.nx[in][st];
    if (nx & kTerm) {
        a.nx[out][st] = nx;
        a.cn[out][st] = a.cn[in][st];
        a.ws[out][st] = a.ws[in][st];
        a.mx[out][st] = a.mx[in][st];
    } else {
        a.nx[out][st] = a.nx[in][nx];
        a.cn[out][st] = a.cn[in][st] + a.cn[in][nx];
        a.ws[out][st] = a.ws[in][st] + a.ws[in][nx];
        a.mx[out][st] = max(a.mx[in][st], a.mx[in][nx]);
    }
}

// States still in a cycle after the jumps: the cycle's largest key ends it.
__global__ void k_sm_cut(SimplifyArgs a, int in) {
    const uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= a.m.lines || !sm_m(a, q) || (a.nx[in][2 * q] & kTerm)) return;
    agg_inc(&a.ctr[3]);
    if (a.m.key[q] == a.mx[in][2 * q]) {
        a.fl[q] &= (unsigned char)~1u;
        agg_inc(&a.ctr[1]);
    }
}

__device__ __forceinline__ bool sm_arc_less(const SimplifyArgs &a, uint64_t x, uint64_t y) {
    const unsigned long long kx = a.m.key[x >> 3], ky = a.m.key[y >> 3];
    return kx < ky || (kx == ky && (x & 7) < (y & 7));
}

struct SmPos {
    unsigned m, pos;
    uint64_t alpha, beta;  // end arcs reached going back / forward
    bool fwd;              // the chain runs through the node leaving by its right arc
};

__device__ __forceinline__ SmPos sm_pos(const SimplifyArgs &a, int in, uint64_t q) {
    SmPos c;
    const unsigned la = a.cn[in][2 * q], lb = a.cn[in][2 * q + 1];
    c.beta = a.nx[in][2 * q] & ~kTerm;
    c.alpha = a.nx[in][2 * q + 1] & ~kTerm;
    c.m = la + lb - 1;
    c.fwd = sm_arc_less(a, c.alpha, c.beta);
    c.pos = c.fwd ? lb : la;
    return c;
}

__device__ __forceinline__ int sm_class(unsigned m) { return m == 0 ? 0 : 64 - __clzll((unsigned long long)m); }

__global__ void k_sm_chain_count(SimplifyArgs a, int in) {
    const uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= a.m.lines || !sm_m(a, q)) return;
    const SmPos c = sm_pos(a, in, q);
    if (c.pos == 1) agg_add_labeled(a.cls_count, sm_class(c.m), 1);
}

__global__ void k_sm_chain_alloc(SimplifyArgs a, int in) {
    const uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= a.m.lines || !sm_m(a, q)) return;
    const SmPos c = sm_pos(a, in, q);
    if (c.pos != 1) return;
    const int cl = sm_class(c.m);
    const unsigned id = (unsigned)agg_inc(&a.ctr[2]);
    a.ch_eoff[id] = agg_add_labeled(a.cls_cursor, cl, 1ull << cl);
    a.ch_m[id] = c.m;
    a.chain_of[c.fwd ? c.alpha : c.beta] = id;
}

// Unit arc p of a chain (multiplicity, length): node p's arc towards the far
// end; node 1 also stores the arc back to the start.
__global__ void k_sm_entries(SimplifyArgs a, int in) {
    const uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= a.m.lines || !sm_m(a, q)) return;
    const SmPos c = sm_pos(a, in, q);
    const unsigned id = a.chain_of[c.fwd ? c.alpha : c.beta];
    const uint64_t e = a.ch_eoff[id];
    const unsigned char f = a.fl[q];
    const int out = c.fwd ? sm_rs(f) : sm_ls(f), back = c.fwd ? sm_ls(f) : sm_rs(f);
    a.ent_m[e + c.pos] = a.m.mult[8 * q + out];
    a.ent_l[e + c.pos] = a.m.len[8 * q + out];
    a.ent_chain[e + c.pos] = id;
    if (c.pos == 1) {
        a.ent_m[e] = a.m.mult[8 * q + back];
        a.ent_l[e] = a.m.len[8 * q + back];
        a.ent_chain[e] = id;
    }
}

// One level of the weighted pairwise reduction (graph.cpp:2157-2163).
__global__ void k_sm_level(SimplifyArgs a, uint64_t n_pairs, int t) {
    const uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n_pairs) return;
    const uint64_t e = q << (t + 1);
    const unsigned id = a.ent_chain[e];
    if (id == kNone) return;
    const uint64_t b = (e - a.ch_eoff[id]) >> t;
    if (((b + 1) << t) > a.ch_m[id]) return;
    const uint64_t r = e + (1ull << t);
    const uint64_t ll = a.ent_l[e], lr = a.ent_l[r];
    a.ent_m[e] = (unsigned char)(((uint64_t)a.ent_m[e] * ll + (uint64_t)a.ent_m[r] * lr) / (ll + lr));
    a.ent_l[e] = ll + lr;
}

// The two end arcs of every chain take the chain: its total length and
// multiplicity, each other as the arc back; every merged node hands its two
// arc strings to them as pieces at the offsets its walk states summed (the
// arcs between it and the far start, which mirror the arcs before it). own[]
// keeps the ends' old string lengths for the rewrite.
__global__ void k_sm_apply(SimplifyArgs a, int in) {
    const uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= a.m.lines || !sm_m(a, q)) return;
    const SmPos c = sm_pos(a, in, q);
    const uint64_t start = c.fwd ? c.alpha : c.beta, end = c.fwd ? c.beta : c.alpha;
    const unsigned id = a.chain_of[start];
    const uint64_t e = a.ch_eoff[id];
    const unsigned char f = a.fl[q];
    const int out = c.fwd ? sm_rs(f) : sm_ls(f), back = c.fwd ? sm_ls(f) : sm_rs(f);
    const int d_out = c.fwd ? 0 : 1;
    a.xsrc[2 * q] = a.m.src[8 * q + out];
    a.xlen[2 * q] = a.m.len[8 * q + out];
    a.xarc[2 * q] = (unsigned)start;
    a.xat[2 * q] = a.ws[in][2 * q + (d_out ^ 1)];
    a.xsrc[2 * q + 1] = a.m.src[8 * q + back];
    a.xlen[2 * q + 1] = a.m.len[8 * q + back];
    a.xarc[2 * q + 1] = (unsigned)end;
    a.xat[2 * q + 1] = a.ws[in][2 * q + d_out];
    if (c.pos == 1 || c.pos == c.m) {
        const unsigned char mm = a.ent_m[e];
        const unsigned long long tl = a.ent_l[e];
        if (c.pos == 1) {
            a.m.len[start] = (unsigned)tl;
            a.m.mult[start] = mm;
            a.m.back[start] = (unsigned)end;
        }
        if (c.pos == c.m) {
            a.m.len[end] = (unsigned)tl;
            a.m.mult[end] = mm;
            a.m.back[end] = (unsigned)start;
        }
    }
}

__global__ void k_sm_delete(SimplifyArgs a) {
    const uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= a.m.lines || !sm_m(a, q)) return;
    a.m.del[q] = 1;
}

int sm_ceil_log2(uint64_t v) {
    int r = 0;
    while ((1ull << r) < v) ++r;
    return r;
}


// ---- printContigs (graph.cpp:1139-1202): every arc of at least
// Contig_Length - k bases (Contig_Length = 100, sequence.h:15) is printed
// once, from the end whose key is not smaller than the far end's, as
// ">proc0: " + the node's k-mer oriented for the arc's side + the arc string.
constexpr int kContigLength = 100;

__device__ __forceinline__ bool ct_prints(const MergedGraph &m, uint64_t a) {
    const uint64_t q = a >> 3;
    const unsigned l = m.len[a];
    if (m.del[q] || l == 0 || (int)l < kContigLength - m.k) return false;
    return m.key[q] >= m.key[m.back[a] >> 3];
}

__global__ void k_ct_len(MergedGraph m, uint64_t *__restrict__ out, unsigned long long *count) {
    const uint64_t a = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= 8 * m.lines) return;
    const bool p = ct_prints(m, a);
    out[a] = p ? 8 + (uint64_t)m.k + m.len[a] + 1 : 0;
    if (p) agg_add(count, 1);
}

__global__ void k_ct_write(MergedGraph m, const uint64_t *__restrict__ off, char *__restrict__ text) {
    const uint64_t a = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= 8 * m.lines || off[a + 1] == off[a]) return;
    char *p = text + off[a];
    const char head[8] = {'>', 'p', 'r', 'o', 'c', '0', ':', ' '};
    for (int i = 0; i < 8; ++i) *p++ = head[i];
    const uint64_t key = m.key[a >> 3];
    const uint64_t o = (a & 7) < 4 ? key : rc_dev(key, m.k);
    for (int i = m.k - 1; i >= 0; --i) *p++ = "ACGT"[(o >> (2 * i)) & 3];
    p[m.len[a]] = '\n';  // the arc string itself is copied in chunks
}

__global__ void k_ct_chunks(MergedGraph m, const uint64_t *__restrict__ off, uint64_t *__restrict__ chunks) {
    const uint64_t a = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a < 8 * m.lines) chunks[a] = off[a + 1] == off[a] ? 0 : (m.len[a] + kChunk - 1) / kChunk;
}

__global__ void k_ct_copy(MergedGraph m, const uint64_t *__restrict__ off, const uint64_t *__restrict__ first,
                          uint64_t n_chunks, char *__restrict__ out) {
    const uint64_t arcs = 8 * m.lines;
    for (uint64_t c = blockIdx.x; c < n_chunks; c += gridDim.x) {
        uint64_t lo = 0, hi = arcs;
        while (hi - lo > 1) {
            const uint64_t mid = (lo + hi) / 2;
            if (first[mid] <= c) lo = mid;
            else hi = mid;
        }
        const uint64_t at = (c - first[lo]) * kChunk;
        const uint64_t rest = m.len[lo] - at;
        const unsigned l = rest < kChunk ? (unsigned)rest : kChunk;
        const char *a = m.text + m.src[lo] + at;
        char *b = out + off[lo] + 8 + m.k + at;
        for (unsigned i = threadIdx.x; i < l; i += blockDim.x) b[i] = a[i];
    }
}
}  // namespace

swg_status prune_tips(MergedGraph *m, cudaStream_t s, uint64_t *count) {
    Scratch scr(s, m->pool);
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

swg_status simplify_lines(MergedGraph *m, cudaStream_t s, uint64_t *count) {
    *count = 0;
    Scratch scr(s, m->pool);
    const uint64_t L = m->lines;
    SimplifyArgs a{};
    a.m = *m;
    constexpr int kCls = 40;
    if (!scr.get(&a.fl, L) || !scr.get(&a.nx[0], 2 * L) || !scr.get(&a.nx[1], 2 * L) ||
        !scr.get(&a.ws[0], 2 * L) || !scr.get(&a.ws[1], 2 * L) || !scr.get(&a.mx[0], 2 * L) ||
        !scr.get(&a.mx[1], 2 * L) || !scr.get(&a.cn[0], 2 * L) || !scr.get(&a.cn[1], 2 * L) ||
        !scr.get(&a.chain_of, 8 * L) || !scr.get(&a.ctr, 8 + 2 * kCls) || !scr.get(&a.own, 8 * L) ||
        !scr.get(&a.xsrc, 2 * L) || !scr.get(&a.xat, 2 * L) || !scr.get(&a.xlen, 2 * L) ||
        !scr.get(&a.xarc, 2 * L))
        return cuda_err(cudaErrorMemoryAllocation, "simplify workspace");
    a.cls_count = a.ctr + 8;
    a.cls_cursor = a.ctr + 8 + kCls;
    EMIT_CUDA(cudaMemsetAsync(a.ctr, 0, (8 + 2 * kCls) * 8, s), "simplify");
    EMIT_CUDA(cudaMemsetAsync(a.xlen, 0, std::max<uint64_t>(2 * L, 1) * 4, s), "simplify");
    if (L == 0) return rewrite(m, s, scr);
    const int rounds = sm_ceil_log2(2 * L) + 1;
    unsigned long long h[4] = {0, 0, 0, 0};
    int in = 0;
    k_sm_classify<<<blocks(L), 256, 0, s>>>(a);
    for (int attempt = 0; attempt < 2; ++attempt) {  // again after cutting cycles
        k_sm_init<<<blocks(L), 256, 0, s>>>(a);
        in = 0;
        for (int r = 0; r < rounds; ++r, in ^= 1) k_sm_jump<<<blocks(2 * L), 256, 0, s>>>(a, in);
        if (attempt == 1) break;
        k_sm_cut<<<blocks(L), 256, 0, s>>>(a, in);
        EMIT_CUDA(cudaMemcpyAsync(h, a.ctr, sizeof(h), cudaMemcpyDeviceToHost, s), "simplify");
        EMIT_CUDA(cudaStreamSynchronize(s), "simplify");
        if (!h[3]) break;
    }
    k_sm_chain_count<<<blocks(L), 256, 0, s>>>(a, in);
    unsigned long long cls[kCls];
    EMIT_CUDA(cudaMemcpyAsync(cls, a.cls_count, sizeof(cls), cudaMemcpyDeviceToHost, s), "simplify");
    EMIT_CUDA(cudaMemcpyAsync(h, a.ctr, sizeof(h), cudaMemcpyDeviceToHost, s), "simplify");
    EMIT_CUDA(cudaStreamSynchronize(s), "simplify");
    unsigned long long cursor[kCls];
    uint64_t total = 0, n_chains = 0;
    int top = 0;
    for (int c = kCls - 1; c >= 0; --c) {
        cursor[c] = total;
        total += cls[c] << c;
        n_chains += cls[c];
        if (cls[c] && !top) top = c;
    }
    EMIT_CUDA(cudaMemcpyAsync(a.cls_cursor, cursor, sizeof(cursor), cudaMemcpyHostToDevice, s), "simplify");
    if (!scr.get(&a.ch_eoff, n_chains) || !scr.get(&a.ch_m, n_chains) || !scr.get(&a.ent_m, total) ||
        !scr.get(&a.ent_l, total) || !scr.get(&a.ent_chain, total))
        return cuda_err(cudaErrorMemoryAllocation, "simplify chains");
    EMIT_CUDA(cudaMemsetAsync(a.ent_chain, 0xff, std::max<uint64_t>(total, 1) * 4, s), "simplify");
    EMIT_CUDA(cudaMemcpyAsync(a.own, m->len, 8 * L * 4, cudaMemcpyDeviceToDevice, s), "simplify");
    k_sm_chain_alloc<<<blocks(L), 256, 0, s>>>(a, in);
    k_sm_entries<<<blocks(L), 256, 0, s>>>(a, in);
    for (int t = 0; t < top; ++t) {
        const uint64_t pairs = total >> (t + 1);
        if (!pairs) break;
        k_sm_level<<<blocks(pairs), 256, 0, s>>>(a, pairs, t);
    }
    k_sm_apply<<<blocks(L), 256, 0, s>>>(a, in);
    k_sm_delete<<<blocks(L), 256, 0, s>>>(a);
    EMIT_CUDA(cudaGetLastError(), "simplify kernels");
    *count = h[0] - h[1];
    Pieces x;
    x.own = a.own;
    x.n = 2 * L;
    x.src = a.xsrc;
    x.len = a.xlen;
    x.arc = a.xarc;
    x.at = a.xat;
    return rewrite(m, s, scr, x);
}

swg_status write_contigs(MergedGraph *m, const char *path, cudaStream_t s, uint64_t *count) {
    *count = 0;
    Scratch scr(s, m->pool);
    const uint64_t arcs = 8 * m->lines;
    uint64_t *len = nullptr, *off = nullptr, *chunks = nullptr, *first = nullptr;
    unsigned long long *ctr = nullptr;
    if (!scr.get(&len, arcs) || !scr.get(&off, arcs + 1) || !scr.get(&chunks, arcs) ||
        !scr.get(&first, arcs + 1) || !scr.get(&ctr, 1))
        return cuda_err(cudaErrorMemoryAllocation, "contig workspace");
    EMIT_CUDA(cudaMemsetAsync(ctr, 0, 8, s), "contigs");
    if (arcs) k_ct_len<<<blocks(arcs), 256, 0, s>>>(*m, len, ctr);
    swg_status st = scan_lengths(len, off, arcs, scr, s);
    if (st) return st;
    uint64_t h[2] = {0, 0};
    EMIT_CUDA(cudaMemcpyAsync(&h[0], off + arcs, 8, cudaMemcpyDeviceToHost, s), "contigs");
    EMIT_CUDA(cudaMemcpyAsync(&h[1], ctr, 8, cudaMemcpyDeviceToHost, s), "contigs");
    EMIT_CUDA(cudaStreamSynchronize(s), "contigs");
    char *text = nullptr;
    if (!scr.get(&text, h[0])) return cuda_err(cudaErrorMemoryAllocation, "contig text");
    if (arcs) {
        k_ct_write<<<blocks(arcs), 256, 0, s>>>(*m, off, text);
        k_ct_chunks<<<blocks(arcs), 256, 0, s>>>(*m, off, chunks);
        st = scan_lengths(chunks, first, arcs, scr, s);
        if (st) return st;
        uint64_t n_chunks = 0;
        EMIT_CUDA(cudaMemcpyAsync(&n_chunks, first + arcs, 8, cudaMemcpyDeviceToHost, s), "contigs");
        EMIT_CUDA(cudaStreamSynchronize(s), "contigs");
        if (n_chunks)
            k_ct_copy<<<(unsigned)std::min<uint64_t>(n_chunks, 1u << 20), 256, 0, s>>>(*m, off, first, n_chunks,
                                                                                      text);
    }
    EMIT_CUDA(cudaGetLastError(), "contig kernels");
    *count = h[1];
    return stream_to_file(text, h[0], path, s);
}

swg_status prune_low_coverage(MergedGraph *m, cudaStream_t s, uint64_t *count) {
    Scratch scr(s, m->pool);
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
