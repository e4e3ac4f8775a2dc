// Merging of semi-extended k-molecules on the device: the result of the
// reference's SWAP merge loop (simplifyDistNodeGraph, graph.cpp:1392-1566,
// with the edge messages of recvProc, graph.cpp:1204-1389) over the filtered
// k-mer graph, written as the gathered node lines of its -d file
// contigGraph.txt (gatherDistNodeGraph, graph.cpp:576-696).
//
// A node with exactly one arc on each side whose arcs do not lead back to
// itself is merged away; all other nodes end the chains of merged nodes, and
// each end arc finally spells the whole chain up to the next end node (the
// arc strings do not depend on the order the merge visits nodes in). The
// multiplicity of a merged arc is the reference's running weighted average
// (graph.cpp:1322-1324: 64-bit sum kept in an int, divided by the new length,
// truncated to 8 bits), which does depend on that order. The device follows
// one fixed order: a chain of m merged nodes is numbered 1..m from its
// smaller end arc (node key, then slot) and node p is visited at level
// ctz(p), so each level merges disjoint pairs of neighbouring segments — a
// pairwise tree reduction of the chain's unit arcs. A cycle made only of
// mergeable nodes is cut at its largest key, which is visited last and keeps
// the whole cycle on its two arcs.
//
// Steps (one stream): open-addressing index key -> node (16-byte entries);
// per node the neighbour of each arc; for every mergeable node two
// directed walk states; list ranking of the walks with a sparse ruling set
// (one state in 16..256 — up to about 2^20 rulers — plus every walk head starts a ruler; a ruler
// walks to the next one, then the rulers' own list is ranked by pointer
// jumping); cycles (states no ruler reaches, or rulers whose list never
// ends) are found, cut and ranked by pointer jumping; chains are laid out in
// power-of-two aligned segments so the tree reduction runs level by level in
// place; finally the surviving nodes are ordered by key, each formats its
// line and every merged node writes its two bases straight into the arc
// strings of the two ends. Node indices follow the build's output order,
// which the result does not depend on: chains are numbered by the keys of
// their end nodes.
#include <cuda_runtime.h>

#include <cooperative_groups.h>
#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <cstdint>
#include <cstring>

#include "swg_internal.h"
#include "text_dev.cuh"

namespace swg {
namespace {

constexpr unsigned long long kTerm = 1ull << 63;  // walk successor: end arc code (node * 8 + slot)
constexpr unsigned kNone = 0xffffffffu;
constexpr unsigned long long kEmptyKey = ~0ull;
constexpr int kClasses = 40;  // chain segment size classes 2^0 .. 2^39

// error bits
constexpr unsigned kErrIndex = 1u, kErrNeighbour = 2u, kErrWalk = 4u, kErrCycle = 8u, kErrOrder = 16u;

// Per chain position of a merge in a given visiting order: the visit time of
// the node at the position, and the two segments that meet there (the first
// arc of the left one, the last arc of the right one, their multiplicities)
// once both are merged; `arrive` counts the sides that have arrived.
struct CartSlot {
    unsigned t;
    unsigned lb, rb;
    unsigned arrive;
    unsigned char lv, rv;
};

__device__ __forceinline__ uint64_t fmix64(uint64_t x) {  // MurmurHash3 finaliser
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return x;
}

namespace cg = cooperative_groups;

// Counter increments aggregated over the threads of a warp that make them
// together (one atomic per counter per warp); returns this thread's slot.
__device__ __forceinline__ unsigned long long agg_inc(unsigned long long *ctr) {
    cg::coalesced_group g = cg::coalesced_threads();
    unsigned long long base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(ctr, (unsigned long long)g.size());
    return g.shfl(base, 0) + g.thread_rank();
}

// The same for threads that target different counters ctr[label], each
// adding step(label).
__device__ __forceinline__ unsigned long long agg_add_labeled(unsigned long long *ctr, int label,
                                                              unsigned long long step) {
    cg::coalesced_group g = cg::labeled_partition(cg::coalesced_threads(), label);
    unsigned long long base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(ctr + label, step * g.size());
    return g.shfl(base, 0) + step * g.thread_rank();
}

struct MergeArgs {
    int k;
    uint64_t n;
    uint64_t rmask;  // ruler sampling: one state in rmask + 1
    const unsigned long long *keys;
    const unsigned long long *mult;  // byte s = multiplicity of slot s
    ulonglong2 *ht;                  // index: x = key (kEmptyKey when free), y = node
    uint64_t hmask;
    unsigned *nb;              // n*8: (neighbour << 1) | arrival side, kNone for an empty slot
    unsigned char *fl;         // bit0 mergeable, bits1-2 right slot, bits3-4 left slot - 4
    unsigned long long *succ;  // 2n walk states: next state or kTerm | end arc
    unsigned long long *oo;    // per state: its ruler << 32 | distance from it (~0: none)
    unsigned *rpos;            // ruler list position of a ruler state
    unsigned *rlist;
    unsigned long long *rn0, *rn1, *rl0, *rl1;  // ruler list: next ruler / end arc, states to the end
    unsigned *len;             // per state: states from it to the end of its walk
    unsigned long long *term;  // per state: kTerm | end arc reached
    unsigned *clist;
    unsigned long long *cx0, *cx1, *cy0, *cy1;  // cycle pointer jumping
    unsigned *chain_of;        // per arc code: chain id (set at the chain's start arc)
    unsigned long long *ch_eoff;
    unsigned *ch_m;
    unsigned long long *ch_dfwd, *ch_drev;
    unsigned char *ent;        // chain unit-arc multiplicities, reduced in place
    unsigned *ent_chain;
    unsigned long long *cls_count, *cls_cursor;
    unsigned long long *ctr;   // [0] rulers [1] cycle states [2] chains [3] cycles cut [4] merged nodes
                               // [5] surviving nodes
    unsigned long long *skey;  // surviving nodes: keys, then (sorted) node indices
    unsigned *sidx;
    unsigned *err;
    // merge in a given visiting order (null: the fixed tree order)
    unsigned long long *vt;    // per node: its visit time
    CartSlot *cart;            // per chain position (the ent layout)
};

__device__ __forceinline__ unsigned lookup(const MergeArgs &a, uint64_t key) {
    uint64_t h = fmix64(key) & a.hmask;
    for (uint64_t probe = 0; probe <= a.hmask; ++probe) {
        const ulonglong2 e = a.ht[h];
        if (e.x == key) return (unsigned)e.y;
        if (e.x == kEmptyKey) return kNone;
        h = (h + 1) & a.hmask;
    }
    return kNone;
}

__device__ __forceinline__ unsigned mbyte(uint64_t m, int s) { return (unsigned)(m >> (8 * s)) & 0xffu; }
__device__ __forceinline__ bool is_m(const MergeArgs &a, uint64_t i) { return a.fl[i] & 1u; }
__device__ __forceinline__ int rslot(unsigned char f) { return (f >> 1) & 3; }
__device__ __forceinline__ int lslot(unsigned char f) { return 4 + ((f >> 3) & 3); }

__global__ void k_mg_index(MergeArgs a) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const unsigned long long key = a.keys[i];
    uint64_t h = fmix64(key) & a.hmask;
    for (uint64_t probe = 0; probe <= a.hmask; ++probe) {
        const unsigned long long prev = atomicCAS(&a.ht[h].x, kEmptyKey, key);
        if (prev == kEmptyKey || prev == key) {
            a.ht[h].y = i;
            return;
        }
        h = (h + 1) & a.hmask;
    }
    atomicOr(a.err, kErrIndex);
}

// Neighbour of every arc (node::getNodeID, graph.cpp:164-196: oriented k-mer
// plus the arc base, last k bases, canonical id and the side reached) and
// whether the node is merged away.
__global__ void k_mg_classify(MergeArgs a) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int k = a.k;
    const uint64_t kmask = (1ull << (2 * k)) - 1;
    const uint64_t key = a.keys[i], m = a.mult[i], rk = rc_dev(key, k);
    int rc = 0, lc = 0, rs = 0, ls = 4;
    bool self = false;
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        unsigned v = kNone;
        if (mbyte(m, s)) {
            const uint64_t e = (((s < 4 ? key : rk) << 2) | (uint64_t)(s & 3)) & kmask;
            const uint64_t r = rc_dev(e, k);
            const unsigned side = e >= r;
            const unsigned j = lookup(a, side ? e : r);
            if (j == kNone) {
                atomicOr(a.err, kErrNeighbour);
            } else {
                v = (j << 1) | side;
                self |= (uint64_t)j == i;
            }
            if (s < 4) ++rc, rs = s;
            else ++lc, ls = s;
        }
        a.nb[i * 8 + s] = v;
    }
    const bool merged = rc == 1 && lc == 1 && !self;
    a.fl[i] = (unsigned char)((merged ? 1 : 0) | (rs << 1) | ((ls - 4) << 3));
    if (merged) agg_inc(&a.ctr[4]);
}

// Walk state 2i+d of a merged node: d = 0 traverses it as its key (leaves by
// the right arc), d = 1 as the reverse complement (leaves by the left arc).
// The successor is the next merged node's state, or the end arc that points
// back from the end node reached: its side of arrival picks the half, the
// first base of the k-mer just left gives the slot.
__device__ __forceinline__ unsigned long long walk_next(const MergeArgs &a, uint64_t i, int d) {
    const unsigned char f = a.fl[i];
    const unsigned v = a.nb[i * 8 + (d ? lslot(f) : rslot(f))];
    const uint64_t j = v >> 1;
    const unsigned side = v & 1u;
    if (is_m(a, j)) return 2 * j + (side ? 0 : 1);
    const uint64_t o = d ? rc_dev(a.keys[i], a.k) : a.keys[i];
    const unsigned first = (unsigned)(o >> (2 * (a.k - 1))) & 3u;
    return kTerm | (j * 8 + (side ? 4 : 0) + 3 - first);
}

__device__ __forceinline__ bool ruler_of(const MergeArgs &a, uint64_t st, const ulonglong2 &pair);

// Both walk states of a merged node, and which of them start rulers.
__global__ void k_mg_states(MergeArgs a) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n || !is_m(a, i)) return;
    const ulonglong2 pair = make_ulonglong2(walk_next(a, i, 0), walk_next(a, i, 1));
    *reinterpret_cast<ulonglong2 *>(a.succ + 2 * i) = pair;
    for (int d = 0; d < 2; ++d) {
        if (!ruler_of(a, 2 * i + d, pair)) continue;
        const unsigned p = (unsigned)agg_inc(&a.ctr[0]);
        a.rlist[p] = (unsigned)(2 * i + d);
    }
}

// The successors of a node's two states sit side by side: one 16-byte load.
__device__ __forceinline__ ulonglong2 succ_pair(const MergeArgs &a, uint64_t st) {
    return *reinterpret_cast<const ulonglong2 *>(a.succ + (st & ~1ull));
}

// A ruler: the first state of a walk (its twin leaves to an end) or, on
// average, one state in rmask + 1 (16..256, chosen for at most about 2^20 rulers:
// enough walkers to keep the SMs' warp slots busy while each walk's loads
// wait on memory one after the other, and a ruler list small enough for L2).
__device__ __forceinline__ bool ruler_of(const MergeArgs &a, uint64_t st, const ulonglong2 &pair) {
    const unsigned long long twin = (st & 1) ? pair.x : pair.y;
    return (twin & kTerm) || (fmix64(st) & a.rmask) == 0;
}

// The ruler list position of every ruler state (read when a walk meets it).
__global__ void k_mg_rpos(MergeArgs a) {
    const uint64_t n_rul = a.ctr[0];
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n_rul;
         p += (uint64_t)gridDim.x * blockDim.x)
        a.rpos[a.rlist[p]] = (unsigned)p;
}

// Each ruler walks to the next ruler or the walk's end, labelling the states
// on the way with (its list position, distance); per step one 16-byte load
// and one 8-byte store. Grid-stride over the ruler count on the device.
__global__ void k_mg_walk(MergeArgs a) {
    const uint64_t n_rul = a.ctr[0];
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n_rul;
         p += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned r = a.rlist[p];
        const unsigned long long tag = p << 32;
        a.oo[r] = tag;
        uint64_t cur = r;
        ulonglong2 pr = succ_pair(a, r);
        bool done = false;
        for (unsigned o = 1; o <= 2 * a.n; ++o) {
            const unsigned long long nx = (cur & 1) ? pr.y : pr.x;
            if (nx & kTerm) {
                a.rn0[p] = nx;
                a.rl0[p] = o;
                done = true;
                break;
            }
            const ulonglong2 pn = succ_pair(a, nx);
            if (ruler_of(a, nx, pn)) {
                a.rn0[p] = a.rpos[nx];
                a.rl0[p] = o;
                done = true;
                break;
            }
            a.oo[nx] = tag | o;
            cur = nx;
            pr = pn;
        }
        if (!done) atomicOr(a.err, kErrWalk);
    }
}

__global__ void k_mg_rjump(const unsigned long long *__restrict__ rn_in, const unsigned long long *__restrict__ rl_in,
                           unsigned long long *__restrict__ rn_out, unsigned long long *__restrict__ rl_out,
                           const unsigned long long *__restrict__ count) {
    const uint64_t n_rul = *count;
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n_rul;
         p += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long nx = rn_in[p];
        if (nx & kTerm) {
            rn_out[p] = nx;
            rl_out[p] = rl_in[p];
        } else {
            rn_out[p] = rn_in[nx];
            rl_out[p] = rl_in[p] + rl_in[nx];
        }
    }
}

__global__ void k_mg_finish(MergeArgs a, const unsigned long long *__restrict__ rn,
                            const unsigned long long *__restrict__ rl) {
    const uint64_t st = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (st >= 2 * a.n || !is_m(a, st >> 1)) return;
    const unsigned long long oo = a.oo[st];
    if (oo != ~0ull) {
        const unsigned p = (unsigned)(oo >> 32);
        if (rn[p] & kTerm) {
            a.len[st] = (unsigned)(rl[p] - (oo & 0xffffffffull));
            a.term[st] = rn[p];
            return;
        }
    }
    a.len[st] = 0;
    a.term[st] = 0;
    a.clist[agg_inc(&a.ctr[1])] = (unsigned)st;
}

// ---- cycles of merged nodes: largest key by pointer jumping, cut there
// A cycle keeps the node the merge visits last: the largest key in the fixed
// order, the latest visit time in a given one.
__device__ __forceinline__ unsigned long long cut_rank(const MergeArgs &a, uint64_t node) {
    return a.vt ? a.vt[node] : a.keys[node];
}

__global__ void k_mg_cyc_init(MergeArgs a, uint64_t c) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= c) return;
    const unsigned st = a.clist[t];
    a.cx0[st] = cut_rank(a, st >> 1);
    a.cy0[st] = a.succ[st];
}

__global__ void k_mg_cyc_max(MergeArgs a, uint64_t c, const unsigned long long *__restrict__ mx_in,
                             const unsigned long long *__restrict__ nx_in, unsigned long long *__restrict__ mx_out,
                             unsigned long long *__restrict__ nx_out) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= c) return;
    const unsigned st = a.clist[t];
    const unsigned long long nx = nx_in[st];
    mx_out[st] = max(mx_in[st], mx_in[nx]);
    nx_out[st] = nx_in[nx];
}

__global__ void k_mg_cyc_cut(MergeArgs a, uint64_t c, const unsigned long long *__restrict__ mx) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= c) return;
    const unsigned st = a.clist[t];
    if (cut_rank(a, st >> 1) == mx[st]) {
        a.fl[st >> 1] &= (unsigned char)~1u;  // both states of the node store the same
        if (!(st & 1)) atomicAdd(&a.ctr[3], 1ull);
    }
}

__global__ void k_mg_cyc_succ(MergeArgs a, uint64_t c) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= c) return;
    const unsigned st = a.clist[t];
    if (!is_m(a, st >> 1)) return;
    a.cy0[st] = walk_next(a, st >> 1, (int)(st & 1));
    a.cx0[st] = 1;
}

__global__ void k_mg_cyc_rank(MergeArgs a, uint64_t c, const unsigned long long *__restrict__ ln_in,
                              const unsigned long long *__restrict__ nx_in, unsigned long long *__restrict__ ln_out,
                              unsigned long long *__restrict__ nx_out) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= c) return;
    const unsigned st = a.clist[t];
    if (!is_m(a, st >> 1)) return;
    const unsigned long long nx = nx_in[st];
    if (nx & kTerm) {
        ln_out[st] = ln_in[st];
        nx_out[st] = nx;
    } else {
        ln_out[st] = ln_in[st] + ln_in[nx];
        nx_out[st] = nx_in[nx];
    }
}

__global__ void k_mg_cyc_done(MergeArgs a, uint64_t c, const unsigned long long *__restrict__ ln,
                              const unsigned long long *__restrict__ nx) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= c) return;
    const unsigned st = a.clist[t];
    if (!is_m(a, st >> 1)) return;
    if (!(nx[st] & kTerm)) atomicOr(a.err, kErrCycle);
    a.len[st] = (unsigned)ln[st];
    a.term[st] = nx[st];
}

// ---- chains
// End arcs compare by (key of the end node, slot). Only end nodes' keys are
// read here: a small, cache-resident set.
__device__ __forceinline__ bool arc_less(const MergeArgs &a, uint64_t x, uint64_t y) {
    const unsigned long long kx = a.keys[x >> 3], ky = a.keys[y >> 3];
    return kx < ky || (kx == ky && (x & 7) < (y & 7));
}

struct ChainPos {
    unsigned m, pos;
    uint64_t start;  // the smaller end arc code: the chain's start
    bool fwd;        // the chain runs through this node as its key (state 2i)
};

__device__ __forceinline__ ChainPos chain_pos(const MergeArgs &a, uint64_t i) {
    ChainPos c;
    const unsigned la = a.len[2 * i], lb = a.len[2 * i + 1];
    const uint64_t beta = a.term[2 * i] & ~kTerm, alpha = a.term[2 * i + 1] & ~kTerm;
    c.m = la + lb - 1;
    c.fwd = arc_less(a, alpha, beta);
    c.pos = c.fwd ? lb : la;
    c.start = c.fwd ? alpha : beta;
    return c;
}

__device__ __forceinline__ int size_class(unsigned m) {  // ceil(log2(m + 1))
    return m == 0 ? 0 : 64 - __clzll((unsigned long long)m);
}

__global__ void k_mg_chain_count(MergeArgs a) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n || !is_m(a, i)) return;
    const ChainPos c = chain_pos(a, i);
    if (c.pos == 1) agg_add_labeled(a.cls_count, size_class(c.m), 1);
}

__global__ void k_mg_chain_alloc(MergeArgs a) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n || !is_m(a, i)) return;
    const ChainPos c = chain_pos(a, i);
    if (c.pos != 1) return;
    const int cl = size_class(c.m);
    const unsigned id = (unsigned)agg_inc(&a.ctr[2]);
    a.ch_eoff[id] = agg_add_labeled(a.cls_cursor, cl, 1ull << cl);
    a.ch_m[id] = c.m;
    a.chain_of[c.start] = id;
}

// Unit arc p (0..m) of a chain: between its nodes at positions p and p+1
// (0 and m+1 are the end nodes); node p stores the arc it leaves by, node 1
// also the arc it enters by.
__global__ void k_mg_entries(MergeArgs a) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n || !is_m(a, i)) return;
    const ChainPos c = chain_pos(a, i);
    const unsigned id = a.chain_of[c.start];
    const uint64_t e = a.ch_eoff[id];
    const unsigned char f = a.fl[i];
    const uint64_t m = a.mult[i];
    a.ent[e + c.pos] = (unsigned char)mbyte(m, c.fwd ? rslot(f) : lslot(f));
    a.ent_chain[e + c.pos] = id;
    if (a.cart) {
        CartSlot z;
        z.t = (unsigned)a.vt[i];
        z.lb = z.rb = z.arrive = 0;
        z.lv = z.rv = 0;
        a.cart[e + c.pos] = z;
    }
    if (c.pos == 1) {
        a.ent[e] = (unsigned char)mbyte(m, c.fwd ? lslot(f) : rslot(f));
        a.ent_chain[e] = id;
    }
}

// One level of the pairwise reduction: the node at position (2b+1)*2^t
// merges segment b (left) with segment b+1 (right), graph.cpp:1322-1324.
__global__ void k_mg_level(MergeArgs a, uint64_t n_pairs, int t) {
    const uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n_pairs) return;
    const uint64_t e = q << (t + 1);
    const unsigned id = a.ent_chain[e];
    if (id == kNone) return;
    const uint64_t m = a.ch_m[id];
    const uint64_t b = (e - a.ch_eoff[id]) >> t;
    if (((b + 1) << t) > m) return;  // no node in the middle: the segment carries over
    const uint64_t ll = 1ull << t;
    const uint64_t lr = min((b + 2) << t, m + 1) - ((b + 1) << t);
    const uint64_t sum = (uint64_t)a.ent[e] * ll + (uint64_t)a.ent[e + ll] * lr;
    const int pre = (int)(unsigned)sum;
    a.ent[e] = (unsigned char)((uint64_t)(int64_t)pre / (ll + lr));
}

// Merge in a given visiting order. Visiting the node at position p merges the
// segment of unit arcs to its left with the one to its right, each spanning
// up to the nearest node on that side still unvisited (or the chain's end):
// the chain's merge tree is the Cartesian tree of the visit times. One thread
// starts at every unit arc; a segment belongs to whichever of its two
// bounding nodes is visited first; a thread publishes its segment there, and
// the second of the two sides to arrive combines them (the weighted average
// of graph.cpp:1322-1324) and carries the merged segment on. The root (no
// unvisited bound left) writes the chain's multiplicity to its first entry.
__global__ void k_mg_cart(MergeArgs a, uint64_t total) {
    const uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= total) return;
    const unsigned id = a.ent_chain[e];
    if (id == kNone) return;
    const uint64_t e0 = a.ch_eoff[id], m = a.ch_m[id];
    uint64_t l = e - e0, r = l;  // the segment: unit arcs l..r
    unsigned v = a.ent[e];
    for (uint64_t step = 0; step <= m; ++step) {
        const unsigned tl = l == 0 ? kNone : a.cart[e0 + l].t;      // node l bounds it on the left
        const unsigned tr = r == m ? kNone : a.cart[e0 + r + 1].t;  // node r+1 on the right
        if (tl == kNone && tr == kNone) {
            a.ent[e0] = (unsigned char)v;
            return;
        }
        const bool as_right = tl < tr;  // node l is visited first: this is its right side
        const uint64_t p = as_right ? l : r + 1;
        CartSlot *cs = a.cart + e0 + p;
        if (as_right) {
            cs->rv = (unsigned char)v;
            cs->rb = (unsigned)r;
        } else {
            cs->lv = (unsigned char)v;
            cs->lb = (unsigned)l;
        }
        __threadfence();
        if (atomicAdd(&cs->arrive, 1u) == 0) return;  // the other side carries on
        __threadfence();
        volatile CartSlot *vs = cs;
        const uint64_t L = as_right ? vs->lb : l, R = as_right ? r : vs->rb;
        const unsigned vl = as_right ? vs->lv : v, vr = as_right ? v : vs->rv;
        const uint64_t ll = p - L, lr = R - p + 1;
        const uint64_t sum = (uint64_t)vl * ll + (uint64_t)vr * lr;
        const int pre = (int)(unsigned)sum;
        v = (unsigned)(unsigned char)((uint64_t)(int64_t)pre / (ll + lr));
        l = L;
        r = R;
    }
    atomicOr(a.err, kErrWalk);
}

// Visit times from a list of keys in visiting order: every node exactly once.
__global__ void k_mg_vtime(MergeArgs a, const unsigned long long *__restrict__ order, uint64_t n_order) {
    const uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n_order) return;
    const unsigned i = lookup(a, order[q]);
    if (i == kNone || atomicCAS(&a.vt[i], ~0ull, (unsigned long long)q) != ~0ull) atomicOr(a.err, kErrOrder);
}

// ---- the gathered node lines (graph.cpp:615-645): id, per slot " " + arc + "#",
// 8 multiplicities, blanks up to sum(len+1)+61 bytes, '\n' as the last byte.
__device__ __forceinline__ uint64_t first_state(unsigned v) {
    return 2 * (uint64_t)(v >> 1) + ((v & 1u) ? 0 : 1);
}

// The nodes left (not merged away), listed for the key-order sort.
__global__ void k_mg_survivors(MergeArgs a) {
    const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= a.n || is_m(a, j)) return;
    const unsigned long long q = agg_inc(&a.ctr[5]);
    a.skey[q] = a.keys[j];
    a.sidx[q] = (unsigned)j;
}

__global__ void k_mg_line_len(MergeArgs a, const unsigned *__restrict__ order, uint64_t n_lines,
                              uint64_t *__restrict__ out) {
    const uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n_lines) return;
    const uint64_t j = order[q];
    const uint64_t m = a.mult[j];
    uint64_t l = 69;
    for (int s = 0; s < 8; ++s) {
        if (!mbyte(m, s)) continue;
        const unsigned v = a.nb[j * 8 + s];
        l += 1 + (is_m(a, v >> 1) ? a.len[first_state(v)] : 0);
    }
    out[q] = l;
}

// Line position of every node left.
__global__ void k_mg_pos(const unsigned *__restrict__ order, uint64_t n_lines, unsigned *__restrict__ pos_of) {
    const uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n_lines) pos_of[order[q]] = (unsigned)q;
}

__global__ void k_mg_line_write(MergeArgs a, const unsigned *__restrict__ order, uint64_t n_lines,
                                const uint64_t *__restrict__ off, char *__restrict__ text,
                                const unsigned *__restrict__ pos_of, MergedGraph mg) {
    const uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n_lines) return;
    const uint64_t j = order[q];
    const uint64_t m = a.mult[j];
    char *const start = text + off[q];
    char *p = put_u64(start, a.keys[j]);
    mg.key[q] = a.keys[j];
    mg.del[q] = 0;
    unsigned mm[8];
    uint64_t vlen = 69;
    const uint64_t key = a.keys[j], rk = rc_dev(key, a.k);
    for (int s = 0; s < 8; ++s) {
        *p++ = ' ';
        mm[s] = mbyte(m, s);
        uint64_t l = 0;
        unsigned back = kNone;
        if (mm[s]) {
            *p = "ACGT"[s & 3];
            const unsigned v = a.nb[j * 8 + s];
            mg.src[8 * q + s] = (unsigned long long)(p - text);
            l = 1;
            if (is_m(a, v >> 1)) {
                const uint64_t st = first_state(v);
                const uint64_t mine = j * 8 + s, other = a.term[st] & ~kTerm;
                const bool first = arc_less(a, mine, other);  // this end starts the chain
                const unsigned id = a.chain_of[first ? mine : other];
                const unsigned long long dest = (unsigned long long)(p - text);
                if (first) a.ch_dfwd[id] = dest;
                else a.ch_drev[id] = dest;
                mm[s] = a.ent[a.ch_eoff[id]];
                l += a.len[st];
                back = pos_of[other >> 3] * 8u + (unsigned)(other & 7);
            } else {  // one base to the next node left: its arc back, as walk_next finds it
                const uint64_t o = s < 4 ? key : rk;
                const unsigned first = (unsigned)(o >> (2 * (a.k - 1))) & 3u;
                back = pos_of[v >> 1] * 8u + ((v & 1u) ? 4u : 0u) + 3u - first;
            }
            p += l;
            vlen += l;
        } else {
            mg.src[8 * q + s] = 0;
        }
        mg.len[8 * q + s] = (unsigned)l;
        mg.mult[8 * q + s] = (unsigned char)mm[s];
        mg.back[8 * q + s] = back;
        *p++ = '#';
    }
    for (int s = 0; s < 8; ++s) {
        *p++ = ' ';
        p = put_u64(p, mm[s]);
    }
    while ((uint64_t)(p - start) < vlen - 1) *p++ = ' ';
    *p = '\n';
}

__global__ void k_mg_chars(MergeArgs a, char *__restrict__ text) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n || !is_m(a, i)) return;
    const ChainPos c = chain_pos(a, i);
    const unsigned id = a.chain_of[c.start];
    const unsigned char f = a.fl[i];
    const int out_fwd = c.fwd ? rslot(f) : lslot(f);  // leaving towards the chain's far end
    const int out_rev = c.fwd ? lslot(f) : rslot(f);
    text[a.ch_dfwd[id] + c.pos] = "ACGT"[out_fwd & 3];
    text[a.ch_drev[id] + (c.m + 1 - c.pos)] = "ACGT"[out_rev & 3];
}

inline unsigned blocks(uint64_t n) { return (unsigned)std::max<uint64_t>((n + 255) / 256, 1); }

int ceil_log2(uint64_t v) {
    int r = 0;
    while ((1ull << r) < v) ++r;
    return r;
}

}  // namespace

// Grows the merged graph's buffers (the text, the spare text for rewrites,
// the per-line arrays) to hold `bytes` of text and `lines` lines.
swg_status merged_reserve(MergedGraph *m, uint64_t bytes, uint64_t lines) {
    if (bytes > m->text_cap) {
        cudaFree(m->text);
        cudaFree(m->text2);
        m->text = m->text2 = nullptr;
        m->text_cap = m->text2_cap = 0;
        EMIT_CUDA(cudaMalloc((void **)&m->text, bytes), "merged text");
        m->text_cap = bytes;
    }
    if (lines > m->line_cap || !m->key) {
        const uint64_t c = std::max<uint64_t>(lines, 1);
        cudaFree(m->key);
        cudaFree(m->len);
        cudaFree(m->mult);
        cudaFree(m->src);
        cudaFree(m->src2);
        cudaFree(m->back);
        cudaFree(m->del);
        m->key = nullptr;
        m->len = nullptr;
        m->mult = nullptr;
        m->src = m->src2 = nullptr;
        m->back = nullptr;
        m->del = nullptr;
        m->line_cap = 0;
        EMIT_CUDA(cudaMalloc((void **)&m->key, c * 8), "merged lines");
        EMIT_CUDA(cudaMalloc((void **)&m->len, c * 32), "merged lines");
        EMIT_CUDA(cudaMalloc((void **)&m->mult, c * 8), "merged lines");
        EMIT_CUDA(cudaMalloc((void **)&m->src, c * 64), "merged lines");
        EMIT_CUDA(cudaMalloc((void **)&m->src2, c * 64), "merged lines");
        EMIT_CUDA(cudaMalloc((void **)&m->back, c * 32), "merged lines");
        EMIT_CUDA(cudaMalloc((void **)&m->del, c), "merged lines");
        m->line_cap = c;
    }
    return SWG_OK;
}

void merged_free(MergedGraph *m) {
    cudaFree(m->text);
    cudaFree(m->text2);
    cudaFree(m->key);
    cudaFree(m->len);
    cudaFree(m->mult);
    cudaFree(m->src);
    cudaFree(m->src2);
    cudaFree(m->back);
    cudaFree(m->del);
    if (m->pool) cudaMemPoolDestroy(m->pool);
    *m = MergedGraph();
}

swg_status merge_graph(const unsigned long long *d_keys, const unsigned long long *d_mult, uint64_t n, int k,
                       cudaStream_t s, MergedGraph *mg, MergeResult *res, const unsigned long long *h_order,
                       uint64_t n_order) {
    *res = MergeResult();
    if (n >= (1ull << 29)) {
        set_error("merge: more than 2^29 k-molecules");
        return SWG_ERR_BAD_INPUT;
    }
    if (k % 2 == 0) {  // the reference's k is odd (sequence.cpp:44): no k-mer is its own reverse complement
        set_error("merge: k must be odd (an even k-mer can be its own reverse complement)");
        return SWG_ERR_BAD_INPUT;
    }
    Scratch scr(s, mg->pool);
    MergeArgs a;
    std::memset(&a, 0, sizeof(a));
    a.k = k;
    a.n = n;
    a.rmask = 15;
    while (a.rmask < 255 && 2 * n / (a.rmask + 1) > (1ull << 20)) a.rmask = 2 * a.rmask + 1;
    unsigned long long *ctr = nullptr;
    uint64_t hcap = 1024;
    while (hcap < 2 * n) hcap *= 2;
    a.hmask = hcap - 1;
    if (!scr.get(&a.ht, hcap) || !scr.get(&a.nb, 8 * n) || !scr.get(&a.fl, n) || !scr.get(&a.succ, 2 * n) ||
        !scr.get(&a.oo, 2 * n) || !scr.get(&a.rpos, 2 * n) || !scr.get(&a.rlist, 2 * n) ||
        !scr.get(&a.len, 2 * n) || !scr.get(&a.term, 2 * n) || !scr.get(&a.clist, 2 * n) ||
        !scr.get(&a.chain_of, 8 * n) || !scr.get(&ctr, 8 + 2 * kClasses) || !scr.get(&a.err, 1))
        return cuda_err(cudaErrorMemoryAllocation, "merge workspace");
    a.ctr = ctr;
    a.cls_count = ctr + 8;
    a.cls_cursor = ctr + 8 + kClasses;
    a.keys = d_keys;
    a.mult = d_mult;
    EMIT_CUDA(cudaMemsetAsync(ctr, 0, (8 + 2 * kClasses) * sizeof(unsigned long long), s), "merge clear");
    EMIT_CUDA(cudaMemsetAsync(a.err, 0, sizeof(unsigned), s), "merge clear");
    EMIT_CUDA(cudaMemsetAsync(a.ht, 0xff, hcap * sizeof(ulonglong2), s), "merge clear");
    EMIT_CUDA(cudaMemsetAsync(a.oo, 0xff, 2 * n * sizeof(unsigned long long), s), "merge clear");
    int launches = 0;
    k_mg_index<<<blocks(n), 256, 0, s>>>(a);
    if (h_order) {  // visit times from the caller's order
        if (n_order != n) {
            set_error("merge: the visiting order must list every k-molecule once");
            return SWG_ERR_BAD_INPUT;
        }
        unsigned long long *d_order = nullptr;
        if (!scr.get(&a.vt, n) || !scr.get(&d_order, n))
            return cuda_err(cudaErrorMemoryAllocation, "visiting order");
        EMIT_CUDA(cudaMemsetAsync(a.vt, 0xff, std::max<uint64_t>(n, 1) * sizeof(unsigned long long), s), "merge clear");
        if (n)
            EMIT_CUDA(cudaMemcpyAsync(d_order, h_order, n * sizeof(unsigned long long), cudaMemcpyHostToDevice, s),
                      "visiting order");
        k_mg_vtime<<<blocks(n), 256, 0, s>>>(a, d_order, n);
        unsigned herr = 0;
        EMIT_CUDA(cudaMemcpyAsync(&herr, a.err, sizeof(unsigned), cudaMemcpyDeviceToHost, s), "merge status");
        EMIT_CUDA(cudaStreamSynchronize(s), "visiting order");
        if (herr & kErrOrder) {
            set_error("merge: the visiting order names a key twice or a key the graph does not hold");
            return SWG_ERR_BAD_INPUT;
        }
        ++launches;
    }
    k_mg_classify<<<blocks(n), 256, 0, s>>>(a);
    k_mg_states<<<blocks(n), 256, 0, s>>>(a);
    launches += 3;
    // rulers: at most one per state; counts stay on the device
    if (!scr.get(&a.rn0, 2 * n) || !scr.get(&a.rn1, 2 * n) || !scr.get(&a.rl0, 2 * n) || !scr.get(&a.rl1, 2 * n))
        return cuda_err(cudaErrorMemoryAllocation, "ruler list");
    int sms = 0;
    EMIT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0), "device attribute");
    const unsigned wgrid = (unsigned)std::max(1, sms * 8);
    k_mg_rpos<<<wgrid, 256, 0, s>>>(a);
    k_mg_walk<<<wgrid, 256, 0, s>>>(a);
    const int rounds = ceil_log2(std::max<uint64_t>(2 * n, 1)) + 1;
    unsigned long long *bn[2] = {a.rn0, a.rn1}, *bl[2] = {a.rl0, a.rl1};
    for (int r = 0; r < rounds; ++r)
        k_mg_rjump<<<wgrid, 256, 0, s>>>(bn[r & 1], bl[r & 1], bn[(r + 1) & 1], bl[(r + 1) & 1], ctr);
    launches += 2 + rounds;
    const unsigned long long *rn = bn[rounds & 1], *rl = bl[rounds & 1];
    k_mg_finish<<<blocks(2 * n), 256, 0, s>>>(a, rn, rl);
    ++launches;
    unsigned long long h[6];
    unsigned herr = 0;
    EMIT_CUDA(cudaMemcpyAsync(h, ctr, sizeof(h), cudaMemcpyDeviceToHost, s), "cycle count");
    EMIT_CUDA(cudaMemcpyAsync(&herr, a.err, sizeof(unsigned), cudaMemcpyDeviceToHost, s), "merge status");
    EMIT_CUDA(cudaStreamSynchronize(s), "cycle count");
    if (herr & (kErrIndex | kErrNeighbour)) {
        set_error("merge: node index or neighbour lookup failed (arc without its neighbour k-molecule)");
        return SWG_ERR_BAD_INPUT;
    }
    if (herr) {
        set_error("merge: a walk did not end (internal error)");
        return SWG_ERR_TIMEOUT;
    }
    const uint64_t n_cyc_states = h[1];
    if (n_cyc_states) {
        if (!scr.get(&a.cx0, 2 * n) || !scr.get(&a.cx1, 2 * n) || !scr.get(&a.cy0, 2 * n) ||
            !scr.get(&a.cy1, 2 * n))
            return cuda_err(cudaErrorMemoryAllocation, "cycle workspace");
        const uint64_t c = n_cyc_states;
        const int rounds = ceil_log2(c) + 1;
        unsigned long long *bx[2] = {a.cx0, a.cx1}, *by[2] = {a.cy0, a.cy1};
        k_mg_cyc_init<<<blocks(c), 256, 0, s>>>(a, c);
        for (int r = 0; r < rounds; ++r)
            k_mg_cyc_max<<<blocks(c), 256, 0, s>>>(a, c, bx[r & 1], by[r & 1], bx[(r + 1) & 1], by[(r + 1) & 1]);
        k_mg_cyc_cut<<<blocks(c), 256, 0, s>>>(a, c, bx[rounds & 1]);
        k_mg_cyc_succ<<<blocks(c), 256, 0, s>>>(a, c);
        for (int r = 0; r < rounds; ++r)
            k_mg_cyc_rank<<<blocks(c), 256, 0, s>>>(a, c, bx[r & 1], by[r & 1], bx[(r + 1) & 1], by[(r + 1) & 1]);
        k_mg_cyc_done<<<blocks(c), 256, 0, s>>>(a, c, bx[rounds & 1], by[rounds & 1]);
        launches += 4 + 2 * rounds;
    }
    k_mg_chain_count<<<blocks(n), 256, 0, s>>>(a);
    ++launches;
    unsigned long long cls[kClasses];
    EMIT_CUDA(cudaMemcpyAsync(cls, a.cls_count, sizeof(cls), cudaMemcpyDeviceToHost, s), "chain classes");
    EMIT_CUDA(cudaMemcpyAsync(h, ctr, sizeof(h), cudaMemcpyDeviceToHost, s), "cycle cuts");
    EMIT_CUDA(cudaMemcpyAsync(&herr, a.err, sizeof(unsigned), cudaMemcpyDeviceToHost, s), "merge status");
    EMIT_CUDA(cudaStreamSynchronize(s), "chain classes");
    if (herr) {
        set_error("merge: a walk did not end (internal error)");
        return SWG_ERR_TIMEOUT;
    }
    // segments of 2^c entries, largest class first: every offset is aligned
    unsigned long long cursor[kClasses];
    uint64_t total = 0, n_chains = 0;
    int top = 0;
    for (int c = kClasses - 1; c >= 0; --c) {
        cursor[c] = total;
        total += cls[c] << c;
        n_chains += cls[c];
        if (cls[c] && !top) top = c;
    }
    EMIT_CUDA(cudaMemcpyAsync(a.cls_cursor, cursor, sizeof(cursor), cudaMemcpyHostToDevice, s), "chain layout");
    if (!scr.get(&a.ch_eoff, n_chains) || !scr.get(&a.ch_m, n_chains) || !scr.get(&a.ch_dfwd, n_chains) ||
        !scr.get(&a.ch_drev, n_chains) || !scr.get(&a.ent, total) || !scr.get(&a.ent_chain, total))
        return cuda_err(cudaErrorMemoryAllocation, "chain workspace");
    EMIT_CUDA(cudaMemsetAsync(a.ent_chain, 0xff, std::max<uint64_t>(total, 1) * sizeof(unsigned), s), "chain clear");
    if (a.vt && !scr.get(&a.cart, total)) return cuda_err(cudaErrorMemoryAllocation, "merge tree");
    k_mg_chain_alloc<<<blocks(n), 256, 0, s>>>(a);
    k_mg_entries<<<blocks(n), 256, 0, s>>>(a);
    launches += 2;
    if (a.vt) {
        if (total) k_mg_cart<<<blocks(total), 256, 0, s>>>(a, total);
        ++launches;
    } else {
        for (int t = 0; t < top; ++t) {
            const uint64_t pairs = total >> (t + 1);
            if (!pairs) break;
            k_mg_level<<<blocks(pairs), 256, 0, s>>>(a, pairs, t);
            ++launches;
        }
    }
    // the nodes left, in key order
    const uint64_t n_lines = n - h[4] + h[3];
    unsigned long long *skey2 = nullptr;
    unsigned *sidx2 = nullptr;
    uint64_t *lens = nullptr, *loff = nullptr;
    if (!scr.get(&a.skey, n_lines) || !scr.get(&a.sidx, n_lines) || !scr.get(&skey2, n_lines) ||
        !scr.get(&sidx2, n_lines) || !scr.get(&lens, n_lines) || !scr.get(&loff, n_lines + 1))
        return cuda_err(cudaErrorMemoryAllocation, "line workspace");
    k_mg_survivors<<<blocks(n), 256, 0, s>>>(a);
    ++launches;
    if (n_lines) {
        size_t tb = 0;
        EMIT_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb, a.skey, skey2, a.sidx, sidx2, (int64_t)n_lines, 0,
                                                  2 * k, s),
                  "sort size");
        unsigned char *tmp = nullptr;
        if (!scr.get(&tmp, tb)) return cuda_err(cudaErrorMemoryAllocation, "sort scratch");
        EMIT_CUDA(cub::DeviceRadixSort::SortPairs(tmp, tb, a.skey, skey2, a.sidx, sidx2, (int64_t)n_lines, 0,
                                                  2 * k, s),
                  "sort");
        k_mg_line_len<<<blocks(n_lines), 256, 0, s>>>(a, sidx2, n_lines, lens);
        ++launches;
    }
    swg_status st = scan_lengths(lens, loff, n_lines, scr, s);
    if (st) return st;
    uint64_t bytes = 0;
    EMIT_CUDA(cudaMemcpyAsync(&bytes, loff + n_lines, 8, cudaMemcpyDeviceToHost, s), "text size");
    EMIT_CUDA(cudaStreamSynchronize(s), "text size");
    swg_status gst = merged_reserve(mg, bytes + 1, n_lines);
    if (gst) return gst;
    mg->k = k;
    mg->lines = n_lines;
    unsigned *pos_of = nullptr;
    if (!scr.get(&pos_of, n)) return cuda_err(cudaErrorMemoryAllocation, "line positions");
    if (n_lines) {
        k_mg_pos<<<blocks(n_lines), 256, 0, s>>>(sidx2, n_lines, pos_of);
        k_mg_line_write<<<blocks(n_lines), 256, 0, s>>>(a, sidx2, n_lines, loff, mg->text, pos_of, *mg);
    }
    k_mg_chars<<<blocks(n), 256, 0, s>>>(a, mg->text);
    launches += 3;
    EMIT_CUDA(cudaMemsetAsync(mg->text + bytes, '\n', 1, s), "merged text");
    EMIT_CUDA(cudaGetLastError(), "merge kernels");
    EMIT_CUDA(cudaMemcpyAsync(&herr, a.err, sizeof(unsigned), cudaMemcpyDeviceToHost, s), "merge status");
    EMIT_CUDA(cudaStreamSynchronize(s), "merge");
    if (herr) {
        set_error("merge: a merge tree did not end (internal error)");
        return SWG_ERR_TIMEOUT;
    }
    res->text_bytes = bytes + 1;
    mg->text_bytes = bytes + 1;
    mg->nodes = n_lines;
    res->nodes = n_lines;
    res->chains = n_chains;
    res->cycles = h[3];
    res->rulers = h[0];
    res->launches = launches + 3;  // + the scan
    return SWG_OK;
}

}  // namespace swg
