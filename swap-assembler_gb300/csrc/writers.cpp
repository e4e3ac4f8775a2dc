// Host-side output of the filtered k-mer graph: sorting, the reference's
// -s adjacency file (kmerGraph.txt), node lines with multiplicities, and the
// graphStatistics totals.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "swg_internal.h"

namespace swg {

// Reverse complement (kmerGraph.cpp:5-14): complement each base, reverse order.
uint64_t revcomp_host(uint64_t a, int k) {
    uint64_t rev = 0;
    for (int i = 0; i < k; i++) {
        rev = (rev << 2) | ((3 - a) & 3);
        a >>= 2;
    }
    return rev;
}

// Neighbour id printed for slot s of key K in kmerGraph.txt.
// node::getNodeID (graph.cpp:164-196): descriptor = K (s < 4) or rc(K)
// (s >= 4), append base "ACGT"[s%4], keep the last k bases N; if N >= rc(N)
// the id is N, else rc(N) with return value -1. printKmerGraph
// (graph.cpp:3387-3396, 3417-3426) then means to reverse-complement the id
// back, but complements character i (the slot) instead of j, k times: the
// printed value is complement(N) with base s flipped back when k is odd.
uint64_t kmer_graph_neighbour(uint64_t key, int slot, int k) {
    const uint64_t kmask = (1ull << (2 * k)) - 1;
    const uint64_t d = slot < 4 ? key : revcomp_host(key, k);
    const uint64_t n = ((d << 2) | (uint64_t)(slot & 3)) & kmask;
    if (n >= revcomp_host(n, k)) return n;
    uint64_t out = n ^ kmask;
    if (k & 1) out ^= 3ull << (2 * (k - 1 - slot));
    return out;
}

// LSD radix sort of (key, payload) by key, 16-bit digits; skips digits that
// are equal in every key.
static void radix_sort_pairs(uint64_t *keys, uint64_t *pay, uint64_t n) {
    if (n < 2) return;
    uint64_t all_or = 0, all_and = ~0ull;
    for (uint64_t i = 0; i < n; i++) {
        all_or |= keys[i];
        all_and &= keys[i];
    }
    std::vector<uint64_t> k2(n), p2(n), hist(65536);
    uint64_t *ks = keys, *ps = pay, *kd = k2.data(), *pd = p2.data();
    for (int pass = 0; pass < 4; pass++) {
        const int sh = 16 * pass;
        if ((((all_or ^ all_and) >> sh) & 0xffff) == 0) continue;
        std::fill(hist.begin(), hist.end(), 0);
        for (uint64_t i = 0; i < n; i++) hist[(ks[i] >> sh) & 0xffff]++;
        uint64_t s = 0;
        for (auto &h : hist) {
            const uint64_t c = h;
            h = s;
            s += c;
        }
        for (uint64_t i = 0; i < n; i++) {
            const uint64_t pos = hist[(ks[i] >> sh) & 0xffff]++;
            kd[pos] = ks[i];
            pd[pos] = ps[i];
        }
        std::swap(ks, kd);
        std::swap(ps, pd);
    }
    if (ks != keys) {
        std::memcpy(keys, ks, n * sizeof(uint64_t));
        std::memcpy(pay, ps, n * sizeof(uint64_t));
    }
}

void sort_records(uint64_t *keys, uint64_t *mult8, uint64_t n) { radix_sort_pairs(keys, mult8, n); }

namespace {

struct OutBuf {
    FILE *fp;
    std::vector<char> buf;
    size_t n = 0;
    bool ok = true;
    explicit OutBuf(FILE *f) : fp(f), buf(1 << 22) {}
    void flush() {
        if (n && std::fwrite(buf.data(), 1, n, fp) != n) ok = false;
        n = 0;
    }
    void reserve(size_t want) {
        if (n + want > buf.size()) flush();
    }
    void put(char c) { buf[n++] = c; }
    void put_u64(uint64_t v) {
        char tmp[24];
        int l = 0;
        do {
            tmp[l++] = (char)('0' + v % 10);
            v /= 10;
        } while (v);
        while (l) buf[n++] = tmp[--l];
    }
};

}  // namespace

// printKmerGraph (graph.cpp:3352-3440): per node, a line "K n.." for the set
// slots 0-3 and a line "rc(K) n.." for the set slots 4-7 (graph.cpp:3369-3376
// computes the second line's head as the reverse complement). The reference
// prints in hash-map order; here lines are sorted by their first token (all
// first tokens are distinct: K is canonical, rc(K) is not).
swg_status write_kmer_graph(const uint64_t *keys, const uint8_t *mult, uint64_t n, int k,
                            const char *path) {
    if (k < 8 || k > 31) {
        set_error("kmerGraph.txt needs 8 <= k <= 31 (the reference indexes the slot as a base position)");
        return SWG_ERR_BAD_INPUT;
    }
    std::vector<uint64_t> first, idx;
    first.reserve(2 * n);
    idx.reserve(2 * n);
    for (uint64_t i = 0; i < n; i++) {
        const uint8_t *m = mult + 8 * i;
        if (m[0] | m[1] | m[2] | m[3]) {
            first.push_back(keys[i]);
            idx.push_back(2 * i);
        }
        if (m[4] | m[5] | m[6] | m[7]) {
            first.push_back(revcomp_host(keys[i], k));
            idx.push_back(2 * i + 1);
        }
    }
    radix_sort_pairs(first.data(), idx.data(), first.size());
    FILE *fp = std::fopen(path, "wb");
    if (!fp) {
        set_error(std::string("cannot open ") + path);
        return SWG_ERR_IO;
    }
    OutBuf ob(fp);
    for (uint64_t q = 0; q < first.size(); q++) {
        const uint64_t i = idx[q] >> 1;
        const int half = (int)(idx[q] & 1);
        const uint8_t *m = mult + 8 * i;
        ob.reserve(5 * 24);
        ob.put_u64(first[q]);
        for (int s = 4 * half; s < 4 * half + 4; s++) {
            if (!m[s]) continue;
            ob.put(' ');
            ob.put_u64(kmer_graph_neighbour(keys[i], s, k));
        }
        ob.put('\n');
    }
    ob.flush();
    const bool ok = ob.ok && std::fclose(fp) == 0;
    if (!ok) {
        set_error(std::string("write failed: ") + path);
        return SWG_ERR_IO;
    }
    return SWG_OK;
}

// printLocalNodeGraph (graph.cpp:569): "%llu %s# ... %s# %d .. %d\n" with the
// arc strings of node::init (graph.cpp:88-96): "ACGT"[s%4] iff mult != 0.
swg_status write_node_lines(const uint64_t *keys, const uint8_t *mult, uint64_t n,
                            const char *path) {
    static const char acgt[4] = {'A', 'C', 'G', 'T'};
    FILE *fp = std::fopen(path, "wb");
    if (!fp) {
        set_error(std::string("cannot open ") + path);
        return SWG_ERR_IO;
    }
    OutBuf ob(fp);
    for (uint64_t i = 0; i < n; i++) {
        const uint8_t *m = mult + 8 * i;
        ob.reserve(24 + 8 * 3 + 8 * 4 + 2);
        ob.put_u64(keys[i]);
        for (int s = 0; s < 8; s++) {
            ob.put(' ');
            if (m[s]) ob.put(acgt[s & 3]);
            ob.put('#');
        }
        for (int s = 0; s < 8; s++) {
            ob.put(' ');
            ob.put_u64(m[s]);
        }
        ob.put('\n');
    }
    ob.flush();
    const bool ok = ob.ok && std::fclose(fp) == 0;
    if (!ok) {
        set_error(std::string("write failed: ") + path);
        return SWG_ERR_IO;
    }
    return SWG_OK;
}

// graphStatistics (graph.cpp:1579-1608) on freshly built nodes: every arc
// string is one base long, so the edge-length sum equals the edge count, a
// tip is a node with exactly one arc (1 < k), and a bubble is a node whose
// smallest arc multiplicity is below 0.2 x its largest.
void graph_stats(const uint8_t *mult, uint64_t n, int k, int64_t out[5]) {
    int64_t nodes = 0, edges = 0, tips = 0, bubbles = 0;
    for (uint64_t i = 0; i < n; i++) {
        const uint8_t *m = mult + 8 * i;
        int local = 0, maxm = -1, minm = 1000000;
        nodes++;
        for (int s = 0; s < 8; s++) {
            if (!m[s]) continue;
            edges++;
            local++;
            maxm = std::max(maxm, (int)m[s]);
            minm = std::min(minm, (int)m[s]);
        }
        if (local == 1 && 1 < k) tips++;
        if (minm < 0.2 * maxm) bubbles++;
    }
    out[0] = nodes;
    out[1] = edges;
    out[2] = edges;
    out[3] = tips;
    out[4] = bubbles;
}

}  // namespace swg
