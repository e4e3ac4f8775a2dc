// Autotuner: picks the counting scheme and its knobs for a (k, read-length
// band) by timing trial builds of a sample on this GPU: the bucketed build
// (the default) at several bucket sizes and scatter block shapes; the direct table at several load factors, in input and in
// minimizer order; hash-partitioned slices. The choices go to a cache file,
// one JSON object per line: {"k": K, "band": B, "load": X, "algorithm": A,
// "read_order": O, "ms": T, "bucket_records": R, "part_bits": P,
// "scatter_shape": S}.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "swg_internal.h"

namespace {

// Read-length bands (upper bounds): 75, 100, 150, 250 bp reads fall in
// different bands.
int band_of(uint32_t len) {
    static const uint32_t edges[] = {80, 125, 175, 275};
    for (int i = 0; i < 4; i++)
        if (len <= edges[i]) return i;
    return 4;
}

struct Cand {
    double load;
    int algorithm;
    int order;
    uint32_t records;  // bucketed knobs (0 = default)
    int part_bits;
    int shape;
};

bool read_entry(const char *line, int *k, int *band, swg_tuning *t) {
    double load = 0, ms = 0;
    int kk = 0, b = 0, alg = 0, ord = 0, pb = 0, sh = 0;
    unsigned rec = 0;
    const int got = std::sscanf(line,
                                " {\"k\": %d, \"band\": %d, \"load\": %lf, \"algorithm\": %d, "
                                "\"read_order\": %d, \"ms\": %lf, \"bucket_records\": %u, \"part_bits\": %d, "
                                "\"scatter_shape\": %d}",
                                &kk, &b, &load, &alg, &ord, &ms, &rec, &pb, &sh);
    if (got != 6 && got != 9) return false;  // 6: an entry written before the bucketed knobs
    *k = kk;
    *band = b;
    t->load_factor = load;
    t->algorithm = alg;
    t->read_order = ord;
    t->ms = (float)ms;
    t->bucket_records = got == 9 ? rec : 0;
    t->part_bits = got == 9 ? pb : 0;
    t->scatter_shape = got == 9 ? sh : 0;
    return true;
}

}  // namespace

extern "C" {

swg_status swg_autotune(const swg_opts *base, const uint32_t *d_packed, uint64_t n_words,
                        const uint64_t *d_read_off, const uint32_t *d_read_len, uint64_t n_reads,
                        uint32_t read_len_hint, const char *cache_path, swg_tuning *best) {
    if (!base || !best || !cache_path) return SWG_ERR_BAD_INPUT;
    // bucketed: bucket size and scatter shape (the partition count follows the
    // input's size, so a count picked on a sample would not fit the full input)
    std::vector<Cand> cands;
    for (uint32_t rec : {4096u, 2048u, 8192u})  // the default first: ties keep it
        for (int sh : {0, 1, 2}) cands.push_back({0.6, SWG_ALGO_BUCKETED, SWG_ORDER_INPUT, rec, 0, sh});
    for (double load : {0.5, 0.6, 0.7, 0.8}) cands.push_back({load, SWG_ALGO_DIRECT, SWG_ORDER_INPUT, 0, 0, 0});
    cands.push_back({0.6, SWG_ALGO_DIRECT, SWG_ORDER_MINIMIZER, 0, 0, 0});
    cands.push_back({0.6, SWG_ALGO_PARTITIONED, SWG_ORDER_INPUT, 0, 0, 0});
    swg_graph *g = nullptr;
    swg_status st = swg_graph_create(&g);
    if (st) return st;
    swg_tuning top;
    std::memset(&top, 0, sizeof(top));
    top.ms = -1;
    for (const Cand &c : cands) {
        swg_opts o = *base;
        o.load_factor = c.load;
        o.algorithm = c.algorithm;
        o.read_order = c.order;
        o.expected_distinct = 0;
        o.bucket_records = c.records;
        o.part_bits = c.part_bits;
        o.scatter_shape = c.shape;
        float ms = 0;
        for (int rep = 0; rep < 3 && st == SWG_OK; rep++) {  // first run allocates; best of two
            st = swg_graph_build_device(g, &o, d_packed, n_words, d_read_off, d_read_len, n_reads);
            swg_build_info info;
            if (st == SWG_OK && swg_graph_build_info(g, &info) == SWG_OK && rep > 0)
                ms = rep == 1 ? info.ms[4] : std::min(ms, info.ms[4]);
        }
        if (st) break;
        if (top.ms < 0 || ms < top.ms) {
            top.load_factor = c.load;
            top.algorithm = c.algorithm;
            top.read_order = c.order;
            top.ms = ms;
            top.bucket_records = c.records;
            top.part_bits = c.part_bits;
            top.scatter_shape = c.shape;
        }
    }
    swg_graph_free(g);
    if (st) return st;
    *best = top;
    FILE *fp = std::fopen(cache_path, "a");
    if (!fp) {
        swg::set_error(std::string("cannot write ") + cache_path);
        return SWG_ERR_IO;
    }
    std::fprintf(fp,
                 "{\"k\": %d, \"band\": %d, \"load\": %.3f, \"algorithm\": %d, \"read_order\": %d, "
                 "\"ms\": %.4f, \"bucket_records\": %u, \"part_bits\": %d, \"scatter_shape\": %d}\n",
                 base->k, band_of(read_len_hint), top.load_factor, top.algorithm, top.read_order,
                 (double)top.ms, top.bucket_records, top.part_bits, top.scatter_shape);
    std::fclose(fp);
    return SWG_OK;
}

swg_status swg_autotune_apply(const char *cache_path, int k, uint32_t read_len, swg_opts *o) {
    if (!cache_path || !o) return SWG_ERR_BAD_INPUT;
    FILE *fp = std::fopen(cache_path, "r");
    if (!fp) return SWG_ERR_NOT_READY;
    char line[512];
    const int want = band_of(read_len);
    bool found = false;
    swg_tuning t, hit;
    while (std::fgets(line, sizeof(line), fp)) {  // the last entry for a key wins
        int kk, b;
        if (read_entry(line, &kk, &b, &t) && kk == k && b == want) {
            hit = t;
            found = true;
        }
    }
    std::fclose(fp);
    if (!found) return SWG_ERR_NOT_READY;
    o->load_factor = hit.load_factor;
    o->algorithm = hit.algorithm;
    o->read_order = hit.read_order;
    o->bucket_records = hit.bucket_records;
    o->part_bits = hit.part_bits;
    o->scatter_shape = hit.scatter_shape;
    return SWG_OK;
}

}  // extern "C"
