// C ABI of the k-mer graph builder (declared in include/swapgb.h).
//
// A build runs on one CUDA stream. It starts with the occurrence prefix (3
// launches; the host reads the occurrence total and the longest read), then
// one of:
//   bucketed (the default): sampled region sizes -> level-1 partition scatter
//     -> level-2 bucket scatter -> shared-memory bucket counting + cutoff ->
//     (host reads the survivor total) -> survivor gather [-> big buckets in a
//     global table]; a region overflow reruns it with exact counts;
//   direct: tile table -> HyperLogLog estimate (host reads it) -> table clear
//     -> K1 extract+count -> K2 cutoff+compaction; a table that fills up is
//     detected on the device and the build is repeated with a larger table;
//   partitioned: record scatter -> waves of L2-resident partition slices.
// A last synchronisation reads the status and the survivor count.
#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "swg_internal.h"

namespace swg {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

}  // namespace swg

using swg::BuildArgs;
using swg::Entry;

struct Control {  // device-side control block
    unsigned status;
    unsigned pad;                    // bucketed build: tier-1 overflow count
    unsigned long long counters[2];  // inserted keys, survivors
    unsigned pad2;                   // bucketed build: tier-2 overflow count
    unsigned pad3;
    unsigned long long work[2];      // bucketed build: read batches handed out (count, scatter)
    unsigned max_len;                // longest read (occurrence scan)
    unsigned pad4;
    unsigned long long host_written; // survivors written to the caller's host arrays
    uint64_t occ_total;              // last: the memsets of the control block stop before it
};

struct swg_graph {
    int device = 0;
    cudaStream_t own = nullptr;
    // device workspace, grown on demand and reused by later builds
    uint32_t *d_packed = nullptr;
    uint64_t packed_cap = 0;
    uint64_t *d_off = nullptr;
    uint32_t *d_len = nullptr;
    uint64_t reads_cap = 0;
    uint64_t *d_prefix = nullptr;
    uint64_t prefix_cap = 0;
    uint64_t *d_scan = nullptr;
    uint64_t scan_cap = 0;
    uint32_t *d_tiles = nullptr;
    uint64_t tiles_cap = 0;
    Entry *d_table = nullptr;
    uint64_t table_cap = 0;
    unsigned long long *d_out_keys = nullptr;
    unsigned long long *d_out_mult = nullptr;
    uint64_t out_cap = 0;
    unsigned *d_hll = nullptr;
    Control *d_ctl = nullptr;
    // pinned host mirrors
    Control *h_ctl = nullptr;
    unsigned *h_hll = nullptr;
    cudaEvent_t ev[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    // result of the last build
    bool built = false;
    int k = 0;
    int cutoff = 0;
    uint64_t n_out = 0;
    uint64_t n_distinct = 0;
    uint64_t cap_used = 0;
    float ms[5] = {0, 0, 0, 0, 0};
    int launches = 0;
    int algorithm = 0;
    uint64_t occurrences = 0;
    double estimate = 0;
    uint32_t retries = 0;
    // partitioned workspace
    unsigned long long *d_part = nullptr;  // count[P] | start[P+1] | cursor[P]
    uint64_t part_cap = 0;
    unsigned long long *h_part = nullptr;  // pinned copy of start[P+1]
    unsigned long long *d_records = nullptr;
    uint64_t records_cap = 0;
    Entry *d_slices = nullptr;
    uint64_t slices_cap = 0;
    uint32_t parts = 0, slots = 0, waves = 0;
    uint32_t bucket_table = 0;  // bucketed: entries of the tier-1 shared table
    uint64_t slot_cap = 0;
    // read-order workspace
    unsigned *d_minhash = nullptr;
    uint64_t minhash_cap = 0;
    unsigned *d_bucket = nullptr;
    uint64_t bucket_cap = 0;
    uint64_t *d_poff = nullptr;
    uint64_t poff_cap = 0;
    uint32_t *d_plen = nullptr;
    uint64_t plen_cap = 0;
    // device framing workspace
    unsigned char *d_text = nullptr;
    uint64_t text_cap = 0;
    uint64_t *d_fw = nullptr;  // chunk counts | scan scratch | newline masks and positions | records x2
    uint64_t fw_cap = 0;
    // bucketed workspace
    unsigned long long *d_rec2 = nullptr;
    uint64_t rec2_cap = 0;
    unsigned long long *d_bk = nullptr;  // bucketed build: bucket cursors, offsets, lists, prefixes
    uint64_t bk_cap = 0;
    Entry *d_arena = nullptr;
    uint64_t arena_cap = 0;
    // batched build (n_samples == 0 after a single-sample build)
    uint32_t n_samples = 0;
    std::vector<uint64_t> s_tbase, s_tcap, s_out, s_distinct, s_occ;
    swg::SegParams *d_segs = nullptr;
    uint64_t segs_cap = 0;
    uint32_t *d_read_seg = nullptr;
    uint64_t read_seg_cap = 0;
    unsigned long long *d_seg_counts = nullptr;
    uint64_t seg_counts_cap = 0;
    unsigned *d_seg_status = nullptr;
    uint64_t seg_status_cap = 0;
    uint64_t *d_seg_meta = nullptr;  // read start [S+1] | offset shift [S] | occurrence prefix [S+1]
    uint64_t seg_meta_cap = 0;
    double *d_est = nullptr;
    uint64_t est_cap = 0;
    // tagged bucketed batch: survivors grouped by sample, per-sample cursors
    unsigned long long *d_out2_keys = nullptr;
    unsigned long long *d_out2_mult = nullptr;
    uint64_t out2_cap = 0;
    unsigned long long *d_seg_cursor = nullptr;
    uint64_t seg_cursor_cap = 0;
    unsigned long long *d_bigmeta = nullptr;  // bucketed: big-bucket ranges for the global table
    uint64_t bigmeta_cap = 0;
    // merged graph (swg_graph_merge): the -d file's text and its lines on the device
    swg::MergedGraph mg;
    bool merged = false;
    swg::MergeResult mres;
    float merge_ms = 0;
    unsigned *d_hll_seg = nullptr;
    uint64_t hll_seg_cap = 0;
    // streamed FASTA build: the copy stream, one event per text piece, and
    // the framing arrays that grow as pieces land
    cudaStream_t copy = nullptr, frame = nullptr;
    std::vector<cudaEvent_t> piece_ev;
    uint64_t *d_sfw = nullptr;  // block counts | block bases | scan scratch | totals
    uint64_t sfw_cap = 0;
    uint64_t *d_nl = nullptr;
    uint64_t nl_cap = 0;
    uint64_t *d_ridx = nullptr, *d_woff = nullptr;  // per record: read index, first word
    uint64_t ridx_cap = 0, woff_cap = 0;
    // swg_graph_build_fasta_file: pinned host buffer the file is read into
    // (kept and reused by later calls of this handle)
    char *h_file = nullptr;
    uint64_t h_file_cap = 0;
    // swg_graph_build_fasta_to_host: the caller's arrays as the device sees
    // them, for the duration of the call; host_out_used: the bucket count wrote them
    unsigned long long *host_keys = nullptr, *host_mult = nullptr;
    uint64_t host_cap = 0;
    bool host_out_used = false;
};

namespace {

swg_status cuda_fail(cudaError_t e, const char *what) {
    swg::set_error(std::string(what) + ": " + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? SWG_ERR_OOM : SWG_ERR_CUDA;
}

#define SWG_CUDA(call, what)                            \
    do {                                                \
        cudaError_t e_ = (call);                        \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

template <typename T>
swg_status ensure(T **p, uint64_t *cap, uint64_t want, const char *what) {
    if (*cap >= want && *p) return SWG_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    const uint64_t n = std::max<uint64_t>(want, 1);
    cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
    if (e != cudaSuccess) {
        cudaGetLastError();
        return cuda_fail(e, what);
    }
    *cap = n;
    return SWG_OK;
}

// Device read offsets and lengths (host-input builds), grown together.
swg_status ensure_reads(swg_graph *g, uint64_t n_reads) {
    if (g->reads_cap >= n_reads && g->d_off && g->d_len) return SWG_OK;
    cudaFree(g->d_off);
    cudaFree(g->d_len);
    g->d_off = nullptr;
    g->d_len = nullptr;
    g->reads_cap = 0;
    SWG_CUDA(cudaMalloc(&g->d_off, std::max<uint64_t>(n_reads, 1) * 8), "read offsets");
    SWG_CUDA(cudaMalloc(&g->d_len, std::max<uint64_t>(n_reads, 1) * 4), "read lengths");
    g->reads_cap = std::max<uint64_t>(n_reads, 1);
    return SWG_OK;
}

swg_status check_opts(const swg_opts *o) {
    if (!o) {
        swg::set_error("opts is NULL");
        return SWG_ERR_BAD_INPUT;
    }
    if (o->k < 1 || o->k > 31) {
        swg::set_error("k must be in 1..31");
        return SWG_ERR_BAD_INPUT;
    }
    if (o->algorithm < 0 || o->algorithm > SWG_ALGO_BUCKETED || o->read_order < 0 ||
        o->read_order > SWG_ORDER_MINIMIZER) {
        swg::set_error("unknown algorithm or read order");
        return SWG_ERR_BAD_INPUT;
    }
    if (o->load_factor < 0 || o->load_factor > 0.9) {
        swg::set_error("load_factor must be in (0, 0.9] (0 = default)");
        return SWG_ERR_BAD_INPUT;
    }
    if (o->bucket_records > 65535 || (o->part_bits && (o->part_bits < 8 || o->part_bits > 10)) ||
        o->scatter_shape < 0 || o->scatter_shape > 4) {
        swg::set_error("bucketed knobs out of range (records per bucket <= 65535, partition bits 8..10, "
                       "scatter shape 0..4)");
        return SWG_ERR_BAD_INPUT;
    }
    return SWG_OK;
}

cudaStream_t stream_of(swg_graph *g, const swg_opts *o) {
    return o->stream ? (cudaStream_t)o->stream : g->own;
}

swg_status build_direct(swg_graph *g, const swg_opts *o, BuildArgs &a, cudaStream_t s, double load);
swg_status build_partitioned(swg_graph *g, const swg_opts *o, BuildArgs &a, cudaStream_t s,
                             double load);
swg_status build_bucketed(swg_graph *g, const swg_opts *o, BuildArgs &a, cudaStream_t s,
                          double load, bool counted = false);

// The default algorithm is the bucketed one while its worst-case workspace
// (two record buffers of at most 1.5 x 8 bytes per occurrence, plus an
// output of up to 16 bytes per occurrence) fits in 80% of the device memory
// that is free or already held by this handle's record buffers; otherwise the
// direct one, whose table grows with the distinct k-molecules instead of the
// occurrences.
constexpr unsigned kBucketedMaxRead = 16384;  // longest read the default sends to the bucketed build

bool bucketed_fits(const swg_graph *g, uint64_t occurrences) {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    const double held = 8.0 * (double)(g->records_cap + g->rec2_cap);
    const double need = 40.0 * (double)occurrences + (64 << 20);
    return need <= 0.8 * ((double)free_b + held);
}

// NVTX range over one call, named after the reference's phase it replaces
// (visible to a profiler; no cost without one).
struct Phase {
    explicit Phase(const char *name) { nvtxRangePushA(name); }
    ~Phase() { nvtxRangePop(); }
    Phase(const Phase &) = delete;
    Phase &operator=(const Phase &) = delete;
};

swg_status build_impl(swg_graph *g, const swg_opts *o, const uint32_t *packed, uint64_t n_words,
                      const uint64_t *off, const uint32_t *len, uint64_t n_reads) {
    Phase phase("constructDistNodeGraph + cutoffGraph");
    swg_status st = check_opts(o);
    if (st) return st;
    if (n_reads >= 0xffffffffull) {
        swg::set_error("at most 2^32-2 reads per build");
        return SWG_ERR_BAD_INPUT;
    }
    if (n_reads && (!packed || !off || !len)) {
        swg::set_error("NULL read buffer");
        return SWG_ERR_BAD_INPUT;
    }
    SWG_CUDA(cudaSetDevice(g->device), "cudaSetDevice");
    cudaStream_t s = stream_of(g, o);
    g->built = false;
    g->merged = false;
    g->n_samples = 0;
    g->k = o->k;
    g->cutoff = o->cutoff;
    g->launches = 0;
    const double load = o->load_factor > 0 ? o->load_factor : 0.6;

    BuildArgs a;
    std::memset(&a, 0, sizeof(a));
    a.packed = packed;
    a.n_words = n_words;
    a.read_off = off;
    a.read_len = len;
    a.n_reads = n_reads;
    a.k = o->k;
    a.cutoff = o->cutoff;

    if ((st = ensure(&g->d_prefix, &g->prefix_cap, n_reads + 1, "occurrence prefix"))) return st;
    if ((st = ensure(&g->d_scan, &g->scan_cap, swg::scan_block_count(n_reads) + 1, "scan scratch")))
        return st;
    a.occ_prefix = g->d_prefix;
    a.scan_blocks = g->d_scan;
    a.hll = g->d_hll;
    a.status = &g->d_ctl->status;
    a.counters = g->d_ctl->counters;

    SWG_CUDA(cudaEventRecord(g->ev[0], s), "event");
    SWG_CUDA(cudaMemsetAsync(g->d_ctl, 0, sizeof(Control), s), "memset control");
    SWG_CUDA(cudaMemsetAsync(g->d_prefix, 0, sizeof(uint64_t), s), "memset prefix");
    a.max_len = &g->d_ctl->max_len;
    g->launches += swg::launch_occ_scan(a, s, false);  // the total; the per-read prefix below if needed
    a.max_len = nullptr;
    SWG_CUDA(cudaGetLastError(), "occurrence scan launch");
    SWG_CUDA(cudaMemcpyAsync(&g->h_ctl->occ_total, g->d_prefix + n_reads, sizeof(uint64_t),
                             cudaMemcpyDeviceToHost, s),
             "read occurrence total");
    SWG_CUDA(cudaMemcpyAsync(&g->h_ctl->max_len, &g->d_ctl->max_len, sizeof(unsigned),
                             cudaMemcpyDeviceToHost, s),
             "read longest read");
    SWG_CUDA(cudaStreamSynchronize(s), "occurrence scan");
    a.total_occ = g->h_ctl->occ_total;
    g->occurrences = a.total_occ;
    g->retries = 0;
    g->estimate = 0;
    // the bucketed build walks one read per thread: reads of more than 16 kbp
    // (long-read data) would leave the GPU waiting on a few threads
    const bool bucketed = o->algorithm == SWG_ALGO_BUCKETED ||
                          (o->algorithm == SWG_ALGO_DEFAULT && o->read_order == SWG_ORDER_INPUT &&
                           g->h_ctl->max_len <= kBucketedMaxRead && bucketed_fits(g, a.total_occ));
    // the per-read occurrence prefix and the tiles of kTileOcc occurrences:
    // every algorithm but the bucketed build's thread-per-read scatter uses them
    if (!bucketed || swg::level1_shape(o->scatter_shape) == 4) {
        g->launches += swg::launch_occ_scan_write(a, s);
        a.n_tiles = (a.total_occ + swg::kTileOcc - 1) / swg::kTileOcc;
        if ((st = ensure(&g->d_tiles, &g->tiles_cap, a.n_tiles, "tile table"))) return st;
        a.tile_first_read = g->d_tiles;
        g->launches += swg::launch_tiles(a, s);
        SWG_CUDA(cudaGetLastError(), "tile launch");
    }
    if (o->algorithm == SWG_ALGO_PARTITIONED) return build_partitioned(g, o, a, s, load);
    if (bucketed) return build_bucketed(g, o, a, s, load);
    return build_direct(g, o, a, s, load);
}

// One pass into a device-wide table in HBM: HyperLogLog sizing, clear, K1, K2.
swg_status build_direct(swg_graph *g, const swg_opts *o, BuildArgs &a, cudaStream_t s,
                        double load) {
    swg_status st;
    g->algorithm = SWG_ALGO_DIRECT;
    // table sizing: caller's hint, else a HyperLogLog estimate on the device
    double est;
    if (o->expected_distinct) {
        est = (double)o->expected_distinct;
    } else if (a.total_occ == 0) {
        est = 0;
    } else {
        est = -1;  // from the sketch below
    }
    // One pass computes the HyperLogLog registers and every read's minimizer;
    // the reads are then counted in minimizer order (reads sharing a
    // minimizer overlap, so their shared k-molecules hit entries already in L2).
    const bool reorder = o->read_order == SWG_ORDER_MINIMIZER && a.total_occ > 0;
    if (reorder) {
        if ((st = ensure(&g->d_minhash, &g->minhash_cap, a.n_reads, "read minimizers"))) return st;
        SWG_CUDA(cudaMemsetAsync(g->d_minhash, 0xff, a.n_reads * sizeof(unsigned), s), "clear minimizers");
        SWG_CUDA(cudaMemsetAsync(g->d_hll, 0, sizeof(unsigned) << swg::kHllBits, s), "memset hll");
        g->launches += swg::launch_sketch(a, g->d_minhash, s);
        SWG_CUDA(cudaGetLastError(), "sketch launch");
    } else if (est < 0) {
        SWG_CUDA(cudaMemsetAsync(g->d_hll, 0, sizeof(unsigned) << swg::kHllBits, s), "memset hll");
        g->launches += swg::launch_hll(a, s);
        SWG_CUDA(cudaGetLastError(), "hll launch");
    }
    if (reorder) {
        if ((st = ensure(&g->d_bucket, &g->bucket_cap, swg::bucket_count(), "read buckets"))) return st;
        if ((st = ensure(&g->d_poff, &g->poff_cap, a.n_reads, "ordered offsets"))) return st;
        if ((st = ensure(&g->d_plen, &g->plen_cap, a.n_reads, "ordered lengths"))) return st;
        g->launches += swg::launch_read_order(a, g->d_minhash, g->d_bucket, g->d_poff, g->d_plen, s);
        a.read_off = g->d_poff;
        a.read_len = g->d_plen;
        g->launches += swg::launch_occ_scan(a, s);
        g->launches += swg::launch_tiles(a, s);
        SWG_CUDA(cudaGetLastError(), "read order launch");
    }
    if (est < 0) {
        SWG_CUDA(cudaMemcpyAsync(g->h_hll, g->d_hll, sizeof(unsigned) << swg::kHllBits,
                                 cudaMemcpyDeviceToHost, s),
                 "read hll");
        SWG_CUDA(cudaStreamSynchronize(s), "hll");
        est = swg::hll_estimate(g->h_hll) * 1.06;  // ~3.7 standard errors of margin
    }
    est = std::min(est, (double)a.total_occ);
    g->estimate = est;
    uint64_t cap = (uint64_t)std::ceil(std::max(est, 1.0) / load) + 64;
    for (int attempt = 0; attempt < 6; ++attempt) {
        if ((st = ensure(&g->d_table, &g->table_cap, cap, "hash table"))) return st;
        if (g->out_cap < cap || !g->d_out_keys || !g->d_out_mult) {
            cudaFree(g->d_out_keys);
            cudaFree(g->d_out_mult);
            g->d_out_keys = g->d_out_mult = nullptr;
            g->out_cap = 0;
            SWG_CUDA(cudaMalloc(&g->d_out_keys, cap * sizeof(unsigned long long)), "output keys");
            SWG_CUDA(cudaMalloc(&g->d_out_mult, cap * sizeof(unsigned long long)),
                     "output multiplicities");
            g->out_cap = cap;
        }
        a.table = g->d_table;
        a.cap = cap;
        a.out_keys = g->d_out_keys;
        a.out_mult = g->d_out_mult;
        a.out_cap = cap;
        SWG_CUDA(cudaEventRecord(g->ev[1], s), "event");
        SWG_CUDA(cudaMemsetAsync(g->d_table, 0, cap * sizeof(Entry), s), "clear table");
        SWG_CUDA(cudaMemsetAsync(g->d_ctl, 0, sizeof(Control) - sizeof(uint64_t), s),
                 "clear control");
        SWG_CUDA(cudaEventRecord(g->ev[2], s), "event");
        g->launches += swg::launch_count(a, s);
        SWG_CUDA(cudaGetLastError(), "count launch");
        SWG_CUDA(cudaEventRecord(g->ev[3], s), "event");
        g->launches += swg::launch_compact(a, s);
        SWG_CUDA(cudaGetLastError(), "compact launch");
        SWG_CUDA(cudaEventRecord(g->ev[4], s), "event");
        SWG_CUDA(cudaMemcpyAsync(g->h_ctl, g->d_ctl, sizeof(Control) - sizeof(uint64_t),
                                 cudaMemcpyDeviceToHost, s),
                 "read status");
        SWG_CUDA(cudaStreamSynchronize(s), "build");
        const unsigned status = g->h_ctl->status;
        if (status & swg::kStatusCasLimit) {
            swg::set_error("a bounded CAS retry loop gave up on the device");
            return SWG_ERR_TIMEOUT;
        }
        if (status & swg::kStatusTableFull) {
            // the distinct count never exceeds the occurrence count: retry at
            // that bound first, then double (only a probe-length pathology
            // can fill a table sized by the bound)
            const uint64_t bound = (uint64_t)std::ceil((double)a.total_occ / load) + 64;
            cap = cap < bound ? bound : cap * 2;
            g->retries++;
            continue;
        }
        g->n_distinct = g->h_ctl->counters[0];
        g->n_out = g->h_ctl->counters[1];
        g->cap_used = cap;
        g->built = true;
        float t[5] = {0, 0, 0, 0, 0};
        cudaEventElapsedTime(&t[0], g->ev[0], g->ev[1]);
        cudaEventElapsedTime(&t[1], g->ev[1], g->ev[2]);
        cudaEventElapsedTime(&t[2], g->ev[2], g->ev[3]);
        cudaEventElapsedTime(&t[3], g->ev[3], g->ev[4]);
        cudaEventElapsedTime(&t[4], g->ev[0], g->ev[4]);
        std::memcpy(g->ms, t, sizeof(t));
        return SWG_OK;
    }
    swg::set_error("hash table still full after 6 enlargements");
    return SWG_ERR_TABLE_FULL;
}

// Hash-partitioned counting: every occurrence becomes an 8-byte record
// {low bits of rmix64(key), arc code}, scattered to the partition named by the
// top bits; each partition is then counted in a table slice sized by its
// record count (an upper bound on its distinct keys) that stays resident in
// L2, several partitions (a wave) at a time, and compacted straight from L2.
swg_status build_partitioned(swg_graph *g, const swg_opts *o, BuildArgs &a, cudaStream_t s,
                             double load) {
    swg_status st;
    g->algorithm = SWG_ALGO_PARTITIONED;
    // about 1M slice entries (16 MiB) per partition, 2^8..2^10 partitions
    const double want = (double)a.total_occ / load / (double)(1u << 20);
    int bits = swg::kPartBitsMin;
    while (bits < swg::kPartBitsMax && (double)(1u << bits) < want) bits++;
    swg::PartArgs pa;
    std::memset(&pa, 0, sizeof(pa));
    pa.bits = bits;
    pa.n_parts = 1u << bits;
    pa.work = g->d_ctl->work;
    pa.shape = o ? o->scatter_shape : 0;  // zeroed with the control block at the start of the build
    pa.load_num = 3;  // slice capacity = count / 0.6 + 16
    pa.load_den = 5;
    if (load != 0.6) {
        pa.load_num = (int)std::lround(load * 1000.0);
        pa.load_den = 1000;
    }
    const uint64_t P = pa.n_parts;
    if ((st = ensure(&g->d_part, &g->part_cap, 3 * P + 1, "partition table"))) return st;
    pa.part_count = g->d_part;
    pa.part_start = g->d_part + P;
    pa.part_cursor = g->d_part + 2 * P + 1;
    SWG_CUDA(cudaMemsetAsync(pa.part_count, 0, P * sizeof(unsigned long long), s), "clear partitions");
    g->launches += swg::launch_part_count(a, pa, s);
    g->launches += swg::launch_part_prefix(pa, s);
    SWG_CUDA(cudaGetLastError(), "partition count launch");
    SWG_CUDA(cudaMemcpyAsync(g->h_part, pa.part_start, (P + 1) * sizeof(unsigned long long),
                             cudaMemcpyDeviceToHost, s),
             "read partition offsets");
    SWG_CUDA(cudaEventRecord(g->ev[1], s), "event");
    SWG_CUDA(cudaStreamSynchronize(s), "partition count");
    const unsigned long long *start = g->h_part;
    uint64_t max_count = 0;
    for (uint64_t p = 0; p < P; p++) max_count = std::max<uint64_t>(max_count, start[p + 1] - start[p]);
    const uint64_t chunk = 256 * 8;  // k_part_compact block chunk
    uint64_t slot_cap = max_count * (uint64_t)pa.load_den / (uint64_t)pa.load_num + 16;
    slot_cap = (slot_cap + chunk - 1) / chunk * chunk;
    int dev = g->device, l2 = 0;
    cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev);
    const double budget = 0.55 * (double)(l2 > 0 ? l2 : (126 << 20));
    uint64_t slots = (uint64_t)(budget / (double)(slot_cap * sizeof(Entry)));
    slots = std::max<uint64_t>(1, std::min<uint64_t>(slots, std::min<uint64_t>(P, 64)));
    pa.slot_cap = slot_cap;
    pa.n_slots = (uint32_t)slots;
    if ((st = ensure(&g->d_slices, &g->slices_cap, slots * slot_cap, "partition slices"))) return st;
    if ((st = ensure(&g->d_records, &g->records_cap, std::max<uint64_t>(a.total_occ, 1),
                     "partition records")))
        return st;
    const uint64_t out_want = std::max<uint64_t>(a.total_occ, 1);
    if (g->out_cap < out_want || !g->d_out_keys || !g->d_out_mult) {
        cudaFree(g->d_out_keys);
        cudaFree(g->d_out_mult);
        g->d_out_keys = g->d_out_mult = nullptr;
        g->out_cap = 0;
        SWG_CUDA(cudaMalloc(&g->d_out_keys, out_want * 8), "output keys");
        SWG_CUDA(cudaMalloc(&g->d_out_mult, out_want * 8), "output multiplicities");
        g->out_cap = out_want;
    }
    pa.slices = g->d_slices;
    pa.records = g->d_records;
    a.out_keys = g->d_out_keys;
    a.out_mult = g->d_out_mult;
    a.out_cap = out_want;
    SWG_CUDA(cudaMemsetAsync(g->d_slices, 0, slots * slot_cap * sizeof(Entry), s), "clear slices");
    g->launches += swg::launch_part_scatter(a, pa, s);
    SWG_CUDA(cudaGetLastError(), "scatter launch");
    SWG_CUDA(cudaEventRecord(g->ev[2], s), "event");
    uint32_t waves = 0;
    for (uint64_t p0 = 0; p0 < P; p0 += slots) {
        const uint32_t n = (uint32_t)std::min<uint64_t>(slots, P - p0);
        g->launches += swg::launch_part_wave(a, pa, (uint32_t)p0, n, start[p0], start[p0 + n], s);
        waves++;
    }
    SWG_CUDA(cudaGetLastError(), "wave launch");
    SWG_CUDA(cudaEventRecord(g->ev[3], s), "event");
    SWG_CUDA(cudaEventRecord(g->ev[4], s), "event");
    SWG_CUDA(cudaMemcpyAsync(g->h_ctl, g->d_ctl, sizeof(Control) - sizeof(uint64_t),
                             cudaMemcpyDeviceToHost, s),
             "read status");
    SWG_CUDA(cudaStreamSynchronize(s), "build");
    const unsigned status = g->h_ctl->status;
    if (status & swg::kStatusCasLimit) {
        swg::set_error("a bounded CAS retry loop gave up on the device");
        return SWG_ERR_TIMEOUT;
    }
    if (status & swg::kStatusTableFull) {
        swg::set_error("a partition slice reached the probe limit");
        return SWG_ERR_TABLE_FULL;
    }
    g->parts = (uint32_t)P;
    g->slots = (uint32_t)slots;
    g->waves = waves;
    g->slot_cap = slot_cap;
    g->cap_used = slot_cap;
    g->n_distinct = g->h_ctl->counters[0];
    g->n_out = g->h_ctl->counters[1];
    g->built = true;
    float t[5] = {0, 0, 0, 0, 0};
    cudaEventElapsedTime(&t[0], g->ev[0], g->ev[1]);
    cudaEventElapsedTime(&t[1], g->ev[1], g->ev[2]);
    cudaEventElapsedTime(&t[2], g->ev[2], g->ev[3]);
    cudaEventElapsedTime(&t[4], g->ev[0], g->ev[4]);
    std::memcpy(g->ms, t, sizeof(t));
    return SWG_OK;
}

// ---------------------------------------------------------------------
// Batched build: all samples are segments of one build (direct algorithm).
// Batched build on the bucketed scheme: the sample index sits in the top tb
// bits of every key (tb = 0 for one sample), each bucket applies its keys'
// own sample cutoffs and counts per sample, and a final pass moves the
// survivors into per-sample ranges with the tag stripped.
swg_status batch_bucketed(swg_graph *g, const swg_opts *o, const swg_sample *sm, uint32_t S,
                          BuildArgs &a, cudaStream_t s, double load, int tb) {
    swg_status st;
    a.tag_bits = S > 1 ? tb : 0;
    a.cutoff = sm[0].cutoff;  // the single sample's, when untagged
    a.k = sm[0].k;
    SWG_CUDA(cudaMemsetAsync(g->d_ctl, 0, sizeof(Control) - sizeof(uint64_t), s), "clear control");
    SWG_CUDA(cudaMemsetAsync(g->d_seg_counts, 0, 2ull * S * 8, s), "clear counters");
    if ((st = build_bucketed(g, o, a, s, load))) return st;
    g->n_samples = S;
    g->s_tbase.assign(S, 0);
    g->s_tcap.assign(S, 0);
    g->s_out.assign(S, 0);
    g->s_distinct.assign(S, 0);
    if (!a.tag_bits) {
        g->s_out[0] = g->n_out;
        g->s_distinct[0] = g->n_distinct;
        g->s_tcap[0] = g->n_out;
        return SWG_OK;
    }
    std::vector<unsigned long long> counts(2 * (uint64_t)S);
    SWG_CUDA(cudaMemcpyAsync(counts.data(), g->d_seg_counts, counts.size() * 8, cudaMemcpyDeviceToHost, s),
             "read sample counters");
    SWG_CUDA(cudaStreamSynchronize(s), "sample counters");
    std::vector<unsigned long long> cur(S);
    uint64_t total = 0;
    for (uint32_t i = 0; i < S; i++) {
        g->s_distinct[i] = counts[2 * i];
        g->s_out[i] = counts[2 * i + 1];
        g->s_tbase[i] = total;
        g->s_tcap[i] = counts[2 * i + 1];
        cur[i] = total;
        total += counts[2 * i + 1];
    }
    if (total != g->n_out) {
        swg::set_error("batch: per-sample survivor counts disagree with the total");
        return SWG_ERR_CUDA;
    }
    if ((st = ensure(&g->d_seg_cursor, &g->seg_cursor_cap, S, "sample cursors"))) return st;
    if (g->out2_cap < total || !g->d_out2_keys || !g->d_out2_mult) {
        cudaFree(g->d_out2_keys);
        cudaFree(g->d_out2_mult);
        g->d_out2_keys = g->d_out2_mult = nullptr;
        g->out2_cap = 0;
        const uint64_t want = std::max<uint64_t>(total, 1);
        SWG_CUDA(cudaMalloc(&g->d_out2_keys, want * 8), "grouped keys");
        SWG_CUDA(cudaMalloc(&g->d_out2_mult, want * 8), "grouped multiplicities");
        g->out2_cap = want;
    }
    SWG_CUDA(cudaMemcpyAsync(g->d_seg_cursor, cur.data(), S * 8, cudaMemcpyHostToDevice, s), "sample cursors");
    g->launches += swg::launch_group_by_sample(g->d_out_keys, g->d_out_mult, total, a.tag_bits, S,
                                               g->d_seg_cursor, g->d_out2_keys, g->d_out2_mult, s);
    SWG_CUDA(cudaGetLastError(), "group launch");
    SWG_CUDA(cudaStreamSynchronize(s), "group by sample");
    std::swap(g->d_out_keys, g->d_out2_keys);
    std::swap(g->d_out_mult, g->d_out2_mult);
    std::swap(g->out_cap, g->out2_cap);
    return SWG_OK;
}

swg_status batch_impl(swg_graph *g, const swg_opts *o, const swg_sample *sm, uint32_t S) {
    if (!o || !sm || S == 0) {
        swg::set_error("batch: no samples");
        return SWG_ERR_BAD_INPUT;
    }
    if (o->load_factor < 0 || o->load_factor > 0.9) {
        swg::set_error("load_factor must be in (0, 0.9] (0 = default)");
        return SWG_ERR_BAD_INPUT;
    }
    uint64_t W = 0, R = 0;
    std::vector<uint64_t> meta(3 * (uint64_t)S + 2, 0);  // read start [S+1] | shift [S] | prefix [S+1]
    for (uint32_t i = 0; i < S; i++) {
        if (sm[i].k < 1 || sm[i].k > 31) {
            swg::set_error("batch: sample k must be in 1..31");
            return SWG_ERR_BAD_INPUT;
        }
        if (sm[i].n_reads && (!sm[i].packed || !sm[i].read_off || !sm[i].read_len)) {
            swg::set_error("batch: NULL read buffer");
            return SWG_ERR_BAD_INPUT;
        }
        meta[i] = R;
        meta[S + 1 + i] = W * 16;  // base offset of the sample's words in the stream
        R += sm[i].n_reads;
        W += sm[i].n_words;
    }
    meta[S] = R;
    if (R >= 0xffffffffull) {
        swg::set_error("at most 2^32-2 reads per build");
        return SWG_ERR_BAD_INPUT;
    }
    SWG_CUDA(cudaSetDevice(g->device), "cudaSetDevice");
    cudaStream_t s = stream_of(g, o);
    const double load = o->load_factor > 0 ? o->load_factor : 0.6;
    g->built = false;
    g->merged = false;
    g->launches = 0;
    g->retries = 0;
    g->algorithm = SWG_ALGO_DIRECT;
    swg_status st;
    if ((st = ensure(&g->d_packed, &g->packed_cap, std::max<uint64_t>(W, 1), "packed reads"))) return st;
    if ((st = ensure_reads(g, R))) return st;
    if ((st = ensure(&g->d_read_seg, &g->read_seg_cap, std::max<uint64_t>(R, 1), "read samples")))
        return st;
    if ((st = ensure(&g->d_segs, &g->segs_cap, S, "sample table"))) return st;
    if ((st = ensure(&g->d_seg_counts, &g->seg_counts_cap, 2ull * S, "sample counters"))) return st;
    if ((st = ensure(&g->d_seg_status, &g->seg_status_cap, S, "sample status"))) return st;
    if ((st = ensure(&g->d_seg_meta, &g->seg_meta_cap, meta.size(), "sample metadata"))) return st;
    if ((st = ensure(&g->d_est, &g->est_cap, S, "sample estimates"))) return st;
    if ((st = ensure(&g->d_hll_seg, &g->hll_seg_cap, (uint64_t)S << swg::kHllBits, "sample sketches")))
        return st;
    if ((st = ensure(&g->d_prefix, &g->prefix_cap, R + 1, "occurrence prefix"))) return st;
    if ((st = ensure(&g->d_scan, &g->scan_cap, swg::scan_block_count(R) + 1, "scan scratch"))) return st;

    SWG_CUDA(cudaEventRecord(g->ev[0], s), "event");
    uint64_t wofs = 0, rofs = 0;
    for (uint32_t i = 0; i < S; i++) {
        // host or device memory (the request server passes device copies)
        if (sm[i].n_words)
            SWG_CUDA(cudaMemcpyAsync(g->d_packed + wofs, sm[i].packed, sm[i].n_words * 4, cudaMemcpyDefault, s),
                     "copy packed reads");
        if (sm[i].n_reads) {
            SWG_CUDA(cudaMemcpyAsync(g->d_off + rofs, sm[i].read_off, sm[i].n_reads * 8, cudaMemcpyDefault, s),
                     "copy read offsets");
            SWG_CUDA(cudaMemcpyAsync(g->d_len + rofs, sm[i].read_len, sm[i].n_reads * 4, cudaMemcpyDefault, s),
                     "copy read lengths");
        }
        wofs += sm[i].n_words;
        rofs += sm[i].n_reads;
    }
    std::vector<swg::SegParams> segs(S);
    for (uint32_t i = 0; i < S; i++) {
        segs[i].k = sm[i].k;
        segs[i].cutoff = sm[i].cutoff;
        segs[i].tbase = 0;
        segs[i].tcap = 0;
    }
    SWG_CUDA(cudaMemcpyAsync(g->d_seg_meta, meta.data(), (2 * (uint64_t)S + 1) * 8,
                             cudaMemcpyHostToDevice, s), "copy sample metadata");
    SWG_CUDA(cudaMemcpyAsync(g->d_segs, segs.data(), S * sizeof(swg::SegParams),
                             cudaMemcpyHostToDevice, s), "copy sample table");
    BuildArgs a;
    std::memset(&a, 0, sizeof(a));
    a.packed = g->d_packed;
    a.n_words = W;
    a.read_off = g->d_off;
    a.read_len = g->d_len;
    a.n_reads = R;
    a.k = sm[0].k;
    a.occ_prefix = g->d_prefix;
    a.scan_blocks = g->d_scan;
    a.status = &g->d_ctl->status;
    a.counters = g->d_ctl->counters;
    a.read_seg = g->d_read_seg;
    a.segs = g->d_segs;
    a.n_segs = S;
    a.seg_counts = g->d_seg_counts;
    a.seg_status = g->d_seg_status;
    a.hll = g->d_hll_seg;
    g->launches += swg::launch_seg_setup(a, g->d_seg_meta, g->d_seg_meta + S + 1, g->d_read_seg,
                                         g->d_off, s);
    SWG_CUDA(cudaMemsetAsync(g->d_prefix, 0, sizeof(uint64_t), s), "memset prefix");
    g->launches += swg::launch_occ_scan(a, s);
    g->launches += swg::launch_gather_prefix(g->d_prefix, g->d_seg_meta, S + 1,
                                             g->d_seg_meta + 2 * (uint64_t)S + 1, s);
    SWG_CUDA(cudaGetLastError(), "batch setup launch");
    SWG_CUDA(cudaMemcpyAsync(meta.data() + 2 * S + 1, g->d_seg_meta + 2 * (uint64_t)S + 1,
                             (S + 1) * 8, cudaMemcpyDeviceToHost, s), "read sample occurrences");
    SWG_CUDA(cudaStreamSynchronize(s), "batch occurrence scan");
    const uint64_t *occ_pre = meta.data() + 2 * S + 1;
    a.total_occ = occ_pre[S];
    g->occurrences = a.total_occ;
    g->s_occ.assign(S, 0);
    for (uint32_t i = 0; i < S; i++) g->s_occ[i] = occ_pre[i + 1] - occ_pre[i];
    {
        // every key tagged with its sample in one bucketed build, when the tag
        // fits above the longest k-mer
        int kmax = 1, tb = 0;
        for (uint32_t i = 0; i < S; i++) kmax = std::max(kmax, sm[i].k);
        while ((1u << tb) < S) tb++;
        if ((o->algorithm == SWG_ALGO_DEFAULT || o->algorithm == SWG_ALGO_BUCKETED) &&
            o->read_order == SWG_ORDER_INPUT && S <= swg::kMaxTagSamples && 2 * kmax + tb <= 64 &&
            (o->algorithm == SWG_ALGO_BUCKETED || bucketed_fits(g, a.total_occ)))
            return batch_bucketed(g, o, sm, S, a, s, load, tb);
    }
    a.n_tiles = (a.total_occ + swg::kTileOcc - 1) / swg::kTileOcc;
    if ((st = ensure(&g->d_tiles, &g->tiles_cap, a.n_tiles, "tile table"))) return st;
    a.tile_first_read = g->d_tiles;
    g->launches += swg::launch_tiles(a, s);
    std::vector<double> est(S, 0.0);
    if (a.total_occ) {
        SWG_CUDA(cudaMemsetAsync(g->d_hll_seg, 0, ((uint64_t)S << swg::kHllBits) * 4, s), "memset sketches");
        g->launches += swg::launch_hll(a, s);
        g->launches += swg::launch_hll_estimates(g->d_hll_seg, S, g->d_est, s);
        SWG_CUDA(cudaGetLastError(), "sketch launch");
        SWG_CUDA(cudaMemcpyAsync(est.data(), g->d_est, S * sizeof(double), cudaMemcpyDeviceToHost, s),
                 "read estimates");
        SWG_CUDA(cudaStreamSynchronize(s), "batch sketch");
    }
    SWG_CUDA(cudaEventRecord(g->ev[1], s), "event");
    std::vector<uint64_t> cap(S);
    for (uint32_t i = 0; i < S; i++) {
        const double occ = (double)(occ_pre[i + 1] - occ_pre[i]);
        const double e = std::min(est[i] * 1.06, occ);
        cap[i] = (uint64_t)std::ceil(std::max(e, 1.0) / load) + 64;
    }
    const uint64_t chunk = 256 * 8;  // k_compact chunk: sample regions start on it
    for (int attempt = 0; attempt < 6; ++attempt) {
        uint64_t total = 0;
        for (uint32_t i = 0; i < S; i++) {
            segs[i].tbase = total;
            segs[i].tcap = cap[i];
            total += (cap[i] + chunk - 1) / chunk * chunk;
        }
        if ((st = ensure(&g->d_table, &g->table_cap, total, "hash table"))) return st;
        if (g->out_cap < total || !g->d_out_keys || !g->d_out_mult) {
            cudaFree(g->d_out_keys);
            cudaFree(g->d_out_mult);
            g->d_out_keys = g->d_out_mult = nullptr;
            g->out_cap = 0;
            SWG_CUDA(cudaMalloc(&g->d_out_keys, total * 8), "output keys");
            SWG_CUDA(cudaMalloc(&g->d_out_mult, total * 8), "output multiplicities");
            g->out_cap = total;
        }
        SWG_CUDA(cudaMemcpyAsync(g->d_segs, segs.data(), S * sizeof(swg::SegParams),
                                 cudaMemcpyHostToDevice, s), "copy sample table");
        a.table = g->d_table;
        a.cap = total;
        a.out_keys = g->d_out_keys;
        a.out_mult = g->d_out_mult;
        a.out_cap = total;
        SWG_CUDA(cudaMemsetAsync(g->d_table, 0, total * sizeof(Entry), s), "clear table");
        SWG_CUDA(cudaMemsetAsync(g->d_seg_counts, 0, 2ull * S * 8, s), "clear counters");
        SWG_CUDA(cudaMemsetAsync(g->d_seg_status, 0, S * 4, s), "clear status");
        SWG_CUDA(cudaEventRecord(g->ev[2], s), "event");
        g->launches += swg::launch_count(a, s);
        SWG_CUDA(cudaEventRecord(g->ev[3], s), "event");
        g->launches += swg::launch_compact(a, s);
        SWG_CUDA(cudaGetLastError(), "batch count launch");
        SWG_CUDA(cudaEventRecord(g->ev[4], s), "event");
        std::vector<unsigned long long> counts(2 * (uint64_t)S);
        std::vector<unsigned> status(S);
        SWG_CUDA(cudaMemcpyAsync(counts.data(), g->d_seg_counts, counts.size() * 8,
                                 cudaMemcpyDeviceToHost, s), "read counters");
        SWG_CUDA(cudaMemcpyAsync(status.data(), g->d_seg_status, S * 4, cudaMemcpyDeviceToHost, s),
                 "read status");
        SWG_CUDA(cudaStreamSynchronize(s), "batch build");
        bool again = false;
        for (uint32_t i = 0; i < S; i++) {
            if (status[i] & swg::kStatusCasLimit) {
                swg::set_error("a bounded CAS retry loop gave up on the device");
                return SWG_ERR_TIMEOUT;
            }
            if (status[i] & swg::kStatusTableFull) {
                const uint64_t bound = (uint64_t)std::ceil((double)g->s_occ[i] / load) + 64;
                cap[i] = cap[i] < bound ? bound : cap[i] * 2;
                again = true;
            }
        }
        if (again) {
            g->retries++;
            continue;
        }
        g->n_samples = S;
        g->s_tbase.resize(S);
        g->s_tcap.resize(S);
        g->s_out.resize(S);
        g->s_distinct.resize(S);
        for (uint32_t i = 0; i < S; i++) {
            g->s_tbase[i] = segs[i].tbase;
            g->s_tcap[i] = segs[i].tcap;
            g->s_distinct[i] = counts[2 * i];
            g->s_out[i] = counts[2 * i + 1];
        }
        g->n_distinct = 0;
        g->n_out = 0;
        for (uint32_t i = 0; i < S; i++) {
            g->n_distinct += g->s_distinct[i];
            g->n_out += g->s_out[i];
        }
        g->cap_used = total;
        g->built = true;
        float t[5] = {0, 0, 0, 0, 0};
        cudaEventElapsedTime(&t[0], g->ev[0], g->ev[1]);
        cudaEventElapsedTime(&t[1], g->ev[1], g->ev[2]);
        cudaEventElapsedTime(&t[2], g->ev[2], g->ev[3]);
        cudaEventElapsedTime(&t[3], g->ev[3], g->ev[4]);
        cudaEventElapsedTime(&t[4], g->ev[0], g->ev[4]);
        std::memcpy(g->ms, t, sizeof(t));
        return SWG_OK;
    }
    swg::set_error("hash table still full after 6 enlargements");
    return SWG_ERR_TABLE_FULL;
}

// Bucketed counting: the records of the hash partitions (as in the
// partitioned build) are split again into buckets of a few hundred records by
// the next hash bits, and every bucket is counted by one CTA in a
// shared-memory hash table and compacted from there. Buckets too large for
// shared memory (hot k-molecules) are counted in a global-memory table.
// Bucketed build (kernels.cu, k_p1_* / k_sub_* / k_bucket_*). A sampled pass
// (every 16th batch of reads, from 64M occurrences; uniform below) sizes
// every level-1 partition and every bucket;
// the scatters write into those regions, so no exact count pass precedes
// them. A partition or bucket that outgrows its region (a sampling miss) sets
// a status bit, the later kernels skip their work, and the build reruns with
// exact counts (counted = true).
struct BucketPlan {
    int b1 = 0, b2 = 0;
    uint64_t P = 0, NB = 0;
    swg::PartArgs pa;
    swg::BucketArgs bk;
    unsigned long long *scr = nullptr, *sampled = nullptr;
};

// Sizes the bucketed build for N occurrences, allocates its workspace and
// lays out the level-1 partition and bucket regions: from exact counts over
// the reads of a (counted), else from a sample of them (every stride-th
// batch, once N reaches 64M occurrences).
swg_status bucketed_plan(swg_graph *g, const swg_opts *o, const BuildArgs &a, uint64_t N, bool counted,
                         uint32_t stride, cudaStream_t s, BucketPlan &pl) {
    swg_status st;
    // level-1 partitions: 256, 512 past 400M occurrences (a level-1 round of
    // 4096 records still writes runs of 8), 1024 only past 6.4G; the options
    // (then SWG_PART_BITS) override
    int b1 = N <= (400ull << 20) ? 8 : (N <= (6400ull << 20) ? 9 : 10);
    if (const char *e = std::getenv("SWG_PART_BITS")) b1 = std::min(10, std::max(8, std::atoi(e)));
    if (o && o->part_bits) b1 = std::min(10, std::max(8, o->part_bits));
    // sub-buckets of about `target` records (the options, then SWG_BUCKET_RECORDS, override)
    double target = 4096.0;
    if (const char *e = std::getenv("SWG_BUCKET_RECORDS")) target = std::max(64.0, std::atof(e));
    if (o && o->bucket_records) target = std::min(65535.0, std::max(64.0, (double)o->bucket_records));
    // more partitions when even 1024 sub-buckets each would leave buckets past
    // twice the target (they would outgrow the shared-memory tables)
    while (b1 < 10 && (double)N / (double)((1ull << b1) << 10) > 2 * target) b1++;
    const uint64_t P = 1ull << b1;
    int b2 = 0;
    while (b2 < 10 && (double)N / (double)(P << b2) > target) b2++;
    // at most 512 sub-buckets (level-2 runs of >= 8 records per 4096-record
    // chunk) while the buckets stay under 4x the target
    if (b2 == 10 && (double)N / (double)(P << 9) <= 4 * target) b2 = 9;
    const uint64_t NB = P << b2;
    // region bounds: partitions <= 1.25 N + 4097 P, buckets <= 1.5 N + 257 NB;
    // the level-1 buffer also stages survivor keys at bucket offsets
    const uint64_t rec1_bound = counted ? N : N + N / 4 + 4097 * P;
    const uint64_t rec2_bound = counted ? N : N + N / 2 + 257 * NB;
    swg::PartArgs pa;
    std::memset(&pa, 0, sizeof(pa));
    pa.bits = b1;
    pa.n_parts = (uint32_t)P;
    pa.load_num = 3;
    pa.load_den = 5;
    pa.work = g->d_ctl->work;
    pa.shape = o ? o->scatter_shape : 0;
    if ((st = ensure(&g->d_part, &g->part_cap, 4 * P + 1, "partition table"))) return st;
    pa.part_count = g->d_part;
    pa.part_start = g->d_part + P;
    pa.part_cursor = g->d_part + 2 * P + 1;
    // +2: the level-2 bulk copies may round a chunk's end up to an even record
    if ((st = ensure(&g->d_records, &g->records_cap, std::max(rec1_bound, rec2_bound) + 2, "records")))
        return st;
    if ((st = ensure(&g->d_rec2, &g->rec2_cap, std::max<uint64_t>(rec2_bound, 1), "bucket records"))) return st;
    const uint64_t scratch = swg::gscan_scratch(NB);
    // d_bk: cursors [NB] | regions [NB+1] | big list [NB] | survivor prefix
    // [NB+1] | scan scratch | sampled total [2] | chunk prefix [P+1] | second
    // big list [NB] | survivors per bucket [NB]
    if ((st = ensure(&g->d_bk, &g->bk_cap, 6 * NB + 2 + scratch + 2 + P + 1, "bucket table"))) return st;
    pa.records = g->d_records;
    swg::BucketArgs bk;
    std::memset(&bk, 0, sizeof(bk));
    bk.b1 = b1;
    bk.b2 = b2;
    bk.shape = o ? o->scatter_shape : 0;
    bk.n_parts = (uint32_t)P;
    bk.part_start = pa.part_start;
    bk.part_cursor = pa.part_cursor;
    bk.part_end = g->d_part + 3 * P + 1;
    bk.status = &g->d_ctl->status;
    bk.rec1 = g->d_records;
    bk.rec2 = g->d_rec2;
    bk.cursor2 = g->d_bk;
    bk.off2 = g->d_bk + NB;
    bk.big = g->d_bk + 2 * NB + 1;
    bk.big_cap = (uint32_t)std::min<uint64_t>(NB, 0xffffffffu);
    bk.big_count = &g->d_ctl->pad;
    bk.n_rec = N;
    bk.surv_off = g->d_bk + 3 * NB + 1;
    bk.stage_keys = g->d_records;  // level-1 records are spent by then
    unsigned long long *scr = bk.surv_off + NB + 1;
    unsigned long long *sampled = scr + scratch;
    bk.chunk_start = sampled + 2;
    bk.big2 = bk.chunk_start + P + 1;
    bk.big2_count = &g->d_ctl->pad2;
    bk.surv = bk.big2 + NB;

    SWG_CUDA(cudaMemsetAsync(pa.part_count, 0, P * 8, s), "clear partitions");
    if (counted) {
        g->launches += swg::launch_part_count(a, pa, s);
        g->launches += swg::launch_part_prefix(pa, s);
    } else {
        SWG_CUDA(cudaMemsetAsync(bk.cursor2, 0, NB * 8, s), "clear bucket samples");
        // from 64M occurrences every stride-th batch of reads is sampled;
        // smaller inputs get uniform regions (an empty sample), whose slack
        // covers their spread (a skewed one recounts)
        if (N >= (64ull << 20)) g->launches += swg::launch_p1_sample(a, pa, bk, stride, s);
        g->launches += swg::launch_part_caps(pa, N, sampled, s);
        // bucket regions from the same sample (surv serves as scratch)
        g->launches += swg::launch_bucket_caps(bk.cursor2, sampled, N, NB, bk.surv, s);
        g->launches += swg::launch_gscan(reinterpret_cast<const uint64_t *>(bk.surv),
                                         reinterpret_cast<uint64_t *>(bk.off2), NB,
                                         reinterpret_cast<uint64_t *>(scr),
                                         reinterpret_cast<uint64_t *>(bk.off2 + NB), s);
        SWG_CUDA(cudaMemcpyAsync(bk.cursor2, bk.off2, NB * 8, cudaMemcpyDeviceToDevice, s), "bucket cursors");
    }
    pl.b1 = b1;
    pl.b2 = b2;
    pl.P = P;
    pl.NB = NB;
    pl.pa = pa;
    pl.bk = bk;
    pl.scr = scr;
    pl.sampled = sampled;
    return SWG_OK;
}

swg_status bucketed_finish(swg_graph *g, const swg_opts *o, BuildArgs &a, cudaStream_t s, double load,
                           bool counted, BucketPlan &pl);

swg_status build_bucketed(swg_graph *g, const swg_opts *o, BuildArgs &a, cudaStream_t s,
                          double load, bool counted) {
    swg_status st;
    g->algorithm = SWG_ALGO_BUCKETED;
    BucketPlan pl;
    if ((st = bucketed_plan(g, o, a, a.total_occ, counted, 16, s, pl))) return st;
    SWG_CUDA(cudaEventRecord(g->ev[1], s), "event");
    g->launches += swg::launch_part_scatter(a, pl.pa, s);
    SWG_CUDA(cudaEventRecord(g->ev[2], s), "event");
    return bucketed_finish(g, o, a, s, load, counted, pl);
}

// Everything after the level-1 scatter: level-2 scatter, bucket counting,
// survivor packing, the big buckets; an overflowed region reruns the build
// with exact counts.
swg_status bucketed_finish(swg_graph *g, const swg_opts *o, BuildArgs &a, cudaStream_t s, double load,
                           bool counted, BucketPlan &pl) {
    swg_status st;
    g->algorithm = SWG_ALGO_BUCKETED;
    if (g->host_keys && !a.tag_bits) {  // survivors also straight to the caller's host arrays
        a.host_keys = g->host_keys;
        a.host_mult = g->host_mult;
        a.host_cap = g->host_cap;
        a.host_written = &g->d_ctl->host_written;
        g->host_out_used = true;
    }
    const uint64_t N = a.total_occ;
    const int b1 = pl.b1, b2 = pl.b2;
    const uint64_t P = pl.P, NB = pl.NB;
    swg::BucketArgs &bk = pl.bk;
    unsigned long long *scr = pl.scr;
    (void)P;
    g->launches += swg::launch_chunk_prefix(bk, s);
    if (counted) {  // exact bucket regions
        SWG_CUDA(cudaMemsetAsync(bk.cursor2, 0, NB * 8, s), "clear bucket counts");
        g->launches += swg::launch_sub_hist(bk, s);
        g->launches += swg::launch_gscan(reinterpret_cast<const uint64_t *>(bk.cursor2),
                                         reinterpret_cast<uint64_t *>(bk.off2), NB,
                                         reinterpret_cast<uint64_t *>(scr),
                                         reinterpret_cast<uint64_t *>(bk.off2 + NB), s);
        SWG_CUDA(cudaMemcpyAsync(bk.cursor2, bk.off2, NB * 8, cudaMemcpyDeviceToDevice, s), "bucket cursors");
    }
    g->launches += swg::launch_sub_scatter(bk, s);
    SWG_CUDA(cudaGetLastError(), "bucket scatter launch");
    SWG_CUDA(cudaEventRecord(g->ev[3], s), "event");
    g->launches += swg::launch_bucket_count(a, bk, s);
    g->bucket_table = (uint32_t)swg::bucket_count_table(a, bk);
    SWG_CUDA(cudaEventRecord(g->ev[5], s), "event");
    g->launches += swg::launch_gscan(reinterpret_cast<const uint64_t *>(bk.surv),
                                     reinterpret_cast<uint64_t *>(bk.surv_off), NB,
                                     reinterpret_cast<uint64_t *>(scr),
                                     reinterpret_cast<uint64_t *>(bk.surv_off + NB), s);
    SWG_CUDA(cudaGetLastError(), "bucket count launch");
    SWG_CUDA(cudaMemcpyAsync(&g->h_ctl->occ_total, bk.surv_off + NB, sizeof(uint64_t),
                             cudaMemcpyDeviceToHost, s), "read survivor total");
    SWG_CUDA(cudaMemcpyAsync(g->h_ctl, g->d_ctl, sizeof(Control) - sizeof(uint64_t),
                             cudaMemcpyDeviceToHost, s), "read status");
    SWG_CUDA(cudaStreamSynchronize(s), "bucket count");
    if (!counted && (g->h_ctl->status & swg::kStatusPartOverflow)) {
        // a partition or bucket outgrew its sampled region: recount exactly,
        // from a clear control block
        g->h_ctl->occ_total = N;
        SWG_CUDA(cudaMemsetAsync(g->d_ctl, 0, sizeof(Control) - sizeof(uint64_t), s), "clear control");
        if (a.tag_bits)
            SWG_CUDA(cudaMemsetAsync(a.seg_counts, 0, 2ull * a.n_segs * 8, s), "clear sample counters");
        return build_bucketed(g, o, a, s, load, true);
    }
    if (g->h_ctl->status & swg::kStatusPartOverflow) {
        swg::set_error("bucketed build: a region overflowed with exact counts");
        return SWG_ERR_CUDA;
    }
    const uint64_t n_small = g->h_ctl->occ_total;
    g->h_ctl->occ_total = N;
    const unsigned nbig = g->h_ctl->pad2;  // buckets no shared-memory table held
    std::vector<unsigned long long> meta;   // rb [n] | hash prefix [n] | record prefix [n+1]
    uint64_t big_records = 0;
    if (nbig) {
        std::vector<unsigned long long> big(nbig), off(NB + 1), cur(NB);
        SWG_CUDA(cudaMemcpyAsync(big.data(), bk.big2, nbig * 8, cudaMemcpyDeviceToHost, s), "read big buckets");
        SWG_CUDA(cudaMemcpyAsync(off.data(), bk.off2, (NB + 1) * 8, cudaMemcpyDeviceToHost, s), "read regions");
        SWG_CUDA(cudaMemcpyAsync(cur.data(), bk.cursor2, NB * 8, cudaMemcpyDeviceToHost, s), "read cursors");
        SWG_CUDA(cudaStreamSynchronize(s), "big buckets");
        meta.resize(3 * (uint64_t)nbig + 1);
        for (unsigned i = 0; i < nbig; i++) {
            const uint64_t bb = big[i], rb = off[bb], re = std::min<uint64_t>(cur[bb], off[bb + 1]);
            meta[i] = rb;
            meta[nbig + i] = (unsigned long long)(bb >> b2) << (64 - b1);
            meta[2 * nbig + i] = big_records;
            big_records += re - rb;
        }
        meta[3 * (uint64_t)nbig] = big_records;
    }
    // output: the survivors of the shared-memory buckets, then at most one
    // per record of the big buckets
    const uint64_t out_want = std::max<uint64_t>(n_small + big_records, 1);
    if (g->out_cap < out_want || !g->d_out_keys || !g->d_out_mult) {
        cudaFree(g->d_out_keys);
        cudaFree(g->d_out_mult);
        g->d_out_keys = g->d_out_mult = nullptr;
        g->out_cap = 0;
        SWG_CUDA(cudaMalloc(&g->d_out_keys, out_want * 8), "output keys");
        SWG_CUDA(cudaMalloc(&g->d_out_mult, out_want * 8), "output multiplicities");
        g->out_cap = out_want;
    }
    a.out_keys = g->d_out_keys;
    a.out_mult = g->d_out_mult;
    a.out_cap = g->out_cap;
    g->launches += swg::launch_bucket_gather(a, bk, NB, s);
    if (nbig) {  // all big buckets in one global-memory table (disjoint keys)
        if ((st = ensure(&g->d_bigmeta, &g->bigmeta_cap, meta.size(), "big-bucket list"))) return st;
        SWG_CUDA(cudaMemcpyAsync(g->d_bigmeta, meta.data(), meta.size() * 8, cudaMemcpyHostToDevice, s),
                 "big-bucket list");
        const uint64_t cap = (uint64_t)std::ceil((double)big_records / load) + 64;
        if ((st = ensure(&g->d_arena, &g->arena_cap, cap, "big-bucket table"))) return st;
        SWG_CUDA(cudaMemsetAsync(g->d_arena, 0, cap * sizeof(Entry), s), "clear big-bucket table");
        g->launches += swg::launch_big_multi(a, bk, g->d_bigmeta, nbig, big_records, g->d_arena, cap, s);
    }
    SWG_CUDA(cudaGetLastError(), "gather launch");
    SWG_CUDA(cudaMemcpyAsync(g->h_ctl, g->d_ctl, sizeof(Control) - sizeof(uint64_t),
                             cudaMemcpyDeviceToHost, s), "read status");
    SWG_CUDA(cudaEventRecord(g->ev[4], s), "event");
    SWG_CUDA(cudaStreamSynchronize(s), "build");
    const unsigned status = g->h_ctl->status;
    if (status & swg::kStatusCasLimit) {
        swg::set_error("a bounded CAS retry loop gave up on the device");
        return SWG_ERR_TIMEOUT;
    }
    if (status & swg::kStatusTableFull) {
        swg::set_error("a big-bucket table reached the probe limit");
        return SWG_ERR_TABLE_FULL;
    }
    g->retries = g->h_ctl->pad;
    g->estimate = counted ? 1.0 : 0.0;  // bucketed: 1 when the exact-count rerun was needed
    g->parts = (uint32_t)P;
    g->slots = (uint32_t)(1u << b2);
    g->waves = nbig;
    g->cap_used = NB;
    g->n_distinct = g->h_ctl->counters[0];
    g->n_out = g->h_ctl->counters[1];
    g->built = true;
    float t[5] = {0, 0, 0, 0, 0};
    // [0] setup, [1] level-1 scatter, [2] level-2 scatter, [3] bucket count
    cudaEventElapsedTime(&t[0], g->ev[0], g->ev[1]);
    cudaEventElapsedTime(&t[1], g->ev[1], g->ev[2]);
    cudaEventElapsedTime(&t[2], g->ev[2], g->ev[3]);
    cudaEventElapsedTime(&t[3], g->ev[3], g->ev[5]);
    cudaEventElapsedTime(&t[4], g->ev[0], g->ev[4]);
    std::memcpy(g->ms, t, sizeof(t));
    return SWG_OK;
}

// Grows a device array to want elements, keeping its first keep. Called
// only where the stream that uses the array is idle (after a synchronize).
template <typename T>
swg_status grow_keep(T **p, uint64_t *cap, uint64_t want, uint64_t keep, const char *what) {
    if (*p && *cap >= want) return SWG_OK;
    T *q = nullptr;
    const uint64_t n = std::max<uint64_t>(want, 1);
    cudaError_t e = cudaMalloc((void **)&q, n * sizeof(T));
    if (e == cudaSuccess && *p && keep) e = cudaMemcpy(q, *p, keep * sizeof(T), cudaMemcpyDeviceToDevice);
    if (e != cudaSuccess) {
        cudaGetLastError();
        cudaFree(q);
        return cuda_fail(e, what);
    }
    cudaFree(*p);
    *p = q;
    *cap = n;
    return SWG_OK;
}

constexpr uint64_t kStreamMin = 96ull << 20;    // shorter texts go up and are framed in one piece
constexpr uint64_t kStreamPiece = 40ull << 20;  // target bytes per piece
constexpr uint64_t kStreamMaxPieces = 16;

// Streamed FASTA build (texts of kStreamMin bytes and more). The text goes
// up in pieces on a copy stream; a framing stream frames each piece as it
// lands — newline counts, newline positions, the records completed so far,
// their packing — and, on the bucketed path, the build stream scatters that
// piece's reads to the level-1 partitions while the next pieces are copied
// and framed. The first piece is framed with host round trips: its totals
// size the build. Its occurrences per text byte scale to the whole text (a
// region that the estimate or the sample misses overflows, and the build
// recounts exactly, as the one-shot build does), its reads are the sample,
// and its densities, with slack, size the framing arrays for the whole text.
// The later pieces of a bucketed build are then framed on the device alone
// (the running totals and each piece's reads kept in device memory); a text
// that outgrows the arrays is framed again with round trips (synced). Any
// piece with a read longer than the bucketed build takes, another algorithm
// or read order, or a graph the bucketed workspace does not fit, falls back
// to the one-shot build over the reads framed here. Results are those of the
// one-shot build.
swg_status build_fasta_streamed(swg_graph *g, const swg_opts *o, const char *first, uint64_t n,
                                cudaStream_t s, bool synced = false) {
    swg_status st;
    const uint64_t nc = swg::framing_chunks(n);
    uint64_t C = std::min<uint64_t>(kStreamMaxPieces, std::max<uint64_t>(2, n / kStreamPiece));
    if (const char *e = std::getenv("SWG_STREAM_PIECES"))  // at most 16: the first piece is the sample
        C = std::min<uint64_t>(kStreamMaxPieces, std::max(2, std::atoi(e)));
    // piece c: bytes [cut[c], cut[c+1]), on framing-chunk bounds. The first
    // piece, whose copy nothing overlaps, is half a piece but at least 1/16
    // of the text (its reads are the sample: at least 1/16 of all reads)
    std::vector<uint64_t> cut(C + 1);
    const uint64_t first_blocks = std::max<uint64_t>(1, std::max(nc / (2 * C), nc / 16));
    cut[0] = 0;
    for (uint64_t c = 1; c < C; ++c)
        cut[c] = (first_blocks + (nc - first_blocks) * (c - 1) / (C - 1)) * swg::kFramingChunk;
    cut[C] = n;
    if (!g->copy) SWG_CUDA(cudaStreamCreateWithFlags(&g->copy, cudaStreamNonBlocking), "copy stream");
    if (!g->frame) {  // highest priority; the scatters of earlier pieces leave it an SM slot
        int least = 0, greatest = 0;
        SWG_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest), "stream priorities");
        SWG_CUDA(cudaStreamCreateWithPriority(&g->frame, cudaStreamNonBlocking, greatest), "framing stream");
    }
    cudaStream_t F = g->frame;
    while (g->piece_ev.size() < 2 * C) {  // copied [C] | packed [C]
        cudaEvent_t e = nullptr;
        SWG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "piece event");
        g->piece_ev.push_back(e);
    }
    cudaEvent_t *copied = g->piece_ev.data(), *packed_ev = copied + C;
    // +64: the packing kernel's aligned 16-byte loads read up to 31 bytes past a record
    if ((st = ensure(&g->d_text, &g->text_cap, n + 64, "FASTA text"))) return st;
    // the copies and the framing wait for earlier work on the build stream
    SWG_CUDA(cudaEventRecord(g->ev[6], s), "event");
    SWG_CUDA(cudaStreamWaitEvent(g->copy, g->ev[6], 0), "copy stream wait");
    SWG_CUDA(cudaStreamWaitEvent(F, g->ev[6], 0), "framing stream wait");
    for (uint64_t c = 0; c < C; ++c) {
        SWG_CUDA(cudaMemcpyAsync(g->d_text + cut[c], first + cut[c], cut[c + 1] - cut[c],
                                 cudaMemcpyHostToDevice, g->copy),
                 "copy FASTA piece");
        SWG_CUDA(cudaEventRecord(copied[c], g->copy), "piece event");
    }
    // the caller's buffer is read until the last copy ends, and the framing
    // stream's work must end before the arrays it writes are reused: no
    // return before both streams are idle
    struct Drain {
        cudaStream_t c, f;
        ~Drain() {
            cudaStreamSynchronize(c);
            cudaStreamSynchronize(f);
        }
    } drain{g->copy, F};
    // workspace: block counts [nc] | block bases [nc] | scan scratch [S] |
    // framing state [16] | each piece's reads [2 kStreamMaxPieces] | newline masks
    const uint64_t S = std::max(swg::gscan_scratch(nc), swg::rec_scan_scratch(n / 2 + 1));
    constexpr uint64_t kStateWords = 16;
    static_assert(sizeof(swg::StreamState) <= kStateWords * 8, "framing state");
    if ((st = ensure(&g->d_sfw, &g->sfw_cap,
                     2 * nc + S + kStateWords + 2 * kStreamMaxPieces + swg::newline_mask_words(n),
                     "framing workspace")))
        return st;
    uint64_t *counts = g->d_sfw, *cbase = counts + nc, *scratch = cbase + nc, *tot = scratch + S;
    auto *fs = reinterpret_cast<swg::StreamState *>(tot);  // tot[0..5]: newlines, piece reads, words, occ, longest, NUL
    auto *piece_reads = reinterpret_cast<unsigned long long *>(tot + kStateWords);
    uint64_t *masks = tot + kStateWords + 2 * kStreamMaxPieces;
    auto *acc = reinterpret_cast<unsigned long long *>(tot + 3);
    unsigned *nul_flag = reinterpret_cast<unsigned *>(tot + 5);
    SWG_CUDA(cudaMemsetAsync(tot, 0, kStateWords * 8, F), "clear framing state");

    // build state, as build_impl sets it
    g->built = false;
    g->merged = false;
    g->n_samples = 0;
    g->k = o->k;
    g->cutoff = o->cutoff;
    g->launches = 0;
    g->retries = 0;
    g->estimate = 0;
    const double load = o->load_factor > 0 ? o->load_factor : 0.6;
    SWG_CUDA(cudaEventRecord(g->ev[0], s), "event");
    SWG_CUDA(cudaMemsetAsync(g->d_ctl, 0, sizeof(Control), s), "memset control");
    BuildArgs a;
    std::memset(&a, 0, sizeof(a));
    a.k = o->k;
    a.cutoff = o->cutoff;
    a.hll = g->d_hll;
    a.status = &g->d_ctl->status;
    a.counters = g->d_ctl->counters;
    BucketPlan pl;
    bool stream = o->algorithm == SWG_ALGO_BUCKETED ||
                  (o->algorithm == SWG_ALGO_DEFAULT && o->read_order == SWG_ORDER_INPUT);
    int launches = 0;
    uint64_t NL = 0, R = 0, reads = 0, words = 0, occ = 0, longest = 0;
    // after the first piece (framed with host round trips: it sizes the
    // build), the pieces of a bucketed build are framed on the device alone,
    // into capacities for the whole text estimated from the first piece; a
    // text that outgrows them is framed again with round trips (synced)
    bool fast = stream && !synced;
    uint64_t nl_cap = 0, rec_cap = 0;
    for (uint64_t c = 0; c < C; ++c) {
        SWG_CUDA(cudaStreamWaitEvent(F, copied[c], 0), "piece wait");
        const uint64_t j0 = cut[c] / swg::kFramingChunk, end = cut[c + 1];
        if (fast && c > 0) {
            launches += swg::launch_nl_count(g->d_text, end, counts, masks, nul_flag, F, j0);
            launches += swg::launch_gscan(counts, cbase, swg::framing_chunks(end), scratch, tot, F);
            launches += swg::launch_nl_pos(masks, end, cbase, g->d_nl, F, j0, nl_cap,
                                           reinterpret_cast<uint64_t *>(&fs->overflow));
            launches += swg::launch_frame_piece(g->d_nl, nl_cap, fs, rec_cap, o->k, scratch, g->d_ridx, g->d_woff,
                                                g->d_text, g->d_off, g->d_len, g->d_packed, g->reads_cap,
                                                g->packed_cap, piece_reads + 2 * c, F);
            SWG_CUDA(cudaGetLastError(), "framing launch");
            SWG_CUDA(cudaEventRecord(packed_ev[c], F), "packed event");
            // the piece's reads to the level-1 partitions (the range the
            // framing left on the device), leaving room for the next piece's
            // framing but for the last piece
            SWG_CUDA(cudaStreamWaitEvent(s, packed_ev[c], 0), "build stream wait");
            BuildArgs ac = a;
            ac.packed = g->d_packed;
            ac.n_words = g->packed_cap;
            ac.read_off = g->d_off;
            ac.read_len = g->d_len;
            ac.n_reads = g->reads_cap;  // bounds only: the piece's reads are in piece_reads
            ac.total_occ = 1;
            ac.read_range = piece_reads + 2 * c;
            SWG_CUDA(cudaMemsetAsync(&g->d_ctl->work[1], 0, sizeof(unsigned long long), s), "clear work");
            g->launches += swg::launch_part_scatter(ac, pl.pa, s,
                                                    c + 1 < C ? swg::kScatterShared : swg::kScatterResident);
            SWG_CUDA(cudaGetLastError(), "scatter launch");
            continue;
        }
        launches += swg::launch_nl_count(g->d_text, end, counts, masks, nul_flag, F, j0);
        launches += swg::launch_gscan(counts, cbase, swg::framing_chunks(end), scratch, tot, F);
        uint64_t h[6] = {0, 0, 0, 0, 0, 0};
        SWG_CUDA(cudaMemcpyAsync(h, tot, sizeof(h), cudaMemcpyDeviceToHost, F), "read newline count");
        SWG_CUDA(cudaStreamSynchronize(F), "framing count");
        if ((unsigned)h[5]) {
            swg::set_error("NUL byte in the FASTA input");
            return SWG_ERR_BAD_INPUT;
        }
        const uint64_t NLc = h[0], Rc = NLc / 2;
        // capacities from the first piece, scaled to the whole text with slack
        // (the device-framed pieces need the whole text's from the start)
        const double scale = (double)n / (double)end, slack = fast ? 1.25 : 1.1;
        const uint64_t nl_want = std::max<uint64_t>(NLc, (uint64_t)(scale * slack * (double)NLc) + 4096);
        if ((st = grow_keep(&g->d_nl, &g->nl_cap, g->nl_cap >= NLc && !fast ? NLc : nl_want, NL,
                            "newline positions")))
            return st;
        const uint64_t r_want = std::max<uint64_t>(Rc, (uint64_t)(scale * slack * (double)Rc) + 4096);
        const uint64_t rw = g->ridx_cap >= Rc && !fast ? Rc : r_want;
        if ((st = grow_keep(&g->d_ridx, &g->ridx_cap, rw, R, "read index")) ||
            (st = grow_keep(&g->d_woff, &g->woff_cap, rw, R, "word offsets")))
            return st;
        launches += swg::launch_nl_pos(masks, end, cbase, g->d_nl, F, j0);
        // this piece's records only: prefixes from 0, the totals so far added when packing
        launches += swg::launch_rec_scan(g->d_nl, R, Rc, o->k, scratch, g->d_ridx, g->d_woff, tot + 1, acc, F);
        SWG_CUDA(cudaGetLastError(), "framing launch");
        SWG_CUDA(cudaMemcpyAsync(h, tot, sizeof(h), cudaMemcpyDeviceToHost, F), "read framing totals");
        SWG_CUDA(cudaStreamSynchronize(F), "framing scan");
        const uint64_t reads_c = reads + h[1], words_c = words + h[2], occ_c = h[3];
        longest = std::max<uint64_t>(longest, h[4]);
        // the reads' arrays grow only with the build stream idle: its
        // scatters of earlier pieces read them
        const uint64_t p_want = std::max<uint64_t>(words_c + 4, (uint64_t)(scale * slack * (double)words_c) + 4096);
        const uint64_t rd_want = std::max<uint64_t>(reads_c, (uint64_t)(scale * slack * (double)reads_c) + 4096);
        const bool grow_packed = g->packed_cap < (fast ? p_want : words_c + 4) || !g->d_packed;
        const bool grow_reads = g->reads_cap < (fast ? rd_want : reads_c) || !g->d_off || !g->d_len;
        if (grow_packed || grow_reads) SWG_CUDA(cudaStreamSynchronize(s), "build stream");
        if (grow_packed) {
            if ((st = grow_keep(&g->d_packed, &g->packed_cap, p_want, words, "packed reads"))) return st;
        }
        if (grow_reads) {
            uint64_t c1 = g->reads_cap, c2 = g->reads_cap;
            if ((st = grow_keep(&g->d_off, &c1, rd_want, reads, "read offsets")) ||
                (st = grow_keep(&g->d_len, &c2, rd_want, reads, "read lengths")))
                return st;
            g->reads_cap = std::min(c1, c2);
        }
        launches += swg::launch_rec_pack(g->d_text, g->d_nl, Rc, o->k, g->d_ridx, g->d_woff, g->d_off,
                                         g->d_len, g->d_packed, F, R, reads, words);
        SWG_CUDA(cudaGetLastError(), "pack launch");
        SWG_CUDA(cudaEventRecord(packed_ev[c], F), "packed event");
        if (stream && o->algorithm == SWG_ALGO_DEFAULT && longest > kBucketedMaxRead) stream = false;
        if (stream && c == 0) {
            // the first piece sizes the build: its occurrences per byte, and its reads as the sample
            const uint64_t N_est = occ_c ? (uint64_t)(scale * (double)occ_c * 1.02) + 65536 : 0;
            if (!N_est || (o->algorithm == SWG_ALGO_DEFAULT && !bucketed_fits(g, N_est))) {
                stream = false;
            } else {
                SWG_CUDA(cudaStreamWaitEvent(s, packed_ev[0], 0), "build stream wait");
                BuildArgs a0 = a;
                a0.packed = g->d_packed;
                a0.n_words = words_c;
                a0.read_off = g->d_off;
                a0.read_len = g->d_len;
                a0.n_reads = reads_c;
                a0.total_occ = occ_c;
                g->algorithm = SWG_ALGO_BUCKETED;
                // every stride-th batch of the first piece: 1/16 to 1/8 of all reads
                const uint32_t stride = (uint32_t)std::max<uint64_t>(1, 16 * first_blocks / nc);
                if ((st = bucketed_plan(g, o, a0, N_est, false, stride, s, pl))) return st;
                SWG_CUDA(cudaEventRecord(g->ev[1], s), "event");
            }
        }
        if (stream && reads_c > reads) {  // this piece's reads to the level-1 partitions
            SWG_CUDA(cudaStreamWaitEvent(s, packed_ev[c], 0), "build stream wait");
            BuildArgs ac = a;
            ac.packed = g->d_packed;
            ac.n_words = words_c;
            ac.read_off = g->d_off + reads;
            ac.read_len = g->d_len + reads;
            ac.n_reads = reads_c - reads;
            ac.total_occ = occ_c - occ;
            SWG_CUDA(cudaMemsetAsync(&g->d_ctl->work[1], 0, sizeof(unsigned long long), s), "clear work");
            // all but the last piece leave room for the framing of the next
            // one (its kernels would otherwise wait for this scatter to end)
            g->launches += swg::launch_part_scatter(ac, pl.pa, s,
                                                    c + 1 < C ? swg::kScatterShared : swg::kScatterPerBatch);
            SWG_CUDA(cudaGetLastError(), "scatter launch");
        }
        NL = NLc;
        R = Rc;
        reads = reads_c;
        words = words_c;
        occ = occ_c;
        fast = fast && stream;
        if (fast && c == 0) {  // the device-framed pieces go on from this piece's totals
            nl_cap = g->nl_cap;
            rec_cap = std::min(g->ridx_cap, g->woff_cap);
            const uint64_t from[4] = {Rc, reads_c, words_c, 0};  // records, reads, words, overflow
            SWG_CUDA(cudaMemcpyAsync(&fs->records, from, sizeof(from), cudaMemcpyHostToDevice, F), "framing state");
        }
    }
    if (fast) {  // the device-framed pieces' totals
        uint64_t hs[12];
        SWG_CUDA(cudaMemcpyAsync(hs, tot, sizeof(hs), cudaMemcpyDeviceToHost, F), "read framing state");
        SWG_CUDA(cudaStreamSynchronize(F), "framing");
        if ((unsigned)hs[5]) {
            swg::set_error("NUL byte in the FASTA input");
            return SWG_ERR_BAD_INPUT;
        }
        if (hs[9]) {  // the text outgrew the capacities from the first piece
            SWG_CUDA(cudaStreamSynchronize(s), "build stream");
            return build_fasta_streamed(g, o, first, n, s, true);
        }
        NL = hs[0];
        occ = hs[3];
        longest = std::max<uint64_t>(longest, hs[4]);
        reads = hs[7];
        words = hs[8];
        if (o->algorithm == SWG_ALGO_DEFAULT && longest > kBucketedMaxRead) stream = false;
    }
    // the build stream goes on after all framing
    SWG_CUDA(cudaStreamWaitEvent(s, packed_ev[C - 1], 0), "build stream wait");
    if (NL & 1) {
        swg::set_error("the last record has a header line but no sequence line");
        return SWG_ERR_BAD_INPUT;
    }
    if (stream && o->algorithm == SWG_ALGO_DEFAULT && !bucketed_fits(g, occ)) stream = false;
    if (!stream) {  // the one-shot build over the reads framed here
        st = build_impl(g, o, g->d_packed, words, g->d_off, g->d_len, reads);
        if (st == SWG_OK) g->launches += launches;
        return st;
    }
    SWG_CUDA(cudaEventRecord(g->ev[2], s), "event");
    a.packed = g->d_packed;
    a.n_words = words;
    a.read_off = g->d_off;
    a.read_len = g->d_len;
    a.n_reads = reads;
    a.total_occ = occ;
    g->occurrences = occ;
    pl.bk.n_rec = occ;
    g->launches += launches;
    return bucketed_finish(g, o, a, s, load, false, pl);
}

swg_status fetch_sorted(const swg_graph *g, std::vector<uint64_t> &keys,
                        std::vector<uint64_t> &mult) {
    if (!g || !g->built || g->n_samples) {
        swg::set_error(g && g->n_samples ? "batched build: use the swg_batch_* calls"
                                         : "graph has not been built");
        return SWG_ERR_BAD_STATE;
    }
    keys.resize(g->n_out);
    mult.resize(g->n_out);
    if (g->n_out) {
        SWG_CUDA(cudaSetDevice(g->device), "cudaSetDevice");
        SWG_CUDA(cudaMemcpy(keys.data(), g->d_out_keys, g->n_out * 8, cudaMemcpyDeviceToHost),
                 "copy keys");
        SWG_CUDA(cudaMemcpy(mult.data(), g->d_out_mult, g->n_out * 8, cudaMemcpyDeviceToHost),
                 "copy multiplicities");
    }
    swg::sort_records(keys.data(), mult.data(), g->n_out);
    return SWG_OK;
}

}  // namespace

extern "C" {

const char *swg_status_string(swg_status s) {
    switch (s) {
        case SWG_OK: return "ok";
        case SWG_ERR_BAD_INPUT: return "bad input";
        case SWG_ERR_TABLE_FULL: return "hash table full";
        case SWG_ERR_OOM: return "out of memory";
        case SWG_ERR_ADMISSION: return "admission denied";
        case SWG_ERR_TIMEOUT: return "device retry limit";
        case SWG_ERR_CUDA: return "CUDA error";
        case SWG_ERR_NO_DEVICE: return "no CUDA device";
        case SWG_ERR_BAD_STATE: return "bad state";
        case SWG_ERR_IO: return "I/O error";
        case SWG_ERR_NOT_READY: return "not ready";
    }
    return "unknown status";
}

const char *swg_last_error(void) { return swg::g_last_error.c_str(); }

const char *swg_version(void) { return "swapgb 0.1 (sm_103a)"; }

swg_status swg_graph_create(swg_graph **out) {
    if (!out) return SWG_ERR_BAD_INPUT;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        swg::set_error("no CUDA device visible");
        return SWG_ERR_NO_DEVICE;
    }
    swg_graph *g = new (std::nothrow) swg_graph;
    if (!g) return SWG_ERR_OOM;
    cudaError_t e = cudaGetDevice(&g->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&g->own, cudaStreamNonBlocking);
    for (int i = 0; e == cudaSuccess && i < 7; i++) e = cudaEventCreate(&g->ev[i]);
    if (e == cudaSuccess) e = cudaMalloc(&g->d_hll, sizeof(unsigned) << swg::kHllBits);
    if (e == cudaSuccess) e = cudaMalloc(&g->d_ctl, sizeof(Control));
    if (e == cudaSuccess) e = cudaMallocHost(&g->h_ctl, sizeof(Control));
    if (e == cudaSuccess) e = cudaMallocHost(&g->h_hll, sizeof(unsigned) << swg::kHllBits);
    if (e == cudaSuccess)
        e = cudaMallocHost(&g->h_part, sizeof(unsigned long long) * ((1u << swg::kPartBitsMax) + 1));
    if (e != cudaSuccess) {
        swg_status st = cuda_fail(e, "graph create");
        swg_graph_free(g);
        return st;
    }
    *out = g;
    return SWG_OK;
}

void swg_graph_free(swg_graph *g) {
    if (!g) return;
    cudaSetDevice(g->device);
    if (g->own) cudaStreamSynchronize(g->own);
    cudaFree(g->d_packed);
    cudaFree(g->d_off);
    cudaFree(g->d_len);
    cudaFree(g->d_prefix);
    cudaFree(g->d_scan);
    cudaFree(g->d_tiles);
    cudaFree(g->d_table);
    cudaFree(g->d_out_keys);
    cudaFree(g->d_out_mult);
    cudaFree(g->d_hll);
    cudaFree(g->d_ctl);
    cudaFree(g->d_part);
    cudaFree(g->d_minhash);
    cudaFree(g->d_text);
    cudaFree(g->d_rec2);
    cudaFree(g->d_bk);
    cudaFree(g->d_arena);
    cudaFree(g->d_fw);
    cudaFree(g->d_segs);
    cudaFree(g->d_read_seg);
    cudaFree(g->d_seg_counts);
    cudaFree(g->d_seg_status);
    cudaFree(g->d_seg_meta);
    cudaFree(g->d_est);
    cudaFree(g->d_out2_keys);
    cudaFree(g->d_out2_mult);
    cudaFree(g->d_seg_cursor);
    cudaFree(g->d_bigmeta);
    swg::merged_free(&g->mg);
    cudaFree(g->d_hll_seg);
    cudaFree(g->d_bucket);
    cudaFree(g->d_poff);
    cudaFree(g->d_plen);
    cudaFree(g->d_records);
    cudaFree(g->d_slices);
    cudaFree(g->d_sfw);
    cudaFree(g->d_nl);
    cudaFree(g->d_ridx);
    cudaFree(g->d_woff);
    if (g->h_file) cudaFreeHost(g->h_file);
    if (g->copy) cudaStreamSynchronize(g->copy);
    if (g->frame) cudaStreamSynchronize(g->frame);
    for (auto &e : g->piece_ev)
        if (e) cudaEventDestroy(e);
    if (g->copy) cudaStreamDestroy(g->copy);
    if (g->frame) cudaStreamDestroy(g->frame);
    if (g->h_part) cudaFreeHost(g->h_part);
    if (g->h_ctl) cudaFreeHost(g->h_ctl);
    if (g->h_hll) cudaFreeHost(g->h_hll);
    for (auto &e : g->ev)
        if (e) cudaEventDestroy(e);
    if (g->own) cudaStreamDestroy(g->own);
    delete g;
}

swg_status swg_graph_build_device(swg_graph *g, const swg_opts *o, const uint32_t *d_packed,
                                  uint64_t n_words, const uint64_t *d_read_off,
                                  const uint32_t *d_read_len, uint64_t n_reads) {
    if (!g) return SWG_ERR_BAD_INPUT;
    return build_impl(g, o, d_packed, n_words, d_read_off, d_read_len, n_reads);
}

swg_status swg_graph_build(swg_graph *g, const swg_opts *o, const uint32_t *packed,
                           uint64_t n_words, const uint64_t *read_off, const uint32_t *read_len,
                           uint64_t n_reads) {
    if (!g) return SWG_ERR_BAD_INPUT;
    swg_status st = check_opts(o);
    if (st) return st;
    if (n_reads && (!packed || !read_off || !read_len)) {
        swg::set_error("NULL read buffer");
        return SWG_ERR_BAD_INPUT;
    }
    SWG_CUDA(cudaSetDevice(g->device), "cudaSetDevice");
    cudaStream_t s = stream_of(g, o);
    if ((st = ensure(&g->d_packed, &g->packed_cap, n_words, "packed reads"))) return st;
    if ((st = ensure_reads(g, n_reads))) return st;
    if (n_words)
        SWG_CUDA(cudaMemcpyAsync(g->d_packed, packed, n_words * 4, cudaMemcpyHostToDevice, s),
                 "copy packed reads");
    if (n_reads) {
        SWG_CUDA(cudaMemcpyAsync(g->d_off, read_off, n_reads * 8, cudaMemcpyHostToDevice, s),
                 "copy read offsets");
        SWG_CUDA(cudaMemcpyAsync(g->d_len, read_len, n_reads * 4, cudaMemcpyHostToDevice, s),
                 "copy read lengths");
    }
    return build_impl(g, o, g->d_packed, n_words, g->d_off, g->d_len, n_reads);
}

swg_status swg_graph_build_fasta(swg_graph *g, const swg_opts *o, const char *text, uint64_t len) {
    Phase phase("constructKmerGraph framing + build");
    if (!g) return SWG_ERR_BAD_INPUT;
    swg_status st = check_opts(o);
    if (st) return st;
    if (!text || len == 0) {
        swg::set_error("empty FASTA input");
        return SWG_ERR_BAD_INPUT;
    }
    const char *first = (const char *)std::memchr(text, '>', len);
    if (!first) {
        swg::set_error("no '>' record start in the input");
        return SWG_ERR_BAD_INPUT;
    }
    if (text[len - 1] != '\n') {
        swg::set_error("the last record is not terminated by a newline");
        return SWG_ERR_BAD_INPUT;
    }
    const uint64_t n = len - (uint64_t)(first - text);
    SWG_CUDA(cudaSetDevice(g->device), "cudaSetDevice");
    cudaStream_t s = stream_of(g, o);
    if (n >= kStreamMin && !std::getenv("SWG_NO_STREAM")) return build_fasta_streamed(g, o, first, n, s);
    // +64: the packing kernel's aligned 16-byte loads read up to 31 bytes past a record
    if ((st = ensure(&g->d_text, &g->text_cap, n + 64, "FASTA text"))) return st;
    SWG_CUDA(cudaMemcpyAsync(g->d_text, first, n, cudaMemcpyHostToDevice, s), "copy FASTA text");
    const uint64_t nc = swg::framing_chunks(n);
    // workspace: counts [nc] | scratch [S] | total [2] | newline masks [MW] |
    // newline positions [nl] | per record: read index, first word
    const uint64_t S = std::max(swg::gscan_scratch(nc), swg::rec_scan_scratch(n / 2 + 1));
    const uint64_t MW = swg::newline_mask_words(n);
    uint64_t want = nc + S + 2 + MW;
    if ((st = ensure(&g->d_fw, &g->fw_cap, want, "framing workspace"))) return st;
    uint64_t *counts = g->d_fw, *scratch = counts + nc, *tot = scratch + S;
    SWG_CUDA(cudaMemsetAsync(g->d_ctl, 0, sizeof(unsigned), s), "clear flag");
    int launches = swg::launch_nl_count(g->d_text, n, counts, tot + 2, &g->d_ctl->status, s);
    launches += swg::launch_gscan(counts, counts, nc, scratch, tot, s);
    uint64_t h[2] = {0, 0};
    unsigned nul = 0;
    SWG_CUDA(cudaMemcpyAsync(h, tot, 8, cudaMemcpyDeviceToHost, s), "read newline count");
    SWG_CUDA(cudaMemcpyAsync(&nul, &g->d_ctl->status, 4, cudaMemcpyDeviceToHost, s), "read flag");
    SWG_CUDA(cudaStreamSynchronize(s), "framing count");
    if (nul) {
        swg::set_error("NUL byte in the FASTA input");
        return SWG_ERR_BAD_INPUT;
    }
    const uint64_t NL = h[0];
    if (NL & 1) {
        swg::set_error("the last record has a header line but no sequence line");
        return SWG_ERR_BAD_INPUT;
    }
    const uint64_t R = NL / 2;
    want = nc + S + 2 + MW + NL + 2 * std::max<uint64_t>(R, 1);
    if (want > g->fw_cap) {  // grow, keeping the chunk bases and the newline masks computed above
        uint64_t *nw = nullptr;
        SWG_CUDA(cudaMalloc(&nw, want * 8), "framing workspace");
        SWG_CUDA(cudaMemcpyAsync(nw, g->d_fw, (nc + S + 2 + MW) * 8, cudaMemcpyDeviceToDevice, s),
                 "copy framing workspace");
        SWG_CUDA(cudaStreamSynchronize(s), "framing workspace");
        cudaFree(g->d_fw);
        g->d_fw = nw;
        g->fw_cap = want;
        counts = g->d_fw;
        scratch = counts + nc;
        tot = scratch + S;
    }
    uint64_t *masks = tot + 2, *nl = masks + MW, *idx = nl + NL, *words = idx + R;
    launches += swg::launch_nl_pos(masks, n, counts, nl, s);
    launches += swg::launch_rec_scan(nl, 0, R, o->k, scratch, idx, words, tot, nullptr, s);
    SWG_CUDA(cudaGetLastError(), "framing launch");
    SWG_CUDA(cudaMemcpyAsync(h, tot, 16, cudaMemcpyDeviceToHost, s), "read framing totals");
    SWG_CUDA(cudaStreamSynchronize(s), "framing scan");
    const uint64_t n_reads = h[0], n_words = h[1];
    if ((st = ensure(&g->d_packed, &g->packed_cap, n_words + 4, "packed reads"))) return st;
    if ((st = ensure_reads(g, n_reads))) return st;
    launches += swg::launch_rec_pack(g->d_text, nl, R, o->k, idx, words, g->d_off, g->d_len,
                                     g->d_packed, s);
    SWG_CUDA(cudaGetLastError(), "pack launch");
    st = build_impl(g, o, g->d_packed, n_words, g->d_off, g->d_len, n_reads);
    if (st == SWG_OK) g->launches += launches;
    return st;
}

swg_status swg_graph_build_fasta_to_host(swg_graph *g, const swg_opts *o, const char *text, uint64_t len,
                                         uint64_t *keys, uint8_t *mult, uint64_t cap, uint64_t *n_out) {
    if (!g || !n_out || (cap && (!keys || !mult))) return SWG_ERR_BAD_INPUT;
    *n_out = 0;
    SWG_CUDA(cudaSetDevice(g->device), "cudaSetDevice");
    // the arrays as the device sees them (pinned host memory); otherwise the
    // graph is copied out after the build
    void *dk = nullptr, *dm = nullptr;
    const bool mapped = cap && cudaHostGetDevicePointer(&dk, keys, 0) == cudaSuccess &&
                        cudaHostGetDevicePointer(&dm, mult, 0) == cudaSuccess;
    if (!mapped) cudaGetLastError();
    g->host_keys = mapped ? static_cast<unsigned long long *>(dk) : nullptr;
    g->host_mult = mapped ? static_cast<unsigned long long *>(dm) : nullptr;
    g->host_cap = mapped ? cap : 0;
    g->host_out_used = false;
    swg_status st = swg_graph_build_fasta(g, o, text, len);
    const bool wrote = g->host_out_used;
    g->host_keys = g->host_mult = nullptr;
    g->host_cap = 0;
    g->host_out_used = false;
    if (st) return st;
    *n_out = g->n_out;
    if (g->n_out > cap) {
        swg::set_error("output arrays too small: n_out holds the survivor count needed");
        return SWG_ERR_BAD_INPUT;
    }
    if (!wrote) return swg_graph_copy_out(g, keys, mult, cap, 0, n_out);
    if (g->h_ctl->host_written != g->n_out) {
        swg::set_error("survivors written to the host arrays disagree with the graph (internal error)");
        return SWG_ERR_CUDA;
    }
    return SWG_OK;
}

swg_status swg_graph_build_fasta_file(swg_graph *g, const swg_opts *o, const char *path) {
    if (!g || !path) return SWG_ERR_BAD_INPUT;
    swg_status st = check_opts(o);
    if (st) return st;
    const int fd = ::open(path, O_RDONLY);
    if (fd < 0) {
        swg::set_error(std::string("cannot open ") + path);
        return SWG_ERR_IO;
    }
    struct stat sb;
    if (::fstat(fd, &sb) != 0 || sb.st_size <= 0) {
        ::close(fd);
        swg::set_error(std::string(sb.st_size == 0 ? "empty FASTA input: " : "cannot stat ") + path);
        return sb.st_size == 0 ? SWG_ERR_BAD_INPUT : SWG_ERR_IO;
    }
    const uint64_t len = (uint64_t)sb.st_size;
    SWG_CUDA(cudaSetDevice(g->device), "cudaSetDevice");
    if (g->h_file_cap < len) {
        if (g->h_file) cudaFreeHost(g->h_file);
        g->h_file = nullptr;
        g->h_file_cap = 0;
        cudaError_t e = cudaHostAlloc((void **)&g->h_file, len, cudaHostAllocDefault);
        if (e != cudaSuccess) {
            ::close(fd);
            g->h_file = nullptr;
            return cuda_fail(e, "pinned buffer for the FASTA file");
        }
        g->h_file_cap = len;
    }
    // read in parallel slices of at least 16 MiB
    const uint64_t slice = 16ull << 20;
    const unsigned nt = (unsigned)std::min<uint64_t>(8, (len + slice - 1) / slice);
    std::vector<int> ok(nt, 1);
    {
        std::vector<std::thread> th;
        for (unsigned t = 0; t < nt; t++)
            th.emplace_back([&, t] {
                uint64_t a = len * t / nt;
                const uint64_t b = len * (t + 1) / nt;
                while (a < b) {
                    const ssize_t r = ::pread(fd, g->h_file + a, (size_t)std::min<uint64_t>(b - a, 1ull << 30), (off_t)a);
                    if (r <= 0) {
                        ok[t] = 0;
                        return;
                    }
                    a += (uint64_t)r;
                }
            });
        for (auto &x : th) x.join();
    }
    ::close(fd);
    for (unsigned t = 0; t < nt; t++)
        if (!ok[t]) {
            swg::set_error(std::string("short read from ") + path);
            return SWG_ERR_IO;
        }
    return swg_graph_build_fasta(g, o, g->h_file, len);
}

swg_status swg_build(const swg_opts *o, const uint32_t *packed, uint64_t n_words,
                     const uint64_t *read_off, const uint32_t *read_len, uint64_t n_reads,
                     swg_graph **out) {
    if (!out) return SWG_ERR_BAD_INPUT;
    *out = nullptr;
    swg_graph *g = nullptr;
    swg_status st = swg_graph_create(&g);
    if (st) return st;
    st = swg_graph_build(g, o, packed, n_words, read_off, read_len, n_reads);
    if (st) {
        swg_graph_free(g);
        return st;
    }
    *out = g;
    return SWG_OK;
}

swg_status swg_build_fasta(const swg_opts *o, const char *text, uint64_t len, swg_graph **out) {
    if (!out) return SWG_ERR_BAD_INPUT;
    *out = nullptr;
    swg_status st = check_opts(o);
    if (st) return st;
    swg_graph *g = nullptr;
    if ((st = swg_graph_create(&g))) return st;
    if ((st = swg_graph_build_fasta(g, o, text, len))) {
        swg_graph_free(g);
        return st;
    }
    *out = g;
    return SWG_OK;
}

swg_status swg_graph_size(const swg_graph *g, uint64_t *n) {
    if (!g || !n) return SWG_ERR_BAD_INPUT;
    if (!g->built || g->n_samples) return SWG_ERR_BAD_STATE;
    *n = g->n_out;
    return SWG_OK;
}

swg_status swg_graph_distinct(const swg_graph *g, uint64_t *n) {
    if (!g || !n) return SWG_ERR_BAD_INPUT;
    if (!g->built || g->n_samples) return SWG_ERR_BAD_STATE;
    *n = g->n_distinct;
    return SWG_OK;
}

swg_status swg_graph_device_view(const swg_graph *g, const uint64_t **d_keys,
                                 const uint64_t **d_mult, uint64_t *n) {
    if (!g) return SWG_ERR_BAD_INPUT;
    if (!g->built || g->n_samples) return SWG_ERR_BAD_STATE;
    if (d_keys) *d_keys = reinterpret_cast<const uint64_t *>(g->d_out_keys);
    if (d_mult) *d_mult = reinterpret_cast<const uint64_t *>(g->d_out_mult);
    if (n) *n = g->n_out;
    return SWG_OK;
}

swg_status swg_graph_copy_out(const swg_graph *g, uint64_t *keys, uint8_t *mult, uint64_t cap,
                              int sorted, uint64_t *n) {
    if (!g) return SWG_ERR_BAD_INPUT;
    if (!g->built || g->n_samples) return SWG_ERR_BAD_STATE;
    if (n) *n = g->n_out;
    if (cap < g->n_out) {
        swg::set_error("output capacity smaller than the survivor count");
        return SWG_ERR_BAD_INPUT;
    }
    if (g->n_out == 0) return SWG_OK;
    if (!sorted) {
        SWG_CUDA(cudaSetDevice(g->device), "cudaSetDevice");
        if (keys)
            SWG_CUDA(cudaMemcpy(keys, g->d_out_keys, g->n_out * 8, cudaMemcpyDeviceToHost),
                     "copy keys");
        if (mult)
            SWG_CUDA(cudaMemcpy(mult, g->d_out_mult, g->n_out * 8, cudaMemcpyDeviceToHost),
                     "copy multiplicities");
        return SWG_OK;
    }
    std::vector<uint64_t> k, m;
    swg_status st = fetch_sorted(g, k, m);
    if (st) return st;
    if (keys) std::memcpy(keys, k.data(), g->n_out * 8);
    if (mult) std::memcpy(mult, m.data(), g->n_out * 8);
    return SWG_OK;
}

swg_status swg_graph_stats(const swg_graph *g, int64_t out[5]) {
    if (!g || !out) return SWG_ERR_BAD_INPUT;
    std::vector<uint64_t> k, m;
    swg_status st = fetch_sorted(g, k, m);
    if (st) return st;
    swg::graph_stats(reinterpret_cast<const uint8_t *>(m.data()), g->n_out, g->k, out);
    return SWG_OK;
}

// Both text outputs are formatted on the device (emit.cu) from the
// device-resident records and streamed to the file.
static swg_status writable(const swg_graph *g) {
    if (!g->built || g->n_samples) {
        swg::set_error(g->n_samples ? "batched build: use the swg_batch_* calls" : "graph has not been built");
        return SWG_ERR_BAD_STATE;
    }
    return SWG_OK;
}

swg_status swg_graph_write_kmer_graph(const swg_graph *g, const char *path) {
    Phase phase("printKmerGraph");
    if (!g || !path) return SWG_ERR_BAD_INPUT;
    swg_status st = writable(g);
    if (st) return st;
    SWG_CUDA(cudaSetDevice(g->device), "cudaSetDevice");
    return swg::emit_kmer_graph(g->d_out_keys, g->d_out_mult, g->n_out, g->k, path, g->own);
}

swg_status swg_graph_write_node_lines(const swg_graph *g, const char *path) {
    Phase phase("printLocalNodeGraph");
    if (!g || !path) return SWG_ERR_BAD_INPUT;
    swg_status st = writable(g);
    if (st) return st;
    SWG_CUDA(cudaSetDevice(g->device), "cudaSetDevice");
    return swg::emit_node_lines(g->d_out_keys, g->d_out_mult, g->n_out, g->k, path, g->own);
}

// Merging of semi-extended k-molecules (merge.cu) over the built graph; the
// result is the -d file's text, kept on the device until the next build.
static swg_status merge_impl(swg_graph *g, const uint64_t *order, uint64_t n_order);

swg_status swg_graph_merge(swg_graph *g) { return merge_impl(g, nullptr, 0); }

swg_status swg_graph_merge_in_order(swg_graph *g, const uint64_t *order_keys, uint64_t n_order) {
    if (!order_keys && n_order) return SWG_ERR_BAD_INPUT;
    static const uint64_t none = 0;
    return merge_impl(g, order_keys ? order_keys : &none, n_order);
}

static swg_status merge_impl(swg_graph *g, const uint64_t *order, uint64_t n_order) {
    Phase phase("simplifyDistNodeGraph");
    if (!g) return SWG_ERR_BAD_INPUT;
    swg_status st = writable(g);
    if (st) return st;
    SWG_CUDA(cudaSetDevice(g->device), "cudaSetDevice");
    g->merged = false;
    if (!g->mg.pool) {  // the handle's own pool: merge scratch stays mapped between calls
        cudaMemPoolProps props;
        std::memset(&props, 0, sizeof(props));
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = g->device;
        SWG_CUDA(cudaMemPoolCreate(&g->mg.pool, &props), "merge memory pool");
        uint64_t keep = ~0ull;
        SWG_CUDA(cudaMemPoolSetAttribute(g->mg.pool, cudaMemPoolAttrReleaseThreshold, &keep), "merge memory pool");
    }
    cudaEvent_t e0 = g->ev[0], e1 = g->ev[1];
    SWG_CUDA(cudaEventRecord(e0, g->own), "merge timing");
    st = swg::merge_graph(g->d_out_keys, g->d_out_mult, g->n_out, g->k, g->own, &g->mg, &g->mres,
                          reinterpret_cast<const unsigned long long *>(order), n_order);
    if (st) return st;
    SWG_CUDA(cudaEventRecord(e1, g->own), "merge timing");
    SWG_CUDA(cudaEventSynchronize(e1), "merge timing");
    SWG_CUDA(cudaEventElapsedTime(&g->merge_ms, e0, e1), "merge timing");
    g->merged = true;
    return SWG_OK;
}

static swg_status merged_state(const swg_graph *g) {
    if (!g->merged) {
        swg::set_error("no merged graph: call swg_graph_merge after the build");
        return SWG_ERR_BAD_STATE;
    }
    return SWG_OK;
}

swg_status swg_graph_merge_info(const swg_graph *g, swg_merge_info *info) {
    if (!g || !info) return SWG_ERR_BAD_INPUT;
    swg_status st = merged_state(g);
    if (st) return st;
    info->nodes = g->mg.nodes;
    info->chains = g->mres.chains;
    info->cycles = g->mres.cycles;
    info->text_bytes = g->mg.text_bytes;
    info->ms = g->merge_ms;
    info->launches = g->mres.launches;
    return SWG_OK;
}

swg_status swg_graph_copy_merged(const swg_graph *g, char *buf, uint64_t cap, uint64_t *n) {
    if (!g || !n) return SWG_ERR_BAD_INPUT;
    swg_status st = merged_state(g);
    if (st) return st;
    *n = g->mg.text_bytes;
    if (cap < *n || (*n && !buf)) {
        swg::set_error("buffer smaller than the merged text");
        return SWG_ERR_BAD_INPUT;
    }
    SWG_CUDA(cudaSetDevice(g->device), "cudaSetDevice");
    SWG_CUDA(cudaMemcpyAsync(buf, g->mg.text, *n, cudaMemcpyDeviceToHost, g->own), "merged text copy");
    SWG_CUDA(cudaStreamSynchronize(g->own), "merged text copy");
    return SWG_OK;
}

swg_status swg_graph_write_merged(const swg_graph *g, const char *path) {
    if (!g || !path) return SWG_ERR_BAD_INPUT;
    swg_status st = merged_state(g);
    if (st) return st;
    SWG_CUDA(cudaSetDevice(g->device), "cudaSetDevice");
    return swg::stream_to_file(g->mg.text, g->mg.text_bytes, path, g->own);
}

// Rank-0 passes of the reference over the merged graph (prune.cu).
swg_status swg_graph_remove_tips(swg_graph *g, uint64_t *removed) {
    Phase phase("masterTipsRemoval");
    if (!g) return SWG_ERR_BAD_INPUT;
    swg_status st = merged_state(g);
    if (st) return st;
    SWG_CUDA(cudaSetDevice(g->device), "cudaSetDevice");
    uint64_t n = 0;
    st = swg::prune_tips(&g->mg, g->own, &n);
    if (st) g->merged = false;  // lines edited, text not rewritten: drop both
    if (removed) *removed = st ? 0 : n;
    return st;
}

swg_status swg_graph_remove_low_coverage(swg_graph *g, uint64_t *cut) {
    Phase phase("masterLowCoverageEdgeRemoval");
    if (!g) return SWG_ERR_BAD_INPUT;
    swg_status st = merged_state(g);
    if (st) return st;
    SWG_CUDA(cudaSetDevice(g->device), "cudaSetDevice");
    uint64_t n = 0;
    st = swg::prune_low_coverage(&g->mg, g->own, &n);
    if (st) g->merged = false;  // lines edited, text not rewritten: drop both
    if (cut) *cut = st ? 0 : n;
    return st;
}

swg_status swg_graph_simplify(swg_graph *g, uint64_t *merged) {
    Phase phase("masterSimplifyNodeGraph");
    if (!g) return SWG_ERR_BAD_INPUT;
    swg_status st = merged_state(g);
    if (st) return st;
    SWG_CUDA(cudaSetDevice(g->device), "cudaSetDevice");
    uint64_t n = 0;
    st = swg::simplify_lines(&g->mg, g->own, &n);
    if (st) g->merged = false;  // lines edited, text not rewritten: drop both
    if (merged) *merged = st ? 0 : n;
    return st;
}

swg_status swg_graph_write_contigs(swg_graph *g, const char *path, uint64_t *n) {
    Phase phase("printContigs");
    if (!g || !path) return SWG_ERR_BAD_INPUT;
    swg_status st = merged_state(g);
    if (st) return st;
    SWG_CUDA(cudaSetDevice(g->device), "cudaSetDevice");
    uint64_t c = 0;
    st = swg::write_contigs(&g->mg, path, g->own, &c);
    if (n) *n = st ? 0 : c;
    return st;
}

static swg_status sorted_copy(const uint64_t *keys, const uint8_t *mult, uint64_t n,
                              std::vector<uint64_t> &k, std::vector<uint64_t> &m) {
    if (n && (!keys || !mult)) return SWG_ERR_BAD_INPUT;
    k.assign(keys, keys + n);
    m.resize(n);
    if (n) std::memcpy(m.data(), mult, n * 8);
    swg::sort_records(k.data(), m.data(), n);
    return SWG_OK;
}

swg_status swg_records_write_kmer_graph(const uint64_t *keys, const uint8_t *mult, uint64_t n,
                                        int k, const char *path) {
    if (!path) return SWG_ERR_BAD_INPUT;
    std::vector<uint64_t> kk, mm;
    swg_status st = sorted_copy(keys, mult, n, kk, mm);
    if (st) return st;
    return swg::write_kmer_graph(kk.data(), reinterpret_cast<const uint8_t *>(mm.data()), n, k, path);
}

swg_status swg_records_write_node_lines(const uint64_t *keys, const uint8_t *mult, uint64_t n,
                                        const char *path) {
    if (!path) return SWG_ERR_BAD_INPUT;
    std::vector<uint64_t> kk, mm;
    swg_status st = sorted_copy(keys, mult, n, kk, mm);
    if (st) return st;
    return swg::write_node_lines(kk.data(), reinterpret_cast<const uint8_t *>(mm.data()), n, path);
}

swg_status swg_graph_last_timings(const swg_graph *g, float ms[5], int *launches) {
    if (!g) return SWG_ERR_BAD_INPUT;
    if (!g->built) return SWG_ERR_BAD_STATE;
    if (ms) std::memcpy(ms, g->ms, sizeof(g->ms));
    if (launches) *launches = g->launches;
    return SWG_OK;
}

swg_status swg_batch_build(swg_graph *g, const swg_opts *o, const swg_sample *samples,
                           uint32_t n_samples) {
    if (!g) return SWG_ERR_BAD_INPUT;
    return batch_impl(g, o, samples, n_samples);
}

swg_status swg_batch_samples(const swg_graph *g, uint32_t *n_samples) {
    if (!g || !n_samples) return SWG_ERR_BAD_INPUT;
    if (!g->built || !g->n_samples) return SWG_ERR_BAD_STATE;
    *n_samples = g->n_samples;
    return SWG_OK;
}

swg_status swg_batch_sample_info(const swg_graph *g, uint32_t s, uint64_t *occurrences,
                                 uint64_t *distinct, uint64_t *survivors) {
    if (!g) return SWG_ERR_BAD_INPUT;
    if (!g->built || !g->n_samples) return SWG_ERR_BAD_STATE;
    if (s >= g->n_samples) return SWG_ERR_BAD_INPUT;
    if (occurrences) *occurrences = g->s_occ[s];
    if (distinct) *distinct = g->s_distinct[s];
    if (survivors) *survivors = g->s_out[s];
    return SWG_OK;
}

swg_status swg_batch_device_view(const swg_graph *g, uint32_t s, const uint64_t **d_keys,
                                 const uint64_t **d_mult, uint64_t *n) {
    if (!g) return SWG_ERR_BAD_INPUT;
    if (!g->built || !g->n_samples) return SWG_ERR_BAD_STATE;
    if (s >= g->n_samples) return SWG_ERR_BAD_INPUT;
    if (d_keys) *d_keys = reinterpret_cast<const uint64_t *>(g->d_out_keys + g->s_tbase[s]);
    if (d_mult) *d_mult = reinterpret_cast<const uint64_t *>(g->d_out_mult + g->s_tbase[s]);
    if (n) *n = g->s_out[s];
    return SWG_OK;
}

swg_status swg_batch_copy_out(const swg_graph *g, uint32_t s, uint64_t *keys, uint8_t *mult,
                              uint64_t cap, int sorted, uint64_t *n) {
    if (!g) return SWG_ERR_BAD_INPUT;
    if (!g->built || !g->n_samples) return SWG_ERR_BAD_STATE;
    if (s >= g->n_samples) return SWG_ERR_BAD_INPUT;
    const uint64_t cnt = g->s_out[s];
    if (n) *n = cnt;
    if (cap < cnt) {
        swg::set_error("output capacity smaller than the survivor count");
        return SWG_ERR_BAD_INPUT;
    }
    if (!cnt) return SWG_OK;
    std::vector<uint64_t> k(cnt), m(cnt);
    SWG_CUDA(cudaSetDevice(g->device), "cudaSetDevice");
    SWG_CUDA(cudaMemcpy(k.data(), g->d_out_keys + g->s_tbase[s], cnt * 8, cudaMemcpyDeviceToHost),
             "copy keys");
    SWG_CUDA(cudaMemcpy(m.data(), g->d_out_mult + g->s_tbase[s], cnt * 8, cudaMemcpyDeviceToHost),
             "copy multiplicities");
    if (sorted) swg::sort_records(k.data(), m.data(), cnt);
    if (keys) std::memcpy(keys, k.data(), cnt * 8);
    if (mult) std::memcpy(mult, m.data(), cnt * 8);
    return SWG_OK;
}

swg_status swg_graph_build_info(const swg_graph *g, swg_build_info *info) {
    if (!g || !info) return SWG_ERR_BAD_INPUT;
    if (!g->built) return SWG_ERR_BAD_STATE;
    std::memset(info, 0, sizeof(*info));
    info->algorithm = g->algorithm;
    info->launches = g->launches;
    info->occurrences = g->occurrences;
    info->distinct = g->n_distinct;
    info->survivors = g->n_out;
    info->table_entries = g->cap_used;
    const bool parted = g->algorithm == SWG_ALGO_PARTITIONED || g->algorithm == SWG_ALGO_BUCKETED;
    info->partitions = parted ? g->parts : 0;
    info->slots = parted ? g->slots : 0;
    info->waves = parted ? g->waves : 0;
    info->retries = g->retries;
    info->estimate = g->estimate;
    std::memcpy(info->ms, g->ms, sizeof(g->ms));
    info->bucket_table = g->algorithm == SWG_ALGO_BUCKETED ? g->bucket_table : 0;
    return SWG_OK;
}

swg_status swg_probe_random_access(int kind, uint64_t table_bytes, uint64_t n_ops, void *stream,
                                   double *ops_per_s) {
    if (!ops_per_s || kind < 0 || kind > 6 || n_ops == 0 || table_bytes < 4096)
        return SWG_ERR_BAD_INPUT;
    float ms = 0;
    cudaError_t e = swg::run_probe(kind, table_bytes, n_ops, (cudaStream_t)stream, &ms);
    if (e != cudaSuccess) return cuda_fail(e, "random-access probe");
    const double per = kind == 5 ? 4.0 : (kind == 6 ? 2.0 : 1.0);  // accesses per operation
    *ops_per_s = ms > 0 ? per * (double)n_ops / (ms * 1e-3) : 0;
    return SWG_OK;
}

swg_status swg_probe_shared_atomics(int kind, uint64_t n_ops, void *stream, double *ops_per_s) {
    if (!ops_per_s || kind < 0 || kind > 1 || n_ops == 0) return SWG_ERR_BAD_INPUT;
    float ms = 0;
    cudaError_t e = swg::run_smem_probe(kind, n_ops, (cudaStream_t)stream, &ms);
    if (e != cudaSuccess) return cuda_fail(e, "shared-memory atomic probe");
    *ops_per_s = ms > 0 ? (double)n_ops / (ms * 1e-3) : 0;
    return SWG_OK;
}

}  // extern "C"
