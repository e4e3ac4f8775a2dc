// Internal declarations shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "swapgb.h"

namespace swg {

// Hash-table entry: one canonical k-molecule and its 8 saturating uint8 edge
// multiplicities (byte t = slot t, the reference's arc::multiplicity[t],
// graph.cpp:36-40). Key 0 marks an empty entry: a canonical key is
// max(kmer, revcomp(kmer)) and revcomp(0) = 4^k-1 > 0, so 0 is never a key.
struct __align__(16) Entry {
    unsigned long long key;
    unsigned long long cnt;
};

// Device status bits (set by kernels, read by the host after a build).
enum : unsigned {
    kStatusTableFull = 1u,  // probe limit reached or table nearly full
    kStatusCasLimit = 2u,   // a bounded CAS retry loop gave up
    kStatusPartOverflow = 4u,  // a partition or bucket outgrew its region (bucketed build)
};

constexpr int kK1Block = 256;
constexpr int kK1Items = 16;
constexpr uint64_t kTileOcc = (uint64_t)kK1Block * kK1Items;  // occurrences per tile
constexpr int kHllBits = 12;                                  // 4096 registers

// Per-sample parameters of a batched build (samples = segments of one
// build): the sample's table region (its output uses the same offsets), its
// k and its cutoff.
struct SegParams {
    unsigned long long tbase;
    unsigned long long tcap;
    int k;
    int cutoff;
};

// Per-build launch parameters.
struct BuildArgs {
    const uint32_t *packed;
    uint64_t n_words;
    const uint64_t *read_off;
    const uint32_t *read_len;
    uint64_t n_reads;
    int k;
    int cutoff;
    // workspace
    uint64_t *occ_prefix;      // n_reads + 1
    uint64_t *scan_blocks;     // scratch for the scan
    uint32_t *tile_first_read; // n_tiles
    uint64_t n_tiles;
    uint64_t total_occ;
    Entry *table;
    uint64_t cap;
    unsigned *hll;             // 1 << kHllBits registers
    unsigned *status;
    unsigned long long *counters;  // [0] inserted, [1] survivors
    unsigned long long *out_keys;
    unsigned long long *out_mult;
    uint64_t out_cap;
    // batched builds only (all null / 0 for a single sample)
    const uint32_t *read_seg;          // [n_reads] sample of each read
    const SegParams *segs;             // [n_segs]
    uint32_t n_segs;
    unsigned long long *seg_counts;    // [2 * n_segs]: inserted, survivors
    unsigned *seg_status;              // [n_segs]
    int tag_bits;                      // bucketed batch: the read's sample index sits in the
                                       // top tag_bits bits of every key (0 = no tag)
    unsigned *max_len;                 // if set, the occurrence scan records the longest read
    // level-1 scatter of a streamed piece: if set, the reads read_range[0] <=
    // r < read_range[1] (device values; n_reads and total_occ are then only
    // bounds for the launch)
    const unsigned long long *read_range;
    // bucketed single-sample build only: survivors also written, as each bucket
    // is compacted, to host memory the device can reach (unordered, at most
    // host_cap; host_written counts them), so the copy-out overlaps the count
    unsigned long long *host_keys;
    unsigned long long *host_mult;
    uint64_t host_cap;
    unsigned long long *host_written;
};

constexpr uint32_t kMaxTagSamples = 1024;  // samples of one tagged bucketed batch

// Partitioned build: records {hash low bits, arc code} scattered by the top
// bits of mix64(key) into n_parts partitions, each counted in a table slice
// small enough to stay in L2, a wave of n_slots partitions at a time.
constexpr int kPartBitsMin = 8;
constexpr int kPartBitsMax = 10;

struct PartArgs {
    int bits;                          // log2(n_parts)
    uint32_t n_parts;
    unsigned long long *part_count;    // [n_parts] records per partition
    unsigned long long *part_start;    // [n_parts + 1] exclusive prefix
    unsigned long long *part_cursor;   // [n_parts] scatter cursors
    unsigned long long *records;       // [total_occ]
    Entry *slices;                     // [n_slots * slot_cap]
    uint64_t slot_cap;
    uint32_t n_slots;
    int load_num, load_den;            // slice capacity = count * den / num + 16
    unsigned long long *work;          // bucketed: [2] read-batch counters (count, scatter), zeroed
    int shape;                         // scatter block shape (swg_opts::scatter_shape; 0 = default)
};

// Bucketed build: the level-1 partition records are split again by the next
// b2 bits of the hash into sub-buckets small enough for a shared-memory table.
struct BucketArgs {
    int b1, b2;                            // partition bits, sub-bucket bits
    uint32_t n_parts;                      // 1 << b1
    const unsigned long long *part_start;  // [n_parts + 1] level-1 offsets
    const unsigned long long *part_cursor; // [n_parts] level-1 cursors after the scatter
    unsigned long long *part_end;          // [n_parts] end of each partition's records
    unsigned *status;
    const unsigned long long *rec1;        // level-1 records
    unsigned long long *rec2;              // records grouped by bucket
    unsigned long long *off2;              // [n_buckets + 1] bucket regions (region j = [off2[j], off2[j+1]))
    unsigned long long *cursor2;           // [n_buckets] scatter cursors
    unsigned long long *chunk_start;       // [n_parts + 1] level-2 chunks per partition, prefix
    unsigned long long *surv;              // [n_buckets] survivors per bucket
    unsigned long long *surv_off;          // [n_buckets + 1] their exclusive prefix
    unsigned long long *stage_keys;        // [n_rec] survivor keys, staged at the bucket's offset
    uint64_t n_rec;
    unsigned long long *big;               // buckets too large for a tier-1 table
    unsigned *big_count;
    unsigned long long *big2;              // ... and for a tier-2 table
    unsigned *big2_count;
    uint32_t big_cap;                      // capacity of each list
    int shape;                             // scatter block shape (swg_opts::scatter_shape; 0 = default)
};

// Kernel launchers (kernels.cu). Each returns the number of launches made.
// The occurrence total (into occ_prefix[n_reads]) and, with write, the
// per-read prefix; launch_occ_scan_write adds the prefix to a scan made
// without it.
int launch_occ_scan(const BuildArgs &a, cudaStream_t s, bool write = true);
int launch_occ_scan_write(const BuildArgs &a, cudaStream_t s);
// The level-1 scatter's block shape for swg_opts::scatter_shape (0: the
// SWG_SCATTER_SHAPE default).
int level1_shape(int opt_shape);
uint64_t scan_block_count(uint64_t n_reads);
int launch_tiles(const BuildArgs &a, cudaStream_t s);
int launch_hll(const BuildArgs &a, cudaStream_t s);
double hll_estimate(const unsigned *regs_host);
int launch_sketch(const BuildArgs &a, unsigned *minhash, cudaStream_t s);
uint64_t bucket_count();
int launch_read_order(const BuildArgs &a, const unsigned *minhash, unsigned *hist,
                      uint64_t *out_off, uint32_t *out_len, cudaStream_t s);
int launch_count(const BuildArgs &a, cudaStream_t s);
int launch_seg_setup(const BuildArgs &a, const uint64_t *seg_read_start,
                     const uint64_t *seg_base_shift, uint32_t *read_seg, uint64_t *read_off,
                     cudaStream_t s);
int launch_hll_estimates(const unsigned *regs, uint32_t n_segs, double *est, cudaStream_t s);
int launch_gather_prefix(const uint64_t *prefix, const uint64_t *idx, uint32_t n, uint64_t *out,
                         cudaStream_t s);
int launch_compact(const BuildArgs &a, cudaStream_t s);
int launch_part_count(const BuildArgs &a, const PartArgs &p, cudaStream_t s);
int launch_part_prefix(const PartArgs &p, cudaStream_t s);
int launch_p1_sample(const BuildArgs &a, const PartArgs &p, const BucketArgs &b, uint32_t stride,
                     cudaStream_t s);
int launch_part_caps(const PartArgs &p, uint64_t n_rec, unsigned long long *sampled, cudaStream_t s);
int launch_bucket_caps(const unsigned long long *counts, const unsigned long long *sampled, uint64_t n_rec,
                       uint64_t nb, unsigned long long *caps, cudaStream_t s);
int launch_big_multi(const BuildArgs &a, const BucketArgs &b, const unsigned long long *meta, uint32_t n,
                     uint64_t records, Entry *table, uint64_t cap, cudaStream_t s);
// persistent: at most the resident blocks, each taking read batches until
// none is left; else one block per batch (blocks retire as they finish, so
// other streams' kernels get SMs during the scatter)
// Grid of the level-1 scatter: one block per batch of reads (blocks retire
// as they finish), as many blocks as stay resident (each takes batches until
// none are left), or one block per SM fewer than that, leaving room on every
// SM for the kernels of a concurrent stream (the streamed build's framing;
// with 256 partitions this mode takes a block shape of at most 64 registers).
enum { kScatterPerBatch = 0, kScatterResident = 1, kScatterShared = 2 };
int launch_part_scatter(const BuildArgs &a, const PartArgs &p, cudaStream_t s, int grid_mode = kScatterResident);
int launch_part_wave(const BuildArgs &a, const PartArgs &p, uint32_t p0, uint32_t n,
                     uint64_t rec_begin, uint64_t rec_end, cudaStream_t s);
// Device FASTA framing (framing.cu).
uint64_t framing_chunks(uint64_t n);
uint64_t gscan_scratch(uint64_t n);
int launch_gscan(const uint64_t *in, uint64_t *out, uint64_t n, uint64_t *scratch, uint64_t *total,
                 cudaStream_t s);
// The text's 16 KiB chunks from j0 up to the end n; records from r0 up to
// n_rec (a streamed build frames the text a piece at a time); a record's
// read index and first word are read_base + read_idx[r], word_base +
// word_off[r].
// The newline count leaves a bit mask of the newlines (newline_mask_words(n)
// words for a text of n bytes) that the newline positions are read from.
uint64_t newline_mask_words(uint64_t n);
int launch_nl_count(const unsigned char *t, uint64_t n, uint64_t *counts, uint64_t *masks, unsigned *flag,
                    cudaStream_t s, uint64_t j0 = 0);
int launch_nl_pos(const uint64_t *masks, uint64_t n, const uint64_t *chunk_base, uint64_t *nl,
                  cudaStream_t s, uint64_t j0 = 0, uint64_t cap = ~0ull, uint64_t *ovf = nullptr);
// Device state of a streamed framing, in the order the framing kernels write
// it (the chunk-count scan's total, the record scan's two totals, the
// occurrence and longest-read accumulators, the NUL flag first).
struct StreamState {
    unsigned long long newlines;                  // through the current piece
    unsigned long long piece_reads, piece_words;  // kept reads and their words in the piece
    unsigned long long occ, longest;              // kept reads' k-mer occurrences, longest read
    unsigned long long nul;                       // a NUL byte was seen (low 32 bits)
    unsigned long long records;                   // records framed before the piece
    unsigned long long reads, words;              // kept reads and words framed so far
    unsigned long long overflow;                  // a capacity below the text's needs
    unsigned long long rec_range[2];              // the piece's records
};
// One streamed piece framed with no host round trip (its newlines counted,
// scanned and located already): the records it completes are scanned and
// packed with the running totals as bases, the totals advanced, and the
// piece's reads written to piece_reads as [first, end) for the level-1
// scatter. Capacities the text outgrows set st->overflow instead of being
// written past.
int launch_frame_piece(const uint64_t *nl, uint64_t nl_cap, StreamState *st, uint64_t rec_cap, int k,
                       uint64_t *scratch,
                       uint64_t *read_idx, uint64_t *word_off, const unsigned char *t, uint64_t *off,
                       uint32_t *len, uint32_t *packed, uint64_t reads_cap, uint64_t words_cap,
                       unsigned long long *piece_reads, cudaStream_t s);
// Records r0 <= r < n_rec: read_idx[r] / word_off[r] = kept records (length
// >= k) / their 16-base words before r, from r0; totals to tot[0], tot[1];
// with acc, the kept reads' k-mer occurrences added to acc[0] and their
// longest length maxed into acc[1]. scratch holds rec_scan_scratch(n) words.
uint64_t rec_scan_scratch(uint64_t n_rec);
int launch_rec_scan(const uint64_t *nl, uint64_t r0, uint64_t n_rec, int k, uint64_t *scratch,
                    uint64_t *read_idx, uint64_t *word_off, uint64_t *tot, unsigned long long *acc,
                    cudaStream_t s);
int launch_rec_pack(const unsigned char *t, const uint64_t *nl, uint64_t n_rec, int k,
                    const uint64_t *read_idx, const uint64_t *word_off, uint64_t *off,
                    uint32_t *len, uint32_t *packed, cudaStream_t s, uint64_t r0 = 0,
                    uint64_t read_base = 0, uint64_t word_base = 0);
constexpr uint64_t kFramingChunk = 16384;  // bytes per block of k_nl_count / k_nl_pos
int launch_chunk_prefix(const BucketArgs &b, cudaStream_t s);
int launch_sub_hist(const BucketArgs &b, cudaStream_t s);
int launch_sub_scatter(const BucketArgs &b, cudaStream_t s);
int launch_bucket_count(const BuildArgs &a, const BucketArgs &b, cudaStream_t s);
// Entries of the tier-1 shared table launch_bucket_count uses for this build
// (2048 for small untagged buckets, else 4096).
int bucket_count_table(const BuildArgs &a, const BucketArgs &b);
int launch_bucket_gather(const BuildArgs &a, const BucketArgs &b, uint64_t n_buckets, cudaStream_t s);
int launch_group_by_sample(const unsigned long long *in_keys, const unsigned long long *in_mult,
                           uint64_t n, int tag_bits, uint32_t n_samples, unsigned long long *cursor,
                           unsigned long long *out_keys, unsigned long long *out_mult, cudaStream_t s);
cudaError_t run_probe(int kind, uint64_t table_bytes, uint64_t n_ops, cudaStream_t s, float *ms);
cudaError_t run_smem_probe(int kind, uint64_t n_ops, cudaStream_t s, float *ms);
int device_sm_count();

// Thread-local error message (api.cpp).
void set_error(const std::string &msg);

// Host framing / packing (reads.cpp).
swg_status pack_fasta(const char *text, uint64_t len, int k, swg_reads **out);

// Host writers (writers.cpp): records sorted by key.
swg_status write_kmer_graph(const uint64_t *keys, const uint8_t *mult, uint64_t n, int k,
                            const char *path);
swg_status write_node_lines(const uint64_t *keys, const uint8_t *mult, uint64_t n,
                            const char *path);
void graph_stats(const uint8_t *mult, uint64_t n, int k, int64_t out[5]);
void sort_records(uint64_t *keys, uint64_t *mult8, uint64_t n);
uint64_t revcomp_host(uint64_t x, int k);
// Device emission of the text outputs (emit.cu), byte-identical with the host
// writers: records on the device, any order.
// Device text -> file through two pinned 64 MiB buffers (emit.cu).
swg_status stream_to_file(const char *d_text, uint64_t bytes, const char *path, cudaStream_t s);
// The merged graph on the device: the -d file's text (gathered node lines in
// key order + final '\n') and, per line, its node key and per arc slot the
// arc's length, multiplicity, offset of its string in the text and the arc
// at the far end pointing back (far line * 8 + slot; ~0u for an empty slot).
struct MergedGraph {
    int k = 0;
    char *text = nullptr, *text2 = nullptr;  // current text, spare for rewrites
    uint64_t text_cap = 0, text2_cap = 0, text_bytes = 0;
    uint64_t lines = 0, line_cap = 0, nodes = 0;  // lines held; nodes printed
    unsigned long long *key = nullptr;
    unsigned *len = nullptr;
    unsigned char *mult = nullptr;
    unsigned long long *src = nullptr, *src2 = nullptr;
    unsigned *back = nullptr;
    unsigned char *del = nullptr;  // deleted by a pass
    cudaMemPool_t pool = nullptr;   // scratch of the merge and the passes, kept for reuse
};
void merged_free(MergedGraph *m);
swg_status merged_reserve(MergedGraph *m, uint64_t bytes, uint64_t lines);
// Merging of semi-extended k-molecules (merge.cu) into *mg.
struct MergeResult {
    uint64_t text_bytes = 0, nodes = 0, chains = 0, cycles = 0, rulers = 0;
    int launches = 0;
};
// h_order: if set, the n keys in the order the merge visits them (host memory)
swg_status merge_graph(const unsigned long long *d_keys, const unsigned long long *d_mult, uint64_t n, int k,
                       cudaStream_t s, MergedGraph *mg, MergeResult *res,
                       const unsigned long long *h_order = nullptr, uint64_t n_order = 0);
// masterTipsRemoval / masterLowCoverageEdgeRemoval on the merged graph
// (prune.cu); the text is rewritten. *count = tips removed / arcs cut.
swg_status prune_tips(MergedGraph *mg, cudaStream_t s, uint64_t *count);
swg_status prune_low_coverage(MergedGraph *mg, cudaStream_t s, uint64_t *count);
// masterSimplifyNodeGraph on the merged graph (prune.cu); *count = nodes merged away.
swg_status simplify_lines(MergedGraph *mg, cudaStream_t s, uint64_t *count);
// printContigs of the merged graph into a file (prune.cu); *count = contigs.
swg_status write_contigs(MergedGraph *mg, const char *path, cudaStream_t s, uint64_t *count);
swg_status emit_node_lines(const unsigned long long *d_keys, const unsigned long long *d_mult, uint64_t n,
                           int k, const char *path, cudaStream_t s);
swg_status emit_kmer_graph(const unsigned long long *d_keys, const unsigned long long *d_mult, uint64_t n, int k,
                           const char *path, cudaStream_t s);
uint64_t kmer_graph_neighbour(uint64_t key, int slot, int k);

}  // namespace swg
