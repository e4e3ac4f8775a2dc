/*
 * swapgb.h — C ABI of the GB300 k-mer graph builder.
 *
 * The library builds SWAP-Assembler's filtered k-mer graph (every canonical
 * k-molecule with its 8 strand-oriented edge multiplicities, after the -c
 * cutoff) on one GPU. All entry points are plain C: pointers, sizes and
 * status codes; no exceptions cross the boundary and nothing calls exit().
 *
 * Reference seams each entry point replaces (files of the reference project):
 *   parameter::getopt / getParameters ......... sequence.cpp:4-183 (CLI `swap`)
 *   MPIEnviroment::File_read + read framing .... mympi.cpp:108-120,
 *                                                kmerGraph.cpp:95-233 -> swg_reads_from_fasta
 *   kmerGraph::constructKmerGraph +
 *   distNodeGraph::constructDistNodeGraph +
 *   distNodeGraph::cutoffGraph ................. kmerGraph.cpp:95-310, graph.cpp:1049-1114
 *                                                -> swg_build, swg_build_device, swg_graph_build*
 *   distNodeGraph::kmolecules (hash_map<u64,arc>) graph.cpp:36-40,353 -> swg_graph_copy_out,
 *                                                swg_graph_device_view
 *   distNodeGraph::graphStatistics ............. graph.cpp:1569-1627 -> swg_graph_stats
 *   distNodeGraph::printKmerGraph (-s output) .. graph.cpp:3352-3440 -> swg_graph_write_kmer_graph
 *   distNodeGraph::printLocalNodeGraph ......... graph.cpp:555-572 -> swg_graph_write_node_lines
 *   distNodeGraph::simplifyDistNodeGraph ....... graph.cpp:1392-1566 (+ recvProc 1204-1389)
 *                                                -> swg_graph_merge
 *   distNodeGraph::gatherDistNodeGraph, -d file  graph.cpp:576-696, 3617-3621
 *                                                -> swg_graph_write_merged / swg_graph_copy_merged
 *   distNodeGraph::masterTipsRemoval ........... graph.cpp:2194-2265 -> swg_graph_remove_tips
 *   distNodeGraph::masterLowCoverageEdgeRemoval  graph.cpp:2267-2300 -> swg_graph_remove_low_coverage
 *   distNodeGraph::masterSimplifyNodeGraph ..... graph.cpp:2089-2192 -> swg_graph_simplify
 *   distNodeGraph::printContigs ................ graph.cpp:1139-1202 -> swg_graph_write_contigs
 *
 * Packed read layout (host or device memory):
 *   packed   uint32 words; base i of the concatenated read stream sits in
 *            word i/16 at bits [31-2*(i%16), 30-2*(i%16)] (first base most
 *            significant, the reference's encoding order, kmerGraph.cpp:16-24),
 *            codes A=0 C=1 G=2 T=3 (sequence.cpp:164-168).
 *   read_off base offset of each read in the stream (uint64).
 *   read_len length of each read (uint32). Reads shorter than k contribute
 *            nothing (kmerGraph.cpp:182-187).
 *
 * Results: keys are canonical k-molecules, max(kmer, reverse complement)
 * (kmerGraph.cpp:246-247); mult holds 8 bytes per key, slot t = the
 * reference's arc::multiplicity[t] (graph.cpp:36-40): saturating uint8
 * counts (graph.cpp:1076) after the cutoff (graph.cpp:1105).
 *
 * Threading: distinct handles may be used from distinct host threads; one
 * handle must not be used concurrently. Every device operation of a call is
 * ordered on the stream given in swg_opts (or the library's own stream).
 */
#ifndef SWAPGB_H
#define SWAPGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum swg_status {
    SWG_OK = 0,
    SWG_ERR_BAD_INPUT = 1,  /* bad argument, k out of range, malformed FASTA */
    SWG_ERR_TABLE_FULL = 2, /* hash table probe limit hit after all internal retries */
    SWG_ERR_OOM = 3,        /* device or host allocation failed */
    SWG_ERR_ADMISSION = 4,  /* server: request larger than the memory budget */
    SWG_ERR_TIMEOUT = 5,    /* a bounded device-side retry loop gave up */
    SWG_ERR_CUDA = 6,       /* CUDA runtime error (message in swg_last_error) */
    SWG_ERR_NO_DEVICE = 7,  /* no CUDA device visible */
    SWG_ERR_BAD_STATE = 8,  /* handle used in a state that does not allow the call */
    SWG_ERR_IO = 9,         /* file could not be read or written */
    SWG_ERR_NOT_READY = 10  /* server: result not finished yet */
} swg_status;

/* Counting algorithms (same results, different memory traffic). */
#define SWG_ALGO_DEFAULT 0     /* bucketed when its workspace (at most 40 bytes per
                                  k-mer occurrence) fits in device memory and no
                                  read is longer than 16384 bases, else direct;
                                  direct for SWG_ORDER_MINIMIZER */
#define SWG_ALGO_DIRECT 1      /* one pass into a device-wide table in HBM */
#define SWG_ALGO_PARTITIONED 2 /* hash-partitioned records, each partition counted in L2 */
#define SWG_ALGO_BUCKETED 3    /* records split into buckets counted in shared memory */

/* Order in which the direct algorithm counts the reads (same results). */
#define SWG_ORDER_INPUT 0     /* input order (default) */
#define SWG_ORDER_MINIMIZER 1 /* reads sharing a minimizer k-molecule counted together:
                                 fewer DRAM misses, more CAS contention; slower on GB300 */

typedef struct swg_opts {
    int k;                      /* 1..31; the CLI enforces the reference's odd 19..31 */
    int cutoff;                 /* -c: slot kept iff multiplicity >= cutoff */
    double load_factor;         /* target hash-table load, (0,0.9]; 0 selects 0.6 */
    uint64_t expected_distinct; /* direct algorithm: table sizing hint; 0 = estimate on the device */
    void *stream;               /* cudaStream_t; NULL = the library's own stream */
    int algorithm;              /* SWG_ALGO_*; 0 = default */
    int read_order;             /* direct: SWG_ORDER_*; 0 = input order */
    /* Bucketed build knobs (0 = the default; swg_autotune picks them per k and
     * read-length band): target records per bucket (64..65535), level-1
     * partition bits (8..10; more are used when the buckets would otherwise
     * pass twice the target), block shape of the two scatter passes (the
     * default is 256 threads x 16 records each; 1 = 512 x 8 for both, 2 =
     * 256 x 8 for level 1 and 512 x 8 for level 2, 3 = level 2 staged by
     * bulk copies, 4 = level 1 with warp-cooperative extraction: the lanes of
     * a warp on consecutive k-mers, each cut from a window of the packed
     * words; single-sample builds from packed reads). */
    uint32_t bucket_records;
    int part_bits;
    int scatter_shape;
} swg_opts;

/* What the last build did (for measurement and tests). */
typedef struct swg_build_info {
    int algorithm;        /* SWG_ALGO_DIRECT, _PARTITIONED or _BUCKETED */
    int launches;         /* kernel launches of the build */
    uint64_t occurrences; /* k-mer occurrences counted */
    uint64_t distinct;    /* distinct k-molecules before the cutoff */
    uint64_t survivors;   /* after the cutoff */
    uint64_t table_entries; /* direct: table capacity; partitioned: entries per slice slot;
                               bucketed: number of buckets */
    uint32_t partitions;  /* partitioned, bucketed: number of (level-1) partitions */
    uint32_t slots;       /* partitioned: partitions counted at once (one wave);
                             bucketed: sub-buckets per partition */
    uint32_t waves;       /* partitioned: waves; bucketed: buckets counted in a
                             global-memory table */
    uint32_t retries;     /* direct: rebuilds after a full table; bucketed: buckets
                             recounted in the larger (tier-2) shared-memory table */
    double estimate;      /* direct: distinct-count estimate used for sizing;
                             bucketed: 1 when a partition or bucket outgrew its
                             sampled region and the build reran with exact counts */
    float ms[5];          /* as swg_graph_last_timings */
    uint32_t bucket_table; /* bucketed: entries of the shared table the first
                              counting pass used (2048 when the buckets average
                              at most 3072 records, else 4096); 0 otherwise */
} swg_build_info;

typedef struct swg_reads swg_reads; /* host-side packed reads */
typedef struct swg_graph swg_graph; /* device-resident filtered k-mer graph + workspace */

/* ---- status ---------------------------------------------------------- */
const char *swg_status_string(swg_status s);
/* Last error message of the calling thread ("" if none). */
const char *swg_last_error(void);
/* Library version string. */
const char *swg_version(void);

/* ---- host FASTA framing and 2-bit packing ----------------------------- */
/* Reproduces the reference's framing (kmerGraph.cpp:113-114,160-233): from the
 * first '>', alternating header / single sequence line, each ended by '\n';
 * acgt upper-cased, any other byte read as 'A'; reads shorter than k dropped.
 * Input the reference never finishes (last record without '\n', NUL bytes,
 * no '>') returns SWG_ERR_BAD_INPUT. */
swg_status swg_reads_from_fasta(const char *text, uint64_t len, int k, swg_reads **out);
swg_status swg_reads_from_fasta_file(const char *path, int k, swg_reads **out);
/* Borrowed views into the packed read set (valid until swg_reads_free). */
swg_status swg_reads_view(const swg_reads *r, const uint32_t **packed, uint64_t *n_words,
                          const uint64_t **read_off, const uint32_t **read_len,
                          uint64_t *n_reads, uint64_t *n_bases);
/* Records seen while framing, including those shorter than k. */
uint64_t swg_reads_records(const swg_reads *r);
void swg_reads_free(swg_reads *r);

/* ---- graph build ------------------------------------------------------ */
/* Create an empty graph handle on the current CUDA device. Its device
 * workspace (table, tiles, outputs) is kept and reused by later builds. */
swg_status swg_graph_create(swg_graph **out);
void swg_graph_free(swg_graph *g);

/* Build from packed reads in HOST memory: copies them to the device, builds,
 * leaves the result on the device. */
swg_status swg_graph_build(swg_graph *g, const swg_opts *o, const uint32_t *packed,
                           uint64_t n_words, const uint64_t *read_off,
                           const uint32_t *read_len, uint64_t n_reads);
/* Same with the packed reads already in DEVICE memory. */
swg_status swg_graph_build_device(swg_graph *g, const swg_opts *o, const uint32_t *d_packed,
                                  uint64_t n_words, const uint64_t *d_read_off,
                                  const uint32_t *d_read_len, uint64_t n_reads);
/* Build from a FASTA held in HOST memory, framed and packed ON THE DEVICE: the
 * text is copied to the GPU, lines are found and paired there with the same
 * framing as swg_reads_from_fasta (same errors), reads are 2-bit packed, then
 * built as swg_graph_build_device. A text of 96 MiB or more is copied in
 * pieces, each framed and scattered while the rest is still copying (the
 * result is the same); from pinned host memory (cudaHostAlloc) the copies
 * overlap the work. The call returns after every copy from `text` has ended.
 * Environment: SWG_NO_STREAM=1 copies and frames the text in one piece;
 * SWG_STREAM_PIECES=2..16 sets the number of pieces. */
swg_status swg_graph_build_fasta(swg_graph *g, const swg_opts *o, const char *text, uint64_t len);

/* As swg_graph_build_fasta, then the filtered graph into the caller's host
 * arrays (keys[n], mult[8 n], unordered, as swg_graph_copy_out with sorted =
 * 0): the end-to-end form of constructDistNodeGraph + cutoffGraph
 * (graph.cpp:1049-1114) for a caller that wants the graph in host memory.
 * When keys and mult are pinned host memory the device can address
 * (cudaHostAlloc, cudaHostRegister) and the bucketed build runs, every
 * bucket's survivors are written there as the bucket is counted, so the copy
 * overlaps the counting; the order may then differ between calls. Otherwise
 * the graph is copied after the build. The graph also stays on the device as
 * after swg_graph_build_fasta. More than cap survivors: SWG_ERR_BAD_INPUT with
 * *n_out set to the count needed. */
swg_status swg_graph_build_fasta_to_host(swg_graph *g, const swg_opts *o, const char *text, uint64_t len,
                                         uint64_t *keys, uint8_t *mult, uint64_t cap, uint64_t *n_out);

/* As swg_graph_build_fasta, on the FASTA file at path: the file is read (in
 * parallel slices) into a pinned host buffer the handle keeps for later calls,
 * then uploaded, framed and built on the device. The reference's reader takes
 * the file by name too (parameter::fastaPath, kmerGraph.cpp:95-156); this is
 * the one-call replacement for constructDistNodeGraph + cutoffGraph
 * (graph.cpp:1049-1114) on a file. SWG_ERR_IO if the file cannot be read. */
swg_status swg_graph_build_fasta_file(swg_graph *g, const swg_opts *o, const char *path);
/* Convenience: create + build from host packed reads. */
swg_status swg_build(const swg_opts *o, const uint32_t *packed, uint64_t n_words,
                     const uint64_t *read_off, const uint32_t *read_len, uint64_t n_reads,
                     swg_graph **out);
/* Convenience: create a handle and build from a FASTA text in host memory
 * (swg_graph_build_fasta: framed and packed on the device). */
swg_status swg_build_fasta(const swg_opts *o, const char *text, uint64_t len, swg_graph **out);

/* ---- batched build ---------------------------------------------------- */
/* One sample of a batch: its packed reads in HOST memory (layout as above,
 * offsets relative to its own packed words) and its own k and cutoff. */
typedef struct swg_sample {
    const uint32_t *packed;
    uint64_t n_words;
    const uint64_t *read_off;
    const uint32_t *read_len;
    uint64_t n_reads;
    int k;
    int cutoff;
} swg_sample;

/* Build many independent samples at once: their reads (host or device
 * memory) are copied into one device stream and every kernel runs once over
 * all samples. By default (2 * largest k + ceil(log2 samples) <= 64, at most
 * 1024 samples) every key carries its sample's index in its top bits and one
 * bucketed build counts all samples, each bucket applying each key's own
 * sample cutoff; otherwise each sample counts into its own partition of one
 * direct table. Each sample gets its own output region, and its result equals
 * a plain build of that sample alone. opts->k and opts->cutoff are ignored
 * (each sample has its own). */
swg_status swg_batch_build(swg_graph *g, const swg_opts *o, const swg_sample *samples,
                           uint32_t n_samples);
swg_status swg_batch_samples(const swg_graph *g, uint32_t *n_samples);
/* Per-sample results of the last batched build (sample s < n_samples). */
swg_status swg_batch_sample_info(const swg_graph *g, uint32_t s, uint64_t *occurrences,
                                 uint64_t *distinct, uint64_t *survivors);
swg_status swg_batch_device_view(const swg_graph *g, uint32_t s, const uint64_t **d_keys,
                                 const uint64_t **d_mult, uint64_t *n);
swg_status swg_batch_copy_out(const swg_graph *g, uint32_t s, uint64_t *keys, uint8_t *mult,
                              uint64_t cap, int sorted, uint64_t *n);

/* ---- request server (continuous batching) ------------------------------ */
/* Graph-build requests arrive at any time; worker threads batch every queued
 * request that fits the memory budget into one batched build (several batches
 * overlap on the device, one per worker) and keep each result on the device
 * until it is fetched or released. Admission charges a request an estimate of
 * its footprint (sized by its k-mer occurrence count, an upper bound on its
 * distinct k-molecules) while its batch runs and its exact result size while
 * resident; a request larger than the whole budget is refused
 * (SWG_ERR_ADMISSION). Each result equals the plain build of that request. */
typedef struct swg_server swg_server;

typedef struct swg_server_opts {
    uint64_t memory_budget; /* device bytes for in-flight batches + resident results; 0 = 150 GiB */
    uint32_t workers;       /* batches in flight at once; 0 = 2 */
    uint32_t max_batch;     /* requests per batch; 0 = no limit */
    double load_factor;     /* 0 = 0.6 */
} swg_server_opts;

typedef struct swg_server_stats {
    uint64_t submitted, completed, failed, rejected, batches, max_batch_requests;
    uint64_t queued, bytes_reserved, bytes_resident;
} swg_server_stats;

#define SWG_REQ_QUEUED 0
#define SWG_REQ_RUNNING 1
#define SWG_REQ_DONE 2
#define SWG_REQ_FAILED 3

swg_status swg_server_create(const swg_server_opts *o, swg_server **out);
/* Uploads the request's reads to device memory (they wait there until a
 * worker builds them); the caller may free its buffers on return. SWG_ERR_OOM
 * if the device cannot hold them. If no
 * worker could set itself up (graph handle or stream creation failed), queued
 * requests fail with that reason and submit returns SWG_ERR_BAD_STATE. */
swg_status swg_server_submit(swg_server *srv, const swg_sample *req, uint64_t *ticket);
/* Non-blocking: state (SWG_REQ_*) and latency so far (submit to completion). */
swg_status swg_server_poll(swg_server *srv, uint64_t ticket, int *state, double *latency_s);
/* Blocks at most timeout_s seconds; SWG_ERR_NOT_READY on timeout. */
swg_status swg_server_wait(swg_server *srv, uint64_t ticket, double timeout_s);
swg_status swg_server_result_info(swg_server *srv, uint64_t ticket, uint64_t *survivors,
                                  uint64_t *distinct);
/* Copies the result to host memory (sorted by key when sorted != 0) and frees
 * it on the device; the ticket is then gone. */
swg_status swg_server_fetch(swg_server *srv, uint64_t ticket, uint64_t *keys, uint8_t *mult,
                            uint64_t cap, int sorted, uint64_t *n);
/* Drops a finished result without copying it. */
swg_status swg_server_release(swg_server *srv, uint64_t ticket);
swg_status swg_server_get_stats(swg_server *srv, swg_server_stats *out);
/* Finishes the batches in flight, drops queued requests and results, frees. */
void swg_server_free(swg_server *srv);

/* ---- results ---------------------------------------------------------- */
/* The swg_graph_* result calls below refer to a single-sample build
 * (SWG_ERR_BAD_STATE after a batched build; use swg_batch_* there). */
/* Number of surviving k-molecules (after the cutoff). */
swg_status swg_graph_size(const swg_graph *g, uint64_t *n);
/* Distinct k-molecules before the cutoff (all keys ever inserted). */
swg_status swg_graph_distinct(const swg_graph *g, uint64_t *n);
/* Device pointers to the unordered result: keys[n], mult[n] (8 bytes per key
 * packed in a uint64, byte t = slot t). Valid until the next build or free. */
swg_status swg_graph_device_view(const swg_graph *g, const uint64_t **d_keys,
                                 const uint64_t **d_mult, uint64_t *n);
/* Copy the result to host memory, sorted by key when sorted != 0.
 * keys[cap], mult[8*cap]; *n receives the count (SWG_ERR_BAD_INPUT if cap < n). */
swg_status swg_graph_copy_out(const swg_graph *g, uint64_t *keys, uint8_t *mult, uint64_t cap,
                              int sorted, uint64_t *n);
/* graph.cpp:1613-1625 totals: nodes, edges, edge-length sum, tips, bubbles. */
swg_status swg_graph_stats(const swg_graph *g, int64_t out[5]);
/* kmerGraph.txt exactly as the reference's -s run writes it (graph.cpp:3352-3440,
 * including its neighbour-id quirk), lines sorted by their first token. */
swg_status swg_graph_write_kmer_graph(const swg_graph *g, const char *path);
/* Node lines "K A# # ...# m0 .. m7" (graph.cpp:569), sorted by key; readable by
 * the reference's readDistNodeGraph (graph.cpp:898-941). */
swg_status swg_graph_write_node_lines(const swg_graph *g, const char *path);
/* Merging of semi-extended k-molecules over the built graph: the reference's
 * SWAP merge (simplifyDistNodeGraph, graph.cpp:1392-1566, edge messages
 * graph.cpp:1289-1345). Every node with exactly one arc on each side that does
 * not lead back to itself is merged into its neighbours; the remaining nodes'
 * arcs then spell whole chains up to the next remaining node. Arc strings are
 * those of any complete merge order; a merged arc's multiplicity is the
 * reference's running weighted average (graph.cpp:1322-1324, including its
 * int truncation) taken in one fixed visiting order: a chain of m merged
 * nodes numbered 1..m from its smaller end arc (key, then slot), node p at
 * level ctz(p), levels in increasing order. A cycle of merged nodes is cut at
 * its largest key, which keeps the cycle on its two arcs. The result stays on
 * the device (as the -d file's text) until the next build; the handle keeps
 * the merge's device workspace in its own memory pool until swg_graph_free, so
 * later merges and passes need not map it again. SWG_ERR_BAD_STATE
 * without a single-sample build; SWG_ERR_BAD_INPUT for an even k (the
 * reference's k is odd, sequence.cpp:44) or more than 2^29 k-molecules. */
swg_status swg_graph_merge(swg_graph *g);
/* The same merge with the nodes visited in the caller's order: order_keys
 * lists every k-molecule of the built graph once (host memory), in the order
 * the reference's merge loop meets them (its node map's iteration order,
 * graph.cpp:1412). Each chain's multiplicities are then those of that order
 * with every edge message applied as it is sent: the chain's merge tree is
 * the Cartesian tree of the visit times (a node merges the segments that
 * reach, on each side, the nearest node visited after it); a cycle keeps the
 * node visited last. Arc strings and surviving nodes are those of
 * swg_graph_merge. SWG_ERR_BAD_INPUT if the order misses a key, repeats one
 * or names one the graph does not hold. */
swg_status swg_graph_merge_in_order(swg_graph *g, const uint64_t *order_keys, uint64_t n_order);
typedef struct swg_merge_info {
    uint64_t nodes;      /* nodes left (lines of the -d file) */
    uint64_t chains;     /* chains of merged nodes */
    uint64_t cycles;     /* cycles of merged nodes (cut at their largest key) */
    uint64_t text_bytes; /* size of the -d file */
    float ms;            /* device time of the merge, including its text */
    int launches;        /* kernel launches of the merge */
} swg_merge_info;
swg_status swg_graph_merge_info(const swg_graph *g, swg_merge_info *info);
/* The merged graph as the reference's -d file contigGraph.txt
 * (gatherDistNodeGraph lines, graph.cpp:615-645: id, 8 arcs each closed by
 * '#', 8 multiplicities, blank-padded to sum(arc length + 1) + 61 bytes; then
 * the final '\n' of graph.cpp:3620), lines in key order. copy_merged needs
 * cap >= the text size (*n receives it either way). */
swg_status swg_graph_write_merged(const swg_graph *g, const char *path);
swg_status swg_graph_copy_merged(const swg_graph *g, char *buf, uint64_t cap, uint64_t *n);
/* Two of the reference's rank-0 passes over the merged graph (after
 * swg_graph_merge; the merged text is rewritten, deleted and arc-less nodes
 * left out as gatherDistNodeGraph does):
 * remove_tips = masterTipsRemoval (graph.cpp:2194-2265): a node with exactly
 *   one arc, shorter than k, loses it, the far node loses its arc back, and
 *   the node is deleted. Every node that is a tip when the pass starts is
 *   judged on that state (the reference's one pass visiting all other nodes
 *   first, then the tips in key order); of two tips joined only to each other
 *   the smaller key is deleted. *removed = nodes deleted.
 * remove_low_coverage = masterLowCoverageEdgeRemoval (graph.cpp:2267-2300):
 *   avg = sum(len*m)/sum(len) over the arcs left (integer division); every
 *   arc shorter than 2k with m < avg/4 is cut. *cut = arcs cut (both ends of
 *   an edge count). With no arc left nothing is cut (the reference divides by
 *   zero). Neither pass merges the nodes it leaves with one arc per side (the
 *   reference's masterSimplifyNodeGraph does that next). */
swg_status swg_graph_remove_tips(swg_graph *g, uint64_t *removed);
swg_status swg_graph_remove_low_coverage(swg_graph *g, uint64_t *cut);
/* masterSimplifyNodeGraph (graph.cpp:2089-2192) on the merged graph, as the
 * reference runs it after those passes: a node left with exactly one arc on
 * each side whose neighbours are not itself is merged into its neighbours;
 * each end arc of a chain of such nodes becomes the concatenation of the
 * chain's arcs, with the weighted average multiplicity in size_t arithmetic
 * (graph.cpp:2157-2163) taken in swg_graph_merge's visiting order (chain
 * positions from the smaller end arc, node p at level ctz(p)); a cycle of such
 * nodes is cut at its largest key. *merged = nodes merged away. */
swg_status swg_graph_simplify(swg_graph *g, uint64_t *merged);
/* The reference's printContigs (graph.cpp:1139-1202, noCEcontigs.fasta) on the
 * merged graph as it stands: every arc of at least 100 - k bases
 * (Contig_Length, sequence.h:15), once, from the end whose key is not smaller
 * than the far end's, as the line ">proc0: " + that node's k-mer (its reverse
 * complement for slots 4-7) + the arc string; nodes in key order. *n =
 * contigs written. */
swg_status swg_graph_write_contigs(swg_graph *g, const char *path, uint64_t *n);
/* Host-only writers for records already in host memory (keys[n], mult[8*n],
 * any order): the same two file formats as above. */
swg_status swg_records_write_kmer_graph(const uint64_t *keys, const uint8_t *mult, uint64_t n,
                                        int k, const char *path);
swg_status swg_records_write_node_lines(const uint64_t *keys, const uint8_t *mult, uint64_t n,
                                        const char *path);
/* Device times (ms) of the last build's phases, from CUDA events on the build
 * stream. Direct / partitioned: [0] sizing (occurrence prefix, tiles, distinct
 * estimate or partition histogram), [1] preparation (table clear, or record
 * scatter), [2] counting (K1, or every wave's partition count + compaction),
 * [3] cutoff+compaction (direct only). Bucketed: [0] setup, [1] level-1
 * scatter kernel, [2] level-2 scatter, [3] bucket counting kernels. [4] whole
 * build. Also the launch count of the last build. */
swg_status swg_graph_last_timings(const swg_graph *g, float ms[5], int *launches);
swg_status swg_graph_build_info(const swg_graph *g, swg_build_info *info);

/* ---- build without device allocation ------------------------------------ */
/* No counterpart in the reference. For callers that must not have the library
 * allocate device memory (their memory is reserved by another allocator or a
 * fixed budget, or they cannot accept cudaMalloc's device-wide synchronisation
 * mid-run): the whole build runs in one file-scope device array of about
 * 72 MiB that every GPU loading the library holds until exit. The reads and the
 * output arrays (keys[out_cap], mult[out_cap] as in swg_graph_device_view) are
 * the caller's device memory. At most 1048576 reads and 2516505 k-mer
 * occurrences per call, else SWG_ERR_BAD_INPUT; more than out_cap survivors
 * gives SWG_ERR_BAD_INPUT with *n_out set to the count needed. The first call
 * on a device resolves the array's address, and so does the first call after
 * the device's context was destroyed (cudaDeviceReset): make those calls
 * before any stream capture. Calls share the array: calls whose device work
 * overlaps race. */
swg_status swg_build_device_noalloc(const swg_opts *o, const uint32_t *d_packed, uint64_t n_words,
                                    const uint64_t *d_read_off, const uint32_t *d_read_len,
                                    uint64_t n_reads, uint64_t *d_keys_out, uint64_t *d_mult_out,
                                    uint64_t out_cap, uint64_t *n_out);

/* ---- autotuner ---------------------------------------------------------- */
/* Times trial builds of a sample (device packed reads, as for
 * swg_graph_build_device) for each candidate: the bucketed build (the default
 * scheme) with records per bucket 2048 / 4096 / 8192 and each scatter block
 * shape (the level-1 partition count follows the input's size); the direct table at load factors
 * 0.5-0.8, in input and in minimizer order; hash-partitioned slices. Appends
 * the fastest to a cache file as one JSON line keyed by (k, read-length band
 * of read_len_hint). */
typedef struct swg_tuning {
    double load_factor;
    int algorithm;
    int read_order;
    float ms;
    uint32_t bucket_records; /* bucketed knobs, as in swg_opts (0 = default) */
    int part_bits;
    int scatter_shape;
} swg_tuning;

swg_status swg_autotune(const swg_opts *base, const uint32_t *d_packed, uint64_t n_words,
                        const uint64_t *d_read_off, const uint32_t *d_read_len, uint64_t n_reads,
                        uint32_t read_len_hint, const char *cache_path, swg_tuning *best);
/* Sets o's load factor, algorithm, read order and bucketed knobs from the
 * cache entry for (k, band of read_len); SWG_ERR_NOT_READY when the cache has
 * none. */
swg_status swg_autotune_apply(const char *cache_path, int k, uint32_t read_len, swg_opts *o);

/* ---- roofline probe ----------------------------------------------------- */
/* Random-access throughput on this GPU: n_ops operations at uniformly random
 * 16-byte-aligned addresses of a table of table_bytes bytes (allocated and
 * freed inside). kind: 0 = 32-bit atomicAdd (no return), 1 = 64-bit CAS,
 * 2 = 128-bit CAS, 3 = 16-byte load, 4 = 16-byte load + 128-bit CAS on the
 * same address, 5 = as 3 with four independent loads in flight per thread,
 * 6 = as 4 with two independent chains per thread. Writes accesses (kinds
 * 5/6: loads, load+CAS pairs) per second (device time). */
swg_status swg_probe_random_access(int kind, uint64_t table_bytes, uint64_t n_ops, void *stream,
                                   double *ops_per_s);
/* Shared-memory atomic throughput on this GPU (lane operations per second,
 * whole GPU): n_ops random operations in per-CTA tables laid out like the
 * bucket count's (two CTAs of 512 threads per SM, 4096 64-bit key slots and
 * 16384 32-bit counter words each). kind: 0 = 32-bit atomicAdd, 1 = 64-bit
 * atomicCAS. The bucket count's on-chip floor is its CAS and counter adds at
 * these rates. No counterpart in the reference (a measurement tool). */
swg_status swg_probe_shared_atomics(int kind, uint64_t n_ops, void *stream, double *ops_per_s);

#ifdef __cplusplus
}
#endif
#endif /* SWAPGB_H */
