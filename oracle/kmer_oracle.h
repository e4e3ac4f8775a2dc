/*
 * kmer_oracle — CPU restatement of SWAP-Assembler's k-mer graph construction.
 *
 * TEST INFRASTRUCTURE ONLY. This code is the parity checker for the GPU
 * library: only the tests, the smoke check and the CPU-baseline leg of the
 * benchmark load it. The product path never calls it.
 *
 * Semantics restated (all citations are files of the reference project):
 *   read framing / normalisation   kmerGraph.cpp:113-114,160-192,201-233
 *   2-bit encoding, MASK           kmerGraph.cpp:16-24,240-244; sequence.cpp:164-180
 *   reverse complement             kmerGraph.cpp:5-14
 *   canonical k-molecule = max     kmerGraph.cpp:246-247
 *   per-occurrence arc mask        kmerGraph.cpp:39-47,249-296
 *   saturating uint8 counting      graph.cpp:1058-1080 (type arc, graph.cpp:36-40)
 *   cutoff                         graph.cpp:1092-1114
 *   node arcs                      graph.cpp:81-102 (node::init)
 *   kmerGraph.txt (-s) lines       graph.cpp:3352-3440 with node::getNodeID 164-196
 *   node lines                     graph.cpp:555-572 (printLocalNodeGraph)
 *   graph statistics               graph.cpp:1569-1627
 */
#ifndef SWG_KMER_ORACLE_H
#define SWG_KMER_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Parse errors (the reference does not terminate or aborts on these). */
#define ORACLE_OK 0
#define ORACLE_ERR_NO_RECORD (-1)   /* no '>' in the input (kmerGraph.cpp:113-114 assert) */
#define ORACLE_ERR_UNTERMINATED (-2) /* last record lacks its '\n' (kmerGraph.cpp:155 never reached) */
#define ORACLE_ERR_NUL_BYTE (-3)    /* NUL byte before the end (strstr stops there) */
#define ORACLE_ERR_BAD_K (-4)
#define ORACLE_ERR_OOM (-5)

typedef struct oracle_reads {
    uint8_t *codes;     /* 0..3 per base, reads concatenated */
    uint64_t *off;      /* base offset of read i in codes */
    uint32_t *len;      /* length of read i (>= k) */
    uint64_t n_reads;
    uint64_t n_bases;
    uint64_t n_records; /* records seen, including those shorter than k */
} oracle_reads;

typedef struct oracle_graph oracle_graph;

/* Framing + normalisation of a single-line FASTA held in memory. Keeps only
 * reads of length >= k. Returns ORACLE_OK or a negative error. */
int oracle_parse_fasta(const char *buf, uint64_t len, int k, oracle_reads *out);
void oracle_reads_free(oracle_reads *r);

/* Count every occurrence and (when apply_cutoff != 0) apply the -c cutoff.
 * threads <= 0 means all online cores. With apply_cutoff == 0 the graph holds
 * every distinct k-molecule including those whose 8 counts are all zero. */
oracle_graph *oracle_build(const oracle_reads *r, int k, int cutoff, int apply_cutoff, int threads);
oracle_graph *oracle_build_fasta(const char *buf, uint64_t len, int k, int cutoff, int threads,
                                 int *err);

/* Records sorted by key ascending; mult holds 8 bytes per key (slot 0..7). */
uint64_t oracle_graph_size(const oracle_graph *g);
void oracle_graph_get(const oracle_graph *g, uint64_t *keys, uint8_t *mult);
void oracle_graph_free(oracle_graph *g);

/* Output files; lines sorted by their first token. */
int oracle_write_kmer_graph(const oracle_graph *g, int k, const char *path);
int oracle_write_node_lines(const oracle_graph *g, const char *path);

/* graph.cpp:1569-1627 totals: nodes, edges, edge-length sum, tips, bubbles. */
void oracle_graph_stats(const oracle_graph *g, int k, int64_t out[5]);

/* Merging of semi-extended k-molecules (merge_oracle.c, graph.cpp:1204-1566)
 * over n nodes (keys, 8 multiplicities each, as the build leaves them),
 * visited in `order` (n node indices). Writes the gathered node lines of the
 * surviving nodes in visiting order, plus the closing '\n' of the -d file
 * (graph.cpp:576-696, 3617-3621), into *text (free with oracle_free_text).
 * Returns 0 or a negative error (-10 neighbour missing, -11 no arc back to
 * the sender, -12 unlock of an unlocked node: the reference exits on each). */
#define MERGE_TIMING_REFERENCE 0 /* one rank's lazy message handling */
#define MERGE_TIMING_IMMEDIATE 1 /* every message applied when sent */
int oracle_merge(int k, uint64_t n, const uint64_t *keys, const uint8_t *mult, const uint64_t *order,
                 int timing, char **text, uint64_t *text_len, uint64_t *n_lines);
void oracle_free_text(char *text);
/* The visiting order the GPU merge follows (see merge_oracle.c). */
int oracle_merge_tree_order(int k, uint64_t n, const uint64_t *keys, const uint8_t *mult, uint64_t *order);

/* Rank-0 passes over a merged graph given as gathered node lines (the -d
 * file): passes bit 0 = masterTipsRemoval (graph.cpp:2194-2265), bit 1 =
 * masterLowCoverageEdgeRemoval (graph.cpp:2267-2300), in that order. Nodes are
 * visited in `order` (indices of the input's lines; NULL = file order); the
 * result is written as gathered lines in that order (+ '\n'). *count receives
 * the tips removed plus the arcs cut. */
int oracle_prune(int k, const char *text, uint64_t len, const uint64_t *order, int passes, char **out,
                 uint64_t *out_len, uint64_t *count);

/* masterSimplifyNodeGraph (graph.cpp:2089-2192) once over gathered lines,
 * visiting them in `order` (NULL = file order); *merged = nodes merged away. */
int oracle_simplify_lines(int k, const char *text, uint64_t len, const uint64_t *order, char **out,
                          uint64_t *out_len, uint64_t *merged);
/* The GPU's visiting order for that pass (chains numbered from their smaller
 * end arc, level ctz(position)), as line indices; *n = lines. */
int oracle_lines_tree_order(int k, const char *text, uint64_t len, uint64_t *order, uint64_t cap, uint64_t *n);

/* Neighbour id printed in kmerGraph.txt for slot s of key K (graph.cpp:3380-3427). */
uint64_t oracle_kmer_graph_neighbour(uint64_t key, int slot, int k);
uint64_t oracle_revcomp(uint64_t x, int k);

#ifdef __cplusplus
}
#endif
#endif
