/*
 * kmer_oracle.c — CPU restatement of SWAP-Assembler's k-mer graph
 * construction. TEST INFRASTRUCTURE ONLY (the parity checker and the timed CPU
 * baseline); the product path never links it. Each function names the
 * reference lines it restates; see kmer_oracle.h for the full map.
 *
 * Parallel form: the reads are split into chunks, every thread extracts the
 * (k-molecule, arc-mask) pairs of its chunk and routes them to the owner
 * partition of the key; each partition is then counted by one thread in its
 * own open-addressing table. This is the reference's own np=N scheme
 * (distributeKmerGraph, kmerGraph.cpp:337-432, then the per-rank hash_map
 * count, graph.cpp:1058-1080) with threads in place of ranks. Counting is
 * order independent, so the result does not depend on the thread count.
 */
#define _GNU_SOURCE
#include "kmer_oracle.h"

#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

/* ------------------------------------------------------------------ */
/* A1: read framing and normalisation (kmerGraph.cpp:113-114,160-233). */
/* ------------------------------------------------------------------ */

/* Base code after the reference's normalisation (kmerGraph.cpp:228-233:
 * ACGT kept, acgt upper-cased, anything else becomes 'A') and the A=0 C=1
 * G=2 T=3 table (sequence.cpp:164-168). */
static uint8_t base_code(unsigned char ch) {
    switch (ch) {
        case 'C': case 'c': return 1;
        case 'G': case 'g': return 2;
        case 'T': case 't': return 3;
        default: return 0;
    }
}

/* The reference consumes the text as alternating lines from the first '>'
 * (kmerGraph.cpp:113-114): a header line, then ONE sequence line, both ended
 * by '\n' (strstr at 173 and 177). Sequences shorter than k are skipped
 * (182-187). A record without its final '\n' leaves bytes in the window that
 * are never consumed, so the reference loops forever (readEnd never reaches
 * 0 at kmerGraph.cpp:155); that is reported as ORACLE_ERR_UNTERMINATED. */
int oracle_parse_fasta(const char *buf, uint64_t len, int k, oracle_reads *out) {
    memset(out, 0, sizeof(*out));
    if (k < 1 || k > 31) return ORACLE_ERR_BAD_K;
    if (len && memchr(buf, 0, len)) return ORACLE_ERR_NUL_BYTE;
    const char *end = buf + len;
    const char *p = len ? memchr(buf, '>', len) : NULL;
    if (!p) return ORACLE_ERR_NO_RECORD;
    const char *start = p;
    uint64_t n_reads = 0, n_bases = 0, n_records = 0;
    while (p < end) {
        const char *h = memchr(p, '\n', (size_t)(end - p));
        if (!h) return ORACLE_ERR_UNTERMINATED;
        const char *s = h + 1;
        const char *e = s < end ? memchr(s, '\n', (size_t)(end - s)) : NULL;
        if (!e) return ORACLE_ERR_UNTERMINATED;
        uint64_t L = (uint64_t)(e - s);
        n_records++;
        if (L >= (uint64_t)k) { n_reads++; n_bases += L; }
        p = e + 1;
    }
    out->codes = (uint8_t *)malloc(n_bases ? n_bases : 1);
    out->off = (uint64_t *)malloc((n_reads ? n_reads : 1) * sizeof(uint64_t));
    out->len = (uint32_t *)malloc((n_reads ? n_reads : 1) * sizeof(uint32_t));
    if (!out->codes || !out->off || !out->len) { oracle_reads_free(out); return ORACLE_ERR_OOM; }
    p = start;
    uint64_t r = 0, b = 0;
    while (p < end) {
        const char *h = memchr(p, '\n', (size_t)(end - p));
        const char *s = h + 1;
        const char *e = memchr(s, '\n', (size_t)(end - s));
        uint64_t L = (uint64_t)(e - s);
        if (L >= (uint64_t)k) {
            out->off[r] = b;
            out->len[r] = (uint32_t)L;
            for (uint64_t i = 0; i < L; i++) out->codes[b + i] = base_code((unsigned char)s[i]);
            b += L;
            r++;
        }
        p = e + 1;
    }
    out->n_reads = n_reads;
    out->n_bases = n_bases;
    out->n_records = n_records;
    return ORACLE_OK;
}

void oracle_reads_free(oracle_reads *r) {
    free(r->codes);
    free(r->off);
    free(r->len);
    memset(r, 0, sizeof(*r));
}

/* ------------------------------------------------------------------ */
/* A2-A5: encoding, reverse complement, canonical key, arc mask.       */
/* ------------------------------------------------------------------ */

/* kmerGraph.cpp:5-14: reverse the base order and complement each base
 * ((3-a)&3). */
uint64_t oracle_revcomp(uint64_t a, int k) {
    uint64_t rev = 0;
    for (int i = 0; i < k; i++) {
        rev = (rev << 2) | ((3 - a) & 3);
        a >>= 2;
    }
    return rev;
}

typedef struct {
    uint64_t key;
    uint8_t mask;
} occ_t;

/* Emit the (key, mask) of every k-mer of one read.
 * kmerGraph.cpp:240-299 restated per occurrence j (0 <= j <= L-k):
 *   C = 2-bit code of bases j..j+k-1 (first base most significant, 240-244),
 *   K = max(C, rc(C)) (246-247), f = (C == K);
 *   right arc (j+k < L): slot (f ? 0 : 4) + code[j+k];
 *   left arc  (j >= 1):  slot (f ? 4 : 0) + 3 - code[j-1].
 * The four orientation cases at 261-296 with arcPos (39-47) reduce to these
 * two rules; the OR of the two bits (265/268) equals two independent counts
 * because the two slots always fall in opposite halves. */
typedef void (*occ_sink)(void *ctx, uint64_t key, uint8_t mask);

static void read_occurrences(const uint8_t *c, uint32_t L, int k, occ_sink sink, void *ctx) {
    const uint64_t kmask = (k == 32) ? ~0ull : ((1ull << (2 * k)) - 1);
    uint64_t fwd = 0;
    for (int i = 0; i < k - 1; i++) fwd = (fwd << 2) | c[i];
    for (uint32_t j = 0; j + (uint32_t)k <= L; j++) {
        fwd = ((fwd << 2) | c[j + k - 1]) & kmask;
        uint64_t rc = oracle_revcomp(fwd, k);
        uint64_t key = fwd > rc ? fwd : rc;
        int f = (fwd == key);
        uint8_t mask = 0;
        if (j + (uint32_t)k < L) mask |= (uint8_t)(1u << ((f ? 0 : 4) + c[j + k]));
        if (j >= 1) mask |= (uint8_t)(1u << ((f ? 4 : 0) + 3 - c[j - 1]));
        sink(ctx, key, mask);
    }
}

/* ------------------------------------------------------------------ */
/* A6: counting (graph.cpp:1058-1080).                                 */
/* ------------------------------------------------------------------ */

/* Open-addressing table; cnt holds the 8 uint8 multiplicities of the
 * reference's arc (graph.cpp:36-40), byte t = slot t. */
typedef struct {
    uint64_t *keys;
    uint64_t *cnt;
    uint64_t cap; /* power of two */
    uint64_t n;
} otable;

#define EMPTY_KEY (~0ull)

static uint64_t mix64(uint64_t x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return x;
}

static int otable_init(otable *t, uint64_t cap) {
    t->cap = cap;
    t->n = 0;
    t->keys = (uint64_t *)malloc(cap * sizeof(uint64_t));
    t->cnt = (uint64_t *)calloc(cap, sizeof(uint64_t));
    if (!t->keys || !t->cnt) return -1;
    memset(t->keys, 0xff, cap * sizeof(uint64_t));
    return 0;
}

static void otable_free(otable *t) {
    free(t->keys);
    free(t->cnt);
    memset(t, 0, sizeof(*t));
}

static uint64_t *otable_slot(otable *t, uint64_t key, int *is_new) {
    uint64_t m = t->cap - 1, h = mix64(key) & m;
    for (;;) {
        if (t->keys[h] == key) { *is_new = 0; return &t->cnt[h]; }
        if (t->keys[h] == EMPTY_KEY) {
            t->keys[h] = key;
            t->n++;
            *is_new = 1;
            return &t->cnt[h];
        }
        h = (h + 1) & m;
    }
}

static int otable_grow(otable *t) {
    otable nt;
    if (otable_init(&nt, t->cap * 2)) return -1;
    for (uint64_t i = 0; i < t->cap; i++) {
        if (t->keys[i] == EMPTY_KEY) continue;
        int is_new;
        *otable_slot(&nt, t->keys[i], &is_new) = t->cnt[i];
    }
    otable_free(t);
    *t = nt;
    return 0;
}

/* First occurrence: multiplicity[t] = bit t of the mask (graph.cpp:1062-1070);
 * later ones: ++ while below 255 (1074-1078). Net effect per slot:
 * min(occurrences with bit t, 255). */
static int otable_add(otable *t, uint64_t key, uint8_t mask) {
    if ((t->n + 1) * 10 > t->cap * 7 && otable_grow(t)) return -1;
    int is_new;
    uint64_t *c = otable_slot(t, key, &is_new);
    uint64_t v = *c;
    for (int s = 0; s < 8; s++) {
        if (!(mask & (1u << s))) continue;
        uint64_t b = (v >> (8 * s)) & 0xff;
        if (b < 255) v += 1ull << (8 * s);
    }
    *c = v;
    return 0;
}

/* ------------------------------------------------------------------ */
/* Parallel driver.                                                    */
/* ------------------------------------------------------------------ */

typedef struct {
    occ_t *v;
    uint64_t n, cap;
} occvec;

static int occvec_push(occvec *o, uint64_t key, uint8_t mask) {
    if (o->n == o->cap) {
        uint64_t nc = o->cap ? o->cap * 2 : 4096;
        occ_t *nv = (occ_t *)realloc(o->v, nc * sizeof(occ_t));
        if (!nv) return -1;
        o->v = nv;
        o->cap = nc;
    }
    o->v[o->n].key = key;
    o->v[o->n].mask = mask;
    o->n++;
    return 0;
}

struct oracle_graph {
    uint64_t n;
    uint64_t *keys;
    uint8_t *mult; /* 8 per key */
};

typedef struct shared_s shared_t;

typedef struct {
    shared_t *sh;
    int tid;
    occvec *out; /* [nparts] */
    int failed;
} worker_t;

struct shared_s {
    const oracle_reads *r;
    int k;
    int nthreads;
    int nparts;
    uint64_t batch_begin, batch_end; /* read range of the current batch */
    worker_t *w;
    otable *tables; /* [nparts] */
    pthread_barrier_t bar;
    int done;
};

typedef struct {
    occvec *out;
    int nparts;
    int failed;
} sink_ctx;

static int part_of(uint64_t key, int nparts) {
    return (int)((mix64(key ^ 0x5bd1e9955bd1e995ull) >> 40) % (uint64_t)nparts);
}

static void sink_route(void *vctx, uint64_t key, uint8_t mask) {
    sink_ctx *ctx = (sink_ctx *)vctx;
    if (occvec_push(&ctx->out[part_of(key, ctx->nparts)], key, mask)) ctx->failed = 1;
}

static void *worker_main(void *arg) {
    worker_t *w = (worker_t *)arg;
    shared_t *sh = w->sh;
    for (;;) {
        pthread_barrier_wait(&sh->bar); /* batch published */
        if (sh->done) break;
        /* phase 1: extract my slice of the batch, route by owner */
        uint64_t nb = sh->batch_end - sh->batch_begin;
        uint64_t lo = sh->batch_begin + nb * (uint64_t)w->tid / (uint64_t)sh->nthreads;
        uint64_t hi = sh->batch_begin + nb * (uint64_t)(w->tid + 1) / (uint64_t)sh->nthreads;
        sink_ctx ctx = {w->out, sh->nparts, 0};
        for (uint64_t i = lo; i < hi; i++)
            read_occurrences(sh->r->codes + sh->r->off[i], sh->r->len[i], sh->k, sink_route, &ctx);
        if (ctx.failed) w->failed = 1;
        pthread_barrier_wait(&sh->bar);
        /* phase 2: count the partitions I own */
        for (int p = w->tid; p < sh->nparts; p += sh->nthreads) {
            for (int t = 0; t < sh->nthreads; t++) {
                occvec *o = &sh->w[t].out[p];
                for (uint64_t i = 0; i < o->n; i++)
                    if (otable_add(&sh->tables[p], o->v[i].key, o->v[i].mask)) w->failed = 1;
            }
        }
        pthread_barrier_wait(&sh->bar);
        /* phase 3: clear my own buffers for the next batch */
        for (int p = 0; p < sh->nparts; p++) w->out[p].n = 0;
    }
    return NULL;
}

static int online_cores(void) {
    long n = sysconf(_SC_NPROCESSORS_ONLN);
    return n > 0 ? (int)n : 1;
}

/* LSD radix sort of (key, 8-byte counts) pairs by key. */
static int sort_pairs(uint64_t *keys, uint64_t *cnt, uint64_t n) {
    if (n < 2) return 0;
    uint64_t *k2 = (uint64_t *)malloc(n * sizeof(uint64_t));
    uint64_t *c2 = (uint64_t *)malloc(n * sizeof(uint64_t));
    uint64_t *hist = (uint64_t *)malloc(65536 * sizeof(uint64_t));
    if (!k2 || !c2 || !hist) { free(k2); free(c2); free(hist); return -1; }
    for (int pass = 0; pass < 4; pass++) {
        int sh = 16 * pass;
        memset(hist, 0, 65536 * sizeof(uint64_t));
        for (uint64_t i = 0; i < n; i++) hist[(keys[i] >> sh) & 0xffff]++;
        uint64_t s = 0;
        for (int d = 0; d < 65536; d++) { uint64_t h = hist[d]; hist[d] = s; s += h; }
        for (uint64_t i = 0; i < n; i++) {
            uint64_t pos = hist[(keys[i] >> sh) & 0xffff]++;
            k2[pos] = keys[i];
            c2[pos] = cnt[i];
        }
        memcpy(keys, k2, n * sizeof(uint64_t));
        memcpy(cnt, c2, n * sizeof(uint64_t));
    }
    free(k2); free(c2); free(hist);
    return 0;
}

/* A7: cutoff (graph.cpp:1092-1114). multiplicity < threshold -> 0 (the
 * comparison is int against the uint8 value, 1105); the key survives iff some
 * slot is nonzero (1106-1108). */
static uint64_t apply_cutoff_counts(uint64_t v, int cutoff) {
    uint64_t out = 0;
    for (int s = 0; s < 8; s++) {
        int b = (int)((v >> (8 * s)) & 0xff);
        if (b < cutoff) b = 0;
        out |= (uint64_t)b << (8 * s);
    }
    return out;
}

oracle_graph *oracle_build(const oracle_reads *r, int k, int cutoff, int apply_cutoff, int threads) {
    if (k < 1 || k > 31) return NULL;
    int nt = threads > 0 ? threads : online_cores();
    if (nt > 256) nt = 256;
    shared_t sh;
    memset(&sh, 0, sizeof(sh));
    sh.r = r;
    sh.k = k;
    sh.nthreads = nt;
    sh.nparts = nt * 4;
    sh.w = (worker_t *)calloc((size_t)nt, sizeof(worker_t));
    sh.tables = (otable *)calloc((size_t)sh.nparts, sizeof(otable));
    pthread_t *tids = (pthread_t *)calloc((size_t)nt, sizeof(pthread_t));
    int fail = (!sh.w || !sh.tables || !tids);
    for (int p = 0; !fail && p < sh.nparts; p++) fail |= otable_init(&sh.tables[p], 1024) != 0;
    for (int t = 0; !fail && t < nt; t++) {
        sh.w[t].sh = &sh;
        sh.w[t].tid = t;
        sh.w[t].out = (occvec *)calloc((size_t)sh.nparts, sizeof(occvec));
        fail |= sh.w[t].out == NULL;
    }
    oracle_graph *g = NULL;
    if (!fail) {
        pthread_barrier_init(&sh.bar, NULL, (unsigned)nt + 1);
        for (int t = 0; t < nt; t++) pthread_create(&tids[t], NULL, worker_main, &sh.w[t]);
        /* batches of about 32M k-mer occurrences bound the routing buffers */
        uint64_t i = 0;
        while (i < r->n_reads) {
            uint64_t j = i, occ = 0;
            while (j < r->n_reads && occ < (32ull << 20)) { occ += r->len[j] - (uint64_t)k + 1; j++; }
            sh.batch_begin = i;
            sh.batch_end = j;
            pthread_barrier_wait(&sh.bar); /* start */
            pthread_barrier_wait(&sh.bar); /* phase 1 done */
            pthread_barrier_wait(&sh.bar); /* phase 2 done */
            i = j;
        }
        sh.done = 1;
        pthread_barrier_wait(&sh.bar);
        for (int t = 0; t < nt; t++) pthread_join(tids[t], NULL);
        pthread_barrier_destroy(&sh.bar);
        for (int t = 0; t < nt; t++) fail |= sh.w[t].failed;
    }
    if (!fail) {
        uint64_t total = 0;
        for (int p = 0; p < sh.nparts; p++) total += sh.tables[p].n;
        g = (oracle_graph *)calloc(1, sizeof(oracle_graph));
        uint64_t *keys = (uint64_t *)malloc((total ? total : 1) * sizeof(uint64_t));
        uint64_t *cnt = (uint64_t *)malloc((total ? total : 1) * sizeof(uint64_t));
        if (!g || !keys || !cnt) {
            free(g); free(keys); free(cnt);
            g = NULL;
        } else {
            uint64_t n = 0;
            for (int p = 0; p < sh.nparts; p++) {
                otable *t = &sh.tables[p];
                for (uint64_t s = 0; s < t->cap; s++) {
                    if (t->keys[s] == EMPTY_KEY) continue;
                    uint64_t v = t->cnt[s];
                    if (apply_cutoff) {
                        v = apply_cutoff_counts(v, cutoff);
                        if (v == 0) continue;
                    }
                    keys[n] = t->keys[s];
                    cnt[n] = v;
                    n++;
                }
            }
            if (sort_pairs(keys, cnt, n)) {
                free(g); free(keys); free(cnt);
                g = NULL;
            } else {
                g->n = n;
                g->keys = keys;
                g->mult = (uint8_t *)malloc((n ? n : 1) * 8);
                for (uint64_t q = 0; q < n; q++)
                    for (int s = 0; s < 8; s++) g->mult[q * 8 + s] = (uint8_t)(cnt[q] >> (8 * s));
                free(cnt);
            }
        }
    }
    for (int t = 0; sh.w && t < nt; t++) {
        if (!sh.w[t].out) continue;
        for (int p = 0; p < sh.nparts; p++) free(sh.w[t].out[p].v);
        free(sh.w[t].out);
    }
    for (int p = 0; sh.tables && p < sh.nparts; p++) otable_free(&sh.tables[p]);
    free(sh.w);
    free(sh.tables);
    free(tids);
    return g;
}

oracle_graph *oracle_build_fasta(const char *buf, uint64_t len, int k, int cutoff, int threads,
                                 int *err) {
    oracle_reads r;
    int e = oracle_parse_fasta(buf, len, k, &r);
    if (err) *err = e;
    if (e != ORACLE_OK) return NULL;
    oracle_graph *g = oracle_build(&r, k, cutoff, 1, threads);
    oracle_reads_free(&r);
    if (!g && err) *err = ORACLE_ERR_OOM;
    return g;
}

uint64_t oracle_graph_size(const oracle_graph *g) { return g ? g->n : 0; }

void oracle_graph_get(const oracle_graph *g, uint64_t *keys, uint8_t *mult) {
    if (!g) return;
    if (keys) memcpy(keys, g->keys, g->n * sizeof(uint64_t));
    if (mult) memcpy(mult, g->mult, g->n * 8);
}

void oracle_graph_free(oracle_graph *g) {
    if (!g) return;
    free(g->keys);
    free(g->mult);
    free(g);
}

/* ------------------------------------------------------------------ */
/* A9: kmerGraph.txt (graph.cpp:3352-3440, node::getNodeID 164-196).   */
/* ------------------------------------------------------------------ */

/* getNodeID(s): descriptor = K (s < 4) or rc(K) (s >= 4) plus the arc base
 * "ACGT"[s%4]; N = its last k bases (177-181). If N >= rc(N) the id is N
 * (ret 1). Otherwise the id is rc(N) (ret -1, 187-191) and printKmerGraph
 * tries to reverse-complement it back, but its loop complements
 * nReverseStr[i] (i = the slot) instead of [j] (3393, 3423): the printed id is
 * reverse(string(rc(N))) = complement(N), with base i complemented k times.
 * k is odd (sequence.cpp:44), so base i ends as N's own base there. */
uint64_t oracle_kmer_graph_neighbour(uint64_t key, int slot, int k) {
    const uint64_t kmask = (1ull << (2 * k)) - 1;
    uint64_t d = slot < 4 ? key : oracle_revcomp(key, k);
    uint64_t n = ((d << 2) | (uint64_t)(slot & 3)) & kmask;
    uint64_t rn = oracle_revcomp(n, k);
    if (n >= rn) return n;
    /* string position i holds the base at bit offset 2*(k-1-i) */
    uint64_t out = n ^ kmask;
    if (k & 1) out ^= 3ull << (2 * (k - 1 - slot));
    return out;
}

typedef struct {
    uint64_t first;
    char *text;
} line_t;

static int line_cmp(const void *a, const void *b) {
    uint64_t x = ((const line_t *)a)->first, y = ((const line_t *)b)->first;
    return x < y ? -1 : (x > y ? 1 : 0);
}

/* Each node gives up to two lines: "K n.." over slots 0-3, then
 * "rc(K) n.." over slots 4-7 (3401-3437); hash-map order in the reference,
 * sorted by first token here. */
int oracle_write_kmer_graph(const oracle_graph *g, int k, const char *path) {
    FILE *fp = fopen(path, "w");
    if (!fp) return -1;
    line_t *lines = (line_t *)malloc((g->n * 2 + 1) * sizeof(line_t));
    uint64_t nl = 0;
    char tmp[256];
    for (uint64_t i = 0; i < g->n; i++) {
        uint64_t key = g->keys[i];
        const uint8_t *m = g->mult + 8 * i;
        for (int half = 0; half < 2; half++) {
            int any = 0;
            int pos = snprintf(tmp, sizeof(tmp), "%llu",
                               (unsigned long long)(half ? oracle_revcomp(key, k) : key));
            for (int s = 4 * half; s < 4 * half + 4; s++) {
                if (!m[s]) continue;
                any = 1;
                pos += snprintf(tmp + pos, sizeof(tmp) - (size_t)pos, " %llu",
                                (unsigned long long)oracle_kmer_graph_neighbour(key, s, k));
            }
            if (!any) continue;
            lines[nl].first = half ? oracle_revcomp(key, k) : key;
            lines[nl].text = strdup(tmp);
            nl++;
        }
    }
    qsort(lines, nl, sizeof(line_t), line_cmp);
    for (uint64_t i = 0; i < nl; i++) {
        fputs(lines[i].text, fp);
        fputc('\n', fp);
        free(lines[i].text);
    }
    free(lines);
    fclose(fp);
    return 0;
}

/* A10: printLocalNodeGraph (graph.cpp:569) — key, the 8 arc strings each
 * followed by '#' (arc = "ACGT"[s%4] iff multiplicity != 0, node::init
 * graph.cpp:88-96), then the 8 multiplicities. Sorted by key here. */
int oracle_write_node_lines(const oracle_graph *g, const char *path) {
    FILE *fp = fopen(path, "w");
    if (!fp) return -1;
    static const char acgt[4] = {'A', 'C', 'G', 'T'};
    for (uint64_t i = 0; i < g->n; i++) {
        const uint8_t *m = g->mult + 8 * i;
        fprintf(fp, "%llu", (unsigned long long)g->keys[i]);
        for (int s = 0; s < 8; s++) {
            if (m[s]) fprintf(fp, " %c#", acgt[s & 3]);
            else fputs(" #", fp);
        }
        for (int s = 0; s < 8; s++) fprintf(fp, " %d", m[s]);
        fputc('\n', fp);
    }
    fclose(fp);
    return 0;
}

/* graph.cpp:1579-1608 over the built nodes (every arc string has length 1). */
void oracle_graph_stats(const oracle_graph *g, int k, int64_t out[5]) {
    int64_t nodes = 0, edges = 0, tips = 0, bubbles = 0;
    for (uint64_t i = 0; i < g->n; i++) {
        const uint8_t *m = g->mult + 8 * i;
        nodes++;
        int local = 0, maxm = -1, minm = 1000000;
        for (int s = 0; s < 8; s++) {
            if (!m[s]) continue;
            edges++;
            local++;
            if (m[s] > maxm) maxm = m[s];
            if (m[s] < minm) minm = m[s];
        }
        if (local == 1 && 1 < k) tips++;
        /* arcs[minIndex].length() < 2k holds for every one-base arc */
        if (minm < 0.2 * maxm) bubbles++;
    }
    out[0] = nodes;
    out[1] = edges;
    out[2] = edges;
    out[3] = tips;
    out[4] = bubbles;
}
