/*
 * merge_oracle — CPU restatement of SWAP-Assembler's merging of
 * semi-extended k-molecules.
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker for the GPU merge. Only the
 * tests, the smoke check and the CPU-baseline leg of the benchmark load it.
 *
 * Restated (files of the reference project):
 *   node arcs / multiplicities          graph.cpp:42-102 (node, node::init)
 *   getLeftNodeID / getRightNodeID      graph.cpp:228-248
 *   getNodeID (arc end point)           graph.cpp:164-196
 *   getSrcNodeEdge (arc back to src)    graph.cpp:250-309, called with
 *                                       direction 2, no edge/multiplicity filter
 *   getLeftEdge / getRightEdge          graph.cpp:135-161
 *   merge loop                          graph.cpp:1392-1566 (simplifyDistNodeGraph)
 *   lock / unlock / edge messages       graph.cpp:1204-1389 (recvProc)
 *   gathered node lines                 graph.cpp:576-696 (gatherDistNodeGraph),
 *                                       written as by graph.cpp:3617-3621
 *
 * The merge visits the nodes in a given order. At one rank the reference
 * visits them in its node map's iteration order, and its messages to itself
 * are handled lazily: a merge's two edge messages (and an unlock message)
 * are applied only when the next node that reaches a lock exchange services
 * its queue, so the neighbours of the last merge stay locked until then, and
 * the messages of the very last merge are never applied (the final barrier
 * completes at once at one rank). MERGE_TIMING_REFERENCE reproduces that;
 * MERGE_TIMING_IMMEDIATE applies every message at once, which is the merge
 * the GPU implements.
 *
 * Multiplicity arithmetic follows graph.cpp:1322-1324 exactly: the weighted
 * sum is formed in 64 bits, stored in an int (low 32 bits), widened back to
 * 64 bits for the division by the new arc length, and truncated to 8 bits.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "kmer_oracle.h"

typedef struct {
    uint8_t *s; /* base codes 0..3 */
    uint32_t len, cap;
} mstr;

typedef struct {
    int type; /* 4 = edge, 3 = unlock */
    uint64_t dst, src;
    int side;
    uint8_t *str;
    uint32_t len;
    uint8_t mult;
} mmsg;

typedef struct {
    int k;
    uint64_t n;
    const uint64_t *keys;
    uint8_t (*mult)[8];
    mstr (*arcs)[8];
    uint8_t *deleted, *locked;
    uint64_t hcap;
    uint64_t *hk;
    int64_t *hv;
    mmsg *q;
    uint64_t qn, qcap;
    int err;
} mgraph;

static uint64_t mmix(uint64_t x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33;
    return x;
}

static int64_t mfind(const mgraph *g, uint64_t key) {
    uint64_t h = mmix(key) & (g->hcap - 1);
    for (;;) {
        if (g->hv[h] < 0) return -1;
        if (g->hk[h] == key) return g->hv[h];
        h = (h + 1) & (g->hcap - 1);
    }
}

static int mstr_append(mstr *a, const uint8_t *s, uint32_t len) {
    if (a->len + len > a->cap) {
        uint32_t c = a->cap ? a->cap : 4;
        while (c < a->len + len) c *= 2;
        uint8_t *p = (uint8_t *)realloc(a->s, c);
        if (!p) return -1;
        a->s = p;
        a->cap = c;
    }
    memcpy(a->s + a->len, s, len);
    a->len += len;
    return 0;
}

/* End point of arc `slot` of node x: the last k bases of the oriented
 * k-mer followed by the arc string, as a canonical id plus the side it is
 * reached on (1: the id itself, 0: its reverse complement) — graph.cpp:164-196
 * and 270-293. An empty arc ends at the node itself. */
static void arc_end(const mgraph *g, uint64_t x, int slot, uint64_t *id, int *side) {
    const int k = g->k;
    const uint64_t mask = (k == 32) ? ~0ULL : ((1ULL << (2 * k)) - 1);
    uint64_t v = slot < 4 ? g->keys[x] : oracle_revcomp(g->keys[x], k);
    const mstr *a = &g->arcs[x][slot];
    uint32_t from = a->len > (uint32_t)k ? a->len - (uint32_t)k : 0;
    for (uint32_t i = from; i < a->len; ++i) v = ((v << 2) | a->s[i]) & mask;
    uint64_t r = oracle_revcomp(v, k);
    if (v < r) {
        *id = r;
        *side = 0;
    } else {
        *id = v;
        *side = 1;
    }
}

static int src_edge(const mgraph *g, uint64_t dst, uint64_t src, int side) {
    for (int i = 0; i < 8; ++i) {
        uint64_t id;
        int sd;
        arc_end(g, dst, i, &id, &sd);
        if (id == g->keys[src] && sd == side) return i;
    }
    return -1;
}

static void apply(mgraph *g, const mmsg *m) {
    if (m->type == 3) {
        if (!g->locked[m->dst]) g->err = -12; /* graph.cpp:1282-1287 exits */
        g->locked[m->dst] = 0;
        return;
    }
    int i = src_edge(g, m->dst, m->src, m->side);
    if (i < 0) {
        g->err = -11; /* graph.cpp:1333-1343 asserts */
        return;
    }
    mstr *a = &g->arcs[m->dst][i];
    if (m->len) {
        uint64_t sum = (uint64_t)g->mult[m->dst][i] * a->len + (uint64_t)m->mult * m->len;
        int32_t pre = (int32_t)(uint32_t)sum;
        if (mstr_append(a, m->str, m->len)) {
            g->err = ORACLE_ERR_OOM;
            return;
        }
        g->mult[m->dst][i] = (uint8_t)((uint64_t)(int64_t)pre / a->len);
    } else {
        g->mult[m->dst][i] = 0;
        a->len = 0;
    }
    g->locked[m->dst] = 0;
}

static void push(mgraph *g, int type, uint64_t dst, uint64_t src, int side, const mstr *s, uint8_t mult) {
    if (g->qn == g->qcap) {
        uint64_t c = g->qcap ? 2 * g->qcap : 16;
        mmsg *p = (mmsg *)realloc(g->q, c * sizeof(mmsg));
        if (!p) {
            g->err = ORACLE_ERR_OOM;
            return;
        }
        g->q = p;
        g->qcap = c;
    }
    mmsg *m = &g->q[g->qn++];
    memset(m, 0, sizeof(*m));
    m->type = type;
    m->dst = dst;
    m->src = src;
    m->side = side;
    m->mult = mult;
    if (s && s->len) {
        m->str = (uint8_t *)malloc(s->len); /* the send copies the string as it is now */
        if (!m->str) {
            g->err = ORACLE_ERR_OOM;
            return;
        }
        memcpy(m->str, s->s, s->len);
        m->len = s->len;
    }
}

static void drain(mgraph *g) {
    for (uint64_t i = 0; i < g->qn && !g->err; ++i) apply(g, &g->q[i]);
    for (uint64_t i = 0; i < g->qn; ++i) free(g->q[i].str);
    g->qn = 0;
}

static void one_sided(const mgraph *g, uint64_t x, int *lslot, int *rslot, int *lc, int *rc) {
    *lc = *rc = 0;
    *lslot = *rslot = -1;
    for (int i = 0; i < 4; ++i)
        if (g->arcs[x][i].len) *rslot = i, ++*rc;
    for (int i = 4; i < 8; ++i)
        if (g->arcs[x][i].len) *lslot = i, ++*lc;
}

static void simplify(mgraph *g, const uint64_t *order, int timing) {
    for (uint64_t t = 0; t < g->n && !g->err; ++t) {
        const uint64_t x = order[t];
        if (g->deleted[x]) continue;
        if (g->locked[x]) continue; /* locked by a neighbour's pending merge */
        g->locked[x] = 1;
        int ls, rs, lc, rc;
        one_sided(g, x, &ls, &rs, &lc, &rc);
        if (lc != 1 || rc != 1) {
            g->locked[x] = 0;
            continue;
        }
        uint64_t lid, rid;
        int lsd, rsd;
        arc_end(g, x, ls, &lid, &lsd);
        arc_end(g, x, rs, &rid, &rsd);
        int64_t li = mfind(g, lid), ri = mfind(g, rid);
        if (li < 0 || ri < 0) {
            g->err = -10; /* graph.cpp:1270-1274 exits */
            return;
        }
        drain(g); /* the lock exchange services the queue first */
        int lres = g->locked[li] ? 2 : (g->locked[li] = 1, 1);
        int rres;
        if (ri != li)
            rres = g->locked[ri] ? 2 : (g->locked[ri] = 1, 1);
        else
            rres = lres;
        if (lres == 1 && rres == 1) {
            push(g, 4, (uint64_t)ri, x, 0, &g->arcs[x][ls], g->mult[x][ls]);
            push(g, 4, (uint64_t)li, x, 1, &g->arcs[x][rs], g->mult[x][rs]);
            g->deleted[x] = 1;
        } else if (lres == 1 || rres == 1) {
            push(g, 3, lres == 1 ? (uint64_t)li : (uint64_t)ri, x, 0, NULL, 0);
        }
        if (timing == MERGE_TIMING_IMMEDIATE) drain(g);
        g->locked[x] = 0;
    }
    /* MERGE_TIMING_REFERENCE: whatever is still queued is never applied */
    for (uint64_t i = 0; i < g->qn; ++i) free(g->q[i].str);
    g->qn = 0;
}

/* One gathered node line (graph.cpp:615-645): id, 8 arcs each closed by '#',
 * 8 multiplicities, padded with blanks to sum(len+1)+61 bytes, '\n' last. */
static char *put_line(char *p, const mgraph *g, uint64_t x) {
    static const char acgt[4] = {'A', 'C', 'G', 'T'};
    uint64_t vlen = 61;
    for (int i = 0; i < 8; ++i) vlen += g->arcs[x][i].len + 1;
    char *start = p;
    p += sprintf(p, "%llu", (unsigned long long)g->keys[x]);
    for (int i = 0; i < 8; ++i) {
        *p++ = ' ';
        for (uint32_t j = 0; j < g->arcs[x][i].len; ++j) *p++ = acgt[g->arcs[x][i].s[j]];
        *p++ = '#';
    }
    for (int i = 0; i < 8; ++i) p += sprintf(p, " %d", g->mult[x][i]);
    while ((uint64_t)(p - start) < vlen - 1) *p++ = ' ';
    *p++ = '\n';
    return p;
}

static int has_arc(const mgraph *g, uint64_t x) {
    for (int i = 0; i < 8; ++i)
        if (g->arcs[x][i].len) return 1;
    return 0;
}

static int mgraph_init(mgraph *g, int k, uint64_t n, const uint64_t *keys, const uint8_t *mult) {
    memset(g, 0, sizeof(*g));
    g->k = k;
    g->n = n;
    g->keys = keys;
    g->mult = (uint8_t(*)[8])calloc(n ? n : 1, 8);
    g->arcs = (mstr(*)[8])calloc(n ? n : 1, sizeof(mstr[8]));
    g->deleted = (uint8_t *)calloc(n ? n : 1, 1);
    g->locked = (uint8_t *)calloc(n ? n : 1, 1);
    g->hcap = 16;
    while (g->hcap < 2 * n) g->hcap *= 2;
    g->hk = (uint64_t *)malloc(g->hcap * sizeof(uint64_t));
    g->hv = (int64_t *)malloc(g->hcap * sizeof(int64_t));
    if (!g->mult || !g->arcs || !g->deleted || !g->locked || !g->hk || !g->hv) return ORACLE_ERR_OOM;
    for (uint64_t h = 0; h < g->hcap; ++h) g->hv[h] = -1;
    for (uint64_t x = 0; x < n; ++x) {
        uint64_t h = mmix(keys[x]) & (g->hcap - 1);
        while (g->hv[h] >= 0) h = (h + 1) & (g->hcap - 1);
        g->hk[h] = keys[x];
        g->hv[h] = (int64_t)x;
        for (int i = 0; i < 8; ++i) {
            g->mult[x][i] = mult[8 * x + i];
            if (mult[8 * x + i]) { /* node::init: arc = the slot's base */
                uint8_t b = (uint8_t)(i & 3);
                if (mstr_append(&g->arcs[x][i], &b, 1)) return ORACLE_ERR_OOM;
            }
        }
    }
    return 0;
}

static void mgraph_free(mgraph *g) {
    if (g->arcs)
        for (uint64_t x = 0; x < g->n; ++x)
            for (int i = 0; i < 8; ++i) free(g->arcs[x][i].s);
    free(g->arcs);
    free(g->mult);
    free(g->deleted);
    free(g->locked);
    free(g->hk);
    free(g->hv);
    free(g->q);
}

int oracle_merge(int k, uint64_t n, const uint64_t *keys, const uint8_t *mult, const uint64_t *order,
                 int timing, char **text, uint64_t *text_len, uint64_t *n_lines) {
    *text = NULL;
    *text_len = 0;
    if (n_lines) *n_lines = 0;
    if (k < 1 || k > 31) return ORACLE_ERR_BAD_K;
    mgraph g;
    int rc = mgraph_init(&g, k, n, keys, mult);
    if (!rc) {
        simplify(&g, order, timing);
        rc = g.err;
    }
    if (!rc) {
        uint64_t total = 2, lines = 0;
        for (uint64_t x = 0; x < n; ++x) {
            if (g.deleted[x] || !has_arc(&g, x)) continue;
            total += 61;
            for (int i = 0; i < 8; ++i) total += g.arcs[x][i].len + 1;
            ++lines;
        }
        char *buf = (char *)malloc(total + 64);
        if (!buf) {
            rc = ORACLE_ERR_OOM;
        } else {
            char *p = buf;
            for (uint64_t t = 0; t < n; ++t) { /* gathered in visiting order */
                uint64_t x = order[t];
                if (g.deleted[x] || !has_arc(&g, x)) continue;
                p = put_line(p, &g, x);
            }
            *p++ = '\n'; /* fprintf(fp, "%s\n", rBuf) */
            *text = buf;
            *text_len = (uint64_t)(p - buf);
            if (n_lines) *n_lines = lines;
        }
    }
    mgraph_free(&g);
    return rc;
}

void oracle_free_text(char *text) { free(text); }

/* ---------------------------------------------------------------------------
 * The visiting order the GPU merge follows. A node is mergeable when it has
 * exactly one arc on each side and neither arc leads back to itself; every
 * other node ends chains. Each chain is numbered from its smaller end arc
 * (end node key, then slot); its interior node at position p (1..m) is
 * visited at level ctz(p), levels in increasing order, so each level merges
 * disjoint pairs of neighbouring segments. A cycle made only of mergeable
 * nodes is cut at its largest key, which is visited after everything else
 * and is left holding the whole cycle on its two arcs.
 * ------------------------------------------------------------------------- */

typedef struct {
    uint64_t level, ckey, cslot, pos, node;
} tord;

static int tord_cmp(const void *a, const void *b) {
    const tord *x = (const tord *)a, *y = (const tord *)b;
    if (x->level != y->level) return x->level < y->level ? -1 : 1;
    if (x->ckey != y->ckey) return x->ckey < y->ckey ? -1 : 1;
    if (x->cslot != y->cslot) return x->cslot < y->cslot ? -1 : 1;
    if (x->pos != y->pos) return x->pos < y->pos ? -1 : 1;
    return 0;
}

/* Step along arc `slot` of node x: the neighbour index, and the slot of the
 * neighbour that continues in the same direction when the neighbour has one
 * arc per side (-1 when it does not). */
static int64_t step(const mgraph *g, uint64_t x, int slot, int *arrive_side) {
    uint64_t id;
    int side;
    arc_end(g, x, slot, &id, &side);
    *arrive_side = side;
    return mfind(g, id);
}

static int ctz64(uint64_t v) {
    int c = 0;
    while (!(v & 1)) v >>= 1, ++c;
    return c;
}

int oracle_merge_tree_order(int k, uint64_t n, const uint64_t *keys, const uint8_t *mult, uint64_t *order) {
    if (k < 1 || k > 31) return ORACLE_ERR_BAD_K;
    mgraph g;
    int rc = mgraph_init(&g, k, n, keys, mult);
    uint8_t *mg = (uint8_t *)calloc(n ? n : 1, 1);
    int8_t *ls = (int8_t *)malloc(n ? n : 1), *rs = (int8_t *)malloc(n ? n : 1);
    tord *to = (tord *)malloc((n ? n : 1) * sizeof(tord));
    uint8_t *seen = (uint8_t *)calloc(n ? n : 1, 1);
    if (!mg || !ls || !rs || !to || !seen) rc = ORACLE_ERR_OOM;
    for (uint64_t x = 0; !rc && x < n; ++x) {
        int l, r, lc, rcnt;
        one_sided(&g, x, &l, &r, &lc, &rcnt);
        ls[x] = (int8_t)l;
        rs[x] = (int8_t)r;
        if (lc == 1 && rcnt == 1) {
            int s1, s2;
            int64_t a = step(&g, x, l, &s1), b = step(&g, x, r, &s2);
            if (a < 0 || b < 0) rc = -10;
            else mg[x] = ((uint64_t)a != x && (uint64_t)b != x);
        }
    }
    uint64_t nt = 0, ncyc = 0;
    uint64_t *cyc = (uint64_t *)malloc((n ? n : 1) * sizeof(uint64_t));
    if (!cyc) rc = ORACLE_ERR_OOM;
    /* Walk one chain from end arc (x, slot); fill positions when `fill`. */
    for (int pass = 0; !rc && pass < 2; ++pass) {
        for (uint64_t x = 0; !rc && x < n; ++x) {
            if (pass == 0 && mg[x]) continue;          /* chains start at end nodes */
            if (pass == 1 && (!mg[x] || seen[x])) continue; /* leftover: cycles */
            uint64_t start = x;
            if (pass == 1) { /* find the cycle's largest key, cut there */
                uint64_t best = x, cur = x;
                int dslot = rs[x];
                for (;;) {
                    int side;
                    int64_t y = step(&g, cur, dslot, &side);
                    if ((uint64_t)y == x) break;
                    if (keys[y] > keys[best]) best = (uint64_t)y;
                    dslot = side ? rs[y] : ls[y];
                    cur = (uint64_t)y;
                }
                start = best;
                mg[start] = 0;
                seen[start] = 1;
                cyc[ncyc++] = start;
            }
            for (int slot = 0; slot < 8 && !rc; ++slot) {
                if (!g.arcs[start][slot].len) continue;
                /* walk to the other end, then number from the smaller end arc */
                int side;
                int64_t y = step(&g, start, slot, &side);
                if (y < 0) { rc = -10; break; }
                if (!mg[y]) continue;
                uint64_t m = 0, cur = (uint64_t)y;
                int dir = side; /* 1: leave through the right arc */
                uint64_t ekey = 0, eslot = 0;
                for (;;) {
                    ++m;
                    int out = dir ? rs[cur] : ls[cur];
                    int s2;
                    int64_t z = step(&g, cur, out, &s2);
                    if (!mg[z]) {
                        /* the end arc pointing back: side of arrival and the
                         * first base of the oriented k-mer we left */
                        uint64_t ok = dir ? keys[cur] : oracle_revcomp(keys[cur], k);
                        int first = (int)((ok >> (2 * (k - 1))) & 3);
                        ekey = keys[z];
                        eslot = (uint64_t)((s2 ? 4 : 0) + 3 - first);
                        break;
                    }
                    dir = s2;
                    cur = (uint64_t)z;
                }
                int fwd = keys[start] < ekey || (keys[start] == ekey && (uint64_t)slot < eslot);
                if (!fwd) continue; /* numbered from the other end */
                cur = (uint64_t)y;
                dir = side;
                for (uint64_t p = 1; p <= m; ++p) {
                    to[nt].level = (uint64_t)ctz64(p);
                    to[nt].ckey = keys[start];
                    to[nt].cslot = (uint64_t)slot;
                    to[nt].pos = p;
                    to[nt].node = cur;
                    ++nt;
                    seen[cur] = 1;
                    int out = dir ? rs[cur] : ls[cur];
                    int s2;
                    int64_t z = step(&g, cur, out, &s2);
                    dir = s2;
                    cur = (uint64_t)z;
                }
            }
        }
    }
    if (!rc) {
        qsort(to, nt, sizeof(tord), tord_cmp);
        uint64_t o = 0;
        for (uint64_t x = 0; x < n; ++x)
            if (!mg[x] && !seen[x]) order[o++] = x; /* ends: never merged */
        for (uint64_t i = 0; i < nt; ++i) order[o++] = to[i].node;
        for (uint64_t i = 0; i < ncyc; ++i) order[o++] = cyc[i];
        if (o != n) rc = -13;
    }
    free(cyc);
    free(mg);
    free(ls);
    free(rs);
    free(to);
    free(seen);
    mgraph_free(&g);
    return rc;
}

/* ---------------------------------------------------------------------------
 * Two of the reference's rank-0 passes over a merged graph, restated:
 *   masterTipsRemoval            graph.cpp:2194-2265 (one pass)
 *   masterLowCoverageEdgeRemoval graph.cpp:2267-2300
 * The graph comes as gathered node lines (the -d file, parsed as
 * recvBufDistNodeGraph does, graph.cpp:845-896); nodes are visited in a
 * given order of its lines, and the result is written as gathered lines in
 * that order (deleted and arc-less nodes skipped, graph.cpp:587-596).
 * ------------------------------------------------------------------------- */

static int parse_lines(mgraph *g, int k, const char *text, uint64_t len, uint64_t **keys_out) {
    static const int8_t code[256] = {['A'] = 1, ['C'] = 2, ['G'] = 3, ['T'] = 4};
    uint64_t cap = 1024, n = 0;
    uint64_t *keys = (uint64_t *)malloc(cap * 8);
    uint8_t(*mult)[8] = (uint8_t(*)[8])malloc(cap * 8);
    mstr(*arcs)[8] = (mstr(*)[8])calloc(cap, sizeof(mstr[8]));
    const char *p = text, *end = text + len;
    int rc = 0;
    while (!rc && p < end) {
        while (p < end && (*p == '\n' || *p == ' ')) ++p;
        if (p >= end || *p == 0) break;
        if (n == cap) {
            cap *= 2;
            keys = (uint64_t *)realloc(keys, cap * 8);
            mult = (uint8_t(*)[8])realloc(mult, cap * 8);
            arcs = (mstr(*)[8])realloc(arcs, cap * sizeof(mstr[8]));
            memset(arcs + n, 0, (cap - n) * sizeof(mstr[8]));
        }
        uint64_t id = 0;
        while (p < end && *p >= '0' && *p <= '9') id = id * 10 + (uint64_t)(*p++ - '0');
        while (p < end && *p == ' ') ++p;
        for (int i = 0; i < 8 && !rc; ++i) {
            const char *e = p;
            while (e < end && *e != '#') ++e;
            if (e >= end) {
                rc = ORACLE_ERR_NO_RECORD;
                break;
            }
            for (const char *q = p; q < e; ++q) {
                uint8_t b = (uint8_t)(code[(unsigned char)*q] - 1);
                if (mstr_append(&arcs[n][i], &b, 1)) rc = ORACLE_ERR_OOM;
            }
            p = e + 2; /* '#' and the blank after it */
        }
        for (int i = 0; i < 8 && !rc; ++i) {
            int v = 0;
            while (p < end && *p >= '0' && *p <= '9') v = v * 10 + (*p++ - '0');
            mult[n][i] = (uint8_t)v;
            while (p < end && *p == ' ') ++p;
        }
        keys[n++] = id;
        while (p < end && *p == '\n') ++p;
    }
    memset(g, 0, sizeof(*g));
    g->k = k;
    g->n = n;
    g->keys = keys;
    g->mult = mult;
    g->arcs = arcs;
    g->deleted = (uint8_t *)calloc(n ? n : 1, 1);
    g->locked = (uint8_t *)calloc(n ? n : 1, 1);
    g->hcap = 16;
    while (g->hcap < 2 * n) g->hcap *= 2;
    g->hk = (uint64_t *)malloc(g->hcap * 8);
    g->hv = (int64_t *)malloc(g->hcap * 8);
    for (uint64_t h = 0; h < g->hcap; ++h) g->hv[h] = -1;
    for (uint64_t x = 0; x < n; ++x) {
        uint64_t h = mmix(keys[x]) & (g->hcap - 1);
        while (g->hv[h] >= 0) h = (h + 1) & (g->hcap - 1);
        g->hk[h] = keys[x];
        g->hv[h] = (int64_t)x;
    }
    *keys_out = keys;
    return rc;
}

static void tips_pass(mgraph *g, const uint64_t *order, uint64_t *removed) {
    for (uint64_t t = 0; t < g->n; ++t) {
        const uint64_t x = order[t];
        if (g->deleted[x]) continue;
        int num = 0, index = -1;
        for (int i = 0; i < 8; ++i)
            if (g->arcs[x][i].len) ++num, index = i;
        if (num != 1 || g->arcs[x][index].len >= (uint32_t)g->k) continue;
        uint64_t id;
        int side;
        arc_end(g, x, index, &id, &side);
        const int64_t nx = mfind(g, id);
        const int ret = nx < 0 ? -1 : src_edge(g, (uint64_t)nx, x, index < 4 ? 0 : 1);
        if (ret < 0) { /* no arc back: only the tip's own arc goes */
            g->mult[x][index] = 0;
            g->arcs[x][index].len = 0;
            continue;
        }
        if ((uint64_t)nx == x) continue;
        g->mult[nx][ret] = 0;
        g->arcs[nx][ret].len = 0;
        g->mult[x][index] = 0;
        g->arcs[x][index].len = 0;
        g->deleted[x] = 1;
        if (removed) ++*removed;
    }
}

static void low_coverage_pass(mgraph *g, const uint64_t *order, uint64_t *cleared) {
    uint64_t cov = 0, nuc = 0;
    for (uint64_t x = 0; x < g->n; ++x) {
        if (g->deleted[x]) continue;
        for (int i = 0; i < 8; ++i) {
            nuc += g->arcs[x][i].len;
            cov += (uint64_t)g->arcs[x][i].len * g->mult[x][i];
        }
    }
    /* the reference divides by zero when no arc is left; here nothing is cut */
    const uint64_t avg = nuc ? cov / nuc : 0;
    for (uint64_t t = 0; t < g->n; ++t) {
        const uint64_t x = order[t];
        if (g->deleted[x]) continue;
        for (int i = 0; i < 8; ++i) {
            /* multiplicity < 0.25 * avgCoverage, exactly: 4 * m < avg */
            if (g->arcs[x][i].len < 2u * (uint32_t)g->k && 4ull * g->mult[x][i] < avg) {
                if (g->arcs[x][i].len && cleared) ++*cleared;
                g->arcs[x][i].len = 0;
                g->mult[x][i] = 0;
            }
        }
    }
}

int oracle_prune(int k, const char *text, uint64_t len, const uint64_t *order, int passes, char **out,
                 uint64_t *out_len, uint64_t *count) {
    *out = NULL;
    *out_len = 0;
    if (count) *count = 0;
    if (k < 1 || k > 31) return ORACLE_ERR_BAD_K;
    mgraph g;
    uint64_t *keys = NULL;
    int rc = parse_lines(&g, k, text, len, &keys);
    uint64_t *ord = NULL;
    if (!rc) {
        ord = (uint64_t *)malloc((g.n ? g.n : 1) * 8);
        if (!ord) rc = ORACLE_ERR_OOM;
        for (uint64_t t = 0; !rc && t < g.n; ++t) ord[t] = order ? order[t] : t;
    }
    if (!rc && (passes & 1)) tips_pass(&g, ord, count);
    if (!rc && (passes & 2)) low_coverage_pass(&g, ord, count);
    if (!rc) {
        uint64_t total = 2;
        for (uint64_t x = 0; x < g.n; ++x) {
            total += 61;
            for (int i = 0; i < 8; ++i) total += g.arcs[x][i].len + 1;
        }
        char *buf = (char *)malloc(total + 64);
        if (!buf) {
            rc = ORACLE_ERR_OOM;
        } else {
            char *p = buf;
            for (uint64_t t = 0; t < g.n; ++t) {
                const uint64_t x = ord[t];
                if (g.deleted[x] || !has_arc(&g, x)) continue;
                p = put_line(p, &g, x);
            }
            *p++ = '\n';
            *out = buf;
            *out_len = (uint64_t)(p - buf);
        }
    }
    free(ord);
    mgraph_free(&g);
    free(keys);
    return rc;
}

/* ---------------------------------------------------------------------------
 * masterSimplifyNodeGraph (graph.cpp:2089-2192) over gathered lines: in the
 * given order, a node left with exactly one arc on each side whose two
 * neighbours both hold an arc back to it (getSrcNodeEdge, graph.cpp:250-309)
 * and neither of which is itself is merged away; each neighbour's arc back
 * gets the node's other arc appended, its multiplicity the weighted average
 * in size_t arithmetic (graph.cpp:2157-2163, no int step here).
 * ------------------------------------------------------------------------- */

static void master_append(mgraph *g, uint64_t d, int slot, const mstr *s, uint8_t m) {
    mstr *a = &g->arcs[d][slot];
    const uint64_t sum = (uint64_t)g->mult[d][slot] * a->len + (uint64_t)m * s->len;
    g->mult[d][slot] = (uint8_t)(sum / (a->len + s->len));
    if (mstr_append(a, s->s, s->len)) g->err = ORACLE_ERR_OOM;
}

static void simplify_master(mgraph *g, const uint64_t *order, uint64_t *merged) {
    for (uint64_t t = 0; t < g->n && !g->err; ++t) {
        const uint64_t x = order[t];
        if (g->deleted[x]) continue;
        int ls, rs, lc, rc;
        one_sided(g, x, &ls, &rs, &lc, &rc);
        if (lc != 1 || rc != 1) continue;
        uint64_t rid, lid;
        int rsd, lsd;
        arc_end(g, x, rs, &rid, &rsd);
        arc_end(g, x, ls, &lid, &lsd);
        const int64_t ri = mfind(g, rid), li = mfind(g, lid);
        if (ri < 0 || li < 0) continue; /* a missing neighbour holds no arc back */
        const int rret = src_edge(g, (uint64_t)ri, x, 0), lret = src_edge(g, (uint64_t)li, x, 1);
        if (rret < 0 || lret < 0) continue;
        if ((uint64_t)li == x || (uint64_t)ri == x) continue;
        mstr xl = g->arcs[x][ls], xr = g->arcs[x][rs]; /* read before ri/li change */
        master_append(g, (uint64_t)ri, rret, &xl, g->mult[x][ls]);
        master_append(g, (uint64_t)li, lret, &xr, g->mult[x][rs]);
        g->deleted[x] = 1;
        if (merged) ++*merged;
    }
}

/* The GPU's visiting order on a graph of arbitrary arcs: as
 * oracle_merge_tree_order, the chain end's arc back found by getSrcNodeEdge. */
static int tree_order_graph(mgraph *g, uint64_t *order) {
    const uint64_t n = g->n;
    int rc = 0;
    uint8_t *mg = (uint8_t *)calloc(n ? n : 1, 1);
    int8_t *ls = (int8_t *)malloc(n ? n : 1), *rs = (int8_t *)malloc(n ? n : 1);
    tord *to = (tord *)malloc((n ? n : 1) * sizeof(tord));
    uint8_t *seen = (uint8_t *)calloc(n ? n : 1, 1);
    uint64_t *cyc = (uint64_t *)malloc((n ? n : 1) * sizeof(uint64_t));
    if (!mg || !ls || !rs || !to || !seen || !cyc) rc = ORACLE_ERR_OOM;
    for (uint64_t x = 0; !rc && x < n; ++x) {
        int l, r, lc, rcnt;
        one_sided(g, x, &l, &r, &lc, &rcnt);
        ls[x] = (int8_t)l;
        rs[x] = (int8_t)r;
        if (g->deleted[x] || lc != 1 || rcnt != 1) continue;
        int s1, s2;
        const int64_t a = step(g, x, l, &s1), b = step(g, x, r, &s2);
        if (a < 0 || b < 0) continue;
        if (src_edge(g, (uint64_t)b, x, 0) < 0 || src_edge(g, (uint64_t)a, x, 1) < 0) continue;
        mg[x] = (uint64_t)a != x && (uint64_t)b != x;
    }
    uint64_t nt = 0, ncyc = 0;
    for (int pass = 0; !rc && pass < 2; ++pass) {
        for (uint64_t x = 0; !rc && x < n; ++x) {
            if (pass == 0 && (mg[x] || g->deleted[x])) continue;
            if (pass == 1 && (!mg[x] || seen[x])) continue;
            uint64_t start = x;
            if (pass == 1) {
                uint64_t best = x, cur = x;
                int dslot = rs[x];
                for (;;) {
                    int side;
                    const int64_t y = step(g, cur, dslot, &side);
                    if ((uint64_t)y == x) break;
                    if (g->keys[y] > g->keys[best]) best = (uint64_t)y;
                    dslot = side ? rs[y] : ls[y];
                    cur = (uint64_t)y;
                }
                start = best;
                mg[start] = 0;
                seen[start] = 1;
                cyc[ncyc++] = start;
            }
            for (int slot = 0; slot < 8 && !rc; ++slot) {
                if (!g->arcs[start][slot].len) continue;
                int side;
                const int64_t y = step(g, start, slot, &side);
                if (y < 0 || !mg[y]) continue;
                uint64_t m = 0, cur = (uint64_t)y, ekey = 0, eslot = 0;
                int dir = side;
                for (;;) {
                    ++m;
                    const int out = dir ? rs[cur] : ls[cur];
                    int s2;
                    const int64_t z = step(g, cur, out, &s2);
                    if (!mg[z]) {
                        ekey = g->keys[z];
                        eslot = (uint64_t)src_edge(g, (uint64_t)z, cur, dir ? 0 : 1);
                        break;
                    }
                    dir = s2;
                    cur = (uint64_t)z;
                }
                const int fwd = g->keys[start] < ekey || (g->keys[start] == ekey && (uint64_t)slot < eslot);
                if (!fwd) continue;
                cur = (uint64_t)y;
                dir = side;
                for (uint64_t p = 1; p <= m; ++p) {
                    to[nt].level = (uint64_t)ctz64(p);
                    to[nt].ckey = g->keys[start];
                    to[nt].cslot = (uint64_t)slot;
                    to[nt].pos = p;
                    to[nt].node = cur;
                    ++nt;
                    seen[cur] = 1;
                    const int out = dir ? rs[cur] : ls[cur];
                    int s2;
                    const int64_t z = step(g, cur, out, &s2);
                    dir = s2;
                    cur = (uint64_t)z;
                }
            }
        }
    }
    if (!rc) {
        qsort(to, nt, sizeof(tord), tord_cmp);
        uint64_t o = 0;
        for (uint64_t x = 0; x < n; ++x)
            if (!mg[x] && !seen[x]) order[o++] = x;
        for (uint64_t i = 0; i < nt; ++i) order[o++] = to[i].node;
        for (uint64_t i = 0; i < ncyc; ++i) order[o++] = cyc[i];
        if (o != n) rc = -13;
    }
    free(cyc);
    free(mg);
    free(ls);
    free(rs);
    free(to);
    free(seen);
    return rc;
}

static int lines_out(mgraph *g, const uint64_t *ord, char **out, uint64_t *out_len) {
    uint64_t total = 2;
    for (uint64_t x = 0; x < g->n; ++x) {
        total += 61;
        for (int i = 0; i < 8; ++i) total += g->arcs[x][i].len + 1;
    }
    char *buf = (char *)malloc(total + 64);
    if (!buf) return ORACLE_ERR_OOM;
    char *p = buf;
    for (uint64_t t = 0; t < g->n; ++t) {
        const uint64_t x = ord[t];
        if (g->deleted[x] || !has_arc(g, x)) continue;
        p = put_line(p, g, x);
    }
    *p++ = '\n';
    *out = buf;
    *out_len = (uint64_t)(p - buf);
    return 0;
}

int oracle_simplify_lines(int k, const char *text, uint64_t len, const uint64_t *order, char **out,
                          uint64_t *out_len, uint64_t *merged) {
    *out = NULL;
    *out_len = 0;
    if (merged) *merged = 0;
    if (k < 1 || k > 31) return ORACLE_ERR_BAD_K;
    mgraph g;
    uint64_t *keys = NULL;
    int rc = parse_lines(&g, k, text, len, &keys);
    uint64_t *ord = (uint64_t *)malloc((g.n ? g.n : 1) * 8);
    if (!ord) rc = ORACLE_ERR_OOM;
    for (uint64_t t = 0; !rc && t < g.n; ++t) ord[t] = order ? order[t] : t;
    if (!rc) simplify_master(&g, ord, merged);
    if (!rc) rc = g.err;
    if (!rc) rc = lines_out(&g, ord, out, out_len);
    free(ord);
    mgraph_free(&g);
    free(keys);
    return rc;
}

int oracle_lines_tree_order(int k, const char *text, uint64_t len, uint64_t *order, uint64_t cap, uint64_t *n) {
    if (k < 1 || k > 31) return ORACLE_ERR_BAD_K;
    mgraph g;
    uint64_t *keys = NULL;
    int rc = parse_lines(&g, k, text, len, &keys);
    *n = g.n;
    if (!rc && cap < g.n) rc = ORACLE_ERR_OOM;
    if (!rc) rc = tree_order_graph(&g, order);
    mgraph_free(&g);
    free(keys);
    return rc;
}
