/*
 * swap_oracle — command-line front end of the CPU restatement (TEST
 * INFRASTRUCTURE ONLY). Mirrors `swap -k -c -i -o -s` (sequence.cpp:4-119) but
 * writes both outputs sorted: <o>/kmerGraph.txt (graph.cpp:3352-3440) and
 * <o>/nodes.txt (graph.cpp:569 layout). -t sets the thread count (0 = all
 * cores). Prints one JSON line with the phase times.
 */
#define _GNU_SOURCE
#include "kmer_oracle.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <time.h>

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + ts.tv_nsec * 1e-9;
}

int main(int argc, char **argv) {
    int k = 23, c = 5, threads = 0, write = 0;
    const char *in = NULL, *out = NULL;
    for (int i = 1; i < argc; i++) {
        if (!strcmp(argv[i], "-k") && i + 1 < argc) k = atoi(argv[++i]);
        else if (!strcmp(argv[i], "-c") && i + 1 < argc) c = atoi(argv[++i]);
        else if (!strcmp(argv[i], "-i") && i + 1 < argc) in = argv[++i];
        else if (!strcmp(argv[i], "-o") && i + 1 < argc) out = argv[++i];
        else if (!strcmp(argv[i], "-t") && i + 1 < argc) threads = atoi(argv[++i]);
        else if (!strcmp(argv[i], "-s")) write = 1;
    }
    if (!in || !out) {
        fprintf(stderr, "usage: %s -k K -c C -i reads.fa -o outdir [-s] [-t threads]\n", argv[0]);
        return 2;
    }
    double t0 = now_s();
    FILE *fp = fopen(in, "rb");
    if (!fp) { fprintf(stderr, "cannot open %s\n", in); return 1; }
    fseeko(fp, 0, SEEK_END);
    long long sz = ftello(fp);
    fseeko(fp, 0, SEEK_SET);
    char *buf = (char *)malloc((size_t)sz + 1);
    if (!buf || fread(buf, 1, (size_t)sz, fp) != (size_t)sz) { fprintf(stderr, "read failed\n"); return 1; }
    fclose(fp);
    double t1 = now_s();
    oracle_reads r;
    int e = oracle_parse_fasta(buf, (uint64_t)sz, k, &r);
    free(buf);
    if (e) { fprintf(stderr, "parse error %d\n", e); return 1; }
    double t2 = now_s();
    oracle_graph *g = oracle_build(&r, k, c, 1, threads);
    if (!g) { fprintf(stderr, "build failed\n"); return 1; }
    double t3 = now_s();
    if (write) {
        mkdir(out, 0755);
        char path[4096];
        snprintf(path, sizeof(path), "%s/kmerGraph.txt", out);
        oracle_write_kmer_graph(g, k, path);
        snprintf(path, sizeof(path), "%s/nodes.txt", out);
        oracle_write_node_lines(g, path);
    }
    double t4 = now_s();
    int64_t st[5];
    oracle_graph_stats(g, k, st);
    printf("{\"reads\": %llu, \"bases\": %llu, \"survivors\": %llu, \"edges\": %lld, "
           "\"read_s\": %.6f, \"parse_s\": %.6f, \"build_s\": %.6f, \"write_s\": %.6f}\n",
           (unsigned long long)r.n_reads, (unsigned long long)r.n_bases,
           (unsigned long long)oracle_graph_size(g), (long long)st[1], t1 - t0, t2 - t1, t3 - t2,
           t4 - t3);
    oracle_graph_free(g);
    oracle_reads_free(&r);
    return 0;
}
