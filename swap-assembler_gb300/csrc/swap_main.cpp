// swap — command line of the GPU k-mer graph build, with the reference's
// interface: swap -k <kmerlength> -c <cutoff> -i <input fasta> -o <output dir> [-s] [-d]
//
// Flags, defaults (k=23, c=5) and checks follow parameter::getopt and
// getParameters (sequence.cpp:4-183): k odd in 19..31 (sequence.cpp:44), the
// output directory is created and must not exist (sequence.cpp:128-133).
// Outputs in <output dir>:
//   kmerGraph.txt  with -s, the reference's -s adjacency file
//                  (graph.cpp:3352-3440), lines sorted by first token;
//   nodes.txt      every surviving k-molecule with its 8 edge multiplicities
//                  (graph.cpp:569 layout), the input of the merging stage;
//   contigGraph.txt with -d and without -s (graph.cpp:3617-3621), the graph
//                  after merging its semi-extended k-molecules (the merge of
//                  simplifyDistNodeGraph, graph.cpp:1392-1566, run on the GPU);
//   noCEcontigs.fasta with it: the contigs of the merged graph as the
//                  reference's printContigs writes them (graph.cpp:1139-1202);
//   logtime.txt    phase times.
// stdout carries the reference's graph totals (graph.cpp:1621-1625).
// Unlike the reference, every failure exits with a nonzero status.
#include <sys/stat.h>
#include <sys/types.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "swapgb.h"

namespace {

void usage(const char *argv0) {
    std::printf("Usage: %s -k <kmerlength> -c <cutoff Threshod> -i <input Fasta data> -o <output data directory>\n",
                argv0);
}

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int fail(swg_status st, const char *what) {
    std::fprintf(stderr, "Error: %s: %s (%s)\n", what, swg_status_string(st), swg_last_error());
    return 1;
}

}  // namespace

int main(int argc, char **argv) {
    int k = 23, c = 5, kmer_graph = 0, dist_graph = 0;
    std::string in, out;
    for (int i = 1; i < argc; i++) {
        const char *a = argv[i];
        if (a[0] != '-') {
            usage(argv[0]);
            return 2;
        }
        switch (a[1]) {
            case 'h': usage(argv[0]); return 0;
            case 'v': std::printf("SWAP-Assembler version 0.2 (%s)\n", swg_version()); return 0;
            case 'k':
                if (i + 1 == argc || std::sscanf(argv[i + 1], "%d", &k) != 1 || k < 19 || k > 31 ||
                    k % 2 != 1) {
                    std::printf("Error: -k needs a value (odd number between 18 and 32) for the kmer size\n");
                    usage(argv[0]);
                    return 2;
                }
                i++;
                break;
            case 'c':
                if (i + 1 == argc || std::sscanf(argv[i + 1], "%d", &c) != 1) {
                    std::printf("Error: -c needs a value for the cutoff threshold\n");
                    usage(argv[0]);
                    return 2;
                }
                i++;
                break;
            case 'i':
                if (i + 1 == argc) {
                    std::printf("Error: -i needs a path for the file in fasta format\n");
                    usage(argv[0]);
                    return 2;
                }
                in = argv[++i];
                break;
            case 'o':
                if (i + 1 == argc) {
                    std::printf("Error: -o needs a directory name used for the output data\n");
                    usage(argv[0]);
                    return 2;
                }
                out = argv[++i];
                break;
            case 's': kmer_graph = 1; break;
            case 'd': dist_graph = 1; break;
            default: break;  // -j -p select contig-stage outputs, which this build does not run
        }
    }
    if (in.empty() || out.empty()) {
        usage(argv[0]);
        return 2;
    }
    if (mkdir(out.c_str(), S_IRWXU | S_IRWXG | S_IROTH | S_IXOTH) == -1) {
        std::printf("Error: Creating directory %s\n", out.c_str());
        return 1;
    }
    std::printf("Runing command: %s -k %d -c %d -i %s -o %s\n", argv[0], k, c, in.c_str(), out.c_str());

    const double t0 = now_s();
    std::string text;
    {
        FILE *fp = std::fopen(in.c_str(), "rb");
        if (!fp) {
            std::printf("Error: cannot open %s\n", in.c_str());
            return 1;
        }
        std::fseek(fp, 0, SEEK_END);
        const long long sz = ftello(fp);
        std::fseek(fp, 0, SEEK_SET);
        text.resize((size_t)std::max(0LL, sz));
        const size_t got = sz > 0 ? std::fread(&text[0], 1, (size_t)sz, fp) : 0;
        std::fclose(fp);
        if ((long long)got != sz) {
            std::printf("Error: short read from %s\n", in.c_str());
            return 1;
        }
    }
    const double t1 = now_s();
    swg_opts o;
    std::memset(&o, 0, sizeof(o));
    o.k = k;
    o.cutoff = c;
    swg_graph *g = nullptr;
    swg_status st = swg_graph_create(&g);
    if (st) return fail(st, "creating the graph");
    // framing, packing and counting all run on the GPU
    st = swg_graph_build_fasta(g, &o, text.data(), text.size());
    std::string().swap(text);
    if (st) return fail(st, "building the k-mer graph");
    const double t2 = now_s();
    int64_t stats[5];
    if ((st = swg_graph_stats(g, stats))) return fail(st, "graph statistics");
    std::printf("recvNodeNum = %lld\n", (long long)stats[0]);
    std::printf("recvEdgeNum = %lld\n", (long long)stats[1]);
    std::printf("recvEdgeAvgLength = %lld\n", (long long)stats[2]);
    std::printf("recvTipsNum = %lld\n", (long long)stats[3]);
    std::printf("recvBubbleNum = %lld\n", (long long)stats[4]);
    if (kmer_graph && (st = swg_graph_write_kmer_graph(g, (out + "/kmerGraph.txt").c_str())))
        return fail(st, "writing kmerGraph.txt");
    if ((st = swg_graph_write_node_lines(g, (out + "/nodes.txt").c_str())))
        return fail(st, "writing nodes.txt");
    // the reference merges only without -s, and writes the merged graph with -d
    // (graph.cpp:3578, 3617)
    swg_merge_info minfo;
    std::memset(&minfo, 0, sizeof(minfo));
    const bool merge = dist_graph && !kmer_graph;
    if (merge) {
        if ((st = swg_graph_merge(g))) return fail(st, "merging semi-extended k-molecules");
        if ((st = swg_graph_merge_info(g, &minfo))) return fail(st, "merge info");
        if ((st = swg_graph_write_merged(g, (out + "/contigGraph.txt").c_str())))
            return fail(st, "writing contigGraph.txt");
        uint64_t contigs = 0;
        if ((st = swg_graph_write_contigs(g, (out + "/noCEcontigs.fasta").c_str(), &contigs)))
            return fail(st, "writing noCEcontigs.fasta");
        std::printf(">proc0: %llu contigs\n", (unsigned long long)contigs);
    }
    const double t3 = now_s();
    float ms[5];
    int launches = 0;
    swg_graph_last_timings(g, ms, &launches);
    swg_build_info info;
    std::memset(&info, 0, sizeof(info));
    swg_graph_build_info(g, &info);
    static const char *phases_bucketed[4] = {"setup", "level-1 scatter", "level-2 scatter", "bucket counting"};
    static const char *phases_direct[4] = {"sizing", "clear", "count", "cutoff"};
    const char *const *ph = info.algorithm == SWG_ALGO_BUCKETED ? phases_bucketed : phases_direct;
    FILE *lf = std::fopen((out + "/logtime.txt").c_str(), "w");
    if (lf) {
        std::fprintf(lf, "Time spend in Geting Reads (file read) %.5f\n", t1 - t0);
        std::fprintf(lf, "Time spend in Constructing Graph %.5f (framing on the device; build %.5f: %s %.5f, %s %.5f, %s %.5f, %s %.5f)\n",
                     t2 - t1, ms[4] * 1e-3, ph[0], ms[0] * 1e-3, ph[1], ms[1] * 1e-3, ph[2], ms[2] * 1e-3,
                     ph[3], ms[3] * 1e-3);
        if (merge)
            std::fprintf(lf, "Time spend in Simplify DistGraph %.5f (device; %llu nodes left, %llu chains, %llu cycles)\n",
                         minfo.ms * 1e-3, (unsigned long long)minfo.nodes, (unsigned long long)minfo.chains,
                         (unsigned long long)minfo.cycles);
        std::fprintf(lf, "Time spend in writing output %.5f\n", t3 - t2);
        std::fprintf(lf, "Time spend in All step %.5f\n", t3 - t0);
        std::fclose(lf);
    }
    swg_graph_free(g);
    return 0;
}
