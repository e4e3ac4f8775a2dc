// Host code under AddressSanitizer / UndefinedBehaviorSanitizer — TEST
// INFRASTRUCTURE, built and run by tests/test_host.py. The device sanitizer
// is not available on the GPU pool, so the host parts of the library that
// parse untrusted input and format output (csrc/reads.cpp: FASTA framing and
// 2-bit packing, multi-threaded; csrc/writers.cpp: the text writers, sort,
// graph totals) are compiled here with -fsanitize=address,undefined and driven
// over the given FASTA files, a set of malformed inputs, and random records.
// Exit status 0: no sanitizer report (reports abort the process).
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "swapgb.h"
#include "swg_internal.h"

namespace swg {
void set_error(const std::string &) {}  // api.cpp's, not linked here
}

static int check_reads(const swg_reads *r, int k) {
    const uint32_t *packed;
    const uint64_t *off;
    const uint32_t *len;
    uint64_t n_words, n_reads, n_bases;
    if (swg_reads_view(r, &packed, &n_words, &off, &len, &n_reads, &n_bases) != SWG_OK) return 1;
    uint64_t sum = 0;
    for (uint64_t i = 0; i < n_reads; ++i) {
        if (len[i] < (uint32_t)k) return 2;
        if (off[i] + len[i] > 16 * n_words) return 3;
        sum += len[i];
    }
    return sum == n_bases ? 0 : 4;
}

int main(int argc, char **argv) {
    int bad = 0;
    // the given FASTA files, at several k
    for (int a = 1; a < argc; ++a) {
        for (int k : {1, 19, 21, 31}) {
            swg_reads *r = nullptr;
            if (swg_reads_from_fasta_file(argv[a], k, &r) == SWG_OK) {
                bad |= check_reads(r, k);
                swg_reads_free(r);
            }
        }
    }
    // malformed and edge-case inputs held in memory
    const std::vector<std::string> texts = {
        "",
        ">",
        ">a",
        ">a\n",
        ">a\nACGT",
        "no record start\n",
        ">a\nACGTNNNNacgt\n>b\nAC\n",
        ">a\r\nACGTACGTACGTACGTACGTACGT\r\n",
        ">a\n\n>b\nACGTACGTACGTACGTACGTACGTA\n",
        "junk before\n>a\nACGTACGTACGTACGTACGTACGT\n",
        std::string(">a\nACGT\0ACGT\n", 12),
        ">a\nACGTACGTACGTACGTACGTACGTACGTACGTACGTACGTACGTACGTACGTACGTACGTACGTACGTACGTACGTACGT\n"
        ">b\nTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTT\n",
    };
    for (const std::string &t : texts)
        for (int k : {1, 3, 19, 31, 32, 0}) {
            swg_reads *r = nullptr;
            if (swg_reads_from_fasta(t.data(), t.size(), k, &r) == SWG_OK) {
                bad |= check_reads(r, k);
                swg_reads_free(r);
            }
        }
    // a large random input, so that every framing thread gets work
    std::mt19937_64 rng(7);
    std::string big;
    for (int i = 0; i < 20000; ++i) {
        big += ">r" + std::to_string(i) + "\n";
        const int L = 50 + (int)(rng() % 200);
        for (int j = 0; j < L; ++j) big += "ACGTNacgt"[rng() % 9];
        big += "\n";
    }
    swg_reads *r = nullptr;
    if (swg_reads_from_fasta(big.data(), big.size(), 21, &r) == SWG_OK) {
        bad |= check_reads(r, 21);
        swg_reads_free(r);
    } else {
        bad |= 8;
    }
    // the writers, graph totals and sort on random records
    const char *dir = std::getenv("SWG_SANITIZE_OUT");
    const std::string out = dir ? dir : ".";
    for (int k : {9, 21, 31}) {
        const uint64_t n = 3000;
        const uint64_t mask = (1ull << (2 * k)) - 1;
        std::vector<uint64_t> keys(n), mult8(n);
        for (uint64_t i = 0; i < n; ++i) {
            keys[i] = rng() & mask;
            mult8[i] = rng() & 0x0303030303030303ull;
        }
        swg::sort_records(keys.data(), mult8.data(), n);
        const uint8_t *m = reinterpret_cast<const uint8_t *>(mult8.data());
        int64_t st[5];
        swg::graph_stats(m, n, k, st);
        bad |= swg::write_kmer_graph(keys.data(), m, n, k, (out + "/kg.txt").c_str()) != SWG_OK ? 16 : 0;
        bad |= swg::write_node_lines(keys.data(), m, n, (out + "/nodes.txt").c_str()) != SWG_OK ? 32 : 0;
    }
    std::printf("host sanitizer run: %s\n", bad ? "invariant broken" : "clean");
    return bad;
}
