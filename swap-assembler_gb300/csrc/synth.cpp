// swgsynth — seeded synthetic genomes and reads (see synth.h).
#include "synth.h"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

namespace {

struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed) {}
    uint64_t next() {  // splitmix64
        uint64_t z = (s += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
    double uniform() { return (next() >> 11) * (1.0 / 9007199254740992.0); }
    uint64_t below(uint64_t n) { return n ? next() % n : 0; }
    uint64_t range(uint64_t lo, uint64_t hi) { return lo + below(hi - lo + 1); }
    // Approximately log-uniform on [lo, hi] with integer arithmetic only (so
    // the output is identical on every platform): pick one of the doubling
    // intervals [lo*2^i, lo*2^(i+1)) uniformly, the last partial interval
    // weighted by its length relative to a full one, then a uniform value in it.
    uint64_t log_uniform(uint64_t lo, uint64_t hi) {
        if (lo == 0) lo = 1;
        if (hi <= lo) return lo;
        uint64_t n_full = 0, a = lo;
        while (a * 2 <= hi + 1) {
            a *= 2;
            n_full++;
        }
        const uint64_t tail = hi + 1 - a;  // length of the partial interval [a, hi]
        const uint64_t scale = 1u << 20;
        const uint64_t w_tail = a ? tail * scale / a : 0;  // relative to the full interval [a, 2a)
        const uint64_t pick = below(n_full * scale + w_tail);
        const uint64_t i = pick / scale;
        if (i < n_full) {
            const uint64_t base = lo << i;
            return base + below(base);
        }
        return a + below(tail);
    }
};

const char kBases[4] = {'A', 'C', 'G', 'T'};

char random_base(Rng &r, double gc) {
    double u = r.uniform();
    if (u < gc * 0.5) return 'C';
    if (u < gc) return 'G';
    if (u < gc + (1.0 - gc) * 0.5) return 'A';
    return 'T';
}

char other_base(Rng &r, char b) {
    char c;
    do c = kBases[r.below(4)];
    while (c == b);
    return c;
}

char complement(char b) {
    switch (b) {
        case 'A': return 'T';
        case 'C': return 'G';
        case 'G': return 'C';
        default: return 'A';
    }
}

std::string make_genome(const swg_synth_params &p) {
    Rng r(p.seed * 0x2545f4914f6cdd1dull + 1);
    std::string g(p.genome_len, 'A');
    for (auto &ch : g) ch = random_base(r, p.gc);
    const uint64_t G = p.genome_len;
    // repeat families: a unit written (with divergence) at random places
    uint64_t target = (uint64_t)(p.repeat_frac * (double)G), written = 0;
    while (written < target && p.repeat_unit_max > 0 && G > p.repeat_unit_max) {
        uint64_t ulen = r.log_uniform(std::max<uint32_t>(1, p.repeat_unit_min), p.repeat_unit_max);
        uint64_t copies = r.range(std::max<uint32_t>(1, p.repeat_copies_min),
                                  std::max(p.repeat_copies_min, p.repeat_copies_max));
        std::string unit(ulen, 'A');
        for (auto &ch : unit) ch = random_base(r, p.gc);
        for (uint64_t c = 0; c < copies && written < target; c++) {
            uint64_t pos = r.below(G - ulen);
            for (uint64_t i = 0; i < ulen; i++) {
                char b = unit[i];
                if (r.uniform() < p.repeat_divergence) b = other_base(r, b);
                g[pos + i] = b;
            }
            written += ulen;
        }
    }
    // tandem arrays of short units
    target = (uint64_t)(p.tandem_frac * (double)G);
    written = 0;
    while (written < target && p.tandem_unit_max > 0 && G > p.tandem_len_max) {
        uint64_t ulen = r.range(std::max<uint32_t>(1, p.tandem_unit_min),
                                std::max(p.tandem_unit_min, p.tandem_unit_max));
        uint64_t alen = r.log_uniform(std::max<uint32_t>(1, p.tandem_len_min), p.tandem_len_max);
        char unit[64];
        for (uint64_t i = 0; i < ulen && i < 64; i++) unit[i] = random_base(r, p.gc);
        uint64_t pos = r.below(G - alen);
        for (uint64_t i = 0; i < alen; i++) g[pos + i] = unit[i % ulen];
        written += alen;
    }
    return g;
}

// One read: walk the template (forward or reverse-complement strand) from a
// uniform start, applying substitutions and single-base indels.
void make_read(const std::string &g, const swg_synth_params &p, uint64_t idx, std::string &out) {
    Rng r(p.seed ^ (0x9e3779b97f4a7c15ull * (idx + 1)) ^ 0xd1b54a32d192ed03ull);
    const uint64_t L = p.read_len, G = g.size();
    const uint64_t span = L + L / 4 + 8;  // room for deletions
    uint64_t start = G > span ? r.below(G - span + 1) : 0;
    bool rev = r.next() & 1;
    auto tmpl = [&](uint64_t i) -> char {  // i-th base of the read's template strand
        uint64_t gi = rev ? start + span - 1 - i : start + i;
        if (gi >= G) gi = G - 1;
        char b = g[gi];
        return rev ? complement(b) : b;
    };
    out.clear();
    uint64_t t = 0;
    while (out.size() < L) {
        double u = r.uniform();
        if (u < p.indel_rate * 0.5) {  // insertion
            out.push_back(kBases[r.below(4)]);
            continue;
        }
        if (u < p.indel_rate) {  // deletion
            t++;
            continue;
        }
        char b = tmpl(t++);
        if (r.uniform() < p.sub_rate) b = other_base(r, b);
        out.push_back(b);
    }
}

}  // namespace

extern "C" {

void swg_synth_defaults(swg_synth_params *p) {
    std::memset(p, 0, sizeof(*p));
    p->seed = 1;
    p->genome_len = 1000000;
    p->gc = 0.5;
    p->repeat_unit_min = 1000;
    p->repeat_unit_max = 5000;
    p->repeat_copies_min = 2;
    p->repeat_copies_max = 200;
    p->repeat_divergence = 0.01;
    p->tandem_unit_min = 2;
    p->tandem_unit_max = 6;
    p->tandem_len_min = 20;
    p->tandem_len_max = 2000;
    p->read_len = 100;
}

int64_t swg_synth_fasta(const swg_synth_params *pp, char **out) {
    if (!pp || !out || pp->genome_len < 2 || pp->read_len == 0) return -1;
    const swg_synth_params p = *pp;
    const std::string g = make_genome(p);
    int nt = p.threads > 0 ? p.threads : (int)std::max(1u, std::thread::hardware_concurrency());
    nt = (int)std::min<uint64_t>((uint64_t)nt, std::max<uint64_t>(1, p.n_reads / 4096 + 1));
    std::vector<std::string> parts(nt);
    std::vector<std::thread> th;
    for (int t = 0; t < nt; t++) {
        th.emplace_back([&, t] {
            uint64_t lo = p.n_reads * t / nt, hi = p.n_reads * (t + 1) / nt;
            std::string &s = parts[t];
            s.reserve((hi - lo) * (p.read_len + 16));
            std::string read;
            char hdr[32];
            for (uint64_t i = lo; i < hi; i++) {
                make_read(g, p, i, read);
                int n = std::snprintf(hdr, sizeof(hdr), ">r%llu\n", (unsigned long long)i);
                s.append(hdr, n);
                s.append(read);
                s.push_back('\n');
            }
        });
    }
    for (auto &x : th) x.join();
    uint64_t total = 0;
    for (auto &s : parts) total += s.size();
    char *buf = (char *)std::malloc(total + 1);
    if (!buf) return -1;
    uint64_t pos = 0;
    for (auto &s : parts) {
        std::memcpy(buf + pos, s.data(), s.size());
        pos += s.size();
    }
    buf[total] = 0;
    *out = buf;
    return (int64_t)total;
}

int64_t swg_synth_fasta_file(const swg_synth_params *p, const char *path) {
    char *buf = nullptr;
    int64_t n = swg_synth_fasta(p, &buf);
    if (n < 0) return -1;
    FILE *fp = std::fopen(path, "wb");
    if (!fp) {
        std::free(buf);
        return -1;
    }
    size_t w = std::fwrite(buf, 1, (size_t)n, fp);
    std::fclose(fp);
    std::free(buf);
    return w == (size_t)n ? n : -1;
}

void swg_synth_free(char *buf) { std::free(buf); }

}  // extern "C"
