// Host FASTA framing and 2-bit packing.
//
// Framing follows the reference's reader (kmerGraph.cpp:113-114,160-233):
// from the first '>' the text is read as alternating lines, a header line and
// then ONE sequence line, each ended by '\n' (strstr at kmerGraph.cpp:173,177);
// a second sequence line of a multi-line record is therefore taken as the next
// header, exactly as the reference does. Sequence bytes are normalised as at
// kmerGraph.cpp:228-233 (ACGT kept, acgt upper-cased, anything else 'A') and
// coded A=0 C=1 G=2 T=3 (sequence.cpp:164-168). Sequences shorter than k are
// dropped (kmerGraph.cpp:182-187). Input the reference never finishes — a
// last record without its '\n' (kmerGraph.cpp:155 is then never reached), a
// NUL byte, no '>' at all (the assert at kmerGraph.cpp:114) — is rejected.
//
// Large inputs are framed in parallel: the text is cut into chunks at line
// starts; a first pass counts, per chunk, its newlines and the reads/bases it
// would hold under either line parity; a prefix over the chunks fixes each
// chunk's parity and output offsets; a second pass packs.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <thread>
#include <utility>
#include <vector>

#include "swg_internal.h"

// Allocator that leaves elements uninitialised on resize: the framing threads
// write every element (the packed words after a parallel clear), so the
// single-threaded zero fill of std::vector is skipped.
template <typename T>
struct NoInitAlloc : std::allocator<T> {
    template <typename U>
    struct rebind {
        using other = NoInitAlloc<U>;
    };
    NoInitAlloc() = default;
    template <typename U>
    NoInitAlloc(const NoInitAlloc<U> &) {}
    template <typename U>
    void construct(U *) noexcept {}
    template <typename U, typename... A>
    void construct(U *p, A &&...a) {
        ::new ((void *)p) U(std::forward<A>(a)...);
    }
};

struct swg_reads {
    std::vector<uint32_t, NoInitAlloc<uint32_t>> packed;
    std::vector<uint64_t, NoInitAlloc<uint64_t>> off;
    std::vector<uint32_t, NoInitAlloc<uint32_t>> len;
    uint64_t n_bases = 0;
    uint64_t n_records = 0;
};

namespace swg {
namespace {

struct CodeTable {
    uint8_t v[256];
    CodeTable() {
        std::memset(v, 0, sizeof(v));
        v['C'] = v['c'] = 1;
        v['G'] = v['g'] = 2;
        v['T'] = v['t'] = 3;
    }
};
const CodeTable kCodes;

struct ChunkStats {
    uint64_t newlines = 0;
    // [p] = totals if the chunk's first line has global parity p (0 = header)
    uint64_t reads[2] = {0, 0};
    uint64_t bases[2] = {0, 0};
    uint64_t records[2] = {0, 0};
};

// Pass 1 over the lines that start in [b, e): count them by parity.
void count_chunk(const char *b, const char *e, int k, ChunkStats &st) {
    const char *p = b;
    uint64_t line = 0;
    while (p < e) {
        // chunks end right after a '\n', so every line starting here ends here
        const char *nl = (const char *)std::memchr(p, '\n', (size_t)(e - p));
        uint64_t L = nl ? (uint64_t)(nl - p) : (uint64_t)(e - p);
        // local line index `line`: it is a sequence line when (parity + line) is odd
        int seq_if_parity0 = (int)(line & 1);
        if (nl) {
            int par = seq_if_parity0 ? 0 : 1;  // parity making this line a sequence line
            st.records[par]++;
            if (L >= (uint64_t)k) {
                st.reads[par]++;
                st.bases[par] += L;
            }
            st.newlines++;
        }
        line++;
        if (!nl) break;
        p = nl + 1;
    }
}

// Eight sequence bytes (first base in the lowest byte) to their 2-bit codes,
// first base in bits 15..14, with portable 64-bit arithmetic: a byte's code
// is ((c >> 1) ^ (c >> 2)) & 3 for A/C/G/T in either case (A=0 C=1 G=2 T=3);
// every other byte is read as A (kmerGraph.cpp:228-233).
inline uint64_t bytes_equal(uint64_t v, uint64_t t) {  // 0x80 in each byte of v equal to t's
    const uint64_t z = v ^ t;
    return ~(((z & 0x7f7f7f7f7f7f7f7full) + 0x7f7f7f7f7f7f7f7full) | z | 0x7f7f7f7f7f7f7f7full);
}
inline uint32_t pack8(uint64_t x) {
    const uint64_t lc = x | 0x2020202020202020ull;  // lower case (only the four letters count)
    const uint64_t ok = bytes_equal(lc, 0x6161616161616161ull) | bytes_equal(lc, 0x6363636363636363ull) |
                        bytes_equal(lc, 0x6767676767676767ull) | bytes_equal(lc, 0x7474747474747474ull);
    const uint64_t y = ((x >> 1) ^ (x >> 2)) & ((ok >> 7) * 3);  // code i in bits 8i..8i+1
    const uint64_t y2 = ((y & 0x0003000300030003ull) << 2) | ((y >> 8) & 0x0003000300030003ull);
    const uint64_t y3 = ((y2 & 0x0000000f0000000full) << 4) | ((y2 >> 16) & 0x0000000f0000000full);
    return (uint32_t)(((y3 & 0xffu) << 8) | ((y3 >> 32) & 0xffu));
}
inline uint32_t pack16(const char *p) {
    uint64_t a, b;
    std::memcpy(&a, p, 8);
    std::memcpy(&b, p + 8, 8);
    return (pack8(a) << 16) | pack8(b);
}

inline void put_word(uint32_t *w, uint64_t idx, uint32_t val, bool shared) {
    if (!val) return;
    if (shared) __atomic_fetch_or(&w[idx], val, __ATOMIC_RELAXED);
    else w[idx] |= val;
}

// Pass 2: pack the sequence lines of [b, e) given the chunk's parity.
void pack_chunk(const char *b, const char *e, int parity, int k, uint64_t read0, uint64_t base0,
                uint64_t base_end, swg_reads *r) {
    uint32_t *words = r->packed.data();
    const uint64_t first_word = base0 >> 4;
    const uint64_t last_word = base_end ? (base_end - 1) >> 4 : 0;
    const char *p = b;
    uint64_t line = 0, rd = read0, base = base0;
    while (p < e) {
        // chunks end right after a '\n', so every line starting here ends here
        const char *nl = (const char *)std::memchr(p, '\n', (size_t)(e - p));
        uint64_t L = (uint64_t)(nl - p);
        bool is_seq = ((line + (uint64_t)parity) & 1) != 0;
        if (is_seq && L >= (uint64_t)k) {
            r->off[rd] = base;
            r->len[rd] = (uint32_t)L;
            rd++;
            uint64_t widx = base >> 4;
            uint32_t acc = 0;
            int fill = (int)(base & 15);
            uint64_t i = 0;
            for (; i < L && fill; i++) {  // up to the read's first whole word
                acc |= (uint32_t)kCodes.v[(unsigned char)p[i]] << (30 - 2 * fill);
                if (++fill == 16) {
                    put_word(words, widx, acc, widx == first_word || widx == last_word);
                    widx++;
                    acc = 0;
                    fill = 0;
                }
            }
            for (; i + 16 <= L; i += 16, widx++)  // whole words, 16 bases at a time
                put_word(words, widx, pack16(p + i), widx == first_word || widx == last_word);
            for (; i < L; i++) {
                acc |= (uint32_t)kCodes.v[(unsigned char)p[i]] << (30 - 2 * fill);
                fill++;
            }
            if (fill) put_word(words, widx, acc, widx == first_word || widx == last_word);
            base += L;
        }
        line++;
        p = nl + 1;
    }
}

}  // namespace

swg_status pack_fasta(const char *text, uint64_t len, int k, swg_reads **out) {
    *out = nullptr;
    if (k < 1 || k > 31) {
        set_error("k must be in 1..31");
        return SWG_ERR_BAD_INPUT;
    }
    if (!text || len == 0) {
        set_error("empty FASTA input");
        return SWG_ERR_BAD_INPUT;
    }
    const char *end = text + len;
    const char *first = (const char *)std::memchr(text, '>', len);
    if (!first) {
        set_error("no '>' record start in the input");
        return SWG_ERR_BAD_INPUT;
    }
    if (end[-1] != '\n') {
        set_error("the last record is not terminated by a newline");
        return SWG_ERR_BAD_INPUT;
    }
    const uint64_t body = (uint64_t)(end - first);
    int nt = (int)std::max(1u, std::thread::hardware_concurrency());
    nt = (int)std::min<uint64_t>((uint64_t)nt, body / (4u << 20) + 1);
    // chunk starts at line starts
    std::vector<const char *> cs(nt + 1);
    cs[0] = first;
    cs[nt] = end;
    for (int t = 1; t < nt; t++) {
        const char *nominal = first + body * (uint64_t)t / (uint64_t)nt;
        nominal = std::max(nominal, cs[t - 1]);
        const char *nl = (const char *)std::memchr(nominal, '\n', (size_t)(end - nominal));
        cs[t] = nl ? nl + 1 : end;
    }
    std::vector<ChunkStats> st(nt);
    std::vector<int> has_nul(nt, 0);
    {
        std::vector<std::thread> th;
        for (int t = 0; t < nt; t++)
            th.emplace_back([&, t] {
                has_nul[t] = std::memchr(cs[t], 0, (size_t)(cs[t + 1] - cs[t])) != nullptr;
                count_chunk(cs[t], cs[t + 1], k, st[t]);
            });
        for (auto &x : th) x.join();
    }
    for (int t = 0; t < nt; t++)
        if (has_nul[t]) {
            set_error("NUL byte in the FASTA input");
            return SWG_ERR_BAD_INPUT;
        }
    std::vector<int> parity(nt);
    std::vector<uint64_t> read0(nt + 1), base0(nt + 1);
    uint64_t lines = 0, nrec = 0;
    read0[0] = base0[0] = 0;
    for (int t = 0; t < nt; t++) {
        parity[t] = (int)(lines & 1);
        read0[t + 1] = read0[t] + st[t].reads[parity[t]];
        base0[t + 1] = base0[t] + st[t].bases[parity[t]];
        nrec += st[t].records[parity[t]];
        lines += st[t].newlines;
    }
    if (lines & 1) {
        set_error("the last record has a header line but no sequence line");
        return SWG_ERR_BAD_INPUT;
    }
    swg_reads *r = new (std::nothrow) swg_reads;
    if (!r) return SWG_ERR_OOM;
    try {
        r->n_bases = base0[nt];
        r->n_records = nrec;
        r->off.resize(read0[nt]);
        r->len.resize(read0[nt]);
        r->packed.resize((r->n_bases + 15) / 16 + 4);  // 4 words of tail padding
    } catch (...) {
        delete r;
        set_error("host allocation failed while packing reads");
        return SWG_ERR_OOM;
    }
    {
        // every thread clears a share of the words, then (after all have)
        // packs its chunk: chunks share their boundary words
        const uint64_t nw = r->packed.size();
        std::vector<std::thread> th;
        for (int t = 0; t < nt; t++)
            th.emplace_back([&, t] {
                const uint64_t w0 = nw * (uint64_t)t / (uint64_t)nt, w1 = nw * (uint64_t)(t + 1) / (uint64_t)nt;
                std::memset(r->packed.data() + w0, 0, (size_t)(w1 - w0) * sizeof(uint32_t));
            });
        for (auto &x : th) x.join();
        th.clear();
        for (int t = 0; t < nt; t++)
            th.emplace_back([&, t] {
                pack_chunk(cs[t], cs[t + 1], parity[t], k, read0[t], base0[t], base0[t + 1], r);
            });
        for (auto &x : th) x.join();
    }
    *out = r;
    return SWG_OK;
}

}  // namespace swg

extern "C" {

swg_status swg_reads_from_fasta(const char *text, uint64_t len, int k, swg_reads **out) {
    if (!out) return SWG_ERR_BAD_INPUT;
    return swg::pack_fasta(text, len, k, out);
}

swg_status swg_reads_from_fasta_file(const char *path, int k, swg_reads **out) {
    if (!out || !path) return SWG_ERR_BAD_INPUT;
    *out = nullptr;
    FILE *fp = std::fopen(path, "rb");
    if (!fp) {
        swg::set_error(std::string("cannot open ") + path);
        return SWG_ERR_IO;
    }
    std::fseek(fp, 0, SEEK_END);
    long long sz = ftello(fp);
    std::fseek(fp, 0, SEEK_SET);
    std::vector<char> buf;
    try {
        buf.resize((size_t)std::max(0LL, sz));
    } catch (...) {
        std::fclose(fp);
        return SWG_ERR_OOM;
    }
    size_t got = sz > 0 ? std::fread(buf.data(), 1, (size_t)sz, fp) : 0;
    std::fclose(fp);
    if ((long long)got != sz) {
        swg::set_error(std::string("short read from ") + path);
        return SWG_ERR_IO;
    }
    return swg::pack_fasta(buf.data(), (uint64_t)buf.size(), k, out);
}

swg_status swg_reads_view(const swg_reads *r, const uint32_t **packed, uint64_t *n_words,
                          const uint64_t **read_off, const uint32_t **read_len, uint64_t *n_reads,
                          uint64_t *n_bases) {
    if (!r) return SWG_ERR_BAD_INPUT;
    if (packed) *packed = r->packed.data();
    if (n_words) *n_words = r->packed.size();
    if (read_off) *read_off = r->off.data();
    if (read_len) *read_len = r->len.data();
    if (n_reads) *n_reads = r->off.size();
    if (n_bases) *n_bases = r->n_bases;
    return SWG_OK;
}

uint64_t swg_reads_records(const swg_reads *r) { return r ? r->n_records : 0; }

void swg_reads_free(swg_reads *r) { delete r; }

}  // extern "C"
