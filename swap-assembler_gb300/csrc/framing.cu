// FASTA framing and 2-bit packing on the device.
//
// Same framing as the host path (and the reference, kmerGraph.cpp:113-114,
// 160-233): from the first '>', lines alternate header / ONE sequence line;
// acgt upper-cased, any other byte read as 'A'; sequences shorter than k
// dropped. Steps: newlines per 16 KiB chunk (and a newline bit mask) -> scan
// -> every newline's position -> record r = (line 2r, line 2r+1) -> keep
// sequences of length >= k -> one scan of kept reads and of their 16-base
// words -> pack. Every read starts on a word boundary of the packed stream
// (read_off is a multiple of 16), so each packed word belongs to one read and
// is written by one thread. A streamed text is framed a piece at a time; past
// its first piece the records' ranges and the running totals can stay in
// device memory (StreamState), with no host round trip per piece.
#include <cuda_runtime.h>

#include <algorithm>

#include "dev_util.cuh"
#include "swg_internal.h"

namespace swg {
namespace {

constexpr int kFBlock = 256;
constexpr int kFVec = 4;                                    // 16-byte loads per thread
constexpr int kFBytes = 16 * kFVec;                         // bytes per thread
constexpr uint64_t kFChunk = (uint64_t)kFBlock * kFBytes;  // bytes per block
static_assert(kFChunk == kFramingChunk, "the streamed build splits the text on framing chunks");
constexpr int kGItems = 8;
constexpr uint64_t kGChunk = (uint64_t)kFBlock * kGItems;  // items per scan block

// A thread's kFBytes bytes at i (a multiple of 16) as 32-bit words; bytes
// past n read as 1 (neither a newline nor a NUL).
__device__ __forceinline__ void load_words(const unsigned char *__restrict__ t, uint64_t n, uint64_t i,
                                           uint32_t w[kFBytes / 4]) {
#pragma unroll
    for (int v = 0; v < kFVec; ++v) {
        const uint64_t a = i + 16 * (uint64_t)v;
        if (a + 16 <= n) {
            const uint4 x = *reinterpret_cast<const uint4 *>(t + a);
            w[4 * v] = x.x;
            w[4 * v + 1] = x.y;
            w[4 * v + 2] = x.z;
            w[4 * v + 3] = x.w;
        } else {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                uint32_t x = 0;
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    const uint64_t at = a + 4 * q + b;
                    x |= (uint32_t)(at < n ? t[at] : (unsigned char)1) << (8 * b);
                }
                w[4 * v + q] = x;
            }
        }
    }
}

// 0xff in every byte of x equal to '\n'.
__device__ __forceinline__ uint32_t nl_mask(uint32_t x) { return __vcmpeq4(x, 0x0a0a0a0au); }

// Newlines per chunk (chunks j0 + blockIdx.x), and per thread's kFBytes
// bytes a bit mask of them (bit b: byte b is a newline) for k_nl_pos, which
// then reads 1/8 of what the text is; any NUL byte raises flag.
static_assert(kFBytes == 64, "one 64-bit newline mask per thread");
__global__ void __launch_bounds__(kFBlock) k_nl_count(const unsigned char *__restrict__ t, uint64_t n,
                                                      uint64_t *__restrict__ counts,
                                                      unsigned long long *__restrict__ masks,
                                                      unsigned *__restrict__ flag, uint64_t j0) {
    __shared__ uint64_t wb[kFBlock / 32];
    const uint64_t j = j0 + blockIdx.x;
    uint32_t w[kFBytes / 4];
    load_words(t, n, j * kFChunk + (uint64_t)threadIdx.x * kFBytes, w);
    unsigned z = 0;
    unsigned long long m = 0;
#pragma unroll
    for (int q = 0; q < kFBytes / 4; ++q) {
        const uint32_t e = nl_mask(w[q]);  // 0xff per newline byte
        const uint32_t b = ((e >> 7) & 1u) | ((e >> 14) & 2u) | ((e >> 21) & 4u) | ((e >> 28) & 8u);
        m |= (unsigned long long)b << (4 * q);
        z |= __vcmpeq4(w[q], 0u);
    }
    masks[j * kFBlock + threadIdx.x] = m;
    uint64_t total;
    block_exclusive_scan<kFBlock>((uint64_t)__popcll(m), wb, &total);
    if (threadIdx.x == 0) counts[j] = total;
    if (z) atomicOr(flag, 1u);
}

// Position of every newline of chunks j0 + blockIdx.x, in order, from the
// masks k_nl_count left; positions from cap on are not written and set *ovf.
__global__ void __launch_bounds__(kFBlock) k_nl_pos(const unsigned long long *__restrict__ masks,
                                                    const uint64_t *__restrict__ chunk_base,
                                                    uint64_t *__restrict__ nl, uint64_t j0, uint64_t cap,
                                                    uint64_t *__restrict__ ovf) {
    __shared__ uint64_t wb[kFBlock / 32];
    const uint64_t j = j0 + blockIdx.x;
    const uint64_t base = j * kFChunk + (uint64_t)threadIdx.x * kFBytes;
    unsigned long long m = masks[j * kFBlock + threadIdx.x];
    uint64_t pos = chunk_base[j] + block_exclusive_scan<kFBlock>((uint64_t)__popcll(m), wb, nullptr);
    while (m) {
        if (pos < cap) nl[pos] = base + (uint64_t)(__ffsll((long long)m) - 1);
        else if (ovf) *ovf = 1;
        pos++;
        m &= m - 1;
    }
}

// Exclusive scan of at most a few kGChunk items by one block (in place
// allowed): one launch where the three-kernel scan would take three.
__global__ void __launch_bounds__(kFBlock) k_gscan_small(const uint64_t *in, uint64_t n, uint64_t *out,
                                                         uint64_t *total) {
    __shared__ uint64_t wb[kFBlock / 32];
    uint64_t carry = 0;
    for (uint64_t b0 = 0; b0 < n; b0 += kGChunk) {
        const uint64_t base = b0 + (uint64_t)threadIdx.x * kGItems;
        uint64_t v[kGItems];
        uint64_t s = 0;
#pragma unroll
        for (int it = 0; it < kGItems; ++it) {
            v[it] = base + it < n ? in[base + it] : 0;
            s += v[it];
        }
        uint64_t t;
        uint64_t run = carry + block_exclusive_scan<kFBlock>(s, wb, &t);
#pragma unroll
        for (int it = 0; it < kGItems; ++it) {
            if (base + it < n) out[base + it] = run;
            run += v[it];
        }
        carry += t;
    }
    if (threadIdx.x == 0) *total = carry;
}

// Generic exclusive scan of uint64 (in place allowed).
__global__ void __launch_bounds__(kFBlock) k_gscan_reduce(const uint64_t *__restrict__ in, uint64_t n,
                                                          uint64_t *__restrict__ sums) {
    __shared__ uint64_t wb[kFBlock / 32];
    const uint64_t base = (uint64_t)blockIdx.x * kGChunk;
    uint64_t s = 0;
    for (int it = 0; it < kGItems; ++it) {
        const uint64_t i = base + (uint64_t)it * kFBlock + threadIdx.x;
        if (i < n) s += in[i];
    }
    uint64_t total;
    block_exclusive_scan<kFBlock>(s, wb, &total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// One block of kFBlock threads: a block this size finds room on an SM that
// a concurrent kernel of the same block size leaves (the streamed build's
// framing runs beside the level-1 scatter).
__global__ void __launch_bounds__(kFBlock) k_gscan_blocks(uint64_t *sums, uint64_t nb, uint64_t *total) {
    __shared__ uint64_t wb[kFBlock / 32];
    __shared__ uint64_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint64_t base = 0; base < nb; base += kFBlock) {
        const uint64_t i = base + threadIdx.x;
        const uint64_t v = i < nb ? sums[i] : 0;
        uint64_t t;
        const uint64_t ex = block_exclusive_scan<kFBlock>(v, wb, &t);
        const uint64_t c = carry;
        if (i < nb) sums[i] = c + ex;
        __syncthreads();
        if (threadIdx.x == 0) carry = c + t;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void __launch_bounds__(kFBlock) k_gscan_write(const uint64_t *in, uint64_t n,
                                                         const uint64_t *__restrict__ sums,
                                                         uint64_t *out) {
    __shared__ uint64_t wb[kFBlock / 32];
    const uint64_t base = (uint64_t)blockIdx.x * kGChunk + (uint64_t)threadIdx.x * kGItems;
    uint64_t v[kGItems];
    uint64_t s = 0;
#pragma unroll
    for (int it = 0; it < kGItems; ++it) {
        v[it] = base + it < n ? in[base + it] : 0;
        s += v[it];
    }
    uint64_t run = sums[blockIdx.x] + block_exclusive_scan<kFBlock>(s, wb, nullptr);
#pragma unroll
    for (int it = 0; it < kGItems; ++it) {
        if (base + it < n) out[base + it] = run;
        run += v[it];
    }
}

// Record r's sequence length (line 2r+1; header line 2r before it).
__device__ __forceinline__ uint64_t rec_length(const uint64_t *__restrict__ nl, uint64_t r) {
    return nl[2 * r + 1] - nl[2 * r] - 1;
}

// The record scan in three kernels (a scan of records r0 <= r < r1 in blocks
// of kGChunk): per block the kept records (length >= k) and their 16-base
// words are summed (and, with acc, the kept reads' k-mer occurrences added
// to acc[0] and their longest length maxed into acc[1]); one block scans the
// two columns of block sums (totals to tot[0], tot[1]); then every record
// gets its read index (kept records before it) and first word, from r0 on.
// With rr, the range is rr[0] <= r < rr[1] (device values, a streamed
// piece's records); the blocks stride over the range's blocks of records.
__device__ __forceinline__ void rec_range(const uint64_t *rr, uint64_t &r0, uint64_t &r1) {
    if (rr) {
        r0 = rr[0];
        r1 = rr[1];
    }
}

__global__ void __launch_bounds__(kFBlock) k_rec_reduce(const uint64_t *__restrict__ nl, uint64_t r0,
                                                        uint64_t r1, const uint64_t *rr, int k,
                                                        uint64_t *__restrict__ sums,
                                                        unsigned long long *__restrict__ acc) {
    __shared__ uint64_t wb[kFBlock / 32];
    rec_range(rr, r0, r1);
    const uint64_t nb = r1 > r0 ? (r1 - r0 + kGChunk - 1) / kGChunk : 0;
    for (uint64_t q = blockIdx.x; q < nb; q += gridDim.x) {
        const uint64_t base = r0 + q * kGChunk;
        uint64_t keep = 0, words = 0;
        unsigned long long occ = 0, mx = 0;
        for (int it = 0; it < kGItems; ++it) {
            const uint64_t r = base + (uint64_t)it * kFBlock + threadIdx.x;
            if (r < r1) {
                const uint64_t L = rec_length(nl, r);
                if (L >= (uint64_t)k) {
                    keep++;
                    words += (L + 15) / 16;
                    occ += L - (uint64_t)k + 1;
                    mx = L > mx ? L : mx;
                }
            }
        }
        uint64_t tk, tw;
        block_exclusive_scan<kFBlock>(keep, wb, &tk);
        block_exclusive_scan<kFBlock>(words, wb, &tw);
        if (threadIdx.x == 0) {
            sums[2 * q] = tk;
            sums[2 * q + 1] = tw;
        }
        if (acc) {
#pragma unroll
            for (int d = 16; d; d >>= 1) {
                occ += __shfl_down_sync(0xffffffffu, occ, d);
                const unsigned long long y = __shfl_down_sync(0xffffffffu, mx, d);
                mx = y > mx ? y : mx;
            }
            if ((threadIdx.x & 31) == 0 && occ) {
                atomicAdd(&acc[0], occ);
                atomicMax(&acc[1], mx);
            }
        }
    }
}

__global__ void __launch_bounds__(kFBlock) k_rec_blocks(uint64_t *sums, uint64_t r0, uint64_t r1,
                                                        const uint64_t *rr, uint64_t *tot) {
    __shared__ uint64_t wb[kFBlock / 32];
    __shared__ uint64_t carry[2];
    rec_range(rr, r0, r1);
    const uint64_t nb = r1 > r0 ? (r1 - r0 + kGChunk - 1) / kGChunk : 0;
    if (threadIdx.x < 2) carry[threadIdx.x] = 0;
    __syncthreads();
    for (uint64_t b0 = 0; b0 < nb; b0 += kFBlock) {
        const uint64_t i = b0 + threadIdx.x;
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            const uint64_t v = i < nb ? sums[2 * i + c] : 0;
            uint64_t t;
            const uint64_t ex = block_exclusive_scan<kFBlock>(v, wb, &t);
            const uint64_t cc = carry[c];
            if (i < nb) sums[2 * i + c] = cc + ex;
            __syncthreads();
            if (threadIdx.x == 0) carry[c] = cc + t;
            __syncthreads();
        }
    }
    if (threadIdx.x < 2) tot[threadIdx.x] = carry[threadIdx.x];
}

__global__ void __launch_bounds__(kFBlock) k_rec_write(const uint64_t *__restrict__ nl, uint64_t r0,
                                                       uint64_t r1, const uint64_t *rr, int k,
                                                       const uint64_t *__restrict__ sums,
                                                       uint64_t *__restrict__ read_idx,
                                                       uint64_t *__restrict__ word_off) {
    __shared__ uint64_t wb[kFBlock / 32];
    rec_range(rr, r0, r1);
    const uint64_t nb = r1 > r0 ? (r1 - r0 + kGChunk - 1) / kGChunk : 0;
    for (uint64_t q = blockIdx.x; q < nb; q += gridDim.x) {
        const uint64_t base = r0 + q * kGChunk + (uint64_t)threadIdx.x * kGItems;
        uint32_t kept = 0;  // bit i: record base + i kept
        uint64_t wds[kGItems];
        uint64_t sk = 0, sw = 0;
#pragma unroll
        for (int it = 0; it < kGItems; ++it) {
            wds[it] = 0;
            if (base + it < r1) {
                const uint64_t L = rec_length(nl, base + it);
                if (L >= (uint64_t)k) {
                    kept |= 1u << it;
                    wds[it] = (L + 15) / 16;
                }
            }
            sk += (kept >> it) & 1u;
            sw += wds[it];
        }
        uint64_t rk = sums[2 * q] + block_exclusive_scan<kFBlock>(sk, wb, nullptr);
        uint64_t rw = sums[2 * q + 1] + block_exclusive_scan<kFBlock>(sw, wb, nullptr);
#pragma unroll
        for (int it = 0; it < kGItems; ++it) {
            if (base + it < r1) {
                read_idx[base + it] = rk;
                word_off[base + it] = rw;
            }
            rk += (kept >> it) & 1u;
            rw += wds[it];
        }
    }
}

// Streamed framing state (one thread). k_frame_prep: this piece's records
// are rr = [records framed so far, complete records through the piece),
// capped at rec_cap and at the newline positions written (nl_cap; past
// either, st->overflow). k_frame_advance: the piece's kept reads
// and words are added to the running totals, and its reads' range is put
// in piece_reads for the level-1 scatter (empty after an overflow).
__global__ void k_frame_prep(StreamState *st, uint64_t rec_cap, uint64_t nl_cap) {
    uint64_t r1 = st->newlines / 2;
    const uint64_t cap = rec_cap < nl_cap / 2 ? rec_cap : nl_cap / 2;
    if (r1 > cap || st->newlines > nl_cap) {
        r1 = r1 < cap ? r1 : cap;
        st->overflow = 1;
    }
    st->rec_range[0] = st->records;
    st->rec_range[1] = r1 > st->records ? r1 : st->records;
}

__global__ void k_frame_advance(StreamState *st, unsigned long long *piece_reads) {
    const uint64_t before = st->reads;
    st->reads += st->piece_reads;
    st->words += st->piece_words;
    st->records = st->rec_range[1];
    piece_reads[0] = before;
    piece_reads[1] = st->overflow ? before : st->reads;
}

__device__ __forceinline__ uint32_t code_of(unsigned char ch) {
    switch (ch) {
        case 'C': case 'c': return 1u;
        case 'G': case 'g': return 2u;
        case 'T': case 't': return 3u;
        default: return 0u;
    }
}

// Kept reads get their offset/length and packed words. A warp takes 32
// records at a time: each lane loads one record's newline positions, packed
// offset and read index (coalesced), a warp scan lays the 32 records' packed
// words out, and the lanes then build those words round-robin — every lane
// busy, each on the record its word falls in (binary search over the 33
// prefixes). A word (16 bases, first base in the top bits) comes from two
// aligned 16-byte loads of the text shifted by the record's alignment; four
// upper-case ACGT bytes at a time are mapped arithmetically, any other group
// of four byte by byte through a 256-entry table. Bases past the read are
// cleared. The text buffer has 64 bytes of slack past its end.
__global__ void __launch_bounds__(256) k_rec_pack(const unsigned char *__restrict__ t,
                                                  const uint64_t *__restrict__ nl, uint64_t r0,
                                                  uint64_t n_rec, int k,
                                                  const uint64_t *__restrict__ read_idx,
                                                  const uint64_t *__restrict__ word_off,
                                                  uint64_t read_base, uint64_t word_base,
                                                  uint64_t *__restrict__ off, uint32_t *__restrict__ len,
                                                  uint32_t *__restrict__ packed, StreamState *sst,
                                                  uint64_t reads_cap, uint64_t words_cap) {
    __shared__ unsigned char lut[256];
    __shared__ uint32_t s_pre[8][33];
    __shared__ uint64_t s_start[8][32], s_w0[8][32];
    __shared__ uint32_t s_len[8][32];
    lut[threadIdx.x] = (unsigned char)code_of((unsigned char)threadIdx.x);
    __syncthreads();
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    if (sst) {  // a streamed piece: its records, and the reads and words framed before it
        r0 = sst->rec_range[0];
        n_rec = sst->rec_range[1];
        read_base = sst->reads;
        word_base = sst->words;
    }
    for (uint64_t g0 = r0 + (((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; g0 < n_rec;
         g0 += nwarps * 32) {
        const uint64_t r = g0 + lane;
        uint64_t my_start = 0, my_w0 = 0;
        uint32_t my_len = 0, my_nw = 0;
        if (r < n_rec) {
            my_start = nl[2 * r] + 1;
            const uint64_t L = nl[2 * r + 1] - my_start;
            if (L >= (uint64_t)k) {
                const uint64_t ri = read_base + read_idx[r], w0 = word_base + word_off[r];
                const uint32_t nw = (uint32_t)((L + 15) / 16);
                if (ri < reads_cap && w0 + nw <= words_cap) {
                    my_len = (uint32_t)L;
                    my_nw = nw;
                    my_w0 = w0;
                    off[ri] = my_w0 * 16;
                    len[ri] = my_len;
                } else if (sst) {
                    sst->overflow = 1;  // only a streamed piece has caps below its totals
                }
            }
        }
        uint32_t inc = my_nw;  // inclusive warp scan of the word counts
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, inc, d);
            if (lane >= d) inc += y;
        }
        s_pre[wp][lane] = inc - my_nw;
        if (lane == 31) s_pre[wp][32] = inc;
        s_start[wp][lane] = my_start;
        s_w0[wp][lane] = my_w0;
        s_len[wp][lane] = my_len;
        __syncwarp();
        const uint32_t T = s_pre[wp][32];
        for (uint32_t tw = lane; tw < T; tw += 32) {
            uint32_t lo = 0, hi = 32;  // last record j with s_pre[j] <= tw
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) >> 1;
                if (s_pre[wp][mid] <= tw) lo = mid;
                else hi = mid;
            }
            const uint64_t start = s_start[wp][lo];
            const uint32_t w = tw - s_pre[wp][lo];
            const uint32_t q = (uint32_t)(start & 15) >> 2, sh = 8 * (uint32_t)(start & 3);
            const uint4 *a16 = reinterpret_cast<const uint4 *>(t + (start & ~15ull));
            const uint4 a = a16[w], b = a16[w + 1];
            const uint32_t win[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
            uint32_t sel[5];  // win[q .. q+4], selected without divergence
#pragma unroll
            for (int i = 0; i < 5; ++i)
                sel[i] = q == 0 ? win[i] : (q == 1 ? win[i + 1] : (q == 2 ? win[i + 2] : win[i + 3]));
            const uint32_t left = s_len[wp][lo] - 16 * w;  // bases of the read from this word on
            uint32_t word = 0;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const uint32_t x = __funnelshift_r(sel[i], sel[i + 1], sh);
                // upper-case A, C, G, T give ((b >> 1) ^ (b >> 2)) & 3 = 0, 1, 2, 3: four
                // such bytes are recognised by mapping their codes back to letters
                const uint32_t c = ((x >> 1) ^ (x >> 2)) & 0x03030303u;
                const uint32_t pick = __byte_perm(c | (c >> 4), 0, 0x0020);  // codes as selector nibbles
                uint32_t q4;
                if (__byte_perm(0x54474341u, 0, pick) == x) {  // "ACGT" indexed by the codes
                    q4 = (c * 0x40100401u) >> 24;                // code of byte b to bits 6-2b
                } else {
                    q4 = 0;
#pragma unroll
                    for (int bb = 0; bb < 4; ++bb) q4 |= (uint32_t)lut[(x >> (8 * bb)) & 0xffu] << (6 - 2 * bb);
                }
                word |= q4 << (24 - 8 * i);
            }
            if (left < 16) word &= 0xffffffffu << (32 - 2 * left);  // 1 <= left: bases past the read
            packed[s_w0[wp][lo] + w] = word;
        }
        __syncwarp();
    }
}

}  // namespace

uint64_t framing_chunks(uint64_t n) { return (n + kFChunk - 1) / kFChunk; }

uint64_t gscan_scratch(uint64_t n) { return (n + kGChunk - 1) / kGChunk + 1; }

int launch_gscan(const uint64_t *in, uint64_t *out, uint64_t n, uint64_t *scratch, uint64_t *total,
                 cudaStream_t s) {
    const uint64_t nb = (n + kGChunk - 1) / kGChunk;
    if (nb == 0) {
        cudaMemsetAsync(total, 0, sizeof(uint64_t), s);
        return 0;
    }
    if (nb <= 2) {
        k_gscan_small<<<1, kFBlock, 0, s>>>(in, n, out, total);
        return 1;
    }
    k_gscan_reduce<<<(unsigned)nb, kFBlock, 0, s>>>(in, n, scratch);
    k_gscan_blocks<<<1, kFBlock, 0, s>>>(scratch, nb, total);
    k_gscan_write<<<(unsigned)nb, kFBlock, 0, s>>>(in, n, scratch, out);
    return 3;
}

uint64_t rec_scan_scratch(uint64_t n_rec) { return 2 * ((n_rec + kGChunk - 1) / kGChunk) + 2; }

int launch_rec_scan(const uint64_t *nl, uint64_t r0, uint64_t n_rec, int k, uint64_t *scratch,
                    uint64_t *read_idx, uint64_t *word_off, uint64_t *tot, unsigned long long *acc,
                    cudaStream_t s) {
    const uint64_t nb = n_rec > r0 ? (n_rec - r0 + kGChunk - 1) / kGChunk : 0;
    if (nb == 0) {
        cudaMemsetAsync(tot, 0, 2 * sizeof(uint64_t), s);
        return 0;
    }
    k_rec_reduce<<<(unsigned)nb, kFBlock, 0, s>>>(nl, r0, n_rec, nullptr, k, scratch, acc);
    k_rec_blocks<<<1, kFBlock, 0, s>>>(scratch, r0, n_rec, nullptr, tot);
    k_rec_write<<<(unsigned)nb, kFBlock, 0, s>>>(nl, r0, n_rec, nullptr, k, scratch, read_idx, word_off);
    return 3;
}

int launch_frame_piece(const uint64_t *nl, uint64_t nl_cap, StreamState *st, uint64_t rec_cap, int k,
                       uint64_t *scratch,
                       uint64_t *read_idx, uint64_t *word_off, const unsigned char *t, uint64_t *off,
                       uint32_t *len, uint32_t *packed, uint64_t reads_cap, uint64_t words_cap,
                       unsigned long long *piece_reads, cudaStream_t s) {
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const unsigned grid = (unsigned)std::max(sms, 1) * 4;
    const uint64_t *rr = reinterpret_cast<const uint64_t *>(st->rec_range);
    uint64_t *piece_tot = reinterpret_cast<uint64_t *>(&st->piece_reads);  // piece_reads, piece_words
    k_frame_prep<<<1, 1, 0, s>>>(st, rec_cap, nl_cap);
    k_rec_reduce<<<grid, kFBlock, 0, s>>>(nl, 0, 0, rr, k, scratch, &st->occ);
    k_rec_blocks<<<1, kFBlock, 0, s>>>(scratch, 0, 0, rr, piece_tot);
    k_rec_write<<<grid, kFBlock, 0, s>>>(nl, 0, 0, rr, k, scratch, read_idx, word_off);
    k_rec_pack<<<grid * 4, 256, 0, s>>>(t, nl, 0, 0, k, read_idx, word_off, 0, 0, off, len, packed, st,
                                        reads_cap, words_cap);
    k_frame_advance<<<1, 1, 0, s>>>(st, piece_reads);
    return 6;
}

uint64_t newline_mask_words(uint64_t n) { return framing_chunks(n) * kFBlock; }

int launch_nl_count(const unsigned char *t, uint64_t n, uint64_t *counts, uint64_t *masks, unsigned *flag,
                    cudaStream_t s, uint64_t j0) {
    const uint64_t nc = framing_chunks(n);
    if (nc <= j0) return 0;
    k_nl_count<<<(unsigned)(nc - j0), kFBlock, 0, s>>>(t, n, counts, reinterpret_cast<unsigned long long *>(masks),
                                                      flag, j0);
    return 1;
}

int launch_nl_pos(const uint64_t *masks, uint64_t n, const uint64_t *chunk_base, uint64_t *nl, cudaStream_t s,
                  uint64_t j0, uint64_t cap, uint64_t *ovf) {
    const uint64_t nc = framing_chunks(n);
    if (nc <= j0) return 0;
    k_nl_pos<<<(unsigned)(nc - j0), kFBlock, 0, s>>>(reinterpret_cast<const unsigned long long *>(masks),
                                                    chunk_base, nl, j0, cap, ovf);
    return 1;
}

int launch_rec_pack(const unsigned char *t, const uint64_t *nl, uint64_t n_rec, int k,
                    const uint64_t *read_idx, const uint64_t *word_off, uint64_t *off,
                    uint32_t *len, uint32_t *packed, cudaStream_t s, uint64_t r0, uint64_t read_base,
                    uint64_t word_base) {
    if (n_rec <= r0) return 0;
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint64_t blocks = std::min<uint64_t>((n_rec - r0 + 255) / 256, (uint64_t)std::max(sms, 1) * 16);
    k_rec_pack<<<(unsigned)blocks, 256, 0, s>>>(t, nl, r0, n_rec, k, read_idx, word_off, read_base, word_base,
                                                off, len, packed, nullptr, ~0ull, ~0ull);
    return 1;
}

}  // namespace swg
