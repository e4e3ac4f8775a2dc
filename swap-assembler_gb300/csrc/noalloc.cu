// swg_build_device_noalloc: the graph build without any device allocation.
//
// Some callers cannot let a library call cudaMalloc: a service that reserves
// all of a GPU's memory for its own allocator at start-up (another runtime's
// caching pool or a fixed per-request budget) and must not have memory taken
// behind its back, or a pipeline where the device-wide synchronisation and
// the possible mid-run failure of cudaMalloc/cudaFree are not acceptable.
// For them this entry point keeps every scratch buffer of the build (hash
// table, occurrence prefix, tile table, control block) in one file-scope
// __device__ array of fixed size; the caller passes the reads and the output
// arrays, all in device memory.
//
// Limits: at most kNaMaxReads reads and kNaMaxOcc k-mer occurrences per call
// (the table then stays at most 60% full even if every occurrence is a new
// k-molecule); larger inputs are rejected with SWG_ERR_BAD_INPUT before any
// device work. The array (about 72 MiB) is held by every GPU that loads this
// code until the process exits.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "swg_internal.h"

namespace swg {
namespace {

constexpr uint64_t kNaTableEntries = 1ull << 22;  // 4,194,304 entries x 16 B = 64 MiB
constexpr uint64_t kNaMaxReads = 1ull << 20;      // 1,048,576 reads
constexpr uint64_t kNaMaxOcc = (kNaTableEntries - 128) * 3 / 5;
constexpr uint64_t kNaMaxTiles = kNaMaxOcc / kTileOcc + 2;
constexpr uint64_t kNaScanBlocks = kNaMaxReads / 2048 + 2;
constexpr int kNaMaxDevices = 64;

struct NaControl {
    unsigned status;
    unsigned pad;
    unsigned long long counters[2];  // inserted keys, survivors
};

struct NaScratch {
    Entry table[kNaTableEntries];
    uint64_t prefix[kNaMaxReads + 1];
    uint64_t scan[kNaScanBlocks];
    uint32_t tiles[kNaMaxTiles];
    NaControl ctl;
};

// The scratch itself. In host code this name is only a stand-in for the
// symbol; its device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) NaScratch g_noalloc_scratch;

// The array's device address per device, with the id of the context it was
// resolved in: a context destroyed and made again (cudaDeviceReset) gets a new
// id, and the address is resolved again in it.
struct NaSlot {
    unsigned long long ctx_id;
    NaScratch *ptr;
};
std::mutex g_na_mu;
NaSlot g_na_slot[kNaMaxDevices] = {};

// The driver's cuCtxGetCurrent / cuCtxGetId, looked up through the runtime
// (the library does not link the driver library itself). Result codes are the
// driver's CUresult: 0 = success.
typedef int (*CtxGetCurrentFn)(void **ctx);
typedef int (*CtxGetIdFn)(void *ctx, unsigned long long *id);

bool current_context_id(unsigned long long *id) {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    if (!get_current || !get_id) {
        void *f0 = nullptr, *f1 = nullptr;
        cudaDriverEntryPointQueryResult q0, q1;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 12000, cudaEnableDefault, &q0) != cudaSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
            q0 != cudaDriverEntryPointSuccess || q1 != cudaDriverEntryPointSuccess || !f0 || !f1)
            return false;
        get_current = reinterpret_cast<CtxGetCurrentFn>(f0);
        get_id = reinterpret_cast<CtxGetIdFn>(f1);
    }
    void *ctx = nullptr;
    if (get_current(&ctx) != 0 || !ctx) return false;
    return get_id(ctx, id) == 0;
}

swg_status na_resolve(NaScratch **p) {
    void *q = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&q, g_noalloc_scratch);
    if (e != cudaSuccess || !q) {
        set_error(std::string("cudaGetSymbolAddress of the no-allocation scratch: ") + cudaGetErrorString(e));
        return SWG_ERR_CUDA;
    }
    *p = static_cast<NaScratch *>(q);
    return SWG_OK;
}

// Once per device (and context), with that device current: resolve the
// array's device address. The first call on a device does this (it may load
// this module), and so does the first call after the device's context was
// destroyed; make those calls before any stream capture.
swg_status na_scratch(int dev, NaScratch **out) {
    if (dev < 0 || dev >= kNaMaxDevices) {
        set_error("device ordinal out of range for the no-allocation scratch");
        return SWG_ERR_BAD_INPUT;
    }
    std::lock_guard<std::mutex> lock(g_na_mu);
    NaSlot &slot = g_na_slot[dev];
    unsigned long long id = 0;
    if (!current_context_id(&id)) {
        // no context current in this thread yet: resolving the symbol makes the
        // device's primary context current, then its id can be read
        swg_status st = na_resolve(out);
        if (st) return st;
        if (!current_context_id(&id)) return SWG_OK;  // no id to cache by: resolved per call
        slot.ctx_id = id;
        slot.ptr = *out;
        return SWG_OK;
    }
    if (!slot.ptr || slot.ctx_id != id) {
        swg_status st = na_resolve(&slot.ptr);
        if (st) {
            slot.ptr = nullptr;
            return st;
        }
        slot.ctx_id = id;
    }
    *out = slot.ptr;
    return SWG_OK;
}

swg_status na_cuda(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return SWG_OK;
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    return SWG_ERR_CUDA;
}

}  // namespace
}  // namespace swg

// Calls share the one scratch array, which keeps the previous call's contents:
// the table and the control block are cleared at the start of every call.
// Two calls whose device work overlaps (different streams or host threads)
// race on the array and corrupt each other's results.
extern "C" swg_status swg_build_device_noalloc(const swg_opts *o, const uint32_t *d_packed,
                                               uint64_t n_words, const uint64_t *d_read_off,
                                               const uint32_t *d_read_len, uint64_t n_reads,
                                               uint64_t *d_keys_out, uint64_t *d_mult_out,
                                               uint64_t out_cap, uint64_t *n_out) {
    using namespace swg;
    if (!o || !n_out || o->k < 1 || o->k > 31) {
        set_error("bad arguments (opts, n_out, or k outside 1..31)");
        return SWG_ERR_BAD_INPUT;
    }
    *n_out = 0;
    if (n_reads > kNaMaxReads) {
        set_error("no-allocation build: at most 1048576 reads per call");
        return SWG_ERR_BAD_INPUT;
    }
    if (n_reads && (!d_packed || !d_read_off || !d_read_len)) {
        set_error("NULL read buffer");
        return SWG_ERR_BAD_INPUT;
    }
    int dev = 0;
    swg_status st = na_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    if (st) return st;
    NaScratch *sc = nullptr;
    if ((st = na_scratch(dev, &sc))) return st;
    cudaStream_t s = (cudaStream_t)o->stream;

    BuildArgs a;
    std::memset(&a, 0, sizeof(a));
    a.packed = d_packed;
    a.n_words = n_words;
    a.read_off = d_read_off;
    a.read_len = d_read_len;
    a.n_reads = n_reads;
    a.k = o->k;
    a.cutoff = o->cutoff;
    a.occ_prefix = sc->prefix;
    a.scan_blocks = sc->scan;
    a.tile_first_read = sc->tiles;
    a.status = &sc->ctl.status;
    a.counters = sc->ctl.counters;

    if ((st = na_cuda(cudaMemsetAsync(&sc->ctl, 0, sizeof(NaControl), s), "clear control"))) return st;
    if ((st = na_cuda(cudaMemsetAsync(sc->prefix, 0, sizeof(uint64_t), s), "clear prefix"))) return st;
    launch_occ_scan(a, s);
    if ((st = na_cuda(cudaGetLastError(), "occurrence scan launch"))) return st;
    uint64_t total = 0;
    if ((st = na_cuda(cudaMemcpyAsync(&total, sc->prefix + n_reads, sizeof(total),
                                      cudaMemcpyDeviceToHost, s), "read occurrence total")))
        return st;
    if ((st = na_cuda(cudaStreamSynchronize(s), "occurrence scan"))) return st;
    if (total > kNaMaxOcc) {
        set_error("no-allocation build: at most 2516505 k-mer occurrences per call");
        return SWG_ERR_BAD_INPUT;
    }
    a.total_occ = total;
    a.n_tiles = (total + kTileOcc - 1) / kTileOcc;
    uint64_t cap = (uint64_t)std::ceil((double)total / 0.6) + 64;
    if (cap > kNaTableEntries) cap = kNaTableEntries;
    a.table = sc->table;
    a.cap = cap;
    a.out_keys = reinterpret_cast<unsigned long long *>(d_keys_out);
    a.out_mult = reinterpret_cast<unsigned long long *>(d_mult_out);
    a.out_cap = d_keys_out && d_mult_out ? out_cap : 0;
    launch_tiles(a, s);
    if ((st = na_cuda(cudaMemsetAsync(sc->table, 0, cap * sizeof(Entry), s), "clear table")))
        return st;
    launch_count(a, s);
    launch_compact(a, s);
    if ((st = na_cuda(cudaGetLastError(), "build launch"))) return st;
    NaControl ctl;
    if ((st = na_cuda(cudaMemcpyAsync(&ctl, &sc->ctl, sizeof(ctl), cudaMemcpyDeviceToHost, s),
                      "read status")))
        return st;
    if ((st = na_cuda(cudaStreamSynchronize(s), "build"))) return st;
    if (ctl.status & kStatusCasLimit) {
        set_error("a bounded CAS retry loop gave up on the device");
        return SWG_ERR_TIMEOUT;
    }
    if (ctl.status & kStatusTableFull) {
        set_error("no-allocation build: hash table probe limit reached");
        return SWG_ERR_TABLE_FULL;
    }
    *n_out = ctl.counters[1];
    if (ctl.counters[1] > a.out_cap) {
        set_error("output arrays too small: n_out holds the survivor count needed");
        return SWG_ERR_BAD_INPUT;
    }
    return SWG_OK;
}
