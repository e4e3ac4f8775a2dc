// Request server: continuous batching of graph builds on one GPU.
//
// Clients submit single-sample requests (packed reads in host memory, their
// own k and cutoff) at any time. Submission uploads the reads to device
// memory (an upload runs at the host link's rate; a host copy into fresh
// pages was the submitting thread's bottleneck), so the caller may free them
// on return. Worker threads, each with its own graph handle and CUDA stream,
// repeatedly take every queued request that fits the device-memory budget (in
// arrival order) and build them as one batch (swg_batch_build on the
// device-resident reads); with two or more workers, batches overlap on the device.
// Each request's filtered graph is then copied to its own device buffer and
// stays resident until the client fetches or releases it. Admission: a
// request is charged an estimated footprint while its batch runs (inputs,
// table and outputs sized by its k-mer occurrence count, an upper bound on its
// distinct k-molecules) and its exact result size while resident; a request
// larger than the whole budget is refused at submission.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "swg_internal.h"

namespace {

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Request {
    uint64_t ticket = 0;
    uint32_t *d_packed = nullptr;  // the reads, uploaded at submission (freed after the build)
    uint64_t *d_off = nullptr;
    uint32_t *d_len = nullptr;
    uint64_t n_words = 0, n_reads = 0;
    uint64_t in_bytes = 0;  // device bytes of the uploaded reads
    int k = 0, cutoff = 0;
    uint64_t occ = 0;
    uint64_t footprint = 0;
    int state = SWG_REQ_QUEUED;
    swg_status status = SWG_OK;
    std::string error;
    uint64_t n_out = 0, distinct = 0;
    unsigned long long *d_keys = nullptr, *d_mult = nullptr;
    uint64_t resident = 0;
    double t_submit = 0, t_done = 0;
};

}  // namespace

struct swg_server {
    swg_server_opts opts;
    int device = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request *> queue;
    std::unordered_map<uint64_t, Request *> reqs;
    uint64_t next_ticket = 1;
    uint64_t reserved = 0;  // in-flight footprints
    uint64_t resident = 0;  // results waiting to be fetched
    uint64_t queued = 0;    // device bytes of the uploaded reads of queued requests (charged to the
                            // budget with the rest of the footprint once a worker takes the request)
    std::mutex upload_mu;   // one upload at a time on upload_stream
    cudaStream_t upload_stream = nullptr;
    swg_server_stats st;
    bool stop = false;
    uint32_t live_workers = 0;  // workers whose set-up succeeded or is still under way
    std::string dead_error;     // set when every worker failed its set-up
    std::vector<std::thread> workers;
    cudaStream_t fetch_stream = nullptr;
};

namespace {

// Inputs + 32 B per table slot at the load factor (about 53 B per k-mer
// occurrence at 0.6: covers the direct build's table and output and the
// bucketed build's record buffers and output, at most 40 B per occurrence)
// + 16 MiB for the bucketed build's fixed region slack.
uint64_t footprint_of(uint64_t reads, uint64_t words, uint64_t occ, double load) {
    const uint64_t cap = (uint64_t)((double)occ / load) + 2048;
    return words * 4 + reads * (8 + 4 + 8 + 4) + cap * 16 * 2 + (16ull << 20);
}

void free_inputs(Request *r, cudaStream_t s) {
    if (r->d_packed) cudaFreeAsync(r->d_packed, s);
    if (r->d_off) cudaFreeAsync(r->d_off, s);
    if (r->d_len) cudaFreeAsync(r->d_len, s);
    r->d_packed = nullptr;
    r->d_off = nullptr;
    r->d_len = nullptr;
}

// A worker whose set-up failed leaves; when the last one does, every queued
// request fails with the reason and later submissions are refused with it.
void worker_setup_failed(swg_server *srv, swg_status st, const std::string &why) {
    std::lock_guard<std::mutex> lock(srv->mu);
    if (--srv->live_workers == 0) {
        srv->dead_error = "request server has no working worker: " + why;
        for (Request *r : srv->queue) {
            srv->queued -= r->in_bytes;
            free_inputs(r, srv->upload_stream);
            r->state = SWG_REQ_FAILED;
            r->status = st;
            r->error = srv->dead_error;
            r->t_done = now_s();
            srv->st.failed++;
        }
        srv->queue.clear();
    }
    srv->cv_done.notify_all();
}

void worker_main(swg_server *srv) {
    cudaError_t ce = cudaSetDevice(srv->device);
    if (ce != cudaSuccess) {
        worker_setup_failed(srv, SWG_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(ce));
        return;
    }
    swg_graph *g = nullptr;
    swg_status gs = swg_graph_create(&g);
    if (gs != SWG_OK) {
        worker_setup_failed(srv, gs, std::string("graph handle: ") + swg_last_error());
        return;
    }
    cudaStream_t stream = nullptr;
    ce = cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
    if (ce != cudaSuccess) {
        swg_graph_free(g);
        worker_setup_failed(srv, SWG_ERR_CUDA, std::string("stream creation: ") + cudaGetErrorString(ce));
        return;
    }
    swg_opts o;
    std::memset(&o, 0, sizeof(o));
    o.load_factor = srv->opts.load_factor;
    o.stream = stream;
    for (;;) {
        std::vector<Request *> batch;
        {
            std::unique_lock<std::mutex> lock(srv->mu);
            for (;;) {
                if (srv->stop) break;
                // Requests in arrival order while they fit the budget. A batch
                // runs as one tagged bucketed build only while its samples'
                // indices fit above the largest k-mer (2 k_max + ceil(log2
                // samples) <= 64 bits): a request that would break that waits
                // for a later batch, and the requests behind it may join.
                int kmax = 0;
                for (auto it = srv->queue.begin(); it != srv->queue.end();) {
                    Request *r = *it;
                    if (srv->reserved + srv->resident + r->footprint > srv->opts.memory_budget)
                        break;  // waits until memory frees up (arrival order is kept)
                    const int km = std::max(kmax, r->k);
                    int tb = 0;
                    while ((size_t(1) << tb) < batch.size() + 1) tb++;
                    if (!batch.empty() && (2 * km + tb > 64 || batch.size() + 1 > swg::kMaxTagSamples)) {
                        ++it;
                        continue;
                    }
                    kmax = km;
                    it = srv->queue.erase(it);
                    srv->queued -= r->in_bytes;
                    srv->reserved += r->footprint;
                    r->state = SWG_REQ_RUNNING;
                    batch.push_back(r);
                    if (srv->opts.max_batch && batch.size() >= srv->opts.max_batch) break;
                }
                if (!batch.empty()) break;
                srv->cv_work.wait(lock);
            }
            if (batch.empty()) break;  // stopping
            srv->st.batches++;
            srv->st.max_batch_requests = std::max<uint64_t>(srv->st.max_batch_requests, batch.size());
        }
        std::vector<swg_sample> samples(batch.size());
        for (size_t i = 0; i < batch.size(); i++) {
            Request *r = batch[i];
            samples[i].packed = r->d_packed;
            samples[i].n_words = r->n_words;
            samples[i].read_off = r->d_off;
            samples[i].read_len = r->d_len;
            samples[i].n_reads = r->n_reads;
            samples[i].k = r->k;
            samples[i].cutoff = r->cutoff;
        }
        swg_status bs = swg_batch_build(g, &o, samples.data(), (uint32_t)samples.size());
        std::string berr = bs ? swg_last_error() : "";
        std::vector<swg_status> rs(batch.size(), bs);
        for (size_t i = 0; bs == SWG_OK && i < batch.size(); i++) {
            Request *r = batch[i];
            const uint64_t *dk = nullptr, *dm = nullptr;
            uint64_t n = 0, occ = 0, distinct = 0;
            swg_batch_device_view(g, (uint32_t)i, &dk, &dm, &n);
            swg_batch_sample_info(g, (uint32_t)i, &occ, &distinct, nullptr);
            r->n_out = n;
            r->distinct = distinct;
            if (n) {
                cudaError_t e = cudaMallocAsync(&r->d_keys, n * 8, stream);
                if (e == cudaSuccess) e = cudaMallocAsync(&r->d_mult, n * 8, stream);
                if (e == cudaSuccess)
                    e = cudaMemcpyAsync(r->d_keys, dk, n * 8, cudaMemcpyDeviceToDevice, stream);
                if (e == cudaSuccess)
                    e = cudaMemcpyAsync(r->d_mult, dm, n * 8, cudaMemcpyDeviceToDevice, stream);
                if (e != cudaSuccess) {
                    cudaGetLastError();
                    rs[i] = e == cudaErrorMemoryAllocation ? SWG_ERR_OOM : SWG_ERR_CUDA;
                    r->error = cudaGetErrorString(e);
                }
            }
        }
        for (Request *r : batch) free_inputs(r, stream);  // the inputs are no longer needed
        cudaStreamSynchronize(stream);
        {
            std::lock_guard<std::mutex> lock(srv->mu);
            const double t = now_s();
            for (size_t i = 0; i < batch.size(); i++) {
                Request *r = batch[i];
                srv->reserved -= r->footprint;
                r->t_done = t;
                r->status = rs[i];
                if (rs[i] == SWG_OK) {
                    r->state = SWG_REQ_DONE;
                    r->resident = r->n_out * 16;
                    srv->resident += r->resident;
                    srv->st.completed++;
                } else {
                    r->state = SWG_REQ_FAILED;
                    if (r->error.empty()) r->error = berr;
                    srv->st.failed++;
                }
            }
        }
        srv->cv_done.notify_all();
        srv->cv_work.notify_all();
    }
    cudaStreamSynchronize(stream);
    cudaStreamDestroy(stream);
    swg_graph_free(g);
}

void free_result(swg_server *srv, Request *r) {
    if (r->d_keys) cudaFreeAsync(r->d_keys, srv->fetch_stream);
    if (r->d_mult) cudaFreeAsync(r->d_mult, srv->fetch_stream);
    r->d_keys = r->d_mult = nullptr;
}

}  // namespace

extern "C" {

swg_status swg_server_create(const swg_server_opts *o, swg_server **out) {
    if (!out) return SWG_ERR_BAD_INPUT;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        swg::set_error("no CUDA device visible");
        return SWG_ERR_NO_DEVICE;
    }
    swg_server *srv = new (std::nothrow) swg_server;
    if (!srv) return SWG_ERR_OOM;
    std::memset(&srv->opts, 0, sizeof(srv->opts));
    if (o) srv->opts = *o;
    if (!srv->opts.memory_budget) srv->opts.memory_budget = 150ull << 30;
    if (!srv->opts.workers) srv->opts.workers = 2;
    if (srv->opts.load_factor <= 0 || srv->opts.load_factor > 0.9) srv->opts.load_factor = 0.6;
    std::memset(&srv->st, 0, sizeof(srv->st));
    cudaGetDevice(&srv->device);
    if (cudaStreamCreateWithFlags(&srv->fetch_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&srv->upload_stream, cudaStreamNonBlocking) != cudaSuccess) {
        if (srv->fetch_stream) cudaStreamDestroy(srv->fetch_stream);
        delete srv;
        swg::set_error("stream creation failed");
        return SWG_ERR_CUDA;
    }
    srv->live_workers = srv->opts.workers;
    for (uint32_t i = 0; i < srv->opts.workers; i++) srv->workers.emplace_back(worker_main, srv);
    *out = srv;
    return SWG_OK;
}

swg_status swg_server_submit(swg_server *srv, const swg_sample *req, uint64_t *ticket) {
    if (!srv || !req || !ticket) return SWG_ERR_BAD_INPUT;
    if (req->k < 1 || req->k > 31) {
        swg::set_error("k must be in 1..31");
        return SWG_ERR_BAD_INPUT;
    }
    if (req->n_reads && (!req->packed || !req->read_off || !req->read_len)) {
        swg::set_error("NULL read buffer");
        return SWG_ERR_BAD_INPUT;
    }
    const double t0 = now_s();
    Request *r = new (std::nothrow) Request;
    if (!r) return SWG_ERR_OOM;
    r->k = req->k;
    r->cutoff = req->cutoff;
    r->n_words = req->n_words;
    r->n_reads = req->n_reads;
    r->in_bytes = req->n_words * 4 + req->n_reads * 12;
    const uint32_t k = (uint32_t)req->k;
    uint64_t occ = 0;
    for (uint64_t i = 0; i < req->n_reads; i++) {
        const uint32_t L = req->read_len[i];
        occ += L >= k ? L - k + 1 : 0;
    }
    r->occ = occ;
    r->footprint = footprint_of(req->n_reads, req->n_words, r->occ, srv->opts.load_factor);
    r->t_submit = t0;
    {
        std::lock_guard<std::mutex> lock(srv->mu);
        swg_status refuse = SWG_OK;
        if (r->footprint > srv->opts.memory_budget) {
            srv->st.rejected++;
            swg::set_error("request footprint exceeds the server's memory budget");
            refuse = SWG_ERR_ADMISSION;
        } else if (srv->stop) {
            refuse = SWG_ERR_BAD_STATE;
        } else if (!srv->dead_error.empty()) {
            swg::set_error(srv->dead_error);
            refuse = SWG_ERR_BAD_STATE;
        }
        if (refuse) {
            delete r;
            return refuse;
        }
        srv->queued += r->in_bytes;
    }
    // upload the reads (the caller may free its buffers once this returns)
    cudaError_t e = cudaSetDevice(srv->device);
    {
        std::lock_guard<std::mutex> up(srv->upload_mu);
        cudaStream_t us = srv->upload_stream;
        if (e == cudaSuccess && r->n_words) e = cudaMallocAsync((void **)&r->d_packed, r->n_words * 4, us);
        if (e == cudaSuccess && r->n_reads) e = cudaMallocAsync((void **)&r->d_off, r->n_reads * 8, us);
        if (e == cudaSuccess && r->n_reads) e = cudaMallocAsync((void **)&r->d_len, r->n_reads * 4, us);
        if (e == cudaSuccess && r->n_words)
            e = cudaMemcpyAsync(r->d_packed, req->packed, r->n_words * 4, cudaMemcpyHostToDevice, us);
        if (e == cudaSuccess && r->n_reads)
            e = cudaMemcpyAsync(r->d_off, req->read_off, r->n_reads * 8, cudaMemcpyHostToDevice, us);
        if (e == cudaSuccess && r->n_reads)
            e = cudaMemcpyAsync(r->d_len, req->read_len, r->n_reads * 4, cudaMemcpyHostToDevice, us);
        if (e == cudaSuccess) e = cudaStreamSynchronize(us);
        if (e != cudaSuccess) {
            cudaGetLastError();
            free_inputs(r, us);
            cudaStreamSynchronize(us);
        }
    }
    std::lock_guard<std::mutex> lock(srv->mu);
    if (e != cudaSuccess) {
        srv->queued -= r->in_bytes;
        delete r;
        swg::set_error(std::string("request upload: ") + cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? SWG_ERR_OOM : SWG_ERR_CUDA;
    }
    if (srv->stop) {
        srv->queued -= r->in_bytes;
        free_inputs(r, srv->upload_stream);
        delete r;
        return SWG_ERR_BAD_STATE;
    }
    r->ticket = srv->next_ticket++;
    srv->reqs[r->ticket] = r;
    srv->queue.push_back(r);
    srv->st.submitted++;
    *ticket = r->ticket;
    srv->cv_work.notify_one();
    return SWG_OK;
}

swg_status swg_server_poll(swg_server *srv, uint64_t ticket, int *state, double *latency_s) {
    if (!srv) return SWG_ERR_BAD_INPUT;
    std::lock_guard<std::mutex> lock(srv->mu);
    auto it = srv->reqs.find(ticket);
    if (it == srv->reqs.end()) return SWG_ERR_BAD_INPUT;
    Request *r = it->second;
    if (state) *state = r->state;
    if (latency_s) *latency_s = r->t_done > 0 ? r->t_done - r->t_submit : now_s() - r->t_submit;
    return SWG_OK;
}

swg_status swg_server_wait(swg_server *srv, uint64_t ticket, double timeout_s) {
    if (!srv) return SWG_ERR_BAD_INPUT;
    std::unique_lock<std::mutex> lock(srv->mu);
    auto it = srv->reqs.find(ticket);
    if (it == srv->reqs.end()) return SWG_ERR_BAD_INPUT;
    Request *r = it->second;
    const auto until = std::chrono::steady_clock::now() +
                       std::chrono::duration_cast<std::chrono::steady_clock::duration>(
                           std::chrono::duration<double>(timeout_s));
    while (r->state == SWG_REQ_QUEUED || r->state == SWG_REQ_RUNNING) {
        if (srv->cv_done.wait_until(lock, until) == std::cv_status::timeout &&
            (r->state == SWG_REQ_QUEUED || r->state == SWG_REQ_RUNNING))
            return SWG_ERR_NOT_READY;
    }
    if (r->state == SWG_REQ_FAILED) {
        swg::set_error(r->error);
        return r->status;
    }
    return SWG_OK;
}

swg_status swg_server_result_info(swg_server *srv, uint64_t ticket, uint64_t *survivors,
                                  uint64_t *distinct) {
    if (!srv) return SWG_ERR_BAD_INPUT;
    std::lock_guard<std::mutex> lock(srv->mu);
    auto it = srv->reqs.find(ticket);
    if (it == srv->reqs.end()) return SWG_ERR_BAD_INPUT;
    Request *r = it->second;
    if (r->state == SWG_REQ_FAILED) return r->status;
    if (r->state != SWG_REQ_DONE) return SWG_ERR_NOT_READY;
    if (survivors) *survivors = r->n_out;
    if (distinct) *distinct = r->distinct;
    return SWG_OK;
}

swg_status swg_server_fetch(swg_server *srv, uint64_t ticket, uint64_t *keys, uint8_t *mult,
                            uint64_t cap, int sorted, uint64_t *n) {
    if (!srv) return SWG_ERR_BAD_INPUT;
    Request *r = nullptr;
    {
        std::lock_guard<std::mutex> lock(srv->mu);
        auto it = srv->reqs.find(ticket);
        if (it == srv->reqs.end()) return SWG_ERR_BAD_INPUT;
        r = it->second;
        if (r->state == SWG_REQ_FAILED) {
            swg::set_error(r->error);
            return r->status;
        }
        if (r->state != SWG_REQ_DONE) return SWG_ERR_NOT_READY;
        if (n) *n = r->n_out;
        if (cap < r->n_out) {
            swg::set_error("output capacity smaller than the survivor count");
            return SWG_ERR_BAD_INPUT;
        }
        srv->reqs.erase(it);  // the caller owns the result from here
    }
    swg_status st = SWG_OK;
    cudaSetDevice(srv->device);
    if (r->n_out) {
        std::vector<uint64_t> k(r->n_out), m(r->n_out);
        cudaError_t e = cudaMemcpyAsync(k.data(), r->d_keys, r->n_out * 8, cudaMemcpyDeviceToHost,
                                        srv->fetch_stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(m.data(), r->d_mult, r->n_out * 8, cudaMemcpyDeviceToHost,
                                srv->fetch_stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(srv->fetch_stream);
        if (e != cudaSuccess) {
            swg::set_error(std::string("fetch: ") + cudaGetErrorString(e));
            st = SWG_ERR_CUDA;
        } else {
            if (sorted) swg::sort_records(k.data(), m.data(), r->n_out);
            if (keys) std::memcpy(keys, k.data(), r->n_out * 8);
            if (mult) std::memcpy(mult, m.data(), r->n_out * 8);
        }
    }
    free_result(srv, r);
    {
        std::lock_guard<std::mutex> lock(srv->mu);
        srv->resident -= r->resident;
    }
    srv->cv_work.notify_all();
    delete r;
    return st;
}

swg_status swg_server_release(swg_server *srv, uint64_t ticket) {
    if (!srv) return SWG_ERR_BAD_INPUT;
    Request *r = nullptr;
    {
        std::lock_guard<std::mutex> lock(srv->mu);
        auto it = srv->reqs.find(ticket);
        if (it == srv->reqs.end()) return SWG_ERR_BAD_INPUT;
        r = it->second;
        if (r->state == SWG_REQ_QUEUED || r->state == SWG_REQ_RUNNING) return SWG_ERR_NOT_READY;
        srv->reqs.erase(it);
        srv->resident -= r->resident;
    }
    cudaSetDevice(srv->device);
    free_result(srv, r);
    srv->cv_work.notify_all();
    delete r;
    return SWG_OK;
}

swg_status swg_server_get_stats(swg_server *srv, swg_server_stats *out) {
    if (!srv || !out) return SWG_ERR_BAD_INPUT;
    std::lock_guard<std::mutex> lock(srv->mu);
    *out = srv->st;
    out->queued = srv->queue.size();
    out->bytes_reserved = srv->reserved;
    out->bytes_resident = srv->resident;
    return SWG_OK;
}

void swg_server_free(swg_server *srv) {
    if (!srv) return;
    {
        std::lock_guard<std::mutex> lock(srv->mu);
        srv->stop = true;
    }
    srv->cv_work.notify_all();
    for (auto &t : srv->workers) t.join();
    cudaSetDevice(srv->device);
    for (auto &kv : srv->reqs) {
        free_inputs(kv.second, srv->fetch_stream);
        free_result(srv, kv.second);
        delete kv.second;
    }
    cudaStreamSynchronize(srv->fetch_stream);
    cudaStreamDestroy(srv->fetch_stream);
    cudaStreamSynchronize(srv->upload_stream);
    cudaStreamDestroy(srv->upload_stream);
    delete srv;
}

}  // extern "C"
