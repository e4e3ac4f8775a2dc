// Single-rank MPI shim — TEST INFRASTRUCTURE ONLY (see mpi.h for scope).
//
// Semantics with one rank:
//   * collectives copy the send buffer to the receive buffer (root/peer is 0);
//   * Send/Isend to self are buffered in a FIFO per tag and matched by
//     Recv/Irecv (first matching tag, or any tag); a Send that matches an
//     already-posted Irecv completes it directly (graph.cpp:667,677 posts the
//     receive before the send);
//   * a wait that can never complete with one rank aborts the process with a
//     message (never blocks).
#include "mpi.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <string>
#include <vector>

namespace {

struct Msg {
    int tag;
    std::vector<char> data;
};

struct Req {
    bool active = false;
    bool done = false;
    bool is_recv = false;
    void *buf = nullptr;
    long long cap = 0;
    int tag = 0;
    long long got = 0;
    int got_tag = 0;
};

std::deque<Msg> g_inbox;
std::vector<Req> g_reqs;
std::vector<long long> g_type_size(6, 0);

[[noreturn]] void die(const char *what) {
    std::fprintf(stderr, "mpi shim: %s (single-rank shim)\n", what);
    std::fflush(stderr);
    std::abort();
}

long long tsize(MPI_Datatype t) {
    if (t <= 0 || (size_t)t >= g_type_size.size() || g_type_size[t] == 0) die("unknown datatype");
    return g_type_size[t];
}

void init_types() {
    if (g_type_size[MPI_CHAR]) return;
    g_type_size[MPI_CHAR] = 1;
    g_type_size[MPI_INT] = sizeof(int);
    g_type_size[MPI_UNSIGNED_LONG_LONG] = sizeof(unsigned long long);
    g_type_size[MPI_LONG_LONG_INT] = sizeof(long long);
    g_type_size[MPI_DOUBLE] = sizeof(double);
}

void copy_n(void *dst, const void *src, long long bytes) {
    if (bytes > 0 && dst != src) std::memmove(dst, src, (size_t)bytes);
}

bool tag_match(int want, int have) { return want == MPI_ANY_TAG || want == have; }

int new_req() {
    for (size_t i = 0; i < g_reqs.size(); ++i)
        if (!g_reqs[i].active) { g_reqs[i] = Req(); g_reqs[i].active = true; return (int)i; }
    g_reqs.emplace_back();
    g_reqs.back().active = true;
    return (int)g_reqs.size() - 1;
}

void fill_status(MPI_Status *st, int tag, long long bytes) {
    if (!st) return;
    st->MPI_SOURCE = 0;
    st->MPI_TAG = tag;
    st->MPI_ERROR = MPI_SUCCESS;
    st->shim_bytes = bytes;
}

// Deliver a message: complete the oldest posted receive with a matching tag,
// else queue it.
void deliver(const void *buf, long long bytes, int tag) {
    for (auto &r : g_reqs) {
        if (r.active && r.is_recv && !r.done && tag_match(r.tag, tag)) {
            if (bytes > r.cap) die("message larger than posted receive");
            copy_n(r.buf, buf, bytes);
            r.got = bytes;
            r.got_tag = tag;
            r.done = true;
            return;
        }
    }
    Msg m;
    m.tag = tag;
    m.data.assign((const char *)buf, (const char *)buf + bytes);
    g_inbox.push_back(std::move(m));
}

bool take(void *buf, long long cap, int tag, long long *got, int *got_tag) {
    for (auto it = g_inbox.begin(); it != g_inbox.end(); ++it) {
        if (tag_match(tag, it->tag)) {
            if ((long long)it->data.size() > cap) die("message larger than receive buffer");
            copy_n(buf, it->data.data(), (long long)it->data.size());
            *got = (long long)it->data.size();
            *got_tag = it->tag;
            g_inbox.erase(it);
            return true;
        }
    }
    return false;
}

}  // namespace

struct shim_mpi_file {
    FILE *fp;
};

extern "C" {

int MPI_Init(int *, char ***) { init_types(); return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Abort(MPI_Comm, int code) { std::exit(code); }
int MPI_Comm_rank(MPI_Comm, int *rank) { *rank = 0; return MPI_SUCCESS; }
int MPI_Comm_size(MPI_Comm, int *size) { *size = 1; return MPI_SUCCESS; }
int MPI_Get_processor_name(char *name, int *len) {
    std::strcpy(name, "shim-rank0");
    *len = (int)std::strlen(name);
    return MPI_SUCCESS;
}

int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype *out) {
    init_types();
    g_type_size.push_back(tsize(old) * count);
    *out = (MPI_Datatype)g_type_size.size() - 1;
    return MPI_SUCCESS;
}
int MPI_Type_commit(MPI_Datatype *) { return MPI_SUCCESS; }

int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
int MPI_Ibarrier(MPI_Comm, MPI_Request *req) {
    *req = new_req();
    g_reqs[*req].done = true;
    return MPI_SUCCESS;
}
int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }
int MPI_Reduce(const void *s, void *r, int count, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
    copy_n(r, s, count * tsize(t));
    return MPI_SUCCESS;
}
int MPI_Allreduce(const void *s, void *r, int count, MPI_Datatype t, MPI_Op, MPI_Comm) {
    copy_n(r, s, count * tsize(t));
    return MPI_SUCCESS;
}
int MPI_Scan(const void *s, void *r, int count, MPI_Datatype t, MPI_Op, MPI_Comm) {
    copy_n(r, s, count * tsize(t));
    return MPI_SUCCESS;
}
int MPI_Gather(const void *s, int scount, MPI_Datatype st, void *r, int, MPI_Datatype, int, MPI_Comm) {
    copy_n(r, s, scount * tsize(st));
    return MPI_SUCCESS;
}
int MPI_Alltoall(const void *s, int scount, MPI_Datatype st, void *r, int, MPI_Datatype, MPI_Comm) {
    copy_n(r, s, scount * tsize(st));
    return MPI_SUCCESS;
}
int MPI_Alltoallv(const void *s, const int *scounts, const int *sdispls, MPI_Datatype st, void *r,
                  const int *, const int *rdispls, MPI_Datatype, MPI_Comm) {
    long long e = tsize(st);
    copy_n((char *)r + (long long)rdispls[0] * e, (const char *)s + (long long)sdispls[0] * e,
           (long long)scounts[0] * e);
    return MPI_SUCCESS;
}

int MPI_Send(const void *buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm) {
    if (dest != 0) die("send to a rank other than 0");
    deliver(buf, (long long)count * tsize(t), tag);
    return MPI_SUCCESS;
}
int MPI_Isend(const void *buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm c,
              MPI_Request *req) {
    MPI_Send(buf, count, t, dest, tag, c);
    *req = new_req();
    g_reqs[*req].done = true;
    return MPI_SUCCESS;
}
int MPI_Recv(void *buf, int count, MPI_Datatype t, int src, int tag, MPI_Comm, MPI_Status *st) {
    if (src != 0 && src != MPI_ANY_SOURCE) die("receive from a rank other than 0");
    long long got = 0;
    int got_tag = 0;
    if (!take(buf, (long long)count * tsize(t), tag, &got, &got_tag))
        die("blocking receive with no matching message would wait forever");
    fill_status(st, got_tag, got);
    return MPI_SUCCESS;
}
int MPI_Irecv(void *buf, int count, MPI_Datatype t, int src, int tag, MPI_Comm, MPI_Request *req) {
    if (src != 0 && src != MPI_ANY_SOURCE) die("receive from a rank other than 0");
    int id = new_req();
    Req &r = g_reqs[id];
    r.is_recv = true;
    r.buf = buf;
    r.cap = (long long)count * tsize(t);
    r.tag = tag;
    if (take(buf, r.cap, tag, &r.got, &r.got_tag)) r.done = true;
    *req = id;
    return MPI_SUCCESS;
}
int MPI_Test(MPI_Request *req, int *flag, MPI_Status *st) {
    Req &r = g_reqs.at(*req);
    *flag = r.done ? 1 : 0;
    if (r.done) {
        fill_status(st, r.got_tag, r.got);
        r.active = false;
    }
    return MPI_SUCCESS;
}
// The status array is left untouched: the merge stage's service loop
// (graph.cpp:1214, 1232) allocates one status per rank but tests up to four
// requests, and never reads the statuses. Filling n of them would write past
// that allocation when the job has fewer than four ranks.
int MPI_Testall(int n, MPI_Request *reqs, int *flag, MPI_Status *) {
    int all = 1;
    for (int i = 0; i < n; ++i) all &= g_reqs.at(reqs[i]).done ? 1 : 0;
    *flag = all;
    if (all)
        for (int i = 0; i < n; ++i) {
            int f;
            MPI_Test(&reqs[i], &f, nullptr);
        }
    return MPI_SUCCESS;
}
int MPI_Wait(MPI_Request *req, MPI_Status *st) {
    int f = 0;
    MPI_Test(req, &f, st);
    if (!f) die("wait on a request that no rank can complete");
    return MPI_SUCCESS;
}
int MPI_Waitall(int n, MPI_Request *reqs, MPI_Status *sts) {
    for (int i = 0; i < n; ++i) MPI_Wait(&reqs[i], sts ? &sts[i] : nullptr);
    return MPI_SUCCESS;
}
int MPI_Iprobe(int, int tag, MPI_Comm, int *flag, MPI_Status *st) {
    *flag = 0;
    for (auto &m : g_inbox)
        if (tag_match(tag, m.tag)) {
            *flag = 1;
            fill_status(st, m.tag, (long long)m.data.size());
            break;
        }
    return MPI_SUCCESS;
}

int MPI_File_open(MPI_Comm, const char *name, int amode, MPI_Info, MPI_File *fh) {
    const char *mode = (amode & MPI_MODE_RDONLY) ? "rb" : ((amode & MPI_MODE_CREATE) ? "wb" : "r+b");
    FILE *fp = std::fopen(name, mode);
    if (!fp) return MPI_ERR_OTHER;
    *fh = new shim_mpi_file{fp};
    return MPI_SUCCESS;
}
int MPI_File_close(MPI_File *fh) {
    if (fh && *fh) {
        std::fclose((*fh)->fp);
        delete *fh;
        *fh = nullptr;
    }
    return MPI_SUCCESS;
}
int MPI_File_get_size(MPI_File fh, MPI_Offset *size) {
    long long cur = ftello(fh->fp);
    fseeko(fh->fp, 0, SEEK_END);
    *size = ftello(fh->fp);
    fseeko(fh->fp, cur, SEEK_SET);
    return MPI_SUCCESS;
}
int MPI_File_read_at_all(MPI_File fh, MPI_Offset off, void *buf, int count, MPI_Datatype t,
                         MPI_Status *st) {
    long long bytes = (long long)count * tsize(t);
    fseeko(fh->fp, off, SEEK_SET);
    size_t got = bytes > 0 ? std::fread(buf, 1, (size_t)bytes, fh->fp) : 0;
    fill_status(st, 0, (long long)got);
    return MPI_SUCCESS;
}
int MPI_File_write_at_all(MPI_File fh, MPI_Offset off, const void *buf, int count, MPI_Datatype t,
                          MPI_Status *st) {
    long long bytes = (long long)count * tsize(t);
    fseeko(fh->fp, off, SEEK_SET);
    size_t put = bytes > 0 ? std::fwrite(buf, 1, (size_t)bytes, fh->fp) : 0;
    fill_status(st, 0, (long long)put);
    return MPI_SUCCESS;
}

}  // extern "C"
