/*
 * Single-rank MPI shim — TEST INFRASTRUCTURE ONLY.
 *
 * This header and mpi_shim.cpp are project-written. They exist so that the
 * unmodified SWAP-Assembler sources (graph.cpp, kmerGraph.cpp, sequence.cpp,
 * mympi.cpp) can be compiled and run in a container that has no MPI library,
 * and used as the correctness oracle for the GPU k-mer graph build.
 *
 * Only the subset of MPI that those four files reference is declared
 * (mympi.cpp:12-15,52,71-72,113,138,142,151; kmerGraph.cpp:52-53,121-122,134,
 * 150,372,412,414; graph.cpp:616-679,1204-1566,1613-1617,3464-3696).
 * There is exactly one rank (rank 0 of 1). Point-to-point messages are to
 * self and are buffered; collectives degenerate to copies. Calls that can
 * only make progress with a second rank abort with a message instead of
 * blocking forever.
 */
#ifndef SWG_ORACLE_MPI_SHIM_H
#define SWG_ORACLE_MPI_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef int MPI_Info;
typedef long long MPI_Offset;
typedef struct shim_mpi_file *MPI_File;

typedef struct {
    int MPI_SOURCE;
    int MPI_TAG;
    int MPI_ERROR;
    long long shim_bytes;
} MPI_Status;

#define MPI_SUCCESS 0
#define MPI_ERR_OTHER 15
#define MPI_COMM_WORLD 0
#define MPI_INFO_NULL 0
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
#define MPI_MAX_PROCESSOR_NAME 256

#define MPI_CHAR 1
#define MPI_INT 2
#define MPI_UNSIGNED_LONG_LONG 3
#define MPI_LONG_LONG_INT 4
#define MPI_DOUBLE 5
#define MPI_LONG_LONG MPI_LONG_LONG_INT

#define MPI_SUM 1

#define MPI_MODE_RDONLY 2
#define MPI_MODE_WRONLY 4
#define MPI_MODE_CREATE 1

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Abort(MPI_Comm comm, int code);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Get_processor_name(char *name, int *len);

int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype *out);
int MPI_Type_commit(MPI_Datatype *t);

int MPI_Barrier(MPI_Comm comm);
int MPI_Ibarrier(MPI_Comm comm, MPI_Request *req);
int MPI_Bcast(void *buf, int count, MPI_Datatype t, int root, MPI_Comm comm);
int MPI_Reduce(const void *s, void *r, int count, MPI_Datatype t, MPI_Op op, int root, MPI_Comm comm);
int MPI_Allreduce(const void *s, void *r, int count, MPI_Datatype t, MPI_Op op, MPI_Comm comm);
int MPI_Scan(const void *s, void *r, int count, MPI_Datatype t, MPI_Op op, MPI_Comm comm);
int MPI_Gather(const void *s, int scount, MPI_Datatype st, void *r, int rcount, MPI_Datatype rt,
               int root, MPI_Comm comm);
int MPI_Alltoall(const void *s, int scount, MPI_Datatype st, void *r, int rcount, MPI_Datatype rt,
                 MPI_Comm comm);
int MPI_Alltoallv(const void *s, const int *scounts, const int *sdispls, MPI_Datatype st,
                  void *r, const int *rcounts, const int *rdispls, MPI_Datatype rt, MPI_Comm comm);

int MPI_Send(const void *buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm);
int MPI_Isend(const void *buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm,
              MPI_Request *req);
int MPI_Recv(void *buf, int count, MPI_Datatype t, int src, int tag, MPI_Comm comm, MPI_Status *st);
int MPI_Irecv(void *buf, int count, MPI_Datatype t, int src, int tag, MPI_Comm comm, MPI_Request *req);
int MPI_Wait(MPI_Request *req, MPI_Status *st);
int MPI_Waitall(int n, MPI_Request *reqs, MPI_Status *sts);
int MPI_Test(MPI_Request *req, int *flag, MPI_Status *st);
int MPI_Testall(int n, MPI_Request *reqs, int *flag, MPI_Status *sts);
int MPI_Iprobe(int src, int tag, MPI_Comm comm, int *flag, MPI_Status *st);

int MPI_File_open(MPI_Comm comm, const char *name, int amode, MPI_Info info, MPI_File *fh);
int MPI_File_close(MPI_File *fh);
int MPI_File_get_size(MPI_File fh, MPI_Offset *size);
int MPI_File_read_at_all(MPI_File fh, MPI_Offset off, void *buf, int count, MPI_Datatype t,
                         MPI_Status *st);
int MPI_File_write_at_all(MPI_File fh, MPI_Offset off, const void *buf, int count, MPI_Datatype t,
                          MPI_Status *st);

#ifdef __cplusplus
}
#endif
#endif
