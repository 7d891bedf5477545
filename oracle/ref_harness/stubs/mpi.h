/* Single-rank MPI for running the reference CPU worker in-process (test
 * infrastructure).  Rank 0 of size 1; point-to-point messages go to a
 * thread-safe loopback mailbox; collectives copy the caller's buffer. */
#ifndef SG_REF_MPI_STUB_H_
#define SG_REF_MPI_STUB_H_
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct {
  int MPI_SOURCE;
  int MPI_TAG;
  int MPI_ERROR;
  int sg_bytes;
} MPI_Status;
#define MPI_SUCCESS 0
#define MPI_COMM_NULL 0
#define MPI_COMM_WORLD 1
#define MPI_REQUEST_NULL (-1)
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
#define MPI_IN_PLACE ((void*)1)
#define MPI_MAX_PROCESSOR_NAME 256
#define MPI_THREAD_SINGLE 0
#define MPI_THREAD_FUNNELED 1
#define MPI_THREAD_SERIALIZED 2
#define MPI_THREAD_MULTIPLE 3
/* datatypes encode their byte size */
#define MPI_CHAR 1
#define MPI_BYTE 1
#define MPI_UNSIGNED_CHAR 1
#define MPI_SHORT 2
#define MPI_INT 4
#define MPI_UNSIGNED 4
#define MPI_FLOAT 4
#define MPI_LONG 8
#define MPI_UNSIGNED_LONG 8
#define MPI_LONG_LONG 8
#define MPI_LONG_LONG_INT 8
#define MPI_UNSIGNED_LONG_LONG 8
#define MPI_UINT64_T 8
#define MPI_INT64_T 8
#define MPI_UINT32_T 4
#define MPI_INT32_T 4
#define MPI_DOUBLE 8
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3
int MPI_Init(int* argc, char*** argv);
int MPI_Init_thread(int* argc, char*** argv, int required, int* provided);
int MPI_Initialized(int* flag);
int MPI_Finalize(void);
int MPI_Comm_rank(MPI_Comm comm, int* rank);
int MPI_Comm_size(MPI_Comm comm, int* size);
int MPI_Comm_dup(MPI_Comm comm, MPI_Comm* out);
int MPI_Comm_free(MPI_Comm* comm);
int MPI_Comm_split(MPI_Comm comm, int color, int key, MPI_Comm* out);
int MPI_Barrier(MPI_Comm comm);
int MPI_Send(const void* buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm);
int MPI_Isend(const void* buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm,
              MPI_Request* req);
int MPI_Recv(void* buf, int count, MPI_Datatype t, int src, int tag, MPI_Comm comm,
             MPI_Status* st);
int MPI_Irecv(void* buf, int count, MPI_Datatype t, int src, int tag, MPI_Comm comm,
              MPI_Request* req);
int MPI_Probe(int src, int tag, MPI_Comm comm, MPI_Status* st);
int MPI_Iprobe(int src, int tag, MPI_Comm comm, int* flag, MPI_Status* st);
int MPI_Get_count(const MPI_Status* st, MPI_Datatype t, int* count);
int MPI_Test(MPI_Request* req, int* flag, MPI_Status* st);
int MPI_Wait(MPI_Request* req, MPI_Status* st);
int MPI_Waitall(int n, MPI_Request* reqs, MPI_Status* sts);
int MPI_Waitany(int n, MPI_Request* reqs, int* index, MPI_Status* st);
int MPI_Cancel(MPI_Request* req);
int MPI_Allreduce(const void* sb, void* rb, int count, MPI_Datatype t, MPI_Op op, MPI_Comm comm);
int MPI_Reduce(const void* sb, void* rb, int count, MPI_Datatype t, MPI_Op op, int root,
               MPI_Comm comm);
int MPI_Allgather(const void* sb, int sc, MPI_Datatype st, void* rb, int rc, MPI_Datatype rt,
                  MPI_Comm comm);
int MPI_Allgatherv(const void* sb, int sc, MPI_Datatype st, void* rb, const int* rcs,
                   const int* displs, MPI_Datatype rt, MPI_Comm comm);
int MPI_Gather(const void* sb, int sc, MPI_Datatype st, void* rb, int rc, MPI_Datatype rt,
               int root, MPI_Comm comm);
int MPI_Bcast(void* buf, int count, MPI_Datatype t, int root, MPI_Comm comm);
int MPI_Get_processor_name(char* name, int* len);
double MPI_Wtime(void);
int MPI_Abort(MPI_Comm comm, int code);
#ifdef __cplusplus
}
#endif
#endif
