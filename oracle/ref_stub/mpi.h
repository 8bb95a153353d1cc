/* Single-rank stand-in for <mpi.h>, used only to compile the reference's own
 * local-multiply sources into oracle/_ref (a CPU checker, never shipped).
 * With one rank every collective is a local copy and no point-to-point peer
 * exists, so point-to-point and RMA calls abort.  The hot path (spgemm(),
 * serialSpgemm, LocalAccumulator) calls none of them. */
#ifndef ORACLE_REF_STUB_MPI_H
#define ORACLE_REF_STUB_MPI_H

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Request;
typedef int MPI_Win;
typedef int MPI_Op;
typedef int MPI_Info;
typedef std::int64_t MPI_Aint;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_SUCCESS 0
#define MPI_COMM_NULL 0
#define MPI_COMM_WORLD 1
#define MPI_REQUEST_NULL 0
#define MPI_INFO_NULL 0
#define MPI_COMM_TYPE_SHARED 1
#define MPI_MAX_ERROR_STRING 64
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
#define MPI_THREAD_SINGLE 0
#define MPI_THREAD_FUNNELED 1
#define MPI_THREAD_SERIALIZED 2
#define MPI_THREAD_MULTIPLE 3
#define MPI_INT 4
#define MPI_INT64_T 8
#define MPI_DOUBLE 9
#define MPI_MAX 1
#define MPI_MIN 2
#define MPI_SUM 3

inline std::size_t stub_mpi_size(MPI_Datatype t) { return t == MPI_INT ? 4 : 8; }
[[noreturn]] inline void stub_mpi_no_peer(const char* call) {
    std::fprintf(stderr, "single-rank MPI stub: %s needs a peer\n", call);
    std::abort();
}
inline int MPI_Comm_rank(MPI_Comm, int* rank) { *rank = 0; return MPI_SUCCESS; }
inline int MPI_Comm_size(MPI_Comm, int* size) { *size = 1; return MPI_SUCCESS; }
inline int MPI_Comm_dup(MPI_Comm c, MPI_Comm* out) { *out = c; return MPI_SUCCESS; }
inline int MPI_Comm_free(MPI_Comm* c) { *c = MPI_COMM_NULL; return MPI_SUCCESS; }
inline int MPI_Comm_split(MPI_Comm c, int, int, MPI_Comm* out) { *out = c; return MPI_SUCCESS; }
inline int MPI_Comm_split_type(MPI_Comm c, int, int, MPI_Info, MPI_Comm* out) { *out = c; return MPI_SUCCESS; }
inline int MPI_Abort(MPI_Comm, int) { std::abort(); }
inline int MPI_Error_string(int, char* s, int* n) { std::strcpy(s, "stub"); *n = 4; return MPI_SUCCESS; }
inline double MPI_Wtime() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }
inline int MPI_Reduce(const void* in, void* out, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
    std::memmove(out, in, n * stub_mpi_size(t));
    return MPI_SUCCESS;
}
inline int MPI_Allreduce(const void* in, void* out, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
    std::memmove(out, in, n * stub_mpi_size(t));
    return MPI_SUCCESS;
}
inline int MPI_Allgather(const void* in, int n, MPI_Datatype t, void* out, int, MPI_Datatype, MPI_Comm) {
    std::memmove(out, in, n * stub_mpi_size(t));
    return MPI_SUCCESS;
}
inline int MPI_Waitall(int, MPI_Request*, MPI_Status*) { return MPI_SUCCESS; }
inline int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm) { stub_mpi_no_peer("MPI_Send"); }
inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) { stub_mpi_no_peer("MPI_Recv"); }
inline int MPI_Isend(const void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*) { stub_mpi_no_peer("MPI_Isend"); }
inline int MPI_Irecv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*) { stub_mpi_no_peer("MPI_Irecv"); }
inline int MPI_Get(void*, int, MPI_Datatype, int, MPI_Aint, int, MPI_Datatype, MPI_Win) { stub_mpi_no_peer("MPI_Get"); }
inline int MPI_Put(const void*, int, MPI_Datatype, int, MPI_Aint, int, MPI_Datatype, MPI_Win) { stub_mpi_no_peer("MPI_Put"); }

#endif
