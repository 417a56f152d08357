/* Single-rank stand-in for <mpi.h>, used only to compile the reference aMat
 * headers into the CPU oracle library (oracle/_ref). Test infrastructure, not
 * product code.
 *
 * Every collective the reference issues at set-up (Maps::buildScatterMap:
 * Allgather, Alltoall, Alltoallv; include/maps.hpp:547-548, 704, 738) becomes
 * a copy of the caller's own contribution, which is what MPI does on a
 * communicator of size one. Point-to-point calls are never reached on one
 * rank (every halo routine returns early when size==1,
 * include/aMatFree.hpp:1428, 1505, 1554, 1633); they abort if they are. */
#ifndef ORACLE_SHIM_MPI_H
#define ORACLE_SHIM_MPI_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 1
#define MPI_COMM_SELF 2
#define MPI_COMM_NULL 0
#define MPI_SUCCESS 0
#define MPI_STATUS_IGNORE ((MPI_Status*)0)

/* datatype handle == element size in bytes; derived types get their size */
#define MPI_BYTE 1
#define MPI_CHAR 1
#define MPI_INT 4
#define MPI_UNSIGNED 4
#define MPI_FLOAT 4
#define MPI_LONG 8
#define MPI_UNSIGNED_LONG 8
#define MPI_DOUBLE 8
#define MPI_LONG_DOUBLE 16
#define MPI_MAX 1
#define MPI_MIN 2
#define MPI_SUM 3

static inline int MPI_Init(int*, char***) { return 0; }
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm, unsigned int* r) { *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, unsigned int* s) { *s = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Abort(MPI_Comm, int c) { fprintf(stderr, "MPI_Abort(%d)\n", c); abort(); }
static inline int MPI_Type_contiguous(int n, MPI_Datatype t, MPI_Datatype* out) { *out = n * t; return 0; }
static inline int MPI_Type_commit(MPI_Datatype*) { return 0; }
static inline double MPI_Wtime() { return 0.0; }

static inline int MPI_Allgather(const void* s, int sc, MPI_Datatype st, void* r, int, MPI_Datatype, MPI_Comm) {
    memcpy(r, s, (size_t)sc * (size_t)st); return 0;
}
static inline int MPI_Alltoall(const void* s, int sc, MPI_Datatype st, void* r, int, MPI_Datatype, MPI_Comm) {
    memcpy(r, s, (size_t)sc * (size_t)st); return 0;
}
static inline int MPI_Alltoallv(const void* s, const int* sc, const int* sd, MPI_Datatype st,
                                void* r, const int*, const int* rd, MPI_Datatype, MPI_Comm) {
    if (sc[0] > 0) memmove((char*)r + (size_t)rd[0] * st, (const char*)s + (size_t)sd[0] * st, (size_t)sc[0] * st);
    return 0;
}
static inline int MPI_Reduce(const void* s, void* r, int c, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
    if (s != r) memcpy(r, s, (size_t)c * (size_t)t); return 0;
}
static inline int MPI_Allreduce(const void* s, void* r, int c, MPI_Datatype t, MPI_Op, MPI_Comm) {
    if (s != r) memcpy(r, s, (size_t)c * (size_t)t); return 0;
}
static inline int oracle_mpi_p2p_unreachable() { fprintf(stderr, "oracle mpi shim: point-to-point on one rank\n"); abort(); }
static inline int MPI_Isend(const void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*) { return oracle_mpi_p2p_unreachable(); }
static inline int MPI_Irecv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*) { return oracle_mpi_p2p_unreachable(); }
static inline int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm) { return oracle_mpi_p2p_unreachable(); }
static inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) { return oracle_mpi_p2p_unreachable(); }
static inline int MPI_Wait(MPI_Request*, MPI_Status*) { return 0; }
static inline int MPI_Waitall(int, MPI_Request*, MPI_Status*) { return 0; }

#endif
