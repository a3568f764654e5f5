/*
 * Single-process stand-in for the handful of MPI symbols the reference's
 * explicit finite-volume sources name (src/global.h:9, src/global.cpp:590-687).
 * Test infrastructure only: it lets the oracle recipe compile the reference's
 * own FVM_TVD path without an MPI installation. One rank, no communication:
 * sends/receives/broadcasts are no-ops, which is exactly what the FVM_TVD path
 * sees at procCount == 1 (it never calls Method::exchange). FEM_RKDG's time step
 * (src/methods/fem_rkdg.cpp:413) reduces with MPI_Allreduce: one rank, a copy.
 */
#ifndef ORACLE_STUB_MPI_H
#define ORACLE_STUB_MPI_H

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 1
#define MPI_INT 2
#define MPI_MIN 3
#define MPI_MAX 4
#define MPI_SUM 5
#define MPI_SUCCESS 0

static inline int MPI_Init(int*, char***) { return MPI_SUCCESS; }
static inline int MPI_Finalize() { return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm, int* n) { *n = 1; return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return MPI_SUCCESS; }
static inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) { return MPI_SUCCESS; }
static inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }
/* one rank: the reduction of one contribution is that contribution */
static inline int MPI_Allreduce(const void* in, void* out, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
    const unsigned long bytes = (unsigned long)n * (t == MPI_DOUBLE ? 8u : 4u);
    for (unsigned long i = 0; i < bytes; i++) ((char*)out)[i] = ((const char*)in)[i];
    return MPI_SUCCESS;
}

#endif
