// oracle/shim/mpi.h -- TEST INFRASTRUCTURE ONLY.
//
// A single-rank stand-in for the handful of MPI calls the reference's
// src/StaticBTESolver.cpp makes (:33-34 size/rank, :42,:760,:811,:813,:872,:875
// barriers, :761-768 Allgather, :844 Gather), so that the reference's CPU solver
// compiles without an MPI installation.  With one rank, Allgather and Gather
// are plain copies and everything else is a no-op.
#pragma once
#include <cstring>

typedef int MPI_Comm;
typedef int MPI_Datatype;
#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 8
#define MPI_UNSIGNED_CHAR 1
#define MPI_UNSIGNED_SHORT 2
#define MPI_UNSIGNED 4
#define MPI_UNSIGNED_LONG 108
#define MPI_UNSIGNED_LONG_LONG 208

static inline int shim_mpi_type_size(MPI_Datatype t) { return t % 100; }
static inline int MPI_Init(int*, char***) { return 0; }
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Comm_size(MPI_Comm, int* n) { *n = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Allgather(const void* send, int count, MPI_Datatype t, void* recv, int,
                                MPI_Datatype, MPI_Comm) {
    if (send != recv) std::memmove(recv, send, (size_t)count * shim_mpi_type_size(t));
    return 0;
}
static inline int MPI_Gather(const void* send, int count, MPI_Datatype t, void* recv, int,
                             MPI_Datatype, int, MPI_Comm) {
    if (recv && send != recv) std::memmove(recv, send, (size_t)count * shim_mpi_type_size(t));
    return 0;
}
