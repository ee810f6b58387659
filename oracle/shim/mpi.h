/*
 * Single-rank MPI stand-in used only to compile the reference solver as a CPU
 * oracle (test infrastructure; never linked into the product).
 *
 * With one rank every collective is a copy and no point-to-point message is
 * ever posted: the reference's halo maps (include/comm.hpp:209-265) are empty
 * when there is one rank, so Isend/Irecv/Probe are never reached.  The gold
 * files of the reference were produced with 2 ranks and are matched bit-for-bit
 * by 1 rank (the decomposition only reorders independent per-cell work).
 */
#pragma once
#include <cstring>
#include <cstdint>
#include <stdexcept>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
struct MPI_Status { int MPI_SOURCE; int MPI_TAG; int MPI_ERROR; int count; };

#define MPI_COMM_WORLD 0
#define MPI_INT 1
#define MPI_FLOAT 2
#define MPI_DOUBLE 3
#define MPI_LONG_LONG 4
#define MPI_C_BOOL 5
#define MPI_SUM 10
#define MPI_MAX 11
#define MPI_ANY_SOURCE (-1)
#define MPI_STATUS_IGNORE ((MPI_Status *)nullptr)
#define MPI_STATUSES_IGNORE ((MPI_Status *)nullptr)

static inline size_t mpi_shim_size(MPI_Datatype t)
{
    switch (t) {
    case MPI_INT: return sizeof(int);
    case MPI_FLOAT: return sizeof(float);
    case MPI_DOUBLE: return sizeof(double);
    case MPI_LONG_LONG: return sizeof(long long);
    case MPI_C_BOOL: return sizeof(bool);
    default: throw std::runtime_error("mpi shim: unknown datatype");
    }
}

static inline int MPI_Init(int *, char ***) { return 0; }
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int *s) { *s = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Bcast(void *, long long, MPI_Datatype, int, MPI_Comm) { return 0; }
static inline int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm)
{
    std::memcpy(r, s, (size_t)n * mpi_shim_size(t));
    return 0;
}
static inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm)
{
    std::memcpy(r, s, (size_t)n * mpi_shim_size(t));
    return 0;
}
static inline int MPI_Gather(const void *s, int n, MPI_Datatype t, void *r, int, MPI_Datatype, int, MPI_Comm)
{
    std::memcpy(r, s, (size_t)n * mpi_shim_size(t));
    return 0;
}
static inline int MPI_Gatherv(const void *s, int n, MPI_Datatype t, void *r, const int *, const int *,
                              MPI_Datatype, int, MPI_Comm)
{
    if (n > 0) std::memcpy(r, s, (size_t)n * mpi_shim_size(t));
    return 0;
}
static inline int MPI_Isend(const void *, long long, MPI_Datatype, int, int, MPI_Comm, MPI_Request *)
{
    throw std::runtime_error("mpi shim: point-to-point send with one rank");
}
static inline int MPI_Irecv(void *, long long, MPI_Datatype, int, int, MPI_Comm, MPI_Request *)
{
    throw std::runtime_error("mpi shim: point-to-point receive with one rank");
}
static inline int MPI_Wait(MPI_Request *, MPI_Status *) { return 0; }
static inline int MPI_Waitall(int, MPI_Request *, MPI_Status *) { return 0; }
static inline int MPI_Probe(int, int, MPI_Comm, MPI_Status *)
{
    throw std::runtime_error("mpi shim: probe with one rank");
}
static inline int MPI_Get_count(const MPI_Status *, MPI_Datatype, int *c) { *c = 0; return 0; }
static inline int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *)
{
    throw std::runtime_error("mpi shim: receive with one rank");
}
