/* Single-rank stand-in for the MPI calls the reference's hot path makes.
 *
 * Test infrastructure only: lets the reference's own src/*.cpp compile and
 * run as one rank so that its results can serve as the oracle.  Semantics:
 * one process, rank 0, size 1.  MPI_Cart_shift returns MPI_PROC_NULL for a
 * non-periodic dimension and the caller itself for a periodic one, so
 * MPI_Sendrecv to self copies the send buffer into the receive buffer (the
 * reference's periodic boundary exchange, src/fields.cpp:413-422).
 */
#pragma once
#include <string.h>
#include <stddef.h>
#include <unistd.h> /* real MPI headers pull this in; the reference relies on it */

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Info;
typedef struct { int source, tag, error; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_INFO_NULL 0
#define MPI_PROC_NULL (-2)
#define MPI_DOUBLE 8
#define MPI_INT 4
#define MPI_SUM 1
#define MPI_SUCCESS 0

/* one definition shared by every translation unit (C++17 inline variable) */
inline int ffip_shim_periods[3] = {0, 0, 0};

static inline int MPI_Init(int *, char ***) { return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int *s) { *s = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Cart_create(MPI_Comm, int ndims, const int *, const int *periods, int, MPI_Comm *c)
{
    for (int i = 0; i < ndims && i < 3; ++i) ffip_shim_periods[i] = periods[i];
    *c = 0;
    return 0;
}
static inline int MPI_Cart_coords(MPI_Comm, int, int maxdims, int *coords)
{
    for (int i = 0; i < maxdims; ++i) coords[i] = 0;
    return 0;
}
static inline int MPI_Cart_shift(MPI_Comm, int dir, int, int *src, int *dst)
{
    int r = ffip_shim_periods[dir] ? 0 : MPI_PROC_NULL;
    *src = r;
    *dst = r;
    return 0;
}
static inline int MPI_Sendrecv(const void *sbuf, int scount, MPI_Datatype stype, int dst, int,
                               void *rbuf, int rcount, MPI_Datatype, int src, int, MPI_Comm, MPI_Status *)
{
    if (dst == 0 && src == 0 && scount > 0 && rcount > 0)
        memcpy(rbuf, sbuf, (size_t)(scount < rcount ? scount : rcount) * (size_t)stype);
    return 0;
}
static inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm)
{
    memcpy(r, s, (size_t)n * (size_t)t);
    return 0;
}
static inline int MPI_Scan(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm)
{
    memcpy(r, s, (size_t)n * (size_t)t);
    return 0;
}
