/*
 * Single-rank stand-in for <mpi.h>, just enough to compile the reference's
 * Orthogonalization.c (3D-GreenIteration/src/utilities/Orthogonalization.c)
 * as a CPU checker.  With one rank, MPI_Allreduce(SUM) is a copy.
 * Test infrastructure only.
 */
#ifndef TAGI_ORACLE_MPI_STUB_H
#define TAGI_ORACLE_MPI_STUB_H
#include <string.h>
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 8
#define MPI_SUM 1
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
static inline int MPI_Allreduce(const void *in, void *out, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c)
{
    (void)op; (void)c;
    memcpy(out, in, (size_t)n * (size_t)t);
    return 0;
}
#endif
