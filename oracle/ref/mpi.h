/* Single-rank stand-in for <mpi.h>, used only to compile the reference's own
 * CPU sources as a test oracle (the image ships no MPI).  Every call behaves as
 * it would on a communicator of size 1: rank 0, size 1, Allgather copies the
 * send buffer, point-to-point calls never run (the reference guards them with
 * nRanks > 1).  Written for this project; not part of the reference. */
#ifndef QMIN_ORACLE_MPI_SHIM_H
#define QMIN_ORACLE_MPI_SHIM_H
#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Request;
typedef int MPI_Info;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_INT 1
#define MPI_FLOAT 2
#define MPI_DOUBLE 3
#define MPI_ANY_SOURCE (-1)
#define MPI_COMM_TYPE_SHARED 0
#define MPI_INFO_NULL 0
#define MPI_MAX_PROCESSOR_NAME 64
#define MPI_SUCCESS 0

static inline int qmin_shim_type_size(MPI_Datatype t)
{
    return t == MPI_INT ? (int)sizeof(int) : t == MPI_FLOAT ? (int)sizeof(float) : (int)sizeof(double);
}
static inline int MPI_Init(int *, char ***) { return MPI_SUCCESS; }
static inline int MPI_Finalize(void) { return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm, int *size) { *size = 1; return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm, int *rank) { *rank = 0; return MPI_SUCCESS; }
static inline int MPI_Get_processor_name(char *name, int *len)
{
    strcpy(name, "oracle");
    *len = 6;
    return MPI_SUCCESS;
}
static inline int MPI_Comm_split_type(MPI_Comm, int, int, MPI_Info, MPI_Comm *out)
{
    *out = 0;
    return MPI_SUCCESS;
}
static inline int MPI_Allgather(const void *s, int n, MPI_Datatype t, void *r, int, MPI_Datatype, MPI_Comm)
{
    memmove(r, s, (size_t)n * (size_t)qmin_shim_type_size(t));
    return MPI_SUCCESS;
}
static inline int MPI_Isend(const void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) { return MPI_SUCCESS; }
static inline int MPI_Irecv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) { return MPI_SUCCESS; }
static inline int MPI_Wait(MPI_Request *, MPI_Status *) { return MPI_SUCCESS; }
#endif
