/* Test infrastructure: a stand-in for the MPI declarations that the
 * reference's include/comm.hpp names, so that its host ogs operator compiles
 * at one rank without an MPI installation.  The operator path the oracle
 * drives makes no MPI call; each function here aborts if it is ever reached.
 */
#ifndef OGSREF_MPI_STANDIN_H
#define OGSREF_MPI_STANDIN_H
#include <stdio.h>
#include <stdlib.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_SUCCESS 0
#define MPI_COMM_WORLD 0
#define MPI_COMM_NULL (-1)
#define MPI_MAX_PROCESSOR_NAME 256
#define MPI_IN_PLACE ((void*)1)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
#define MPI_REQUEST_NULL 0
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)

enum { MPI_CHAR = 1, MPI_INT, MPI_LONG, MPI_LONG_LONG_INT, MPI_LONG_LONG, MPI_FLOAT, MPI_DOUBLE, MPI_BYTE,
       MPI_UNSIGNED, MPI_UNSIGNED_LONG, MPI_UNSIGNED_LONG_LONG, MPI_C_BOOL, MPI_CXX_BOOL, MPI_SHORT,
       MPI_UNSIGNED_CHAR, MPI_SIGNED_CHAR, MPI_UNSIGNED_SHORT, MPI_LONG_DOUBLE, MPI_INT8_T, MPI_INT16_T,
       MPI_INT32_T, MPI_INT64_T, MPI_UINT8_T, MPI_UINT16_T, MPI_UINT32_T, MPI_UINT64_T };
enum { MPI_SUM = 1, MPI_PROD, MPI_MAX, MPI_MIN, MPI_LAND, MPI_LOR, MPI_LXOR, MPI_BAND, MPI_BOR, MPI_BXOR };

static inline int ogsref_mpi_unreached(const char* fn) {
  fprintf(stderr, "ogsref: %s called; the one-rank operator path makes no MPI call\n", fn);
  abort();
  return 1;
}
#define OGSREF_MPI_FN(name, ...) \
  static inline int name(__VA_ARGS__) { return ogsref_mpi_unreached(#name); }

OGSREF_MPI_FN(MPI_Init, int*, char***)
OGSREF_MPI_FN(MPI_Finalize, void)
OGSREF_MPI_FN(MPI_Initialized, int*)
OGSREF_MPI_FN(MPI_Abort, MPI_Comm, int)
OGSREF_MPI_FN(MPI_Comm_rank, MPI_Comm, int*)
OGSREF_MPI_FN(MPI_Comm_size, MPI_Comm, int*)
OGSREF_MPI_FN(MPI_Comm_dup, MPI_Comm, MPI_Comm*)
OGSREF_MPI_FN(MPI_Comm_free, MPI_Comm*)
OGSREF_MPI_FN(MPI_Comm_delete, MPI_Comm*)
OGSREF_MPI_FN(MPI_Comm_split, MPI_Comm, int, int, MPI_Comm*)
OGSREF_MPI_FN(MPI_Barrier, MPI_Comm)
OGSREF_MPI_FN(MPI_Get_processor_name, char*, int*)
OGSREF_MPI_FN(MPI_Type_contiguous, int, MPI_Datatype, MPI_Datatype*)
OGSREF_MPI_FN(MPI_Type_commit, MPI_Datatype*)
OGSREF_MPI_FN(MPI_Type_free, MPI_Datatype*)
OGSREF_MPI_FN(MPI_Send, const void*, int, MPI_Datatype, int, int, MPI_Comm)
OGSREF_MPI_FN(MPI_Recv, void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*)
OGSREF_MPI_FN(MPI_Isend, const void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*)
OGSREF_MPI_FN(MPI_Irecv, void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*)
OGSREF_MPI_FN(MPI_Wait, MPI_Request*, MPI_Status*)
OGSREF_MPI_FN(MPI_Waitall, int, MPI_Request*, MPI_Status*)
OGSREF_MPI_FN(MPI_Bcast, void*, int, MPI_Datatype, int, MPI_Comm)
OGSREF_MPI_FN(MPI_Reduce, const void*, void*, int, MPI_Datatype, MPI_Op, int, MPI_Comm)
OGSREF_MPI_FN(MPI_Allreduce, const void*, void*, int, MPI_Datatype, MPI_Op, MPI_Comm)
OGSREF_MPI_FN(MPI_Iallreduce, const void*, void*, int, MPI_Datatype, MPI_Op, MPI_Comm, MPI_Request*)
OGSREF_MPI_FN(MPI_Scan, const void*, void*, int, MPI_Datatype, MPI_Op, MPI_Comm)
OGSREF_MPI_FN(MPI_Exscan, const void*, void*, int, MPI_Datatype, MPI_Op, MPI_Comm)
OGSREF_MPI_FN(MPI_Gather, const void*, int, MPI_Datatype, void*, int, MPI_Datatype, int, MPI_Comm)
OGSREF_MPI_FN(MPI_Gatherv, const void*, int, MPI_Datatype, void*, const int*, const int*, MPI_Datatype, int, MPI_Comm)
OGSREF_MPI_FN(MPI_Scatter, const void*, int, MPI_Datatype, void*, int, MPI_Datatype, int, MPI_Comm)
OGSREF_MPI_FN(MPI_Scatterv, const void*, const int*, const int*, MPI_Datatype, void*, int, MPI_Datatype, int,
              MPI_Comm)
OGSREF_MPI_FN(MPI_Allgather, const void*, int, MPI_Datatype, void*, int, MPI_Datatype, MPI_Comm)
OGSREF_MPI_FN(MPI_Allgatherv, const void*, int, MPI_Datatype, void*, const int*, const int*, MPI_Datatype, MPI_Comm)
OGSREF_MPI_FN(MPI_Alltoall, const void*, int, MPI_Datatype, void*, int, MPI_Datatype, MPI_Comm)
OGSREF_MPI_FN(MPI_Alltoallv, const void*, const int*, const int*, MPI_Datatype, void*, const int*, const int*,
              MPI_Datatype, MPI_Comm)
OGSREF_MPI_FN(MPI_Ialltoallv, const void*, const int*, const int*, MPI_Datatype, void*, const int*, const int*,
              MPI_Datatype, MPI_Comm, MPI_Request*)
#undef OGSREF_MPI_FN
#endif
