/*
 * Minimal MPI stand-in used ONLY to compile the reference POREMAPS sources
 * (the src directory of krachdd/poremaps) unmodified into a CPU oracle binary.
 *
 * Test infrastructure: nothing in the poremaps_gb300 product links this.
 *
 * Ranks are POSIX threads inside one process (world size from the environment
 * variable PM_SHIM_NP, default 1).  Every MPI call the reference makes is
 * covered: Cartesian topology, Sendrecv (mailbox), Allreduce (rank-ordered,
 * deterministic), subarray MPI-IO (pread/pwrite), Wtime.  The reference's
 * own main() runs as rank 0; MPI_Init starts ranks 1..P-1 as threads that
 * enter main() again with their own thread-local rank.
 */
#ifndef PM_MPI_SHIM_H
#define PM_MPI_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Info;
typedef long long MPI_Offset;
typedef struct { int MPI_SOURCE; int MPI_TAG; int MPI_ERROR; } MPI_Status;
typedef struct pm_shim_file* MPI_File;

#define MPI_COMM_WORLD 1
#define MPI_COMM_CART_BASE 2

#define MPI_C_BOOL 1
#define MPI_INT 2
#define MPI_DOUBLE 3
/* derived (subarray) datatypes are numbered from here */
#define PM_SHIM_FIRST_DERIVED 16

#define MPI_SUM 1
#define MPI_MAX 2

#define MPI_INFO_NULL 0
#define MPI_PROC_NULL (-2)
#define MPI_ORDER_C 56
#define MPI_ORDER_FORTRAN 57

#define MPI_MODE_RDONLY 2
#define MPI_MODE_RDWR 8
#define MPI_MODE_CREATE 1
#define MPI_MODE_SEQUENTIAL 256

#define MPI_IN_PLACE ((void*)1)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)

int MPI_Init(int* argc, char*** argv);
int MPI_Finalize(void);
int MPI_Comm_rank(MPI_Comm comm, int* rank);
int MPI_Comm_size(MPI_Comm comm, int* size);
int MPI_Barrier(MPI_Comm comm);
int MPI_Dims_create(int nnodes, int ndims, int* dims);
int MPI_Cart_create(MPI_Comm old, int ndims, const int* dims, const int* periods,
                    int reorder, MPI_Comm* comm_cart);
int MPI_Cart_coords(MPI_Comm comm, int rank, int maxdims, int* coords);
int MPI_Cart_shift(MPI_Comm comm, int direction, int disp, int* source, int* dest);
int MPI_Sendrecv(const void* sendbuf, int sendcount, MPI_Datatype sendtype, int dest,
                 int sendtag, void* recvbuf, int recvcount, MPI_Datatype recvtype,
                 int source, int recvtag, MPI_Comm comm, MPI_Status* status);
int MPI_Allreduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype type,
                  MPI_Op op, MPI_Comm comm);
int MPI_Type_create_subarray(int ndims, const int* sizes, const int* subsizes,
                             const int* starts, int order, MPI_Datatype oldtype,
                             MPI_Datatype* newtype);
int MPI_Type_commit(MPI_Datatype* type);
int MPI_Type_free(MPI_Datatype* type);
int MPI_File_open(MPI_Comm comm, const char* filename, int amode, MPI_Info info,
                  MPI_File* fh);
int MPI_File_set_view(MPI_File fh, MPI_Offset disp, MPI_Datatype etype,
                      MPI_Datatype filetype, const char* datarep, MPI_Info info);
int MPI_File_read_at_all(MPI_File fh, MPI_Offset offset, void* buf, int count,
                         MPI_Datatype type, MPI_Status* status);
int MPI_File_write_at_all(MPI_File fh, MPI_Offset offset, const void* buf, int count,
                          MPI_Datatype type, MPI_Status* status);
int MPI_File_close(MPI_File* fh);
double MPI_Wtime(void);

#ifdef __cplusplus
}
#endif

#endif
