/*
 * mpi.h -- a single-process stand-in for the MPI calls of the reference's
 * Filter stack (cxx/Filter.cpp, upwind/cxx/upwindMpi.cxx,
 * laplacian/cxx/laplacian.cxx, laplacian/cxx/testStencil2d.cxx).
 *
 * TEST INFRASTRUCTURE ONLY.  It lets oracle/Makefile compile those reference
 * sources unchanged, by path, for ONE rank, so that their output can pin the
 * Filter restatement (oracle/filter_oracle.c).  Semantics for one rank:
 * rank 0 of size 1; a window exposes its base buffer and MPI_Get copies from
 * it (the target rank is always 0); fences do nothing; a reduction or a
 * gather over one rank copies the send buffer.  Only MPI_DOUBLE is served.
 * Nothing here is taken from an MPI implementation: it is written from the
 * calls' documented single-rank meaning.
 */
#ifndef FDB_ORACLE_MPI_STUB_H
#define FDB_ORACLE_MPI_STUB_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Info;
typedef int MPI_Win;
typedef ptrdiff_t MPI_Aint;

#define MPI_SUCCESS 0
#define MPI_COMM_WORLD 1
#define MPI_DOUBLE 1
#define MPI_SUM 1
#define MPI_MIN 2
#define MPI_MAX 3
#define MPI_INFO_NULL 0
#define MPI_MODE_NOCHECK 1
#define MPI_MODE_NOSTORE 2
#define MPI_MODE_NOPUT 4
#define MPI_MODE_NOPRECEDE 8
#define MPI_MODE_NOSUCCEED 16
#define MPI_THREAD_SINGLE 0
#define MPI_THREAD_FUNNELED 1
#define MPI_THREAD_SERIALIZED 2
#define MPI_THREAD_MULTIPLE 3

int MPI_Init(int* argc, char*** argv);
int MPI_Init_thread(int* argc, char*** argv, int required, int* provided);
int MPI_Finalize(void);
int MPI_Comm_rank(MPI_Comm comm, int* rank);
int MPI_Comm_size(MPI_Comm comm, int* size);
double MPI_Wtime(void);
int MPI_Alloc_mem(MPI_Aint size, MPI_Info info, void* baseptr);
int MPI_Free_mem(void* base);
int MPI_Win_create(void* base, MPI_Aint size, int disp_unit, MPI_Info info, MPI_Comm comm,
                   MPI_Win* win);
int MPI_Win_fence(int assert_, MPI_Win win);
int MPI_Win_free(MPI_Win* win);
int MPI_Get(void* origin, int origin_count, MPI_Datatype origin_type, int target_rank,
            MPI_Aint target_disp, int target_count, MPI_Datatype target_type, MPI_Win win);
int MPI_Reduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype type, MPI_Op op,
               int root, MPI_Comm comm);
int MPI_Gather(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf,
               int recvcount, MPI_Datatype recvtype, int root, MPI_Comm comm);

#ifdef __cplusplus
}
#endif
#endif /* FDB_ORACLE_MPI_STUB_H */
