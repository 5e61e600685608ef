/* mpi_stub.c -- the single-rank MPI stand-in declared in mpi.h (test
 * infrastructure only; see that header). */
#include "mpi.h"

#include <stdlib.h>
#include <string.h>
#include <time.h>

#define STUB_MAX_WINDOWS 256

static struct {
  void* base;
  MPI_Aint size;
  int disp_unit;
  int used;
} g_win[STUB_MAX_WINDOWS];

int MPI_Init(int* argc, char*** argv) {
  (void)argc;
  (void)argv;
  return MPI_SUCCESS;
}

int MPI_Init_thread(int* argc, char*** argv, int required, int* provided) {
  (void)argc;
  (void)argv;
  if (provided) *provided = required;
  return MPI_SUCCESS;
}

int MPI_Finalize(void) { return MPI_SUCCESS; }

int MPI_Comm_rank(MPI_Comm comm, int* rank) {
  (void)comm;
  *rank = 0;
  return MPI_SUCCESS;
}

int MPI_Comm_size(MPI_Comm comm, int* size) {
  (void)comm;
  *size = 1;
  return MPI_SUCCESS;
}

double MPI_Wtime(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

int MPI_Alloc_mem(MPI_Aint size, MPI_Info info, void* baseptr) {
  (void)info;
  void* p = malloc(size > 0 ? (size_t)size : 1);
  if (!p) return 1;
  memcpy(baseptr, &p, sizeof(void*));
  return MPI_SUCCESS;
}

int MPI_Free_mem(void* base) {
  free(base);
  return MPI_SUCCESS;
}

int MPI_Win_create(void* base, MPI_Aint size, int disp_unit, MPI_Info info, MPI_Comm comm,
                   MPI_Win* win) {
  (void)info;
  (void)comm;
  for (int k = 0; k < STUB_MAX_WINDOWS; ++k) {
    if (!g_win[k].used) {
      g_win[k].base = base;
      g_win[k].size = size;
      g_win[k].disp_unit = disp_unit;
      g_win[k].used = 1;
      *win = k;
      return MPI_SUCCESS;
    }
  }
  return 1;
}

int MPI_Win_fence(int assert_, MPI_Win win) {
  (void)assert_;
  (void)win;
  return MPI_SUCCESS;
}

int MPI_Win_free(MPI_Win* win) {
  if (*win >= 0 && *win < STUB_MAX_WINDOWS) g_win[*win].used = 0;
  *win = -1;
  return MPI_SUCCESS;
}

int MPI_Get(void* origin, int origin_count, MPI_Datatype origin_type, int target_rank,
            MPI_Aint target_disp, int target_count, MPI_Datatype target_type, MPI_Win win) {
  if (origin_type != MPI_DOUBLE || target_type != MPI_DOUBLE || target_rank != 0) return 1;
  if (win < 0 || win >= STUB_MAX_WINDOWS || !g_win[win].used) return 1;
  const int n = origin_count < target_count ? origin_count : target_count;
  const size_t off = (size_t)target_disp * (size_t)g_win[win].disp_unit;
  if (off + (size_t)n * sizeof(double) > (size_t)g_win[win].size) return 1;
  memcpy(origin, (const char*)g_win[win].base + off, (size_t)n * sizeof(double));
  return MPI_SUCCESS;
}

int MPI_Reduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype type, MPI_Op op,
               int root, MPI_Comm comm) {
  (void)op;
  (void)root;
  (void)comm;
  if (type != MPI_DOUBLE) return 1;
  memcpy(recvbuf, sendbuf, (size_t)count * sizeof(double));
  return MPI_SUCCESS;
}

int MPI_Gather(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf,
               int recvcount, MPI_Datatype recvtype, int root, MPI_Comm comm) {
  (void)recvcount;
  (void)recvtype;
  (void)root;
  (void)comm;
  if (sendtype != MPI_DOUBLE) return 1;
  if (recvbuf) memcpy(recvbuf, sendbuf, (size_t)sendcount * sizeof(double));
  return MPI_SUCCESS;
}
