/*
 * Single-rank MPI stand-in used ONLY to compile the reference's MPI classes
 * (ThreadSharedMemory, ParticleSystem*Ptr, *StepperPtr) unmodified as a CPU
 * oracle.  Test infrastructure: nothing in the product links this.
 *
 * Semantics are those of MPI_COMM_WORLD with exactly one rank:
 *   - rank 0, size 1; the shared-memory split returns the world communicator;
 *   - MPI_Win_allocate_shared is calloc, MPI_Win_shared_query returns it;
 *   - Gather/Allreduce/Reduce copy the send buffer; Bcast/Barrier/fences and
 *     window locks do nothing;
 *   - Put/Get copy between the caller's buffer and the window's base;
 *   - point-to-point calls are never reached with one rank and do nothing.
 */
#ifndef SPSS_ORACLE_MPI_STUB_H
#define SPSS_ORACLE_MPI_STUB_H

#include <stdlib.h>
#include <string.h>

#ifdef __cplusplus
extern "C++" {
#endif

typedef int MPI_Comm;
typedef int MPI_Info;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef long MPI_Aint;
typedef long long MPI_Offset;
typedef int MPI_File;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 1
#define MPI_COMM_SELF 2
#define MPI_COMM_TYPE_SHARED 1
#define MPI_INFO_NULL 0
#define MPI_DOUBLE 8
#define MPI_INT 4
#define MPI_FLOAT 5
#define MPI_SUM 1
#define MPI_MODE_APPEND 128
#define MPI_MODE_WRONLY 4
#define MPI_MODE_CREATE 1
#define MPI_STATUS_IGNORE ((MPI_Status *) 0)
#define MPI_STATUSES_IGNORE ((MPI_Status *) 0)
#define MPI_SUCCESS 0

/* A window is an index into a small table of (base, bytes, owned). */
struct spss_mpi_window { void *base; long bytes; int owned; int used; };
typedef int MPI_Win;

static inline spss_mpi_window *spss_mpi_windows()
{
  static spss_mpi_window table[256];
  return table;
}

static inline int spss_mpi_new_window(void *base, long bytes, int owned)
{
  spss_mpi_window *t = spss_mpi_windows();
  for (int i = 1; i < 256; ++i)
  {
    if (!t[i].used)
    {
      t[i].base = base;
      t[i].bytes = bytes;
      t[i].owned = owned;
      t[i].used = 1;
      return i;
    }
  }
  abort();
}

static inline int spss_mpi_type_size(MPI_Datatype t)
{
  return t == MPI_DOUBLE ? 8 : 4;
}

static inline int MPI_Init(int *, char ***) { return 0; }
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int *rank) { *rank = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int *size) { *size = 1; return 0; }
static inline int MPI_Comm_split_type(MPI_Comm comm, int, int, MPI_Info, MPI_Comm *newcomm)
{
  *newcomm = comm;
  return 0;
}
static inline int MPI_Comm_free(MPI_Comm *) { return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return 0; }
static inline int MPI_Gather(const void *sendbuf, int sendcount, MPI_Datatype sendtype,
                             void *recvbuf, int, MPI_Datatype, int, MPI_Comm)
{
  if (sendbuf != recvbuf) memmove(recvbuf, sendbuf, (size_t) sendcount * spss_mpi_type_size(sendtype));
  return 0;
}
static inline int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype t, MPI_Op, MPI_Comm)
{
  if (sendbuf != recvbuf) memmove(recvbuf, sendbuf, (size_t) count * spss_mpi_type_size(t));
  return 0;
}
static inline int MPI_Reduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype t, MPI_Op, int, MPI_Comm)
{
  if (sendbuf != recvbuf) memmove(recvbuf, sendbuf, (size_t) count * spss_mpi_type_size(t));
  return 0;
}
static inline int MPI_Win_allocate_shared(MPI_Aint size, int, MPI_Info, MPI_Comm, void *baseptr, MPI_Win *win)
{
  void *p = calloc(size > 0 ? (size_t) size : 1, 1);
  *(void **) baseptr = p;
  *win = spss_mpi_new_window(p, size, 1);
  return 0;
}
static inline int MPI_Win_shared_query(MPI_Win win, int, MPI_Aint *size, int *disp_unit, void *baseptr)
{
  spss_mpi_window &w = spss_mpi_windows()[win];
  *size = w.bytes;
  *disp_unit = 1;
  *(void **) baseptr = w.base;
  return 0;
}
static inline int MPI_Win_create(void *base, MPI_Aint size, int, MPI_Info, MPI_Comm, MPI_Win *win)
{
  *win = spss_mpi_new_window(base, size, 0);
  return 0;
}
static inline int MPI_Win_free(MPI_Win *win)
{
  spss_mpi_window &w = spss_mpi_windows()[*win];
  if (w.used && w.owned) free(w.base);
  w.used = 0;
  w.base = 0;
  return 0;
}
static inline int MPI_Win_fence(int, MPI_Win) { return 0; }
static inline int MPI_Win_lock_all(int, MPI_Win) { return 0; }
static inline int MPI_Win_unlock_all(MPI_Win) { return 0; }
static inline int MPI_Win_sync(MPI_Win) { return 0; }
static inline int MPI_Put(const void *origin, int count, MPI_Datatype t, int, MPI_Aint disp, int, MPI_Datatype,
                          MPI_Win win)
{
  spss_mpi_window &w = spss_mpi_windows()[win];
  char *dst = (char *) w.base + disp * spss_mpi_type_size(t);
  if (dst != origin) memmove(dst, origin, (size_t) count * spss_mpi_type_size(t));
  return 0;
}
static inline int MPI_Get(void *origin, int count, MPI_Datatype t, int, MPI_Aint disp, int, MPI_Datatype,
                          MPI_Win win)
{
  spss_mpi_window &w = spss_mpi_windows()[win];
  const char *src = (const char *) w.base + disp * spss_mpi_type_size(t);
  if (src != origin) memmove(origin, src, (size_t) count * spss_mpi_type_size(t));
  return 0;
}
static inline int MPI_Isend(const void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *r) { *r = 0; return 0; }
static inline int MPI_Irecv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *r) { *r = 0; return 0; }
static inline int MPI_Send(const void *, int, MPI_Datatype, int, int, MPI_Comm) { return 0; }
static inline int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *) { return 0; }
static inline int MPI_Waitall(int, MPI_Request *, MPI_Status *) { return 0; }

#ifdef __cplusplus
}
#endif

#endif
