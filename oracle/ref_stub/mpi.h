/* Single-rank stand-in for the MPI API, used only to compile the reference
 * metaLBM CPU path as a test oracle (no MPI runtime exists in this image).
 * Everything is a no-op returning 0 except the point-to-point pair: with one
 * rank, metaLBM's X halo exchange (Communication.h:134-180) posts an
 * MPI_Irecv into the halo plane and then an MPI_Isend of the opposite
 * interior plane with the same tag; this stub copies the send buffer into the
 * pending receive buffer, which is the periodic self-exchange one rank needs. */
#pragma once
#include <cstring>
typedef int MPI_Comm;
typedef int MPI_Info;
typedef int MPI_Status;
typedef int MPI_Request;
typedef int MPI_Datatype;
typedef int MPI_Op;
#define MPI_SUCCESS 0
#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 8
#define MPI_SUM 0
#define MPI_IN_PLACE ((void*)1)
#define MPI_MAX_PROCESSOR_NAME 64
#define MPI_THREAD_FUNNELED 1
#define MPI_COMM_TYPE_SHARED 0
#define MPI_INFO_NULL 0
template <class... A> inline int mlbm_mpi_noop(A...) { return 0; }
#define MPI_Init_thread mlbm_mpi_noop
#define MPI_Get_processor_name mlbm_mpi_noop
#define MPI_Abort mlbm_mpi_noop
#define MPI_Finalize mlbm_mpi_noop
#define MPI_Barrier mlbm_mpi_noop
#define MPI_Scatter mlbm_mpi_noop
#define MPI_Gather mlbm_mpi_noop
#define MPI_Waitall mlbm_mpi_noop
#define MPI_Info_create mlbm_mpi_noop
#define MPI_Info_free mlbm_mpi_noop
#define MPI_Comm_split_type mlbm_mpi_noop
#define MPI_Comm_free mlbm_mpi_noop
inline int MPI_Comm_size(MPI_Comm, int* n) { *n = 1; return 0; }
inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
/* One rank: a reduction to rank 0 is a copy (count doubles). */
inline int MPI_Reduce(const void* s, void* r, int count, MPI_Datatype, MPI_Op, int, MPI_Comm) {
  if (s != MPI_IN_PLACE && s != r) std::memmove(r, s, sizeof(double) * (size_t)count);
  return 0;
}
struct MlbmPendingRecv { void* buf; int count; int tag; };
inline MlbmPendingRecv& mlbm_pending_recv() { static MlbmPendingRecv p{nullptr, 0, -1}; return p; }
inline int MPI_Irecv(void* buf, int count, MPI_Datatype, int, int tag, MPI_Comm, MPI_Request*) {
  mlbm_pending_recv() = {buf, count, tag};
  return 0;
}
inline int MPI_Isend(const void* buf, int count, MPI_Datatype, int, int tag, MPI_Comm, MPI_Request*) {
  MlbmPendingRecv& p = mlbm_pending_recv();
  if (p.tag == tag && p.buf) { std::memmove(p.buf, buf, sizeof(double) * (size_t)count); p.tag = -1; }
  return 0;
}
