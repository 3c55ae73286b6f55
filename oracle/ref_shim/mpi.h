/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * The subset of the MPI C interface that the reference simulator
 * (c++/src/NetworkGrowthSimulator.cpp) calls, implemented over threads of one
 * process so that the reference's own trial code can be compiled and run where
 * no MPI library exists.  Each rank is a thread; a rank's number is
 * thread-local (ugmpi_set_rank).  With the default world of one rank every
 * collective is a copy, which is the reference's `mpirun -np 1` semantics.
 *
 * Datatypes are MPI_INT, MPI_DOUBLE and the struct types the reference builds
 * with MPI_Type_create_struct; the only reduction is MPI_SUM, applied in rank
 * order so results do not depend on thread timing.  Point-to-point sends are
 * buffered (a send returns once its data is copied), which standard-mode MPI
 * permits.
 */
#ifndef UG_REF_SHIM_MPI_H
#define UG_REF_SHIM_MPI_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef ptrdiff_t MPI_Aint;

typedef struct {
    int MPI_SOURCE;
    int MPI_TAG;
    int MPI_ERROR;
    long bytes; /* size of the received message */
} MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_SUM 1
#define MPI_SUCCESS 0

int MPI_Init(int* argc, char*** argv);
int MPI_Finalize(void);
int MPI_Comm_size(MPI_Comm comm, int* size);
int MPI_Comm_rank(MPI_Comm comm, int* rank);
int MPI_Barrier(MPI_Comm comm);
int MPI_Bcast(void* buf, int count, MPI_Datatype type, int root, MPI_Comm comm);
int MPI_Allreduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype type, MPI_Op op, MPI_Comm comm);
int MPI_Allgather(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, int recvcount,
                  MPI_Datatype recvtype, MPI_Comm comm);
int MPI_Allgatherv(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, const int* recvcounts,
                   const int* displs, MPI_Datatype recvtype, MPI_Comm comm);
int MPI_Gatherv(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, const int* recvcounts,
                const int* displs, MPI_Datatype recvtype, int root, MPI_Comm comm);
int MPI_Scatterv(const void* sendbuf, const int* sendcounts, const int* displs, MPI_Datatype sendtype, void* recvbuf,
                 int recvcount, MPI_Datatype recvtype, int root, MPI_Comm comm);
int MPI_Send(const void* buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm);
int MPI_Recv(void* buf, int count, MPI_Datatype type, int source, int tag, MPI_Comm comm, MPI_Status* status);
int MPI_Get_count(const MPI_Status* status, MPI_Datatype type, int* count);
int MPI_Type_create_struct(int count, const int* blocklens, const MPI_Aint* displs, const MPI_Datatype* types,
                           MPI_Datatype* newtype);
int MPI_Type_commit(MPI_Datatype* type);

/* Thread world control (not MPI): set up a world of `size` ranks before any
 * rank thread starts, and give each rank thread its number. */
void ugmpi_init_world(int size);
void ugmpi_set_rank(int rank);

#ifdef __cplusplus
}
#endif

#endif
