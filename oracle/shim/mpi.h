/*
 * Single-rank stand-in for <mpi.h>, used ONLY to compile the reference's own
 * AREC3D sources into oracle/_ref (test infrastructure; never linked into the
 * product library).  Every collective is the identity on one rank.
 *
 * Covers the MPI symbols the reference path references
 * (AREC3D/AREC3D/{arecImage,arecproject,areccgls,areccgls_KB,arecsirt,
 * arecsirt_KB,align2dstack,imagetools,arecImageIO,arecImageIO_mpi}.cpp).
 */
#pragma once
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct {
    int MPI_SOURCE, MPI_TAG, MPI_ERROR, count;
} MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_CHAR 1
#define MPI_INT 2
#define MPI_FLOAT 3
#define MPI_DOUBLE 4
#define MPI_BYTE 5
#define MPI_SUM 1
#define MPI_MIN 2
#define MPI_MAX 3
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype type, MPI_Op op,
                  MPI_Comm comm);
int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm);
int MPI_Barrier(MPI_Comm comm);
int MPI_Send(const void *buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm);
int MPI_Recv(void *buf, int count, MPI_Datatype type, int source, int tag, MPI_Comm comm,
             MPI_Status *status);
int MPI_Gatherv(const void *sendbuf, int sendcount, MPI_Datatype sendtype, void *recvbuf,
                const int *recvcounts, const int *displs, MPI_Datatype recvtype, int root,
                MPI_Comm comm);
int MPI_Abort(MPI_Comm comm, int errorcode);
double MPI_Wtime(void);

#ifdef __cplusplus
}
#endif
