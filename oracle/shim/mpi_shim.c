/* Single-rank MPI stand-in (see mpi.h).  Test infrastructure only. */
#define _POSIX_C_SOURCE 199309L
#include "mpi.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

static size_t type_size(MPI_Datatype t) {
    switch (t) {
    case MPI_CHAR:
    case MPI_BYTE: return 1;
    case MPI_INT: return sizeof(int);
    case MPI_FLOAT: return sizeof(float);
    case MPI_DOUBLE: return sizeof(double);
    default: return 0;
    }
}

int MPI_Init(int *argc, char ***argv) {
    (void)argc;
    (void)argv;
    return MPI_SUCCESS;
}
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm comm, int *rank) {
    (void)comm;
    *rank = 0;
    return MPI_SUCCESS;
}
int MPI_Comm_size(MPI_Comm comm, int *size) {
    (void)comm;
    *size = 1;
    return MPI_SUCCESS;
}
int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype type, MPI_Op op,
                  MPI_Comm comm) {
    (void)op;
    (void)comm;
    if (sendbuf != recvbuf) memmove(recvbuf, sendbuf, (size_t)count * type_size(type));
    return MPI_SUCCESS;
}
int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm) {
    (void)buf;
    (void)count;
    (void)type;
    (void)root;
    (void)comm;
    return MPI_SUCCESS;
}
int MPI_Barrier(MPI_Comm comm) {
    (void)comm;
    return MPI_SUCCESS;
}
int MPI_Send(const void *buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm) {
    (void)buf;
    (void)count;
    (void)type;
    (void)dest;
    (void)tag;
    (void)comm;
    fprintf(stderr, "mpi shim: MPI_Send on a single rank\n");
    abort();
}
int MPI_Recv(void *buf, int count, MPI_Datatype type, int source, int tag, MPI_Comm comm,
             MPI_Status *status) {
    (void)buf;
    (void)count;
    (void)type;
    (void)source;
    (void)tag;
    (void)comm;
    (void)status;
    fprintf(stderr, "mpi shim: MPI_Recv on a single rank\n");
    abort();
}
int MPI_Gatherv(const void *sendbuf, int sendcount, MPI_Datatype sendtype, void *recvbuf,
                const int *recvcounts, const int *displs, MPI_Datatype recvtype, int root,
                MPI_Comm comm) {
    (void)recvcounts;
    (void)recvtype;
    (void)root;
    (void)comm;
    memmove((char *)recvbuf + (size_t)displs[0] * type_size(sendtype), sendbuf,
            (size_t)sendcount * type_size(sendtype));
    return MPI_SUCCESS;
}
int MPI_Abort(MPI_Comm comm, int errorcode) {
    (void)comm;
    fprintf(stderr, "mpi shim: MPI_Abort(%d)\n", errorcode);
    abort();
}
double MPI_Wtime(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
