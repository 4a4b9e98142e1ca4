/*
 * Single-rank MPI stand-in, test infrastructure only: lets the reference's
 * own sources compile and run as one process (rank 0 of 1) for the oracle
 * pinning harness. Point-to-point calls to oneself copy the send buffer into
 * the receive buffer; reductions over one rank copy the input.
 * A datatype is its element size in bytes.
 */
#ifndef BT_MPI_STUB_H
#define BT_MPI_STUB_H
#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_CHAR 1
#define MPI_INT 4
#define MPI_FLOAT 4
#define MPI_DOUBLE 8
#define MPI_SUM 0
#define MPI_MAX 1
#define MPI_MIN 2

static inline int MPI_Init(int* argc, char*** argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int* n) { (void)c; *n = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int* r) { (void)c; *r = 0; return 0; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }

static inline int MPI_Sendrecv(const void* sbuf, int scount, MPI_Datatype stype, int dest, int stag,
                               void* rbuf, int rcount, MPI_Datatype rtype, int src, int rtag,
                               MPI_Comm c, MPI_Status* st) {
    (void)scount; (void)stype; (void)dest; (void)stag; (void)src; (void)rtag; (void)c; (void)st;
    memmove(rbuf, sbuf, (size_t)rcount * (size_t)rtype);
    return 0;
}

static inline int MPI_Reduce(const void* sbuf, void* rbuf, int count, MPI_Datatype t, MPI_Op op,
                             int root, MPI_Comm c) {
    (void)op; (void)root; (void)c;
    memmove(rbuf, sbuf, (size_t)count * (size_t)t);
    return 0;
}

static inline int MPI_Allreduce(const void* sbuf, void* rbuf, int count, MPI_Datatype t, MPI_Op op,
                                MPI_Comm c) {
    (void)op; (void)c;
    memmove(rbuf, sbuf, (size_t)count * (size_t)t);
    return 0;
}
#endif
