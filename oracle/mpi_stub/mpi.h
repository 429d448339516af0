/*
 * Single-rank stand-in for <mpi.h>.
 *
 * Test infrastructure only: lets the reference lbsolver/io headers compile and
 * run as one rank (rank 0 of 1) so that the reference time loop can be executed
 * on the host and used as the oracle.  Collective calls copy send buffers to
 * receive buffers; point-to-point calls are never reached at one rank (the
 * reference's BndMpi list is empty there) and report an error if they are.
 * MPI-IO calls used by the PVTU writer map onto stdio.
 */
#ifndef BCLBM_ORACLE_MPI_STUB_H
#define BCLBM_ORACLE_MPI_STUB_H

#include <stdio.h>
#include <string.h>
#include <stdlib.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Info;
typedef long long MPI_Offset;
typedef FILE* MPI_File;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_INFO_NULL 0
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3

#define MPI_CHAR 1
#define MPI_INT 4
#define MPI_LONG 8
#define MPI_DOUBLE 108
#define MPI_FLOAT 104

#define MPI_MODE_APPEND 1
#define MPI_MODE_WRONLY 2
#define MPI_MODE_CREATE 4
#define MPI_SEEK_SET 0

static inline size_t bclbm_stub_type_size(MPI_Datatype t) {
    switch (t) {
        case MPI_CHAR: return 1;
        case MPI_INT: return sizeof(int);
        case MPI_LONG: return sizeof(long);
        case MPI_FLOAT: return sizeof(float);
        case MPI_DOUBLE: return sizeof(double);
        default: return 1;
    }
}

static inline int MPI_Init(int*, char***) { return 0; }
static inline int MPI_Initialized(int* flag) { *flag = 1; return 0; }
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Comm_size(MPI_Comm, int* n) { *n = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }

static inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
    if (s != r) memcpy(r, s, (size_t)n * bclbm_stub_type_size(t));
    return 0;
}
static inline int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
    if (s != r) memcpy(r, s, (size_t)n * bclbm_stub_type_size(t));
    return 0;
}
static inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return 0; }

static inline int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm) {
    fprintf(stderr, "mpi stub: MPI_Send reached at one rank\n");
    abort();
}
static inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) {
    fprintf(stderr, "mpi stub: MPI_Recv reached at one rank\n");
    abort();
}

static inline int MPI_File_open(MPI_Comm, const char* name, int, MPI_Info, MPI_File* fh) {
    *fh = fopen(name, "r+b");
    return *fh ? 0 : 1;
}
static inline int MPI_File_seek(MPI_File fh, MPI_Offset off, int) {
    return fseek(fh, (long)off, SEEK_SET);
}
static inline int MPI_File_write(MPI_File fh, const void* buf, int n, MPI_Datatype t, MPI_Status*) {
    fwrite(buf, bclbm_stub_type_size(t), (size_t)n, fh);
    return 0;
}
static inline int MPI_File_close(MPI_File* fh) { fclose(*fh); *fh = 0; return 0; }

#endif
