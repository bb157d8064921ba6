/*
 * ORACLE — test infrastructure only.  Single-rank stand-in for <mpi.h> so the
 * reference's block and driver sources build and run as one process: collective
 * reductions copy, point-to-point calls are never reached without CONNECT
 * boundaries and complete immediately.
 */
#ifndef ORACLE_STUB_MPI_H
#define ORACLE_STUB_MPI_H

#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_SUCCESS 0
#define MPI_COMM_WORLD 0
#define MPI_REQUEST_NULL (-1)
#define MPI_FLOAT 4
#define MPI_DOUBLE 8
#define MPI_INT 5
#define MPI_MIN 1
#define MPI_MAX 2
#define MPI_SUM 3
#define MPI_THREAD_MULTIPLE 3
#define MPI_STATUS_IGNORE ((MPI_Status *)0)

static inline int oracle_mpi_size(MPI_Datatype t) { return t == MPI_DOUBLE ? 8 : 4; }
static inline int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Init_thread(int *argc, char ***argv, int req, int *prov) { (void)argc; (void)argv; *prov = req; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
static inline int MPI_Allreduce(const void *in, void *out, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c) {
    (void)op; (void)c; memmove(out, in, (size_t)n * (size_t)oracle_mpi_size(t)); return 0;
}
static inline int MPI_Isend(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c, MPI_Request *r) {
    (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; *r = MPI_REQUEST_NULL; return 0;
}
static inline int MPI_Irecv(void *b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Request *r) {
    (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; *r = MPI_REQUEST_NULL; return 0;
}
static inline int MPI_Request_free(MPI_Request *r) { *r = MPI_REQUEST_NULL; return 0; }
static inline int MPI_Waitall(int n, MPI_Request *r, MPI_Status *s) { (void)n; (void)r; (void)s; return 0; }
static inline int MPI_Type_vector(int n, int bl, int st, MPI_Datatype o, MPI_Datatype *t) { (void)n; (void)bl; (void)st; *t = o; return 0; }
static inline int MPI_Type_commit(MPI_Datatype *t) { (void)t; return 0; }
static inline int MPI_Type_free(MPI_Datatype *t) { (void)t; return 0; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }

#endif
