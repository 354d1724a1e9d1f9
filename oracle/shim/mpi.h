/*
 * Single-rank MPI stand-in, used only to compile the reference tools/ sources
 * in place for the pinned CPU oracle (oracle/build_ref.py).  With one rank no
 * message is ever sent: point-to-point calls are unreachable, reductions copy.
 * Test infrastructure, not part of the product.
 */
#ifndef GADE_ORACLE_MPI_STUB_H
#define GADE_ORACLE_MPI_STUB_H
#include <string.h>
#include <stdio.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int source, tag, error; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 1
#define MPI_INT 2
#define MPI_SUM 0
#define MPI_REQUEST_NULL 0
#define MPI_DATATYPE_NULL 0
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
#define MPI_IN_PLACE ((void *)1)
#define MPI_MAX_ERROR_STRING 256

static inline int mpi_stub_size(MPI_Datatype t) { return t == MPI_DOUBLE ? 8 : 4; }
static inline int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
static inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op o, MPI_Comm c)
{ (void)o; (void)c; if (s != MPI_IN_PLACE) memcpy(r, s, (size_t)n * mpi_stub_size(t)); return 0; }
static inline int MPI_Allgather(const void *s, int sn, MPI_Datatype st, void *r, int rn, MPI_Datatype rt, MPI_Comm c)
{ (void)rn; (void)rt; (void)c; if (s != MPI_IN_PLACE) memcpy(r, s, (size_t)sn * mpi_stub_size(st)); return 0; }
static inline int mpi_stub_unreachable(const char *f) { fprintf(stderr, "MPI stub: %s called with one rank\n", f); return 1; }
static inline int MPI_Isend(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c, MPI_Request *q)
{ (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; (void)q; return mpi_stub_unreachable("MPI_Isend"); }
static inline int MPI_Irecv(void *b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Request *q)
{ (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; (void)q; return mpi_stub_unreachable("MPI_Irecv"); }
static inline int MPI_Send(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c)
{ (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; return mpi_stub_unreachable("MPI_Send"); }
static inline int MPI_Waitall(int n, MPI_Request *q, MPI_Status *s) { (void)n; (void)q; (void)s; return 0; }
static inline int MPI_Type_indexed(int n, const int *bl, const int *d, MPI_Datatype o, MPI_Datatype *t)
{ (void)n; (void)bl; (void)d; (void)o; *t = 0; return 0; }
static inline int MPI_Type_commit(MPI_Datatype *t) { (void)t; return 0; }
static inline int MPI_Error_string(int e, char *s, int *l) { *l = sprintf(s, "MPI stub error %d", e); return 0; }
#endif
