/*
 * Single-rank stand-in for the MPI interface used by the reference solve
 * path (checker build only).  With one rank every Allreduce is a copy,
 * point-to-point calls move zero values, and barriers are no-ops.
 */
#ifndef FEMREF_STUB_MPI_H
#define FEMREF_STUB_MPI_H
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_CHAR 1
#define MPI_INT 4
#define MPI_DOUBLE 8
#define MPI_SUM 0
#define MPI_MIN 1
#define MPI_MAX 2
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_SUCCESS 0

static inline int femref_dtsize(MPI_Datatype t) { return t == MPI_CHAR ? 1 : t; }
static inline int MPI_Init(int *a, char ***b) { (void)a; (void)b; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
static inline int MPI_Abort(MPI_Comm c, int code)
{ (void)c; fprintf(stderr, "reference called MPI_Abort(%d)\n", code); abort(); return code; }
static inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op o, MPI_Comm c)
{ (void)o; (void)c; memmove(r, s, (size_t)n * femref_dtsize(t)); return 0; }
static inline int MPI_Send(const void *b, int n, MPI_Datatype t, int d, int g, MPI_Comm c)
{ (void)b; (void)n; (void)t; (void)d; (void)g; (void)c; return 0; }
static inline int MPI_Isend(const void *b, int n, MPI_Datatype t, int d, int g, MPI_Comm c, MPI_Request *q)
{ (void)b; (void)n; (void)t; (void)d; (void)g; (void)c; *q = 0; return 0; }
static inline int MPI_Recv(void *b, int n, MPI_Datatype t, int s, int g, MPI_Comm c, MPI_Status *st)
{ (void)b; (void)n; (void)t; (void)s; (void)g; (void)c; (void)st; return 0; }
static inline int MPI_Request_free(MPI_Request *q) { (void)q; return 0; }
static inline int MPI_Wait(MPI_Request *q, MPI_Status *s) { (void)q; (void)s; return 0; }
static inline double MPI_Wtime(void) { return 0.0; }
#endif
