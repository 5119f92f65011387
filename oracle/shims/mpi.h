/*
 * Single-process stand-in for the MPI interface, used only to compile the
 * reference FMD sources as a CPU oracle on a machine without an MPI library.
 *
 * Test infrastructure: nothing in the product links against this header.
 *
 * With exactly one rank every collective is a copy from the send buffer to
 * the receive buffer, a broadcast is a no-op, and pack/unpack are memcpy with
 * a running byte offset.  Datatypes are represented by their size in bytes
 * (derived types take the extent given to MPI_Type_create_resized).
 * Point-to-point calls are never reached when the box is split into a single
 * subdomain (1,1,1); if one is reached anyway the process aborts with a message.
 */
#ifndef ORACLE_SHIM_MPI_H
#define ORACLE_SHIM_MPI_H

#include <limits.h>
#include <stdarg.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef int MPI_Comm;
typedef int MPI_Group;
typedef long MPI_Datatype;   /* byte size of one element */
typedef int MPI_Op;
typedef int MPI_Request;
typedef long MPI_Aint;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; int count_bytes; } MPI_Status;

#define MPI_SUCCESS 0
#define MPI_COMM_WORLD 1
#define MPI_COMM_NULL 0
#define MPI_PROC_NULL (-2)
#define MPI_UNDEFINED (-32766)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)

#define MPI_CHAR ((MPI_Datatype)sizeof(char))
#define MPI_INT ((MPI_Datatype)sizeof(int))
#define MPI_UNSIGNED ((MPI_Datatype)sizeof(unsigned))
#define MPI_FLOAT ((MPI_Datatype)sizeof(float))
#define MPI_DOUBLE ((MPI_Datatype)sizeof(double))
#define MPI_PACKED ((MPI_Datatype)1)

#define MPI_SUM 1
#define MPI_MIN 2
#define MPI_MAX 3

static inline void oshim_unreachable(const char *what)
{
    fprintf(stderr, "oracle mpi shim: %s is not available with one rank\n", what);
    abort();
}

static inline int MPI_Initialized(int *flag) { *flag = 1; return 0; }
static inline int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Finalized(int *flag) { *flag = 1; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *n) { (void)c; *n = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_group(MPI_Comm c, MPI_Group *g) { (void)c; *g = 1; return 0; }
static inline int MPI_Group_incl(MPI_Group g, int n, const int *r, MPI_Group *out)
{ (void)g; (void)n; (void)r; *out = 1; return 0; }
static inline int MPI_Group_free(MPI_Group *g) { *g = 0; return 0; }
static inline int MPI_Comm_create(MPI_Comm c, MPI_Group g, MPI_Comm *out)
{ (void)c; (void)g; *out = 1; return 0; }
static inline int MPI_Comm_create_group(MPI_Comm c, MPI_Group g, int tag, MPI_Comm *out)
{ (void)c; (void)g; (void)tag; *out = 1; return 0; }
static inline int MPI_Comm_split(MPI_Comm c, int color, int key, MPI_Comm *out)
{ (void)c; (void)key; *out = (color == MPI_UNDEFINED) ? MPI_COMM_NULL : 1; return 0; }
static inline int MPI_Comm_free(MPI_Comm *c) { *c = MPI_COMM_NULL; return 0; }

static inline double MPI_Wtime(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* derived datatypes: only their byte extent matters for one rank */
static inline int MPI_Type_contiguous(int n, MPI_Datatype old, MPI_Datatype *out)
{ *out = n * old; return 0; }
static inline int MPI_Type_create_struct(int n, const int *bl, const MPI_Aint *disp,
                                         const MPI_Datatype *types, MPI_Datatype *out)
{
    MPI_Aint end = 0;
    for (int i = 0; i < n; i++)
    {
        MPI_Aint e = disp[i] + bl[i] * types[i];
        if (e > end) end = e;
    }
    *out = end;
    return 0;
}
static inline int MPI_Type_create_resized(MPI_Datatype old, MPI_Aint lb, MPI_Aint ext, MPI_Datatype *out)
{ (void)old; (void)lb; *out = ext; return 0; }
static inline int MPI_Type_commit(MPI_Datatype *t) { (void)t; return 0; }
static inline int MPI_Type_free(MPI_Datatype *t) { *t = 0; return 0; }

static inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c)
{ (void)op; (void)c; if (n > 0 && s != r) memmove(r, s, (size_t)n * (size_t)t); return 0; }
static inline int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c)
{ (void)op; (void)root; (void)c; if (n > 0 && s != r) memmove(r, s, (size_t)n * (size_t)t); return 0; }
static inline int MPI_Bcast(void *b, int n, MPI_Datatype t, int root, MPI_Comm c)
{ (void)b; (void)n; (void)t; (void)root; (void)c; return 0; }
static inline int MPI_Gather(const void *s, int sn, MPI_Datatype st, void *r, int rn, MPI_Datatype rt,
                             int root, MPI_Comm c)
{ (void)rn; (void)rt; (void)root; (void)c; if (sn > 0 && r != NULL) memmove(r, s, (size_t)sn * (size_t)st); return 0; }
static inline int MPI_Gatherv(const void *s, int sn, MPI_Datatype st, void *r, const int *rc, const int *displs,
                              MPI_Datatype rt, int root, MPI_Comm c)
{
    (void)rc; (void)root; (void)c;
    if (sn > 0 && r != NULL)
        memmove((char *)r + (size_t)displs[0] * (size_t)rt, s, (size_t)sn * (size_t)st);
    return 0;
}

static inline int MPI_Pack_size(int n, MPI_Datatype t, MPI_Comm c, int *size)
{ (void)c; *size = n * (int)t; return 0; }
static inline int MPI_Pack(const void *in, int n, MPI_Datatype t, void *out, int outsize, int *pos, MPI_Comm c)
{
    (void)outsize; (void)c;
    size_t b = (size_t)n * (size_t)t;
    memcpy((char *)out + *pos, in, b);
    *pos += (int)b;
    return 0;
}
static inline int MPI_Unpack(const void *in, int insize, int *pos, void *out, int n, MPI_Datatype t, MPI_Comm c)
{
    (void)insize; (void)c;
    size_t b = (size_t)n * (size_t)t;
    memcpy(out, (const char *)in + *pos, b);
    *pos += (int)b;
    return 0;
}

static inline int MPI_Send(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c)
{ (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; oshim_unreachable("MPI_Send"); return 1; }
static inline int MPI_Recv(void *b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Status *st)
{ (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; (void)st; oshim_unreachable("MPI_Recv"); return 1; }
static inline int MPI_Isend(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c, MPI_Request *rq)
{ (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; (void)rq; oshim_unreachable("MPI_Isend"); return 1; }
static inline int MPI_Wait(MPI_Request *rq, MPI_Status *st)
{ (void)rq; (void)st; oshim_unreachable("MPI_Wait"); return 1; }
static inline int MPI_Probe(int s, int tag, MPI_Comm c, MPI_Status *st)
{ (void)s; (void)tag; (void)c; (void)st; oshim_unreachable("MPI_Probe"); return 1; }
static inline int MPI_Get_count(const MPI_Status *st, MPI_Datatype t, int *n)
{ (void)st; (void)t; *n = 0; oshim_unreachable("MPI_Get_count"); return 1; }
/* a Sendrecv with both peers MPI_PROC_NULL moves nothing */
static inline int MPI_Sendrecv(const void *sb, int sn, MPI_Datatype st, int d, int stag,
                               void *rb, int rn, MPI_Datatype rt, int s, int rtag, MPI_Comm c, MPI_Status *status)
{
    (void)sb; (void)sn; (void)st; (void)stag; (void)rb; (void)rn; (void)rt; (void)rtag; (void)c;
    if (status) status->count_bytes = 0;
    if (d != MPI_PROC_NULL || s != MPI_PROC_NULL) oshim_unreachable("MPI_Sendrecv to a peer");
    return 0;
}

#endif
