/*
 * mpi.h -- single-rank stand-in for MPI, used only to compile the reference's
 * own generator, CSR build, CPU BFS and validator sources into oracle/_ref.
 *
 * TEST INFRASTRUCTURE ONLY.  There is one process and one rank: every
 * collective is a copy from the send buffer to the receive buffer (or a no-op
 * in place), communicator splits return the world, and point-to-point or
 * one-sided calls, which a 1x1 process grid never issues, abort.
 */
#ifndef G5_REFSHIM_MPI_H
#define G5_REFSHIM_MPI_H

#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MPI_VERSION 3
#define MPI_SUBVERSION 0
#define MPI_SUCCESS 0
#define MPI_MAX_ERROR_STRING 256
#define MPI_UNDEFINED (-32766)
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
#define MPI_MODE_NOPRECEDE 1
#define MPI_MODE_NOSUCCEED 2
#define MPI_MODE_NOPUT 4
#define MPI_MODE_NOSTORE 8

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Info;
typedef int MPI_Request;
typedef intptr_t MPI_Aint;
typedef struct { int count_bytes; int MPI_SOURCE; int MPI_TAG; int MPI_ERROR; } MPI_Status;
typedef struct g5_shim_win { char *base; MPI_Aint size; int disp; } *MPI_Win;

#define MPI_COMM_WORLD 1
#define MPI_COMM_SELF 2
#define MPI_COMM_NULL 0
#define MPI_INFO_NULL 0
#define MPI_REQUEST_NULL 0
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
#define MPI_IN_PLACE ((void *)(intptr_t)-1)

enum {
    MPI_DATATYPE_NULL = 0, MPI_CHAR, MPI_SIGNED_CHAR, MPI_UNSIGNED_CHAR, MPI_BYTE,
    MPI_SHORT, MPI_UNSIGNED_SHORT, MPI_INT, MPI_UNSIGNED, MPI_LONG,
    MPI_UNSIGNED_LONG, MPI_LONG_LONG, MPI_UNSIGNED_LONG_LONG, MPI_FLOAT,
    MPI_DOUBLE, MPI_INT8_T, MPI_INT16_T, MPI_INT32_T, MPI_INT64_T, MPI_UINT8_T,
    MPI_UINT16_T, MPI_UINT32_T, MPI_UINT64_T, MPI_AINT, MPI_C_BOOL,
    G5_SHIM_FIRST_DERIVED
};
#define MPI_LONG_LONG_INT MPI_LONG_LONG

enum { MPI_OP_NULL = 0, MPI_SUM, MPI_MAX, MPI_MIN, MPI_LOR, MPI_LAND, MPI_BOR,
       MPI_BAND, MPI_REPLACE };

#define G5_SHIM_MAXTYPES 64
static int g5_shim_derived_size[G5_SHIM_MAXTYPES];
static int g5_shim_ntypes = G5_SHIM_FIRST_DERIVED;

static inline int g5_shim_size(MPI_Datatype t)
{
    static const int sz[] = {0, 1, 1, 1, 1, 2, 2, 4, 4, (int)sizeof(long),
                             (int)sizeof(unsigned long), 8, 8, 4, 8, 1, 2, 4, 8,
                             1, 2, 4, 8, (int)sizeof(MPI_Aint), 1};
    if (t >= 0 && t < G5_SHIM_FIRST_DERIVED) return sz[t];
    if (t >= G5_SHIM_FIRST_DERIVED && t < G5_SHIM_MAXTYPES) return g5_shim_derived_size[t];
    return 0;
}

static inline void g5_shim_unsupported(const char *what)
{
    fprintf(stderr, "single-rank MPI shim: %s is not available\n", what);
    abort();
}

static inline int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
static inline int MPI_Comm_split(MPI_Comm c, int color, int key, MPI_Comm *out)
{ (void)color; (void)key; *out = c; return 0; }
static inline int MPI_Comm_dup(MPI_Comm c, MPI_Comm *out) { *out = c; return 0; }
static inline int MPI_Comm_free(MPI_Comm *c) { *c = MPI_COMM_NULL; return 0; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
static inline int MPI_Abort(MPI_Comm c, int code) { (void)c; exit(code ? code : 1); }
static inline double MPI_Wtime(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
static inline int MPI_Error_string(int code, char *s, int *len)
{ *len = snprintf(s, MPI_MAX_ERROR_STRING, "error %d", code); return 0; }

static inline int MPI_Alloc_mem(MPI_Aint n, MPI_Info info, void *baseptr)
{ (void)info; *(void **)baseptr = malloc(n ? (size_t)n : 1); return 0; }
static inline int MPI_Free_mem(void *p) { free(p); return 0; }

static inline int MPI_Type_size(MPI_Datatype t, int *s) { *s = g5_shim_size(t); return 0; }
static inline int MPI_Type_create_struct(int n, const int *bl, const MPI_Aint *disp,
                                         const MPI_Datatype *types, MPI_Datatype *out)
{
    int ext = 0;
    for (int i = 0; i < n; ++i) {
        int end = (int)disp[i] + bl[i] * g5_shim_size(types[i]);
        if (end > ext) ext = end;
    }
    if (g5_shim_ntypes >= G5_SHIM_MAXTYPES) g5_shim_unsupported("more derived types");
    g5_shim_derived_size[g5_shim_ntypes] = ext;
    *out = g5_shim_ntypes++;
    return 0;
}
static inline int MPI_Type_contiguous(int n, MPI_Datatype t, MPI_Datatype *out)
{
    if (g5_shim_ntypes >= G5_SHIM_MAXTYPES) g5_shim_unsupported("more derived types");
    g5_shim_derived_size[g5_shim_ntypes] = n * g5_shim_size(t);
    *out = g5_shim_ntypes++;
    return 0;
}
static inline int MPI_Type_commit(MPI_Datatype *t) { (void)t; return 0; }
static inline int MPI_Type_free(MPI_Datatype *t) { *t = MPI_DATATYPE_NULL; return 0; }
static inline int MPI_Get_count(const MPI_Status *st, MPI_Datatype t, int *count)
{ *count = st->count_bytes / g5_shim_size(t); return 0; }

static inline void g5_shim_copy(const void *s, void *r, size_t bytes)
{
    if (s != MPI_IN_PLACE && s != r && bytes) memmove(r, s, bytes);
}

static inline int MPI_Bcast(void *b, int n, MPI_Datatype t, int root, MPI_Comm c)
{ (void)b; (void)n; (void)t; (void)root; (void)c; return 0; }
static inline int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c)
{ (void)op; (void)root; (void)c; g5_shim_copy(s, r, (size_t)n * g5_shim_size(t)); return 0; }
static inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c)
{ (void)op; (void)c; g5_shim_copy(s, r, (size_t)n * g5_shim_size(t)); return 0; }
static inline int MPI_Allgather(const void *s, int sn, MPI_Datatype st, void *r, int rn, MPI_Datatype rt, MPI_Comm c)
{ (void)rn; (void)rt; (void)c; g5_shim_copy(s, r, (size_t)sn * g5_shim_size(st)); return 0; }
static inline int MPI_Allgatherv(const void *s, int sn, MPI_Datatype st, void *r, const int *rc,
                                 const int *displs, MPI_Datatype rt, MPI_Comm c)
{
    (void)rc; (void)c;
    if (s == MPI_IN_PLACE) return 0;
    g5_shim_copy(s, (char *)r + (size_t)displs[0] * g5_shim_size(rt), (size_t)sn * g5_shim_size(st));
    return 0;
}
static inline int MPI_Alltoall(const void *s, int sn, MPI_Datatype st, void *r, int rn, MPI_Datatype rt, MPI_Comm c)
{ (void)rn; (void)rt; (void)c; g5_shim_copy(s, r, (size_t)sn * g5_shim_size(st)); return 0; }
static inline int MPI_Alltoallv(const void *s, const int *sc, const int *sd, MPI_Datatype st, void *r,
                                const int *rc, const int *rd, MPI_Datatype rt, MPI_Comm c)
{
    (void)rc; (void)c;
    g5_shim_copy((const char *)s + (size_t)sd[0] * g5_shim_size(st),
                 (char *)r + (size_t)rd[0] * g5_shim_size(rt), (size_t)sc[0] * g5_shim_size(st));
    return 0;
}
static inline int MPI_Sendrecv(const void *s, int sn, MPI_Datatype st, int dst, int stag, void *r, int rn,
                               MPI_Datatype rt, int src, int rtag, MPI_Comm c, MPI_Status *status)
{
    (void)dst; (void)stag; (void)rn; (void)rt; (void)src; (void)rtag; (void)c;
    g5_shim_copy(s, r, (size_t)sn * g5_shim_size(st));
    if (status) status->count_bytes = sn * g5_shim_size(st);
    return 0;
}

static inline int MPI_Send(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c)
{ (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; g5_shim_unsupported("MPI_Send"); return 1; }
static inline int MPI_Recv(void *b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Status *st)
{ (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; (void)st; g5_shim_unsupported("MPI_Recv"); return 1; }
static inline int MPI_Issend(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c, MPI_Request *rq)
{ (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; (void)rq; g5_shim_unsupported("MPI_Issend"); return 1; }
static inline int MPI_Iprobe(int s, int tag, MPI_Comm c, int *flag, MPI_Status *st)
{ (void)s; (void)tag; (void)c; (void)st; *flag = 0; return 0; }
static inline int MPI_Test(MPI_Request *rq, int *flag, MPI_Status *st)
{ (void)rq; (void)st; *flag = 1; return 0; }
static inline int MPI_Win_create(void *base, MPI_Aint size, int disp, MPI_Info info, MPI_Comm c, MPI_Win *w)
{
    (void)info; (void)c;
    *w = (MPI_Win)malloc(sizeof(struct g5_shim_win));
    (*w)->base = (char *)base; (*w)->size = size; (*w)->disp = disp;
    return 0;
}
static inline int MPI_Win_free(MPI_Win *w) { free(*w); *w = 0; return 0; }
static inline int MPI_Win_fence(int a, MPI_Win w) { (void)a; (void)w; return 0; }
static inline int MPI_Get(void *o, int on, MPI_Datatype ot, int rank, MPI_Aint disp, int tn, MPI_Datatype tt, MPI_Win w)
{ (void)on; (void)rank; (void)tt; memcpy(o, w->base + disp * w->disp, (size_t)tn * g5_shim_size(ot)); return 0; }
static inline int MPI_Put(const void *o, int on, MPI_Datatype ot, int rank, MPI_Aint disp, int tn, MPI_Datatype tt, MPI_Win w)
{ (void)tn; (void)rank; (void)tt; memcpy(w->base + disp * w->disp, o, (size_t)on * g5_shim_size(ot)); return 0; }

#ifdef __cplusplus
}
#endif
#endif
