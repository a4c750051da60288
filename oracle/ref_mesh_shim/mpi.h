/* Single-rank stand-in for the MPI interface, written for the oracle build of
 * the reference's octree mesh (ot::Mesh, src/mesh.cpp and include/mesh.tcc),
 * which includes <mpi.h> throughout.  Test infrastructure only: it lets the
 * reference's own mesh construction, block set-up, unzip and zip run on one
 * rank in one process, so their outputs can pin this project's mesh.
 *
 * Semantics on one rank: the communicator has rank 0 and size 1; every
 * collective copies the caller's own contribution to the receive buffer
 * (a reduction over one rank is the identity); a point-to-point message to
 * oneself is matched by tag through a small mailbox; datatypes carry their
 * size in bytes.  Communicator and group management returns the same
 * communicator.  Nothing here is used by the product library.
 */
#ifndef DGB_ORACLE_MPI_STUB_H
#define DGB_ORACLE_MPI_STUB_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef int MPI_Comm;
typedef int MPI_Group;
typedef long MPI_Datatype; /* size in bytes */
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct {
    int MPI_SOURCE;
    int MPI_TAG;
    int MPI_ERROR;
    int count_bytes;
} MPI_Status;
typedef void(MPI_User_function)(void *, void *, int *, MPI_Datatype *);

#define MPI_COMM_WORLD 1
#define MPI_COMM_SELF 2
#define MPI_COMM_NULL 0
#define MPI_GROUP_NULL 0
#define MPI_SUCCESS 0
#define MPI_ERR_OTHER 15
#define MPI_MAX_ERROR_STRING 256
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
#define MPI_PROC_NULL (-2)
#define MPI_UNDEFINED (-32766)
#define MPI_REQUEST_NULL 0
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
#define MPI_IN_PLACE ((void *)1)

#define MPI_CHAR ((MPI_Datatype)1)
#define MPI_SIGNED_CHAR ((MPI_Datatype)1)
#define MPI_UNSIGNED_CHAR ((MPI_Datatype)1)
#define MPI_BYTE ((MPI_Datatype)1)
#define MPI_CXX_BOOL ((MPI_Datatype)sizeof(bool))
#define MPI_C_BOOL ((MPI_Datatype)1)
#define MPI_SHORT ((MPI_Datatype)2)
#define MPI_UNSIGNED_SHORT ((MPI_Datatype)2)
#define MPI_INT ((MPI_Datatype)4)
#define MPI_UNSIGNED ((MPI_Datatype)4)
#define MPI_LONG ((MPI_Datatype)sizeof(long))
#define MPI_UNSIGNED_LONG ((MPI_Datatype)sizeof(unsigned long))
#define MPI_LONG_LONG ((MPI_Datatype)8)
#define MPI_LONG_LONG_INT ((MPI_Datatype)8)
#define MPI_UNSIGNED_LONG_LONG ((MPI_Datatype)8)
#define MPI_FLOAT ((MPI_Datatype)4)
#define MPI_DOUBLE ((MPI_Datatype)8)
#define MPI_LONG_DOUBLE ((MPI_Datatype)sizeof(long double))
#define MPI_DOUBLE_INT ((MPI_Datatype)12)

#define MPI_MAX 1
#define MPI_MIN 2
#define MPI_SUM 3
#define MPI_PROD 4
#define MPI_LAND 5
#define MPI_LOR 6
#define MPI_BAND 7
#define MPI_BOR 8
#define MPI_MAXLOC 9
#define MPI_MINLOC 10

namespace dgb_mpi_stub {
struct Msg {
    const void *buf;
    void *rbuf;
    long bytes;
    int tag;
    int live;
};
inline Msg *box(int send)
{
    static Msg s[4096], r[4096];
    return send ? s : r;
}
inline int &nbox(int send)
{
    static int ns = 0, nr = 0;
    return send ? ns : nr;
}
/* match a pending send with a pending receive of the same tag */
inline void match(void)
{
    Msg *s = box(1), *r = box(0);
    for (int i = 0; i < nbox(1); i++) {
        if (!s[i].live) continue;
        for (int j = 0; j < nbox(0); j++) {
            if (!r[j].live || (r[j].tag != s[i].tag && r[j].tag != MPI_ANY_TAG)) continue;
            memcpy(r[j].rbuf, s[i].buf, (size_t)(s[i].bytes < r[j].bytes ? s[i].bytes : r[j].bytes));
            s[i].live = r[j].live = 0;
            break;
        }
    }
}
inline void push(int send, const void *b, void *rb, long bytes, int tag)
{
    if (nbox(send) >= 4096) {
        fprintf(stderr, "mpi stub: mailbox full\n");
        abort();
    }
    Msg m = {b, rb, bytes, tag, 1};
    box(send)[nbox(send)++] = m;
    match();
}
inline void copy(const void *s, void *r, long bytes)
{
    if (s == MPI_IN_PLACE || s == r || bytes <= 0) return;
    memmove(r, s, (size_t)bytes);
}
}  // namespace dgb_mpi_stub

static inline int MPI_Init(int *, char ***) { return MPI_SUCCESS; }
static inline int MPI_Initialized(int *f) { *f = 1; return MPI_SUCCESS; }
static inline int MPI_Finalize(void) { return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm, int *n) { *n = 1; return MPI_SUCCESS; }
static inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
static inline double MPI_Wtime(void)
{
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}
static inline int MPI_Abort(MPI_Comm, int code)
{
    fprintf(stderr, "mpi stub: MPI_Abort(%d)\n", code);
    abort();
    return code;
}
static inline int MPI_Error_string(int code, char *s, int *len)
{
    *len = snprintf(s, MPI_MAX_ERROR_STRING, "mpi stub error %d", code);
    return MPI_SUCCESS;
}
static inline int MPI_Comm_dup(MPI_Comm c, MPI_Comm *o) { *o = c; return MPI_SUCCESS; }
static inline int MPI_Comm_free(MPI_Comm *) { return MPI_SUCCESS; }
static inline int MPI_Comm_split(MPI_Comm c, int color, int, MPI_Comm *o)
{
    *o = color == MPI_UNDEFINED ? MPI_COMM_NULL : c;
    return MPI_SUCCESS;
}
static inline int MPI_Comm_group(MPI_Comm, MPI_Group *g) { *g = 1; return MPI_SUCCESS; }
static inline int MPI_Group_incl(MPI_Group g, int, const int *, MPI_Group *o) { *o = g; return MPI_SUCCESS; }
static inline int MPI_Group_free(MPI_Group *) { return MPI_SUCCESS; }
static inline int MPI_Comm_create(MPI_Comm c, MPI_Group, MPI_Comm *o) { *o = c; return MPI_SUCCESS; }
static inline int MPI_Type_contiguous(int n, MPI_Datatype t, MPI_Datatype *o) { *o = (MPI_Datatype)n * t; return MPI_SUCCESS; }
static inline int MPI_Type_commit(MPI_Datatype *) { return MPI_SUCCESS; }
static inline int MPI_Type_free(MPI_Datatype *) { return MPI_SUCCESS; }
static inline int MPI_Op_create(MPI_User_function *, int, MPI_Op *op)
{
    static int next = 100;
    *op = next++;
    return MPI_SUCCESS;
}
static inline int MPI_Op_free(MPI_Op *) { return MPI_SUCCESS; }

static inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm)
{ dgb_mpi_stub::copy(s, r, (long)n * t); return MPI_SUCCESS; }
static inline int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm)
{ dgb_mpi_stub::copy(s, r, (long)n * t); return MPI_SUCCESS; }
static inline int MPI_Scan(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm)
{ dgb_mpi_stub::copy(s, r, (long)n * t); return MPI_SUCCESS; }
static inline int MPI_Exscan(const void *, void *, int, MPI_Datatype, MPI_Op, MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Alltoall(const void *s, int sn, MPI_Datatype st, void *r, int, MPI_Datatype, MPI_Comm)
{ dgb_mpi_stub::copy(s, r, (long)sn * st); return MPI_SUCCESS; }
static inline int MPI_Alltoallv(const void *s, const int *sc, const int *sd, MPI_Datatype st, void *r,
                                const int *, const int *rd, MPI_Datatype rt, MPI_Comm)
{
    dgb_mpi_stub::copy((const char *)s + (long)sd[0] * st, (char *)r + (long)rd[0] * rt, (long)sc[0] * st);
    return MPI_SUCCESS;
}
static inline int MPI_Allgather(const void *s, int sn, MPI_Datatype st, void *r, int, MPI_Datatype, MPI_Comm)
{ dgb_mpi_stub::copy(s, r, (long)sn * st); return MPI_SUCCESS; }
static inline int MPI_Allgatherv(const void *s, int sn, MPI_Datatype st, void *r, const int *, const int *rd,
                                 MPI_Datatype rt, MPI_Comm)
{ dgb_mpi_stub::copy(s, (char *)r + (long)rd[0] * rt, (long)sn * st); return MPI_SUCCESS; }
static inline int MPI_Gather(const void *s, int sn, MPI_Datatype st, void *r, int, MPI_Datatype, int, MPI_Comm)
{ dgb_mpi_stub::copy(s, r, (long)sn * st); return MPI_SUCCESS; }
static inline int MPI_Gatherv(const void *s, int sn, MPI_Datatype st, void *r, const int *, const int *rd,
                              MPI_Datatype rt, int, MPI_Comm)
{ dgb_mpi_stub::copy(s, (char *)r + (long)rd[0] * rt, (long)sn * st); return MPI_SUCCESS; }
static inline int MPI_Scatter(const void *s, int sn, MPI_Datatype st, void *r, int, MPI_Datatype, int, MPI_Comm)
{ dgb_mpi_stub::copy(s, r, (long)sn * st); return MPI_SUCCESS; }

static inline int MPI_Isend(const void *b, int n, MPI_Datatype t, int, int tag, MPI_Comm, MPI_Request *q)
{ dgb_mpi_stub::push(1, b, 0, (long)n * t, tag); *q = 0; return MPI_SUCCESS; }
static inline int MPI_Issend(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c, MPI_Request *q)
{ return MPI_Isend(b, n, t, d, tag, c, q); }
static inline int MPI_Send(const void *b, int n, MPI_Datatype t, int, int tag, MPI_Comm)
{ dgb_mpi_stub::push(1, b, 0, (long)n * t, tag); return MPI_SUCCESS; }
static inline int MPI_Irecv(void *b, int n, MPI_Datatype t, int, int tag, MPI_Comm, MPI_Request *q)
{ dgb_mpi_stub::push(0, 0, b, (long)n * t, tag); *q = 0; return MPI_SUCCESS; }
static inline int MPI_Recv(void *b, int n, MPI_Datatype t, int, int tag, MPI_Comm, MPI_Status *)
{ dgb_mpi_stub::push(0, 0, b, (long)n * t, tag); return MPI_SUCCESS; }
static inline int MPI_Sendrecv(const void *s, int sn, MPI_Datatype st, int, int, void *r, int rn, MPI_Datatype rt,
                               int, int, MPI_Comm, MPI_Status *)
{
    const long sb = (long)sn * st, rb = (long)rn * rt;
    if (s && r) dgb_mpi_stub::copy(s, r, sb < rb ? sb : rb);
    return MPI_SUCCESS;
}
static inline int MPI_Wait(MPI_Request *, MPI_Status *) { return MPI_SUCCESS; }
static inline int MPI_Waitall(int, MPI_Request *, MPI_Status *) { return MPI_SUCCESS; }
static inline int MPI_Test(MPI_Request *, int *f, MPI_Status *) { *f = 1; return MPI_SUCCESS; }
static inline int MPI_Get_count(const MPI_Status *s, MPI_Datatype t, int *n) { *n = s ? (int)(s->count_bytes / t) : 0; return MPI_SUCCESS; }

#endif
