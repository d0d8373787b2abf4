/*
 * Single-rank MPI stand-in — ORACLE TEST INFRASTRUCTURE ONLY.
 *
 * No MPI implementation is installed on either build machine, yet the
 * reference framework's CPU path (APPFIS_CPU) includes "mpi.h" and calls MPI on
 * every halo exchange and reduction.  This header implements exactly the calls
 * the reference makes (Appfis/Topology.hpp:118-206, Appfis/Communication.hpp:49-828)
 * for a world of ONE rank, so that the reference's own OpenMP code can be built
 * unchanged and used as the parity oracle and as the timed CPU baseline:
 *
 *   Comm_size = 1, rank = 0; Dims_create fills zero entries with 1;
 *   Cart_shift returns self (0) on periodic axes, MPI_PROC_NULL otherwise;
 *   Sendrecv to self copies through the two datatypes (MPI_BYTE / basic types /
 *   C-order subarrays, as used by Scatter, Gather and Exchange);
 *   Allreduce copies; Barrier and Type_free are no-ops.
 *
 * Nothing in the product library includes this file.
 */
#ifndef APPFIS_ORACLE_MPI_STUB_H
#define APPFIS_ORACLE_MPI_STUB_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifdef __cplusplus
extern "C++" {
#endif

typedef int MPI_Comm;
typedef int MPI_Op;
typedef struct { int MPI_SOURCE; int MPI_TAG; int MPI_ERROR; } MPI_Status;
typedef int MPI_Request;

/* A datatype is a small descriptor: a basic element or a C-order subarray. */
struct mpistub_type {
    int basic_size;     /* bytes of one element */
    int is_subarray;
    int ndims;
    int sizes[3];
    int subsizes[3];
    int starts[3];
};
typedef struct mpistub_type* MPI_Datatype;

static struct mpistub_type mpistub_byte = {1, 0, 0, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
static struct mpistub_type mpistub_int = {4, 0, 0, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
static struct mpistub_type mpistub_float = {4, 0, 0, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
static struct mpistub_type mpistub_double = {8, 0, 0, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};

#define MPI_BYTE (&mpistub_byte)
#define MPI_INT (&mpistub_int)
#define MPI_FLOAT (&mpistub_float)
#define MPI_DOUBLE (&mpistub_double)
#define MPI_COMM_WORLD 0
#define MPI_PROC_NULL (-2)
#define MPI_ORDER_C 56
#define MPI_MAX 1
#define MPI_MIN 2
#define MPI_SUM 3
#define MPI_SUCCESS 0

static inline void mpistub_fail(const char* what)
{
    fprintf(stderr, "mpi stand-in: %s is not available with one rank\n", what);
    abort();
}

static inline int MPI_Init(int*, char***) { return MPI_SUCCESS; }
static inline int MPI_Finalize() { return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm, int* n) { *n = 1; return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return MPI_SUCCESS; }
static inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }

static inline int MPI_Dims_create(int nnodes, int ndims, int* dims)
{
    if (nnodes != 1) mpistub_fail("Dims_create with more than one node");
    for (int i = 0; i < ndims; i++)
        if (dims[i] == 0) dims[i] = 1;
    return MPI_SUCCESS;
}

/* periodicity per axis of the one Cartesian communicator */
static int mpistub_periods[3] = {0, 0, 0};

static inline int MPI_Cart_create(MPI_Comm, int ndims, const int*, const int* periods, int, MPI_Comm* out)
{
    for (int i = 0; i < ndims && i < 3; i++) mpistub_periods[i] = periods[i];
    *out = 1;
    return MPI_SUCCESS;
}

static inline int MPI_Cart_coords(MPI_Comm, int, int ndims, int* coords)
{
    for (int i = 0; i < ndims; i++) coords[i] = 0;
    return MPI_SUCCESS;
}

static inline int MPI_Cart_shift(MPI_Comm, int dir, int, int* src, int* dst)
{
    int self = mpistub_periods[dir] ? 0 : MPI_PROC_NULL;
    *src = self;
    *dst = self;
    return MPI_SUCCESS;
}

static inline int MPI_Type_create_subarray(int ndims, const int* sizes, const int* subsizes, const int* starts,
                                           int order, MPI_Datatype old, MPI_Datatype* out)
{
    if (order != MPI_ORDER_C || ndims < 1 || ndims > 3 || old->is_subarray) mpistub_fail("this subarray form");
    struct mpistub_type* t = (struct mpistub_type*)calloc(1, sizeof(struct mpistub_type));
    t->basic_size = old->basic_size;
    t->is_subarray = 1;
    t->ndims = ndims;
    for (int i = 0; i < ndims; i++) {
        t->sizes[i] = sizes[i];
        t->subsizes[i] = subsizes[i];
        t->starts[i] = starts[i];
    }
    *out = t;
    return MPI_SUCCESS;
}

static inline int MPI_Type_commit(MPI_Datatype*) { return MPI_SUCCESS; }

static inline int MPI_Type_free(MPI_Datatype* t)
{
    if (*t && (*t)->is_subarray) free(*t);
    *t = 0;
    return MPI_SUCCESS;
}

/* Bytes a (count, type) message carries. */
static inline size_t mpistub_msg_bytes(int count, MPI_Datatype t)
{
    if (!t->is_subarray) return (size_t)count * (size_t)t->basic_size;
    size_t n = (size_t)t->basic_size;
    for (int i = 0; i < t->ndims; i++) n *= (size_t)t->subsizes[i];
    return n * (size_t)count;
}

/* Walk a C-order subarray (last index fastest); pack==1 copies buf->msg. */
static inline void mpistub_walk(char* buf, char* msg, MPI_Datatype t, int pack)
{
    int sz[3] = {1, 1, 1}, sub[3] = {1, 1, 1}, st[3] = {0, 0, 0};
    int off = 3 - t->ndims;
    for (int i = 0; i < t->ndims; i++) {
        sz[off + i] = t->sizes[i];
        sub[off + i] = t->subsizes[i];
        st[off + i] = t->starts[i];
    }
    size_t es = (size_t)t->basic_size;
    size_t row = (size_t)sub[2] * es;
    for (int a = 0; a < sub[0]; a++)
        for (int b = 0; b < sub[1]; b++) {
            size_t idx = (((size_t)(st[0] + a) * sz[1] + (size_t)(st[1] + b)) * sz[2] + (size_t)st[2]) * es;
            if (pack) memcpy(msg, buf + idx, row);
            else memcpy(buf + idx, msg, row);
            msg += row;
        }
}

static inline int MPI_Sendrecv(const void* sbuf, int scount, MPI_Datatype stype, int dest, int,
                               void* rbuf, int rcount, MPI_Datatype rtype, int source, int,
                               MPI_Comm, MPI_Status*)
{
    if (dest == MPI_PROC_NULL || source == MPI_PROC_NULL) return MPI_SUCCESS;
    size_t sb = mpistub_msg_bytes(scount, stype), rb = mpistub_msg_bytes(rcount, rtype);
    if (sb != rb) mpistub_fail("Sendrecv with mismatched sizes");
    char* tmp = (char*)malloc(sb ? sb : 1);
    if (stype->is_subarray) mpistub_walk((char*)sbuf, tmp, stype, 1);
    else memcpy(tmp, sbuf, sb);
    if (rtype->is_subarray) mpistub_walk((char*)rbuf, tmp, rtype, 0);
    else memcpy(rbuf, tmp, rb);
    free(tmp);
    return MPI_SUCCESS;
}

static inline int MPI_Allreduce(const void* in, void* out, int count, MPI_Datatype t, MPI_Op, MPI_Comm)
{
    memcpy(out, in, mpistub_msg_bytes(count, t));
    return MPI_SUCCESS;
}

static inline int MPI_Isend(const void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*)
{
    mpistub_fail("Isend");
    return 1;
}
static inline int MPI_Irecv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*)
{
    mpistub_fail("Irecv");
    return 1;
}
static inline int MPI_Wait(MPI_Request*, MPI_Status*) { return MPI_SUCCESS; }

#ifdef __cplusplus
}
#endif

#endif
