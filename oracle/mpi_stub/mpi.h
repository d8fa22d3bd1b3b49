/*
 * Single-rank MPI stand-in used only to compile the reference's CPU path
 * (parallel/compute_pool.h and core/parallel.h include <mpi.h>
 * unconditionally).  Written for this oracle; it implements exactly the
 * calls those headers make, for one rank in one process:
 *   - collectives copy send -> receive buffers (world size 1),
 *   - point-to-point calls are never reached with one rank and fail loudly,
 *   - MPI-IO is unsupported (the reference's binary checkpoint path is not
 *     exercised by the oracle).
 * Test infrastructure only: never linked into the product library.
 */
#pragma once
#include <string.h>
#include <stdio.h>
#include <stdlib.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef int MPI_Info;
typedef int MPI_File;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_SUCCESS 0
#define MPI_COMM_WORLD 0
#define MPI_INFO_NULL 0
#define MPI_THREAD_FUNNELED 1
#define MPI_MODE_RDWR 1
#define MPI_MODE_CREATE 2

#define MPI_DOUBLE   1
#define MPI_CHAR     2
#define MPI_FLOAT    3
#define MPI_INT      4
#define MPI_UINT64_T 5
#define MPI_UINT     6

#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3

static inline size_t mpistub_type_size(MPI_Datatype t)
{
    switch (t)
    {
        case MPI_DOUBLE:   return 8;
        case MPI_CHAR:     return 1;
        case MPI_FLOAT:    return 4;
        case MPI_INT:      return 4;
        case MPI_UINT64_T: return 8;
        case MPI_UINT:     return 4;
    }
    return 0;
}

static inline int mpistub_unreachable(const char* what)
{
    fprintf(stderr, "mpi stub: %s is not available with a single rank\n", what);
    abort();
    return 1;
}

static inline int MPI_Init(int*, char***) { return MPI_SUCCESS; }
static inline int MPI_Init_thread(int*, char***, int required, int* provided) { *provided = required; return MPI_SUCCESS; }
static inline int MPI_Finalize(void) { return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return MPI_SUCCESS; }
static inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Error_string(int, char* s, int* len) { static char m[] = "mpi stub error"; (void)s; *len = (int)sizeof(m) - 1; return MPI_SUCCESS; }

static inline int MPI_Allgather(const void* sb, int sc, MPI_Datatype st, void* rb, int, MPI_Datatype, MPI_Comm)
{
    if (sb != rb) memmove(rb, sb, (size_t)sc * mpistub_type_size(st));
    return MPI_SUCCESS;
}
static inline int MPI_Allreduce(const void* sb, void* rb, int c, MPI_Datatype t, MPI_Op, MPI_Comm)
{
    if (sb != rb) memmove(rb, sb, (size_t)c * mpistub_type_size(t));
    return MPI_SUCCESS;
}
static inline int MPI_Gather(const void* sb, int sc, MPI_Datatype st, void* rb, int, MPI_Datatype, int, MPI_Comm)
{
    if (sb != rb) memmove(rb, sb, (size_t)sc * mpistub_type_size(st));
    return MPI_SUCCESS;
}
static inline int MPI_Gatherv(const void* sb, int sc, MPI_Datatype st, void* rb, const int*, const int* displ, MPI_Datatype, int, MPI_Comm)
{
    memmove((char*)rb + (size_t)displ[0] * mpistub_type_size(st), sb, (size_t)sc * mpistub_type_size(st));
    return MPI_SUCCESS;
}
static inline int MPI_Irecv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*) { return mpistub_unreachable("MPI_Irecv"); }
static inline int MPI_Ssend(const void*, int, MPI_Datatype, int, int, MPI_Comm) { return mpistub_unreachable("MPI_Ssend"); }
static inline int MPI_Waitall(int, MPI_Request*, MPI_Status*) { return MPI_SUCCESS; }
static inline int MPI_File_open(MPI_Comm, const char*, int, MPI_Info, MPI_File*) { return mpistub_unreachable("MPI_File_open"); }
static inline int MPI_File_write_at(MPI_File, long long, const void*, int, MPI_Datatype, MPI_Status*) { return mpistub_unreachable("MPI_File_write_at"); }
static inline int MPI_File_read_at(MPI_File, long long, void*, int, MPI_Datatype, MPI_Status*) { return mpistub_unreachable("MPI_File_read_at"); }
static inline int MPI_File_close(MPI_File*) { return MPI_SUCCESS; }
