/*
 * TEST INFRASTRUCTURE ONLY: a single-rank stand-in for the MPI API subset the
 * CudaNavierStokes host code calls (src/comm.cpp, src/main.cpp). It lets the
 * reference build without an MPI installation when it runs on one GPU
 * (pRow = pCol = 1): collectives copy the send buffer, the Cartesian topology has
 * one rank, and MPI-IO writes the local array to a plain file (the single-rank
 * subarray view covers the whole global array). It is staged as `mpi.h` next to the
 * reference sources by oracle/ref_harness.py.
 */
#ifndef CNS_REF_MPI_STUB_H_
#define CNS_REF_MPI_STUB_H_

#include <stdio.h>
#include <string.h>
#include <time.h>

typedef int MPI_Comm;
typedef int MPI_Info;
typedef long long MPI_Offset;
typedef struct { int count; } MPI_Status;
struct cns_stub_type { long long elems; int is_double; };
typedef struct cns_stub_type* MPI_Datatype;
typedef FILE* MPI_File;
typedef int MPI_Op;

static struct cns_stub_type cns_stub_double_type = {1, 1};
static struct cns_stub_type cns_stub_types[64];
static int cns_stub_ntypes = 0;

#define MPI_COMM_WORLD 0
#define MPI_DOUBLE (&cns_stub_double_type)
#define MPI_SUCCESS 0
#define MPI_MAX_ERROR_STRING 64
#define MPI_MAX_PROCESSOR_NAME 64
#define MPI_ORDER_C 0
#define MPI_MODE_CREATE 1
#define MPI_MODE_WRONLY 2
#define MPI_INFO_NULL 0
#define MPI_SUM 0
#define MPI_MIN 1

static inline int MPI_Init(int*, char***) { return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline double MPI_Wtime(void) {
    struct timespec ts; clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}
static inline int MPI_Error_string(int, char* s, int* len) { s[0] = 0; *len = 0; return 0; }
static inline int MPI_Get_processor_name(char* s, int* len) { strcpy(s, "stub"); *len = 4; return 0; }
static inline int MPI_Comm_split(MPI_Comm, int, int, MPI_Comm* n) { *n = 0; return 0; }
static inline int MPI_Cart_create(MPI_Comm, int, const int*, const int*, int, MPI_Comm* c) { *c = 0; return 0; }
static inline int MPI_Cart_coords(MPI_Comm, int, int nd, int* coords) {
    for (int i = 0; i < nd; i++) coords[i] = 0;
    return 0;
}
static inline int MPI_Cart_rank(MPI_Comm, const int*, int* r) { *r = 0; return 0; }
static inline long long cns_stub_elems(MPI_Datatype t) { return t->elems; }
static inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
    memmove(r, s, (size_t)n * cns_stub_elems(t) * sizeof(double)); return 0;
}
static inline int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
    memmove(r, s, (size_t)n * cns_stub_elems(t) * sizeof(double)); return 0;
}
static inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return 0; }
static inline int MPI_Sendrecv(const void* s, int n, MPI_Datatype t, int, int, void* r, int, MPI_Datatype, int, int,
                               MPI_Comm, MPI_Status*) {
    memmove(r, s, (size_t)n * cns_stub_elems(t) * sizeof(double)); return 0;
}
static inline int MPI_Type_create_subarray(int nd, const int*, const int* sub, const int*, int, MPI_Datatype,
                                           MPI_Datatype* out) {
    long long e = 1;
    for (int i = 0; i < nd; i++) e *= sub[i];
    int slot = cns_stub_ntypes++ % 64;
    cns_stub_types[slot].elems = e;
    cns_stub_types[slot].is_double = 1;
    *out = &cns_stub_types[slot];
    return 0;
}
static inline int MPI_Type_commit(MPI_Datatype*) { return 0; }
static inline int MPI_File_open(MPI_Comm, const char* name, int, MPI_Info, MPI_File* fh) {
    *fh = fopen(name, "wb"); return *fh ? 0 : 1;
}
static inline int MPI_File_set_view(MPI_File, MPI_Offset, MPI_Datatype, MPI_Datatype, const char*, MPI_Info) { return 0; }
static inline int MPI_File_write_all(MPI_File fh, const void* buf, int n, MPI_Datatype t, MPI_Status*) {
    size_t cnt = (size_t)n * cns_stub_elems(t);
    return fwrite(buf, sizeof(double), cnt, fh) == cnt ? 0 : 1;
}
static inline int MPI_File_close(MPI_File* fh) { fclose(*fh); return 0; }

#endif
