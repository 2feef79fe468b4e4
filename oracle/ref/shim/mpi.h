/* Single-rank stand-in for the MPI library, written for this project so that the
 * reference's unmodified headers compile and run as one process (rank 0 of 1).
 * Collectives become copies (MPI_IN_PLACE: no-ops), communicator splits are the
 * identity, MPI-IO maps to stdio.  Point-to-point, RMA and inter-communicator calls
 * are only reached with more than one rank or region; they abort if called.
 * Test infrastructure for the oracle harness only. */
#pragma once
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <complex>

typedef int MPI_Comm;
typedef int MPI_Group;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Info;
typedef int MPI_Win;
typedef long long MPI_Offset;
typedef long long MPI_Aint;
typedef FILE* MPI_File;
struct MPI_Status { int MPI_SOURCE, MPI_TAG, MPI_ERROR; };

#define MPI_COMM_WORLD 0
#define MPI_INFO_NULL 0
#define MPI_SUM 1
#define MPI_IN_PLACE ((void*)1)
#define MPI_BOTTOM ((void*)0)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_MAX_PROCESSOR_NAME 64
#define MPI_MAX_LIBRARY_VERSION_STRING 64
#define MPI_MODE_RDONLY 1
#define MPI_MODE_WRONLY 2
#define MPI_MODE_CREATE 4
#define MPI_MODE_NOSUCCEED 8
#define MPI_MODE_NOPRECEDE 16
#define MPI_MODE_NOSTORE 32
#define MPI_MODE_NOPUT 64
#define MPI_SEEK_SET SEEK_SET

enum : int {
  MPI_INT = 4, MPI_DOUBLE = 8, MPI_CXX_DOUBLE_COMPLEX = 16, MPI_CXX_BOOL = 1, MPI_UNSIGNED_CHAR = 1,
  MPI_OFFSET = 8, MPI_BYTE = 1, MPI_INT64_T = 8
};

static inline size_t qsf_shim_type_size(MPI_Datatype t) { return (size_t)t; }
[[noreturn]] static inline void qsf_shim_unreachable(const char* what) {
  fprintf(stderr, "single-rank MPI stand-in: %s is not available\n", what);
  abort();
}

static inline int MPI_Init(int*, char***) { return 0; }
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return 0; }
static inline int MPI_Comm_group(MPI_Comm, MPI_Group* g) { *g = 0; return 0; }
static inline int MPI_Comm_split(MPI_Comm c, int, int, MPI_Comm* o) { *o = c; return 0; }
static inline int MPI_Comm_remote_size(MPI_Comm, int* s) { *s = 1; return 0; }
static inline int MPI_Intercomm_create(MPI_Comm, int, MPI_Comm, int, int, MPI_Comm*) {
  qsf_shim_unreachable("MPI_Intercomm_create");
}
static inline int MPI_Intercomm_merge(MPI_Comm, int, MPI_Comm*) { qsf_shim_unreachable("MPI_Intercomm_merge"); }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Get_processor_name(char* n, int* l) { strcpy(n, "oracle"); *l = 6; return 0; }
static inline int MPI_Get_version(int* v, int* s) { *v = 3; *s = 1; return 0; }
static inline int MPI_Get_library_version(char* v, int* l) { strcpy(v, "single-rank stand-in"); *l = 20; return 0; }

static inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  if (s != MPI_IN_PLACE) memcpy(r, s, (size_t)n * qsf_shim_type_size(t));
  return 0;
}
static inline int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
  if (s != MPI_IN_PLACE && s != r) memcpy(r, s, (size_t)n * qsf_shim_type_size(t));
  return 0;
}
static inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return 0; }
static inline int MPI_Gather(const void* s, int n, MPI_Datatype t, void* r, int, MPI_Datatype, int, MPI_Comm) {
  if (s != MPI_IN_PLACE && s != r) memcpy(r, s, (size_t)n * qsf_shim_type_size(t));
  return 0;
}
static inline int MPI_Allgather(const void* s, int n, MPI_Datatype t, void* r, int, MPI_Datatype, MPI_Comm) {
  if (s != MPI_IN_PLACE && s != r) memcpy(r, s, (size_t)n * qsf_shim_type_size(t));
  return 0;
}
static inline int MPI_Scatter(const void* s, int n, MPI_Datatype t, void* r, int, MPI_Datatype, int, MPI_Comm) {
  if (s != r) memcpy(r, s, (size_t)n * qsf_shim_type_size(t));
  return 0;
}
static inline int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm) { qsf_shim_unreachable("MPI_Send"); }
static inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) { qsf_shim_unreachable("MPI_Recv"); }

static inline int MPI_Type_contiguous(int, MPI_Datatype, MPI_Datatype*) { qsf_shim_unreachable("MPI_Type_contiguous"); }
static inline int MPI_Type_create_struct(int, const int*, const MPI_Aint*, const MPI_Datatype*, MPI_Datatype*) {
  qsf_shim_unreachable("MPI_Type_create_struct");
}
static inline int MPI_Type_commit(MPI_Datatype*) { return 0; }

static inline int MPI_Win_create(void*, MPI_Aint, int, MPI_Info, MPI_Comm, MPI_Win* w) { *w = 0; return 0; }
static inline int MPI_Win_fence(int, MPI_Win) { return 0; }
static inline int MPI_Win_free(MPI_Win*) { return 0; }
static inline int MPI_Get(void*, int, MPI_Datatype, int, MPI_Aint, int, MPI_Datatype, MPI_Win) {
  qsf_shim_unreachable("MPI_Get");
}

static inline int MPI_File_open(MPI_Comm, const char* name, int mode, MPI_Info, MPI_File* fh) {
  *fh = fopen(name, (mode & MPI_MODE_RDONLY) ? "rb" : "wb");
  return *fh ? 0 : 1;
}
static inline int MPI_File_close(MPI_File* fh) { if (*fh) fclose(*fh); *fh = nullptr; return 0; }
static inline int MPI_File_delete(const char* name, MPI_Info) { remove(name); return 0; }
static inline int MPI_File_read(MPI_File fh, void* b, int n, MPI_Datatype t, MPI_Status*) {
  return fread(b, qsf_shim_type_size(t), (size_t)n, fh) == (size_t)n ? 0 : 1;
}
static inline int MPI_File_read_all(MPI_File fh, void* b, int n, MPI_Datatype t, MPI_Status* s) {
  return MPI_File_read(fh, b, n, t, s);
}
static inline int MPI_File_write(MPI_File fh, const void* b, int n, MPI_Datatype t, MPI_Status*) {
  return fwrite(b, qsf_shim_type_size(t), (size_t)n, fh) == (size_t)n ? 0 : 1;
}
static inline int MPI_File_seek(MPI_File fh, MPI_Offset o, int w) { return fseek(fh, (long)o, w); }
static inline int MPI_File_get_position(MPI_File fh, MPI_Offset* o) { *o = ftell(fh); return 0; }
static inline int MPI_File_set_view(MPI_File fh, MPI_Offset disp, MPI_Datatype, MPI_Datatype, const char*, MPI_Info) {
  return fseek(fh, (long)disp, SEEK_SET);
}
