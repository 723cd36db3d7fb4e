/* Single-rank MPI shim for the host-emulation build of the reference
 * (oracle/ref_host): one process, Cartesian coordinates all zero, reductions
 * are copies. Test infrastructure only. */
#pragma once
#include <cstdlib>
#include <cstring>
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Info;
#define MPI_COMM_WORLD 0
#define MPI_COMM_SELF 1
#define MPI_COMM_NULL (-1)
#define MPI_DOUBLE 8
#define MPI_INT 4
#define MPI_SUM 0
#define MPI_INFO_NULL 0
#define MPI_COMM_TYPE_SHARED 0
#define MPI_THREAD_MULTIPLE 3
#define MPI_IN_PLACE ((void*)1)
#define MPI_STATUSES_IGNORE ((void*)0)
#define MPI_SUCCESS 0
typedef int MPI_Request;
inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return 0; }
inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
inline int MPI_Cart_create(MPI_Comm, int, const int*, const int*, int, MPI_Comm* c) { *c = 2; return 0; }
inline int MPI_Cart_coords(MPI_Comm, int, int n, int* c) { for (int i = 0; i < n; ++i) c[i] = 0; return 0; }
inline int MPI_Cart_rank(MPI_Comm, const int*, int* r) { *r = 0; return 0; }
inline int MPI_Comm_dup(MPI_Comm c, MPI_Comm* d) { *d = c; return 0; }
inline int MPI_Comm_free(MPI_Comm*) { return 0; }
inline int MPI_Comm_split_type(MPI_Comm c, int, int, MPI_Info, MPI_Comm* d) { *d = c; return 0; }
inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  if (s != MPI_IN_PLACE) std::memmove(r, s, (std::size_t)n * (std::size_t)t);
  return 0;
}
inline int MPI_Iallreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op o, MPI_Comm c, MPI_Request* q) {
  *q = 0;
  return MPI_Allreduce(s, r, n, t, o, c);
}
inline int MPI_Waitall(int, MPI_Request*, void*) { return 0; }
inline int MPI_Abort(MPI_Comm, int e) { std::exit(e); }
inline double MPI_Wtime() { return 0.0; }
inline int MPI_Init(int*, char***) { return 0; }
inline int MPI_Finalize() { return 0; }
