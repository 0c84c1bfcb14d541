/*
 * Single-rank MPI stand-in used only to compile the unmodified reference
 * sources (Local-DG: MPIUtil.cpp, mesh.cpp, solver.cpp, io.cpp) into the
 * CPU oracle binary oracle/_ref/ldg_ref.  Test infrastructure, not product.
 *
 * Semantics on one rank, matching what a real MPI library does there:
 *  - MPI_Dims_create fills 1s, MPI_Cart_shift on a periodic grid returns
 *    this rank for both neighbours (MPIUtil.cpp:23-28).
 *  - MPI_Isend records (buffer, bytes, tag); MPI_Irecv records its target;
 *    MPI_Waitall copies every receive from the pending send with the same
 *    tag.  The reference posts face iF's send with tag iF and face iF's
 *    receive with tag iF^1 (MPIUtil.cpp:31-34, solver.cpp:951-961), so the
 *    copy realises the periodic self-exchange.
 *  - MPI_Allreduce on one rank is a copy.
 */
#ifndef LDG_REF_SHIM_MPI_H
#define LDG_REF_SHIM_MPI_H

#include <cstring>
#include <cstdlib>
#include <cstdio>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int unused; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_SUM 1
#define MPI_LAND 2
/* Datatype handles index a table of byte sizes. */
#define MPI_DOUBLE 1
#define MPI_INT 2

namespace ldg_mpi_shim {
struct Pending {
  void* buf;
  long bytes;
  int tag;
  int is_send;
  int live;
};
static const int kMaxTypes = 64;
static const int kMaxReq = 256;
inline long* type_bytes() {
  static long t[kMaxTypes] = {0, (long)sizeof(double), (long)sizeof(int)};
  return t;
}
inline int& n_types() { static int n = 3; return n; }
inline Pending* pending() { static Pending p[kMaxReq]; return p; }
inline int& n_pending() { static int n = 0; return n; }
inline int record(void* buf, int count, MPI_Datatype dt, int tag, int is_send) {
  int i = n_pending()++;
  if (i >= kMaxReq) { std::fprintf(stderr, "mpi shim: too many requests\n"); std::exit(3); }
  Pending& p = pending()[i];
  p.buf = buf; p.bytes = (long)count * type_bytes()[dt]; p.tag = tag;
  p.is_send = is_send; p.live = 1;
  return i;
}
}  // namespace ldg_mpi_shim

static inline int MPI_Init(int*, char***) { return 0; }
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Comm_size(MPI_Comm, int* n) { *n = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
static inline int MPI_Dims_create(int, int ndims, int* dims) {
  for (int i = 0; i < ndims; ++i) dims[i] = 1;
  return 0;
}
static inline int MPI_Cart_create(MPI_Comm, int, const int*, const int*, int, MPI_Comm* c) {
  *c = 0; return 0;
}
static inline int MPI_Cart_coords(MPI_Comm, int, int ndims, int* coords) {
  for (int i = 0; i < ndims; ++i) coords[i] = 0;
  return 0;
}
static inline int MPI_Cart_shift(MPI_Comm, int, int, int* src, int* dst) {
  *src = 0; *dst = 0; return 0;
}
static inline int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype* nt) {
  int i = ldg_mpi_shim::n_types()++;
  ldg_mpi_shim::type_bytes()[i] = count * ldg_mpi_shim::type_bytes()[old];
  *nt = i;
  return 0;
}
static inline int MPI_Type_commit(MPI_Datatype*) { return 0; }
static inline int MPI_Isend(const void* buf, int count, MPI_Datatype dt, int, int tag,
                            MPI_Comm, MPI_Request* req) {
  *req = ldg_mpi_shim::record(const_cast<void*>(buf), count, dt, tag, 1);
  return 0;
}
static inline int MPI_Irecv(void* buf, int count, MPI_Datatype dt, int, int tag,
                            MPI_Comm, MPI_Request* req) {
  *req = ldg_mpi_shim::record(buf, count, dt, tag, 0);
  return 0;
}
static inline int MPI_Waitall(int n, MPI_Request* reqs, MPI_Status*) {
  using namespace ldg_mpi_shim;
  for (int i = 0; i < n; ++i) {
    Pending& r = pending()[reqs[i]];
    if (!r.live || r.is_send) continue;
    int found = 0;
    for (int j = 0; j < n_pending(); ++j) {
      Pending& s = pending()[j];
      if (s.live && s.is_send && s.tag == r.tag) {
        if (s.bytes != r.bytes) { std::fprintf(stderr, "mpi shim: size mismatch\n"); std::exit(3); }
        std::memmove(r.buf, s.buf, (size_t)r.bytes);
        found = 1;
        break;
      }
    }
    if (!found) { std::fprintf(stderr, "mpi shim: unmatched receive tag %d\n", r.tag); std::exit(3); }
  }
  for (int i = 0; i < n_pending(); ++i) pending()[i].live = 0;
  n_pending() = 0;
  return 0;
}
static inline int MPI_Allreduce(const void* in, void* out, int count, MPI_Datatype dt, MPI_Op,
                                MPI_Comm) {
  std::memcpy(out, in, (size_t)count * ldg_mpi_shim::type_bytes()[dt]);
  return 0;
}
static inline int MPI_Barrier(MPI_Comm) { return 0; }

#endif
