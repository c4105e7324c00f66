// Single-rank MPI shim: see mpi.h for why it exists and why it is exact.
#include "mpi.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace {

struct Pending {
  bool is_send;
  const void* sbuf;
  void* rbuf;
  size_t bytes;
  int tag;
  bool done;
};

std::vector<Pending> g_pending;

size_t type_size(MPI_Datatype t) { return (size_t)t; }

}  // namespace

extern "C" {

int MPI_Init(int*, char***) { return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Abort(MPI_Comm, int code) {
  std::fprintf(stderr, "MPI_Abort(%d) from the oracle harness\n", code);
  std::exit(code == 0 ? 1 : code);
}
int MPI_Comm_size(MPI_Comm, int* size) { *size = 1; return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm, int* rank) { *rank = 0; return MPI_SUCCESS; }
int MPI_Comm_free(MPI_Comm*) { return MPI_SUCCESS; }
int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }
int MPI_Cart_create(MPI_Comm, int, const int*, const int*, int, MPI_Comm* cart) {
  *cart = MPI_COMM_WORLD;
  return MPI_SUCCESS;
}
int MPI_Cart_coords(MPI_Comm, int, int maxdims, int* coords) {
  for (int d = 0; d < maxdims; ++d) coords[d] = 0;
  return MPI_SUCCESS;
}
int MPI_Cart_shift(MPI_Comm, int, int, int* src, int* dst) {
  *src = 0;
  *dst = 0;
  return MPI_SUCCESS;
}

// A request is an index into g_pending; Waitall matches receives to sends by tag.
int MPI_Isend(const void* buf, int count, MPI_Datatype type, int, int tag, MPI_Comm,
              MPI_Request* req) {
  g_pending.push_back({true, buf, nullptr, (size_t)count * type_size(type), tag, false});
  *req = (MPI_Request)(g_pending.size() - 1);
  return MPI_SUCCESS;
}
int MPI_Irecv(void* buf, int count, MPI_Datatype type, int, int tag, MPI_Comm,
              MPI_Request* req) {
  g_pending.push_back({false, nullptr, buf, (size_t)count * type_size(type), tag, false});
  *req = (MPI_Request)(g_pending.size() - 1);
  return MPI_SUCCESS;
}
int MPI_Waitall(int n, MPI_Request* reqs, MPI_Status*) {
  for (int a = 0; a < n; ++a) {
    Pending& r = g_pending[reqs[a]];
    if (r.is_send || r.done) continue;
    bool matched = false;
    for (int b = 0; b < n && !matched; ++b) {
      Pending& s = g_pending[reqs[b]];
      if (!s.is_send || s.done || s.tag != r.tag) continue;
      if (s.bytes != r.bytes) {
        std::fprintf(stderr, "mpi shim: size mismatch on tag %d\n", r.tag);
        std::exit(2);
      }
      std::memcpy(r.rbuf, s.sbuf, r.bytes);
      s.done = r.done = matched = true;
    }
    if (!matched) {
      std::fprintf(stderr, "mpi shim: unmatched receive on tag %d\n", r.tag);
      std::exit(2);
    }
  }
  g_pending.clear();
  return MPI_SUCCESS;
}
int MPI_Allreduce(const void* in, void* out, int count, MPI_Datatype type, MPI_Op,
                  MPI_Comm) {
  std::memmove(out, in, (size_t)count * type_size(type));
  return MPI_SUCCESS;
}
int MPI_Reduce(const void* in, void* out, int count, MPI_Datatype type, MPI_Op, int,
               MPI_Comm) {
  std::memmove(out, in, (size_t)count * type_size(type));
  return MPI_SUCCESS;
}

}  // extern "C"
