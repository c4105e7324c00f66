/*
 * Single-rank MPI shim (project-written test infrastructure, not product code).
 *
 * The reference solver (chenbei102/cbns3d_cart_mpi) needs an MPI library only for
 * its halo exchange (src/boundary_condition.cpp:52-62, 122-132, 192-202), the dt
 * MIN all-reduce (src/cbns3d.cpp:189) and its start-up/teardown calls
 * (src/cbns3d.cpp:29-35, 80-97, 280-304).  This image has no MPI, so the oracle
 * recipe compiles the reference's own sources against this header instead.  With
 * one rank on a fully periodic Cartesian communicator every neighbour is the rank
 * itself, so a point-to-point message is a memcpy matched by tag, and every
 * reduction is the identity.  Halo copies are exact, so the single-rank run is
 * bitwise what an N-rank run of the reference produces.
 */
#ifndef CBNS_ORACLE_MPI_SHIM_H
#define CBNS_ORACLE_MPI_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD ((MPI_Comm)0)
#define MPI_BYTE ((MPI_Datatype)1)
#define MPI_DOUBLE ((MPI_Datatype)8)
#define MPI_INT ((MPI_Datatype)4)
#define MPI_MIN ((MPI_Op)1)
#define MPI_MAX ((MPI_Op)2)
#define MPI_SUM ((MPI_Op)3)
#define MPI_SUCCESS 0
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)

int MPI_Init(int* argc, char*** argv);
int MPI_Finalize(void);
int MPI_Abort(MPI_Comm comm, int code);
int MPI_Comm_size(MPI_Comm comm, int* size);
int MPI_Comm_rank(MPI_Comm comm, int* rank);
int MPI_Comm_free(MPI_Comm* comm);
int MPI_Bcast(void* buf, int count, MPI_Datatype type, int root, MPI_Comm comm);
int MPI_Cart_create(MPI_Comm old, int ndims, const int* dims, const int* periods,
                    int reorder, MPI_Comm* cart);
int MPI_Cart_coords(MPI_Comm comm, int rank, int maxdims, int* coords);
int MPI_Cart_shift(MPI_Comm comm, int dir, int disp, int* src, int* dst);
int MPI_Isend(const void* buf, int count, MPI_Datatype type, int dest, int tag,
              MPI_Comm comm, MPI_Request* req);
int MPI_Irecv(void* buf, int count, MPI_Datatype type, int src, int tag,
              MPI_Comm comm, MPI_Request* req);
int MPI_Waitall(int n, MPI_Request* reqs, MPI_Status* stats);
int MPI_Allreduce(const void* in, void* out, int count, MPI_Datatype type,
                  MPI_Op op, MPI_Comm comm);
int MPI_Reduce(const void* in, void* out, int count, MPI_Datatype type,
               MPI_Op op, int root, MPI_Comm comm);

#ifdef __cplusplus
}
#endif

#endif
