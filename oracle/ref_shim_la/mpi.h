// One-rank stand-in for <mpi.h>, used only to compile the reference's own
// la/SparsityPattern.cpp and common/IndexMap.cpp (and what they include)
// into oracle/_ref/ as a checker. Test infrastructure: nothing in the
// product links it.
//
// Every communicator has one rank. Collectives copy the send buffer to the
// receive buffer; non-blocking collectives complete at once; neighbourhood
// collectives move each outgoing block to the matching incoming block of
// the (self-only) graph. Point-to-point messages cannot happen on one rank
// and abort.
#pragma once
#include <cstdio>
#include <cstdlib>
#include <cstring>

typedef int MPI_Comm;
typedef long MPI_Datatype; // the size of one element in bytes
typedef int MPI_Op;
typedef int MPI_Info;
typedef int MPI_Request;
struct MPI_Status
{
  int MPI_SOURCE, MPI_TAG, MPI_ERROR;
};

#define MPI_SUCCESS 0
#define MPI_COMM_NULL 0
#define MPI_COMM_WORLD 1
#define MPI_COMM_SELF 2
#define MPI_INFO_NULL 0
#define MPI_REQUEST_NULL 0
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
#define MPI_UNDEFINED (-32766)
#define MPI_MAX_ERROR_STRING 64
#define MPI_COMM_TYPE_SHARED 1
#define MPI_STATUS_IGNORE ((MPI_Status*)nullptr)
#define MPI_STATUSES_IGNORE ((MPI_Status*)nullptr)
#define MPI_UNWEIGHTED ((int*)nullptr)
#define MPI_WEIGHTS_EMPTY ((int*)nullptr)
#define MPI_IN_PLACE ((void*)1)

#define MPI_BYTE ((MPI_Datatype)1)
#define MPI_CHAR ((MPI_Datatype)1)
#define MPI_INT8_T ((MPI_Datatype)1)
#define MPI_UINT8_T ((MPI_Datatype)1)
#define MPI_INT16_T ((MPI_Datatype)2)
#define MPI_UINT16_T ((MPI_Datatype)2)
#define MPI_INT ((MPI_Datatype)4)
#define MPI_UINT ((MPI_Datatype)4)
#define MPI_INT32_T ((MPI_Datatype)4)
#define MPI_UINT32_T ((MPI_Datatype)4)
#define MPI_FLOAT ((MPI_Datatype)4)
#define MPI_INT64_T ((MPI_Datatype)8)
#define MPI_UINT64_T ((MPI_Datatype)8)
#define MPI_DOUBLE ((MPI_Datatype)8)
#define MPI_C_FLOAT_COMPLEX ((MPI_Datatype)8)
#define MPI_C_DOUBLE_COMPLEX ((MPI_Datatype)16)
#define MPI_CXX_BOOL ((MPI_Datatype)1)

#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3
#define MPI_AVG 4
#define MPI_LOR 5
#define MPI_LAND 6
#define MPI_BOR 7

namespace dfx_mpi_shim
{
inline void copy(const void* s, void* r, int count, MPI_Datatype t)
{
  if (s != MPI_IN_PLACE && s != r && count > 0)
    std::memcpy(r, s, (size_t)count * (size_t)t);
}
[[noreturn]] inline void unsupported(const char* what)
{
  std::fprintf(stderr, "one-rank MPI stand-in: %s cannot happen on one rank\n", what);
  std::abort();
}
} // namespace dfx_mpi_shim

inline int MPI_Comm_size(MPI_Comm, int* n) { *n = 1; return 0; }
inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
inline int MPI_Comm_dup(MPI_Comm c, MPI_Comm* n) { *n = c; return 0; }
inline int MPI_Comm_free(MPI_Comm* c) { *c = MPI_COMM_NULL; return 0; }
inline int MPI_Comm_split_type(MPI_Comm c, int, int, MPI_Info, MPI_Comm* n) { *n = c; return 0; }
inline int MPI_Abort(MPI_Comm, int e) { std::exit(e); }
inline int MPI_Error_string(int, char* s, int* len)
{
  std::snprintf(s, MPI_MAX_ERROR_STRING, "one-rank MPI stand-in");
  *len = (int)std::strlen(s);
  return 0;
}
inline int MPI_Type_contiguous(int count, MPI_Datatype t, MPI_Datatype* n)
{
  *n = count * t;
  return 0;
}
inline int MPI_Type_commit(MPI_Datatype*) { return 0; }
inline int MPI_Type_free(MPI_Datatype*) { return 0; }

inline int MPI_Barrier(MPI_Comm) { return 0; }
inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm)
{
  dfx_mpi_shim::copy(s, r, n, t);
  return 0;
}
inline int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm)
{
  dfx_mpi_shim::copy(s, r, n, t);
  return 0;
}
inline int MPI_Exscan(const void*, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm)
{
  std::memset(r, 0, (size_t)n * (size_t)t); // rank 0: nothing before it
  return 0;
}
inline int MPI_Allgather(const void* s, int n, MPI_Datatype t, void* r, int, MPI_Datatype, MPI_Comm)
{
  dfx_mpi_shim::copy(s, r, n, t);
  return 0;
}
inline int MPI_Gather(const void* s, int n, MPI_Datatype t, void* r, int, MPI_Datatype, int, MPI_Comm)
{
  dfx_mpi_shim::copy(s, r, n, t);
  return 0;
}
inline int MPI_Gatherv(const void* s, int n, MPI_Datatype t, void* r, const int*, const int* displs,
                       MPI_Datatype rt, int, MPI_Comm)
{
  dfx_mpi_shim::copy(s, (char*)r + (size_t)displs[0] * (size_t)rt, n, t);
  return 0;
}
inline int MPI_Alltoall(const void* s, int n, MPI_Datatype t, void* r, int, MPI_Datatype, MPI_Comm)
{
  dfx_mpi_shim::copy(s, r, n, t);
  return 0;
}
inline int MPI_Iallreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm,
                          MPI_Request* q)
{
  dfx_mpi_shim::copy(s, r, n, t);
  *q = MPI_REQUEST_NULL;
  return 0;
}
inline int MPI_Iexscan(const void*, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm,
                       MPI_Request* q)
{
  std::memset(r, 0, (size_t)n * (size_t)t);
  *q = MPI_REQUEST_NULL;
  return 0;
}
inline int MPI_Ibarrier(MPI_Comm, MPI_Request* q) { *q = MPI_REQUEST_NULL; return 0; }
inline int MPI_Ireduce_scatter_block(const void* s, void* r, int n, MPI_Datatype t, MPI_Op,
                                     MPI_Comm, MPI_Request* q)
{
  dfx_mpi_shim::copy(s, r, n, t);
  *q = MPI_REQUEST_NULL;
  return 0;
}

// Graph communicators: one rank, so every neighbour is rank 0 itself.
inline int MPI_Dist_graph_create_adjacent(MPI_Comm c, int indeg, const int*, const int*,
                                          int outdeg, const int*, const int*, MPI_Info, int,
                                          MPI_Comm* n)
{
  if (indeg != outdeg)
    dfx_mpi_shim::unsupported("a graph with different in- and out-degree");
  *n = c + 16 * (indeg + 1); // degree recorded in the handle
  return 0;
}
inline int dfx_mpi_degree(MPI_Comm c) { return c >= 16 ? c / 16 - 1 : 0; }
inline int MPI_Neighbor_alltoall(const void* s, int n, MPI_Datatype t, void* r, int,
                                 MPI_Datatype, MPI_Comm c)
{
  dfx_mpi_shim::copy(s, r, n * dfx_mpi_degree(c), t);
  return 0;
}
inline int MPI_Ineighbor_alltoall(const void* s, int n, MPI_Datatype t, void* r, int rn,
                                  MPI_Datatype rt, MPI_Comm c, MPI_Request* q)
{
  *q = MPI_REQUEST_NULL;
  return MPI_Neighbor_alltoall(s, n, t, r, rn, rt, c);
}
inline int MPI_Neighbor_alltoallv(const void* s, const int* sc, const int* sd, MPI_Datatype t,
                                  void* r, const int* rc, const int* rd, MPI_Datatype rt,
                                  MPI_Comm c)
{
  for (int i = 0; i < dfx_mpi_degree(c); ++i)
  {
    if (sc[i] != rc[i])
      dfx_mpi_shim::unsupported("a neighbour exchange with unequal counts");
    dfx_mpi_shim::copy((const char*)s + (size_t)sd[i] * (size_t)t,
                       (char*)r + (size_t)rd[i] * (size_t)rt, sc[i], t);
  }
  return 0;
}
inline int MPI_Ineighbor_alltoallv(const void* s, const int* sc, const int* sd, MPI_Datatype t,
                                   void* r, const int* rc, const int* rd, MPI_Datatype rt,
                                   MPI_Comm c, MPI_Request* q)
{
  *q = MPI_REQUEST_NULL;
  return MPI_Neighbor_alltoallv(s, sc, sd, t, r, rc, rd, rt, c);
}

inline int MPI_Wait(MPI_Request* q, MPI_Status*) { *q = MPI_REQUEST_NULL; return 0; }
inline int MPI_Waitall(int n, MPI_Request* q, MPI_Status*)
{
  for (int i = 0; i < n; ++i)
    q[i] = MPI_REQUEST_NULL;
  return 0;
}
inline int MPI_Test(MPI_Request* q, int* f, MPI_Status*) { *q = MPI_REQUEST_NULL; *f = 1; return 0; }
inline int MPI_Testall(int n, MPI_Request* q, int* f, MPI_Status* s)
{
  *f = 1;
  return MPI_Waitall(n, q, s);
}
inline int MPI_Test_cancelled(const MPI_Status*, int* f) { *f = 0; return 0; }
inline int MPI_Cancel(MPI_Request*) { return 0; }
inline int MPI_Isend(const void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*)
{
  dfx_mpi_shim::unsupported("MPI_Isend");
}
inline int MPI_Issend(const void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*)
{
  dfx_mpi_shim::unsupported("MPI_Issend");
}
inline int MPI_Irecv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*)
{
  dfx_mpi_shim::unsupported("MPI_Irecv");
}
inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*)
{
  dfx_mpi_shim::unsupported("MPI_Recv");
}
