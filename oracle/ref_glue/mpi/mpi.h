/* Stand-in for the MPI header (test oracle only): the types, constants and calls the reference's
 * server and block sources name, for one process that never sends a message. The grid harness
 * (oracle/ref_glue/grid_harness.cc) drives only BlockBase::GetZoneOffset and the Cartesian
 * server's stencil construction, neither of which communicates; every call that would move data
 * reports failure (MPI_ERR_OTHER) so that an unexpected use shows, unless the harness answers it (the reader's
 * interpolation of SERVER_INTERP_ORDER -1, which the front end asks of the boss). */
#ifndef SPX_MPI_STANDIN_H
#define SPX_MPI_STANDIN_H

#include <cstddef>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Request;
typedef int MPI_Info;
typedef int MPI_Op;
typedef std::ptrdiff_t MPI_Aint;
struct MPI_Status {
   int MPI_SOURCE, MPI_TAG, MPI_ERROR;
};

#define MPI_SUCCESS 0
#define MPI_ERR_OTHER 15
#define MPI_COMM_NULL 0
#define MPI_COMM_WORLD 1
#define MPI_REQUEST_NULL 0
#define MPI_INFO_NULL 0
#define MPI_DATATYPE_NULL 0
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_BYTE 3
#define MPI_SUM 1
#define MPI_UNDEFINED (-32766)
#define MPI_ANY_TAG (-1)
#define MPI_ANY_SOURCE (-2)
#define MPI_COMM_TYPE_SHARED 1
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)

inline int MPI_Init(int*, char***) { return MPI_SUCCESS; }
inline int MPI_Finalize(void) { return MPI_SUCCESS; }
inline int MPI_Comm_size(MPI_Comm, int* size) { *size = 1; return MPI_SUCCESS; }
inline int MPI_Comm_rank(MPI_Comm, int* rank) { *rank = 0; return MPI_SUCCESS; }
inline int MPI_Comm_dup(MPI_Comm c, MPI_Comm* out) { *out = c; return MPI_SUCCESS; }
inline int MPI_Comm_free(MPI_Comm* c) { *c = MPI_COMM_NULL; return MPI_SUCCESS; }
inline int MPI_Comm_split(MPI_Comm c, int, int, MPI_Comm* out) { *out = c; return MPI_SUCCESS; }
inline int MPI_Comm_split_type(MPI_Comm c, int, int, MPI_Info, MPI_Comm* out) { *out = c; return MPI_SUCCESS; }
inline int MPI_Get_address(const void* p, MPI_Aint* a) { *a = (MPI_Aint)p; return MPI_SUCCESS; }
inline int MPI_Type_create_struct(int, const int*, const MPI_Aint*, const MPI_Datatype*, MPI_Datatype* t) { *t = MPI_BYTE; return MPI_SUCCESS; }
inline int MPI_Type_commit(MPI_Datatype*) { return MPI_SUCCESS; }
inline int MPI_Type_free(MPI_Datatype* t) { *t = MPI_DATATYPE_NULL; return MPI_SUCCESS; }
inline int MPI_Request_free(MPI_Request* r) { *r = MPI_REQUEST_NULL; return MPI_SUCCESS; }
inline int MPI_Cancel(MPI_Request*) { return MPI_SUCCESS; }
inline int MPI_Waitall(int, MPI_Request*, MPI_Status*) { return MPI_SUCCESS; }
inline int MPI_Testsome(int, MPI_Request*, int* outcount, int*, MPI_Status*) { *outcount = MPI_UNDEFINED; return MPI_SUCCESS; }
// A harness that plays the other side in process: the last buffer sent, and a hook that answers a receive
// (tag, buffer, count); without a hook a receive fails.
inline const void*& spx_mpi_last_send() { static const void* p = nullptr; return p; }
typedef int (*spx_mpi_recv_fn)(int tag, void* buf, int count);
inline spx_mpi_recv_fn& spx_mpi_recv_hook() { static spx_mpi_recv_fn h = nullptr; return h; }

inline int MPI_Send(const void* buf, int, MPI_Datatype, int, int, MPI_Comm)
{
   spx_mpi_last_send() = buf;
   return MPI_SUCCESS;
}
inline int MPI_Recv(void* buf, int count, MPI_Datatype, int, int tag, MPI_Comm, MPI_Status*)
{
   return spx_mpi_recv_hook() ? spx_mpi_recv_hook()(tag, buf, count) : MPI_ERR_OTHER;
}
inline int MPI_Irecv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request* r) { *r = MPI_REQUEST_NULL; return MPI_ERR_OTHER; }
inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }
inline int MPI_Allreduce(const void*, void*, int, MPI_Datatype, MPI_Op, MPI_Comm) { return MPI_ERR_OTHER; }

#endif
