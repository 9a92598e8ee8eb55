/*
 * Single-rank stand-in for the subset of MPI the reference sampler calls.
 *
 * TEST INFRASTRUCTURE ONLY.  This header lets the reference's header-only
 * C++ library (include/*.hxx of MarcJos/RSA_MPI) compile and run as ONE
 * process without an MPI library, so that its outputs can pin the oracle.
 * It is never linked into the GPU library.
 *
 * Semantics (one rank, rank 0, communicator size 1):
 *  - reductions / gathers copy the send buffer to the receive buffer;
 *  - Isend copies the message eagerly into a FIFO keyed by tag, Irecv pops
 *    the oldest message with the same tag (MPI's non-overtaking rule for one
 *    source; every ghost message of one exchange phase shares a tag, see
 *    include/operator_ghost.ixx:70-77 of the reference);
 *  - Cartesian topology calls describe a 1x1x...x1 periodic grid.
 */
#pragma once

#include <cstddef>
#include <cstdint>
#include <cstring>
#include <deque>
#include <map>
#include <stdexcept>
#include <vector>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_SUCCESS 0
#define MPI_COMM_WORLD 0
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)

#define MPI_CHAR 1
#define MPI_INT 4
#define MPI_UINT 104
#define MPI_DOUBLE 8
#define MPI_LONG_LONG 108
#define MPI_UINT64_T 208
#define MPI_C_BOOL 101

#define MPI_SUM 1
#define MPI_MAX 2

namespace mpi_standin {
inline size_t type_size(MPI_Datatype t) {
    switch (t) {
    case MPI_CHAR: return 1;
    case MPI_C_BOOL: return 1;
    case MPI_INT: return 4;
    case MPI_UINT: return 4;
    case MPI_DOUBLE: return 8;
    case MPI_LONG_LONG: return 8;
    case MPI_UINT64_T: return 8;
    default: throw std::runtime_error("mpi stand-in: unknown datatype");
    }
}
inline std::map<int, std::deque<std::vector<char>>>& mailbox() {
    static std::map<int, std::deque<std::vector<char>>> box;
    return box;
}
} // namespace mpi_standin

inline int MPI_Init(int*, char***) { return MPI_SUCCESS; }
inline int MPI_Finalize() { return MPI_SUCCESS; }
inline int MPI_Comm_size(MPI_Comm, int* size) { *size = 1; return MPI_SUCCESS; }
inline int MPI_Comm_rank(MPI_Comm, int* rank) { *rank = 0; return MPI_SUCCESS; }
inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }

inline int MPI_Allreduce(const void* send, void* recv, int count, MPI_Datatype t, MPI_Op, MPI_Comm) {
    std::memmove(recv, send, count * mpi_standin::type_size(t));
    return MPI_SUCCESS;
}
inline int MPI_Allgather(const void* send, int scount, MPI_Datatype st, void* recv, int, MPI_Datatype, MPI_Comm) {
    std::memmove(recv, send, scount * mpi_standin::type_size(st));
    return MPI_SUCCESS;
}
inline int MPI_Ibcast(void*, int, MPI_Datatype, int, MPI_Comm, MPI_Request* req) {
    *req = 0;
    return MPI_SUCCESS;
}
inline int MPI_Isend(const void* buf, int count, MPI_Datatype t, int, int tag, MPI_Comm, MPI_Request* req) {
    const char* p = static_cast<const char*>(buf);
    mpi_standin::mailbox()[tag].emplace_back(p, p + count * mpi_standin::type_size(t));
    *req = 0;
    return MPI_SUCCESS;
}
inline int MPI_Irecv(void* buf, int count, MPI_Datatype t, int, int tag, MPI_Comm, MPI_Request* req) {
    auto& q = mpi_standin::mailbox()[tag];
    if (q.empty()) throw std::runtime_error("mpi stand-in: receive with no matching send");
    const std::vector<char>& m = q.front();
    size_t want = count * mpi_standin::type_size(t);
    if (m.size() > want) throw std::runtime_error("mpi stand-in: message truncated");
    std::memcpy(buf, m.data(), m.size());
    q.pop_front();
    *req = 0;
    return MPI_SUCCESS;
}
inline int MPI_Waitall(int, MPI_Request*, MPI_Status*) { return MPI_SUCCESS; }

inline int MPI_Dims_create(int, int ndims, int* dims) {
    for (int i = 0; i < ndims; i++)
        if (dims[i] == 0) dims[i] = 1;
    return MPI_SUCCESS;
}
inline int MPI_Cart_create(MPI_Comm, int, const int*, const int*, int, MPI_Comm* cart) {
    *cart = 1;
    return MPI_SUCCESS;
}
inline int MPI_Cart_coords(MPI_Comm, int, int maxdims, int* coords) {
    for (int i = 0; i < maxdims; i++) coords[i] = 0;
    return MPI_SUCCESS;
}
inline int MPI_Cart_rank(MPI_Comm, const int*, int* rank) { *rank = 0; return MPI_SUCCESS; }
