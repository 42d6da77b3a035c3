// Single-process stand-in for the MPI calls SLATE's tile panel code makes
// (src/internal/Tile_getrf.hh, src/internal/internal_swap.hh).  On one rank
// every reduction is a copy, every broadcast from the root a no-op, and no
// point-to-point exchange happens: the calls that would need a peer abort.
// Test infrastructure only (compiled by oracle/build_ref.sh).
#ifndef ORACLE_REFSHIM_MPI_H
#define ORACLE_REFSHIM_MPI_H
#include <cstdio>
#include <cstdlib>
#include <cstring>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_SUCCESS 0
#define MPI_MAX_ERROR_STRING 64
#define MPI_COMM_WORLD 0
#define MPI_MAXLOC 1
#define MPI_BYTE 1
#define MPI_INT 4
#define MPI_INT64_T 8
#define MPI_FLOAT 4
#define MPI_DOUBLE 8
#define MPI_C_COMPLEX 8
#define MPI_C_DOUBLE_COMPLEX 16
#define MPI_FLOAT_INT 8
#define MPI_DOUBLE_INT 16
#define MPI_STATUS_IGNORE ((MPI_Status*) 0)

#include <chrono>
inline double MPI_Wtime()
{ return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count(); }
inline int MPI_Error_string(int, char* s, int* len) { std::strcpy(s, "stand-in"); *len = 8; return 0; }
// Datatype values are element sizes in bytes.
inline int MPI_Allreduce(const void* in, void* out, int count, MPI_Datatype type, MPI_Op, MPI_Comm)
{ std::memmove(out, in, size_t(count) * size_t(type)); return MPI_SUCCESS; }
inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }
inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return MPI_SUCCESS; }
inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return MPI_SUCCESS; }
inline int no_peer(const char* f) { std::fprintf(stderr, "refshim mpi: %s needs a peer\n", f); std::abort(); }
inline int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm) { return no_peer("MPI_Send"); }
inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) { return no_peer("MPI_Recv"); }
inline int MPI_Sendrecv(const void*, int, MPI_Datatype, int, int, void*, int, MPI_Datatype, int, int, MPI_Comm,
                        MPI_Status*) { return no_peer("MPI_Sendrecv"); }
inline int MPI_Sendrecv_replace(void*, int, MPI_Datatype, int, int, int, int, MPI_Comm, MPI_Status*)
{ return no_peer("MPI_Sendrecv_replace"); }
#endif
