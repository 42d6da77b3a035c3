// Stand-in for src/internal/internal_swap.hh: swaps of partial rows between
// local tiles; the remote form needs a second MPI process and aborts.
// Test infrastructure only.
#ifndef ORACLE_REFSHIM_INTERNAL_SWAP_HH
#define ORACLE_REFSHIM_INTERNAL_SWAP_HH
#include <cstdlib>
#include "slate/Tile.hh"
namespace slate {
template <typename T>
void swapLocalRow(int64_t j, int64_t n, Tile<T>& A, int64_t i1, Tile<T>& B, int64_t i2)
{
    if (n <= 0) return;
    blas::swap(n, &A.at(i1, j), A.rowIncrement(), &B.at(i2, j), B.rowIncrement());
}
template <typename T>
void swapLocalRow(int64_t j, int64_t n, Tile<T>&& A, int64_t i1, Tile<T>&& B, int64_t i2)
{ swapLocalRow(j, n, A, i1, B, i2); }
template <typename T>
void swapRemoteRow(int64_t, int64_t, Tile<T>&, int64_t, int, MPI_Comm, int = 0) { no_peer("swapRemoteRow"); }
} // namespace slate
#endif
