// Stand-in for the slate/types.hh names SLATE's tile panel code uses: the
// BLAS enums in namespace slate, and the MPI datatype traits (values here
// are element sizes, which the single-process mpi.h stand-in copies).
// Test infrastructure only.
#ifndef ORACLE_REFSHIM_SLATE_TYPES_HH
#define ORACLE_REFSHIM_SLATE_TYPES_HH
#include <mpi.h>
#include <blas.hh>
#include <lapack.hh>
namespace slate {
using blas::Layout;
using blas::Op;
using blas::Uplo;
using blas::Diag;
using blas::Side;
template <typename T> struct mpi_type { static constexpr MPI_Datatype value = MPI_Datatype(sizeof(T)); };
template <typename real_t> struct max_loc_type { real_t x; int i; };
template <typename real_t> struct mpi_type<max_loc_type<real_t>> {
    static constexpr MPI_Datatype value = MPI_Datatype(sizeof(max_loc_type<real_t>));
};
namespace trace {
struct Block { explicit Block(const char*) {} };
}
} // namespace slate
#endif
