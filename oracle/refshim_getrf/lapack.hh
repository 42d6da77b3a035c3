// Stand-in for the part of LAPACK++ (an empty submodule in the SLATE tree)
// that SLATE's tile panel code calls: lacpy.  Test infrastructure only.
#ifndef ORACLE_REFSHIM_GETRF_LAPACK_HH
#define ORACLE_REFSHIM_GETRF_LAPACK_HH
#include <cstdint>
namespace lapack {
enum class MatrixType : char { General = 'G', Lower = 'L', Upper = 'U' };
template <typename T> void lacpy(MatrixType, int64_t m, int64_t n, const T* A, int64_t lda, T* B, int64_t ldb)
{ for (int64_t j = 0; j < n; ++j) for (int64_t i = 0; i < m; ++i) B[i + j * ldb] = A[i + j * lda]; }
} // namespace lapack
#endif
