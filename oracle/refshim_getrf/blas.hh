// Stand-in for the part of BLAS++ (the icl-utk-edu blaspp library, an empty
// submodule in the SLATE tree) that SLATE's tile panel code calls: the enums
// and column-major copy / swap / scal / geru / trsm / gemm, written here as
// plain loops.  Test infrastructure only (compiled by oracle/build_ref.sh).
#ifndef ORACLE_REFSHIM_GETRF_BLAS_HH
#define ORACLE_REFSHIM_GETRF_BLAS_HH
#include <complex>
#include <cstdint>
#include <utility>

namespace blas {
template <typename T> struct real_type_s { using type = T; };
template <typename T> struct real_type_s<std::complex<T>> { using type = T; };
template <typename T> using real_type = typename real_type_s<T>::type;

enum class Layout : char { ColMajor = 'C', RowMajor = 'R' };
enum class Op : char { NoTrans = 'N', Trans = 'T', ConjTrans = 'C' };
enum class Uplo : char { Upper = 'U', Lower = 'L', General = 'G' };
enum class Diag : char { NonUnit = 'N', Unit = 'U' };
enum class Side : char { Left = 'L', Right = 'R' };

template <typename T> void copy(int64_t n, const T* x, int64_t incx, T* y, int64_t incy)
{ for (int64_t i = 0; i < n; ++i) y[i * incy] = x[i * incx]; }

template <typename T> void swap(int64_t n, T* x, int64_t incx, T* y, int64_t incy)
{ for (int64_t i = 0; i < n; ++i) std::swap(x[i * incx], y[i * incy]); }

template <typename T> void scal(int64_t n, T alpha, T* x, int64_t incx)
{ for (int64_t i = 0; i < n; ++i) x[i * incx] *= alpha; }

// A += alpha x y^T (column-major)
template <typename T> void geru(Layout, int64_t m, int64_t n, T alpha, const T* x, int64_t incx,
                                const T* y, int64_t incy, T* A, int64_t lda)
{
    for (int64_t j = 0; j < n; ++j) {
        const T t = alpha * y[j * incy];
        for (int64_t i = 0; i < m; ++i) A[i + j * lda] += x[i * incx] * t;
    }
}

// B <- alpha op(A)^{-1} B, left side, column-major, no transpose (the only form the panel uses)
template <typename T> void trsm(Layout, Side, Uplo uplo, Op, Diag diag, int64_t m, int64_t n, T alpha,
                                const T* A, int64_t lda, T* B, int64_t ldb)
{
    for (int64_t j = 0; j < n; ++j) {
        T* b = B + j * ldb;
        for (int64_t i = 0; i < m; ++i) b[i] *= alpha;
        if (uplo == Uplo::Lower) {
            for (int64_t k = 0; k < m; ++k) {
                if (diag == Diag::NonUnit) b[k] /= A[k + k * lda];
                for (int64_t i = k + 1; i < m; ++i) b[i] -= b[k] * A[i + k * lda];
            }
        }
        else {
            for (int64_t k = m - 1; k >= 0; --k) {
                if (diag == Diag::NonUnit) b[k] /= A[k + k * lda];
                for (int64_t i = 0; i < k; ++i) b[i] -= b[k] * A[i + k * lda];
            }
        }
    }
}

// C <- alpha A B + beta C, column-major, no transposes (the only form the panel uses)
template <typename T> void gemm(Layout, Op, Op, int64_t m, int64_t n, int64_t k, T alpha, const T* A,
                                int64_t lda, const T* B, int64_t ldb, T beta, T* C, int64_t ldc)
{
    for (int64_t j = 0; j < n; ++j) {
        T* c = C + j * ldc;
        for (int64_t i = 0; i < m; ++i) c[i] *= beta;
        for (int64_t l = 0; l < k; ++l) {
            const T t = alpha * B[l + j * ldb];
            for (int64_t i = 0; i < m; ++i) c[i] += A[i + l * lda] * t;
        }
    }
}
} // namespace blas
#endif
