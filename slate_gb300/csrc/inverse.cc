// inverse.cc -- inverses and condition numbers from the factors:
// slate::getri (src/getri.cc), slate::potri (src/potri.cc), and the LAPACK-API
// front doors slate_dgetri / slate_dpotri (lapack_api/lapack_getri.cc,
// lapack_potri.cc) and slate_dgecon / slate_dpocon (lapack_gecon.cc,
// lapack_pocon.cc).
//
// The inverse is the solution of A X = I with the existing factors, 16
// columns per pair of triangular sweeps, written back over A (getri: all of
// A; potri: the triangle the factor occupied).  gecon / pocon take the
// factors without pivots, as LAPACK's do: ||A^{-1}|| in the 1- and infinity
// norms does not depend on the row order, so the estimate runs with identity
// pivots.

#include "drivers.h"
#include "lapack_opts.h"

#include <algorithm>
#include <cstring>
#include <vector>

using namespace slt;

namespace {

int identity_into(int64_t n, double* X, cudaStream_t s)
{
    SLT_CUDA_TRY(cudaMemsetAsync(X, 0, sizeof(double) * size_t(n) * size_t(n), s));
    return slt_dshift_diag(n, 1.0, X, n, s);
}

// First exactly-zero diagonal entry of U (1-based), or 0.
int zero_diag(int64_t n, const double* A, int64_t lda, cudaStream_t s, int64_t* where)
{
    std::vector<double> d(static_cast<size_t>(n));
    SLT_CUDA_TRY(cudaMemcpy2DAsync(d.data(), sizeof(double), A, sizeof(double) * size_t(lda + 1), sizeof(double),
                                   size_t(n), cudaMemcpyDeviceToHost, s));
    SLT_CUDA_TRY(cudaStreamSynchronize(s));
    *where = 0;
    for (int64_t i = 0; i < n; ++i)
        if (d[size_t(i)] == 0.0) { *where = i + 1; break; }
    return SLT_OK;
}

}  // namespace

// slate::getri: A (getrf's LU factors, per-panel pivots ipiv) <- A^{-1}.
// *info = i > 0 when U(i, i) is exactly zero (A singular; A unchanged).
extern "C" int slt_dgetri_device(int64_t n, double* dA, int64_t lda, const int* d_ipiv, const slt_options* opts,
                                 slt_stream_t stream, int64_t* info)
{
    if (!info || n < 0 || lda < std::max<int64_t>(1, n)) return SLT_ERR_ARG;
    *info = 0;
    if (n == 0) return SLT_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    TRY(zero_diag(n, dA, lda, s, info));
    if (*info) return SLT_OK;
    DevBuf X;
    TRY(X.alloc(sizeof(double) * size_t(n) * size_t(n), s));
    TRY(identity_into(n, X.as<double>(), s));
    TRY(slt_dgetrs_device(n, n, dA, lda, d_ipiv, X.as<double>(), n, opts, stream));
    SLT_CUDA_TRY(cudaMemcpy2DAsync(dA, sizeof(double) * size_t(lda), X.p, sizeof(double) * size_t(n),
                                   sizeof(double) * size_t(n), size_t(n), cudaMemcpyDeviceToDevice, s));
    SLT_CUDA_TRY(cudaStreamSynchronize(s));
    return SLT_OK;
}

// slate::potri (lower): A (potrf's lower factor) <- lower triangle of A^{-1}.
extern "C" int slt_dpotri_device(int64_t n, double* dA, int64_t lda, const slt_options* opts, slt_stream_t stream,
                                 int64_t* info)
{
    if (!info || n < 0 || lda < std::max<int64_t>(1, n)) return SLT_ERR_ARG;
    *info = 0;
    if (n == 0) return SLT_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    TRY(zero_diag(n, dA, lda, s, info));
    if (*info) return SLT_OK;
    DevBuf X;
    TRY(X.alloc(sizeof(double) * size_t(n) * size_t(n), s));
    TRY(identity_into(n, X.as<double>(), s));
    TRY(slt_dpotrs_device(n, n, dA, lda, X.as<double>(), n, opts, stream));
    TRY(slt_dcopy_tri(1, n, X.as<double>(), n, dA, lda, s));
    SLT_CUDA_TRY(cudaStreamSynchronize(s));
    return SLT_OK;
}

// ---- LAPACK-API front doors (host arrays, Fortran by-pointer arguments) ----
namespace {

struct Stream {
    cudaStream_t s = nullptr;
    Stream() { if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) s = nullptr; }
    ~Stream() { if (s) cudaStreamDestroy(s); }
};

cudaStream_t stream_()
{
    static thread_local Stream st;
    return st.s;
}


int upload(const double* a, int64_t n, int64_t lda, DevBuf& d, cudaStream_t s)
{
    TRY(d.alloc(sizeof(double) * size_t(n) * size_t(n), s));
    SLT_CUDA_TRY(cudaMemcpy2DAsync(d.p, sizeof(double) * size_t(n), a, sizeof(double) * size_t(lda),
                                   sizeof(double) * size_t(n), size_t(n), cudaMemcpyHostToDevice, s));
    return SLT_OK;
}

// identity per-panel pivots (row r of panel k is pivot r - k nb)
int identity_pivots(int64_t n, int64_t nb, DevBuf& d, cudaStream_t s)
{
    std::vector<int> rel(static_cast<size_t>(n));
    for (int64_t r = 0; r < n; ++r) rel[size_t(r)] = int(r % nb);
    TRY(d.alloc(sizeof(int) * size_t(n), s));
    SLT_CUDA_TRY(cudaMemcpyAsync(d.p, rel.data(), sizeof(int) * size_t(n), cudaMemcpyHostToDevice, s));
    return SLT_OK;
}

void getri_impl(int n, double* a, int lda, const int* ipiv, int* info)
{
    *info = 0;
    if (n < 0) { *info = -1; return; }
    if (lda < std::max(1, n)) { *info = -3; return; }
    if (n == 0) return;
    cudaStream_t s = stream_();
    const slt_options o = lapack_opts();
    std::vector<int> rel(static_cast<size_t>(n));
    for (int r = 0; r < n; ++r) rel[size_t(r)] = int(ipiv[r] - 1 - (r / o.nb) * o.nb);
    DevBuf dA, dP;
    if (upload(a, n, lda, dA, s) || dP.alloc(sizeof(int) * size_t(n), s) ||
        cudaMemcpyAsync(dP.p, rel.data(), sizeof(int) * size_t(n), cudaMemcpyHostToDevice, s) != cudaSuccess) {
        *info = -100;
        return;
    }
    int64_t inf = 0;
    const int rc = slt_dgetri_device(n, dA.as<double>(), n, dP.as<int>(), &o, s, &inf);
    if (rc) { *info = -1000 + rc; return; }
    if (inf == 0 &&
        cudaMemcpy2DAsync(a, sizeof(double) * size_t(lda), dA.p, sizeof(double) * size_t(n),
                          sizeof(double) * size_t(n), size_t(n), cudaMemcpyDeviceToHost, s) != cudaSuccess) {
        *info = -100;
        return;
    }
    cudaStreamSynchronize(s);
    *info = int(inf);
}

// The referenced triangle of a (uplo) as a lower-triangular device array.
int lower_factor(char uplo, int n, const double* a, int lda, DevBuf& d, cudaStream_t s)
{
    TRY(upload(a, n, lda, d, s));
    if (uplo == 'U' || uplo == 'u') {
        DevBuf t;
        TRY(t.alloc(sizeof(double) * size_t(n) * size_t(n), s));
        TRY(slt_dtranspose(n, n, d.as<double>(), n, t.as<double>(), n, s));
        std::swap(d.p, t.p);
    }
    return SLT_OK;
}

void potri_impl(char uplo, int n, double* a, int lda, int* info)
{
    *info = 0;
    const bool up = (uplo == 'U' || uplo == 'u');
    if (!up && uplo != 'L' && uplo != 'l') { *info = -1; return; }
    if (n < 0) { *info = -2; return; }
    if (lda < std::max(1, n)) { *info = -4; return; }
    if (n == 0) return;
    cudaStream_t s = stream_();
    const slt_options o = lapack_opts();
    DevBuf dL;
    if (lower_factor(uplo, n, a, lda, dL, s)) { *info = -100; return; }
    int64_t inf = 0;
    const int rc = slt_dpotri_device(n, dL.as<double>(), n, &o, s, &inf);
    if (rc) { *info = -1000 + rc; return; }
    if (inf) { *info = int(inf); return; }
    std::vector<double> h(size_t(n) * size_t(n));
    if (cudaMemcpyAsync(h.data(), dL.p, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        *info = -100;
        return;
    }
    // dL holds the lower triangle of A^{-1} (symmetric): write the referenced triangle
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i)
            if (up ? (i <= j) : (i >= j))
                a[i + size_t(j) * lda] = up ? h[size_t(j) + size_t(i) * n] : h[size_t(i) + size_t(j) * n];
}

void gecon_impl(char norm, int n, const double* a, int lda, double anorm, double* rcond, int* info)
{
    *info = 0;
    const bool ok = std::strchr("1OoIi", norm) != nullptr && norm != 0;
    if (!ok) { *info = -1; return; }
    if (n < 0) { *info = -2; return; }
    if (lda < std::max(1, n)) { *info = -4; return; }
    if (anorm < 0) { *info = -5; return; }
    cudaStream_t s = stream_();
    const slt_options o = lapack_opts();
    if (n == 0) { *rcond = 1.0; return; }
    DevBuf dA, dP;
    if (upload(a, n, lda, dA, s) || identity_pivots(n, o.nb, dP, s)) { *info = -100; return; }
    const int rc = slt_dgecondest_device(norm == 'O' || norm == 'o' ? '1' : norm, n, dA.as<double>(), n,
                                         dP.as<int>(), anorm, rcond, &o, s);
    if (rc) *info = -1000 + rc;
}

void pocon_impl(char uplo, int n, const double* a, int lda, double anorm, double* rcond, int* info)
{
    *info = 0;
    if (uplo != 'U' && uplo != 'u' && uplo != 'L' && uplo != 'l') { *info = -1; return; }
    if (n < 0) { *info = -2; return; }
    if (lda < std::max(1, n)) { *info = -4; return; }
    if (anorm < 0) { *info = -5; return; }
    if (n == 0) { *rcond = 1.0; return; }
    cudaStream_t s = stream_();
    const slt_options o = lapack_opts();
    DevBuf dL;
    if (lower_factor(uplo, n, a, lda, dL, s)) { *info = -100; return; }
    const int rc = slt_dpocondest_device('1', n, dL.as<double>(), n, anorm, rcond, &o, s);
    if (rc) *info = -1000 + rc;
}

}  // namespace

extern "C" {

void slate_dgetri(const int* n, double* a, const int* lda, int* ipiv, double*, const int*, int* info)
{ getri_impl(*n, a, *lda, ipiv, info); }
void slate_dgetri_(const int* n, double* a, const int* lda, int* ipiv, double*, const int*, int* info)
{ getri_impl(*n, a, *lda, ipiv, info); }
void slate_dpotri(const char* uplo, const int* n, double* a, const int* lda, int* info)
{ potri_impl(*uplo, *n, a, *lda, info); }
void slate_dpotri_(const char* uplo, const int* n, double* a, const int* lda, int* info)
{ potri_impl(*uplo, *n, a, *lda, info); }
void slate_dgecon(const char* norm, const int* n, double* a, const int* lda, double* anorm, double* rcond, double*,
                  int*, int* info)
{ gecon_impl(*norm, *n, a, *lda, *anorm, rcond, info); }
void slate_dgecon_(const char* norm, const int* n, double* a, const int* lda, double* anorm, double* rcond, double*,
                   int*, int* info)
{ gecon_impl(*norm, *n, a, *lda, *anorm, rcond, info); }
void slate_dpocon(const char* uplo, const int* n, double* a, const int* lda, double* anorm, double* rcond, double*,
                  int*, int* info)
{ pocon_impl(*uplo, *n, a, *lda, *anorm, rcond, info); }
void slate_dpocon_(const char* uplo, const int* n, double* a, const int* lda, double* anorm, double* rcond, double*,
                   int*, int* info)
{ pocon_impl(*uplo, *n, a, *lda, *anorm, rcond, info); }

}  // extern "C"
