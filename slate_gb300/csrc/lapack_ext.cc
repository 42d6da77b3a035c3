// lapack_ext.cc -- the LAPACK-compatible entry points of the other
// precisions: slate_sgetrs / sposv / spotrf and the complex c / z forms of
// gesv, getrf, getrs, posv and potrf, plus slate_zcgesv
// (lapack_api/lapack_gesv.cc:25-45, lapack_getrf.cc, lapack_getrs.cc:19-22,
// lapack_posv.cc:22-25, lapack_potrf.cc:20-23, lapack_gesv_mixed.cc:30-33).
//
// Same contract as the d forms in capi.cc: host arrays, Fortran by-pointer
// arguments, 32-bit int, 1-based ipiv, info = -i for the i-th bad argument,
// the SLATE_LAPACK_* environment for nb and the mixed solver's options, and
// both manglings BLAS_FORTRAN_NAME can produce (slate_cgesv, slate_cgesv_).
// Complex arrays are interleaved (real, imaginary) pairs: std::complex,
// C99 _Complex and Fortran COMPLEX share that layout.

#include "drivers.h"
#include "lapack_opts.h"

#include <algorithm>
#include <cstring>
#include <vector>

using namespace slt;

namespace {

struct C32 { float re, im; };
struct C64 { double re, im; };

// Per-type device entry points and the type code of the generic helpers.
template <typename T> struct Dev;
template <> struct Dev<float> {
    static constexpr int type = 0;
    static int getrf(int64_t m, int64_t n, float* A, int64_t lda, int* ip, const slt_options* o, cudaStream_t s, int64_t* info)
    { return slt_sgetrf_device(m, n, A, lda, ip, o, s, info); }
    static int getrs(char t, int64_t n, int64_t r, const float* A, int64_t lda, const int* ip, float* B, int64_t ldb,
                     const slt_options* o, cudaStream_t s)
    { return slt_sgetrs_trans_device(t, n, r, A, lda, ip, B, ldb, o, s); }
    static int potrf(int64_t n, float* A, int64_t lda, const slt_options* o, cudaStream_t s, int64_t* info)
    { return slt_spotrf_device(n, A, lda, o, s, info); }
    static int potrs(int64_t n, int64_t r, const float* A, int64_t lda, float* B, int64_t ldb, const slt_options* o,
                     cudaStream_t s)
    { return slt_spotrs_device(n, r, A, lda, B, ldb, o, s); }
};
template <> struct Dev<C32> {
    static constexpr int type = 2;
    static int getrf(int64_t m, int64_t n, C32* A, int64_t lda, int* ip, const slt_options* o, cudaStream_t s, int64_t* info)
    { return slt_cgetrf_device(m, n, A, lda, ip, o, s, info); }
    static int getrs(char t, int64_t n, int64_t r, const C32* A, int64_t lda, const int* ip, C32* B, int64_t ldb,
                     const slt_options* o, cudaStream_t s)
    { return slt_cgetrs_device(t, n, r, A, lda, ip, B, ldb, o, s); }
    static int potrf(int64_t n, C32* A, int64_t lda, const slt_options* o, cudaStream_t s, int64_t* info)
    { return slt_cpotrf_device(n, A, lda, o, s, info); }
    static int potrs(int64_t n, int64_t r, const C32* A, int64_t lda, C32* B, int64_t ldb, const slt_options* o,
                     cudaStream_t s)
    { return slt_cpotrs_device(n, r, A, lda, B, ldb, o, s); }
};
template <> struct Dev<C64> {
    static constexpr int type = 3;
    static int getrf(int64_t m, int64_t n, C64* A, int64_t lda, int* ip, const slt_options* o, cudaStream_t s, int64_t* info)
    { return slt_zgetrf_device(m, n, A, lda, ip, o, s, info); }
    static int getrs(char t, int64_t n, int64_t r, const C64* A, int64_t lda, const int* ip, C64* B, int64_t ldb,
                     const slt_options* o, cudaStream_t s)
    { return slt_zgetrs_device(t, n, r, A, lda, ip, B, ldb, o, s); }
    static int potrf(int64_t n, C64* A, int64_t lda, const slt_options* o, cudaStream_t s, int64_t* info)
    { return slt_zpotrf_device(n, A, lda, o, s, info); }
    static int potrs(int64_t n, int64_t r, const C64* A, int64_t lda, C64* B, int64_t ldb, const slt_options* o,
                     cudaStream_t s)
    { return slt_zpotrs_device(n, r, A, lda, B, ldb, o, s); }
};

struct XStream {
    cudaStream_t s = nullptr;
    XStream() { if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) s = nullptr; }
    ~XStream() { if (s) cudaStreamDestroy(s); }
};

cudaStream_t xstream()
{
    static thread_local XStream st;
    return st.s;
}

template <typename T>
int up(const T* h, int64_t m, int64_t n, int64_t ld, DevBuf& d, cudaStream_t s)
{
    TRY(d.alloc(sizeof(T) * size_t(std::max<int64_t>(m, 1)) * size_t(std::max<int64_t>(n, 1)), s));
    if (m > 0 && n > 0)
        SLT_CUDA_TRY(cudaMemcpy2DAsync(d.p, size_t(m) * sizeof(T), h, size_t(ld) * sizeof(T), size_t(m) * sizeof(T),
                                       size_t(n), cudaMemcpyHostToDevice, s));
    return SLT_OK;
}

template <typename T>
int down(const DevBuf& d, T* h, int64_t m, int64_t n, int64_t ld, cudaStream_t s)
{
    if (m > 0 && n > 0)
        SLT_CUDA_TRY(cudaMemcpy2DAsync(h, size_t(ld) * sizeof(T), d.p, size_t(m) * sizeof(T), size_t(m) * sizeof(T),
                                       size_t(n), cudaMemcpyDeviceToHost, s));
    return SLT_OK;
}

void to_lapack(const std::vector<int>& rel, int64_t nb, int* ipiv, int64_t cnt)
{
    for (int64_t r = 0; r < cnt; ++r) ipiv[r] = int((r / nb) * nb + rel[r] + 1);
}

void from_lapack(const int* ipiv, int64_t nb, std::vector<int>& rel, int64_t cnt)
{
    rel.resize(cnt);
    for (int64_t r = 0; r < cnt; ++r) rel[r] = int(ipiv[r] - 1 - (r / nb) * nb);
}

template <typename T>
void getrf_impl(int m, int n, T* a, int lda, int* ipiv, int* info)
{
    *info = 0;
    if (m < 0) { *info = -1; return; }
    if (n < 0) { *info = -2; return; }
    if (lda < std::max(1, m)) { *info = -4; return; }
    if (m == 0 || n == 0) return;
    cudaStream_t s = xstream();
    slt_options o = lapack_opts();
    const int mn = std::min(m, n);
    DevBuf dA, dP;
    if (up(a, m, n, lda, dA, s) || dP.alloc(sizeof(int) * size_t(mn), s)) { *info = -100; return; }
    int64_t inf = 0;
    const int rc = Dev<T>::getrf(m, n, dA.as<T>(), m, dP.as<int>(), &o, s, &inf);
    if (rc) { *info = -1000 + rc; return; }
    std::vector<int> rel(mn);
    if (down(dA, a, m, n, lda, s) ||
        cudaMemcpyAsync(rel.data(), dP.p, sizeof(int) * size_t(mn), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) { *info = -100; return; }
    to_lapack(rel, o.nb, ipiv, mn);
    *info = int(inf);
}

template <typename T>
void gesv_impl(int n, int nrhs, T* a, int lda, int* ipiv, T* b, int ldb, int* info)
{
    *info = 0;
    if (n < 0) { *info = -1; return; }
    if (nrhs < 0) { *info = -2; return; }
    if (lda < std::max(1, n)) { *info = -4; return; }
    if (ldb < std::max(1, n)) { *info = -7; return; }
    if (n == 0) return;
    cudaStream_t s = xstream();
    slt_options o = lapack_opts();
    DevBuf dA, dB, dP;
    if (up(a, n, n, lda, dA, s) || up(b, n, nrhs, ldb, dB, s) || dP.alloc(sizeof(int) * size_t(n), s)) {
        *info = -100;
        return;
    }
    int64_t inf = 0;
    int rc = Dev<T>::getrf(n, n, dA.as<T>(), n, dP.as<int>(), &o, s, &inf);
    if (!rc && inf == 0 && nrhs > 0) rc = Dev<T>::getrs('N', n, nrhs, dA.as<T>(), n, dP.as<int>(), dB.as<T>(), n, &o, s);
    if (rc) { *info = -1000 + rc; return; }
    std::vector<int> rel(n);
    if (down(dA, a, n, n, lda, s) || down(dB, b, n, nrhs, ldb, s) ||
        cudaMemcpyAsync(rel.data(), dP.p, sizeof(int) * size_t(n), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) { *info = -100; return; }
    to_lapack(rel, o.nb, ipiv, n);
    *info = int(inf);
}

template <typename T>
void getrs_impl(char trans, int n, int nrhs, T* a, int lda, int* ipiv, T* b, int ldb, int* info)
{
    *info = 0;
    if (std::strchr("NnTtCc", trans) == nullptr || trans == 0) { *info = -1; return; }
    if (n < 0) { *info = -2; return; }
    if (nrhs < 0) { *info = -3; return; }
    if (lda < std::max(1, n)) { *info = -5; return; }
    if (ldb < std::max(1, n)) { *info = -8; return; }
    if (n == 0 || nrhs == 0) return;
    cudaStream_t s = xstream();
    slt_options o = lapack_opts();
    std::vector<int> rel;
    from_lapack(ipiv, o.nb, rel, n);
    DevBuf dA, dB, dP;
    if (up(a, n, n, lda, dA, s) || up(b, n, nrhs, ldb, dB, s) || up(rel.data(), n, 1, n, dP, s)) {
        *info = -100;
        return;
    }
    const int rc = Dev<T>::getrs(trans, n, nrhs, dA.as<T>(), n, dP.as<int>(), dB.as<T>(), n, &o, s);
    if (rc) { *info = -1000 + rc; return; }
    if (down(dB, b, n, nrhs, ldb, s) || cudaStreamSynchronize(s) != cudaSuccess) { *info = -100; return; }
}

// potrf / posv: an upper-stored matrix is conjugate-transposed on the device
// into lower storage (SLATE: A = conj_transpose(A), src/potrf.cc:45-47) and
// the factor back; only the referenced triangle is written to the caller.
template <typename T>
void potrf_impl(char uplo, int n, T* a, int lda, int* info, int nrhs, T* b, int ldb)
{
    *info = 0;
    const bool upper = (uplo == 'U' || uplo == 'u');
    if (!upper && uplo != 'L' && uplo != 'l') { *info = -1; return; }
    if (n < 0) { *info = -2; return; }
    if (nrhs < 0) { *info = -3; return; }
    if (lda < std::max(1, n)) { *info = b ? -5 : -4; return; }
    if (b && ldb < std::max(1, n)) { *info = -7; return; }
    if (n == 0) return;
    cudaStream_t s = xstream();
    slt_options o = lapack_opts();
    DevBuf dA, dB, tmp;
    if (up(a, n, n, lda, dA, s) || (b && up(b, n, nrhs, ldb, dB, s))) { *info = -100; return; }
    if (upper) {
        if (tmp.alloc(sizeof(T) * size_t(n) * size_t(n), s) ||
            slt_xtranspose(Dev<T>::type, n, n, dA.p, n, tmp.p, n, 1, s)) { *info = -100; return; }
        std::swap(dA.p, tmp.p);
    }
    int64_t inf = 0;
    int rc = Dev<T>::potrf(n, dA.as<T>(), n, &o, s, &inf);
    if (!rc && inf == 0 && b && nrhs > 0) rc = Dev<T>::potrs(n, nrhs, dA.as<T>(), n, dB.as<T>(), n, &o, s);
    if (rc) { *info = -1000 + rc; return; }
    if (upper && slt_xtranspose(Dev<T>::type, n, n, dA.p, n, tmp.p, n, 1, s)) { *info = -100; return; }
    const DevBuf& F = upper ? tmp : dA;
    std::vector<T> h(size_t(n) * size_t(n));
    if (cudaMemcpyAsync(h.data(), F.p, sizeof(T) * h.size(), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        (b && down(dB, b, n, nrhs, ldb, s)) || cudaStreamSynchronize(s) != cudaSuccess) { *info = -100; return; }
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i)
            if (upper ? (i <= j) : (i >= j)) a[i + size_t(j) * lda] = h[i + size_t(j) * n];
    *info = int(inf);
}

void zcgesv_impl(int n, int nrhs, C64* a, int lda, int* ipiv, C64* b, int ldb, C64* x, int ldx, int* iter, int* info)
{
    *info = 0;
    *iter = 0;
    if (n < 0) { *info = -1; return; }
    if (nrhs < 0) { *info = -2; return; }
    if (lda < std::max(1, n)) { *info = -4; return; }
    if (ldb < std::max(1, n)) { *info = -7; return; }
    if (ldx < std::max(1, n)) { *info = -9; return; }
    if (n == 0) return;
    cudaStream_t s = xstream();
    slt_options o = lapack_opts();
    DevBuf dA, dB, dX, dP;
    if (up(a, n, n, lda, dA, s) || up(b, n, nrhs, ldb, dB, s) ||
        dX.alloc(sizeof(C64) * size_t(n) * size_t(std::max(nrhs, 1)), s) || dP.alloc(sizeof(int) * size_t(n), s)) {
        *info = -100;
        return;
    }
    int64_t inf = 0;
    int it = 0;
    const int rc = slt_zcgesv_device(n, nrhs, dA.p, n, dP.as<int>(), dB.p, n, dX.p, n, &o, s, &it, &inf);
    if (rc) { *info = -1000 + rc; return; }
    std::vector<int> rel(n);
    if (down(dX, x, n, nrhs, ldx, s) || down(dA, a, n, n, lda, s) ||
        cudaMemcpyAsync(rel.data(), dP.p, sizeof(int) * size_t(n), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) { *info = -100; return; }
    to_lapack(rel, o.nb, ipiv, n);
    *iter = it;
    *info = int(inf);
}

} // namespace

extern "C" {

#define SLT_BOTH(name, params, call) void name params call void name##_ params call

SLT_BOTH(slate_sgetrs, (const char* trans, const int* n, const int* nrhs, float* a, const int* lda, int* ipiv,
                        float* b, const int* ldb, int* info),
         { getrs_impl<float>(*trans, *n, *nrhs, a, *lda, ipiv, b, *ldb, info); })
SLT_BOTH(slate_cgetrs, (const char* trans, const int* n, const int* nrhs, void* a, const int* lda, int* ipiv,
                        void* b, const int* ldb, int* info),
         { getrs_impl<C32>(*trans, *n, *nrhs, static_cast<C32*>(a), *lda, ipiv, static_cast<C32*>(b), *ldb, info); })
SLT_BOTH(slate_zgetrs, (const char* trans, const int* n, const int* nrhs, void* a, const int* lda, int* ipiv,
                        void* b, const int* ldb, int* info),
         { getrs_impl<C64>(*trans, *n, *nrhs, static_cast<C64*>(a), *lda, ipiv, static_cast<C64*>(b), *ldb, info); })
SLT_BOTH(slate_cgesv, (const int* n, const int* nrhs, void* a, const int* lda, int* ipiv, void* b, const int* ldb,
                       int* info),
         { gesv_impl<C32>(*n, *nrhs, static_cast<C32*>(a), *lda, ipiv, static_cast<C32*>(b), *ldb, info); })
SLT_BOTH(slate_zgesv, (const int* n, const int* nrhs, void* a, const int* lda, int* ipiv, void* b, const int* ldb,
                       int* info),
         { gesv_impl<C64>(*n, *nrhs, static_cast<C64*>(a), *lda, ipiv, static_cast<C64*>(b), *ldb, info); })
SLT_BOTH(slate_cgetrf, (const int* m, const int* n, void* a, const int* lda, int* ipiv, int* info),
         { getrf_impl<C32>(*m, *n, static_cast<C32*>(a), *lda, ipiv, info); })
SLT_BOTH(slate_zgetrf, (const int* m, const int* n, void* a, const int* lda, int* ipiv, int* info),
         { getrf_impl<C64>(*m, *n, static_cast<C64*>(a), *lda, ipiv, info); })
SLT_BOTH(slate_sposv, (const char* uplo, const int* n, const int* nrhs, float* a, const int* lda, float* b,
                       const int* ldb, int* info),
         { potrf_impl<float>(*uplo, *n, a, *lda, info, *nrhs, b, *ldb); })
SLT_BOTH(slate_cposv, (const char* uplo, const int* n, const int* nrhs, void* a, const int* lda, void* b,
                       const int* ldb, int* info),
         { potrf_impl<C32>(*uplo, *n, static_cast<C32*>(a), *lda, info, *nrhs, static_cast<C32*>(b), *ldb); })
SLT_BOTH(slate_zposv, (const char* uplo, const int* n, const int* nrhs, void* a, const int* lda, void* b,
                       const int* ldb, int* info),
         { potrf_impl<C64>(*uplo, *n, static_cast<C64*>(a), *lda, info, *nrhs, static_cast<C64*>(b), *ldb); })
SLT_BOTH(slate_spotrf, (const char* uplo, const int* n, float* a, const int* lda, int* info),
         { potrf_impl<float>(*uplo, *n, a, *lda, info, 0, nullptr, 1); })
SLT_BOTH(slate_cpotrf, (const char* uplo, const int* n, void* a, const int* lda, int* info),
         { potrf_impl<C32>(*uplo, *n, static_cast<C32*>(a), *lda, info, 0, nullptr, 1); })
SLT_BOTH(slate_zpotrf, (const char* uplo, const int* n, void* a, const int* lda, int* info),
         { potrf_impl<C64>(*uplo, *n, static_cast<C64*>(a), *lda, info, 0, nullptr, 1); })
SLT_BOTH(slate_zcgesv, (const int* n, const int* nrhs, void* a, const int* lda, int* ipiv, void* b, const int* ldb,
                        void* x, const int* ldx, void* work, void* swork, int* iter, int* info),
         { (void) work; (void) swork;
           zcgesv_impl(*n, *nrhs, static_cast<C64*>(a), *lda, ipiv, static_cast<C64*>(b), *ldb,
                       static_cast<C64*>(x), *ldx, iter, info); })

#undef SLT_BOTH

} // extern "C"
