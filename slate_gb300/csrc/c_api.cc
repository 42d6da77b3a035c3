// c_api.cc -- SLATE's C API (opaque Options / Pivots / Matrix handles and
// the simplified lu_* / chol_* drivers) over the device entry points.
//
// SLATE generates these wrappers (tools/c_api/generate_matrix.py,
// src/c_api/wrappers.cc:692-1080): each casts the handle back to a
// slate::Matrix and calls the C++ driver.  Here a handle records the user's
// column-major array (host or device memory), its sizes and tile size; each
// call makes a device view of it (the array itself when the CUDA runtime can
// address it, else a staged copy), runs the device driver on the library's
// per-thread stream and writes back what the driver changed.

#include "drivers.h"
#include "slate_c_api.h"

#include <algorithm>
#include <cstring>
#include <vector>

using namespace slt;

struct slate_Pivots_struct {
    std::vector<int> rel;   // per-panel relative pivots (SLATE's Pivot(tile, offset) as tile*nb + offset)
    int64_t nb = 0, n = 0;
};

namespace {

thread_local int64_t g_info = 0;
thread_local int g_status = 0;

struct COpts {
    slt_options o;
    int64_t chunk = 0, panel_threads = 1;
    char target = 'D', method_lu = '*';
    bool hold = false;
    COpts() { slt_options_default(&o); }
};

template <typename T>
struct CMat {
    int64_t m, n, nb, ld;
    T* data;
    bool dev;
    char uplo;   // 'G' general, 'L' / 'U' Hermitian
};

struct CStream {
    cudaStream_t s = nullptr;
    CStream() { if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) s = nullptr; }
    ~CStream() { if (s) cudaStreamDestroy(s); }
};

cudaStream_t cstream()
{
    static thread_local CStream cs;
    return cs.s;
}

bool device_accessible(const void* p)
{
    cudaPointerAttributes a;
    if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

slt_options opts_for(slate_Options h, int64_t nb)
{
    slt_options o;
    if (h) o = static_cast<COpts*>(h)->o;
    else slt_options_default(&o);
    o.nb = nb;        // the matrix's tile size, as in SLATE
    // MethodLU::NoPiv (src/getrf_nopiv.cc) and CALU (src/getrf_tntpiv.cc)
    if (h && static_cast<COpts*>(h)->method_lu == 'N') o.method_lu = 'N';
    if (h && static_cast<COpts*>(h)->method_lu == 'C') o.method_lu = 'C';
    return o;
}

// MethodLU::PartialPiv (and Auto), NoPiv and CALU are served; RBT is
// gesv_rbt's own driver and BEAM is not built.
bool lu_method_ok(slate_Options h)
{
    if (!h) return true;
    const char m = static_cast<COpts*>(h)->method_lu;
    return m == '*' || m == 'P' || m == 'N' || m == 'C';
}

void finish(int status, int64_t info)
{
    g_status = status;
    g_info = status ? -1 : info;
}

// A device copy (or the array itself) of an m x n matrix.
template <typename T>
struct View {
    DevBuf buf;
    T* p = nullptr;
    int64_t ld = 1;
    int open(const CMat<T>& M, cudaStream_t s) {
        if (M.dev) { p = M.data; ld = M.ld; return SLT_OK; }
        ld = std::max<int64_t>(1, M.m);
        TRY(buf.alloc(sizeof(T) * size_t(ld) * size_t(std::max<int64_t>(1, M.n)), s));
        p = buf.as<T>();
        if (M.m > 0 && M.n > 0)
            SLT_CUDA_TRY(cudaMemcpy2DAsync(p, size_t(ld) * sizeof(T), M.data, size_t(M.ld) * sizeof(T),
                                           size_t(M.m) * sizeof(T), size_t(M.n), cudaMemcpyHostToDevice, s));
        return SLT_OK;
    }
    int close(const CMat<T>& M, cudaStream_t s) {
        if (!M.dev && M.m > 0 && M.n > 0)
            SLT_CUDA_TRY(cudaMemcpy2DAsync(M.data, size_t(M.ld) * sizeof(T), p, size_t(ld) * sizeof(T),
                                           size_t(M.m) * sizeof(T), size_t(M.n), cudaMemcpyDeviceToHost, s));
        SLT_CUDA_TRY(cudaStreamSynchronize(s));
        return SLT_OK;
    }
};

template <typename T>
int getrf_dev_any(int64_t n, T* A, int64_t lda, int* ipiv, const slt_options* o, cudaStream_t s, int64_t* info);
template <>
int getrf_dev_any<double>(int64_t n, double* A, int64_t lda, int* ipiv, const slt_options* o, cudaStream_t s,
                          int64_t* info)
{ return slt_dgetrf_device(n, n, A, lda, ipiv, o, s, info); }
template <>
int getrf_dev_any<float>(int64_t n, float* A, int64_t lda, int* ipiv, const slt_options* o, cudaStream_t s,
                         int64_t* info)
{ return slt_sgetrf_device(n, n, A, lda, ipiv, o, s, info); }

template <typename T>
int getrs_dev_any(int64_t n, int64_t nrhs, const T* A, int64_t lda, const int* ipiv, T* B, int64_t ldb,
                  const slt_options* o, cudaStream_t s);
template <>
int getrs_dev_any<double>(int64_t n, int64_t nrhs, const double* A, int64_t lda, const int* ipiv, double* B,
                          int64_t ldb, const slt_options* o, cudaStream_t s)
{ return slt_dgetrs_device(n, nrhs, A, lda, ipiv, B, ldb, o, s); }
template <>
int getrs_dev_any<float>(int64_t n, int64_t nrhs, const float* A, int64_t lda, const int* ipiv, float* B,
                         int64_t ldb, const slt_options* o, cudaStream_t s)
{ return slt_sgetrs_device(n, nrhs, A, lda, ipiv, B, ldb, o, s); }

// complex elements as the C API passes them (interleaved real, imaginary)
struct CX32 { float re, im; };
struct CX64 { double re, im; };

template <>
int getrf_dev_any<CX32>(int64_t n, CX32* A, int64_t lda, int* ipiv, const slt_options* o, cudaStream_t s,
                        int64_t* info)
{ return slt_cgetrf_device(n, n, A, lda, ipiv, o, s, info); }
template <>
int getrf_dev_any<CX64>(int64_t n, CX64* A, int64_t lda, int* ipiv, const slt_options* o, cudaStream_t s,
                        int64_t* info)
{ return slt_zgetrf_device(n, n, A, lda, ipiv, o, s, info); }
template <>
int getrs_dev_any<CX32>(int64_t n, int64_t nrhs, const CX32* A, int64_t lda, const int* ipiv, CX32* B,
                        int64_t ldb, const slt_options* o, cudaStream_t s)
{ return slt_cgetrs_device('N', n, nrhs, A, lda, ipiv, B, ldb, o, s); }
template <>
int getrs_dev_any<CX64>(int64_t n, int64_t nrhs, const CX64* A, int64_t lda, const int* ipiv, CX64* B,
                        int64_t ldb, const slt_options* o, cudaStream_t s)
{ return slt_zgetrs_device('N', n, nrhs, A, lda, ipiv, B, ldb, o, s); }

// Cholesky device entry points and type code (slt_xtranspose) per type.
template <typename T> struct CholDev;
template <> struct CholDev<float> {
    static constexpr int type = 0;
    static int potrf(int64_t n, float* A, int64_t lda, const slt_options* o, cudaStream_t s, int64_t* info)
    { return slt_spotrf_device(n, A, lda, o, s, info); }
    static int potrs(int64_t n, int64_t r, const float* A, int64_t lda, float* B, int64_t ldb, const slt_options* o,
                     cudaStream_t s)
    { return slt_spotrs_device(n, r, A, lda, B, ldb, o, s); }
};
template <> struct CholDev<CX32> {
    static constexpr int type = 2;
    static int potrf(int64_t n, CX32* A, int64_t lda, const slt_options* o, cudaStream_t s, int64_t* info)
    { return slt_cpotrf_device(n, A, lda, o, s, info); }
    static int potrs(int64_t n, int64_t r, const CX32* A, int64_t lda, CX32* B, int64_t ldb, const slt_options* o,
                     cudaStream_t s)
    { return slt_cpotrs_device(n, r, A, lda, B, ldb, o, s); }
};
template <> struct CholDev<CX64> {
    static constexpr int type = 3;
    static int potrf(int64_t n, CX64* A, int64_t lda, const slt_options* o, cudaStream_t s, int64_t* info)
    { return slt_zpotrf_device(n, A, lda, o, s, info); }
    static int potrs(int64_t n, int64_t r, const CX64* A, int64_t lda, CX64* B, int64_t ldb, const slt_options* o,
                     cudaStream_t s)
    { return slt_zpotrs_device(n, r, A, lda, B, ldb, o, s); }
};

// lu_factor (+ lu_solve_using_factor when B is given): A <- LU, pivots
// recorded in P, B <- X.  SLATE skips the solve when info != 0.
template <typename T>
int lu_run(CMat<T>* A, slate_Pivots P, CMat<T>* B, slate_Options h, int64_t* info, char method = 0)
{
    *info = 0;
    if (!A || A->m != A->n) return SLT_ERR_ARG;
    if (B && B->m != A->n) return SLT_ERR_ARG;
    if (!method && !lu_method_ok(h)) return SLT_ERR_NOT_SUPPORTED;
    const int64_t n = A->n;
    cudaStream_t s = cstream();
    if (!s) return SLT_ERR_NO_DEVICE;
    slt_options o = opts_for(h, A->nb);
    if (method) o.method_lu = method;
    View<T> va, vb;
    DevBuf piv;
    TRY(va.open(*A, s));
    if (B) TRY(vb.open(*B, s));
    TRY(piv.alloc(sizeof(int) * size_t(std::max<int64_t>(1, n)), s));
    TRY(getrf_dev_any<T>(n, va.p, va.ld, piv.as<int>(), &o, s, info));
    if (B && *info == 0 && B->n > 0) TRY(getrs_dev_any<T>(n, B->n, va.p, va.ld, piv.as<int>(), vb.p, vb.ld, &o, s));
    std::vector<int> rel(size_t(std::max<int64_t>(1, n)));
    SLT_CUDA_TRY(cudaMemcpyAsync(rel.data(), piv.p, sizeof(int) * rel.size(), cudaMemcpyDeviceToHost, s));
    TRY(va.close(*A, s));
    if (B) TRY(vb.close(*B, s));
    if (P) {
        P->rel.assign(rel.begin(), rel.begin() + n);
        P->nb = A->nb;
        P->n = n;
    }
    return SLT_OK;
}

// Identity pivots in the per-panel form (row r of panel k stays: r - k nb).
void identity_pivots(slate_Pivots_struct& P, int64_t n, int64_t nb)
{
    P.rel.resize(size_t(n));
    for (int64_t r = 0; r < n; ++r) P.rel[size_t(r)] = int(r % nb);
    P.n = n;
    P.nb = nb;
}

template <typename T>
int lu_solve_factored(CMat<T>* A, slate_Pivots P, CMat<T>* B, slate_Options h)
{
    if (!A || !B || !P || A->m != A->n || B->m != A->n || P->n != A->n || P->nb != A->nb) return SLT_ERR_ARG;
    cudaStream_t s = cstream();
    if (!s) return SLT_ERR_NO_DEVICE;
    slt_options o = opts_for(h, A->nb);
    View<T> va, vb;
    DevBuf piv;
    TRY(va.open(*A, s));
    TRY(vb.open(*B, s));
    TRY(piv.alloc(sizeof(int) * size_t(std::max<int64_t>(1, A->n)), s));
    if (A->n > 0)
        SLT_CUDA_TRY(cudaMemcpyAsync(piv.p, P->rel.data(), sizeof(int) * size_t(A->n), cudaMemcpyHostToDevice, s));
    if (A->n > 0 && B->n > 0) TRY(getrs_dev_any<T>(A->n, B->n, va.p, va.ld, piv.as<int>(), vb.p, vb.ld, &o, s));
    TRY(vb.close(*B, s));
    return SLT_OK;
}

// getri on the factors of A (in place, or into Ainv) with the recorded pivots.
int lu_inverse(CMat<double>* A, slate_Pivots P, CMat<double>* Ainv, slate_Options h, int64_t* info)
{
    *info = 0;
    if (!A || !P || A->m != A->n || P->n != A->n || P->nb != A->nb) return SLT_ERR_ARG;
    if (Ainv && (Ainv->m != A->n || Ainv->n != A->n)) return SLT_ERR_ARG;
    const int64_t n = A->n;
    if (n == 0) return SLT_OK;
    cudaStream_t s = cstream();
    if (!s) return SLT_ERR_NO_DEVICE;
    slt_options o = opts_for(h, A->nb);
    CMat<double>* dst = Ainv ? Ainv : A;
    View<double> v;
    DevBuf piv;
    if (Ainv) {
        // the factors into the output's device view
        TRY(v.open(*Ainv, s));
        SLT_CUDA_TRY(cudaMemcpy2DAsync(v.p, size_t(v.ld) * sizeof(double), A->data, size_t(A->ld) * sizeof(double),
                                       size_t(n) * sizeof(double), size_t(n),
                                       A->dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
    }
    else {
        TRY(v.open(*A, s));
    }
    TRY(piv.alloc(sizeof(int) * size_t(n), s));
    SLT_CUDA_TRY(cudaMemcpyAsync(piv.p, P->rel.data(), sizeof(int) * size_t(n), cudaMemcpyHostToDevice, s));
    TRY(slt_dgetri_device(n, v.p, v.ld, piv.as<int>(), &o, s, info));
    return v.close(*dst, s);
}

double lu_rcond(slate_Norm norm, CMat<double>* A, double anorm, slate_Options h, int* st)
{
    *st = SLT_ERR_ARG;
    const char nm = (norm == 'O' || norm == 'o' || norm == '1') ? '1' : (norm == 'I' || norm == 'i') ? 'I' : 0;
    if (!A || A->m != A->n || !nm) return 0.0;
    if (A->n == 0) { *st = SLT_OK; return 1.0; }
    cudaStream_t s = cstream();
    if (!s) { *st = SLT_ERR_NO_DEVICE; return 0.0; }
    slt_options o = opts_for(h, A->nb);
    slate_Pivots_struct P;
    identity_pivots(P, A->n, A->nb);
    View<double> v;
    DevBuf piv;
    double rc = 0.0;
    int r = v.open(*A, s);
    if (!r) r = piv.alloc(sizeof(int) * size_t(A->n), s);
    if (!r) r = slt_from_cuda(cudaMemcpyAsync(piv.p, P.rel.data(), sizeof(int) * size_t(A->n), cudaMemcpyHostToDevice, s));
    if (!r) r = slt_dgecondest_device(nm, A->n, v.p, v.ld, piv.as<int>(), anorm, &rc, &o, s);
    if (!r) r = slt_from_cuda(cudaStreamSynchronize(s));
    *st = r;
    return rc;
}

// Cholesky on a Hermitian handle: the referenced triangle is brought to a
// lower-triangular device array (transposed when uplo = 'U'), the driver
// runs on it, and only the referenced triangle is written back.
enum CholOp { kFactor, kSolve, kSolveFactored, kInverse };

int chol_run(CMat<double>* A, CMat<double>* B, slate_Options h, CholOp op, int64_t* info)
{
    *info = 0;
    const bool needs_b = op == kSolve || op == kSolveFactored;
    if (!A || A->m != A->n || (needs_b && (!B || B->m != A->n))) return SLT_ERR_ARG;
    const int64_t n = A->n;
    if (n == 0) return SLT_OK;
    cudaStream_t s = cstream();
    if (!s) return SLT_ERR_NO_DEVICE;
    slt_options o = opts_for(h, A->nb);
    const bool up = A->uplo == 'U';
    DevBuf L, T2;
    TRY(L.alloc(sizeof(double) * size_t(n) * size_t(n), s));
    SLT_CUDA_TRY(cudaMemcpy2DAsync(L.p, size_t(n) * sizeof(double), A->data, size_t(A->ld) * sizeof(double),
                                   size_t(n) * sizeof(double), size_t(n),
                                   A->dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
    if (up) {
        TRY(T2.alloc(sizeof(double) * size_t(n) * size_t(n), s));
        TRY(slt_dtranspose(n, n, L.as<double>(), n, T2.as<double>(), n, s));
        std::swap(L.p, T2.p);
    }
    View<double> vb;
    if (B) TRY(vb.open(*B, s));
    if (op == kFactor) TRY(slt_dpotrf_device(n, L.as<double>(), n, &o, s, info));
    else if (op == kInverse) TRY(slt_dpotri_device(n, L.as<double>(), n, &o, s, info));
    else if (op == kSolve) TRY(slt_dposv_device(n, B->n, L.as<double>(), n, vb.p, vb.ld, &o, s, info));
    else TRY(slt_dpotrs_device(n, B->n, L.as<double>(), n, vb.p, vb.ld, &o, s));
    if (op != kSolveFactored) {
        const double* src = L.as<double>();
        if (up) {
            TRY(slt_dtranspose(n, n, L.as<double>(), n, T2.as<double>(), n, s));
            src = T2.as<double>();
        }
        if (A->dev) {
            TRY(slt_dcopy_tri(up ? 0 : 1, n, src, n, A->data, A->ld, s));
        }
        else {
            std::vector<double> hbuf(size_t(n) * size_t(n));
            SLT_CUDA_TRY(cudaMemcpyAsync(hbuf.data(), src, sizeof(double) * hbuf.size(), cudaMemcpyDeviceToHost, s));
            SLT_CUDA_TRY(cudaStreamSynchronize(s));
            for (int64_t j = 0; j < n; ++j)
                for (int64_t i = up ? 0 : j; i < (up ? j + 1 : n); ++i)
                    A->data[i + j * A->ld] = hbuf[size_t(i) + size_t(j) * size_t(n)];
        }
    }
    if (B) TRY(vb.close(*B, s));
    SLT_CUDA_TRY(cudaStreamSynchronize(s));
    return SLT_OK;
}

// chol_run for the other precisions (no inverse): the referenced triangle is
// brought to lower storage (conjugate-transposed when uplo = 'U'), factored
// or solved with, and written back to the referenced triangle only.
template <typename T>
int chol_run_any(CMat<T>* A, CMat<T>* B, slate_Options h, CholOp op, int64_t* info)
{
    *info = 0;
    if (op == kInverse) return SLT_ERR_NOT_SUPPORTED;
    const bool needs_b = op == kSolve || op == kSolveFactored;
    if (!A || A->m != A->n || (needs_b && (!B || B->m != A->n))) return SLT_ERR_ARG;
    const int64_t n = A->n;
    if (n == 0) return SLT_OK;
    cudaStream_t s = cstream();
    if (!s) return SLT_ERR_NO_DEVICE;
    slt_options o = opts_for(h, A->nb);
    const bool up = A->uplo == 'U';
    constexpr int ty = CholDev<T>::type;
    DevBuf L, T2;
    TRY(L.alloc(sizeof(T) * size_t(n) * size_t(n), s));
    SLT_CUDA_TRY(cudaMemcpy2DAsync(L.p, size_t(n) * sizeof(T), A->data, size_t(A->ld) * sizeof(T),
                                   size_t(n) * sizeof(T), size_t(n),
                                   A->dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
    if (up) {
        TRY(T2.alloc(sizeof(T) * size_t(n) * size_t(n), s));
        TRY(slt_xtranspose(ty, n, n, L.p, n, T2.p, n, 1, s));
        std::swap(L.p, T2.p);
    }
    View<T> vb;
    if (B) TRY(vb.open(*B, s));
    if (op == kFactor || op == kSolve) TRY(CholDev<T>::potrf(n, L.as<T>(), n, &o, s, info));
    if (needs_b && *info == 0 && B->n > 0) TRY(CholDev<T>::potrs(n, B->n, L.as<T>(), n, vb.p, vb.ld, &o, s));
    if (op != kSolveFactored) {
        const void* src = L.p;
        if (up) {
            TRY(slt_xtranspose(ty, n, n, L.p, n, T2.p, n, 1, s));
            src = T2.p;
        }
        if (A->dev) {
            TRY(slt_xcopy_tri(ty, up ? 1 : 0, n, src, n, A->data, A->ld, s));
        }
        else {
            std::vector<T> hbuf(size_t(n) * size_t(n));
            SLT_CUDA_TRY(cudaMemcpyAsync(hbuf.data(), src, sizeof(T) * hbuf.size(), cudaMemcpyDeviceToHost, s));
            SLT_CUDA_TRY(cudaStreamSynchronize(s));
            for (int64_t j = 0; j < n; ++j)
                for (int64_t i = up ? 0 : j; i < (up ? j + 1 : n); ++i)
                    A->data[i + j * A->ld] = hbuf[size_t(i) + size_t(j) * size_t(n)];
        }
    }
    if (B) TRY(vb.close(*B, s));
    SLT_CUDA_TRY(cudaStreamSynchronize(s));
    return SLT_OK;
}

double chol_rcond(slate_Norm norm, CMat<double>* A, double anorm, slate_Options h, int* st)
{
    *st = SLT_ERR_ARG;
    const char nm = (norm == 'O' || norm == 'o' || norm == '1' || norm == 'I' || norm == 'i') ? '1' : 0;
    if (!A || A->m != A->n || !nm) return 0.0;       // A symmetric: one and infinity norms agree
    const int64_t n = A->n;
    if (n == 0) { *st = SLT_OK; return 1.0; }
    cudaStream_t s = cstream();
    if (!s) { *st = SLT_ERR_NO_DEVICE; return 0.0; }
    slt_options o = opts_for(h, A->nb);
    DevBuf L, T2;
    double rc = 0.0;
    int r = L.alloc(sizeof(double) * size_t(n) * size_t(n), s);
    if (!r) r = slt_from_cuda(cudaMemcpy2DAsync(L.p, size_t(n) * sizeof(double), A->data, size_t(A->ld) * sizeof(double),
                                                size_t(n) * sizeof(double), size_t(n),
                                                A->dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
    if (!r && A->uplo == 'U') {
        r = T2.alloc(sizeof(double) * size_t(n) * size_t(n), s);
        if (!r) r = slt_dtranspose(n, n, L.as<double>(), n, T2.as<double>(), n, s);
        if (!r) std::swap(L.p, T2.p);
    }
    if (!r) r = slt_dpocondest_device('1', n, L.as<double>(), n, anorm, &rc, &o, s);
    if (!r) r = slt_from_cuda(cudaStreamSynchronize(s));
    *st = r;
    return rc;
}

template <typename T>
CMat<T>* make(int64_t m, int64_t n, T* A, int64_t lda, int64_t mb, int64_t nb, int p, int q, char uplo)
{
    if (m < 0 || n < 0 || nb <= 0 || mb != nb || p != 1 || q != 1 || lda < std::max<int64_t>(1, m)) return nullptr;
    if (!A && m > 0 && n > 0) return nullptr;
    return new CMat<T>{m, n, nb, lda, A, device_accessible(A), uplo};
}

} // namespace

extern "C" {

slate_Options slate_Options_create(void) { return new COpts(); }
void slate_Options_destroy(slate_Options opts) { delete static_cast<COpts*>(opts); }
void slate_Options_copy(slate_Options opts1, slate_Options opts2)
{
    if (opts1 && opts2) *static_cast<COpts*>(opts1) = *static_cast<COpts*>(opts2);
}

#define SLT_OPT(Name, Type, field)                                                   \
    void slate_Options_set_##Name(slate_Options opts, Type value)                    \
    { if (opts) static_cast<COpts*>(opts)->field = value; }                          \
    Type slate_Options_get_##Name(slate_Options opts, Type defval)                   \
    { return opts ? static_cast<COpts*>(opts)->field : defval; }

SLT_OPT(ChunkSize, int64_t, chunk)
SLT_OPT(Lookahead, int64_t, o.lookahead)
SLT_OPT(BlockSize, int64_t, o.nb)
SLT_OPT(InnerBlocking, int64_t, o.ib)
SLT_OPT(MaxPanelThreads, int64_t, panel_threads)
SLT_OPT(Tolerance, double, o.tolerance)
SLT_OPT(Target, slate_Target, target)
SLT_OPT(Depth, int64_t, o.depth)
SLT_OPT(MaxIterations, int64_t, o.max_iterations)
SLT_OPT(PivotThreshold, double, o.pivot_threshold)
SLT_OPT(MethodLU, slate_MethodLU, method_lu)
#undef SLT_OPT

void slate_Options_set_HoldLocalWorkspace(slate_Options opts, bool value)
{ if (opts) static_cast<COpts*>(opts)->hold = value; }
bool slate_Options_get_HoldLocalWorkspace(slate_Options opts, bool defval)
{ return opts ? static_cast<COpts*>(opts)->hold : defval; }
void slate_Options_set_UseFallbackSolver(slate_Options opts, bool value)
{ if (opts) static_cast<COpts*>(opts)->o.use_fallback = value ? 1 : 0; }
bool slate_Options_get_UseFallbackSolver(slate_Options opts, bool defval)
{ return opts ? static_cast<COpts*>(opts)->o.use_fallback != 0 : defval; }

slate_Pivots slate_Pivots_create(void) { return new slate_Pivots_struct(); }
void slate_Pivots_destroy(slate_Pivots pivots) { delete pivots; }

slate_Matrix_r64 slate_Matrix_create_fromScaLAPACK_r64(int64_t m, int64_t n, double* A, int64_t lda, int64_t mb,
                                                       int64_t nb, int p, int q, slate_mpi_comm_t)
{ return reinterpret_cast<slate_Matrix_r64>(make<double>(m, n, A, lda, mb, nb, p, q, 'G')); }
slate_Matrix_r32 slate_Matrix_create_fromScaLAPACK_r32(int64_t m, int64_t n, float* A, int64_t lda, int64_t mb,
                                                       int64_t nb, int p, int q, slate_mpi_comm_t)
{ return reinterpret_cast<slate_Matrix_r32>(make<float>(m, n, A, lda, mb, nb, p, q, 'G')); }
void slate_Matrix_destroy_r64(slate_Matrix_r64 A) { delete reinterpret_cast<CMat<double>*>(A); }
void slate_Matrix_destroy_r32(slate_Matrix_r32 A) { delete reinterpret_cast<CMat<float>*>(A); }
int64_t slate_Matrix_m_r64(slate_Matrix_r64 A) { return A ? reinterpret_cast<CMat<double>*>(A)->m : 0; }
int64_t slate_Matrix_n_r64(slate_Matrix_r64 A) { return A ? reinterpret_cast<CMat<double>*>(A)->n : 0; }

slate_HermitianMatrix_r64 slate_HermitianMatrix_create_fromScaLAPACK_r64(slate_Uplo uplo, int64_t n, double* A,
                                                                         int64_t lda, int64_t nb, int p, int q,
                                                                         slate_mpi_comm_t)
{
    const char u = (uplo == 'u' || uplo == 'U') ? 'U' : (uplo == 'l' || uplo == 'L') ? 'L' : 0;
    if (!u) return nullptr;
    return reinterpret_cast<slate_HermitianMatrix_r64>(make<double>(n, n, A, lda, nb, nb, p, q, u));
}
void slate_HermitianMatrix_destroy_r64(slate_HermitianMatrix_r64 A) { delete reinterpret_cast<CMat<double>*>(A); }

void slate_lu_solve_r64(slate_Matrix_r64 A, slate_Matrix_r64 B, slate_Options opts)
{
    int64_t info = 0;
    slate_Pivots_struct P;
    const int rc = lu_run<double>(reinterpret_cast<CMat<double>*>(A), &P, reinterpret_cast<CMat<double>*>(B),
                                  opts, &info);
    finish(rc, info);
}
void slate_lu_factor_r64(slate_Matrix_r64 A, slate_Pivots pivots, slate_Options opts)
{
    int64_t info = 0;
    const int rc = lu_run<double>(reinterpret_cast<CMat<double>*>(A), pivots, nullptr, opts, &info);
    finish(rc, info);
}
void slate_lu_solve_using_factor_r64(slate_Matrix_r64 A, slate_Pivots pivots, slate_Matrix_r64 B,
                                     slate_Options opts)
{
    finish(lu_solve_factored<double>(reinterpret_cast<CMat<double>*>(A), pivots,
                                     reinterpret_cast<CMat<double>*>(B), opts), 0);
}
void slate_lu_solve_r32(slate_Matrix_r32 A, slate_Matrix_r32 B, slate_Options opts)
{
    int64_t info = 0;
    slate_Pivots_struct P;
    const int rc = lu_run<float>(reinterpret_cast<CMat<float>*>(A), &P, reinterpret_cast<CMat<float>*>(B),
                                 opts, &info);
    finish(rc, info);
}
void slate_lu_factor_r32(slate_Matrix_r32 A, slate_Pivots pivots, slate_Options opts)
{
    int64_t info = 0;
    const int rc = lu_run<float>(reinterpret_cast<CMat<float>*>(A), pivots, nullptr, opts, &info);
    finish(rc, info);
}
void slate_lu_solve_using_factor_r32(slate_Matrix_r32 A, slate_Pivots pivots, slate_Matrix_r32 B,
                                     slate_Options opts)
{
    finish(lu_solve_factored<float>(reinterpret_cast<CMat<float>*>(A), pivots,
                                    reinterpret_cast<CMat<float>*>(B), opts), 0);
}

void slate_chol_solve_r64(slate_HermitianMatrix_r64 A, slate_Matrix_r64 B, slate_Options opts)
{
    int64_t info = 0;
    const int rc = chol_run(reinterpret_cast<CMat<double>*>(A), reinterpret_cast<CMat<double>*>(B), opts,
                            kSolve, &info);
    finish(rc, info);
}
void slate_chol_factor_r64(slate_HermitianMatrix_r64 A, slate_Options opts)
{
    int64_t info = 0;
    const int rc = chol_run(reinterpret_cast<CMat<double>*>(A), nullptr, opts, kFactor, &info);
    finish(rc, info);
}
void slate_chol_solve_using_factor_r64(slate_HermitianMatrix_r64 A, slate_Matrix_r64 B, slate_Options opts)
{
    int64_t info = 0;
    const int rc = chol_run(reinterpret_cast<CMat<double>*>(A), reinterpret_cast<CMat<double>*>(B), opts,
                            kSolveFactored, &info);
    finish(rc, info);
}
void slate_chol_inverse_using_factor_r64(slate_HermitianMatrix_r64 A, slate_Options opts)
{
    int64_t info = 0;
    const int rc = chol_run(reinterpret_cast<CMat<double>*>(A), nullptr, opts, kInverse, &info);
    finish(rc, info);
}
double slate_chol_rcondest_using_factor_r64(slate_Norm norm, slate_HermitianMatrix_r64 A, double Anorm,
                                            slate_Options opts)
{
    int st = 0;
    const double r = chol_rcond(norm, reinterpret_cast<CMat<double>*>(A), Anorm, opts, &st);
    finish(st, 0);
    return r;
}

#define SLT_NOPIV(R, T)                                                                                         \
void slate_lu_solve_nopiv_##R(slate_Matrix_##R A, slate_Matrix_##R B, slate_Options opts)                       \
{                                                                                                                \
    int64_t info = 0;                                                                                            \
    slate_Pivots_struct P;                                                                                       \
    const int rc = lu_run<T>(reinterpret_cast<CMat<T>*>(A), &P, reinterpret_cast<CMat<T>*>(B), opts, &info, 'N'); \
    finish(rc, info);                                                                                            \
}                                                                                                                \
void slate_lu_factor_nopiv_##R(slate_Matrix_##R A, slate_Options opts)                                         \
{                                                                                                                \
    int64_t info = 0;                                                                                            \
    const int rc = lu_run<T>(reinterpret_cast<CMat<T>*>(A), nullptr, nullptr, opts, &info, 'N');                \
    finish(rc, info);                                                                                            \
}                                                                                                                \
void slate_lu_solve_using_factor_nopiv_##R(slate_Matrix_##R A, slate_Matrix_##R B, slate_Options opts)         \
{                                                                                                                \
    auto* a = reinterpret_cast<CMat<T>*>(A);                                                                     \
    if (!a) { finish(SLT_ERR_ARG, 0); return; }                                                                  \
    slate_Pivots_struct P;                                                                                       \
    identity_pivots(P, a->n, a->nb);                                                                             \
    finish(lu_solve_factored<T>(a, &P, reinterpret_cast<CMat<T>*>(B), opts), 0);                                \
}
SLT_NOPIV(r64, double)
SLT_NOPIV(r32, float)
#undef SLT_NOPIV

void slate_lu_inverse_using_factor_r64(slate_Matrix_r64 A, slate_Pivots pivots, slate_Options opts)
{
    int64_t info = 0;
    const int rc = lu_inverse(reinterpret_cast<CMat<double>*>(A), pivots, nullptr, opts, &info);
    finish(rc, info);
}
void slate_lu_inverse_using_factor_out_of_place_r64(slate_Matrix_r64 A, slate_Pivots pivots,
                                                    slate_Matrix_r64 A_inverse, slate_Options opts)
{
    int64_t info = 0;
    const int rc = lu_inverse(reinterpret_cast<CMat<double>*>(A), pivots, reinterpret_cast<CMat<double>*>(A_inverse),
                              opts, &info);
    finish(rc, info);
}
double slate_lu_rcondest_using_factor_r64(slate_Norm norm, slate_Matrix_r64 A, double Anorm, slate_Options opts)
{
    int st = 0;
    const double r = lu_rcond(norm, reinterpret_cast<CMat<double>*>(A), Anorm, opts, &st);
    finish(st, 0);
    return r;
}

// ---- complex precisions and single-precision Cholesky (SLATE's c32 / c64 /
// r32 instantiations, src/c_api/wrappers.cc:692-1080)
#define SLT_CMAT(R, T)                                                                                          \
slate_Matrix_##R slate_Matrix_create_fromScaLAPACK_##R(int64_t m, int64_t n, void* A, int64_t lda, int64_t mb, \
                                                       int64_t nb, int p, int q, slate_mpi_comm_t)               \
{ return reinterpret_cast<slate_Matrix_##R>(make<T>(m, n, static_cast<T*>(A), lda, mb, nb, p, q, 'G')); }       \
void slate_Matrix_destroy_##R(slate_Matrix_##R A) { delete reinterpret_cast<CMat<T>*>(A); }                     \
slate_HermitianMatrix_##R slate_HermitianMatrix_create_fromScaLAPACK_##R(slate_Uplo uplo, int64_t n, void* A,   \
                                                                         int64_t lda, int64_t nb, int p, int q,  \
                                                                         slate_mpi_comm_t)                       \
{                                                                                                                \
    const char u = (uplo == 'u' || uplo == 'U') ? 'U' : (uplo == 'l' || uplo == 'L') ? 'L' : 0;                 \
    if (!u) return nullptr;                                                                                      \
    return reinterpret_cast<slate_HermitianMatrix_##R>(make<T>(n, n, static_cast<T*>(A), lda, nb, nb, p, q, u)); \
}                                                                                                                \
void slate_HermitianMatrix_destroy_##R(slate_HermitianMatrix_##R A) { delete reinterpret_cast<CMat<T>*>(A); }
SLT_CMAT(c32, CX32)
SLT_CMAT(c64, CX64)
#undef SLT_CMAT

slate_HermitianMatrix_r32 slate_HermitianMatrix_create_fromScaLAPACK_r32(slate_Uplo uplo, int64_t n, float* A,
                                                                         int64_t lda, int64_t nb, int p, int q,
                                                                         slate_mpi_comm_t)
{
    const char u = (uplo == 'u' || uplo == 'U') ? 'U' : (uplo == 'l' || uplo == 'L') ? 'L' : 0;
    if (!u) return nullptr;
    return reinterpret_cast<slate_HermitianMatrix_r32>(make<float>(n, n, A, lda, nb, nb, p, q, u));
}
void slate_HermitianMatrix_destroy_r32(slate_HermitianMatrix_r32 A) { delete reinterpret_cast<CMat<float>*>(A); }

#define SLT_CLU(R, T)                                                                                           \
void slate_lu_solve_##R(slate_Matrix_##R A, slate_Matrix_##R B, slate_Options opts)                             \
{                                                                                                                \
    int64_t info = 0;                                                                                            \
    slate_Pivots_struct P;                                                                                       \
    const int rc = lu_run<T>(reinterpret_cast<CMat<T>*>(A), &P, reinterpret_cast<CMat<T>*>(B), opts, &info);    \
    finish(rc, info);                                                                                            \
}                                                                                                                \
void slate_lu_factor_##R(slate_Matrix_##R A, slate_Pivots pivots, slate_Options opts)                           \
{                                                                                                                \
    int64_t info = 0;                                                                                            \
    const int rc = lu_run<T>(reinterpret_cast<CMat<T>*>(A), pivots, nullptr, opts, &info);                       \
    finish(rc, info);                                                                                            \
}                                                                                                                \
void slate_lu_solve_using_factor_##R(slate_Matrix_##R A, slate_Pivots pivots, slate_Matrix_##R B,               \
                                     slate_Options opts)                                                         \
{ finish(lu_solve_factored<T>(reinterpret_cast<CMat<T>*>(A), pivots, reinterpret_cast<CMat<T>*>(B), opts), 0); }
SLT_CLU(c32, CX32)
SLT_CLU(c64, CX64)
#undef SLT_CLU

#define SLT_CCHOL(R, T)                                                                                         \
void slate_chol_solve_##R(slate_HermitianMatrix_##R A, slate_Matrix_##R B, slate_Options opts)                  \
{                                                                                                                \
    int64_t info = 0;                                                                                            \
    const int rc = chol_run_any<T>(reinterpret_cast<CMat<T>*>(A), reinterpret_cast<CMat<T>*>(B), opts, kSolve, &info); \
    finish(rc, info);                                                                                            \
}                                                                                                                \
void slate_chol_factor_##R(slate_HermitianMatrix_##R A, slate_Options opts)                                     \
{                                                                                                                \
    int64_t info = 0;                                                                                            \
    const int rc = chol_run_any<T>(reinterpret_cast<CMat<T>*>(A), nullptr, opts, kFactor, &info);               \
    finish(rc, info);                                                                                            \
}                                                                                                                \
void slate_chol_solve_using_factor_##R(slate_HermitianMatrix_##R A, slate_Matrix_##R B, slate_Options opts)     \
{                                                                                                                \
    int64_t info = 0;                                                                                            \
    const int rc = chol_run_any<T>(reinterpret_cast<CMat<T>*>(A), reinterpret_cast<CMat<T>*>(B), opts,           \
                                   kSolveFactored, &info);                                                       \
    finish(rc, info);                                                                                            \
}
SLT_CCHOL(r32, float)
SLT_CCHOL(c32, CX32)
SLT_CCHOL(c64, CX64)
#undef SLT_CCHOL

int64_t slate_gb300_last_info(void) { return g_info; }
int slate_gb300_last_status(void) { return g_status; }

} // extern "C"

// ---- small helpers for the header-only C++ API (include/slate_gb300.hh): the
// per-panel pivot arrays live in device memory and the header stays free of
// CUDA includes.
extern "C" {

int slt_ipiv_alloc(int64_t n, int** d)
{
    if (!d || n < 0) return SLT_ERR_ARG;
    return slt_from_cuda(cudaMalloc(reinterpret_cast<void**>(d), sizeof(int) * size_t(n > 0 ? n : 1)));
}
int slt_ipiv_free(int* d) { return d ? slt_from_cuda(cudaFree(d)) : SLT_OK; }
int slt_ipiv_download(const int* d, int64_t n, int* h)
{
    if (n <= 0) return SLT_OK;
    return slt_from_cuda(cudaMemcpy(h, d, sizeof(int) * size_t(n), cudaMemcpyDeviceToHost));
}
int slt_ipiv_upload(const int* h, int64_t n, int* d)
{
    if (n <= 0) return SLT_OK;
    return slt_from_cuda(cudaMemcpy(d, h, sizeof(int) * size_t(n), cudaMemcpyHostToDevice));
}

}  // extern "C"
