// scalapack.cc -- ScaLAPACK-compatible entry points on a 1 x 1 process grid
// (include/slate_scalapack.h).
//
// SLATE's scalapack_api/ (scalapack_gesv.cc, scalapack_gesv_mixed.cc,
// scalapack_getrf.cc, scalapack_getrs.cc, scalapack_posv.cc,
// scalapack_potrf.cc, scalapack_potrs.cc, scalapack_getri.cc,
// scalapack_potri.cc, scalapack_gecon.cc, scalapack_pocon.cc) wraps the
// caller's block-cyclic local arrays in a SLATE matrix with MB x NB tiles
// (scalapack_gesv.cc:93-99) and runs the driver.  With one process the local
// array is the whole matrix -- element (i, j) of the global matrix at
// a[(i - 1) + (j - 1) LLD] -- so the submatrix starting at (ia, ja) is handed
// to the LAPACK-compatible entry points with the tile size nb = MB and the
// inner blocking SLATE_SCALAPACK_IB (default 16, as scalapack_slate.hh).
// No BLACS is linked: the descriptor's context is not queried, and the
// descriptor must describe a 1 x 1 grid (type 1, RSRC = CSRC = 0,
// LLD >= max(1, M)); anything else is reported as ScaLAPACK reports a bad
// descriptor entry, info = -(100 * argument + entry).
//
// Pivots follow ScaLAPACK: IPIV(ia - 1 + r) is the global row that row
// ia - 1 + r was interchanged with, which for ia = 1 is LAPACK's ipiv (SLATE's
// wrapper fills the first n entries, scalapack_gesv.cc:126-145).  info is the
// driver's (SLATE's pdgesv_ wrapper always returns 0, scalapack_gesv.cc:148).

#include "drivers.h"
#include "lapack_opts.h"
#include "slate_scalapack.h"

#include <algorithm>
#include <cstdlib>
#include <type_traits>
#include <vector>

extern "C" int slt_dtranspose(int64_t m, int64_t n, const double* A, int64_t lda, double* B, int64_t ldb,
                              cudaStream_t stream);

using namespace slt;

namespace {

enum { DTYPE = 0, CTXT, M_, N_, MB_, NB_, RSRC, CSRC, LLD };

// 0, or -(100 * argpos + entry) for the first bad descriptor entry, or
// -(argpos - 2) / -(argpos - 1) when the submatrix starting at (i0, j0) of
// size m x n does not fit (the row and column offsets precede the descriptor).
int check_desc(const int* d, int argpos, int i0, int j0, int m, int n)
{
    if (!d || d[DTYPE] != 1) return -(100 * argpos + 1);
    if (d[M_] < 0) return -(100 * argpos + 3);
    if (d[N_] < 0) return -(100 * argpos + 4);
    if (d[MB_] < 1) return -(100 * argpos + 5);
    if (d[NB_] < 1) return -(100 * argpos + 6);
    if (d[RSRC] != 0) return -(100 * argpos + 7);
    if (d[CSRC] != 0) return -(100 * argpos + 8);
    if (d[LLD] < std::max(1, d[M_])) return -(100 * argpos + 9);
    if (i0 < 1 || int64_t(i0) - 1 + m > d[M_]) return -(argpos - 2);
    if (j0 < 1 || int64_t(j0) - 1 + n > d[N_]) return -(argpos - 1);
    return 0;
}

template <typename T>
T* sub(T* a, int i0, int j0, const int* d)
{
    return a + (int64_t(i0) - 1) + (int64_t(j0) - 1) * d[LLD];
}

int env_int(const char* name, int dflt)
{
    const char* v = std::getenv(name);
    if (!v) return dflt;
    const long x = std::strtol(v, nullptr, 0);
    return x > 0 ? int(x) : dflt;
}

// Options of one ScaLAPACK call: the LAPACK entry points' defaults with the
// descriptor's MB as nb, SLATE_SCALAPACK_IB and SLATE_SCALAPACK_LOOKAHEAD.
struct ScalapackScope {
    slt_options o;
    LapackOptsScope scope;
    static slt_options make(const int* desc)
    {
        slt_options r = lapack_opts();
        r.nb = desc[MB_];
        r.ib = std::min<int64_t>(env_int("SLATE_SCALAPACK_IB", 16), r.nb);
        r.lookahead = env_int("SLATE_SCALAPACK_LOOKAHEAD", int(r.lookahead));
        return r;
    }
    explicit ScalapackScope(const int* desc) : o(make(desc)), scope(o) {}
};

// LAPACK ipiv of the n x n submatrix <-> ScaLAPACK IPIV entries ia - 1 ...
void ipiv_out(const std::vector<int>& lp, int n, int ia, int* ipiv)
{
    for (int r = 0; r < n; ++r) ipiv[ia - 1 + r] = lp[size_t(r)] + ia - 1;
}

std::vector<int> ipiv_in(const int* ipiv, int n, int ia)
{
    std::vector<int> lp(static_cast<size_t>(std::max(n, 1)));
    for (int r = 0; r < n; ++r) lp[size_t(r)] = ipiv[ia - 1 + r] - (ia - 1);
    return lp;
}

template <typename T>
void pgesv(int n, int nrhs, T* a, int ia, int ja, const int* desca, int* ipiv, T* b, int ib, int jb,
           const int* descb, int* info)
{
    *info = 0;
    if (n < 0) { *info = -1; return; }
    if (nrhs < 0) { *info = -2; return; }
    if ((*info = check_desc(desca, 6, ia, ja, n, n))) return;
    if ((*info = check_desc(descb, 11, ib, jb, n, nrhs))) return;
    if (n == 0) return;
    ScalapackScope sc(desca);
    int lda = desca[LLD], ldb = descb[LLD];
    std::vector<int> lp(static_cast<size_t>(n));
    if constexpr (std::is_same<T, double>::value)
        slate_dgesv(&n, &nrhs, sub(a, ia, ja, desca), &lda, lp.data(), sub(b, ib, jb, descb), &ldb, info);
    else
        slate_sgesv(&n, &nrhs, sub(a, ia, ja, desca), &lda, lp.data(), sub(b, ib, jb, descb), &ldb, info);
    if (*info >= 0) ipiv_out(lp, n, ia, ipiv);
}

template <typename T>
void pgetrf(int m, int n, T* a, int ia, int ja, const int* desca, int* ipiv, int* info)
{
    *info = 0;
    if (m < 0) { *info = -1; return; }
    if (n < 0) { *info = -2; return; }
    if ((*info = check_desc(desca, 6, ia, ja, m, n))) return;
    if (m == 0 || n == 0) return;
    ScalapackScope sc(desca);
    int lda = desca[LLD];
    const int mn = std::min(m, n);
    std::vector<int> lp(static_cast<size_t>(mn));
    if constexpr (std::is_same<T, double>::value)
        slate_dgetrf(&m, &n, sub(a, ia, ja, desca), &lda, lp.data(), info);
    else
        slate_sgetrf(&m, &n, sub(a, ia, ja, desca), &lda, lp.data(), info);
    if (*info >= 0) ipiv_out(lp, mn, ia, ipiv);
}

// B = A^{-1} B with A's Cholesky factor in the uplo triangle (LAPACK dpotrs):
// an upper factor U (A = U^T U) is transposed on the device to L = U^T.
void potrs_host(char uplo, int n, int nrhs, const double* a, int lda, double* b, int ldb, int* info)
{
    cudaStream_t s = nullptr;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) { *info = -100; return; }
    int rc = SLT_OK;
    {
        const slt_options o = lapack_opts();
        DevBuf dA, dT, dB;
        rc = dA.alloc(sizeof(double) * size_t(n) * size_t(n), s);
        if (!rc) rc = dB.alloc(sizeof(double) * size_t(n) * size_t(std::max(nrhs, 1)), s);
        if (!rc) rc = slt_from_cuda(cudaMemcpy2DAsync(dA.p, sizeof(double) * size_t(n), a, sizeof(double) * size_t(lda),
                                                      sizeof(double) * size_t(n), size_t(n), cudaMemcpyHostToDevice, s));
        if (!rc && nrhs > 0)
            rc = slt_from_cuda(cudaMemcpy2DAsync(dB.p, sizeof(double) * size_t(n), b, sizeof(double) * size_t(ldb),
                                                 sizeof(double) * size_t(n), size_t(nrhs), cudaMemcpyHostToDevice, s));
        if (!rc && (uplo == 'U' || uplo == 'u')) {
            rc = dT.alloc(sizeof(double) * size_t(n) * size_t(n), s);
            if (!rc) rc = slt_dtranspose(n, n, dA.as<double>(), n, dT.as<double>(), n, s);
            if (!rc) std::swap(dA.p, dT.p);
        }
        if (!rc) rc = slt_dpotrs_device(n, nrhs, dA.as<double>(), n, dB.as<double>(), n, &o, s);
        if (!rc && nrhs > 0)
            rc = slt_from_cuda(cudaMemcpy2DAsync(b, sizeof(double) * size_t(ldb), dB.p, sizeof(double) * size_t(n),
                                                 sizeof(double) * size_t(n), size_t(nrhs), cudaMemcpyDeviceToHost, s));
        if (!rc) rc = slt_from_cuda(cudaStreamSynchronize(s));
    }
    cudaStreamDestroy(s);
    *info = rc ? (rc == SLT_ERR_NOMEM ? -100 : -1000 + rc) : 0;
}

bool uplo_ok(const char* uplo) { return uplo && (*uplo == 'L' || *uplo == 'l' || *uplo == 'U' || *uplo == 'u'); }

} // namespace

extern "C" {

// ---- gesv
void pdgesv_(const int* n, const int* nrhs, double* a, const int* ia, const int* ja, const int* desca, int* ipiv,
             double* b, const int* ib, const int* jb, const int* descb, int* info)
{ pgesv<double>(*n, *nrhs, a, *ia, *ja, desca, ipiv, b, *ib, *jb, descb, info); }
void pdgesv(const int* n, const int* nrhs, double* a, const int* ia, const int* ja, const int* desca, int* ipiv,
            double* b, const int* ib, const int* jb, const int* descb, int* info)
{ pgesv<double>(*n, *nrhs, a, *ia, *ja, desca, ipiv, b, *ib, *jb, descb, info); }
void psgesv_(const int* n, const int* nrhs, float* a, const int* ia, const int* ja, const int* desca, int* ipiv,
             float* b, const int* ib, const int* jb, const int* descb, int* info)
{ pgesv<float>(*n, *nrhs, a, *ia, *ja, desca, ipiv, b, *ib, *jb, descb, info); }
void psgesv(const int* n, const int* nrhs, float* a, const int* ia, const int* ja, const int* desca, int* ipiv,
            float* b, const int* ib, const int* jb, const int* descb, int* info)
{ pgesv<float>(*n, *nrhs, a, *ia, *ja, desca, ipiv, b, *ib, *jb, descb, info); }

// ---- getrf
void pdgetrf_(const int* m, const int* n, double* a, const int* ia, const int* ja, const int* desca, int* ipiv,
              int* info)
{ pgetrf<double>(*m, *n, a, *ia, *ja, desca, ipiv, info); }
void pdgetrf(const int* m, const int* n, double* a, const int* ia, const int* ja, const int* desca, int* ipiv,
             int* info)
{ pgetrf<double>(*m, *n, a, *ia, *ja, desca, ipiv, info); }
void psgetrf_(const int* m, const int* n, float* a, const int* ia, const int* ja, const int* desca, int* ipiv,
              int* info)
{ pgetrf<float>(*m, *n, a, *ia, *ja, desca, ipiv, info); }
void psgetrf(const int* m, const int* n, float* a, const int* ia, const int* ja, const int* desca, int* ipiv,
             int* info)
{ pgetrf<float>(*m, *n, a, *ia, *ja, desca, ipiv, info); }

// ---- getrs
static void pdgetrs_impl(const char* trans, int n, int nrhs, double* a, int ia, int ja, const int* desca,
                         const int* ipiv, double* b, int ib, int jb, const int* descb, int* info)
{
    *info = 0;
    if (!trans || (*trans != 'N' && *trans != 'n' && *trans != 'T' && *trans != 't' && *trans != 'C' &&
                   *trans != 'c')) { *info = -1; return; }
    if (n < 0) { *info = -2; return; }
    if (nrhs < 0) { *info = -3; return; }
    if ((*info = check_desc(desca, 7, ia, ja, n, n))) return;
    if ((*info = check_desc(descb, 12, ib, jb, n, nrhs))) return;
    if (n == 0 || nrhs == 0) return;
    ScalapackScope sc(desca);
    int lda = desca[LLD], ldb = descb[LLD];
    std::vector<int> lp = ipiv_in(ipiv, n, ia);
    slate_dgetrs(trans, &n, &nrhs, sub(a, ia, ja, desca), &lda, lp.data(), sub(b, ib, jb, descb), &ldb, info);
}
void pdgetrs_(const char* trans, const int* n, const int* nrhs, double* a, const int* ia, const int* ja,
              const int* desca, int* ipiv, double* b, const int* ib, const int* jb, const int* descb, int* info)
{ pdgetrs_impl(trans, *n, *nrhs, a, *ia, *ja, desca, ipiv, b, *ib, *jb, descb, info); }
void pdgetrs(const char* trans, const int* n, const int* nrhs, double* a, const int* ia, const int* ja,
             const int* desca, int* ipiv, double* b, const int* ib, const int* jb, const int* descb, int* info)
{ pdgetrs_impl(trans, *n, *nrhs, a, *ia, *ja, desca, ipiv, b, *ib, *jb, descb, info); }

// ---- gesv_mixed
static void pdsgesv_impl(int n, int nrhs, double* a, int ia, int ja, const int* desca, int* ipiv, double* b, int ib,
                         int jb, const int* descb, double* x, int ix, int jx, const int* descx, int* iter, int* info)
{
    *info = 0;
    *iter = 0;
    if (n < 0) { *info = -1; return; }
    if (nrhs < 0) { *info = -2; return; }
    if ((*info = check_desc(desca, 6, ia, ja, n, n))) return;
    if ((*info = check_desc(descb, 11, ib, jb, n, nrhs))) return;
    if ((*info = check_desc(descx, 15, ix, jx, n, nrhs))) return;
    if (n == 0) return;
    ScalapackScope sc(desca);
    int lda = desca[LLD], ldb = descb[LLD], ldx = descx[LLD];
    std::vector<int> lp(static_cast<size_t>(n));
    slate_dsgesv(&n, &nrhs, sub(a, ia, ja, desca), &lda, lp.data(), sub(b, ib, jb, descb), &ldb,
                 sub(x, ix, jx, descx), &ldx, nullptr, nullptr, iter, info);
    if (*info >= 0) ipiv_out(lp, n, ia, ipiv);
}
void pdsgesv_(const int* n, const int* nrhs, double* a, const int* ia, const int* ja, const int* desca, int* ipiv,
              double* b, const int* ib, const int* jb, const int* descb, double* x, const int* ix, const int* jx,
              const int* descx, int* iter, int* info)
{ pdsgesv_impl(*n, *nrhs, a, *ia, *ja, desca, ipiv, b, *ib, *jb, descb, x, *ix, *jx, descx, iter, info); }
void pdsgesv(const int* n, const int* nrhs, double* a, const int* ia, const int* ja, const int* desca, int* ipiv,
             double* b, const int* ib, const int* jb, const int* descb, double* x, const int* ix, const int* jx,
             const int* descx, int* iter, int* info)
{ pdsgesv_impl(*n, *nrhs, a, *ia, *ja, desca, ipiv, b, *ib, *jb, descb, x, *ix, *jx, descx, iter, info); }

// ---- posv / potrf / potrs
static void pdposv_impl(const char* uplo, int n, int nrhs, double* a, int ia, int ja, const int* desca, double* b,
                        int ib, int jb, const int* descb, int* info)
{
    *info = 0;
    if (!uplo_ok(uplo)) { *info = -1; return; }
    if (n < 0) { *info = -2; return; }
    if (nrhs < 0) { *info = -3; return; }
    if ((*info = check_desc(desca, 7, ia, ja, n, n))) return;
    if ((*info = check_desc(descb, 11, ib, jb, n, nrhs))) return;
    if (n == 0) return;
    ScalapackScope sc(desca);
    int lda = desca[LLD], ldb = descb[LLD];
    slate_dposv(uplo, &n, &nrhs, sub(a, ia, ja, desca), &lda, sub(b, ib, jb, descb), &ldb, info);
}
void pdposv_(const char* uplo, const int* n, const int* nrhs, double* a, const int* ia, const int* ja,
             const int* desca, double* b, const int* ib, const int* jb, const int* descb, int* info)
{ pdposv_impl(uplo, *n, *nrhs, a, *ia, *ja, desca, b, *ib, *jb, descb, info); }
void pdposv(const char* uplo, const int* n, const int* nrhs, double* a, const int* ia, const int* ja,
            const int* desca, double* b, const int* ib, const int* jb, const int* descb, int* info)
{ pdposv_impl(uplo, *n, *nrhs, a, *ia, *ja, desca, b, *ib, *jb, descb, info); }

static void pdpotrf_impl(const char* uplo, int n, double* a, int ia, int ja, const int* desca, int* info)
{
    *info = 0;
    if (!uplo_ok(uplo)) { *info = -1; return; }
    if (n < 0) { *info = -2; return; }
    if ((*info = check_desc(desca, 6, ia, ja, n, n))) return;
    if (n == 0) return;
    ScalapackScope sc(desca);
    int lda = desca[LLD];
    slate_dpotrf(uplo, &n, sub(a, ia, ja, desca), &lda, info);
}
void pdpotrf_(const char* uplo, const int* n, double* a, const int* ia, const int* ja, const int* desca, int* info)
{ pdpotrf_impl(uplo, *n, a, *ia, *ja, desca, info); }
void pdpotrf(const char* uplo, const int* n, double* a, const int* ia, const int* ja, const int* desca, int* info)
{ pdpotrf_impl(uplo, *n, a, *ia, *ja, desca, info); }

static void pdpotrs_impl(const char* uplo, int n, int nrhs, double* a, int ia, int ja, const int* desca, double* b,
                         int ib, int jb, const int* descb, int* info)
{
    *info = 0;
    if (!uplo_ok(uplo)) { *info = -1; return; }
    if (n < 0) { *info = -2; return; }
    if (nrhs < 0) { *info = -3; return; }
    if ((*info = check_desc(desca, 7, ia, ja, n, n))) return;
    if ((*info = check_desc(descb, 11, ib, jb, n, nrhs))) return;
    if (n == 0 || nrhs == 0) return;
    ScalapackScope sc(desca);
    potrs_host(*uplo, n, nrhs, sub(a, ia, ja, desca), desca[LLD], sub(b, ib, jb, descb), descb[LLD], info);
}
void pdpotrs_(const char* uplo, const int* n, const int* nrhs, double* a, const int* ia, const int* ja,
              const int* desca, double* b, const int* ib, const int* jb, const int* descb, int* info)
{ pdpotrs_impl(uplo, *n, *nrhs, a, *ia, *ja, desca, b, *ib, *jb, descb, info); }
void pdpotrs(const char* uplo, const int* n, const int* nrhs, double* a, const int* ia, const int* ja,
             const int* desca, double* b, const int* ib, const int* jb, const int* descb, int* info)
{ pdpotrs_impl(uplo, *n, *nrhs, a, *ia, *ja, desca, b, *ib, *jb, descb, info); }

// ---- getri / potri: no host workspace is needed; a query (lwork or liwork
// = -1) returns 1 for both sizes.
static void pdgetri_impl(int n, double* a, int ia, int ja, const int* desca, const int* ipiv, double* work,
                         const int* lwork, int* iwork, const int* liwork, int* info)
{
    *info = 0;
    if (n < 0) { *info = -1; return; }
    if ((*info = check_desc(desca, 5, ia, ja, n, n))) return;
    if ((lwork && *lwork == -1) || (liwork && *liwork == -1)) {
        if (work) work[0] = 1.0;
        if (iwork) iwork[0] = 1;
        return;
    }
    if (n == 0) return;
    ScalapackScope sc(desca);
    int lda = desca[LLD];
    std::vector<int> lp = ipiv_in(ipiv, n, ia);
    slate_dgetri(&n, sub(a, ia, ja, desca), &lda, lp.data(), nullptr, nullptr, info);
}
void pdgetri_(const int* n, double* a, const int* ia, const int* ja, const int* desca, int* ipiv, double* work,
              const int* lwork, int* iwork, const int* liwork, int* info)
{ pdgetri_impl(*n, a, *ia, *ja, desca, ipiv, work, lwork, iwork, liwork, info); }
void pdgetri(const int* n, double* a, const int* ia, const int* ja, const int* desca, int* ipiv, double* work,
             const int* lwork, int* iwork, const int* liwork, int* info)
{ pdgetri_impl(*n, a, *ia, *ja, desca, ipiv, work, lwork, iwork, liwork, info); }

static void pdpotri_impl(const char* uplo, int n, double* a, int ia, int ja, const int* desca, int* info)
{
    *info = 0;
    if (!uplo_ok(uplo)) { *info = -1; return; }
    if (n < 0) { *info = -2; return; }
    if ((*info = check_desc(desca, 6, ia, ja, n, n))) return;
    if (n == 0) return;
    ScalapackScope sc(desca);
    int lda = desca[LLD];
    slate_dpotri(uplo, &n, sub(a, ia, ja, desca), &lda, info);
}
void pdpotri_(const char* uplo, const int* n, double* a, const int* ia, const int* ja, const int* desca, int* info)
{ pdpotri_impl(uplo, *n, a, *ia, *ja, desca, info); }
void pdpotri(const char* uplo, const int* n, double* a, const int* ia, const int* ja, const int* desca, int* info)
{ pdpotri_impl(uplo, *n, a, *ia, *ja, desca, info); }

// ---- gecon / pocon (from the factors, as ScaLAPACK's pdgecon / pdpocon)
static void pcon_impl(bool chol, const char* c, int n, double* a, int ia, int ja, const int* desca,
                      const double* anorm, double* rcond, double* work, const int* lwork, int* iwork,
                      const int* liwork, int* info)
{
    *info = 0;
    if (n < 0) { *info = -2; return; }
    if ((*info = check_desc(desca, 6, ia, ja, n, n))) return;
    if ((lwork && *lwork == -1) || (liwork && *liwork == -1)) {
        if (work) work[0] = 1.0;
        if (iwork) iwork[0] = 1;
        return;
    }
    ScalapackScope sc(desca);
    int lda = desca[LLD];
    double an = *anorm;
    if (chol) slate_dpocon(c, &n, sub(a, ia, ja, desca), &lda, &an, rcond, nullptr, nullptr, info);
    else slate_dgecon(c, &n, sub(a, ia, ja, desca), &lda, &an, rcond, nullptr, nullptr, info);
}
void pdgecon_(const char* norm, const int* n, double* a, const int* ia, const int* ja, const int* desca,
              const double* anorm, double* rcond, double* work, const int* lwork, int* iwork, const int* liwork,
              int* info)
{ pcon_impl(false, norm, *n, a, *ia, *ja, desca, anorm, rcond, work, lwork, iwork, liwork, info); }
void pdgecon(const char* norm, const int* n, double* a, const int* ia, const int* ja, const int* desca,
             const double* anorm, double* rcond, double* work, const int* lwork, int* iwork, const int* liwork,
             int* info)
{ pcon_impl(false, norm, *n, a, *ia, *ja, desca, anorm, rcond, work, lwork, iwork, liwork, info); }
void pdpocon_(const char* uplo, const int* n, double* a, const int* ia, const int* ja, const int* desca,
              const double* anorm, double* rcond, double* work, const int* lwork, int* iwork, const int* liwork,
              int* info)
{ pcon_impl(true, uplo, *n, a, *ia, *ja, desca, anorm, rcond, work, lwork, iwork, liwork, info); }
void pdpocon(const char* uplo, const int* n, double* a, const int* ia, const int* ja, const int* desca,
             const double* anorm, double* rcond, double* work, const int* lwork, int* iwork, const int* liwork,
             int* info)
{ pcon_impl(true, uplo, *n, a, *ia, *ja, desca, anorm, rcond, work, lwork, iwork, liwork, info); }

} // extern "C"
