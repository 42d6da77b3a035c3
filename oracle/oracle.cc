// oracle.cc -- CPU restatement of SLATE's single-node LU / Cholesky solve path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU library: the
// test suite, the package smoke check and the CPU-baseline leg of the benchmark
// call it to produce expected results.  No product code path links or calls it.
//
// Every routine restates the algorithm of the SLATE source it cites (paths are
// relative to the SLATE source tree, release 2025.05.28).  Results are identical
// to SLATE's HostTask target in exact arithmetic; rounding differs only through
// the summation order of the tile BLAS calls, which SLATE delegates to an
// unpinned host BLAS.
//
// Layout: all matrices are column-major with a leading dimension, viewed as a
// grid of nb x nb tiles (the last tile row/column may be ragged), which is the
// tile layout Matrix::fromLAPACK gives (include/slate/Matrix.hh:57-69).
//
// Parity pins:
//   * the Philox generator is checked bit-for-bit against SLATE's own
//     matgen/random.cc (compiled from source by oracle/build_ref.sh), and
//   * the deterministic generators against test/ref/*.txt golden files.
//   * LU/Cholesky/solve results have no golden vectors in SLATE; they are
//     cross-checked against LAPACK (scipy) in the tests.

#include <algorithm>
#include <cmath>
#include <cfloat>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

//==============================================================================
// Philox-2x64-10 counter RNG, restating matgen/random.cc:18-88.
// SLATE's variant multiplies the second state word by 0x9E3779B97F4A7C15 and
// bumps the key by 0xD2B74407B1CE6E93 each round (random.cc:53-75).
inline void philox2x64(uint64_t s0, uint64_t s1, uint64_t key, uint64_t out[2])
{
    const uint64_t key_bump = 0xD2B74407B1CE6E93ull;
    const uint64_t mult = 0x9E3779B97F4A7C15ull;
    for (int r = 0; r < 10; ++r) {
        if (r > 0) key += key_bump;
        unsigned __int128 p = (unsigned __int128) s1 * mult;
        uint64_t lo = (uint64_t) p;
        uint64_t hi = (uint64_t) (p >> 64);
        uint64_t n0 = lo;
        uint64_t n1 = hi ^ key ^ s0;
        s0 = n0;
        s1 = n1;
    }
    out[0] = s0;
    out[1] = s1;
}

// random.cc:80-88: top `digits` bits scaled to [0, 1).
template <typename T> inline T bits_to_unit(uint64_t bits)
{
    const int digits = std::numeric_limits<T>::digits;
    return T(bits >> (64 - digits)) / T(uint64_t(1) << digits);
}

// random.cc:91-160 for real types; dist codes as in matgen/random.hh:14-22.
template <typename T> T philox_entry(int dist, int64_t seed, int64_t i, int64_t j)
{
    uint64_t b[2];
    philox2x64(uint64_t(i), uint64_t(j), uint64_t(seed), b);
    T u1 = bits_to_unit<T>(b[0]);
    T u2 = bits_to_unit<T>(b[1]);
    const T pi = T(3.1415926535897932385);
    switch (dist) {
        case 1: return u1;                                    // Uniform [0,1)
        case 2: return 2*u1 - 1;                              // UniformSigned
        case 3: {                                             // Normal (Box-Muller)
            T mag = std::sqrt(-2 * std::log(1 - u1));
            return mag * std::cos(2 * pi * u2);
        }
        case 4: {                                             // UnitDisk
            T mag = std::sqrt(u1);
            return mag * std::cos(2 * pi * u2);
        }
        case 5: return std::cos(2 * pi * u2);                 // UnitCircle
        case 6: return u1 >= T(0.5) ? T(1) : T(0);            // Binary
        case 7: return u1 >= T(0.5) ? T(1) : T(-1);           // BinarySigned
        default: return T(0);
    }
}

template <typename T>
void philox_fill(int dist, int64_t seed, int64_t m, int64_t n,
                 int64_t ioff, int64_t joff, T* A, int64_t lda)
{
    #pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < n; ++j)
        for (int64_t i = 0; i < m; ++i)
            A[i + j*lda] = philox_entry<T>(dist, seed, i + ioff, j + joff);
}

//==============================================================================
// Tile BLAS used by the restated drivers.  SLATE calls BLAS++ on tiles; here a
// host dgemm/sgemm supplied at run time (Fortran ABI) is used when set,
// otherwise a cache-blocked loop nest.
typedef void (*dgemm_f)(const char*, const char*, const int*, const int*, const int*,
                        const double*, const double*, const int*, const double*, const int*,
                        const double*, double*, const int*);
typedef void (*sgemm_f)(const char*, const char*, const int*, const int*, const int*,
                        const float*, const float*, const int*, const float*, const int*,
                        const float*, float*, const int*);
dgemm_f g_dgemm = nullptr;
sgemm_f g_sgemm = nullptr;
typedef void (*dtrsm_f)(const char*, const char*, const char*, const char*, const int*, const int*,
                        const double*, const double*, const int*, double*, const int*);
typedef void (*strsm_f)(const char*, const char*, const char*, const char*, const int*, const int*,
                        const float*, const float*, const int*, float*, const int*);
typedef void (*dpotrf_f)(const char*, const int*, double*, const int*, int*);
typedef void (*spotrf_f)(const char*, const int*, float*, const int*, int*);
dtrsm_f g_dtrsm = nullptr;
strsm_f g_strsm = nullptr;
dpotrf_f g_dpotrf = nullptr;
spotrf_f g_spotrf = nullptr;

// Host BLAS/LAPACK tile calls (the calls SLATE's HostTask makes), when set.
bool host_trsm(char side, char uplo, char trans, char diag, int64_t m, int64_t n, const double* A,
               int64_t lda, double* B, int64_t ldb)
{
    if (!g_dtrsm || m <= 0 || n <= 0) return false;
    int mi = int(m), ni = int(n), la = int(lda), lb = int(ldb);
    double one = 1.0;
    g_dtrsm(&side, &uplo, &trans, &diag, &mi, &ni, &one, A, &la, B, &lb);
    return true;
}
bool host_trsm(char side, char uplo, char trans, char diag, int64_t m, int64_t n, const float* A,
               int64_t lda, float* B, int64_t ldb)
{
    if (!g_strsm || m <= 0 || n <= 0) return false;
    int mi = int(m), ni = int(n), la = int(lda), lb = int(ldb);
    float one = 1.0f;
    g_strsm(&side, &uplo, &trans, &diag, &mi, &ni, &one, A, &la, B, &lb);
    return true;
}
bool host_potrf(int64_t n, double* A, int64_t lda, int64_t* info)
{
    if (!g_dpotrf) return false;
    int ni = int(n), la = int(lda), inf = 0;
    char u = 'L';
    g_dpotrf(&u, &ni, A, &la, &inf);
    *info = inf;
    return true;
}
bool host_potrf(int64_t n, float* A, int64_t lda, int64_t* info)
{
    if (!g_spotrf) return false;
    int ni = int(n), la = int(lda), inf = 0;
    char u = 'L';
    g_spotrf(&u, &ni, A, &la, &inf);
    *info = inf;
    return true;
}

// C = alpha op(A) op(B) + beta C ; ta/tb in {'N','T'}.
template <typename T>
void gemm_loops(char ta, char tb, int64_t m, int64_t n, int64_t k, T alpha,
                const T* A, int64_t lda, const T* B, int64_t ldb,
                T beta, T* C, int64_t ldc)
{
    for (int64_t j = 0; j < n; ++j) {
        T* c = C + j*ldc;
        if (beta == T(0)) for (int64_t i = 0; i < m; ++i) c[i] = 0;
        else if (beta != T(1)) for (int64_t i = 0; i < m; ++i) c[i] *= beta;
    }
    if (m == 0 || n == 0 || k == 0 || alpha == T(0)) return;
    const int64_t KC = 128, MC = 512;
    if (ta == 'N') {
        for (int64_t l0 = 0; l0 < k; l0 += KC) {
            int64_t l1 = std::min(k, l0 + KC);
            for (int64_t i0 = 0; i0 < m; i0 += MC) {
                int64_t i1 = std::min(m, i0 + MC);
                for (int64_t j = 0; j < n; ++j) {
                    T* c = C + j*ldc;
                    for (int64_t l = l0; l < l1; ++l) {
                        T b = alpha * (tb == 'N' ? B[l + j*ldb] : B[j + l*ldb]);
                        const T* a = A + l*lda;
                        for (int64_t i = i0; i < i1; ++i) c[i] += a[i] * b;
                    }
                }
            }
        }
    }
    else {
        for (int64_t j = 0; j < n; ++j) {
            for (int64_t i = 0; i < m; ++i) {
                const T* a = A + i*lda;
                T s = 0;
                if (tb == 'N') {
                    const T* b = B + j*ldb;
                    for (int64_t l = 0; l < k; ++l) s += a[l] * b[l];
                }
                else {
                    for (int64_t l = 0; l < k; ++l) s += a[l] * B[j + l*ldb];
                }
                C[i + j*ldc] += alpha * s;
            }
        }
    }
}

void gemm(char ta, char tb, int64_t m, int64_t n, int64_t k, double alpha,
          const double* A, int64_t lda, const double* B, int64_t ldb,
          double beta, double* C, int64_t ldc)
{
    if (g_dgemm && m > 0 && n > 0) {
        int mi = int(m), ni = int(n), ki = int(k), la = int(std::max<int64_t>(lda, 1)),
            lb = int(std::max<int64_t>(ldb, 1)), lc = int(ldc);
        g_dgemm(&ta, &tb, &mi, &ni, &ki, &alpha, A, &la, B, &lb, &beta, C, &lc);
        return;
    }
    gemm_loops<double>(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}

void gemm(char ta, char tb, int64_t m, int64_t n, int64_t k, float alpha,
          const float* A, int64_t lda, const float* B, int64_t ldb,
          float beta, float* C, int64_t ldc)
{
    if (g_sgemm && m > 0 && n > 0) {
        int mi = int(m), ni = int(n), ki = int(k), la = int(std::max<int64_t>(lda, 1)),
            lb = int(std::max<int64_t>(ldb, 1)), lc = int(ldc);
        g_sgemm(&ta, &tb, &mi, &ni, &ki, &alpha, A, &la, B, &lb, &beta, C, &lc);
        return;
    }
    gemm_loops<float>(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}

// Left-side triangular solve on a tile: op(T) X = B, T m x m.
// uplo 'L'/'U', trans 'N'/'T', diag 'U'/'N'.
template <typename T>
void trsm_left(char uplo, char trans, char diag, int64_t m, int64_t n,
               const T* A, int64_t lda, T* B, int64_t ldb)
{
    if (host_trsm('L', uplo, trans, diag, m, n, A, lda, B, ldb)) return;
    bool lower_eff = (uplo == 'L') == (trans == 'N');
    for (int64_t j = 0; j < n; ++j) {
        T* b = B + j*ldb;
        if (lower_eff) {
            for (int64_t i = 0; i < m; ++i) {
                T s = b[i];
                if (trans == 'N') { for (int64_t l = 0; l < i; ++l) s -= A[i + l*lda] * b[l]; }
                else              { for (int64_t l = 0; l < i; ++l) s -= A[l + i*lda] * b[l]; }
                b[i] = (diag == 'U') ? s : s / A[i + i*lda];
            }
        }
        else {
            for (int64_t i = m - 1; i >= 0; --i) {
                T s = b[i];
                if (trans == 'N') { for (int64_t l = i+1; l < m; ++l) s -= A[i + l*lda] * b[l]; }
                else              { for (int64_t l = i+1; l < m; ++l) s -= A[l + i*lda] * b[l]; }
                b[i] = (diag == 'U') ? s : s / A[i + i*lda];
            }
        }
    }
}

// Right-side solve X L^T = B with L lower non-unit (Cholesky column panel,
// src/potrf.cc:109-120: A(i,k) <- A(i,k) L(k,k)^{-H}).
template <typename T>
void trsm_right_lower_trans(int64_t m, int64_t n, const T* L, int64_t ldl, T* B, int64_t ldb)
{
    if (host_trsm('R', 'L', 'T', 'N', m, n, L, ldl, B, ldb)) return;
    for (int64_t j = 0; j < n; ++j) {
        T d = L[j + j*ldl];
        for (int64_t l = 0; l < j; ++l) {
            T f = L[j + l*ldl];
            const T* bl = B + l*ldb;
            T* bj = B + j*ldb;
            for (int64_t i = 0; i < m; ++i) bj[i] -= bl[i] * f;
        }
        T* bj = B + j*ldb;
        for (int64_t i = 0; i < m; ++i) bj[i] /= d;
    }
}

struct Tiling {
    int64_t m, n, nb;
    int64_t mt() const { return (m + nb - 1) / nb; }
    int64_t nt() const { return (n + nb - 1) / nb; }
    int64_t tileMb(int64_t i) const { return std::min(nb, m - i*nb); }
    int64_t tileNb(int64_t j) const { return std::min(nb, n - j*nb); }
};

//==============================================================================
// LU panel, restating tile::getrf (src/internal/Tile_getrf.hh:159-447) on one
// MPI rank: per column a threaded max search over the panel tiles with
// strict '>' (thread t scans tiles t, t+T, ...; :197-238), a reduction across
// threads in rank order (:244-251), the pivot-threshold rule that keeps the
// diagonal when |diag| >= |max|*threshold (:253-289), a full-width row swap
// (getrf_swap, :52-95), scaling by the reciprocal pivot when |pivot| >=
// safe_min, else by division (:329-366), and a rank-1 update restricted to
// the ib-wide stripe (:369-385).  After each stripe: a unit-lower trsm of the
// top block and a rank-ib gemm update of the rest of the panel (:390-445).
//
// `panel` points at the diagonal element; rows run to the bottom of A.
// Outputs per panel column j: (tile index relative to the panel, offset) and
// the pivot margin |best| / |second best| among the candidates.
template <typename T>
void panel_getrf(int64_t prows, int64_t nbk, int64_t diag_len, int64_t ib,
                 int64_t nb, T* P, int64_t ld, int nthreads, double threshold,
                 int64_t* piv_tile, int64_t* piv_off, double* margin, int64_t* info)
{
    const int64_t ptiles = (prows + nb - 1) / nb;
    auto tmb = [&](int64_t t) { return std::min(nb, prows - t*nb); };
    auto at = [&](int64_t t, int64_t i, int64_t j) -> T& { return P[t*nb + i + j*ld]; };
    int T_ = int(std::min<int64_t>(std::max(nthreads, 1), ptiles));
    std::vector<T> top(size_t(ib) * size_t(std::max<int64_t>(nbk, 1)));
    const T safe_min = std::numeric_limits<T>::min();
    *info = 0;

    for (int64_t k0 = 0; k0 < diag_len; k0 += ib) {
        int64_t kb = std::min(diag_len - k0, ib);
        for (int64_t j = k0; j < k0 + kb; ++j) {
            // thread max search
            std::vector<T> mv(T_);
            std::vector<int64_t> mi(T_), mo(T_);
            for (int t = 0; t < T_; ++t) {
                if (t == 0) { mv[t] = at(0, j, j); mi[t] = 0; mo[t] = j; }
                else        { mv[t] = at(t, 0, j); mi[t] = t; mo[t] = 0; }
                for (int64_t idx = t; idx < ptiles; idx += T_) {
                    int64_t i0 = (idx == 0) ? j + 1 : 0;
                    for (int64_t i = i0; i < tmb(idx); ++i) {
                        if (std::abs(at(idx, i, j)) > std::abs(mv[t])) {
                            mv[t] = at(idx, i, j); mi[t] = idx; mo[t] = i;
                        }
                    }
                }
            }
            for (int t = 1; t < T_; ++t) {
                if (std::abs(mv[t]) > std::abs(mv[0])) {
                    mv[0] = mv[t]; mi[0] = mi[t]; mo[0] = mo[t];
                }
            }
            // threshold rule with the diagonal (single rank)
            if (std::abs(at(0, j, j)) >= std::abs(mv[0]) * T(threshold)) {
                mi[0] = 0; mo[0] = j; mv[0] = at(0, j, j);
            }
            // pivot margin among all candidates below the diagonal
            if (margin) {
                double best = std::abs(double(mv[0])), second = 0;
                int64_t prow = mi[0]*nb + mo[0];
                for (int64_t r = j; r < prows; ++r) {
                    if (r == prow) continue;
                    second = std::max(second, std::abs(double(P[r + j*ld])));
                }
                margin[j] = second > 0 ? best / second : INFINITY;
            }
            piv_tile[j] = mi[0];
            piv_off[j] = mo[0];
            T pval = mv[0];
            // swap the whole panel row
            if (mi[0] > 0 || mo[0] > j) {
                int64_t r = mi[0]*nb + mo[0];
                for (int64_t c = 0; c < nbk; ++c) std::swap(P[j + c*ld], P[r + c*ld]);
            }
            for (int64_t c = j + 1; c < k0 + kb; ++c) top[c - j - 1] = at(0, j, c);
            // column scaling
            #pragma omp parallel for schedule(static) if(ptiles > 4)
            for (int64_t idx = 0; idx < ptiles; ++idx) {
                int64_t i0 = (idx == 0) ? j + 1 : 0;
                int64_t mb_ = tmb(idx);
                if (std::abs(pval) >= safe_min) {
                    T alpha = T(1) / (idx == 0 ? at(0, j, j) : pval);
                    for (int64_t i = i0; i < mb_; ++i) at(idx, i, j) *= alpha;
                }
                else if (pval != T(0)) {
                    T d = (idx == 0 ? at(0, j, j) : pval);
                    for (int64_t i = i0; i < mb_; ++i) at(idx, i, j) /= d;
                }
                // rank-1 update inside the stripe
                for (int64_t c = j + 1; c < k0 + kb; ++c) {
                    T u = top[c - j - 1];
                    for (int64_t i = i0; i < mb_; ++i) at(idx, i, c) -= at(idx, i, j) * u;
                }
            }
            if (pval == T(0) && *info == 0) *info = j + 1;
        }
        if (k0 + kb < nbk) {
            int64_t nr = nbk - k0 - kb;
            trsm_left<T>('L', 'N', 'U', kb, nr, &at(0, k0, k0), ld, &at(0, k0, k0 + kb), ld);
            int64_t rows = prows - (k0 + kb);
            if (rows > 0) {
                // rank-kb update of the rest of the panel, in row chunks
                const int64_t CH = 256;
                int64_t nch = (rows + CH - 1) / CH;
                #pragma omp parallel for schedule(static) if(nch > 1)
                for (int64_t c = 0; c < nch; ++c) {
                    int64_t r0 = k0 + kb + c*CH;
                    int64_t rr = std::min(CH, prows - r0);
                    gemm('N', 'N', rr, nr, kb, T(-1), &P[r0 + k0*ld], ld,
                         &P[k0 + (k0 + kb)*ld], ld, T(1), &P[r0 + (k0 + kb)*ld], ld);
                }
            }
        }
    }
}

// Forward application of one panel's pivots to a block of columns
// (internal::permuteRows, src/internal/internal_swap.cc:198-435):
// sequential interchanges of row j with row (tile*nb + offset), rows relative
// to the panel's first row.
template <typename T>
void apply_pivots(const int64_t* piv_tile, const int64_t* piv_off, int64_t len,
                  int64_t nb, T* P, int64_t ld, int64_t ncols, bool forward)
{
    if (ncols <= 0) return;
    #pragma omp parallel for schedule(static) if(ncols > 64)
    for (int64_t c = 0; c < ncols; ++c) {
        T* col = P + c*ld;
        if (forward) {
            for (int64_t j = 0; j < len; ++j) {
                int64_t r = piv_tile[j]*nb + piv_off[j];
                if (r != j) std::swap(col[j], col[r]);
            }
        }
        else {
            for (int64_t j = len - 1; j >= 0; --j) {
                int64_t r = piv_tile[j]*nb + piv_off[j];
                if (r != j) std::swap(col[j], col[r]);
            }
        }
    }
}

//==============================================================================
// Right-looking tile LU (impl::getrf, src/getrf.cc:22-244).  The lookahead
// task DAG (:81-236) changes only the order in which independent tile updates
// run, never the operations applied to a tile, so the steps are issued in
// program order here with the tile updates of each step run in parallel.
template <typename T>
int64_t getrf(int64_t m, int64_t n, T* A, int64_t lda, int64_t nb, int64_t ib,
              int nthreads, double threshold, int64_t* piv_tile, int64_t* piv_off,
              double* margin)
{
    Tiling t{m, n, nb};
    int64_t info = 0;
    int64_t minmt = std::min(t.mt(), t.nt());
    for (int64_t k = 0; k < minmt; ++k) {
        int64_t r0 = k*nb;
        int64_t nbk = t.tileNb(k);
        int64_t diag_len = std::min(t.tileMb(k), nbk);
        int64_t iinfo = 0;
        panel_getrf<T>(m - r0, nbk, diag_len, ib, nb, A + r0 + r0*lda, lda, nthreads,
                       threshold, piv_tile + r0, piv_off + r0,
                       margin ? margin + r0 : nullptr, &iinfo);
        if (info == 0 && iinfo > 0) info = r0 + iinfo;
        // pivots to the right and to the left (src/getrf.cc:139-173, :175-215)
        int64_t c1 = r0 + nbk;
        apply_pivots<T>(piv_tile + r0, piv_off + r0, diag_len, nb, A + r0 + c1*lda, lda,
                        n - c1, true);
        apply_pivots<T>(piv_tile + r0, piv_off + r0, diag_len, nb, A + r0, lda, r0, true);
        if (c1 < n) {
            // U row: A(k, j) <- L(k,k)^{-1} A(k, j)
            int64_t ntr = t.nt() - k - 1;
            #pragma omp parallel for schedule(static)
            for (int64_t jj = 0; jj < ntr; ++jj) {
                int64_t cj = c1 + jj*nb;
                trsm_left<T>('L', 'N', 'U', diag_len, t.tileNb(k + 1 + jj),
                             A + r0 + r0*lda, lda, A + r0 + cj*lda, lda);
            }
            // trailing update A(i, j) -= A(i, k) A(k, j) tile by tile
            int64_t mtr = t.mt() - k - 1;
            #pragma omp parallel for collapse(2) schedule(dynamic)
            for (int64_t ii = 0; ii < mtr; ++ii) {
                for (int64_t jj = 0; jj < ntr; ++jj) {
                    int64_t ri = (k + 1 + ii)*nb, cj = c1 + jj*nb;
                    gemm('N', 'N', t.tileMb(k + 1 + ii), t.tileNb(k + 1 + jj), nbk, T(-1),
                         A + ri + r0*lda, lda, A + r0 + cj*lda, lda, T(1), A + ri + cj*lda, lda);
                }
            }
        }
    }
    return info;
}

// getrs, NoTrans (src/getrs.cc:66-117): permute B panel by panel, then tile
// forward (unit L) and backward (U) sweeps (work::trsmA,
// src/work/work_trsmA.cc:147-480).
template <typename T>
void getrs(int64_t n, int64_t nrhs, const T* LU, int64_t lda, const int64_t* piv_tile,
           const int64_t* piv_off, int64_t nb, T* B, int64_t ldb)
{
    Tiling t{n, n, nb};
    int64_t mt = t.mt();
    for (int64_t k = 0; k < mt; ++k)
        apply_pivots<T>(piv_tile + k*nb, piv_off + k*nb, t.tileMb(k), nb, B + k*nb, ldb, nrhs, true);
    for (int64_t k = 0; k < mt; ++k) {
        int64_t r0 = k*nb, mb = t.tileMb(k);
        trsm_left<T>('L', 'N', 'U', mb, nrhs, LU + r0 + r0*lda, lda, B + r0, ldb);
        #pragma omp parallel for schedule(static) if(mt - k > 8)
        for (int64_t i = k + 1; i < mt; ++i)
            gemm('N', 'N', t.tileMb(i), nrhs, mb, T(-1), LU + i*nb + r0*lda, lda,
                 B + r0, ldb, T(1), B + i*nb, ldb);
    }
    for (int64_t k = mt - 1; k >= 0; --k) {
        int64_t r0 = k*nb, mb = t.tileMb(k);
        trsm_left<T>('U', 'N', 'N', mb, nrhs, LU + r0 + r0*lda, lda, B + r0, ldb);
        #pragma omp parallel for schedule(static) if(k > 8)
        for (int64_t i = 0; i < k; ++i)
            gemm('N', 'N', t.tileMb(i), nrhs, mb, T(-1), LU + i*nb + r0*lda, lda,
                 B + r0, ldb, T(1), B + i*nb, ldb);
    }
}

// Diagonal-tile Cholesky, lower (tile::potrf -> lapack::potrf,
// src/internal/Tile_lapack.hh:268-285), restated as the dot-product form of
// LAPACK's unblocked potf2.  Returns the 1-based column of a non-positive
// pivot, else 0.
template <typename T>
int64_t potf2_lower(int64_t n, T* A, int64_t lda)
{
    int64_t hinfo = 0;
    if (host_potrf(n, A, lda, &hinfo)) return hinfo;
    for (int64_t j = 0; j < n; ++j) {
        T ajj = A[j + j*lda];
        for (int64_t l = 0; l < j; ++l) ajj -= A[j + l*lda] * A[j + l*lda];
        if (!(ajj > T(0))) { A[j + j*lda] = ajj; return j + 1; }
        ajj = std::sqrt(ajj);
        A[j + j*lda] = ajj;
        for (int64_t i = j + 1; i < n; ++i) {
            T s = A[i + j*lda];
            for (int64_t l = 0; l < j; ++l) s -= A[i + l*lda] * A[j + l*lda];
            A[i + j*lda] = s / ajj;
        }
    }
    return 0;
}

// Right-looking tile Cholesky, lower (impl::potrf, src/potrf.cc:22-210):
// potrf of A(k,k), trsm of the column below it, then herk on diagonal tiles
// and gemm on off-diagonal tiles of the trailing lower triangle.
template <typename T>
int64_t potrf(int64_t n, T* A, int64_t lda, int64_t nb)
{
    Tiling t{n, n, nb};
    int64_t nt = t.nt();
    for (int64_t k = 0; k < nt; ++k) {
        int64_t r0 = k*nb, kb = t.tileNb(k);
        int64_t iinfo = potf2_lower<T>(kb, A + r0 + r0*lda, lda);
        if (iinfo != 0) return r0 + iinfo;
        #pragma omp parallel for schedule(static)
        for (int64_t i = k + 1; i < nt; ++i)
            trsm_right_lower_trans<T>(t.tileMb(i), kb, A + r0 + r0*lda, lda,
                                      A + i*nb + r0*lda, lda);
        #pragma omp parallel for schedule(dynamic)
        for (int64_t p = 0; p < (nt - k - 1)*(nt - k) / 2; ++p) {
            // enumerate lower-triangle tiles (i >= j) of the trailing matrix
            int64_t jj = 0, rem = p, cnt = nt - k - 1;
            while (rem >= cnt) { rem -= cnt; --cnt; ++jj; }
            int64_t j = k + 1 + jj, i = j + rem;
            gemm('N', 'T', t.tileMb(i), t.tileNb(j), kb, T(-1), A + i*nb + r0*lda, lda,
                 A + j*nb + r0*lda, lda, T(1), A + i*nb + j*nb*lda, lda);
        }
    }
    return 0;
}

// potrs (src/potrs.cc:55-78): forward sweep with L, backward with L^T.
template <typename T>
void potrs(int64_t n, int64_t nrhs, const T* L, int64_t lda, int64_t nb, T* B, int64_t ldb)
{
    Tiling t{n, n, nb};
    int64_t mt = t.mt();
    for (int64_t k = 0; k < mt; ++k) {
        int64_t r0 = k*nb, mb = t.tileMb(k);
        trsm_left<T>('L', 'N', 'N', mb, nrhs, L + r0 + r0*lda, lda, B + r0, ldb);
        for (int64_t i = k + 1; i < mt; ++i)
            gemm('N', 'N', t.tileMb(i), nrhs, mb, T(-1), L + i*nb + r0*lda, lda,
                 B + r0, ldb, T(1), B + i*nb, ldb);
    }
    for (int64_t k = mt - 1; k >= 0; --k) {
        int64_t r0 = k*nb, mb = t.tileMb(k);
        trsm_left<T>('L', 'T', 'N', mb, nrhs, L + r0 + r0*lda, lda, B + r0, ldb);
        for (int64_t i = 0; i < k; ++i)
            gemm('T', 'N', t.tileMb(i), nrhs, mb, T(-1), L + r0 + i*nb*lda, lda,
                 B + r0, ldb, T(1), B + i*nb, ldb);
    }
}

//==============================================================================
// Helpers of the mixed-precision drivers.
double norm_inf(int64_t m, int64_t n, const double* A, int64_t lda)
{
    std::vector<double> rs(m, 0.0);
    for (int64_t j = 0; j < n; ++j)
        for (int64_t i = 0; i < m; ++i) rs[i] += std::abs(A[i + j*lda]);
    double r = 0;
    for (double v : rs) r = std::max(r, v);
    return r;
}

double norm_inf_sym_lower(int64_t n, const double* A, int64_t lda)
{
    std::vector<double> rs(n, 0.0);
    for (int64_t j = 0; j < n; ++j)
        for (int64_t i = j; i < n; ++i) {
            double v = std::abs(A[i + j*lda]);
            rs[i] += v;
            if (i != j) rs[j] += v;
        }
    double r = 0;
    for (double v : rs) r = std::max(r, v);
    return r;
}

void col_max(int64_t m, int64_t n, const double* A, int64_t lda, double* out)
{
    for (int64_t j = 0; j < n; ++j) {
        double r = 0;
        for (int64_t i = 0; i < m; ++i) r = std::max(r, std::abs(A[i + j*lda]));
        out[j] = r;
    }
}

// internal::iterRefConverged (src/internal/internal_util.hh:121-138)
bool converged(const double* cr, const double* cx, int64_t n, double cte)
{
    for (int64_t i = 0; i < n; ++i)
        if (cr[i] > cx[i] * cte) return false;
    return true;
}

// R = B - A X, with A general or symmetric (lower stored).
void residual(int64_t n, int64_t nrhs, const double* A, int64_t lda, bool sym_lower,
              const double* B, int64_t ldb, const double* X, int64_t ldx, double* R)
{
    for (int64_t j = 0; j < nrhs; ++j)
        for (int64_t i = 0; i < n; ++i) R[i + j*n] = B[i + j*ldb];
    if (!sym_lower) {
        gemm('N', 'N', n, nrhs, n, -1.0, A, lda, X, ldx, 1.0, R, n);
        return;
    }
    // Symmetric A with lower storage (SLATE's hemm on a HermitianMatrix):
    // tile (I,J), I > J, contributes A_IJ X_J to R_I and A_IJ^T X_I to R_J;
    // diagonal tiles are expanded to full symmetric blocks.
    const int64_t nb = 512;
    std::vector<double> D(size_t(nb) * nb);
    for (int64_t J = 0; J < n; J += nb) {
        int64_t jb = std::min(nb, n - J);
        for (int64_t c = 0; c < jb; ++c)
            for (int64_t r = 0; r < jb; ++r)
                D[r + c * jb] = (r >= c) ? A[J + r + (J + c) * lda] : A[J + c + (J + r) * lda];
        gemm('N', 'N', jb, nrhs, jb, -1.0, D.data(), jb, X + J, ldx, 1.0, R + J, n);
        if (J + jb < n) {
            int64_t rows = n - J - jb;
            const double* Ab = A + (J + jb) + J * lda;
            gemm('N', 'N', rows, nrhs, jb, -1.0, Ab, lda, X + J, ldx, 1.0, R + J + jb, n);
            gemm('T', 'N', jb, nrhs, rows, -1.0, Ab, lda, X + J + jb, ldx, 1.0, R + J, n);
        }
    }
}

// Low-precision factor + solve used by the mixed drivers.
struct LoFactor {
    bool chol;
    int64_t n, nb, ib;
    int nthreads;
    std::vector<float> A;
    std::vector<int64_t> pt, po;
    int64_t factor(const double* Ahi, int64_t lda) {
        A.assign(size_t(n)*n, 0.f);
        for (int64_t j = 0; j < n; ++j)
            for (int64_t i = 0; i < n; ++i) A[i + j*n] = float(Ahi[i + j*lda]);
        if (chol) return potrf<float>(n, A.data(), n, nb);
        pt.assign(n, 0); po.assign(n, 0);
        return getrf<float>(n, n, A.data(), n, nb, ib, nthreads, 1.0, pt.data(), po.data(), nullptr);
    }
    // X (double, n x nrhs) <- double(M^{-1} float(R))
    void solve(int64_t nrhs, const double* R, int64_t ldr, double* X, int64_t ldx) {
        std::vector<float> w(size_t(n)*nrhs);
        for (int64_t j = 0; j < nrhs; ++j)
            for (int64_t i = 0; i < n; ++i) w[i + j*n] = float(R[i + j*ldr]);
        if (chol) potrs<float>(n, nrhs, A.data(), n, nb, w.data(), n);
        else getrs<float>(n, nrhs, A.data(), n, pt.data(), po.data(), nb, w.data(), n);
        for (int64_t j = 0; j < nrhs; ++j)
            for (int64_t i = 0; i < n; ++i) X[i + j*ldx] = double(w[i + j*n]);
    }
};

// FP64 fallback (src/gesv_mixed.cc:256-278).
int64_t fallback_solve(bool chol, int64_t n, int64_t nrhs, double* A, int64_t lda,
                       int64_t nb, int64_t ib, int nthreads, int64_t* pt, int64_t* po,
                       const double* B, int64_t ldb, double* X, int64_t ldx)
{
    int64_t info = chol ? potrf<double>(n, A, lda, nb)
                        : getrf<double>(n, n, A, lda, nb, ib, nthreads, 1.0, pt, po, nullptr);
    if (info == 0) {
        for (int64_t j = 0; j < nrhs; ++j)
            for (int64_t i = 0; i < n; ++i) X[i + j*ldx] = B[i + j*ldb];
        if (chol) potrs<double>(n, nrhs, A, lda, nb, X, ldx);
        else getrs<double>(n, nrhs, A, lda, pt, po, nb, X, ldx);
    }
    return info;
}

// gesv_mixed / posv_mixed (src/gesv_mixed.cc:105-289, src/posv_mixed.cc:105-320)
int64_t mixed_ir(bool chol, int64_t n, int64_t nrhs, double* A, int64_t lda, int64_t* pt,
                 int64_t* po, const double* B, int64_t ldb, double* X, int64_t ldx,
                 int64_t nb, int64_t ib, int nthreads, int64_t itermax, double tol,
                 int use_fallback, int64_t* iter)
{
    const double eps = std::numeric_limits<double>::epsilon();
    if (tol <= 0) tol = eps * std::sqrt(double(n));
    double Anorm = chol ? norm_inf_sym_lower(n, A, lda) : norm_inf(n, n, A, lda);
    double cte = Anorm * tol;
    LoFactor lo{chol, n, nb, ib, nthreads, {}, {}, {}};
    int64_t info = lo.factor(A, lda);
    bool conv = false;
    *iter = 0;
    std::vector<double> R(size_t(n)*nrhs), cx(nrhs), cr(nrhs);
    if (info != 0) {
        *iter = -3;
    }
    else {
        if (!chol) { std::copy(lo.pt.begin(), lo.pt.end(), pt); std::copy(lo.po.begin(), lo.po.end(), po); }
        lo.solve(nrhs, B, ldb, X, ldx);
        residual(n, nrhs, A, lda, chol, B, ldb, X, ldx, R.data());
        col_max(n, nrhs, X, ldx, cx.data());
        col_max(n, nrhs, R.data(), n, cr.data());
        if (converged(cr.data(), cx.data(), nrhs, cte)) { *iter = 0; conv = true; }
        for (int64_t it = 0; it < itermax && !conv; ++it) {
            std::vector<double> D(size_t(n)*nrhs);
            lo.solve(nrhs, R.data(), n, D.data(), n);
            for (int64_t j = 0; j < nrhs; ++j)
                for (int64_t i = 0; i < n; ++i) X[i + j*ldx] += D[i + j*n];
            residual(n, nrhs, A, lda, chol, B, ldb, X, ldx, R.data());
            col_max(n, nrhs, X, ldx, cx.data());
            col_max(n, nrhs, R.data(), n, cr.data());
            if (converged(cr.data(), cx.data(), nrhs, cte)) { *iter = it + 1; conv = true; }
        }
    }
    if (!conv) {
        if (info == 0) *iter = -itermax - 1;
        if (use_fallback)
            info = fallback_solve(chol, n, nrhs, A, lda, nb, ib, nthreads, pt, po, B, ldb, X, ldx);
    }
    return info;
}

// Classic BLAS drotg: r = sign(roe) * scale * sqrt((a/scale)^2 + (b/scale)^2).
void rotg(double a, double b, double* c, double* s)
{
    double roe = std::abs(a) > std::abs(b) ? a : b;
    double scale = std::abs(a) + std::abs(b);
    if (scale == 0) { *c = 1; *s = 0; return; }
    double r = scale * std::sqrt((a/scale)*(a/scale) + (b/scale)*(b/scale));
    r = std::copysign(1.0, roe) * r;
    *c = a / r;
    *s = b / r;
}

inline void rot(double* x, double* y, double c, double s)
{
    double tx = c * *x + s * *y;
    double ty = c * *y - s * *x;
    *x = tx; *y = ty;
}

// One right-hand side of gesv_mixed_gmres / posv_mixed_gmres
// (src/gesv_mixed_gmres.cc:225-395): right-preconditioned FGMRES with restart
// min(30, itermax, nb-1), CGS2 orthogonalisation and Givens rotations,
// starting from the x it is given.  Returns whether the stopping test held;
// *iter: the Arnoldi steps taken.
bool fgmres_column(bool chol, int64_t n, const double* A, int64_t lda, LoFactor& lo, const double* B,
                   double* X, int64_t itermax, int64_t restart, double cte, int64_t* iter)
{
    int64_t R1 = restart + 1;
    std::vector<double> V(size_t(n)*R1), W(size_t(n)*R1), R(n), z(R1);
    std::vector<double> H(size_t(R1)*R1, 0.0), S(R1, 0.0), gc(std::max<int64_t>(restart, 1)),
                        gs(std::max<int64_t>(restart, 1));
    int64_t iiter = 0;
    double cx = 0, cr = 0;
    *iter = 0;
    while (iiter < itermax) {
        residual(n, 1, A, lda, chol, B, n, X, n, R.data());
        col_max(n, 1, X, n, &cx);
        col_max(n, 1, R.data(), n, &cr);
        if (converged(&cr, &cx, 1, cte)) { *iter = iiter; return true; }
        double* v0 = V.data();
        std::copy(R.begin(), R.end(), v0);
        double ares = 0;
        for (int64_t i = 0; i < n; ++i) ares += v0[i]*v0[i];
        ares = std::sqrt(ares);
        if (ares == 0) { *iter = iiter; return false; }
        double inv = 1.0 / ares;
        for (int64_t i = 0; i < n; ++i) v0[i] *= inv;
        S[0] = ares;
        for (int64_t i = 1; i < R1; ++i) S[i] = 0;
        int64_t j = 0;
        for (; j < restart && iiter < itermax && !converged(&ares, &cx, 1, cte); ++j, ++iiter) {
            double* vj1 = V.data() + (j+1)*n;
            double* wj1 = W.data() + (j+1)*n;
            lo.solve(1, V.data() + j*n, n, wj1, n);
            if (chol) residual(n, 1, A, lda, true, std::vector<double>(n, 0.0).data(), n, wj1, n, vj1);
            else gemm('N', 'N', n, 1, n, 1.0, A, lda, wj1, n, 0.0, vj1, n);
            if (chol) for (int64_t i = 0; i < n; ++i) vj1[i] = -vj1[i];
            // CGS2
            double* hj = H.data() + j*R1;
            gemm('T', 'N', j+1, 1, n, 1.0, V.data(), n, vj1, n, 0.0, hj, R1);
            gemm('N', 'N', n, 1, j+1, -1.0, V.data(), n, hj, R1, 1.0, vj1, n);
            gemm('T', 'N', j+1, 1, n, 1.0, V.data(), n, vj1, n, 0.0, z.data(), R1);
            gemm('N', 'N', n, 1, j+1, -1.0, V.data(), n, z.data(), R1, 1.0, vj1, n);
            for (int64_t i = 0; i <= j; ++i) hj[i] += z[i];
            double nrm = 0;
            for (int64_t i = 0; i < n; ++i) nrm += vj1[i]*vj1[i];
            nrm = std::sqrt(nrm);
            double sc = 1.0 / nrm;
            for (int64_t i = 0; i < n; ++i) vj1[i] *= sc;
            hj[j+1] = nrm;
            for (int64_t i = 0; i < j; ++i) rot(&hj[i], &hj[i+1], gc[i], gs[i]);
            rotg(hj[j], hj[j+1], &gc[j], &gs[j]);
            rot(&hj[j], &hj[j+1], gc[j], gs[j]);
            rot(&S[j], &S[j+1], gc[j], gs[j]);
            ares = std::abs(S[j+1]);
        }
        // X += W(:, 1:j) * (H(0:j-1, 0:j-1)^{-1} S(0:j-1))
        std::vector<double> y(S.begin(), S.begin() + j);
        for (int64_t r = j - 1; r >= 0; --r) {
            double s = y[r];
            for (int64_t c = r + 1; c < j; ++c) s -= H[r + c*R1] * y[c];
            y[r] = s / H[r + r*R1];
        }
        for (int64_t c = 0; c < j; ++c) {
            const double* w = W.data() + (c+1)*n;
            for (int64_t i = 0; i < n; ++i) X[i] += w[i] * y[c];
        }
    }
    *iter = iiter;
    return false;
}

// gesv_mixed_gmres / posv_mixed_gmres (src/gesv_mixed_gmres.cc:110-410,
// src/posv_mixed_gmres.cc:109-436).  SLATE takes one right-hand side; with
// nrhs > 1 every column is an independent instance of that iteration sharing
// the one factorisation.  iter: the largest column count when all converge,
// else -(itermax+1) (the fallback then solves every column); col_iter, when
// given, receives each column's count (-(itermax+1) where it failed).
int64_t mixed_gmres(bool chol, int64_t n, int64_t nrhs, double* A, int64_t lda, int64_t* pt, int64_t* po,
                    const double* B, int64_t ldb, double* X, int64_t ldx, int64_t nb, int64_t ib,
                    int nthreads, int64_t itermax, double tol, int use_fallback, int64_t* iter,
                    int64_t* col_iter = nullptr)
{
    const double eps = std::numeric_limits<double>::epsilon();
    if (tol <= 0) tol = eps * std::sqrt(double(n));
    int64_t restart = std::min<int64_t>(std::min<int64_t>(30, itermax), std::min(nb, n) - 1);
    double Anorm = chol ? norm_inf_sym_lower(n, A, lda) : norm_inf(n, n, A, lda);
    double cte = Anorm * tol;
    LoFactor lo{chol, n, nb, ib, nthreads, {}, {}, {}};
    int64_t info = lo.factor(A, lda);
    bool conv = true;
    *iter = 0;
    if (info != 0) {
        *iter = -3;
        conv = false;
    }
    else {
        if (!chol) { std::copy(lo.pt.begin(), lo.pt.end(), pt); std::copy(lo.po.begin(), lo.po.end(), po); }
        std::vector<double> b(n), x(n);
        for (int64_t c = 0; c < nrhs; ++c) {
            std::copy(B + c*ldb, B + c*ldb + n, b.begin());
            lo.solve(1, b.data(), n, x.data(), n);
            int64_t it = 0;
            const bool cc = fgmres_column(chol, n, A, lda, lo, b.data(), x.data(), itermax, restart, cte, &it);
            std::copy(x.begin(), x.end(), X + c*ldx);
            if (col_iter) col_iter[c] = cc ? it : -itermax - 1;
            conv = conv && cc;
            if (cc) *iter = std::max(*iter, it);
        }
    }
    if (!conv) {
        if (info == 0) *iter = -itermax - 1;
        if (use_fallback)
            info = fallback_solve(chol, n, nrhs, A, lda, nb, ib, nthreads, pt, po, B, ldb, X, ldx);
    }
    return info;
}

// Prescribed-spectrum test matrix, the CPU statement of the library's
// device generator (slate_gb300/csrc/matgen.cu): A = Q1 diag(sigma) Q2^T
// (spd = 0) or Q diag(sigma) Q^T (spd = 1), sigma geo (dist 0) or logrand
// (dist 1) of condition number cond (SLATE's matgen/generate_sigma.hh:73-125),
// Q a product of log2(n) butterfly levels: level l rotates rows (i, i + 2^l)
// inside blocks of 2^(l+1) by the angle 2 pi u (u from Philox(i, l, seed)),
// after a sign flip of row i by the low bit of the second Philox word.
void generate_sigma(int64_t n, double cond, int dist, int spd, int64_t seed, double* A, int64_t lda)
{
    auto unit = [](uint64_t bits) { return double(bits >> 11) / double(uint64_t(1) << 53); };
    for (int64_t j = 0; j < n; ++j)
        std::fill(A + j*lda, A + j*lda + n, 0.0);
    for (int64_t i = 0; i < n; ++i) {
        double sg;
        if (dist == 0) sg = (n > 1) ? std::pow(cond, -double(i) / double(n - 1)) : 1.0;
        else {
            uint64_t b[2];
            philox2x64(uint64_t(i), 0ull, uint64_t(seed), b);
            sg = std::exp(unit(b[0]) * std::log(1.0 / cond));
            if (n >= 2 && i == 0) sg = 1.0;
            if (n >= 2 && i == 1) sg = 1.0 / cond;
        }
        A[i + i*lda] = sg;
    }
    int levels = 0;
    while ((int64_t(1) << levels) < n) ++levels;
    std::vector<int64_t> pi, pk;
    std::vector<double> rc, rs, rsi, qc, qs, qsi;
    auto rots = [&](int l, int64_t sd, std::vector<double>& c, std::vector<double>& sn, std::vector<double>& si) {
        c.resize(pi.size()); sn.resize(pi.size()); si.resize(pi.size());
        for (size_t p = 0; p < pi.size(); ++p) {
            uint64_t b[2];
            philox2x64(uint64_t(pi[p]), uint64_t(l), uint64_t(sd), b);
            const double th = 6.283185307179586 * unit(b[0]);
            c[p] = std::cos(th);
            sn[p] = std::sin(th);
            si[p] = (b[1] & 1) ? -1.0 : 1.0;
        }
    };
    for (int l = 0; l < levels; ++l) {
        const int64_t h = int64_t(1) << l;
        pi.clear(); pk.clear();
        for (int64_t i0 = 0; i0 < n; i0 += 2*h)
            for (int64_t i = i0; i < std::min(i0 + h, n); ++i)
                if (i + h < n) { pi.push_back(i); pk.push_back(i + h); }
        if (pi.empty()) continue;
        rots(l, seed + 101, rc, rs, rsi);
        if (spd) { qc = rc; qs = rs; qsi = rsi; }
        else rots(l, seed + 202, qc, qs, qsi);
        const int64_t np = int64_t(pi.size());
        // rows: A <- R_l A
        #pragma omp parallel for schedule(static)
        for (int64_t j = 0; j < n; ++j) {
            double* col = A + j*lda;
            for (int64_t p = 0; p < np; ++p) {
                const double xi = rsi[p] * col[pi[p]], yk = col[pk[p]];
                col[pi[p]] = rc[p] * xi + rs[p] * yk;
                col[pk[p]] = -rs[p] * xi + rc[p] * yk;
            }
        }
        // columns: A <- A R_l^T
        #pragma omp parallel for schedule(static)
        for (int64_t p = 0; p < np; ++p) {
            double* x = A + pi[p]*lda;
            double* y = A + pk[p]*lda;
            for (int64_t r = 0; r < n; ++r) {
                const double xi = qsi[p] * x[r], yk = y[r];
                x[r] = qc[p] * xi + qs[p] * yk;
                y[r] = -qs[p] * xi + qc[p] * yk;
            }
        }
    }
}

} // namespace

//==============================================================================
// C surface for the test harness (ctypes).
extern "C" {

void orc_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void) n;
#endif
}

int orc_get_threads()
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

// Install a host BLAS gemm (Fortran ABI); null restores the built-in loops.
void orc_set_blas(void* dgemm_ptr, void* sgemm_ptr)
{
    g_dgemm = (dgemm_f) dgemm_ptr;
    g_sgemm = (sgemm_f) sgemm_ptr;
}

// Host trsm / potrf (Fortran ABI) for the tile solves and diagonal tiles.
void orc_set_lapack(void* dtrsm_ptr, void* strsm_ptr, void* dpotrf_ptr, void* spotrf_ptr)
{
    g_dtrsm = (dtrsm_f) dtrsm_ptr;
    g_strsm = (strsm_f) strsm_ptr;
    g_dpotrf = (dpotrf_f) dpotrf_ptr;
    g_spotrf = (spotrf_f) spotrf_ptr;
}

void orc_philox(uint64_t s0, uint64_t s1, uint64_t key, uint64_t* out)
{
    philox2x64(s0, s1, key, out);
}

void orc_generate_d(int dist, int64_t seed, int64_t m, int64_t n, int64_t ioff, int64_t joff,
                    double* A, int64_t lda)
{
    philox_fill<double>(dist, seed, m, n, ioff, joff, A, lda);
}

void orc_generate_s(int dist, int64_t seed, int64_t m, int64_t n, int64_t ioff, int64_t joff,
                    float* A, int64_t lda)
{
    philox_fill<float>(dist, seed, m, n, ioff, joff, A, lda);
}

// Deterministic test matrices (matgen/generate_matrix_ge.cc:80-340).
// kind: 0 zeros, 1 ones, 2 identity, 3 ij, 4 jordan, 5 jordanT, 6 kms,
//       7 minij, 8 hilb, 9 lehmer, 10 lotkin
int orc_generate_kind(int kind, int64_t m, int64_t n, double* A, int64_t lda)
{
    double s_ij = 1.0 / std::pow(10.0, std::ceil(std::log10(double(n))));
    for (int64_t j = 0; j < n; ++j)
        for (int64_t i = 0; i < m; ++i) {
            double v;
            switch (kind) {
                case 0: v = 0; break;
                case 1: v = 1; break;
                case 2: v = (i == j) ? 1 : 0; break;
                case 3: v = double(i) + double(j) * s_ij; break;
                case 4: v = (i == j || i + 1 == j) ? 1 : 0; break;
                case 5: v = (i == j || j + 1 == i) ? 1 : 0; break;
                case 6: v = std::pow(0.5, double(std::abs(j - i))); break;
                case 7: v = double(std::min(i + 1, j + 1)); break;
                case 8: v = 1.0 / double(i + j + 1); break;
                case 9: v = double(std::min(i, j) + 1) / double(std::max(i, j) + 1); break;
                case 10: v = (i == 0) ? 1.0 : 1.0 / double(i + j + 1); break;
                default: return -1;
            }
            A[i + j*lda] = v;
        }
    return 0;
}

// LU with partial pivoting.  Pivots are returned both in SLATE's form
// (tile index relative to the panel, offset; include/slate/types.hh:84-117)
// and as a LAPACK ipiv (1-based, lapack_api/lapack_gesv.cc:90-100).
int64_t orc_dgetrf(int64_t m, int64_t n, double* A, int64_t lda, int64_t nb, int64_t ib,
                   int panel_threads, double threshold, int64_t* piv_tile, int64_t* piv_off,
                   int64_t* ipiv, double* margin)
{
    int64_t mn = std::min(m, n);
    int64_t info = getrf<double>(m, n, A, lda, nb, ib, panel_threads, threshold,
                                 piv_tile, piv_off, margin);
    if (ipiv)
        for (int64_t r = 0; r < mn; ++r) ipiv[r] = (r / nb)*nb + piv_tile[r]*nb + piv_off[r] + 1;
    return info;
}

int64_t orc_sgetrf(int64_t m, int64_t n, float* A, int64_t lda, int64_t nb, int64_t ib,
                   int panel_threads, double threshold, int64_t* piv_tile, int64_t* piv_off,
                   int64_t* ipiv, double* margin)
{
    int64_t mn = std::min(m, n);
    int64_t info = getrf<float>(m, n, A, lda, nb, ib, panel_threads, threshold,
                                piv_tile, piv_off, margin);
    if (ipiv)
        for (int64_t r = 0; r < mn; ++r) ipiv[r] = (r / nb)*nb + piv_tile[r]*nb + piv_off[r] + 1;
    return info;
}

void orc_dgetrs(int64_t n, int64_t nrhs, const double* LU, int64_t lda, const int64_t* piv_tile,
                const int64_t* piv_off, int64_t nb, double* B, int64_t ldb)
{
    getrs<double>(n, nrhs, LU, lda, piv_tile, piv_off, nb, B, ldb);
}

int64_t orc_dgesv(int64_t n, int64_t nrhs, double* A, int64_t lda, int64_t nb, int64_t ib,
                  int panel_threads, int64_t* piv_tile, int64_t* piv_off, double* B, int64_t ldb)
{
    int64_t info = getrf<double>(n, n, A, lda, nb, ib, panel_threads, 1.0, piv_tile, piv_off, nullptr);
    if (info == 0) getrs<double>(n, nrhs, A, lda, piv_tile, piv_off, nb, B, ldb);
    return info;
}

int64_t orc_dpotrf(int64_t n, double* A, int64_t lda, int64_t nb)
{
    return potrf<double>(n, A, lda, nb);
}

int64_t orc_spotrf(int64_t n, float* A, int64_t lda, int64_t nb)
{
    return potrf<float>(n, A, lda, nb);
}

void orc_dpotrs(int64_t n, int64_t nrhs, const double* L, int64_t lda, int64_t nb,
                double* B, int64_t ldb)
{
    potrs<double>(n, nrhs, L, lda, nb, B, ldb);
}

int64_t orc_dposv(int64_t n, int64_t nrhs, double* A, int64_t lda, int64_t nb, double* B, int64_t ldb)
{
    int64_t info = potrf<double>(n, A, lda, nb);
    if (info == 0) potrs<double>(n, nrhs, A, lda, nb, B, ldb);
    return info;
}

int64_t orc_dgesv_mixed(int64_t n, int64_t nrhs, double* A, int64_t lda, int64_t* piv_tile,
                        int64_t* piv_off, const double* B, int64_t ldb, double* X, int64_t ldx,
                        int64_t nb, int64_t ib, int panel_threads, int64_t itermax, double tol,
                        int use_fallback, int64_t* iter)
{
    return mixed_ir(false, n, nrhs, A, lda, piv_tile, piv_off, B, ldb, X, ldx, nb, ib,
                    panel_threads, itermax, tol, use_fallback, iter);
}

int64_t orc_dposv_mixed(int64_t n, int64_t nrhs, double* A, int64_t lda, const double* B,
                        int64_t ldb, double* X, int64_t ldx, int64_t nb, int64_t itermax,
                        double tol, int use_fallback, int64_t* iter)
{
    return mixed_ir(true, n, nrhs, A, lda, nullptr, nullptr, B, ldb, X, ldx, nb, 16, 1,
                    itermax, tol, use_fallback, iter);
}

int64_t orc_dgesv_mixed_gmres(int64_t n, double* A, int64_t lda, int64_t* piv_tile,
                              int64_t* piv_off, const double* B, double* X, int64_t nb,
                              int64_t ib, int panel_threads, int64_t itermax, double tol,
                              int use_fallback, int64_t* iter)
{
    return mixed_gmres(false, n, 1, A, lda, piv_tile, piv_off, B, n, X, n, nb, ib, panel_threads,
                       itermax, tol, use_fallback, iter);
}

int64_t orc_dposv_mixed_gmres(int64_t n, double* A, int64_t lda, const double* B, double* X,
                              int64_t nb, int64_t itermax, double tol, int use_fallback,
                              int64_t* iter)
{
    return mixed_gmres(true, n, 1, A, lda, nullptr, nullptr, B, n, X, n, nb, 16, 1, itermax, tol,
                       use_fallback, iter);
}
// Several right-hand sides, each an independent FGMRES-IR instance sharing
// one factorisation; col_iter (nrhs entries) receives each column's count.
int64_t orc_dgesv_mixed_gmres_nrhs(int64_t n, int64_t nrhs, double* A, int64_t lda, int64_t* piv_tile,
                                   int64_t* piv_off, const double* B, int64_t ldb, double* X, int64_t ldx,
                                   int64_t nb, int64_t ib, int panel_threads, int64_t itermax, double tol,
                                   int use_fallback, int64_t* iter, int64_t* col_iter)
{
    return mixed_gmres(false, n, nrhs, A, lda, piv_tile, piv_off, B, ldb, X, ldx, nb, ib, panel_threads,
                       itermax, tol, use_fallback, iter, col_iter);
}
int64_t orc_dposv_mixed_gmres_nrhs(int64_t n, int64_t nrhs, double* A, int64_t lda, const double* B,
                                   int64_t ldb, double* X, int64_t ldx, int64_t nb, int64_t itermax,
                                   double tol, int use_fallback, int64_t* iter, int64_t* col_iter)
{
    return mixed_gmres(true, n, nrhs, A, lda, nullptr, nullptr, B, ldb, X, ldx, nb, 16, 1, itermax, tol,
                       use_fallback, iter, col_iter);
}
void orc_dgenerate_sigma(int64_t n, double cond, int dist, int spd, int64_t seed, double* A, int64_t lda)
{
    generate_sigma(n, cond, dist, spd, seed, A, lda);
}

// Tester check (test/test_gesv.cc:330-380):
//   ||B - A X||_1 / (n ||A||_1 ||X||_1).  sym_lower: A symmetric, lower stored.
double orc_backward_error(int64_t n, int64_t nrhs, const double* A, int64_t lda, int sym_lower,
                          const double* X, int64_t ldx, const double* B, int64_t ldb)
{
    std::vector<double> R(size_t(n)*nrhs);
    residual(n, nrhs, A, lda, sym_lower != 0, B, ldb, X, ldx, R.data());
    auto norm1 = [&](const double* M, int64_t ld, int64_t rows, int64_t cols) {
        double r = 0;
        for (int64_t j = 0; j < cols; ++j) {
            double s = 0;
            for (int64_t i = 0; i < rows; ++i) s += std::abs(M[i + j*ld]);
            r = std::max(r, s);
        }
        return r;
    };
    double an;
    if (sym_lower) {
        std::vector<double> cs(n, 0.0);
        for (int64_t j = 0; j < n; ++j)
            for (int64_t i = j; i < n; ++i) {
                double v = std::abs(A[i + j*lda]);
                cs[j] += v;
                if (i != j) cs[i] += v;
            }
        an = 0;
        for (double v : cs) an = std::max(an, v);
    }
    else {
        an = norm1(A, lda, n, n);
    }
    double xn = norm1(X, ldx, n, nrhs);
    double rn = norm1(R.data(), n, n, nrhs);
    return rn / (double(n) * an * xn);
}

} // extern "C"
