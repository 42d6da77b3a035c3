/* slt_kernels.h -- the thin extern "C" CUDA layer under the C++ drivers.
 *
 * Stream-ordered launchers over device pointers.  Matrices are column-major
 * with a leading dimension.  Every launcher returns an slt status code
 * (0 = SLT_OK) and never synchronises the stream.
 */
#ifndef SLT_KERNELS_H
#define SLT_KERNELS_H

#include <stdint.h>
#include <stddef.h>
#include <cuda_runtime.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#ifndef SLT_OK
#define SLT_OK                 0
#define SLT_ERR_ARG           -1
#define SLT_ERR_TIMEOUT       -2
#define SLT_ERR_NOMEM         -3
#define SLT_ERR_NOT_SUPPORTED -4
#define SLT_ERR_NO_DEVICE     -5
#define SLT_ERR_LIMIT         -6
#define SLT_ERR_CUDA_BASE   1000
#endif

/* ---- SM budget ---------------------------------------------------------------
 * Number of SMs that the panel and trailing-update launchers may occupy with
 * the launches that the calling thread issues next (0: all).  The lookahead
 * schedule of the drivers gives the panel of step k+1 and the update of step
 * k disjoint shares of the SMs, so the two run side by side.  Returns the
 * previous value. */
int slt_set_sm_cap(int sms);
int slt_sm_cap(void);

/* ---- trailing-matrix update GEMM:  C = alpha A op(B) + beta C --------------
 * transb 'N': B is k x n;  'T': B is n x k (C -= A B^T, the Cholesky update).
 * lower != 0: only the lower triangle (i >= j) of C is computed and written.
 * engine: 0 auto, 1 SIMT FMA, 2 FP64 tensor (DMMA) (double only). */
int slt_dgemm(char transb, int64_t m, int64_t n, int64_t k, double alpha,
              const double* A, int64_t lda, const double* B, int64_t ldb,
              double beta, double* C, int64_t ldc, int lower, int engine,
              cudaStream_t stream);
int slt_sgemm(char transb, int64_t m, int64_t n, int64_t k, float alpha,
              const float* A, int64_t lda, const float* B, int64_t ldb,
              float beta, float* C, int64_t ldc, int lower, cudaStream_t stream);

/* ---- low-precision tensor-core update (tcgen05) ----------------------------
 * C (fp32, m x n) -= A (m x k) op(B), operands rounded to the tier's type
 * (2 TF32, 3 BF16, 4 FP16), fp32 accumulation in TMEM.  transb 'N': B is
 * k x n; 'T': B is n x k.  lower: only C(i,j), i >= j, is updated.  ws may be
 * null.  slt_tc_status() returns (and clears) SLT_ERR_TIMEOUT after a tile
 * gave up waiting. */
int slt_tc_gemm_update(int tier, char transb, int64_t m, int64_t n, int64_t k, const float* A,
                       int64_t lda, const float* B, int64_t ldb, float* C, int64_t ldc, int lower,
                       void* ws, size_t ws_bytes, cudaStream_t stream);
size_t slt_tc_gemm_ws_bytes(int64_t m, int64_t n, int64_t k);
int slt_tc_status(void);

/* ---- LU panel -------------------------------------------------------------
 * Factor the prows x nbk panel P (top-left = diagonal element) with partial
 * pivoting.  ipiv[j] receives the pivot row of column j relative to the
 * panel's first row; *info (device) receives info_offset + j + 1 for the
 * first exactly-zero pivot (if *info is still 0).  ws: device workspace of
 * slt_getrf_panel_ws_bytes() bytes.  *status (device) receives
 * SLT_ERR_TIMEOUT if a grid barrier ever times out.  threshold: SLATE's
 * PivotThreshold (1 = partial pivoting, 0 = keep the diagonal: no pivoting). */
size_t slt_getrf_panel_ws_bytes(int64_t prows, int64_t ib);
int slt_dgetrf_panel(int64_t prows, int64_t nbk, int64_t ib, double* P, int64_t ld,
                     int* ipiv, int* info, int64_t info_offset, double threshold, void* ws,
                     int* status, cudaStream_t stream);
int slt_sgetrf_panel(int64_t prows, int64_t nbk, int64_t ib, float* P, int64_t ld,
                     int* ipiv, int* info, int64_t info_offset, double threshold, void* ws,
                     int* status, cudaStream_t stream);

/* ---- row interchanges -----------------------------------------------------
 * slt_swap_plan: turn one panel's sequential interchanges (ipiv relative to
 * row r0, len entries) into a gather plan of at most 2*len (dst, src) row
 * pairs, written to plan (int[1 + 4*len]): plan[0] = count, then dst rows,
 * then src rows (absolute).  slt_?laswp_plan applies a plan to ncols columns
 * of A. */
int slt_swap_plan(const int* ipiv, int64_t len, int64_t r0, int* plan, cudaStream_t stream);
int slt_dlaswp_plan(const int* plan, int64_t maxcount, double* A, int64_t lda,
                    int64_t ncols, cudaStream_t stream);
int slt_slaswp_plan(const int* plan, int64_t maxcount, float* A, int64_t lda,
                    int64_t ncols, cudaStream_t stream);
/* Compose all panels' interchanges into one row permutation perm (n
 * entries): row i of P A is row perm[i] of A.  ipiv: n entries, relative to
 * each panel's first row (panel k starts at k*nb). */
int slt_perm_from_ipiv(const int* ipiv, int64_t n, int64_t nb, int* perm, cudaStream_t stream);
/* Y(i, :) = X(perm[i], :) for i < n (forward) or Y(perm[i], :) = X(i, :). */
int slt_dpermute_rows(int forward, const int* perm, int64_t n, int64_t ncols,
                      const double* X, int64_t ldx, double* Y, int64_t ldy, cudaStream_t stream);
int slt_spermute_rows(int forward, const int* perm, int64_t n, int64_t ncols,
                      const float* X, int64_t ldx, float* Y, int64_t ldy, cudaStream_t stream);

/* ---- triangular solves ----------------------------------------------------
 * trsm_left_lower_unit: B(kb x n) <- L^{-1} B, L kb x kb unit lower (the LU
 * row panel U12 = L11^{-1} A12, and the getrs forward diagonal blocks). */
int slt_dtrsm_llnu(int64_t kb, int64_t n, const double* L, int64_t ldl, double* B,
                   int64_t ldb, cudaStream_t stream);
int slt_strsm_llnu(int64_t kb, int64_t n, const float* L, int64_t ldl, float* B,
                   int64_t ldb, cudaStream_t stream);
/* Left, upper, non-unit: B <- U^{-1} B (getrs backward diagonal blocks). */
int slt_dtrsm_lunn(int64_t kb, int64_t n, const double* U, int64_t ldu, double* B,
                   int64_t ldb, cudaStream_t stream);
int slt_strsm_lunn(int64_t kb, int64_t n, const float* U, int64_t ldu, float* B,
                   int64_t ldb, cudaStream_t stream);
/* Left, lower, non-unit, op = N or T: B <- op(L)^{-1} B (potrs blocks). */
int slt_dtrsm_llnn(char trans, int64_t kb, int64_t n, const double* L, int64_t ldl,
                   double* B, int64_t ldb, cudaStream_t stream);
int slt_strsm_llnn(char trans, int64_t kb, int64_t n, const float* L, int64_t ldl,
                   float* B, int64_t ldb, cudaStream_t stream);
/* Right, lower^T, non-unit: B(m x kb) <- B L^{-T} (Cholesky column panel). */
int slt_dtrsm_runn(int64_t m, int64_t kb, const double* U, int64_t ldu, double* B, int64_t ldb,
                   cudaStream_t stream);
int slt_strsm_runn(int64_t m, int64_t kb, const float* U, int64_t ldu, float* B, int64_t ldb,
                   cudaStream_t stream);
int slt_dtrsm_rltn(int64_t m, int64_t kb, const double* L, int64_t ldl, double* B,
                   int64_t ldb, cudaStream_t stream);
int slt_strsm_rltn(int64_t m, int64_t kb, const float* L, int64_t ldl, float* B,
                   int64_t ldb, cudaStream_t stream);
/* Cholesky of one diagonal block (kb <= 64, lower, in place, one CTA).
 * *info (device) receives info_offset + j + 1 at the first non-positive
 * pivot if still 0; *flag (device) is set non-zero on failure so later
 * launches become no-ops. */
int slt_dpotrf_small(int64_t kb, double* A, int64_t lda, int* info, int64_t info_offset,
                     cudaStream_t stream);
int slt_spotrf_small(int64_t kb, float* A, int64_t lda, int* info, int64_t info_offset,
                     cudaStream_t stream);

/* ---- auxiliary ------------------------------------------------------------- */
int slt_convert_d2s(int64_t m, int64_t n, const double* A, int64_t lda, float* B, int64_t ldb,
                    cudaStream_t stream);
int slt_convert_s2d(int64_t m, int64_t n, const float* A, int64_t lda, double* B, int64_t ldb,
                    cudaStream_t stream);
/* B = diag(r) A diag(c) cast to float (r, c may be null), and X = diag(r) B */
int slt_convert_d2s_scaled(int64_t m, int64_t n, const double* A, int64_t lda, const double* r,
                           const double* c, float* B, int64_t ldb, cudaStream_t stream);
int slt_convert_s2d_scaled(int64_t m, int64_t n, const float* B, int64_t ldb, const double* r,
                           double* X, int64_t ldx, cudaStream_t stream);
/* power-of-two equilibration scales: general (row r, column c; ws m words),
 * SPD (d from the diagonal) */
int slt_dgeequ(int64_t m, int64_t n, const double* A, int64_t lda, double* r, double* c, void* ws,
               cudaStream_t stream);
int slt_dpoequ(int64_t n, const double* A, int64_t lda, double* d, cudaStream_t stream);
int slt_dcopy2d(int64_t m, int64_t n, const double* A, int64_t lda, double* B, int64_t ldb,
                cudaStream_t stream);
/* B = alpha A + beta B */
int slt_dgeadd(int64_t m, int64_t n, double alpha, const double* A, int64_t lda, double beta,
               double* B, int64_t ldb, cudaStream_t stream);
/* out[j] = max_i |A(i,j)| */
int slt_dcolmax(int64_t m, int64_t n, const double* A, int64_t lda, double* out,
                cudaStream_t stream);
/* *out = ||A||_inf (max row sum); sym_lower: A symmetric with lower storage.
 * ws: at least slt_norm_ws_bytes(m) bytes. */
size_t slt_norm_ws_bytes(int64_t m);
int slt_dnorm_inf(int64_t m, int64_t n, const double* A, int64_t lda, int sym_lower,
                  double* out, void* ws, cudaStream_t stream);
/* R = B - A X  (A n x n general, or symmetric lower-stored), FP64.
 * ws: slt_residual_ws_bytes(n, nrhs) bytes. */
size_t slt_residual_ws_bytes(int64_t n, int64_t nrhs);
int slt_dresidual(int64_t n, int64_t nrhs, const double* A, int64_t lda, int sym_lower,
                  const double* B, int64_t ldb, const double* X, int64_t ldx,
                  double* R, int64_t ldr, void* ws, cudaStream_t stream);
/* R = B - A X with FP64 accuracy on the BF16 tensor cores (digit splitting,
 * digit_residual.cu), nrhs <= 16, one call with its own workspace: the
 * drivers keep the digit planes of A for a whole solve instead.  The _norm
 * form also writes ||A||_inf (d_norm, device) from the split's exact integer
 * row sums. */
int slt_dresidual_digits(int64_t n, int64_t nrhs, const double* A, int64_t lda, int sym_lower,
                         const double* B, int64_t ldb, const double* X, int64_t ldx,
                         double* R, int64_t ldr, cudaStream_t stream);
int slt_dresidual_digits_norm(int64_t n, int64_t nrhs, const double* A, int64_t lda, int sym_lower,
                              const double* B, int64_t ldb, const double* X, int64_t ldx,
                              double* R, int64_t ldr, double* d_norm, cudaStream_t stream);
/* Classical Gram-Schmidt applied twice (CGS2) for the columns of one block
 * FGMRES step (arnoldi.cu).  Column i of the step uses basis slot q[i] of V
 * (slot q: n x R1 doubles at V + q n R1) and its step j[i]: the new vector
 * V_q(:, j+1) = -W(:, i) is orthogonalised against V_q(:, 0:j); the two
 * coefficient vectors go to scal[q SC + 4 ..] and scal[q SC + 4 + R1 ..],
 * the norm of the result to scal[q SC + 3].  R1 <= 32.
 * ws: slt_cgs_ws_bytes(R1) bytes. */
#define kSltCgsMaxCols 16
#define kSltCgsMaxSeg 64
typedef struct slt_cgs_cols {
    int na;                    /* active columns, <= 16 */
    int q[kSltCgsMaxCols];     /* basis slot */
    int j[kSltCgsMaxCols];     /* step: basis vectors 0..j exist */
} slt_cgs_cols;
size_t slt_cgs_ws_bytes(int64_t R1);
int slt_dcgs2(int64_t n, double* V, int64_t R1, const slt_cgs_cols* cols, const double* W, double* scal,
              int64_t SC, void* ws, cudaStream_t stream);
/* Lower triangle of B (float) = diag(d) A diag(d) (d may be null), the
 * strictly upper part of B untouched: the Cholesky factor's working copy. */
int slt_convert_d2s_scaled_lower(int64_t n, const double* A, int64_t lda, const double* d, float* B,
                                 int64_t ldb, cudaStream_t stream);
/* The same for columns [j0, j1) only (rows [j0, n)). */
int slt_convert_d2s_scaled_lower_cols(int64_t n, int64_t j0, int64_t j1, const double* A, int64_t lda,
                                      const double* d, float* B, int64_t ldb, cudaStream_t stream);
/* Tensor-core update on operands already in 16-bit K-major form (tier FP16
 * or BF16): C (fp32, m x n) -= A B^T, row i of A at A16 + i lda16 elements,
 * kpad a multiple of 64; lower: only C(i, j), i >= j.  slt_pack_rows16 writes
 * rows [r0, m) x columns [c0, c1) of a column-major FP32 lower factor into
 * that form (zero above the diagonal). */
int slt_tc_gemm_packed(int tier, int64_t m, int64_t n, int64_t kpad, const void* A16, int64_t lda16,
                       const void* B16, int64_t ldb16, float* C, int64_t ldc, int lower, cudaStream_t stream);
int slt_pack_rows16(int tier, int64_t m, int64_t r0, int64_t c0, int64_t c1, const float* src, int64_t lds,
                    void* dst, int64_t ldd, cudaStream_t stream);
/* Philox matrix generator identical to SLATE's slate::random::generate. */
int slt_dgenerate(int dist, int64_t seed, int64_t m, int64_t n, int64_t ioff, int64_t joff,
                  double* A, int64_t lda, cudaStream_t stream);
/* Test matrix with prescribed singular values (spd = 0: Q1 diag(sigma) Q2^T)
 * or eigenvalues (spd = 1: Q diag(sigma) Q^T), sigma from SLATE's "geo"
 * (dist 0) or "logrand" (dist 1) distribution with condition number cond;
 * Q from log2(n) random butterfly levels (see matgen.cu). */
int slt_dgenerate_sigma(int64_t n, double cond, int dist, int spd, int64_t seed, double* A, int64_t lda,
                        cudaStream_t stream);
/* A(i,i) += alpha for i < n */
int slt_dshift_diag(int64_t n, double alpha, double* A, int64_t lda, cudaStream_t stream);
int slt_sshift_diag(int64_t n, float alpha, float* A, int64_t lda, cudaStream_t stream);
/* Symmetrise from the lower triangle: A(j,i) = A(i,j) for i > j. */
int slt_dsymmetrize_lower(int64_t n, double* A, int64_t lda, cudaStream_t stream);
/* D = S on the lower (lower = 1) or upper triangle, diagonal included */
int slt_dcopy_tri(int lower, int64_t n, const double* S, int64_t lds, double* D, int64_t ldd, cudaStream_t stream);
int slt_dtranspose(int64_t m, int64_t n, const double* A, int64_t lda, double* B, int64_t ldb, cudaStream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* SLT_KERNELS_H */
