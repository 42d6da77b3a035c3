/* slate_gb300.h -- C ABI of the GB300 LU / Cholesky solve library.
 *
 * Three layers, all extern "C", plain pointers and sizes:
 *
 *  1. LAPACK-compatible entry points (host pointers, Fortran by-pointer
 *     arguments, 32-bit int, 1-based ipiv), drop-ins for SLATE's lapack_api.
 *     Exported both as slate_dgesv and slate_dgesv_ (the two manglings
 *     SLATE's BLAS_FORTRAN_NAME can produce).
 *  2. Device entry points (device pointers, column-major, a CUDA stream):
 *     the Matrix::fromDevices / Target::Devices form of SLATE's drivers on a
 *     1 x 1 grid.
 *  3. Options and status helpers.
 *
 * Matrices are column-major; the tile size nb of SLATE's tile layout is an
 * option.  ipiv on the device is stored per panel: ipiv[k*nb + j] is the pivot
 * row of global row k*nb + j, relative to row k*nb (SLATE's Pivot(tile index,
 * offset) flattened, include/slate/types.hh:84-117).
 */
#ifndef SLATE_GB300_H
#define SLATE_GB300_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* CUDA stream, passed as an opaque pointer so this header needs no CUDA. */
typedef void* slt_stream_t;

/* Precision of the O(n^3) factorisation inside the mixed solvers. */
enum slt_precision {
    SLT_PREC_FP64 = 0,   /* plain FP64 factorisation (no refinement)        */
    SLT_PREC_FP32 = 1,   /* FP32 factorisation, SLATE's gesv_mixed<double,float> */
    SLT_PREC_TF32 = 2,   /* FP32 storage, TF32 tensor-core trailing update   */
    SLT_PREC_BF16 = 3,   /* FP32 storage, BF16 tensor-core trailing update   */
    SLT_PREC_FP16 = 4,   /* FP32 storage, FP16 tensor-core trailing update   */
    SLT_PREC_FP8  = 5,   /* FP32 storage, FP8 E4M3 tensor-core trailing update
                            with a power-of-two scale per 128-row tile
                            (experimental)                                   */
    SLT_PREC_TF32X3 = 6  /* FP32 storage, split-precision 3xTF32 tensor-core
                            trailing update (inputs to 22 bits, FP32 sums)   */
};

/* Options (SLATE Option keys, include/slate/enums.hh:453-490). */
typedef struct slt_options {
    int64_t nb;               /* Option::BlockSize (tile size), default 512       */
    int64_t ib;               /* Option::InnerBlocking, default 32                */
    int64_t lookahead;        /* Option::Lookahead, default 1                     */
    int64_t max_iterations;   /* Option::MaxIterations, default 30                */
    double  tolerance;        /* Option::Tolerance; <= 0: eps * sqrt(n)           */
    int     use_fallback;     /* Option::UseFallbackSolver, default 1             */
    double  pivot_threshold;  /* Option::PivotThreshold, default 1 (partial piv.) */
    int     factor_precision; /* slt_precision of mixed solvers, default FP32     */
    int     gemm_engine;      /* FP64 update engine: 0 auto, 1 SIMT, 2 DMMA       */
    int     refine;           /* mixed solvers: slt_refine, default SLT_REFINE_IR */
    int     equilibrate;      /* mixed solvers: -1 auto (on for BF16/FP16), 0, 1  */
    int     lo_retry;         /* 16-bit factor failed or did not converge: retry
                                 with an FP32 factor before the FP64 fallback;
                                 -1 auto (on for BF16/FP16), 0, 1               */
    int64_t depth;            /* Option::Depth of gesv_rbt's butterflies, default 2 */
    int     method_lu;        /* Option::MethodLU: 'P' partial pivoting (default,
                                 also '*'), 'N' no pivoting, 'C' CALU      */
    int     residual_engine;  /* FP64 residuals of the mixed solvers: 0 auto
                                 (tensor cores when a residual covers >= 2
                                 columns at n >= 1024 and the digit planes,
                                 16 n^2 bytes, fit), 1 FP64 FMA (SLATE's FP64
                                 gemm / hemm), 2 tensor cores (FP64-accurate
                                 digit-split products, digit_residual.cu)   */
} slt_options;

/* Refinement of the mixed solvers.  SLT_REFINE_IR is SLATE's gesv_mixed loop
 * (src/gesv_mixed.cc:210-262); SLT_REFINE_GMRES makes slt_dsgesv_device /
 * slt_dsposv_device run SLATE's gesv_mixed_gmres iteration
 * (src/gesv_mixed_gmres.cc:110-410) instead, as the gmres entry points do;
 * SLT_REFINE_IR_GMRES runs the IR loop while the residual falls by at least
 * half per step and, once it stalls, continues each unconverged column with
 * FGMRES-IR preconditioned by the same low-precision factors before any FP64
 * fallback.  The gmres entry points always run FGMRES-IR.  The LAPACK-
 * compatible entry points read it from SLATE_LAPACK_REFINE (ir | gmres |
 * ir+gmres, default ir). */
enum slt_refine {
    SLT_REFINE_IR = 0,
    SLT_REFINE_GMRES = 1,
    SLT_REFINE_IR_GMRES = 2
};

void slt_options_default(slt_options* opts);

/* Status codes returned by the device layer (0 = success; CUDA errors are
 * SLT_ERR_CUDA_BASE + the cudaError_t value). */
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
const char* slt_status_string(int status);

/* Library version string. */
const char* slt_version(void);

/* ------------------------------------------------------------------------- */
/* Device entry points.  Return an slt status (0 ok); *info receives SLATE's   */
/* info (0, or the 1-based column of a zero pivot / non-positive minor).      */
/* All calls are complete (stream synchronised) on return.                    */

/* slate::getrf, src/getrf.cc:319-356 */
int slt_dgetrf_device(int64_t m, int64_t n, double* dA, int64_t lda, int* d_ipiv,
                      const slt_options* opts, slt_stream_t stream, int64_t* info);
int slt_sgetrf_device(int64_t m, int64_t n, float* dA, int64_t lda, int* d_ipiv,
                      const slt_options* opts, slt_stream_t stream, int64_t* info);
/* slate::getrs (NoTrans), src/getrs.cc:66-117 */
int slt_dgetrs_device(int64_t n, int64_t nrhs, const double* dLU, int64_t lda, const int* d_ipiv,
                      double* dB, int64_t ldb, const slt_options* opts, slt_stream_t stream);
int slt_sgetrs_device(int64_t n, int64_t nrhs, const float* dLU, int64_t lda, const int* d_ipiv,
                      float* dB, int64_t ldb, const slt_options* opts, slt_stream_t stream);
/* slate::getrs with Op::Trans / ConjTrans (real: the same), src/getrs.cc:66-117;
 * trans = 'N' is slt_dgetrs_device. */
int slt_dgetrs_trans_device(char trans, int64_t n, int64_t nrhs, const double* dLU, int64_t lda,
                            const int* d_ipiv, double* dB, int64_t ldb, const slt_options* opts,
                            slt_stream_t stream);
/* slate::gecondest (src/gecondest.cc) from getrf's factors and slate::pocondest
 * (src/pocondest.cc) from potrf's: reciprocal condition number estimate in
 * the 1-norm ('1') or infinity norm ('I'); anorm = ||A|| in that norm. */
int slt_dgecondest_device(char norm, int64_t n, const double* dLU, int64_t lda, const int* d_ipiv,
                          double anorm, double* rcond, const slt_options* opts, slt_stream_t stream);
int slt_dpocondest_device(char norm, int64_t n, const double* dL, int64_t lda, double anorm,
                          double* rcond, const slt_options* opts, slt_stream_t stream);
/* slate::getri (src/getri.cc): dA (getrf's factors) <- A^{-1}; slate::potri
 * (src/potri.cc): dA (potrf's lower factor) <- lower triangle of A^{-1}.
 * *info = i > 0 when the i-th diagonal entry of the factor is exactly zero. */
int slt_dgetri_device(int64_t n, double* dA, int64_t lda, const int* d_ipiv, const slt_options* opts,
                      slt_stream_t stream, int64_t* info);
int slt_dpotri_device(int64_t n, double* dA, int64_t lda, const slt_options* opts, slt_stream_t stream,
                      int64_t* info);
/* slate::gesv, src/gesv.cc:85-109 */
int slt_dgesv_device(int64_t n, int64_t nrhs, double* dA, int64_t lda, int* d_ipiv,
                     double* dB, int64_t ldb, const slt_options* opts, slt_stream_t stream,
                     int64_t* info);
/* slate::potrf (lower), src/potrf.cc:261-281 */
int slt_dpotrf_device(int64_t n, double* dA, int64_t lda, const slt_options* opts,
                      slt_stream_t stream, int64_t* info);
int slt_spotrf_device(int64_t n, float* dA, int64_t lda, const slt_options* opts,
                      slt_stream_t stream, int64_t* info);
/* slate::potrs (lower), src/potrs.cc:55-78 */
int slt_dpotrs_device(int64_t n, int64_t nrhs, const double* dL, int64_t lda, double* dB,
                      int64_t ldb, const slt_options* opts, slt_stream_t stream);
/* slate::posv (lower), src/posv.cc:70-94 */
int slt_dposv_device(int64_t n, int64_t nrhs, double* dA, int64_t lda, double* dB, int64_t ldb,
                     const slt_options* opts, slt_stream_t stream, int64_t* info);
/* slate::gesv_mixed, src/gesv_mixed.cc:105-289.  A is left unchanged unless
 * the FP64 fallback runs (then it holds the FP64 LU factors). */
int slt_dsgesv_device(int64_t n, int64_t nrhs, double* dA, int64_t lda, int* d_ipiv,
                      const double* dB, int64_t ldb, double* dX, int64_t ldx,
                      const slt_options* opts, slt_stream_t stream, int* iter, int64_t* info);
/* slate::gesv_mixed_gmres, src/gesv_mixed_gmres.cc:110-410 (nrhs columns are
 * solved as independent single-right-hand-side FGMRES-IR instances). */
int slt_dsgesv_gmres_device(int64_t n, int64_t nrhs, double* dA, int64_t lda, int* d_ipiv,
                            const double* dB, int64_t ldb, double* dX, int64_t ldx,
                            const slt_options* opts, slt_stream_t stream, int* iter,
                            int64_t* info);
/* slate::gesv_rbt, src/gesv_rbt.cc:100-230: random butterfly transform of
 * depth opts->depth, LU without pivoting of the transformed matrix, FP64
 * refinement against A (iter 0..itermax, or -(itermax+1) and the
 * partial-pivoting fallback).  dA receives the factors of the transformed
 * matrix (after the fallback: A itself, as SLATE leaves it). */
int slt_dgesv_rbt_device(int64_t n, int64_t nrhs, double* dA, int64_t lda, const double* dB, int64_t ldb,
                         double* dX, int64_t ldx, const slt_options* opts, slt_stream_t stream, int* iter,
                         int64_t* info);
/* slate::gerbt(U, A, V) and gerbt(U, B) (src/gerbt.cc, Tile_gerbt.hh): one
 * random diagonal of n entries per side (SLATE's packed n x depth storage
 * uses its first column at every level), levels of tiles of nb.
 *   gerbt2: A <- W_U^T A W_V;  gerbt1: B <- W^T B (trans 'T') or W B ('N').
 * rbt_diag: w = exp(r / 20), r uniform(-1, 1) from the Philox stream of seed
 * (internal_rbt_generate.cc:36-50). */
int slt_dgerbt2_device(int64_t n, double* dA, int64_t lda, const double* u, const double* v, int64_t depth,
                       int64_t nb, slt_stream_t stream);
int slt_dgerbt1_device(char trans, int64_t n, int64_t nrhs, double* dB, int64_t ldb, const double* w,
                       int64_t depth, int64_t nb, slt_stream_t stream);
int slt_drbt_diag_device(int64_t n, int64_t seed, double* w, slt_stream_t stream);
/* slate::posv_mixed, src/posv_mixed.cc:105-320 (A lower) */
int slt_dsposv_device(int64_t n, int64_t nrhs, double* dA, int64_t lda, const double* dB,
                      int64_t ldb, double* dX, int64_t ldx, const slt_options* opts,
                      slt_stream_t stream, int* iter, int64_t* info);
/* slate::posv_mixed_gmres, src/posv_mixed_gmres.cc:109-436 (A lower) */
int slt_dsposv_gmres_device(int64_t n, int64_t nrhs, double* dA, int64_t lda, const double* dB,
                            int64_t ldb, double* dX, int64_t ldx, const slt_options* opts,
                            slt_stream_t stream, int* iter, int64_t* info);

/* Single precision forms of getrs (Trans / ConjTrans), potrs and posv
 * (lower), as the double ones above. */
int slt_sgetrs_trans_device(char trans, int64_t n, int64_t nrhs, const float* dLU, int64_t lda,
                            const int* d_ipiv, float* dB, int64_t ldb, const slt_options* opts,
                            slt_stream_t stream);
int slt_spotrs_device(int64_t n, int64_t nrhs, const float* dL, int64_t lda, float* dB, int64_t ldb,
                      const slt_options* opts, slt_stream_t stream);
int slt_sposv_device(int64_t n, int64_t nrhs, float* dA, int64_t lda, float* dB, int64_t ldb,
                     const slt_options* opts, slt_stream_t stream, int64_t* info);

/* Complex precisions: 'c' = complex<float>, 'z' = complex<double>.  Arrays
 * are column-major with interleaved (real, imaginary) pairs, the layout of
 * std::complex, C99 _Complex and cuComplex; pivots and info as for the real
 * forms; the Cholesky forms use the lower triangle of a Hermitian matrix.
 * SLATE's complex instantiations of getrf / getrs (trans 'N', 'T', 'C') /
 * gesv / potrf / potrs / posv (src/getrf.cc, src/getrs.cc, src/gesv.cc,
 * src/potrf.cc, src/potrs.cc, src/posv.cc). */
int slt_cgetrf_device(int64_t m, int64_t n, void* dA, int64_t lda, int* d_ipiv, const slt_options* opts,
                      slt_stream_t stream, int64_t* info);
int slt_zgetrf_device(int64_t m, int64_t n, void* dA, int64_t lda, int* d_ipiv, const slt_options* opts,
                      slt_stream_t stream, int64_t* info);
int slt_cgetrs_device(char trans, int64_t n, int64_t nrhs, const void* dLU, int64_t lda, const int* d_ipiv,
                      void* dB, int64_t ldb, const slt_options* opts, slt_stream_t stream);
int slt_zgetrs_device(char trans, int64_t n, int64_t nrhs, const void* dLU, int64_t lda, const int* d_ipiv,
                      void* dB, int64_t ldb, const slt_options* opts, slt_stream_t stream);
int slt_cgesv_device(int64_t n, int64_t nrhs, void* dA, int64_t lda, int* d_ipiv, void* dB, int64_t ldb,
                     const slt_options* opts, slt_stream_t stream, int64_t* info);
int slt_zgesv_device(int64_t n, int64_t nrhs, void* dA, int64_t lda, int* d_ipiv, void* dB, int64_t ldb,
                     const slt_options* opts, slt_stream_t stream, int64_t* info);
int slt_cpotrf_device(int64_t n, void* dA, int64_t lda, const slt_options* opts, slt_stream_t stream,
                      int64_t* info);
int slt_zpotrf_device(int64_t n, void* dA, int64_t lda, const slt_options* opts, slt_stream_t stream,
                      int64_t* info);
int slt_cpotrs_device(int64_t n, int64_t nrhs, const void* dL, int64_t lda, void* dB, int64_t ldb,
                      const slt_options* opts, slt_stream_t stream);
int slt_zpotrs_device(int64_t n, int64_t nrhs, const void* dL, int64_t lda, void* dB, int64_t ldb,
                      const slt_options* opts, slt_stream_t stream);
int slt_cposv_device(int64_t n, int64_t nrhs, void* dA, int64_t lda, void* dB, int64_t ldb,
                     const slt_options* opts, slt_stream_t stream, int64_t* info);
int slt_zposv_device(int64_t n, int64_t nrhs, void* dA, int64_t lda, void* dB, int64_t ldb,
                     const slt_options* opts, slt_stream_t stream, int64_t* info);
/* slate::gesv_mixed<complex<double>, complex<float>>, src/gesv_mixed.cc:105-289
 * (complex<float> LU, complex<double> refinement, fallback to a complex<double>
 * LU; A unchanged unless the fallback ran). */
int slt_zcgesv_device(int64_t n, int64_t nrhs, void* dA, int64_t lda, int* d_ipiv, const void* dB, int64_t ldb,
                      void* dX, int64_t ldx, const slt_options* opts, slt_stream_t stream, int* iter,
                      int64_t* info);

/* FP64 residual R = B - A X (A n x n general, or symmetric with lower
 * storage when sym_lower != 0), as the kernel layer's slt_dresidual
 * computes it, but with no device allocation and no caller scratch.  It is
 * for callers that cannot allocate device memory where they need a residual:
 * programs whose device memory belongs to their own pool or to a framework
 * allocator that forbids side allocations, and code that must not call
 * cudaMalloc / cudaFree (which can synchronise the whole device) at that
 * point.  Its partial sums live in one 16 MiB library-owned __device__ array
 * per device, held until the process exits, so n * min(nrhs, 16) may not
 * exceed 2,097,152 (else SLT_ERR_LIMIT, nothing launched).  Calls that
 * overlap on the GPU share that array and race: serialise them.  The first
 * call on a device looks up the array's device address (with that device
 * current) and should come before any stream capture.  No counterpart in
 * SLATE. */
int slt_dresidual_noalloc(int64_t n, int64_t nrhs, const double* dA, int64_t lda, int sym_lower,
                          const double* dB, int64_t ldb, const double* dX, int64_t ldx,
                          double* dR, int64_t ldr, slt_stream_t stream);

/* ------------------------------------------------------------------------- */
/* Variable-size batched solves.  No counterpart in SLATE, which has no      */
/* batched routine; each system follows slate::gesv (kind 0: LU with partial */
/* pivoting, lowest row index on ties) or slate::posv (kind 1: SPD, lower    */
/* Cholesky).  Every argument array is a DEVICE array of `batch` entries:    */
/* kind, n (0..2048), nrhs, the column-major matrices A[i] (lda[i] >= n[i]),  */
/* pivots ipiv[i] (LU only, n[i] ints, LAPACK 1-based), right-hand sides     */
/* B[i] (ldb[i]).  The call copies the size and pointer arrays to the host   */
/* once, orders the systems largest first and runs one persistent launch.    */

/* FP64: A[i] <- factors, B[i] <- X[i]; info[i] as slate::gesv / posv. */
int slt_dsolve_vbatched(int64_t batch, const int* d_kind, const int* d_n, const int* d_nrhs,
                        double* const* d_A, const int* d_lda, int* const* d_ipiv,
                        double* const* d_B, const int* d_ldb, int* d_info, slt_stream_t stream);

/* Mixed: FP32 factors (one launch), FP64 refinement with slate::gesv_mixed's
 * stopping test replayed itermax + 1 times from a CUDA graph, FP64 fallback
 * for the systems that do not converge (their A[i] then holds FP64 factors;
 * A[i] and B[i] are untouched otherwise).  X[i] (ldx[i]) receives the
 * solution, iter[i] / info[i] follow slate::gesv_mixed (0..itermax, -3,
 * -(itermax+1)).  nrhs[i] <= 8; tolerance <= 0 means eps * sqrt(n[i]). */
int slt_dsolve_mixed_vbatched(int64_t batch, const int* d_kind, const int* d_n, const int* d_nrhs,
                              double* const* d_A, const int* d_lda, int* const* d_ipiv,
                              double* const* d_B, const int* d_ldb, double* const* d_X,
                              const int* d_ldx, int* d_iter, int* d_info, int64_t itermax,
                              double tolerance, int use_fallback, slt_stream_t stream);

/* Philox test-matrix generator, same values as slate::random::generate
 * (matgen/random.cc:197-230) for the uniform distributions. */
int slt_dgenerate_device(int dist, int64_t seed, int64_t m, int64_t n, int64_t ioff, int64_t joff,
                         double* dA, int64_t lda, slt_stream_t stream);

/* Launch accounting: number of kernels this library has launched so far
 * (all classes), and optional CUDA-event timing of each launch by kernel
 * class (1 FP64 update GEMM, 2 FP32 update GEMM, 3 tensor-core update GEMM,
 * 4 LU panel, 5 triangular solves, 6 row interchanges, 7 skinny products,
 * 8 diagonal-block Cholesky).  slt_profile_enable(1) clears and starts
 * recording; slt_profile_read synchronises the device and sums one class:
 * algorithmic flops and bytes, event-timed seconds and launches. */
long long slt_launch_count(void);
void slt_profile_enable(int on);
int slt_profile_read(int kind, double* flops, double* bytes, double* seconds, long long* launches);

/* Device workspace of the drivers comes from a stream-ordered pool owned by
 * the library, one per device, which keeps freed memory reserved for the
 * next call (a repeated solve does not map its workspace afresh).  This
 * returns the pool's unused memory on the current device to the system
 * (synchronises the device).  SLATE frees its workspace with
 * Matrix::releaseWorkspace (include/slate/BaseMatrix.hh). */
int slt_release_workspace(void);

/* Memory helpers of the header-only C++ API (include/slate_gb300.hh), which
 * keeps SLATE's tile storage (slate::MatrixStorage, include/slate/internal/
 * MatrixStorage.hh) without including CUDA headers: device allocation on the
 * current device, a synchronous 2-D copy between any host / device pointers
 * (unified addressing picks the direction), and whether a pointer is device
 * (or managed) memory. */
int slt_device_malloc(size_t bytes, void** p);
int slt_device_free(void* p);
int slt_memcpy2d(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, size_t height);
int slt_is_device_pointer(const void* p);

/* Type-generic device helpers (type 0 float, 1 double, 2 complex<float>,
 * 3 complex<double>; stream 0 = the default stream): B (n x m) = A^T, or A^H
 * when conj != 0; the lower (upper = 0) or upper (upper = 1) triangle of D
 * <- S.  No counterpart in SLATE (its Tile transposes are host / BLAS++). */
int slt_xtranspose(int type, int64_t m, int64_t n, const void* A, int64_t lda, void* B, int64_t ldb, int conj,
                   slt_stream_t stream);
int slt_xcopy_tri(int type, int upper, int64_t n, const void* S, int64_t lds, void* D, int64_t ldd,
                  slt_stream_t stream);

/* Seconds spent in named phases of the last driver call on this thread
 * (the keys of SLATE's slate::timers map, e.g. "gesv_mixed::getrf_lo");
 * returns -1 if the key is unknown. */
double slt_timer(const char* name);

/* ------------------------------------------------------------------------- */
/* LAPACK-compatible entry points (lapack_api/lapack_*.cc).  Host memory.     */
/* Tile size from SLATE_LAPACK_NB (default 512), inner blocking from          */
/* SLATE_LAPACK_IB (default 32), factorisation precision of the mixed solvers */
/* from SLATE_LAPACK_FACTOR_PRECISION (fp32 | tf32 | tf32x3 | bf16 | fp16 |   */
/* fp8, default fp32), their refinement from SLATE_LAPACK_REFINE (ir | gmres  */
/* | ir+gmres, default ir).                                                   */

/* lapack_api/lapack_gesv.cc:32 */
void slate_dgesv(const int* n, const int* nrhs, double* a, const int* lda, int* ipiv,
                 double* b, const int* ldb, int* info);
void slate_sgesv(const int* n, const int* nrhs, float* a, const int* lda, int* ipiv,
                 float* b, const int* ldb, int* info);
/* lapack_api/lapack_getrf.cc */
void slate_dgetrf(const int* m, const int* n, double* a, const int* lda, int* ipiv, int* info);
void slate_sgetrf(const int* m, const int* n, float* a, const int* lda, int* ipiv, int* info);
/* lapack_api/lapack_getrs.cc:29 (trans 'N' only) */
void slate_dgetrs(const char* trans, const int* n, const int* nrhs, double* a, const int* lda,
                  int* ipiv, double* b, const int* ldb, int* info);
/* lapack_api/lapack_gesv_mixed.cc:24 (dsgesv signature; x receives the solution) */
void slate_dsgesv(const int* n, const int* nrhs, double* a, const int* lda, int* ipiv,
                  double* b, const int* ldb, double* x, const int* ldx, double* work,
                  float* swork, int* iter, int* info);
/* LAPACK dsposv signature (mixed-precision Cholesky solve; SLATE's C++
 * posv_mixed, src/posv_mixed.cc:105-320, has no lapack_api wrapper) */
void slate_dsposv(const char* uplo, const int* n, const int* nrhs, double* a, const int* lda,
                  double* b, const int* ldb, double* x, const int* ldx, double* work,
                  float* swork, int* iter, int* info);
/* lapack_api/lapack_posv.cc:32 (uplo 'L' or 'U') */
void slate_dposv(const char* uplo, const int* n, const int* nrhs, double* a, const int* lda,
                 double* b, const int* ldb, int* info);
/* lapack_api/lapack_potrf.cc:30 */
void slate_dpotrf(const char* uplo, const int* n, double* a, const int* lda, int* info);

void slate_dgesv_(const int* n, const int* nrhs, double* a, const int* lda, int* ipiv,
                  double* b, const int* ldb, int* info);
void slate_sgesv_(const int* n, const int* nrhs, float* a, const int* lda, int* ipiv,
                  float* b, const int* ldb, int* info);
void slate_dgetrf_(const int* m, const int* n, double* a, const int* lda, int* ipiv, int* info);
void slate_sgetrf_(const int* m, const int* n, float* a, const int* lda, int* ipiv, int* info);
void slate_dgetrs_(const char* trans, const int* n, const int* nrhs, double* a, const int* lda,
                   int* ipiv, double* b, const int* ldb, int* info);
void slate_dsgesv_(const int* n, const int* nrhs, double* a, const int* lda, int* ipiv,
                   double* b, const int* ldb, double* x, const int* ldx, double* work,
                   float* swork, int* iter, int* info);
void slate_dsposv_(const char* uplo, const int* n, const int* nrhs, double* a, const int* lda,
                   double* b, const int* ldb, double* x, const int* ldx, double* work,
                   float* swork, int* iter, int* info);
void slate_dposv_(const char* uplo, const int* n, const int* nrhs, double* a, const int* lda,
                  double* b, const int* ldb, int* info);
void slate_dpotrf_(const char* uplo, const int* n, double* a, const int* lda, int* info);
/* The other precisions of the same entry points (lapack_api/lapack_gesv.cc:
 * 25-45, lapack_getrf.cc, lapack_getrs.cc:19-22, lapack_posv.cc:22-25,
 * lapack_potrf.cc:20-23, lapack_gesv_mixed.cc:30-33), each also exported with
 * a trailing underscore.  Complex arrays (void*) hold interleaved (real,
 * imaginary) pairs: std::complex, C99 _Complex, Fortran COMPLEX. */
void slate_sgetrs(const char* trans, const int* n, const int* nrhs, float* a, const int* lda, int* ipiv,
                  float* b, const int* ldb, int* info);
void slate_cgetrs(const char* trans, const int* n, const int* nrhs, void* a, const int* lda, int* ipiv,
                  void* b, const int* ldb, int* info);
void slate_zgetrs(const char* trans, const int* n, const int* nrhs, void* a, const int* lda, int* ipiv,
                  void* b, const int* ldb, int* info);
void slate_cgesv(const int* n, const int* nrhs, void* a, const int* lda, int* ipiv, void* b, const int* ldb,
                 int* info);
void slate_zgesv(const int* n, const int* nrhs, void* a, const int* lda, int* ipiv, void* b, const int* ldb,
                 int* info);
void slate_cgetrf(const int* m, const int* n, void* a, const int* lda, int* ipiv, int* info);
void slate_zgetrf(const int* m, const int* n, void* a, const int* lda, int* ipiv, int* info);
void slate_sposv(const char* uplo, const int* n, const int* nrhs, float* a, const int* lda, float* b,
                 const int* ldb, int* info);
void slate_cposv(const char* uplo, const int* n, const int* nrhs, void* a, const int* lda, void* b,
                 const int* ldb, int* info);
void slate_zposv(const char* uplo, const int* n, const int* nrhs, void* a, const int* lda, void* b,
                 const int* ldb, int* info);
void slate_spotrf(const char* uplo, const int* n, float* a, const int* lda, int* info);
void slate_cpotrf(const char* uplo, const int* n, void* a, const int* lda, int* info);
void slate_zpotrf(const char* uplo, const int* n, void* a, const int* lda, int* info);
void slate_zcgesv(const int* n, const int* nrhs, void* a, const int* lda, int* ipiv, void* b, const int* ldb,
                  void* x, const int* ldx, void* work, void* swork, int* iter, int* info);
void slate_sgetrs_(const char* trans, const int* n, const int* nrhs, float* a, const int* lda, int* ipiv,
                   float* b, const int* ldb, int* info);
void slate_cgetrs_(const char* trans, const int* n, const int* nrhs, void* a, const int* lda, int* ipiv,
                   void* b, const int* ldb, int* info);
void slate_zgetrs_(const char* trans, const int* n, const int* nrhs, void* a, const int* lda, int* ipiv,
                   void* b, const int* ldb, int* info);
void slate_cgesv_(const int* n, const int* nrhs, void* a, const int* lda, int* ipiv, void* b, const int* ldb,
                  int* info);
void slate_zgesv_(const int* n, const int* nrhs, void* a, const int* lda, int* ipiv, void* b, const int* ldb,
                  int* info);
void slate_cgetrf_(const int* m, const int* n, void* a, const int* lda, int* ipiv, int* info);
void slate_zgetrf_(const int* m, const int* n, void* a, const int* lda, int* ipiv, int* info);
void slate_sposv_(const char* uplo, const int* n, const int* nrhs, float* a, const int* lda, float* b,
                  const int* ldb, int* info);
void slate_cposv_(const char* uplo, const int* n, const int* nrhs, void* a, const int* lda, void* b,
                  const int* ldb, int* info);
void slate_zposv_(const char* uplo, const int* n, const int* nrhs, void* a, const int* lda, void* b,
                  const int* ldb, int* info);
void slate_spotrf_(const char* uplo, const int* n, float* a, const int* lda, int* info);
void slate_cpotrf_(const char* uplo, const int* n, void* a, const int* lda, int* info);
void slate_zpotrf_(const char* uplo, const int* n, void* a, const int* lda, int* info);
void slate_zcgesv_(const int* n, const int* nrhs, void* a, const int* lda, int* ipiv, void* b, const int* ldb,
                   void* x, const int* ldx, void* work, void* swork, int* iter, int* info);
/* lapack_api/lapack_getri.cc, lapack_potri.cc, lapack_gecon.cc, lapack_pocon.cc
 * (gecon / pocon take the factors without pivots, as LAPACK's do; work and
 * iwork are not used) */
void slate_dgetri(const int* n, double* a, const int* lda, int* ipiv, double* work, const int* lwork, int* info);
void slate_dgetri_(const int* n, double* a, const int* lda, int* ipiv, double* work, const int* lwork, int* info);
void slate_dpotri(const char* uplo, const int* n, double* a, const int* lda, int* info);
void slate_dpotri_(const char* uplo, const int* n, double* a, const int* lda, int* info);
void slate_dgecon(const char* norm, const int* n, double* a, const int* lda, double* anorm, double* rcond,
                  double* work, int* iwork, int* info);
void slate_dgecon_(const char* norm, const int* n, double* a, const int* lda, double* anorm, double* rcond,
                   double* work, int* iwork, int* info);
void slate_dpocon(const char* uplo, const int* n, double* a, const int* lda, double* anorm, double* rcond,
                  double* work, int* iwork, int* info);
void slate_dpocon_(const char* uplo, const int* n, double* a, const int* lda, double* anorm, double* rcond,
                   double* work, int* iwork, int* info);

#ifdef __cplusplus
}
#endif

#endif /* SLATE_GB300_H */
