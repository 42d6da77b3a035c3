/* slate_scalapack.h -- ScaLAPACK-compatible entry points of libslate_gb300.so
 * on a 1 x 1 process grid.
 *
 * Each replaces the SLATE wrapper of the same name in scalapack_api/ and takes
 * the same arguments (Fortran calling convention: every argument by pointer,
 * 1-based ia / ja, 9-entry descriptors).  With one process the local array is
 * the whole matrix, element (i, j) at a[(i - 1) + (j - 1) * LLD].  The
 * descriptor must be of type 1 (BLOCK_CYCLIC_2D) with RSRC = CSRC = 0 and
 * LLD >= max(1, M); its context is not queried (no BLACS); MB is the tile size
 * nb.  A bad descriptor entry k of argument p gives info = -(100 p + k).
 * Environment: SLATE_SCALAPACK_IB (inner blocking, default 16),
 * SLATE_SCALAPACK_LOOKAHEAD; the factor precision of pdsgesv follows
 * SLATE_LAPACK_FACTOR_PRECISION.
 *
 * IPIV(ia - 1 + r) receives the global row that row ia - 1 + r was swapped
 * with.  info is the driver's: > 0 for an exactly singular / not positive
 * definite matrix (SLATE's pdgesv_ wrapper returns 0 there).
 *
 * Exported with and without the trailing underscore (the two Fortran
 * manglings SLATE exports).
 */
#ifndef SLATE_SCALAPACK_H
#define SLATE_SCALAPACK_H

#ifdef __cplusplus
extern "C" {
#endif

/* scalapack_api/scalapack_gesv.cc:41-56 (pdgesv_), :31-36 (psgesv_) */
void pdgesv_(const int* n, const int* nrhs, double* a, const int* ia, const int* ja, const int* desca, int* ipiv,
             double* b, const int* ib, const int* jb, const int* descb, int* info);
void psgesv_(const int* n, const int* nrhs, float* a, const int* ia, const int* ja, const int* desca, int* ipiv,
             float* b, const int* ib, const int* jb, const int* descb, int* info);
/* scalapack_api/scalapack_getrf.cc:46-54 */
void pdgetrf_(const int* m, const int* n, double* a, const int* ia, const int* ja, const int* desca, int* ipiv,
              int* info);
void psgetrf_(const int* m, const int* n, float* a, const int* ia, const int* ja, const int* desca, int* ipiv,
              int* info);
/* scalapack_api/scalapack_getrs.cc:46-54 */
void pdgetrs_(const char* trans, const int* n, const int* nrhs, double* a, const int* ia, const int* ja,
              const int* desca, int* ipiv, double* b, const int* ib, const int* jb, const int* descb, int* info);
/* scalapack_api/scalapack_gesv_mixed.cc:31-39 */
void pdsgesv_(const int* n, const int* nrhs, double* a, const int* ia, const int* ja, const int* desca, int* ipiv,
              double* b, const int* ib, const int* jb, const int* descb, double* x, const int* ix, const int* jx,
              const int* descx, int* iter, int* info);
/* scalapack_api/scalapack_posv.cc:49-57 */
void pdposv_(const char* uplo, const int* n, const int* nrhs, double* a, const int* ia, const int* ja,
             const int* desca, double* b, const int* ib, const int* jb, const int* descb, int* info);
/* scalapack_api/scalapack_potrf.cc:49-57 */
void pdpotrf_(const char* uplo, const int* n, double* a, const int* ia, const int* ja, const int* desca, int* info);
/* scalapack_api/scalapack_potrs.cc:49-57 */
void pdpotrs_(const char* uplo, const int* n, const int* nrhs, double* a, const int* ia, const int* ja,
              const int* desca, double* b, const int* ib, const int* jb, const int* descb, int* info);
/* scalapack_api/scalapack_getri.cc:46-54 (no host workspace needed: a query returns 1) */
void pdgetri_(const int* n, double* a, const int* ia, const int* ja, const int* desca, int* ipiv, double* work,
              const int* lwork, int* iwork, const int* liwork, int* info);
/* scalapack_api/scalapack_potri.cc:49-57 */
void pdpotri_(const char* uplo, const int* n, double* a, const int* ia, const int* ja, const int* desca, int* info);
/* scalapack_api/scalapack_gecon.cc:46-54, scalapack_pocon.cc:46-54 (from the factors) */
void pdgecon_(const char* norm, const int* n, double* a, const int* ia, const int* ja, const int* desca,
              const double* anorm, double* rcond, double* work, const int* lwork, int* iwork, const int* liwork,
              int* info);
void pdpocon_(const char* uplo, const int* n, double* a, const int* ia, const int* ja, const int* desca,
              const double* anorm, double* rcond, double* work, const int* lwork, int* iwork, const int* liwork,
              int* info);

/* the same entry points without the trailing underscore */
void pdgesv(const int* n, const int* nrhs, double* a, const int* ia, const int* ja, const int* desca, int* ipiv,
            double* b, const int* ib, const int* jb, const int* descb, int* info);
void psgesv(const int* n, const int* nrhs, float* a, const int* ia, const int* ja, const int* desca, int* ipiv,
            float* b, const int* ib, const int* jb, const int* descb, int* info);
void pdgetrf(const int* m, const int* n, double* a, const int* ia, const int* ja, const int* desca, int* ipiv,
             int* info);
void psgetrf(const int* m, const int* n, float* a, const int* ia, const int* ja, const int* desca, int* ipiv,
             int* info);
void pdgetrs(const char* trans, const int* n, const int* nrhs, double* a, const int* ia, const int* ja,
             const int* desca, int* ipiv, double* b, const int* ib, const int* jb, const int* descb, int* info);
void pdsgesv(const int* n, const int* nrhs, double* a, const int* ia, const int* ja, const int* desca, int* ipiv,
             double* b, const int* ib, const int* jb, const int* descb, double* x, const int* ix, const int* jx,
             const int* descx, int* iter, int* info);
void pdposv(const char* uplo, const int* n, const int* nrhs, double* a, const int* ia, const int* ja,
            const int* desca, double* b, const int* ib, const int* jb, const int* descb, int* info);
void pdpotrf(const char* uplo, const int* n, double* a, const int* ia, const int* ja, const int* desca, int* info);
void pdpotrs(const char* uplo, const int* n, const int* nrhs, double* a, const int* ia, const int* ja,
             const int* desca, double* b, const int* ib, const int* jb, const int* descb, int* info);
void pdgetri(const int* n, double* a, const int* ia, const int* ja, const int* desca, int* ipiv, double* work,
             const int* lwork, int* iwork, const int* liwork, int* info);
void pdpotri(const char* uplo, const int* n, double* a, const int* ia, const int* ja, const int* desca, int* info);
void pdgecon(const char* norm, const int* n, double* a, const int* ia, const int* ja, const int* desca,
             const double* anorm, double* rcond, double* work, const int* lwork, int* iwork, const int* liwork,
             int* info);
void pdpocon(const char* uplo, const int* n, double* a, const int* ia, const int* ja, const int* desca,
             const double* anorm, double* rcond, double* work, const int* lwork, int* iwork, const int* liwork,
             int* info);

#ifdef __cplusplus
}
#endif

#endif /* SLATE_SCALAPACK_H */
