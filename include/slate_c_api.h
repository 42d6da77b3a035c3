/* slate_c_api.h -- SLATE's C API (opaque matrices, pivots and options) for
 * the single-GPU LU / Cholesky solve path, served by libslate_gb300.so.
 *
 * Names and argument meaning follow SLATE's generated C API
 * (tools/c_api/generate_matrix.py, src/c_api/wrappers.cc:692-1080,
 * include/slate/c_api/types.h), for single and double precision, real
 * (r32, r64) and complex (c32, c64):
 *   slate_Options_create / _destroy / _copy / _set_<Option> / _get_<Option>
 *   slate_Pivots_create / _destroy
 *   slate_Matrix_create_fromScaLAPACK_{r32,r64} / slate_Matrix_destroy_*
 *   slate_HermitianMatrix_create_fromScaLAPACK_r64 / _destroy_r64
 *   slate_lu_solve_*, slate_lu_factor_*, slate_lu_solve_using_factor_*
 *   slate_chol_solve_r64, slate_chol_factor_r64, slate_chol_solve_using_factor_r64
 *
 * Differences a caller sees:
 *  - the process grid must be 1 x 1 (p = q = 1) and mb = nb; the MPI
 *    communicator argument is accepted and ignored (no MPI is needed);
 *  - the wrapped memory may be host or device memory (any pointer the CUDA
 *    runtime can address); host data are staged to the GPU for each call;
 *  - SLATE's C wrappers return void and report errors by C++ exceptions; here
 *    the calls return void as well and the outcome of the last call on the
 *    calling thread is read with slate_gb300_last_info() (SLATE's info) and
 *    slate_gb300_last_status() (0, or an slt status code).
 */
#ifndef SLATE_GB300_C_API_H
#define SLATE_GB300_C_API_H

#include <stdbool.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef intptr_t slate_mpi_comm_t;   /* MPI_Comm placeholder, ignored */

typedef char slate_Uplo;             /* 'U', 'L' (include/slate/c_api/types.h) */
typedef char slate_Target;           /* 'H', 'T', 'N', 'B', 'D' */
typedef char slate_MethodLU;         /* '*', 'P', 'N' (NoPiv), 'C' (CALU) supported; 'R', 'B' rejected */
typedef char slate_Norm;             /* '1' / 'O' (one norm), 'I' (infinity norm) */

typedef void* slate_Options;
typedef struct slate_Pivots_struct* slate_Pivots;
typedef struct slate_Matrix_struct_r64* slate_Matrix_r64;
typedef struct slate_Matrix_struct_r32* slate_Matrix_r32;
typedef struct slate_HermitianMatrix_struct_r64* slate_HermitianMatrix_r64;
typedef struct slate_Matrix_struct_c32* slate_Matrix_c32;
typedef struct slate_Matrix_struct_c64* slate_Matrix_c64;
typedef struct slate_HermitianMatrix_struct_r32* slate_HermitianMatrix_r32;
typedef struct slate_HermitianMatrix_struct_c32* slate_HermitianMatrix_c32;
typedef struct slate_HermitianMatrix_struct_c64* slate_HermitianMatrix_c64;

slate_Options slate_Options_create(void);
void slate_Options_destroy(slate_Options opts);
void slate_Options_copy(slate_Options opts1, slate_Options opts2);   /* opts1 = opts2 */

void    slate_Options_set_ChunkSize(slate_Options opts, int64_t value);
int64_t slate_Options_get_ChunkSize(slate_Options opts, int64_t defval);
void    slate_Options_set_Lookahead(slate_Options opts, int64_t value);
int64_t slate_Options_get_Lookahead(slate_Options opts, int64_t defval);
void    slate_Options_set_BlockSize(slate_Options opts, int64_t value);
int64_t slate_Options_get_BlockSize(slate_Options opts, int64_t defval);
void    slate_Options_set_InnerBlocking(slate_Options opts, int64_t value);
int64_t slate_Options_get_InnerBlocking(slate_Options opts, int64_t defval);
void    slate_Options_set_MaxPanelThreads(slate_Options opts, int64_t value);
int64_t slate_Options_get_MaxPanelThreads(slate_Options opts, int64_t defval);
void    slate_Options_set_Tolerance(slate_Options opts, double value);
double  slate_Options_get_Tolerance(slate_Options opts, double defval);
void    slate_Options_set_Target(slate_Options opts, slate_Target value);
slate_Target slate_Options_get_Target(slate_Options opts, slate_Target defval);
void    slate_Options_set_HoldLocalWorkspace(slate_Options opts, bool value);
bool    slate_Options_get_HoldLocalWorkspace(slate_Options opts, bool defval);
void    slate_Options_set_Depth(slate_Options opts, int64_t value);
int64_t slate_Options_get_Depth(slate_Options opts, int64_t defval);
void    slate_Options_set_MaxIterations(slate_Options opts, int64_t value);
int64_t slate_Options_get_MaxIterations(slate_Options opts, int64_t defval);
void    slate_Options_set_UseFallbackSolver(slate_Options opts, bool value);
bool    slate_Options_get_UseFallbackSolver(slate_Options opts, bool defval);
void    slate_Options_set_PivotThreshold(slate_Options opts, double value);
double  slate_Options_get_PivotThreshold(slate_Options opts, double defval);
void    slate_Options_set_MethodLU(slate_Options opts, slate_MethodLU value);
slate_MethodLU slate_Options_get_MethodLU(slate_Options opts, slate_MethodLU defval);

slate_Pivots slate_Pivots_create(void);
void slate_Pivots_destroy(slate_Pivots pivots);

slate_Matrix_r64 slate_Matrix_create_fromScaLAPACK_r64(int64_t m, int64_t n, double* A, int64_t lda, int64_t mb,
                                                       int64_t nb, int p, int q, slate_mpi_comm_t mpi_comm);
slate_Matrix_r32 slate_Matrix_create_fromScaLAPACK_r32(int64_t m, int64_t n, float* A, int64_t lda, int64_t mb,
                                                       int64_t nb, int p, int q, slate_mpi_comm_t mpi_comm);
void slate_Matrix_destroy_r64(slate_Matrix_r64 A);
void slate_Matrix_destroy_r32(slate_Matrix_r32 A);
int64_t slate_Matrix_m_r64(slate_Matrix_r64 A);
int64_t slate_Matrix_n_r64(slate_Matrix_r64 A);

slate_HermitianMatrix_r64 slate_HermitianMatrix_create_fromScaLAPACK_r64(slate_Uplo uplo, int64_t n, double* A,
                                                                         int64_t lda, int64_t nb, int p, int q,
                                                                         slate_mpi_comm_t mpi_comm);
void slate_HermitianMatrix_destroy_r64(slate_HermitianMatrix_r64 A);

/* slate::lu_solve = gesv, lu_factor = getrf, lu_solve_using_factor = getrs */
void slate_lu_solve_r64(slate_Matrix_r64 A, slate_Matrix_r64 B, slate_Options opts);
void slate_lu_factor_r64(slate_Matrix_r64 A, slate_Pivots pivots, slate_Options opts);
void slate_lu_solve_using_factor_r64(slate_Matrix_r64 A, slate_Pivots pivots, slate_Matrix_r64 B,
                                     slate_Options opts);
void slate_lu_solve_r32(slate_Matrix_r32 A, slate_Matrix_r32 B, slate_Options opts);
void slate_lu_factor_r32(slate_Matrix_r32 A, slate_Pivots pivots, slate_Options opts);
void slate_lu_solve_using_factor_r32(slate_Matrix_r32 A, slate_Pivots pivots, slate_Matrix_r32 B,
                                     slate_Options opts);

/* MethodLU::NoPiv forms (src/c_api/wrappers.cc:715-880): getrf_nopiv has no
 * pivots; solve_using_factor_nopiv applies none. */
void slate_lu_solve_nopiv_r64(slate_Matrix_r64 A, slate_Matrix_r64 B, slate_Options opts);
void slate_lu_factor_nopiv_r64(slate_Matrix_r64 A, slate_Options opts);
void slate_lu_solve_using_factor_nopiv_r64(slate_Matrix_r64 A, slate_Matrix_r64 B, slate_Options opts);
void slate_lu_solve_nopiv_r32(slate_Matrix_r32 A, slate_Matrix_r32 B, slate_Options opts);
void slate_lu_factor_nopiv_r32(slate_Matrix_r32 A, slate_Options opts);
void slate_lu_solve_using_factor_nopiv_r32(slate_Matrix_r32 A, slate_Matrix_r32 B, slate_Options opts);

/* slate::lu_inverse_using_factor (getri) in place and out of place, and
 * lu_rcondest_using_factor (gecondest: the pivots do not change the 1- or
 * infinity-norm of A^{-1}) (src/c_api/wrappers.cc:882-945). */
void slate_lu_inverse_using_factor_r64(slate_Matrix_r64 A, slate_Pivots pivots, slate_Options opts);
void slate_lu_inverse_using_factor_out_of_place_r64(slate_Matrix_r64 A, slate_Pivots pivots,
                                                    slate_Matrix_r64 A_inverse, slate_Options opts);
double slate_lu_rcondest_using_factor_r64(slate_Norm norm, slate_Matrix_r64 A, double Anorm, slate_Options opts);

/* slate::chol_solve = posv, chol_factor = potrf, chol_solve_using_factor = potrs */
void slate_chol_solve_r64(slate_HermitianMatrix_r64 A, slate_Matrix_r64 B, slate_Options opts);
void slate_chol_factor_r64(slate_HermitianMatrix_r64 A, slate_Options opts);
void slate_chol_solve_using_factor_r64(slate_HermitianMatrix_r64 A, slate_Matrix_r64 B, slate_Options opts);
/* slate::chol_inverse_using_factor (potri) and chol_rcondest_using_factor
 * (pocondest) (src/c_api/wrappers.cc:1083-1130) */
void slate_chol_inverse_using_factor_r64(slate_HermitianMatrix_r64 A, slate_Options opts);
double slate_chol_rcondest_using_factor_r64(slate_Norm norm, slate_HermitianMatrix_r64 A, double Anorm,
                                            slate_Options opts);

/* Complex precisions (c32 = complex<float>, c64 = complex<double>; the
 * arrays hold interleaved real and imaginary parts, the layout of C99
 * float/double _Complex) and the single-precision Cholesky forms: SLATE's
 * c32 / c64 / r32 instantiations of the same wrappers
 * (src/c_api/wrappers.cc:692-1080). */
slate_Matrix_c32 slate_Matrix_create_fromScaLAPACK_c32(int64_t m, int64_t n, void* A, int64_t lda, int64_t mb,
                                                       int64_t nb, int p, int q, slate_mpi_comm_t mpi_comm);
slate_Matrix_c64 slate_Matrix_create_fromScaLAPACK_c64(int64_t m, int64_t n, void* A, int64_t lda, int64_t mb,
                                                       int64_t nb, int p, int q, slate_mpi_comm_t mpi_comm);
void slate_Matrix_destroy_c32(slate_Matrix_c32 A);
void slate_Matrix_destroy_c64(slate_Matrix_c64 A);
slate_HermitianMatrix_r32 slate_HermitianMatrix_create_fromScaLAPACK_r32(slate_Uplo uplo, int64_t n, float* A,
                                                                         int64_t lda, int64_t nb, int p, int q,
                                                                         slate_mpi_comm_t mpi_comm);
slate_HermitianMatrix_c32 slate_HermitianMatrix_create_fromScaLAPACK_c32(slate_Uplo uplo, int64_t n, void* A,
                                                                         int64_t lda, int64_t nb, int p, int q,
                                                                         slate_mpi_comm_t mpi_comm);
slate_HermitianMatrix_c64 slate_HermitianMatrix_create_fromScaLAPACK_c64(slate_Uplo uplo, int64_t n, void* A,
                                                                         int64_t lda, int64_t nb, int p, int q,
                                                                         slate_mpi_comm_t mpi_comm);
void slate_HermitianMatrix_destroy_r32(slate_HermitianMatrix_r32 A);
void slate_HermitianMatrix_destroy_c32(slate_HermitianMatrix_c32 A);
void slate_HermitianMatrix_destroy_c64(slate_HermitianMatrix_c64 A);

void slate_lu_solve_c32(slate_Matrix_c32 A, slate_Matrix_c32 B, slate_Options opts);
void slate_lu_factor_c32(slate_Matrix_c32 A, slate_Pivots pivots, slate_Options opts);
void slate_lu_solve_using_factor_c32(slate_Matrix_c32 A, slate_Pivots pivots, slate_Matrix_c32 B,
                                     slate_Options opts);
void slate_lu_solve_c64(slate_Matrix_c64 A, slate_Matrix_c64 B, slate_Options opts);
void slate_lu_factor_c64(slate_Matrix_c64 A, slate_Pivots pivots, slate_Options opts);
void slate_lu_solve_using_factor_c64(slate_Matrix_c64 A, slate_Pivots pivots, slate_Matrix_c64 B,
                                     slate_Options opts);

void slate_chol_solve_r32(slate_HermitianMatrix_r32 A, slate_Matrix_r32 B, slate_Options opts);
void slate_chol_factor_r32(slate_HermitianMatrix_r32 A, slate_Options opts);
void slate_chol_solve_using_factor_r32(slate_HermitianMatrix_r32 A, slate_Matrix_r32 B, slate_Options opts);
void slate_chol_solve_c32(slate_HermitianMatrix_c32 A, slate_Matrix_c32 B, slate_Options opts);
void slate_chol_factor_c32(slate_HermitianMatrix_c32 A, slate_Options opts);
void slate_chol_solve_using_factor_c32(slate_HermitianMatrix_c32 A, slate_Matrix_c32 B, slate_Options opts);
void slate_chol_solve_c64(slate_HermitianMatrix_c64 A, slate_Matrix_c64 B, slate_Options opts);
void slate_chol_factor_c64(slate_HermitianMatrix_c64 A, slate_Options opts);
void slate_chol_solve_using_factor_c64(slate_HermitianMatrix_c64 A, slate_Matrix_c64 B, slate_Options opts);

/* Outcome of the last C-API call on this thread (no counterpart in SLATE,
 * whose C wrappers throw). */
int64_t slate_gb300_last_info(void);
int slate_gb300_last_status(void);

#ifdef __cplusplus
}
#endif

#endif
