// prof.h -- launch counting and per-kernel event timing (see profile.cc).
#pragma once
#include <cuda_runtime.h>

/* kernel classes for slt_profile_read */
#define SLT_PROF_GEMM64    1   /* FP64 trailing update (DFMA / DMMA)        */
#define SLT_PROF_GEMM32    2   /* FP32 SIMT trailing update                 */
#define SLT_PROF_GEMM_TC   3   /* tcgen05 low-precision trailing update     */
#define SLT_PROF_PANEL     4   /* LU panel (cooperative)                    */
#define SLT_PROF_TRSM      5   /* triangular solves                         */
#define SLT_PROF_LASWP     6   /* row interchanges                          */
#define SLT_PROF_SKINNY    7   /* residual / sweep skinny products (FP64)   */
#define SLT_PROF_POTRF     8   /* diagonal-block Cholesky                   */
#define SLT_PROF_CONVERT   9   /* precision conversion                      */
#define SLT_PROF_SWEEP    10   /* one-launch triangular solve sweeps        */
#define SLT_PROF_DIGIT    11   /* tensor-core digit-split FP64 residual     */

namespace slt {
void count_launch();
int prof_begin(int kind, cudaStream_t s);
void prof_end(int idx, cudaStream_t s, double flops, double bytes);
// The SM count a launcher may use on the calling thread: sms, or the cap set
// by slt_set_sm_cap when it is smaller.
int capped_sms(int sms);
}
