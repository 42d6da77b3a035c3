// status.h -- CUDA error to slt status mapping (host side).
#pragma once
#include <cuda_runtime.h>
#include "slt_kernels.h"

static inline int slt_from_cuda(cudaError_t e)
{
    return e == cudaSuccess ? SLT_OK : (SLT_ERR_CUDA_BASE + int(e));
}

#define SLT_CUDA_TRY(expr)                                        \
    do {                                                          \
        cudaError_t e_ = (expr);                                  \
        if (e_ != cudaSuccess) return slt_from_cuda(e_);          \
    } while (0)

// Propagates a non-zero slt status.
#define TRY(expr) do { int rc_ = (expr); if (rc_ != SLT_OK) return rc_; } while (0)
