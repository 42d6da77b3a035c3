// tc_gemm.cu -- low-precision tensor-core trailing update (tcgen05).
#include "common.cuh"

extern "C" size_t slt_tc_gemm_ws_bytes(int64_t, int64_t, int64_t) { return 0; }

extern "C" int slt_tc_gemm_update(int tier, char transb, int64_t m, int64_t n, int64_t k, const float* A,
                                  int64_t lda, const float* B, int64_t ldb, float* C, int64_t ldc, int lower,
                                  void* ws, size_t ws_bytes, cudaStream_t stream)
{
    (void) tier; (void) transb; (void) m; (void) n; (void) k; (void) A; (void) lda; (void) B; (void) ldb;
    (void) C; (void) ldc; (void) lower; (void) ws; (void) ws_bytes; (void) stream;
    return SLT_ERR_NOT_SUPPORTED;
}
