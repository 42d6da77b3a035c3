// noalloc.cu -- an FP64 residual entry point that allocates nothing.
//
// Some callers cannot allocate device memory at the point where they need a
// residual: applications whose device memory is owned by their own pool or
// by a framework allocator that forbids side allocations, code that must not
// call cudaMalloc / cudaFree at that point (both can synchronise the whole
// device), and latency-critical refinement loops that cannot afford that
// synchronisation.  For them this file keeps the residual's partial-sum
// scratch in a fixed, library-owned __device__ array instead of allocating it
// per call; the caller passes A, B, X and R as usual.
//
// Limits and behaviour:
//  * the scratch holds kNoAllocScratchDoubles doubles (16 MiB); a call needs
//    n * min(nrhs, 16) doubles for one column segment and is rejected with
//    SLT_ERR_LIMIT beyond that (n * min(nrhs, 16) > 2,097,152);
//  * the array exists once per device in every process that loads the
//    library and lives until the process exits;
//  * every call shares it: calls that overlap on the GPU (two streams, or two
//    host threads) race on the scratch and must be serialised by the caller;
//  * the scratch keeps the last call's partial sums; nothing in it has to
//    start at zero, because every partial sum a call reads was written by
//    the same call first;
//  * the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (with that device current) and caches it; make
//    that first call before any stream capture begins.

#include <mutex>

#include "common.cuh"

namespace slt {

int dresidual_into(int64_t n, int64_t nrhs, const double* A, int64_t lda, int sym_lower, const double* B,
                   int64_t ldb, const double* X, int64_t ldx, double* R, int64_t ldr, double* ws,
                   size_t ws_doubles, cudaStream_t stream);

constexpr size_t kNoAllocScratchDoubles = size_t(2) * 1024 * 1024;
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

constexpr int kMaxDevices = 64;
static std::mutex g_noalloc_mtx;
static double* g_noalloc_addr[kMaxDevices] = {};

// Device address of the scratch on the current device (host code cannot use
// the symbol itself: in host code it names a host-side stand-in).
static int noalloc_scratch(double** out)
{
    int dev = 0;
    SLT_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return SLT_ERR_NOT_SUPPORTED;
    std::lock_guard<std::mutex> lk(g_noalloc_mtx);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return slt_from_cuda(e);
        g_noalloc_addr[dev] = static_cast<double*>(p);
    }
    *out = g_noalloc_addr[dev];
    return SLT_OK;
}

} // namespace slt

using namespace slt;

extern "C" int slt_dresidual_noalloc(int64_t n, int64_t nrhs, const double* A, int64_t lda, int sym_lower,
                                     const double* B, int64_t ldb, const double* X, int64_t ldx, double* R,
                                     int64_t ldr, cudaStream_t stream)
{
    if (n < 0 || nrhs < 0) return SLT_ERR_ARG;
    if (n == 0 || nrhs == 0) return SLT_OK;
    if (size_t(n) * size_t(std::min<int64_t>(nrhs, 16)) > kNoAllocScratchDoubles) return SLT_ERR_LIMIT;
    double* ws = nullptr;
    int rc = noalloc_scratch(&ws);
    if (rc) return rc;
    return dresidual_into(n, nrhs, A, lda, sym_lower, B, ldb, X, ldx, R, ldr, ws, kNoAllocScratchDoubles, stream);
}
