// common.cuh -- shared device helpers for the slate_gb300 kernels.
#pragma once

#include <cuda_runtime.h>
#include <atomic>
#include <cstdint>
#include <algorithm>

#include "slt_kernels.h"
#include "status.h"

namespace slt {

// Bound for every spin-wait in this library: about two seconds of wall time
// (%globaltimer), far longer than any legitimate wait, after which the
// waiting block records SLT_ERR_TIMEOUT and leaves.
constexpr unsigned long long kWaitNs = 2000000000ull;

// Kernel attributes set by cudaFuncSetAttribute belong to the current
// device, so a set-up that a launch needs runs once per device: one bit per
// device index.  Thread-safe; two threads racing on a first call both run
// the (idempotent) set-up.
class DeviceOnce {
public:
    template <typename F> int run(F&& f) {
        int dev = 0;
        const cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess) return slt_from_cuda(e);
        const unsigned long long bit = (dev >= 0 && dev < 64) ? (1ull << dev) : 0ull;
        if (bit && (done_.load(std::memory_order_acquire) & bit)) return SLT_OK;
        const int rc = f();
        if (rc == SLT_OK && bit) done_.fetch_or(bit, std::memory_order_acq_rel);
        return rc;
    }
private:
    std::atomic<unsigned long long> done_{0};
};

// Sets a kernel's dynamic shared-memory limit once per device.
#define SLT_SMEM_ONCE(kernel, bytes)                                                              \
    do {                                                                                          \
        static ::slt::DeviceOnce once_;                                                           \
        const int rc_ = once_.run([&] {                                                           \
            return slt_from_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                                      int(bytes)));                               \
        });                                                                                       \
        if (rc_) return rc_;                                                                      \
    } while (0)

// The same, storing the status in rcvar instead of returning it.
#define SLT_SMEM_ONCE_INTO(rcvar, kernel, bytes)                                                  \
    do {                                                                                          \
        static ::slt::DeviceOnce once_;                                                           \
        rcvar = once_.run([&] {                                                                   \
            return slt_from_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                                      int(bytes)));                               \
        });                                                                                       \
    } while (0)

__device__ __forceinline__ unsigned long long globaltimer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned atom_add_acqrel_u32(unsigned* p, unsigned v)
{
    unsigned old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ int ld_volatile_i32(const int* p)
{
    return *(const volatile int*) p;
}

// Grid-wide barrier for a cooperatively launched grid (all blocks are
// co-resident, guaranteed by cudaLaunchCooperativeKernel).  Counter +
// generation word in global memory, zeroed before launch.  Every wait is
// bounded: on timeout the block sets *status = SLT_ERR_TIMEOUT.  Returns
// false when the kernel must stop (status non-zero).
struct GridBarrier {
    unsigned count;
    unsigned gen;
};

__device__ __forceinline__ bool grid_sync(GridBarrier* bar, unsigned nblocks, int* status)
{
    __syncthreads();
    __shared__ int s_ok;
    if (threadIdx.x == 0) {
        unsigned g = ld_acquire_u32(&bar->gen);
        unsigned arrived = atom_add_acqrel_u32(&bar->count, 1u);
        if (arrived == nblocks - 1) {
            atomicExch(&bar->count, 0u);
            __threadfence();
            st_release_u32(&bar->gen, g + 1u);
        }
        else {
            const unsigned long long t0 = globaltimer();
            for (unsigned it = 1; ld_acquire_u32(&bar->gen) == g; ++it) {
                if ((it & 63u) == 0 && (ld_volatile_i32(status) != 0 || globaltimer() - t0 > kWaitNs)) {
                    atomicCAS(status, 0, SLT_ERR_TIMEOUT);
                    break;
                }
                __nanosleep(32);
            }
        }
        s_ok = (ld_volatile_i32(status) == 0);
    }
    __syncthreads();
    return s_ok != 0;
}

// st(e, ld(e)) for e in [0, cnt) by NTHR threads, each issuing NB loads
// before it stores any of their results: an SM issues in order, so a load
// whose result is stored at once costs its full memory latency, and a loop
// of such pairs pays it once per element.
template <int NB, int NTHR, typename Load, typename Store>
__device__ __forceinline__ void staged_copy(int cnt, Load ld, Store st)
{
    for (int e0 = threadIdx.x; e0 < cnt; e0 += NB * NTHR) {
        decltype(ld(0)) v[NB];
        #pragma unroll
        for (int u = 0; u < NB; ++u) {
            const int e = e0 + u * NTHR;
            if (e < cnt) v[u] = ld(e);
        }
        #pragma unroll
        for (int u = 0; u < NB; ++u) {
            const int e = e0 + u * NTHR;
            if (e < cnt) st(e, v[u]);
        }
    }
}

template <typename T> struct Real;
template <> struct Real<double> {
    static __device__ __forceinline__ double safe_min() { return 2.2250738585072014e-308; }
};
template <> struct Real<float> {
    static __device__ __forceinline__ float safe_min() { return 1.17549435e-38f; }
};

__host__ __device__ inline int64_t ceildiv(int64_t a, int64_t b) { return (a + b - 1) / b; }
__host__ __device__ inline int64_t min64(int64_t a, int64_t b) { return a < b ? a : b; }
__host__ __device__ inline int64_t max64(int64_t a, int64_t b) { return a > b ? a : b; }

} // namespace slt
