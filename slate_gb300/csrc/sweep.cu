// sweep.cu -- one-launch triangular solves for few right-hand sides.
//
// Replaces the per-tile trsm + gemm sweeps of SLATE's getrs/potrs
// (work::trsmA, src/work/work_trsmA.cc:147-480; internal::trsmA/gemmA with a
// queue sync per call) by a single persistent kernel per sweep:
//
//   op(M) X = B,  op(M) lower (forward) or upper (backward), unit or not,
//   op(M) = M or M^T, X overwritten in place, nrhs <= 16.
//
// Row blocks of 64 are taken in solve order through an atomic ticket.  The
// block with ticket p accumulates op(M)(i, j) x_j over the blocks already
// solved (tickets < p), waiting on each block's ready flag with a bounded
// acquire spin, then solves its 64 x 64 diagonal block in shared memory and
// publishes x_i with a release flag.  Tickets are taken by running blocks
// in order, so a block only ever waits for blocks that are already running.
// The matrix is read once (HBM-bound); the critical path is one diagonal
// solve per block.

#include "common.cuh"
#include "prof.h"

namespace slt {

constexpr int kSwBS = 64;
constexpr int kSwRhs = 16;

template <typename T>
struct SweepSmem {
    T Ts[kSwBS][kSwBS + 1];    // off-diagonal tile, [col][row]
    T Ds[kSwBS][kSwBS + 1];    // diagonal tile, [row][col]
    T xs[kSwBS][kSwRhs];       // solved block x_j
    T xi[kSwBS][kSwRhs];       // this block's right-hand side / solution
};

__device__ __forceinline__ int ld_acquire_i32(const int* p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_i32(int* p, int v)
{
    asm volatile("st.release.gpu.global.b32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ uint64_t sw_globaltimer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// Inverse of every 64 x 64 diagonal block of op(M) (lower for FORWARD,
// upper otherwise), one block per CTA, 4 lanes per column.  Dinv[b] is
// row-major: Dinv[b][r][c].
template <typename T, bool FORWARD, bool UNIT, bool TRANS>
__global__ void __launch_bounds__(256)
trinv_kernel(int64_t n, const T* __restrict__ M, int64_t ldm, T* __restrict__ Dinv)
{
    extern __shared__ unsigned char ti_smem_raw[];
    T (*Ds)[kSwBS + 1] = reinterpret_cast<T (*)[kSwBS + 1]>(ti_smem_raw);
    T (*Xv)[kSwBS + 1] = Ds + kSwBS;       // Xv[r][c]: inverse being built, column c
    const int t = threadIdx.x;
    const int64_t i0 = int64_t(blockIdx.x) * kSwBS;
    const int ni = int(min64(kSwBS, n - i0));
    for (int e = t; e < kSwBS * kSwBS; e += 256) {
        int r, c;
        if (TRANS) { c = e % kSwBS; r = e / kSwBS; }
        else       { r = e % kSwBS; c = e / kSwBS; }
        T v;
        if (r < ni && c < ni) v = TRANS ? M[(i0 + c) + (i0 + r) * ldm] : M[(i0 + r) + (i0 + c) * ldm];
        else v = (r == c) ? T(1) : T(0);      // identity padding keeps the inverse well defined
        Ds[r][c] = v;
        Xv[r][c] = T(0);
    }
    __syncthreads();
    const int c = t >> 2, q = t & 3;          // column c, lane q of 4
    const T dcc = UNIT ? T(1) : Ds[c][c];
    if (q == 0) Xv[c][c] = T(1) / dcc;
    __syncwarp();
    // Every lane runs the same rows (warp-uniform trip count, so the shuffles
    // and __syncwarp below see all 32 lanes); rows outside the column's
    // triangle contribute nothing.
    for (int s = 1; s < kSwBS; ++s) {
        const int r = FORWARD ? s : kSwBS - 1 - s;
        const bool active = FORWARD ? (r > c) : (r < c);
        T part = T(0);
        if (active) {
            if (FORWARD) { for (int l = c + q; l < r; l += 4) part = fma(Ds[r][l], Xv[l][c], part); }
            else         { for (int l = r + 1 + q; l <= c; l += 4) part = fma(Ds[r][l], Xv[l][c], part); }
        }
        part += __shfl_xor_sync(0xffffffffu, part, 2);
        part += __shfl_xor_sync(0xffffffffu, part, 1);
        if (active && q == 0) Xv[r][c] = -part / (UNIT ? T(1) : Ds[r][r]);
        __syncwarp();
    }
    __syncthreads();
    T* out = Dinv + size_t(blockIdx.x) * kSwBS * kSwBS;
    for (int e = t; e < kSwBS * kSwBS; e += 256) out[e] = Xv[e / kSwBS][e % kSwBS];
}

template <typename T, bool FORWARD, bool UNIT, bool TRANS>
__global__ void __launch_bounds__(256)
sweep_kernel(int64_t n, int nrhs, const T* __restrict__ M, int64_t ldm, const T* __restrict__ Dinv,
             T* X, int64_t ldx, int* ticket, int* ready, int* status)
{
    extern __shared__ unsigned char sw_smem_raw[];
    SweepSmem<T>& sm = *reinterpret_cast<SweepSmem<T>*>(sw_smem_raw);
    __shared__ int s_p, s_ok;
    const int t = threadIdx.x;
    const int nblk = int(ceildiv(n, kSwBS));

    auto opM = [&](int64_t r, int64_t c) -> T {
        return TRANS ? __ldg(&M[c + r * ldm]) : __ldg(&M[r + c * ldm]);
    };

    for (;;) {
        if (t == 0) s_p = atomicAdd(ticket, 1);
        __syncthreads();
        const int p = s_p;
        if (p >= nblk) break;
        const int bi = FORWARD ? p : nblk - 1 - p;
        const int64_t i0 = int64_t(bi) * kSwBS;
        const int ni = int(min64(kSwBS, n - i0));

        // inverse of the diagonal block (row-major), and this block's RHS
        {
            const T* dinv = Dinv + size_t(bi) * kSwBS * kSwBS;
            staged_copy<kSwBS * kSwBS / 256, 256>(kSwBS * kSwBS, [&](int e) { return dinv[e]; },
                                                  [&](int e, T v) { sm.Ds[e / kSwBS][e % kSwBS] = v; });
        }
        staged_copy<kSwBS * kSwRhs / 256, 256>(kSwBS * kSwRhs, [&](int e) {
            const int r = e % kSwBS, q = e / kSwBS;
            return (r < ni && q < nrhs) ? X[i0 + r + q * ldx] : T(0);
        }, [&](int e, T v) { sm.xi[e % kSwBS][e / kSwBS] = v; });

        // accumulate op(M)(i, j) x_j over the solved blocks
        const int r = t % kSwBS, g = t / kSwBS;           // 4 groups x 4 right-hand sides
        T acc[4] = {T(0), T(0), T(0), T(0)};
        for (int pq = 0; pq < p; ++pq) {
            const int bj = FORWARD ? pq : nblk - 1 - pq;
            const int64_t j0 = int64_t(bj) * kSwBS;
            const int nj = int(min64(kSwBS, n - j0));
            __syncthreads();
            staged_copy<kSwBS * kSwBS / 256, 256>(kSwBS * kSwBS, [&](int e) {
                const int rr = TRANS ? e / kSwBS : e % kSwBS, c = TRANS ? e % kSwBS : e / kSwBS;
                return (rr < ni && c < nj) ? opM(i0 + rr, j0 + c) : T(0);
            }, [&](int e, T v) {
                const int rr = TRANS ? e / kSwBS : e % kSwBS, c = TRANS ? e % kSwBS : e / kSwBS;
                sm.Ts[c][rr] = v;
            });
            if (t == 0) {
                int ok = 1;
                if (ld_acquire_i32(&ready[pq]) == 0) {
                    const uint64_t t0 = sw_globaltimer();
                    for (unsigned it = 1; ld_acquire_i32(&ready[pq]) == 0; ++it) {
                        if ((it & 255u) == 0 &&
                            (ld_volatile_i32(status) != 0 || sw_globaltimer() - t0 > 2000000000ull)) {
                            atomicCAS(status, 0, SLT_ERR_TIMEOUT);
                            ok = 0;
                            break;
                        }
                    }
                }
                s_ok = ok;
            }
            __syncthreads();
            if (!s_ok) return;
            staged_copy<kSwBS * kSwRhs / 256, 256>(kSwBS * kSwRhs, [&](int e) {
                const int rr = e % kSwBS, q = e / kSwBS;
                return (rr < nj && q < nrhs) ? __ldcg(&X[j0 + rr + q * ldx]) : T(0);
            }, [&](int e, T v) { sm.xs[e % kSwBS][e / kSwBS] = v; });
            __syncthreads();
            #pragma unroll 4
            for (int c = 0; c < kSwBS; ++c) {
                const T a = sm.Ts[c][r];
                #pragma unroll
                for (int u = 0; u < 4; ++u) acc[u] = fma(a, sm.xs[c][g * 4 + u], acc[u]);
            }
        }
        __syncthreads();
        #pragma unroll
        for (int u = 0; u < 4; ++u) sm.xi[r][g * 4 + u] -= acc[u];
        __syncthreads();

        // x_i = inv(op(M)_ii) (b_i - acc): a 64 x 64 matrix-vector product
        {
            T y[4] = {T(0), T(0), T(0), T(0)};
            #pragma unroll 8
            for (int c = 0; c < kSwBS; ++c) {
                const T d = sm.Ds[r][c];
                #pragma unroll
                for (int u = 0; u < 4; ++u) y[u] = fma(d, sm.xi[c][g * 4 + u], y[u]);
            }
            __syncthreads();
            #pragma unroll
            for (int u = 0; u < 4; ++u) sm.xi[r][g * 4 + u] = y[u];
        }
        __syncthreads();
        for (int e = t; e < kSwBS * kSwRhs; e += 256) {
            int rr = e % kSwBS, q = e / kSwBS;
            if (rr < ni && q < nrhs) X[i0 + rr + q * ldx] = sm.xi[rr][q];
        }
        __threadfence();
        __syncthreads();
        if (t == 0) st_release_i32(&ready[p], 1);
    }
}

template <typename T, bool FORWARD, bool UNIT, bool TRANS>
static int launch_sweep(int64_t n, int64_t nrhs, const T* M, int64_t ldm, T* X, int64_t ldx, int* flags,
                        int* status, cudaStream_t s)
{
    if (n <= 0 || nrhs <= 0) return SLT_OK;
    if (nrhs > kSwRhs) return SLT_ERR_ARG;
    const int64_t nblk = ceildiv(n, kSwBS);
    // flags layout: [ticket][ready x nblk][pad to 256 B][Dinv: nblk x 64 x 64]
    T* Dinv = reinterpret_cast<T*>(reinterpret_cast<char*>(flags) + ((sizeof(int) * size_t(nblk + 1) + 255) & ~size_t(255)));
    const size_t ti_smem = size_t(2) * kSwBS * (kSwBS + 1) * sizeof(T);
    static bool ti_cfg = false;
    if (!ti_cfg) {
        SLT_CUDA_TRY(cudaFuncSetAttribute(trinv_kernel<T, FORWARD, UNIT, TRANS>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, int(ti_smem)));
        ti_cfg = true;
    }
    trinv_kernel<T, FORWARD, UNIT, TRANS><<<unsigned(nblk), 256, ti_smem, s>>>(n, M, ldm, Dinv);
    count_launch();
    SLT_CUDA_TRY(cudaGetLastError());
    SLT_CUDA_TRY(cudaMemsetAsync(flags, 0, sizeof(int) * size_t(nblk + 1), s));
    auto fn = sweep_kernel<T, FORWARD, UNIT, TRANS>;
    const size_t smem = sizeof(SweepSmem<T>);
    static bool cfg = false;
    if (!cfg) {
        SLT_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
        cfg = true;
    }
    int dev = 0, sms = 0, per = 0;
    SLT_CUDA_TRY(cudaGetDevice(&dev));
    SLT_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    SLT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, 256, smem));
    const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(nblk, int64_t(sms) * std::max(per, 1)));
    const int pidx = prof_begin(SLT_PROF_SWEEP, s);
    fn<<<unsigned(grid), 256, smem, s>>>(n, int(nrhs), M, ldm, Dinv, X, ldx, flags, flags + 1, status);
    count_launch();
    prof_end(pidx, s, double(n) * double(n) * double(nrhs), sizeof(T) * (double(n) * double(n) / 2 + 2.0 * n * nrhs));
    return slt_from_cuda(cudaGetLastError());
}

} // namespace slt

using namespace slt;

// flags: device int[ceil(n/64) + 1] scratch; status: device int (timeouts).
// kind: 0 unit lower (L of LU), 1 upper non-unit (U of LU), 2 lower
// non-unit (L of Cholesky), 3 lower^T non-unit (L^T of Cholesky), 4 upper^T
// non-unit (U^T of LU), 5 unit lower^T (L^T of LU).
extern "C" int slt_dsweep(int kind, int64_t n, int64_t nrhs, const double* M, int64_t ldm, double* X,
                          int64_t ldx, int* flags, int* status, cudaStream_t s)
{
    switch (kind) {
        case 0: return launch_sweep<double, true, true, false>(n, nrhs, M, ldm, X, ldx, flags, status, s);
        case 1: return launch_sweep<double, false, false, false>(n, nrhs, M, ldm, X, ldx, flags, status, s);
        case 2: return launch_sweep<double, true, false, false>(n, nrhs, M, ldm, X, ldx, flags, status, s);
        case 3: return launch_sweep<double, false, false, true>(n, nrhs, M, ldm, X, ldx, flags, status, s);
        case 4: return launch_sweep<double, true, false, true>(n, nrhs, M, ldm, X, ldx, flags, status, s);
        case 5: return launch_sweep<double, false, true, true>(n, nrhs, M, ldm, X, ldx, flags, status, s);
        default: return SLT_ERR_ARG;
    }
}

extern "C" int slt_ssweep(int kind, int64_t n, int64_t nrhs, const float* M, int64_t ldm, float* X,
                          int64_t ldx, int* flags, int* status, cudaStream_t s)
{
    switch (kind) {
        case 0: return launch_sweep<float, true, true, false>(n, nrhs, M, ldm, X, ldx, flags, status, s);
        case 1: return launch_sweep<float, false, false, false>(n, nrhs, M, ldm, X, ldx, flags, status, s);
        case 2: return launch_sweep<float, true, false, false>(n, nrhs, M, ldm, X, ldx, flags, status, s);
        case 3: return launch_sweep<float, false, false, true>(n, nrhs, M, ldm, X, ldx, flags, status, s);
        case 4: return launch_sweep<float, true, false, true>(n, nrhs, M, ldm, X, ldx, flags, status, s);
        case 5: return launch_sweep<float, false, true, true>(n, nrhs, M, ldm, X, ldx, flags, status, s);
        default: return SLT_ERR_ARG;
    }
}

// Scratch of one sweep: ticket + ready flags, then the diagonal-block
// inverses (sized for double).
extern "C" size_t slt_sweep_flags_bytes(int64_t n)
{
    const int64_t nblk = ceildiv(n, kSwBS);
    return ((sizeof(int) * size_t(nblk + 1) + 255) & ~size_t(255)) + size_t(nblk) * kSwBS * kSwBS * sizeof(double);
}
