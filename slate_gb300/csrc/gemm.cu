// gemm.cu -- trailing-matrix update GEMMs for the FP64 and FP32 factorizations.
//
// Replaces SLATE's batched tile gemm/herk of the trailing update
// (internal::gemm, src/internal/internal_gemm.cc:354-518, and internal::herk,
// src/internal/internal_herk.cc:350-540), which SLATE hands to cuBLAS as one
// batch of nb x nb tiles per step.  Here the whole trailing matrix is one
// column-major operand and one launch covers it; `lower` restricts the
// output to the lower triangle, which gives the herk-shaped Cholesky update.
//
// Two FP64 engines: a SIMT DFMA kernel and a DMMA tensor kernel
// (mma.sync m16n8k4 .f64).  sm_103a has no FP64 kind of tcgen05.mma, so DMMA is
// the only FP64 tensor instruction on this part.

#include "common.cuh"
#include "prof.h"

namespace slt {

// One BM x BN output tile at (row0, col0).
template <typename T, int BM, int BN, int BK, int TM, int TN, bool TRANSB>
__device__ __forceinline__ void
gemm_simt_tile(int64_t row0, int64_t col0, int64_t m, int64_t n, int64_t k, T alpha, const T* __restrict__ A,
               int64_t lda, const T* __restrict__ B, int64_t ldb, T beta, T* __restrict__ C, int64_t ldc,
               int lower)
{
    constexpr int NT = (BM / TM) * (BN / TN);
    constexpr int RM = BM / TM;          // row groups
    constexpr int LA = BM * BK / NT;     // A elements loaded per thread
    constexpr int LB = BN * BK / NT;
    __shared__ T As[2][BK][BM];
    __shared__ T Bs[2][BK][BN];

    if (lower && row0 + BM - 1 < col0) return;

    const int t = threadIdx.x;
    const int ty = t % RM;
    const int tx = t / RM;

    T ra[LA], rb[LB];
    auto load = [&](int64_t k0) {
        #pragma unroll
        for (int q = 0; q < LA; ++q) {
            int e = t + q * NT;
            int i = e % BM, l = e / BM;
            int64_t gi = row0 + i, gl = k0 + l;
            ra[q] = (gi < m && gl < k) ? A[gi + gl * lda] : T(0);
        }
        #pragma unroll
        for (int q = 0; q < LB; ++q) {
            int e = t + q * NT;
            int l, j;
            if (TRANSB) { j = e % BN; l = e / BN; }
            else        { l = e % BK; j = e / BK; }
            int64_t gj = col0 + j, gl = k0 + l;
            T v = T(0);
            if (gj < n && gl < k) v = TRANSB ? B[gj + gl * ldb] : B[gl + gj * ldb];
            rb[q] = v;
        }
    };
    auto store = [&](int buf) {
        #pragma unroll
        for (int q = 0; q < LA; ++q) {
            int e = t + q * NT;
            As[buf][e / BM][e % BM] = ra[q];
        }
        #pragma unroll
        for (int q = 0; q < LB; ++q) {
            int e = t + q * NT;
            if (TRANSB) Bs[buf][e / BN][e % BN] = rb[q];
            else        Bs[buf][e % BK][e / BK] = rb[q];
        }
    };

    T acc[TM][TN];
    #pragma unroll
    for (int r = 0; r < TM; ++r)
        #pragma unroll
        for (int c = 0; c < TN; ++c) acc[r][c] = T(0);

    int buf = 0;
    load(0);
    store(0);
    __syncthreads();
    for (int64_t k0 = 0; k0 < k; k0 += BK) {
        bool more = k0 + BK < k;
        if (more) load(k0 + BK);
        #pragma unroll
        for (int l = 0; l < BK; ++l) {
            T a[TM], b[TN];
            #pragma unroll
            for (int r = 0; r < TM; ++r) a[r] = As[buf][l][ty + r * RM];
            #pragma unroll
            for (int c = 0; c < TN; ++c) b[c] = Bs[buf][l][tx + c * (BN / TN)];
            #pragma unroll
            for (int r = 0; r < TM; ++r)
                #pragma unroll
                for (int c = 0; c < TN; ++c) acc[r][c] = fma(a[r], b[c], acc[r][c]);
        }
        if (more) {
            store(buf ^ 1);
            __syncthreads();
            buf ^= 1;
        }
    }

    #pragma unroll
    for (int c = 0; c < TN; ++c) {
        int64_t gj = col0 + tx + c * (BN / TN);
        if (gj >= n) continue;
        #pragma unroll
        for (int r = 0; r < TM; ++r) {
            int64_t gi = row0 + ty + r * RM;
            if (gi >= m || (lower && gi < gj)) continue;
            T* p = C + gi + gj * ldc;
            *p = (beta == T(0)) ? alpha * acc[r][c] : fma(alpha, acc[r][c], beta * *p);
        }
    }
}

// The launch walks the output tiles with a grid stride (columns of tiles in
// order, rows fastest), so a grid smaller than the tile count -- an SM budget
// set with slt_set_sm_cap -- still covers C.
template <typename T, int BM, int BN, int BK, int TM, int TN, bool TRANSB>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
gemm_simt_kernel(int64_t m, int64_t n, int64_t k, T alpha, const T* __restrict__ A, int64_t lda,
                 const T* __restrict__ B, int64_t ldb, T beta, T* __restrict__ C, int64_t ldc,
                 int lower)
{
    const int64_t tm = ceildiv(m, BM), tiles = tm * ceildiv(n, BN);
    for (int64_t t = blockIdx.x; t < tiles; t += gridDim.x) {
        __syncthreads();          // the previous tile's shared-memory reads are done
        gemm_simt_tile<T, BM, BN, BK, TM, TN, TRANSB>((t % tm) * BM, (t / tm) * BN, m, n, k, alpha, A, lda,
                                                      B, ldb, beta, C, ldc, lower);
    }
}

// FP64 tensor-core GEMM: mma.sync.m16n8k4 .f64, 64x64 CTA tile, 4 warps of
// 32x32, BK = 16, register-staged double buffering.
template <bool TRANSB>
__device__ __forceinline__ void
dgemm_dmma_tile(int64_t row0, int64_t col0, int64_t m, int64_t n, int64_t k, double alpha,
                const double* __restrict__ A, int64_t lda, const double* __restrict__ B, int64_t ldb,
                double beta, double* __restrict__ C, int64_t ldc, int lower)
{
    constexpr int BM = 64, BN = 64, BK = 16, PAD = 4, NT = 128;
    __shared__ double As[2][BK][BM + PAD];
    __shared__ double Bs[2][BK][BN + PAD];

    if (lower && row0 + BM - 1 < col0) return;

    const int t = threadIdx.x;
    const int warp = t >> 5, lane = t & 31;
    const int g = lane >> 2, tig = lane & 3;
    const int wm = warp & 1, wn = warp >> 1;

    double ra[8], rb[8];
    auto load = [&](int64_t k0) {
        #pragma unroll
        for (int q = 0; q < 8; ++q) {
            int e = t + q * NT;
            int i = e % BM, l = e / BM;
            int64_t gi = row0 + i, gl = k0 + l;
            ra[q] = (gi < m && gl < k) ? A[gi + gl * lda] : 0.0;
        }
        #pragma unroll
        for (int q = 0; q < 8; ++q) {
            int e = t + q * NT;
            int l, j;
            if (TRANSB) { j = e % BN; l = e / BN; }
            else        { l = e % BK; j = e / BK; }
            int64_t gj = col0 + j, gl = k0 + l;
            double v = 0.0;
            if (gj < n && gl < k) v = TRANSB ? B[gj + gl * ldb] : B[gl + gj * ldb];
            rb[q] = v;
        }
    };
    auto store = [&](int buf) {
        #pragma unroll
        for (int q = 0; q < 8; ++q) {
            int e = t + q * NT;
            As[buf][e / BM][e % BM] = ra[q];
        }
        #pragma unroll
        for (int q = 0; q < 8; ++q) {
            int e = t + q * NT;
            if (TRANSB) Bs[buf][e / BN][e % BN] = rb[q];
            else        Bs[buf][e % BK][e / BK] = rb[q];
        }
    };

    double acc[2][4][4];
    #pragma unroll
    for (int a = 0; a < 2; ++a)
        #pragma unroll
        for (int b = 0; b < 4; ++b)
            #pragma unroll
            for (int c = 0; c < 4; ++c) acc[a][b][c] = 0.0;

    int buf = 0;
    load(0);
    store(0);
    __syncthreads();
    for (int64_t k0 = 0; k0 < k; k0 += BK) {
        bool more = k0 + BK < k;
        if (more) load(k0 + BK);
        #pragma unroll
        for (int kk = 0; kk < BK; kk += 4) {
            double af[2][2], bf[4];
            #pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                af[mt][0] = As[buf][kk + tig][wm * 32 + mt * 16 + g];
                af[mt][1] = As[buf][kk + tig][wm * 32 + mt * 16 + g + 8];
            }
            #pragma unroll
            for (int nt = 0; nt < 4; ++nt) bf[nt] = Bs[buf][kk + tig][wn * 32 + nt * 8 + g];
            #pragma unroll
            for (int mt = 0; mt < 2; ++mt)
                #pragma unroll
                for (int nt = 0; nt < 4; ++nt) {
                    asm volatile(
                        "mma.sync.aligned.m16n8k4.row.col.f64.f64.f64.f64 "
                        "{%0,%1,%2,%3}, {%4,%5}, {%6}, {%0,%1,%2,%3};"
                        : "+d"(acc[mt][nt][0]), "+d"(acc[mt][nt][1]),
                          "+d"(acc[mt][nt][2]), "+d"(acc[mt][nt][3])
                        : "d"(af[mt][0]), "d"(af[mt][1]), "d"(bf[nt]));
                }
        }
        if (more) {
            store(buf ^ 1);
            __syncthreads();
            buf ^= 1;
        }
    }

    #pragma unroll
    for (int mt = 0; mt < 2; ++mt)
        #pragma unroll
        for (int nt = 0; nt < 4; ++nt)
            #pragma unroll
            for (int c = 0; c < 4; ++c) {
                int64_t gi = row0 + wm * 32 + mt * 16 + g + ((c & 2) ? 8 : 0);
                int64_t gj = col0 + wn * 32 + nt * 8 + 2 * tig + (c & 1);
                if (gi >= m || gj >= n || (lower && gi < gj)) continue;
                double* p = C + gi + gj * ldc;
                *p = (beta == 0.0) ? alpha * acc[mt][nt][c] : fma(alpha, acc[mt][nt][c], beta * *p);
            }
}

template <bool TRANSB>
__global__ void __launch_bounds__(128)
dgemm_dmma_kernel(int64_t m, int64_t n, int64_t k, double alpha, const double* __restrict__ A,
                  int64_t lda, const double* __restrict__ B, int64_t ldb, double beta,
                  double* __restrict__ C, int64_t ldc, int lower)
{
    const int64_t tm = ceildiv(m, 64), tiles = tm * ceildiv(n, 64);
    for (int64_t t = blockIdx.x; t < tiles; t += gridDim.x) {
        __syncthreads();          // the previous tile's shared-memory reads are done
        dgemm_dmma_tile<TRANSB>((t % tm) * 64, (t / tm) * 64, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc,
                                lower);
    }
}

// Launch shape of a tile-walking GEMM: one block per tile, or, under an SM
// budget, one block per budgeted SM.  Those blocks reserve more than half of
// an SM's shared memory (unused by the kernel), so no two share an SM and the
// SMs outside the budget stay free for the panel that runs beside the update;
// the FP64 and FP32 pipes are saturated by one 256-thread block per SM.
constexpr size_t kCapSmem = 120 * 1024;

struct GemmLaunch {
    unsigned grid;
    size_t smem;
};

template <typename K>
static int gemm_launch(K kernel, int64_t tiles, GemmLaunch* out)
{
    const int cap = slt_sm_cap();
    if (cap <= 0) {
        *out = {unsigned(tiles), 0};
        return SLT_OK;
    }
    // set on every capped launch: kernels of one signature share this
    // template instance, so a once-per-instance flag would miss the second
    SLT_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kCapSmem)));
    *out = {unsigned(std::max<int64_t>(1, std::min<int64_t>(tiles, cap))), kCapSmem};
    return SLT_OK;
}

static int g_dgemm_engine = 0;   // 0: not chosen yet

} // namespace slt

using namespace slt;

extern "C" int slt_dgemm(char transb, int64_t m, int64_t n, int64_t k, double alpha,
                         const double* A, int64_t lda, const double* B, int64_t ldb,
                         double beta, double* C, int64_t ldc, int lower, int engine,
                         cudaStream_t stream)
{
    if (m < 0 || n < 0 || k < 0 || (transb != 'N' && transb != 'T')) return SLT_ERR_ARG;
    if (m == 0 || n == 0) return SLT_OK;
    if (engine == 0) engine = g_dgemm_engine ? g_dgemm_engine : 1;
    const int pidx = prof_begin(SLT_PROF_GEMM64, stream);
    const int64_t tiles = ceildiv(m, 64) * ceildiv(n, 64);
    GemmLaunch L;
    if (engine == 2) {
        auto kf = transb == 'N' ? dgemm_dmma_kernel<false> : dgemm_dmma_kernel<true>;
        const int rc = gemm_launch(kf, tiles, &L);
        if (rc) return rc;
        kf<<<L.grid, 128, L.smem, stream>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, lower);
        slt::count_launch();
    }
    else {
        auto kf = transb == 'N' ? gemm_simt_kernel<double, 64, 64, 8, 4, 4, false>
                                : gemm_simt_kernel<double, 64, 64, 8, 4, 4, true>;
        const int rc = gemm_launch(kf, tiles, &L);
        if (rc) return rc;
        kf<<<L.grid, 256, L.smem, stream>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, lower);
        slt::count_launch();
    }
    {
        double mn = lower ? (double(m) * double(n) - (double(n) * double(n) - double(n)) / 2.0) : double(m) * double(n);
        prof_end(pidx, stream, 2.0 * mn * double(k), 8.0 * (2.0 * mn + double(k) * double(m + n)));
    }
    return slt_from_cuda(cudaGetLastError());
}

extern "C" int slt_sgemm(char transb, int64_t m, int64_t n, int64_t k, float alpha,
                         const float* A, int64_t lda, const float* B, int64_t ldb,
                         float beta, float* C, int64_t ldc, int lower, cudaStream_t stream)
{
    if (m < 0 || n < 0 || k < 0 || (transb != 'N' && transb != 'T')) return SLT_ERR_ARG;
    if (m == 0 || n == 0) return SLT_OK;
    const int64_t tiles = ceildiv(m, 128) * ceildiv(n, 128);
    auto kf = transb == 'N' ? gemm_simt_kernel<float, 128, 128, 8, 8, 8, false>
                            : gemm_simt_kernel<float, 128, 128, 8, 8, 8, true>;
    GemmLaunch L;
    const int rc = gemm_launch(kf, tiles, &L);
    if (rc) return rc;
    const int pidx = prof_begin(SLT_PROF_GEMM32, stream);
    kf<<<L.grid, 256, L.smem, stream>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, lower);
    slt::count_launch();
    {
        double mn = lower ? (double(m) * double(n) - (double(n) * double(n) - double(n)) / 2.0) : double(m) * double(n);
        prof_end(pidx, stream, 2.0 * mn * double(k), 4.0 * (2.0 * mn + double(k) * double(m + n)));
    }
    return slt_from_cuda(cudaGetLastError());
}
