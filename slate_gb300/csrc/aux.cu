// aux.cu -- HBM-bound helpers of the solve and refinement path.
//
// Replaces SLATE's device auxiliary kernels used on this path
// (src/cuda/device_gecopy.cu:40-115 precision conversion, device_genorm.cu
// norms and column maxima, device_geadd.cu, device_gescale.cu) and the
// one-right-hand-side gemm/hemm calls of the refinement residual
// R = B - A X (src/gesv_mixed.cc:198-204, src/posv_mixed.cc:201-205) and of
// the solve sweeps (internal::gemmA, src/internal/internal_gemmA.cc).
//
// Skinny products (few right-hand sides) stream A once: a block owns 64 rows
// and a segment of the columns (64 x 64 tiles, the next tile fetched into
// registers while the current one is used), keeps one accumulator per
// right-hand side per row in registers, and writes a partial sum per
// segment; a second launch adds the segments in a fixed order
// (deterministic, no atomics).  The symmetric variant reads only the lower
// triangle: tile (I,J) with J > I is read as the transpose of the stored
// tile (J,I) through shared memory.

#include "common.cuh"
#include "prof.h"

namespace slt {

constexpr int kRowsPerBlock = 64;
constexpr int kMaxRhs = 16;

// y_seg(i, r) = sum_{j in segment} op(A)(i, j) X(j, r)   (MODE 0)
// y_seg(i, 0) = sum_{j in segment} |op(A)(i, j)|         (MODE 1)
// Tiles of 64 x 64; SYM: A symmetric with lower storage.  The next tile (and
// its slice of X) is fetched into registers while the current one is used,
// so a block keeps a whole tile of loads in flight instead of waiting out one
// load latency per element; the shared tile is reused for the final
// reduction.  Every sum is formed in the same order as a plain loop over the
// tiles (thread group g adds columns g, g + 4, ... of each tile in turn).
constexpr int kRowopPer = 64 * 64 / 256;     // tile elements per thread
constexpr int kRowopTile = 64 * 65;          // padded tile, doubles

template <int MODE, bool SYM, int NR>
__global__ void __launch_bounds__(256)
rowop_kernel(int64_t m, int64_t k, int nrhs, const double* __restrict__ A, int64_t lda,
             const double* __restrict__ X, int64_t ldx, int64_t tiles_per_seg,
             double* __restrict__ part)
{
    extern __shared__ double rowop_smem[];
    double (*As)[65] = reinterpret_cast<double (*)[65]>(rowop_smem);                         // [64][65]
    double (*xs)[NR] = reinterpret_cast<double (*)[NR]>(rowop_smem + kRowopTile);            // [64][NR]
    double (*red)[64][NR + 1] = reinterpret_cast<double (*)[64][NR + 1]>(rowop_smem);        // [4][64][NR+1], after the loop
    constexpr int XPER = (64 * NR + 255) / 256;
    const int t = threadIdx.x;
    const int r = t % 64, g = t / 64;
    const int64_t I = blockIdx.x;
    const int64_t seg = blockIdx.y;
    const int64_t row0 = I * 64;
    const int64_t ktiles = ceildiv(k, 64);
    const int64_t J0 = seg * tiles_per_seg;
    const int64_t J1 = min(ktiles, J0 + tiles_per_seg);
    // NR: compile-time right-hand-side count (1, 2, 4, 8 or 16); MODE 1 uses 1.
    const int nr = (MODE == 0) ? nrhs : 1;

    double pre[kRowopPer];
    double xpre[XPER];
    // element u of this thread: tile row i = t % 64, tile column c = t / 64 + 4 u;
    // a tile above the diagonal is the transpose of the stored tile (J, I), read
    // along its columns (i is then the stored row within tile J).
    auto fetch = [&](int64_t J) {
        const int64_t col0 = J * 64;
        const bool transposed = SYM && (J > I);
        #pragma unroll
        for (int u = 0; u < kRowopPer; ++u) {
            const int i = t % 64, c = t / 64 + 4 * u;
            const int64_t gi = transposed ? col0 + i : row0 + i;     // stored row
            const int64_t gc = transposed ? row0 + c : col0 + c;     // stored column
            const bool in = transposed ? (gi < k && gc < m) : (gi < m && gc < k);
            const bool mirror = SYM && J == I && gi < gc;            // upper half of a diagonal tile
            pre[u] = in ? (mirror ? A[gc + gi * lda] : A[gi + gc * lda]) : 0.0;
        }
        if (MODE == 0) {
            #pragma unroll
            for (int u = 0; u < XPER; ++u) {
                const int e = t + 256 * u, c = e % 64, q = e / 64;
                const int64_t gc = col0 + c;
                xpre[u] = (q < nr && gc < k) ? X[gc + q * ldx] : 0.0;
            }
        }
    };
    auto put = [&](int64_t J) {
        const bool transposed = SYM && (J > I);
        #pragma unroll
        for (int u = 0; u < kRowopPer; ++u) {
            const int i = t % 64, c = t / 64 + 4 * u;
            if (transposed) As[i][c] = pre[u];
            else As[c][i] = pre[u];
        }
        if (MODE == 0) {
            #pragma unroll
            for (int u = 0; u < XPER; ++u) {
                const int e = t + 256 * u, c = e % 64, q = e / 64;
                if (q < NR) xs[c][q] = xpre[u];
            }
        }
    };

    double acc[NR];
    #pragma unroll
    for (int q = 0; q < NR; ++q) acc[q] = 0.0;

    if (J0 < J1) fetch(J0);
    for (int64_t J = J0; J < J1; ++J) {
        __syncthreads();
        put(J);
        __syncthreads();
        if (J + 1 < J1) fetch(J + 1);
        // group g takes tile columns c = g, g+4, ...
        if (MODE == 0) {
            #pragma unroll 4
            for (int c = g; c < 64; c += 4) {
                double a = As[c][r];
                #pragma unroll
                for (int q = 0; q < NR; ++q) acc[q] = fma(a, xs[c][q], acc[q]);
            }
        }
        else {
            for (int c = g; c < 64; c += 4) acc[0] += fabs(As[c][r]);
        }
    }
    __syncthreads();
    #pragma unroll
    for (int q = 0; q < NR; ++q)
        if (q < nr) red[g][r][q] = acc[q];
    __syncthreads();
    for (int e = t; e < 64 * nr; e += 256) {
        int i = e % 64, q = e / 64;
        int64_t gi = row0 + i;
        if (gi < m) {
            double s = red[0][i][q] + red[1][i][q] + red[2][i][q] + red[3][i][q];
            part[(seg * nr + q) * m + gi] = s;
        }
    }
}

// C(i, r) = beta C(i, r) + alpha sum_seg part(seg, r, i)
__global__ void reduce_segments_kernel(int64_t m, int nrhs, int64_t nseg, const double* __restrict__ part,
                                       double alpha, double beta, double* C, int64_t ldc)
{
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    int q = blockIdx.y;
    if (i >= m) return;
    double s = 0.0;
    for (int64_t sg = 0; sg < nseg; ++sg) s += part[(sg * nrhs + q) * m + i];
    double* p = C + i + q * ldc;
    *p = (beta == 0.0) ? alpha * s : fma(alpha, s, beta * *p);
}

__global__ void max_reduce_kernel(int64_t m, int64_t nseg, const double* __restrict__ part, double* out)
{
    __shared__ double red[256];
    double mx = 0.0;
    for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
        double s = 0.0;
        for (int64_t sg = 0; sg < nseg; ++sg) s += part[sg * m + i];
        mx = fmax(mx, s);
    }
    red[threadIdx.x] = mx;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

// padded tile + X slice; the reduction area [4][64][NR+1] reuses the same space
constexpr size_t rowop_smem_bytes(int nr)
{
    return sizeof(double) * size_t(std::max(kRowopTile + 64 * nr, 4 * 64 * (nr + 1)));
}

template <int MODE, bool SYM, int NR>
static int launch_rowop_nr(dim3 grid, cudaStream_t stream, int64_t m, int64_t k, int nrhs, const double* A,
                           int64_t lda, const double* X, int64_t ldx, int64_t tps, double* part)
{
    constexpr size_t smem = rowop_smem_bytes(NR);
    SLT_SMEM_ONCE((rowop_kernel<MODE, SYM, NR>), smem);
    rowop_kernel<MODE, SYM, NR><<<grid, 256, smem, stream>>>(m, k, nrhs, A, lda, X, ldx, tps, part);
    return SLT_OK;
}

template <int MODE, bool SYM>
static int launch_rowop(dim3 grid, cudaStream_t stream, int64_t m, int64_t k, int nrhs, const double* A,
                        int64_t lda, const double* X, int64_t ldx, int64_t tps, double* part)
{
    const int pidx = prof_begin(SLT_PROF_SKINNY, stream);
    int rc;
    if (MODE == 1 || nrhs == 1) rc = launch_rowop_nr<MODE, SYM, 1>(grid, stream, m, k, nrhs, A, lda, X, ldx, tps, part);
    else if (nrhs == 2) rc = launch_rowop_nr<MODE, SYM, 2>(grid, stream, m, k, nrhs, A, lda, X, ldx, tps, part);
    else if (nrhs <= 4) rc = launch_rowop_nr<MODE, SYM, 4>(grid, stream, m, k, nrhs, A, lda, X, ldx, tps, part);
    else if (nrhs <= 8) rc = launch_rowop_nr<MODE, SYM, 8>(grid, stream, m, k, nrhs, A, lda, X, ldx, tps, part);
    else rc = launch_rowop_nr<MODE, SYM, 16>(grid, stream, m, k, nrhs, A, lda, X, ldx, tps, part);
    if (rc) return rc;
    slt::count_launch();
    prof_end(pidx, stream, 2.0 * double(m) * double(k) * (MODE == 0 ? nrhs : 1), 8.0 * (SYM ? double(m) * double(k) / 2 + 64.0 * m : double(m) * double(k)));
    return slt_from_cuda(cudaGetLastError());
}

static void plan_segments(int64_t m, int64_t k, int64_t* nseg, int64_t* tps)
{
    int64_t rowblocks = ceildiv(m, 64);
    int64_t ktiles = ceildiv(k, 64);
    int64_t want = ceildiv(152 * 8, rowblocks);
    int64_t s = std::max<int64_t>(1, std::min<int64_t>(want, ktiles));
    *tps = ceildiv(ktiles, s);
    *nseg = ceildiv(ktiles, *tps);
}

// Skinny transposed product: C(i, r) = beta C + alpha sum_l A(l, i) X(l, r),
// A is kk x m (used for U^T / L^T sweep updates).  One warp per output row i
// reads column i of A contiguously.
template <typename T>
__global__ void __launch_bounds__(256)
skinny_t_kernel(int64_t m, int64_t kk, int nrhs, T alpha, const T* __restrict__ A, int64_t lda,
                const T* __restrict__ X, int64_t ldx, T beta, T* C, int64_t ldc)
{
    const int lane = threadIdx.x & 31;
    const int64_t i = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    if (i >= m) return;
    for (int q = 0; q < nrhs; ++q) {
        T s = T(0);
        for (int64_t l = lane; l < kk; l += 32) s = fma(A[l + i * lda], X[l + q * ldx], s);
        #pragma unroll
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        if (lane == 0) {
            T* p = C + i + q * ldc;
            *p = (beta == T(0)) ? alpha * s : fma(alpha, s, beta * *p);
        }
    }
}

// Skinny product, FP32 (getrs_lo / potrs_lo sweep updates): one thread per
// row, columns split in segments with atomics-free partials is not needed at
// these sizes; each thread keeps nrhs accumulators.
__global__ void __launch_bounds__(256)
sskinny_n_kernel(int64_t m, int64_t kk, int nrhs, float alpha, const float* __restrict__ A, int64_t lda,
                 const float* __restrict__ X, int64_t ldx, float beta, float* C, int64_t ldc)
{
    __shared__ float xs[512][kMaxRhs];
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    float acc[kMaxRhs];
    #pragma unroll
    for (int q = 0; q < kMaxRhs; ++q) acc[q] = 0.f;
    for (int64_t l0 = 0; l0 < kk; l0 += 512) {
        const int nl = int(min64(512, kk - l0));
        __syncthreads();
        for (int e = threadIdx.x; e < nl * nrhs; e += blockDim.x) {
            int l = e % nl, q = e / nl;
            xs[l][q] = X[l0 + l + q * ldx];
        }
        __syncthreads();
        if (i < m) {
            for (int l = 0; l < nl; ++l) {
                float a = A[i + (l0 + l) * lda];
                #pragma unroll
                for (int q = 0; q < kMaxRhs; ++q)
                    if (q < nrhs) acc[q] = fmaf(a, xs[l][q], acc[q]);
            }
        }
    }
    if (i < m)
        for (int q = 0; q < nrhs; ++q) {
            float* p = C + i + q * ldc;
            *p = (beta == 0.f) ? alpha * acc[q] : fmaf(alpha, acc[q], beta * *p);
        }
}

__global__ void geadd_kernel(int64_t m, int64_t n, double alpha, const double* __restrict__ A, int64_t lda,
                             double beta, double* B, int64_t ldb)
{
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    for (int64_t j = blockIdx.y; j < n; j += gridDim.y)
        if (i < m) B[i + j * ldb] = (beta == 0.0) ? alpha * A[i + j * lda] : fma(alpha, A[i + j * lda], beta * B[i + j * ldb]);
}

__global__ void colmax_kernel(int64_t m, const double* __restrict__ A, int64_t lda, double* out)
{
    __shared__ double red[256];
    const int64_t j = blockIdx.x;
    double mx = 0.0;
    for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
        double v = fabs(A[i + j * lda]);
        mx = (v > mx || v != v) ? v : mx;     // NaN propagates, as max_nan
    }
    red[threadIdx.x] = mx;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            double o = red[threadIdx.x + w];
            if (o > red[threadIdx.x] || o != o) red[threadIdx.x] = o;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) out[j] = red[0];
}

// Segment [r0, r0 + rps) of column j: max |A(i, j)| combined with an atomic
// max on the bit pattern (non-negative doubles order like their bits, and a
// NaN, made positive by fabs, orders above +Inf, so it propagates).  out
// (as bits) starts at 0.  grid (ceil(m / rps), n).
__global__ void __launch_bounds__(256)
colmax_seg_kernel(int64_t m, const double* __restrict__ A, int64_t lda, int64_t rps, unsigned long long* out)
{
    __shared__ unsigned long long red[8];
    const int64_t j = blockIdx.y;
    const int64_t r0 = int64_t(blockIdx.x) * rps;
    const int64_t r1 = r0 + rps < m ? r0 + rps : m;
    unsigned long long mx = 0;
    for (int64_t i = r0 + threadIdx.x; i < r1; i += 256) {
        const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(fabs(A[i + j * lda])));
        mx = b > mx ? b : mx;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long v = __shfl_xor_sync(0xffffffffu, mx, o);
        mx = v > mx ? v : mx;
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < 8; ++w) mx = red[w] > mx ? red[w] : mx;
        atomicMax(out + j, mx);
    }
}

// ---- Philox generator (same sequence as slate::random::generate)
__device__ __forceinline__ void philox2x64_dev(uint64_t s0, uint64_t s1, uint64_t key, uint64_t out[2])
{
    const uint64_t key_bump = 0xD2B74407B1CE6E93ull;
    const uint64_t mult = 0x9E3779B97F4A7C15ull;
    #pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) key += key_bump;
        uint64_t lo = s1 * mult;
        uint64_t hi = __umul64hi(s1, mult);
        uint64_t n1 = hi ^ key ^ s0;
        s0 = lo;
        s1 = n1;
    }
    out[0] = s0;
    out[1] = s1;
}

__global__ void generate_kernel(int dist, int64_t seed, int64_t m, int64_t n, int64_t ioff, int64_t joff,
                                double* A, int64_t lda)
{
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= m) return;
    for (int64_t j = blockIdx.y; j < n; j += gridDim.y) {
        uint64_t b[2];
        philox2x64_dev(uint64_t(i + ioff), uint64_t(j + joff), uint64_t(seed), b);
        double u1 = double(b[0] >> 11) / double(uint64_t(1) << 53);
        double u2 = double(b[1] >> 11) / double(uint64_t(1) << 53);
        const double pi = 3.1415926535897932385;
        double v;
        switch (dist) {
            case 1: v = u1; break;
            case 2: v = 2 * u1 - 1; break;
            case 3: v = sqrt(-2 * log(1 - u1)) * cos(2 * pi * u2); break;
            case 4: v = sqrt(u1) * cos(2 * pi * u2); break;
            case 5: v = cos(2 * pi * u2); break;
            case 6: v = u1 >= 0.5 ? 1.0 : 0.0; break;
            case 7: v = u1 >= 0.5 ? 1.0 : -1.0; break;
            default: v = 0.0;
        }
        A[i + j * lda] = v;
    }
}

template <typename T>
__global__ void shift_diag_kernel(int64_t n, T alpha, T* A, int64_t lda)
{
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) A[i + i * lda] += alpha;
}

// D = S on one triangle (lower: i >= j, upper: i <= j), the rest of D untouched.
__global__ void copy_tri_kernel(int lower, int64_t n, const double* __restrict__ S, int64_t lds, double* D,
                                int64_t ldd)
{
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int64_t j = blockIdx.y; j < n; j += gridDim.y)
        if (lower ? (i >= j) : (i <= j)) D[i + j * ldd] = S[i + j * lds];
}

__global__ void symmetrize_lower_kernel(int64_t n, double* A, int64_t lda)
{
    // 32 x 32 tiles through shared memory: upper tile (J, I) <- lower tile (I, J)^T
    __shared__ double tl[32][33];
    int64_t I = blockIdx.x, J = blockIdx.y;
    if (J > I) return;
    int tx = threadIdx.x % 32, ty = threadIdx.x / 32;   // 32 x 8
    for (int q = ty; q < 32; q += 8) {
        int64_t gi = I * 32 + tx, gj = J * 32 + q;
        tl[q][tx] = (gi < n && gj < n) ? A[gi + gj * lda] : 0.0;
    }
    __syncthreads();
    for (int q = ty; q < 32; q += 8) {
        int64_t gi = J * 32 + tx, gj = I * 32 + q;   // destination (row gi, col gj) = A(gj, gi)
        if (gi < n && gj < n && gi < gj) A[gi + gj * lda] = tl[tx][q];
    }
}

} // namespace slt

using namespace slt;

// Partial-sum workspace of the skinny products for any m, k <= n: a
// segment count times m never exceeds min(ceil(n/64) n, 1216*64 + 64 + n)
// per right-hand side (plan_segments targets 1216 blocks).
extern "C" size_t slt_residual_ws_bytes(int64_t n, int64_t nrhs)
{
    int64_t per_rhs = std::min<int64_t>(ceildiv(n, 64) * n, 1216 * 64 + 64 + n);
    return size_t(per_rhs) * size_t(std::max<int64_t>(nrhs, 1)) * sizeof(double) + 256;
}

extern "C" size_t slt_norm_ws_bytes(int64_t m)
{
    int64_t nseg, tps;
    plan_segments(m, m, &nseg, &tps);
    return size_t(nseg) * size_t(m) * sizeof(double) + 256;
}

// C (m x nrhs) = beta C + alpha A X  with A m x k general (sym_lower: m == k,
// symmetric, lower storage).  ws: partial sums.
extern "C" int slt_dgemm_skinny(int64_t m, int64_t nrhs, int64_t k, double alpha, const double* A,
                                int64_t lda, int sym_lower, const double* X, int64_t ldx, double beta,
                                double* C, int64_t ldc, void* ws, cudaStream_t stream)
{
    if (m <= 0 || nrhs <= 0) return SLT_OK;
    if (nrhs > kMaxRhs) return SLT_ERR_ARG;
    if (k <= 0) {
        // C = beta C
        dim3 grid(unsigned(ceildiv(m, 256)), unsigned(nrhs));
        reduce_segments_kernel<<<grid, 256, 0, stream>>>(m, int(nrhs), 0, nullptr, alpha, beta, C, ldc); slt::count_launch();
        return slt_from_cuda(cudaGetLastError());
    }
    int64_t nseg, tps;
    plan_segments(m, k, &nseg, &tps);
    double* part = static_cast<double*>(ws);
    dim3 grid(unsigned(ceildiv(m, 64)), unsigned(nseg));
    int rc = sym_lower ? launch_rowop<0, true>(grid, stream, m, k, int(nrhs), A, lda, X, ldx, tps, part)
                       : launch_rowop<0, false>(grid, stream, m, k, int(nrhs), A, lda, X, ldx, tps, part);
    if (rc) return rc;
    dim3 g2(unsigned(ceildiv(m, 256)), unsigned(nrhs));
    reduce_segments_kernel<<<g2, 256, 0, stream>>>(m, int(nrhs), nseg, part, alpha, beta, C, ldc); slt::count_launch();
    return slt_from_cuda(cudaGetLastError());
}

extern "C" int slt_dresidual(int64_t n, int64_t nrhs, const double* A, int64_t lda, int sym_lower,
                             const double* B, int64_t ldb, const double* X, int64_t ldx,
                             double* R, int64_t ldr, void* ws, cudaStream_t stream)
{
    int rc = slt_dcopy2d(n, nrhs, B, ldb, R, ldr, stream);
    if (rc) return rc;
    return slt_dgemm_skinny(n, nrhs, n, -1.0, A, lda, sym_lower, X, ldx, 1.0, R, ldr, ws, stream);
}

extern "C" int slt_dnorm_inf(int64_t m, int64_t n, const double* A, int64_t lda, int sym_lower,
                             double* out, void* ws, cudaStream_t stream)
{
    if (m <= 0 || n <= 0) return slt_from_cuda(cudaMemsetAsync(out, 0, sizeof(double), stream));
    int64_t nseg, tps;
    plan_segments(m, n, &nseg, &tps);
    double* part = static_cast<double*>(ws);
    dim3 grid(unsigned(ceildiv(m, 64)), unsigned(nseg));
    int rc = sym_lower ? launch_rowop<1, true>(grid, stream, m, n, 1, A, lda, nullptr, 0, tps, part)
                       : launch_rowop<1, false>(grid, stream, m, n, 1, A, lda, nullptr, 0, tps, part);
    if (rc) return rc;
    max_reduce_kernel<<<1, 256, 0, stream>>>(m, nseg, part, out); slt::count_launch();
    return slt_from_cuda(cudaGetLastError());
}

extern "C" int slt_dgemm_skinny_t(int64_t m, int64_t nrhs, int64_t kk, double alpha, const double* A,
                                  int64_t lda, const double* X, int64_t ldx, double beta, double* C,
                                  int64_t ldc, cudaStream_t stream)
{
    if (m <= 0 || nrhs <= 0) return SLT_OK;
    unsigned grid = unsigned(ceildiv(m * 32, 256));
    skinny_t_kernel<double><<<grid, 256, 0, stream>>>(m, kk, int(nrhs), alpha, A, lda, X, ldx, beta, C, ldc); slt::count_launch();
    return slt_from_cuda(cudaGetLastError());
}

extern "C" int slt_sgemm_skinny_t(int64_t m, int64_t nrhs, int64_t kk, float alpha, const float* A,
                                  int64_t lda, const float* X, int64_t ldx, float beta, float* C,
                                  int64_t ldc, cudaStream_t stream)
{
    if (m <= 0 || nrhs <= 0) return SLT_OK;
    unsigned grid = unsigned(ceildiv(m * 32, 256));
    skinny_t_kernel<float><<<grid, 256, 0, stream>>>(m, kk, int(nrhs), alpha, A, lda, X, ldx, beta, C, ldc); slt::count_launch();
    return slt_from_cuda(cudaGetLastError());
}

extern "C" int slt_sgemm_skinny(int64_t m, int64_t nrhs, int64_t k, float alpha, const float* A,
                                int64_t lda, const float* X, int64_t ldx, float beta, float* C,
                                int64_t ldc, cudaStream_t stream)
{
    if (m <= 0 || nrhs <= 0) return SLT_OK;
    if (nrhs > kMaxRhs) return SLT_ERR_ARG;
    sskinny_n_kernel<<<unsigned(ceildiv(m, 256)), 256, 0, stream>>>(m, k, int(nrhs), alpha, A, lda, X, ldx, beta, C, ldc); slt::count_launch();
    return slt_from_cuda(cudaGetLastError());
}

extern "C" int slt_convert_d2s(int64_t m, int64_t n, const double* A, int64_t lda, float* B, int64_t ldb,
                               cudaStream_t stream)
{
    return slt_convert_d2s_scaled(m, n, A, lda, nullptr, nullptr, B, ldb, stream);
}

extern "C" int slt_convert_s2d(int64_t m, int64_t n, const float* A, int64_t lda, double* B, int64_t ldb,
                               cudaStream_t stream)
{
    return slt_convert_s2d_scaled(m, n, A, lda, nullptr, B, ldb, stream);
}

extern "C" int slt_dcopy2d(int64_t m, int64_t n, const double* A, int64_t lda, double* B, int64_t ldb,
                           cudaStream_t stream)
{
    if (m <= 0 || n <= 0) return SLT_OK;
    return slt_from_cuda(cudaMemcpy2DAsync(B, size_t(ldb) * sizeof(double), A, size_t(lda) * sizeof(double),
                                           size_t(m) * sizeof(double), size_t(n), cudaMemcpyDeviceToDevice,
                                           stream));
}

extern "C" int slt_dgeadd(int64_t m, int64_t n, double alpha, const double* A, int64_t lda, double beta,
                          double* B, int64_t ldb, cudaStream_t stream)
{
    if (m <= 0 || n <= 0) return SLT_OK;
    dim3 grid(unsigned(ceildiv(m, 256)), unsigned(std::min<int64_t>(n, 65535)));
    geadd_kernel<<<grid, 256, 0, stream>>>(m, n, alpha, A, lda, beta, B, ldb); slt::count_launch();
    return slt_from_cuda(cudaGetLastError());
}

extern "C" int slt_dcolmax(int64_t m, int64_t n, const double* A, int64_t lda, double* out,
                           cudaStream_t stream)
{
    if (n <= 0) return SLT_OK;
    if (m <= 16384) {
        colmax_kernel<<<unsigned(n), 256, 0, stream>>>(m, A, lda, out); slt::count_launch();
        return slt_from_cuda(cudaGetLastError());
    }
    // long columns: 8192-row segments in parallel
    const int64_t rps = 8192;
    SLT_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(double) * size_t(n), stream));
    colmax_seg_kernel<<<dim3(unsigned(ceildiv(m, rps)), unsigned(n)), 256, 0, stream>>>(
        m, A, lda, rps, reinterpret_cast<unsigned long long*>(out));
    slt::count_launch();
    return slt_from_cuda(cudaGetLastError());
}

extern "C" int slt_dgenerate(int dist, int64_t seed, int64_t m, int64_t n, int64_t ioff, int64_t joff,
                             double* A, int64_t lda, cudaStream_t stream)
{
    if (m <= 0 || n <= 0) return SLT_OK;
    dim3 grid(unsigned(ceildiv(m, 256)), unsigned(std::min<int64_t>(n, 65535)));
    generate_kernel<<<grid, 256, 0, stream>>>(dist, seed, m, n, ioff, joff, A, lda); slt::count_launch();
    return slt_from_cuda(cudaGetLastError());
}

extern "C" int slt_dshift_diag(int64_t n, double alpha, double* A, int64_t lda, cudaStream_t stream)
{
    if (n <= 0) return SLT_OK;
    shift_diag_kernel<double><<<unsigned(ceildiv(n, 256)), 256, 0, stream>>>(n, alpha, A, lda); slt::count_launch();
    return slt_from_cuda(cudaGetLastError());
}

extern "C" int slt_sshift_diag(int64_t n, float alpha, float* A, int64_t lda, cudaStream_t stream)
{
    if (n <= 0) return SLT_OK;
    shift_diag_kernel<float><<<unsigned(ceildiv(n, 256)), 256, 0, stream>>>(n, alpha, A, lda); slt::count_launch();
    return slt_from_cuda(cudaGetLastError());
}

extern "C" int slt_dcopy_tri(int lower, int64_t n, const double* S, int64_t lds, double* D, int64_t ldd,
                             cudaStream_t stream)
{
    if (n <= 0) return SLT_OK;
    dim3 grid(unsigned(ceildiv(n, 256)), unsigned(std::min<int64_t>(n, 65535)));
    copy_tri_kernel<<<grid, 256, 0, stream>>>(lower, n, S, lds, D, ldd); slt::count_launch();
    return slt_from_cuda(cudaGetLastError());
}

extern "C" int slt_dsymmetrize_lower(int64_t n, double* A, int64_t lda, cudaStream_t stream)
{
    if (n <= 0) return SLT_OK;
    dim3 grid(unsigned(ceildiv(n, 32)), unsigned(ceildiv(n, 32)));
    symmetrize_lower_kernel<<<grid, 256, 0, stream>>>(n, A, lda); slt::count_launch();
    return slt_from_cuda(cudaGetLastError());
}

// ---- 2-norm (one block; used on n-vectors of the Arnoldi process)
namespace slt {
__global__ void __launch_bounds__(1024) nrm2_kernel(int64_t n, const double* __restrict__ x, double* out)
{
    __shared__ double red[32];
    double s = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s = fma(x[i], x[i], s);
    #pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
        #pragma unroll
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        if (threadIdx.x == 0) *out = sqrt(s);
    }
}

__global__ void transpose_kernel(int64_t m, int64_t n, const double* __restrict__ A, int64_t lda,
                                 double* __restrict__ B, int64_t ldb)
{
    __shared__ double tl[32][33];
    const int64_t i0 = int64_t(blockIdx.x) * 32, j0 = int64_t(blockIdx.y) * 32;
    const int tx = threadIdx.x % 32, ty = threadIdx.x / 32;
    for (int q = ty; q < 32; q += 8) {
        int64_t gi = i0 + tx, gj = j0 + q;
        if (gi < m && gj < n) tl[q][tx] = A[gi + gj * lda];
    }
    __syncthreads();
    for (int q = ty; q < 32; q += 8) {
        int64_t gi = j0 + tx, gj = i0 + q;   // B(gi, gj) = A(gj, gi)
        if (gi < n && gj < m) B[gi + gj * ldb] = tl[tx][q];
    }
}
} // namespace slt

extern "C" int slt_dnrm2(int64_t n, const double* x, double* out, cudaStream_t stream)
{
    nrm2_kernel<<<1, 1024, 0, stream>>>(n, x, out); slt::count_launch();
    return slt_from_cuda(cudaGetLastError());
}

extern "C" int slt_dtranspose(int64_t m, int64_t n, const double* A, int64_t lda, double* B, int64_t ldb,
                              cudaStream_t stream)
{
    if (m <= 0 || n <= 0) return SLT_OK;
    dim3 grid(unsigned(ceildiv(m, 32)), unsigned(ceildiv(n, 32)));
    transpose_kernel<<<grid, 256, 0, stream>>>(m, n, A, lda, B, ldb); slt::count_launch();
    return slt_from_cuda(cudaGetLastError());
}

// ---------------------------------------------------------------------------
namespace slt {
// Column segments of an n x n residual product with nc right-hand sides whose
// partial sums (nseg x n x nc doubles) must fit in ws_doubles: the usual plan,
// with the segment count lowered (more 64-column tiles per segment) when it
// does not fit.  Requires n x nc <= ws_doubles.
static void plan_segments_fit(int64_t n, int64_t nc, size_t ws_doubles, int64_t* nseg, int64_t* tps)
{
    plan_segments(n, n, nseg, tps);
    const int64_t ktiles = ceildiv(n, 64);
    const int64_t fit = int64_t(ws_doubles / (size_t(n) * size_t(nc)));
    if (*nseg > fit) {
        *tps = ceildiv(ktiles, fit);
        *nseg = ceildiv(ktiles, *tps);
    }
}

// Residual into caller-provided partial-sum scratch (ws_doubles doubles): the
// column-segment count is lowered until the partial sums fit.  Used by the
// allocation-free entry point; returns SLT_ERR_LIMIT when a single segment
// (n x min(nrhs, 16) doubles) does not fit.
int dresidual_into(int64_t n, int64_t nrhs, const double* A, int64_t lda, int sym_lower, const double* B,
                   int64_t ldb, const double* X, int64_t ldx, double* R, int64_t ldr, double* ws,
                   size_t ws_doubles, cudaStream_t stream)
{
    if (n < 0 || nrhs < 0) return SLT_ERR_ARG;
    if (n == 0 || nrhs == 0) return SLT_OK;
    const int64_t chunk = std::min<int64_t>(nrhs, kMaxRhs);
    if (size_t(n) * size_t(chunk) > ws_doubles) return SLT_ERR_LIMIT;
    SLT_CUDA_TRY(cudaMemcpy2DAsync(R, size_t(ldr) * sizeof(double), B, size_t(ldb) * sizeof(double),
                                   size_t(n) * sizeof(double), size_t(nrhs), cudaMemcpyDeviceToDevice, stream));
    // Each chunk of up to 16 columns reuses the scratch from offset 0: its
    // product launch writes the partial sums and its reduction reads them
    // before the next chunk's product overwrites them, which holds only
    // because all of them run in order on the one stream.
    for (int64_t c0 = 0; c0 < nrhs; c0 += kMaxRhs) {
        const int64_t nc = std::min<int64_t>(kMaxRhs, nrhs - c0);
        int64_t nseg, tps;
        plan_segments_fit(n, nc, ws_doubles, &nseg, &tps);
        dim3 grid(unsigned(ceildiv(n, 64)), unsigned(nseg));
        int rc = sym_lower ? launch_rowop<0, true>(grid, stream, n, n, int(nc), A, lda, X + c0 * ldx, ldx, tps, ws)
                           : launch_rowop<0, false>(grid, stream, n, n, int(nc), A, lda, X + c0 * ldx, ldx, tps, ws);
        if (rc) return rc;
        dim3 g2(unsigned(ceildiv(n, 256)), unsigned(nc));
        reduce_segments_kernel<<<g2, 256, 0, stream>>>(n, int(nc), nseg, ws, -1.0, 1.0, R + c0 * ldr, ldr);
        slt::count_launch();
        SLT_CUDA_TRY(cudaGetLastError());
    }
    return SLT_OK;
}
} // namespace slt

// The segment plan of the allocation-free residual (host only, for tests):
// segment count and 64-column tiles per segment for order n, nc <= 16
// right-hand sides and ws_doubles doubles of scratch.  SLT_ERR_LIMIT when one
// segment does not fit.
extern "C" int slt_noalloc_segment_plan(int64_t n, int64_t nc, uint64_t ws_doubles, int64_t* nseg, int64_t* tps)
{
    if (n <= 0 || nc <= 0 || nc > 16 || !nseg || !tps) return SLT_ERR_ARG;
    if (uint64_t(n) * uint64_t(nc) > ws_doubles) return SLT_ERR_LIMIT;
    slt::plan_segments_fit(n, nc, size_t(ws_doubles), nseg, tps);
    return SLT_OK;
}
