// matgen.cu -- test matrices with prescribed singular values / eigenvalues.
//
// SLATE's tester builds kind "svd" (A = U diag(sigma) V^T) and "poev"
// (A = Q diag(lambda) Q^T) from Haar-orthogonal factors, the QR of Gaussian
// matrices (matgen/generate_type_svd.hh, matgen/generate_type_heev.hh), with
// sigma from matgen/generate_sigma.hh:73-125 ("geo": sigma_i =
// cond^(-i/(n-1)); "logrand": exp(u_i log(1/cond)) with sigma_0 = 1,
// sigma_1 = 1/cond).  A Haar factor costs an O(n^3) FP64 QR, about 40 s at
// n = 32768 on this part, so the orthogonal factors here are products of
// log2(n) random butterfly levels instead: level l rotates every pair of rows
// (i, i + 2^l) inside blocks of 2^(l+1) by a Philox-drawn angle, after a
// Philox sign flip per row.  Each level is orthogonal, so the singular values
// (eigenvalues) are exactly sigma (lambda) up to rounding, and after log2(n)
// levels every entry depends on every sigma: the matrix is dense.  Cost:
// O(n^2 log n) FP64, one launch per level and side.

#include "common.cuh"
#include "prof.h"

namespace slt {

__device__ __forceinline__ void mg_philox(uint64_t s0, uint64_t s1, uint64_t key, uint64_t out[2])
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

__device__ __forceinline__ double mg_unit(uint64_t bits) { return double(bits >> 11) / double(uint64_t(1) << 53); }

// sigma / lambda on the diagonal of a zeroed A.  dist 0: geo, 1: logrand.
__global__ void sigma_diag_kernel(int64_t n, double cond, int dist, int64_t seed, double* A, int64_t lda)
{
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s;
    if (dist == 0) {
        s = (n > 1) ? pow(cond, -double(i) / double(n - 1)) : 1.0;
    }
    else {
        uint64_t b[2];
        mg_philox(uint64_t(i), 0ull, uint64_t(seed), b);
        s = exp(mg_unit(b[0]) * log(1.0 / cond));
        if (n >= 2 && i == 0) s = 1.0;
        if (n >= 2 && i == 1) s = 1.0 / cond;
    }
    A[i + i * lda] = s;
}

// One butterfly level.  Rows (COLS = false): A <- R_l A, one thread per row
// pair, looping over columns.  Columns (COLS = true): A <- A R_l^T, one
// thread per row of A, looping over column pairs, so that every access is
// coalesced.  R_l rotates the pair (i, i + h) by a Philox angle after a
// Philox sign flip of i; the same seed gives the same R_l on both sides.
__device__ __forceinline__ void mg_pair(int64_t p, int64_t h, int64_t& i, int64_t& k)
{
    i = (p / h) * 2 * h + (p % h);
    k = i + h;
}

__device__ __forceinline__ void mg_rot(int64_t i, int level, int64_t seed, double& c, double& s, double& si)
{
    uint64_t b[2];
    mg_philox(uint64_t(i), uint64_t(level), uint64_t(seed), b);
    const double th = 6.283185307179586 * mg_unit(b[0]);
    c = cos(th);
    s = sin(th);
    si = (b[1] & 1) ? -1.0 : 1.0;
}

__global__ void butterfly_rows_kernel(int64_t n, int64_t h, int64_t npairs, int level, int64_t seed,
                                      double* A, int64_t lda)
{
    const int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p >= npairs) return;
    int64_t i, k;
    mg_pair(p, h, i, k);
    double c, s, si;
    mg_rot(i, level, seed, c, s, si);
    for (int64_t j = blockIdx.y; j < n; j += gridDim.y) {
        double* x = &A[i + j * lda];
        double* y = &A[k + j * lda];
        const double xi = si * *x, yk = *y;
        *x = c * xi + s * yk;
        *y = -s * xi + c * yk;
    }
}

__global__ void butterfly_cols_kernel(int64_t n, int64_t h, int64_t npairs, int level, int64_t seed,
                                      double* A, int64_t lda)
{
    const int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (r >= n) return;
    for (int64_t p = blockIdx.y; p < npairs; p += gridDim.y) {
        int64_t i, k;
        mg_pair(p, h, i, k);
        double c, s, si;
        mg_rot(i, level, seed, c, s, si);
        double* x = &A[r + i * lda];
        double* y = &A[r + k * lda];
        const double xi = si * *x, yk = *y;
        *x = c * xi + s * yk;
        *y = -s * xi + c * yk;
    }
}

} // namespace slt

using namespace slt;

// A (n x n, column-major) = Q1 diag(sigma) Q2^T (spd = 0) or Q diag(sigma) Q^T
// (spd = 1) with sigma from the geo (dist 0) or logrand (dist 1)
// distribution of condition number cond, Q from random butterfly levels.
extern "C" int slt_dgenerate_sigma(int64_t n, double cond, int dist, int spd, int64_t seed, double* A,
                                   int64_t lda, cudaStream_t stream)
{
    if (n <= 0) return SLT_OK;
    if (lda < n || cond < 1.0 || (dist != 0 && dist != 1)) return SLT_ERR_ARG;
    SLT_CUDA_TRY(cudaMemset2DAsync(A, size_t(lda) * sizeof(double), 0, size_t(n) * sizeof(double), size_t(n), stream));
    sigma_diag_kernel<<<unsigned(ceildiv(n, 256)), 256, 0, stream>>>(n, cond, dist, seed, A, lda);
    count_launch();
    SLT_CUDA_TRY(cudaGetLastError());
    int levels = 0;
    while ((int64_t(1) << levels) < n) ++levels;
    for (int l = 0; l < levels; ++l) {
        const int64_t h = int64_t(1) << l;
        const int64_t npairs = (n / (2 * h)) * h + std::max<int64_t>(0, std::min<int64_t>(h, n % (2 * h) - h));
        if (npairs <= 0) continue;
        dim3 g1(unsigned(ceildiv(npairs, 256)), unsigned(std::min<int64_t>(n, 2048)));
        butterfly_rows_kernel<<<g1, 256, 0, stream>>>(n, h, npairs, l, seed + 101, A, lda);
        count_launch();
        // right factor: the same levels (SPD) or an independent draw
        dim3 g2(unsigned(ceildiv(n, 256)), unsigned(std::min<int64_t>(npairs, 2048)));
        butterfly_cols_kernel<<<g2, 256, 0, stream>>>(n, h, npairs, l, spd ? seed + 101 : seed + 202, A, lda);
        count_launch();
        SLT_CUDA_TRY(cudaGetLastError());
    }
    return SLT_OK;
}
