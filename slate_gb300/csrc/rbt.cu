// rbt.cu -- random butterfly transforms (SLATE's gerbt, src/gerbt.cc,
// src/internal/Tile_gerbt.hh) and their random diagonals
// (src/internal/internal_rbt_generate.cc).
//
// A butterfly of half length H pairs row x (x mod 2H < H) with row x + H:
//     W = 1/sqrt(2) [ D1  D2 ]        W^T = 1/sqrt(2) [ D1  D1 ]
//                   [ D1 -D2 ]                        [ D2 -D2 ]
// with D the random diagonal.  A depth-d transform applies d levels; level k
// (0 = largest) has 2^k butterflies of half length
//     H_k = 2^(d-k-1) * ceil(nt / 2^d) * nb     (nt = ceil(n / nb) tiles)
// (gerbt_iterate_1d / _2d), and a row whose partner x + H_k lies past n is
// only scaled by its diagonal entry (the short-tile branches of
// Tile_gerbt.hh).  As in SLATE every level uses the same diagonal (the first
// column of its packed n x d storage).
//
// Two-sided: A <- W_U^T A W_V, smallest butterflies first.
// One-sided: B <- W^T B (smallest first) or B <- W B (largest first).
// Each element is produced by the arithmetic of Tile_gerbt.hh in the same
// order, with every product and sum rounded separately (no fused
// multiply-add), so the oracle's restatement reproduces it bit for bit.

#include "common.cuh"
#include "prof.h"
#include "slate_gb300.h"

#include <cmath>

namespace slt {

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }

// t-th index of the first halves of the butterflies of half length H
__device__ __forceinline__ int64_t first_half(int64_t t, int64_t H) { return (t / H) * 2 * H + t % H; }

__global__ void rbt_diag_kernel(int64_t n, double* w)
{
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) w[i] = exp(w[i] / 20.0);
}

// One level of A <- W_U^T A W_V.  Thread (tx, ty) owns rows x, x + H and
// columns y, y + H.
__global__ void rbt2_kernel(int64_t n, double* __restrict__ A, int64_t lda, const double* __restrict__ u,
                            const double* __restrict__ v, int64_t H, int64_t T)
{
    const double h = 0.5, r2 = 1.0 / sqrt(2.0);
    const int64_t tx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (tx >= T) return;
    const int64_t x = first_half(tx, H);
    if (x >= n) return;
    const int64_t x2 = x + H;
    const bool px = x2 < n;
    const double u1 = u[x], u2 = px ? u[x2] : 0.0;
    for (int64_t ty = int64_t(blockIdx.y) * blockDim.y + threadIdx.y; ty < T; ty += int64_t(gridDim.y) * blockDim.y) {
        const int64_t y = first_half(ty, H);
        if (y >= n) continue;
        const int64_t y2 = y + H;
        const bool py = y2 < n;
        const double v1 = v[y], v2 = py ? v[y2] : 0.0;
        double* c1 = A + y * lda;
        double* c2 = A + y2 * lda;
        const double a11 = c1[x];
        if (px && py) {
            const double a12 = c2[x], a21 = c1[x2], a22 = c2[x2];
            const double s1 = add(a11, a12), s2 = add(a21, a22);
            const double d1 = sub(a11, a12), d2 = sub(a21, a22);
            c1[x] = mul(mul(mul(h, u1), add(s1, s2)), v1);
            c2[x] = mul(mul(mul(h, u1), add(d1, d2)), v2);
            c1[x2] = mul(mul(mul(h, u2), sub(s1, s2)), v1);
            c2[x2] = mul(mul(mul(h, u2), sub(d1, d2)), v2);
        }
        else if (py) {            // row x unpaired
            const double a12 = c2[x];
            c1[x] = mul(mul(mul(r2, u1), add(a11, a12)), v1);
            c2[x] = mul(mul(mul(r2, u1), sub(a11, a12)), v2);
        }
        else if (px) {            // column y unpaired
            const double a21 = c1[x2];
            c1[x] = mul(mul(mul(r2, u1), add(a11, a21)), v1);
            c1[x2] = mul(mul(mul(r2, u2), sub(a11, a21)), v1);
        }
        else {
            c1[x] = mul(mul(u1, a11), v1);
        }
    }
}

// One level of B <- W^T B (TRANS) or B <- W B.  Thread per (first-half row, column).
template <bool TRANS>
__global__ void rbt1_kernel(int64_t n, int64_t nrhs, double* __restrict__ B, int64_t ldb,
                            const double* __restrict__ w, int64_t H, int64_t T)
{
    const double r2 = 1.0 / sqrt(2.0);
    const int64_t tx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (tx >= T) return;
    const int64_t x = first_half(tx, H);
    if (x >= n) return;
    const int64_t x2 = x + H;
    const bool px = x2 < n;
    const double w1 = w[x], w2 = px ? w[x2] : 0.0;
    for (int64_t j = blockIdx.y; j < nrhs; j += gridDim.y) {
        double* c = B + j * ldb;
        const double b1 = c[x];
        if (!px) {
            c[x] = mul(w1, b1);
            continue;
        }
        const double b2 = c[x2];
        if (TRANS) {
            c[x] = mul(mul(r2, w1), add(b1, b2));
            c[x2] = mul(mul(r2, w2), sub(b1, b2));
        }
        else {
            c[x] = mul(r2, add(mul(w1, b1), mul(w2, b2)));
            c[x2] = mul(r2, sub(mul(w1, b1), mul(w2, b2)));
        }
    }
}

} // namespace slt

using namespace slt;

namespace {

// half length of level k (0 = largest) of a depth-d transform of n rows in tiles of nb
int64_t rbt_half(int64_t n, int64_t nb, int64_t d, int64_t k)
{
    const int64_t nt = (n + nb - 1) / nb;
    const int64_t inner = (nt + (int64_t(1) << d) - 1) >> d;
    return (int64_t(1) << (d - k - 1)) * inner * nb;
}

int check(int64_t n, int64_t nb, int64_t d)
{
    if (n < 0 || nb < 1 || d < 0 || d > 20) return SLT_ERR_ARG;
    return SLT_OK;
}

} // namespace

// w[0 .. n) = exp(r / 20) with r uniform(-1, 1) from the Philox stream of
// `seed` (SLATE: exp(larnv(2) / 20), internal_rbt_generate.cc:36-50).
extern "C" int slt_drbt_diag_device(int64_t n, int64_t seed, double* w, slt_stream_t stream)
{
    if (n < 0) return SLT_ERR_ARG;
    if (n == 0) return SLT_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    TRY(slt_dgenerate_device(2, seed, n, 1, 0, 0, w, n, stream));
    rbt_diag_kernel<<<unsigned(ceildiv(n, 256)), 256, 0, s>>>(n, w);
    count_launch();
    return slt_from_cuda(cudaGetLastError());
}

// A <- W_U^T A W_V, depth d, tiles of nb (slate::gerbt(U, A, V)).
extern "C" int slt_dgerbt2_device(int64_t n, double* dA, int64_t lda, const double* u, const double* v, int64_t d,
                                  int64_t nb, slt_stream_t stream)
{
    TRY(check(n, nb, d));
    if (lda < std::max<int64_t>(1, n)) return SLT_ERR_ARG;
    if (n == 0 || d == 0) return SLT_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    for (int64_t k = d - 1; k >= 0; --k) {
        const int64_t H = rbt_half(n, nb, d, k);
        const int64_t T = ((n + 2 * H - 1) / (2 * H)) * H;
        dim3 blk(64, 4);
        dim3 grd(unsigned(ceildiv(T, 64)), unsigned(std::min<int64_t>(ceildiv(T, 4), 65535)));
        rbt2_kernel<<<grd, blk, 0, s>>>(n, dA, lda, u, v, H, T);
        count_launch();
    }
    return slt_from_cuda(cudaGetLastError());
}

// B <- W^T B (trans = 'T') or W B (trans = 'N') (slate::gerbt(U, B)).
extern "C" int slt_dgerbt1_device(char trans, int64_t n, int64_t nrhs, double* dB, int64_t ldb, const double* w,
                                  int64_t d, int64_t nb, slt_stream_t stream)
{
    TRY(check(n, nb, d));
    const bool tr = trans == 'T' || trans == 't' || trans == 'C' || trans == 'c';
    if (!tr && trans != 'N' && trans != 'n') return SLT_ERR_ARG;
    if (nrhs < 0 || ldb < std::max<int64_t>(1, n)) return SLT_ERR_ARG;
    if (n == 0 || nrhs == 0 || d == 0) return SLT_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    for (int64_t it = 0; it < d; ++it) {
        const int64_t k = tr ? d - 1 - it : it;
        const int64_t H = rbt_half(n, nb, d, k);
        const int64_t T = ((n + 2 * H - 1) / (2 * H)) * H;
        dim3 grd(unsigned(ceildiv(T, 256)), unsigned(std::min<int64_t>(nrhs, 65535)));
        if (tr) rbt1_kernel<true><<<grd, 256, 0, s>>>(n, nrhs, dB, ldb, w, H, T);
        else rbt1_kernel<false><<<grd, 256, 0, s>>>(n, nrhs, dB, ldb, w, H, T);
        count_launch();
    }
    return slt_from_cuda(cudaGetLastError());
}
