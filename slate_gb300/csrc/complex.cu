// complex.cu -- the complex (c = complex<float>, z = complex<double>) LU and
// Cholesky solve path: kernels, drivers and their device entry points.
//
// SLATE instantiates its drivers for complex<float> and complex<double>
// (src/getrf.cc, src/potrf.cc, src/gesv_mixed.cc:293-314); this file is the
// GB300 build of those instantiations.  The algorithms are the real path's:
//  * getrf: right-looking LU in block columns of nb.  The panel is factored
//    in stripes of kLeafW columns as SLATE's tile::getrf does with its ib
//    stripes (src/internal/Tile_getrf.hh:159-447): per column the largest
//    cabs1 = |re| + |im| (first row on ties, SLATE's order with one panel
//    thread) under SLATE's pivot-threshold rule, the row interchange across
//    the stripe, scaling by the reciprocal pivot (division below the safe
//    minimum), a rank-1 update inside the stripe; then the interchanges on
//    the rest of the panel, the stripe's U rows by a unit-lower solve and a
//    rank-kLeafW update of the rest of the panel.  After the panel: the
//    interchanges on the columns left and right of it, the U12 solve and the
//    trailing update (src/getrf.cc:81-236).
//  * potrf: lower, right-looking in block columns: the diagonal block by one
//    CTA, the column below by a right conjugate-transpose solve, the
//    trailing Hermitian update C -= L21 L21^H on the lower triangle
//    (src/potrf.cc:22-210).
//  * getrs / potrs: row interchanges, then blocked triangular solves by
//    block rows of kTriB (a small solve per diagonal block and a GEMM update
//    of the remaining rows); Trans and ConjTrans run the sweeps in reverse.
//  * zcgesv: SLATE's gesv_mixed<complex<double>, complex<float>>
//    (src/gesv_mixed.cc:105-289): complex<float> LU, complex<double>
//    residuals, the same stopping test and iteration codes, and the
//    complex<double> fallback.
// Every kernel here is plain SIMT code: FP64 has no tensor instruction on
// this part, and the complex path is not the benchmarked one.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

#include "common.cuh"
#include "cplx.cuh"
#include "drivers.h"
#include "prof.h"

namespace slt {

constexpr int kLeafW = 16;        // panel stripe width
constexpr int kTriB = 64;         // diagonal block of the triangular solves
constexpr int kLeafThreads = 512;
constexpr int kPotrfThreads = 512;

template <typename T> __host__ __device__ __forceinline__ T zero() { return T(0); }

template <typename T> __device__ __forceinline__ T shfl_xor(T v, int off)
{
    if constexpr (Scalar<T>::complex) {
        v.re = __shfl_xor_sync(0xffffffffu, v.re, off);
        v.im = __shfl_xor_sync(0xffffffffu, v.im, off);
        return v;
    }
    else {
        return __shfl_xor_sync(0xffffffffu, v, off);
    }
}

// ---------------------------------------------------------------------------
// C (m x n) = alpha op(A) op(B) + beta C.  op: 0 none, 1 transpose, 2
// conjugate transpose (A is then k x m, B n x k).  lower: only C(i, j),
// i >= j.  64 x 64 tiles walked with a grid stride, 256 threads, 4 x 4
// outputs per thread.
template <typename T, int OPA, int OPB>
__global__ void __launch_bounds__(256)
cgemm_kernel(int64_t m, int64_t n, int64_t k, T alpha, const T* __restrict__ A, int64_t lda,
             const T* __restrict__ B, int64_t ldb, T beta, T* __restrict__ C, int64_t ldc, int lower)
{
    constexpr int BM = 64, BN = 64, BK = 8;
    __shared__ T As[BK][BM + 1];
    __shared__ T Bs[BK][BN + 1];
    const int t = threadIdx.x;
    const int ty = t % 16, tx = t / 16;
    const int64_t tm = ceildiv(m, BM), tiles = tm * ceildiv(n, BN);
    for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const int64_t row0 = (tile % tm) * BM, col0 = (tile / tm) * BN;
        if (lower && row0 + BM - 1 < col0) continue;
        T acc[4][4];
        #pragma unroll
        for (int r = 0; r < 4; ++r)
            #pragma unroll
            for (int c = 0; c < 4; ++c) acc[r][c] = zero<T>();
        for (int64_t k0 = 0; k0 < k; k0 += BK) {
            __syncthreads();
            for (int e = t; e < BM * BK; e += 256) {
                int i, l;
                if (OPA == 0) { i = e % BM; l = e / BM; }
                else          { l = e % BK; i = e / BK; }
                const int64_t gi = row0 + i, gl = k0 + l;
                T v = zero<T>();
                if (gi < m && gl < k) {
                    v = OPA == 0 ? A[gi + gl * lda] : A[gl + gi * lda];
                    if (OPA == 2) v = conj(v);
                }
                As[l][i] = v;
            }
            for (int e = t; e < BN * BK; e += 256) {
                int l, j;
                if (OPB == 0) { l = e % BK; j = e / BK; }
                else          { j = e % BN; l = e / BN; }
                const int64_t gj = col0 + j, gl = k0 + l;
                T v = zero<T>();
                if (gj < n && gl < k) {
                    v = OPB == 0 ? B[gl + gj * ldb] : B[gj + gl * ldb];
                    if (OPB == 2) v = conj(v);
                }
                Bs[l][j] = v;
            }
            __syncthreads();
            #pragma unroll
            for (int l = 0; l < BK; ++l) {
                T a[4], b[4];
                #pragma unroll
                for (int r = 0; r < 4; ++r) a[r] = As[l][ty + 16 * r];
                #pragma unroll
                for (int c = 0; c < 4; ++c) b[c] = Bs[l][tx + 16 * c];
                #pragma unroll
                for (int r = 0; r < 4; ++r)
                    #pragma unroll
                    for (int c = 0; c < 4; ++c) acc[r][c] = fma(a[r], b[c], acc[r][c]);
            }
        }
        #pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int64_t gj = col0 + tx + 16 * c;
            if (gj >= n) continue;
            #pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int64_t gi = row0 + ty + 16 * r;
                if (gi >= m || (lower && gi < gj)) continue;
                T* p = C + gi + gj * ldc;
                *p = (beta == zero<T>()) ? alpha * acc[r][c] : fma(alpha, acc[r][c], beta * *p);
            }
        }
    }
}

template <typename T, int OPA>
static void cgemm_launch_b(int opb, unsigned grid, cudaStream_t s, int64_t m, int64_t n, int64_t k, T alpha,
                           const T* A, int64_t lda, const T* B, int64_t ldb, T beta, T* C, int64_t ldc, int lower)
{
    if (opb == 0) cgemm_kernel<T, OPA, 0><<<grid, 256, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, lower);
    else if (opb == 1) cgemm_kernel<T, OPA, 1><<<grid, 256, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, lower);
    else cgemm_kernel<T, OPA, 2><<<grid, 256, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, lower);
}

template <typename T>
int cgemm(int opa, int opb, int64_t m, int64_t n, int64_t k, T alpha, const T* A, int64_t lda, const T* B,
          int64_t ldb, T beta, T* C, int64_t ldc, int lower, cudaStream_t s)
{
    if (m <= 0 || n <= 0) return SLT_OK;
    const int64_t tiles = ceildiv(m, 64) * ceildiv(n, 64);
    const unsigned grid = unsigned(std::min<int64_t>(tiles, 152 * 8));
    const int pidx = prof_begin(SLT_PROF_GEMM64, s);
    if (opa == 0) cgemm_launch_b<T, 0>(opb, grid, s, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, lower);
    else if (opa == 1) cgemm_launch_b<T, 1>(opb, grid, s, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, lower);
    else cgemm_launch_b<T, 2>(opb, grid, s, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, lower);
    count_launch();
    prof_end(pidx, s, 8.0 * double(m) * double(n) * double(k), double(sizeof(T)) * double(m * k + k * n + 2 * m * n));
    return slt_from_cuda(cudaGetLastError());
}

// ---------------------------------------------------------------------------
// Small triangular solves op(M) x = b with the kb x kb triangle M (kb <=
// kTriB) for many vectors: vector v has its entries at X[i * si + v * sv]
// (columns of B: si = 1, sv = ldb; rows of B: si = ldb, sv = 1).  LOWER:
// M's lower triangle (else upper); UNIT: unit diagonal; OP: 0 none, 1
// transpose, 2 conjugate transpose; CIO: conjugate each vector on the way in
// and out (the right-side solve X M^H = B is M conj(x)^T = conj(b)^T).  One
// warp per vector with the vector in shared memory; the triangle is staged
// once per block.
template <typename T, bool LOWER, bool UNIT, int OP, bool CIO>
__global__ void __launch_bounds__(256)
ctrsv_small_kernel(int kb, int64_t nvec, const T* __restrict__ M, int64_t ldm, T* X, int64_t si, int64_t sv)
{
    extern __shared__ unsigned char smraw[];
    T* Ms = reinterpret_cast<T*>(smraw);                 // kb x kb, column-major, ld kb
    T* xs = Ms + kb * kb;                                // 8 vectors x kb
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    for (int e = t; e < kb * kb; e += 256) {
        const int i = e % kb, j = e / kb;
        Ms[e] = M[i + j * ldm];
    }
    const int64_t v = int64_t(blockIdx.x) * 8 + warp;
    T* x = xs + warp * kb;
    if (v < nvec)
        for (int i = lane; i < kb; i += 32) {
            const T b = X[i * si + v * sv];
            x[i] = CIO ? conj(b) : b;
        }
    __syncthreads();
    if (v >= nvec) return;
    auto opm = [&](int i, int j) -> T {     // entry (i, j) of op(M)
        if (OP == 0) return Ms[i + j * kb];
        const T a = Ms[j + i * kb];
        return OP == 2 ? conj(a) : a;
    };
    // op(M) is lower triangular when M is lower and not transposed, or upper and transposed
    constexpr bool FWD = (LOWER == (OP == 0));
    for (int s = 0; s < kb; ++s) {
        const int i = FWD ? s : kb - 1 - s;
        T part = zero<T>();
        if (FWD) { for (int j = lane; j < i; j += 32) part = fma(opm(i, j), x[j], part); }
        else     { for (int j = i + 1 + lane; j < kb; j += 32) part = fma(opm(i, j), x[j], part); }
        #pragma unroll
        for (int off = 16; off > 0; off >>= 1) part += shfl_xor(part, off);
        if (lane == 0) {
            T xi = x[i] - part;
            if (!UNIT) xi = xi / opm(i, i);
            x[i] = xi;
        }
        __syncwarp();
    }
    for (int i = lane; i < kb; i += 32) X[i * si + v * sv] = CIO ? conj(x[i]) : x[i];
}

template <typename T, bool LOWER, bool UNIT, int OP, bool CIO>
static int ctrsv_small(int kb, int64_t nvec, const T* M, int64_t ldm, T* X, int64_t si, int64_t sv, cudaStream_t s)
{
    if (kb <= 0 || nvec <= 0) return SLT_OK;
    if (kb > kTriB) return SLT_ERR_ARG;
    const size_t smem = sizeof(T) * size_t(kb) * (kb + 8);
    auto kf = ctrsv_small_kernel<T, LOWER, UNIT, OP, CIO>;
    SLT_SMEM_ONCE(kf, sizeof(T) * size_t(kTriB) * (kTriB + 8));
    const int pidx = prof_begin(SLT_PROF_TRSM, s);
    kf<<<unsigned(ceildiv(nvec, 8)), 256, smem, s>>>(kb, nvec, M, ldm, X, si, sv);
    count_launch();
    prof_end(pidx, s, 4.0 * double(kb) * double(kb) * double(nvec), double(sizeof(T)) * 2.0 * kb * nvec);
    return slt_from_cuda(cudaGetLastError());
}

// Left solve op(M) X = X, M n x n triangular, X n x nrhs, blocked by kTriB:
// a small solve per diagonal block, then a GEMM update of the rows still to
// solve (below the block in a forward sweep, above it in a backward one).
template <typename T, bool LOWER, bool UNIT, int OP>
int ctrsm_left(int64_t n, int64_t nrhs, const T* M, int64_t ldm, T* X, int64_t ldx, cudaStream_t s)
{
    if (n <= 0 || nrhs <= 0) return SLT_OK;
    constexpr bool FWD = (LOWER == (OP == 0));
    const int64_t nblk = ceildiv(n, kTriB);
    for (int64_t q = 0; q < nblk; ++q) {
        const int64_t b = FWD ? q : nblk - 1 - q;
        const int64_t r0 = b * kTriB, kb = std::min<int64_t>(kTriB, n - r0);
        TRY((ctrsv_small<T, LOWER, UNIT, OP, false>(int(kb), nrhs, M + r0 + r0 * ldm, ldm, X + r0, 1, ldx, s)));
        const int64_t o0 = FWD ? r0 + kb : 0, on = FWD ? n - r0 - kb : r0;
        if (on <= 0) continue;
        // X(o, :) -= op(M)(o, blk) X(blk, :); op(M)(o, blk) is M(o, blk), or
        // M(blk, o) transposed / conjugate-transposed
        if (OP == 0)
            TRY(cgemm<T>(0, 0, on, nrhs, kb, T(-1), M + o0 + r0 * ldm, ldm, X + r0, ldx, T(1), X + o0, ldx, 0, s));
        else
            TRY(cgemm<T>(OP, 0, on, nrhs, kb, T(-1), M + r0 + o0 * ldm, ldm, X + r0, ldx, T(1), X + o0, ldx, 0, s));
    }
    return SLT_OK;
}

// Right solve X L^H = X (L lower, non-unit), X m x n: row by row it is
// L conj(x)^T = conj(x)^T, so the same blocked forward sweep on the rows of
// X with the vectors conjugated in and out.
template <typename T>
int ctrsm_right_lower_conjtrans(int64_t m, int64_t n, const T* L, int64_t ldl, T* X, int64_t ldx, cudaStream_t s)
{
    if (m <= 0 || n <= 0) return SLT_OK;
    const int64_t nblk = ceildiv(n, kTriB);
    for (int64_t b = 0; b < nblk; ++b) {
        const int64_t c0 = b * kTriB, kb = std::min<int64_t>(kTriB, n - c0);
        TRY((ctrsv_small<T, true, false, 0, true>(int(kb), m, L + c0 + c0 * ldl, ldl, X + c0 * ldx, ldx, 1, s)));
        const int64_t o0 = c0 + kb, on = n - o0;
        if (on <= 0) continue;
        // X(:, o) -= X(:, blk) L(o, blk)^H
        TRY(cgemm<T>(0, 2, m, on, kb, T(-1), X + c0 * ldx, ldx, L + o0 + c0 * ldl, ldl, T(1), X + o0 * ldx, ldx, 0, s));
    }
    return SLT_OK;
}

// ---------------------------------------------------------------------------
// LU of one stripe: the m x w block P (w <= kLeafW), one CTA, column by
// column.  ipiv[j] receives ioff + the pivot row relative to P's first row
// (ioff: P's row offset in its panel, so ipiv is panel-relative);
// *info (device) is set to info_offset + j + 1 at the first exactly zero
// pivot.  The interchanges are applied across the stripe's w columns only.
template <typename T>
__global__ void __launch_bounds__(kLeafThreads)
cgetrf_leaf_kernel(int64_t m, int w, T* P, int64_t ld, int* ipiv, int ioff, int* info, int64_t info_offset,
                   typename Scalar<T>::real threshold)
{
    using R = typename Scalar<T>::real;
    __shared__ R rv[kLeafThreads / 32];
    __shared__ int64_t ri[kLeafThreads / 32];
    __shared__ int64_t piv_s;
    __shared__ T pv_s;
    __shared__ T row_s[kLeafW];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const R safe_min = Scalar<T>::safe_min();
    for (int j = 0; j < w && j < m; ++j) {
        // largest cabs1 in column j at rows >= j; first row on ties
        R best = R(-1);
        int64_t bi = m;
        for (int64_t i = j + t; i < m; i += kLeafThreads) {
            const R a = cabs1(P[i + j * ld]);
            if (a > best) { best = a; bi = i; }
        }
        #pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const R ob = __shfl_xor_sync(0xffffffffu, best, off);
            const int64_t oi = __shfl_xor_sync(0xffffffffu, bi, off);
            if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        if (lane == 0) { rv[warp] = best; ri[warp] = bi; }
        __syncthreads();
        if (t == 0) {
            for (int q = 1; q < kLeafThreads / 32; ++q)
                if (rv[q] > rv[0] || (rv[q] == rv[0] && ri[q] < ri[0])) { rv[0] = rv[q]; ri[0] = ri[q]; }
            int64_t p = ri[0];
            // SLATE's threshold rule: keep the diagonal when it is within
            // the threshold of the largest entry
            const R d = cabs1(P[j + j * ld]);
            if (p >= m || d >= rv[0] * threshold) p = j;
            piv_s = p;
            ipiv[j] = ioff + int(p);
            pv_s = P[p + j * ld];
            if (pv_s == zero<T>()) atomicCAS(info, 0, int(info_offset + j + 1));
        }
        __syncthreads();
        const int64_t p = piv_s;
        if (p != j && t < w) {
            const T a = P[j + t * ld];
            P[j + t * ld] = P[p + t * ld];
            P[p + t * ld] = a;
        }
        __syncthreads();
        if (t < w) row_s[t] = P[j + t * ld];
        __syncthreads();
        const T pv = pv_s;
        if (pv != zero<T>()) {
            const bool recip = cabs1(pv) >= safe_min;
            const T rp = T(1) / pv;
            for (int64_t i = j + 1 + t; i < m; i += kLeafThreads) {
                T l = P[i + j * ld];
                l = recip ? l * rp : l / pv;
                P[i + j * ld] = l;
                for (int c = j + 1; c < w; ++c) P[i + c * ld] = fma(-l, row_s[c], P[i + c * ld]);
            }
        }
        __syncthreads();
    }
}

// Row interchanges: rows k0 + k and ipiv[k] (both relative to A's first row)
// for k = 0 .. cnt-1 in order, on ncols columns of A.  One thread per column.
template <typename T>
__global__ void claswp_kernel(int64_t ncols, T* A, int64_t lda, const int* ipiv, int cnt, int64_t k0)
{
    const int64_t c = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= ncols) return;
    T* col = A + c * lda;
    for (int k = 0; k < cnt; ++k) {
        const int64_t p = ipiv[k], q = k0 + k;
        if (p != q) {
            const T a = col[q];
            col[q] = col[p];
            col[p] = a;
        }
    }
}

template <typename T>
static int claswp(int64_t ncols, T* A, int64_t lda, const int* ipiv, int cnt, int64_t k0, cudaStream_t s)
{
    if (ncols <= 0 || cnt <= 0) return SLT_OK;
    claswp_kernel<T><<<unsigned(ceildiv(ncols, 128)), 128, 0, s>>>(ncols, A, lda, ipiv, cnt, k0);
    count_launch();
    return slt_from_cuda(cudaGetLastError());
}

// Backward interchanges (k = cnt-1 .. 0): the inverse permutation, for the
// transposed solves.
template <typename T>
__global__ void claswp_back_kernel(int64_t ncols, T* A, int64_t lda, const int* ipiv, int64_t n, int64_t nb)
{
    const int64_t c = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= ncols) return;
    T* col = A + c * lda;
    for (int64_t k = n - 1; k >= 0; --k) {
        const int64_t p = (k / nb) * nb + ipiv[k];
        if (p != k) {
            const T a = col[k];
            col[k] = col[p];
            col[p] = a;
        }
    }
}

// ipiv stored per panel (ipiv[k] relative to row (k / nb) * nb): forward
// interchanges of all panels.
template <typename T>
__global__ void claswp_all_kernel(int64_t ncols, T* A, int64_t lda, const int* ipiv, int64_t n, int64_t nb)
{
    const int64_t c = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= ncols) return;
    T* col = A + c * lda;
    for (int64_t k = 0; k < n; ++k) {
        const int64_t p = (k / nb) * nb + ipiv[k];
        if (p != k) {
            const T a = col[k];
            col[k] = col[p];
            col[p] = a;
        }
    }
}

// ---------------------------------------------------------------------------
// Cholesky of the kb x kb diagonal block (lower, Hermitian) by one CTA,
// right-looking column by column.  *info = info_offset + j + 1 at the first
// non-positive (or NaN) pivot, where the block stops.
template <typename T>
__global__ void __launch_bounds__(kPotrfThreads)
cpotrf_block_kernel(int kb, T* A, int64_t lda, int* info, int64_t info_offset)
{
    using R = typename Scalar<T>::real;
    __shared__ int bad;
    __shared__ R dj;
    const int t = threadIdx.x;
    if (t == 0) bad = 0;
    __syncthreads();
    for (int j = 0; j < kb; ++j) {
        if (t == 0) {
            const R d = real(A[j + j * lda]);
            if (!(d > R(0))) {
                bad = 1;
                atomicCAS(info, 0, int(info_offset + j + 1));
            }
            else {
                dj = sqrt(d);
                A[j + j * lda] = T(dj);
            }
        }
        __syncthreads();
        if (bad) return;
        const R rd = R(1) / dj;
        for (int i = j + 1 + t; i < kb; i += kPotrfThreads) A[i + j * lda] = rd * A[i + j * lda];
        __syncthreads();
        // trailing lower part of the block: A(i, c) -= L(i, j) conj(L(c, j)), i >= c > j
        const int rest = kb - j - 1;
        for (int e = t; e < rest * rest; e += kPotrfThreads) {
            const int i = j + 1 + e % rest, c = j + 1 + e / rest;
            if (i >= c) A[i + c * lda] = fma(-A[i + j * lda], conj(A[c + j * lda]), A[i + c * lda]);
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Elementwise helpers of the mixed solver and the norms of its stopping test.
template <typename S, typename D>
__global__ void cconvert_kernel(int64_t m, int64_t n, const S* A, int64_t lda, D* B, int64_t ldb)
{
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= m) return;
    for (int64_t j = blockIdx.y; j < n; j += gridDim.y) {
        const S a = A[i + j * lda];
        B[i + j * ldb] = D(decltype(D::re)(a.re), decltype(D::re)(a.im));
    }
}

// Y = alpha X + beta Y
template <typename T>
__global__ void caxpby_kernel(int64_t m, int64_t n, T alpha, const T* X, int64_t ldx, T beta, T* Y, int64_t ldy)
{
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= m) return;
    for (int64_t j = blockIdx.y; j < n; j += gridDim.y) {
        T* y = Y + i + j * ldy;
        *y = (beta == zero<T>()) ? alpha * X[i + j * ldx] : fma(alpha, X[i + j * ldx], beta * *y);
    }
}

// out[j] = max_i |A(i, j)| (modulus), one block per column.
template <typename T>
__global__ void ccolmax_kernel(int64_t m, const T* A, int64_t lda, typename Scalar<T>::real* out)
{
    using R = typename Scalar<T>::real;
    __shared__ R red[256];
    const T* a = A + int64_t(blockIdx.x) * lda;
    R mx = 0;
    for (int64_t i = threadIdx.x; i < m; i += 256) mx = fmax(mx, cabs(a[i]));
    red[threadIdx.x] = mx;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}

// Row sums of |A(i, j)| into rs (m entries); the infinity norm is their max.
template <typename T>
__global__ void crowsum_kernel(int64_t m, int64_t n, const T* A, int64_t lda, typename Scalar<T>::real* rs)
{
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= m) return;
    typename Scalar<T>::real s = 0;
    for (int64_t j = 0; j < n; ++j) s += cabs(A[i + j * lda]);
    rs[i] = s;
}

template <typename R>
__global__ void rmax_kernel(int64_t m, const R* x, R* out)
{
    __shared__ R red[256];
    R mx = 0;
    for (int64_t i = threadIdx.x; i < m; i += 256) mx = fmax(mx, x[i]);
    red[threadIdx.x] = mx;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

// ---------------------------------------------------------------------------
// Drivers.
template <typename T>
int cgetrf_dev(int64_t m, int64_t n, T* A, int64_t lda, int* ipiv, const slt_options& o, int* d_info,
               cudaStream_t s)
{
    using R = typename Scalar<T>::real;
    if (m < 0 || n < 0 || lda < std::max<int64_t>(1, m)) return SLT_ERR_ARG;
    const int64_t nb = o.nb > 0 ? o.nb : 512;
    const int64_t mn = std::min(m, n);
    const bool nopiv = o.method_lu == 'N' || o.method_lu == 'n';
    R thr = (o.pivot_threshold >= 0.0 && o.pivot_threshold <= 1.0) ? R(o.pivot_threshold) : R(1);
    if (nopiv) thr = R(0);
    for (int64_t r0 = 0; r0 < mn; r0 += nb) {
        const int64_t nbk = std::min(nb, n - r0), prows = m - r0, diag = std::min(prows, nbk);
        T* P = A + r0 + r0 * lda;
        // the panel, in stripes of kLeafW columns
        for (int64_t j0 = 0; j0 < diag; j0 += kLeafW) {
            const int64_t w = std::min<int64_t>(kLeafW, diag - j0);
            T* S = P + j0 + j0 * lda;
            cgetrf_leaf_kernel<T><<<1, kLeafThreads, 0, s>>>(prows - j0, int(w), S, lda, ipiv + r0 + j0, int(j0),
                                                             d_info, r0 + j0, thr);
            count_launch();
            SLT_CUDA_TRY(cudaGetLastError());
            // the stripe's interchanges on the panel columns left and right of it
            TRY(claswp<T>(j0, P, lda, ipiv + r0 + j0, int(w), j0, s));
            TRY(claswp<T>(nbk - j0 - w, P + (j0 + w) * lda, lda, ipiv + r0 + j0, int(w), j0, s));
            if (j0 + w < nbk) {
                TRY((ctrsm_left<T, true, true, 0>(w, nbk - j0 - w, S, lda, S + w * lda, lda, s)));
                if (j0 + w < prows)
                    TRY(cgemm<T>(0, 0, prows - j0 - w, nbk - j0 - w, w, T(-1), S + w, lda, S + w * lda, lda, T(1),
                                 S + w + w * lda, lda, 0, s));
            }
        }
        // the panel's interchanges on the columns left and right of it
        TRY(claswp<T>(r0, A + r0, lda, ipiv + r0, int(diag), 0, s));
        const int64_t c1 = r0 + nbk;
        TRY(claswp<T>(n - c1, A + r0 + c1 * lda, lda, ipiv + r0, int(diag), 0, s));
        if (c1 < n) {
            TRY((ctrsm_left<T, true, true, 0>(diag, n - c1, P, lda, A + r0 + c1 * lda, lda, s)));
            if (r0 + diag < m)
                TRY(cgemm<T>(0, 0, m - r0 - diag, n - c1, diag, T(-1), A + r0 + diag + r0 * lda, lda,
                             A + r0 + c1 * lda, lda, T(1), A + r0 + diag + c1 * lda, lda, 0, s));
        }
    }
    return SLT_OK;
}

// op(A) X = B with getrf's factors (P A = L U): 'N' X = U^-1 L^-1 P B;
// 'T' / 'C' X = P^T L^-T U^-T B (with conjugates for 'C').
template <typename T>
int cgetrs_dev(char trans, int64_t n, int64_t nrhs, const T* LU, int64_t lda, const int* ipiv, int64_t nb, T* B,
               int64_t ldb, cudaStream_t s)
{
    if (n <= 0 || nrhs <= 0) return SLT_OK;
    const unsigned g = unsigned(ceildiv(nrhs, 128));
    if (trans == 'N' || trans == 'n') {
        claswp_all_kernel<T><<<g, 128, 0, s>>>(nrhs, B, ldb, ipiv, n, nb);
        count_launch();
        TRY((ctrsm_left<T, true, true, 0>(n, nrhs, LU, lda, B, ldb, s)));
        TRY((ctrsm_left<T, false, false, 0>(n, nrhs, LU, lda, B, ldb, s)));
        return slt_from_cuda(cudaGetLastError());
    }
    if (trans == 'C' || trans == 'c') {
        TRY((ctrsm_left<T, false, false, 2>(n, nrhs, LU, lda, B, ldb, s)));
        TRY((ctrsm_left<T, true, true, 2>(n, nrhs, LU, lda, B, ldb, s)));
    }
    else {
        TRY((ctrsm_left<T, false, false, 1>(n, nrhs, LU, lda, B, ldb, s)));
        TRY((ctrsm_left<T, true, true, 1>(n, nrhs, LU, lda, B, ldb, s)));
    }
    claswp_back_kernel<T><<<g, 128, 0, s>>>(nrhs, B, ldb, ipiv, n, nb);
    count_launch();
    return slt_from_cuda(cudaGetLastError());
}

template <typename T>
int cpotrf_dev(int64_t n, T* A, int64_t lda, const slt_options& o, int* d_info, cudaStream_t s)
{
    if (n < 0 || lda < std::max<int64_t>(1, n)) return SLT_ERR_ARG;
    const int64_t nb = std::min<int64_t>(o.nb > 0 ? o.nb : 512, 256);
    for (int64_t r0 = 0; r0 < n; r0 += nb) {
        const int64_t kb = std::min(nb, n - r0);
        T* D = A + r0 + r0 * lda;
        cpotrf_block_kernel<T><<<1, kPotrfThreads, 0, s>>>(int(kb), D, lda, d_info, r0);
        count_launch();
        SLT_CUDA_TRY(cudaGetLastError());
        const int64_t t0 = r0 + kb;
        if (t0 >= n) break;
        // L21 = A21 L11^{-H}; A22 -= L21 L21^H (lower)
        TRY(ctrsm_right_lower_conjtrans<T>(n - t0, kb, D, lda, A + t0 + r0 * lda, lda, s));
        TRY(cgemm<T>(0, 2, n - t0, n - t0, kb, T(-1), A + t0 + r0 * lda, lda, A + t0 + r0 * lda, lda, T(1),
                     A + t0 + t0 * lda, lda, 1, s));
    }
    return SLT_OK;
}

template <typename T>
int cpotrs_dev(int64_t n, int64_t nrhs, const T* L, int64_t lda, T* B, int64_t ldb, cudaStream_t s)
{
    TRY((ctrsm_left<T, true, false, 0>(n, nrhs, L, lda, B, ldb, s)));
    return ctrsm_left<T, true, false, 2>(n, nrhs, L, lda, B, ldb, s);
}

template <typename T>
struct Info {
    DevBuf buf;
    int* d = nullptr;
    int init(cudaStream_t s) {
        TRY(buf.alloc(sizeof(int), s));
        d = buf.as<int>();
        SLT_CUDA_TRY(cudaMemsetAsync(d, 0, sizeof(int), s));
        return SLT_OK;
    }
    int read(int64_t* info, cudaStream_t s) {
        int h = 0;
        SLT_CUDA_TRY(cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost, s));
        SLT_CUDA_TRY(cudaStreamSynchronize(s));
        if (info) *info = h;
        return SLT_OK;
    }
};

// ---------------------------------------------------------------------------
// zcgesv: gesv_mixed<complex<double>, complex<float>> (src/gesv_mixed.cc:105-289).
template <typename TH, typename TL>
int cgesv_mixed_dev(int64_t n, int64_t nrhs, TH* A, int64_t lda, int* ipiv, const TH* B, int64_t ldb, TH* X,
                    int64_t ldx, const slt_options& o, int* iter, int64_t* info, cudaStream_t s)
{
    using R = typename Scalar<TH>::real;
    if (n < 0 || nrhs < 0 || lda < std::max<int64_t>(1, n)) return SLT_ERR_ARG;
    *iter = 0;
    *info = 0;
    if (n == 0 || nrhs == 0) return SLT_OK;
    TimerSet tm(s);
    tm.start("gesv_mixed");
    const R eps = std::numeric_limits<R>::epsilon();
    const R tol = o.tolerance > 0 ? R(o.tolerance) : eps * std::sqrt(R(n));
    const int64_t itermax = o.max_iterations;
    const int64_t nb = o.nb > 0 ? o.nb : 512;
    DevBuf Alo, Xlo, Rr, nrm;
    TRY(Alo.alloc(sizeof(TL) * size_t(n) * size_t(n), s));
    TRY(Xlo.alloc(sizeof(TL) * size_t(n) * size_t(nrhs), s));
    TRY(Rr.alloc(sizeof(TH) * size_t(n) * size_t(nrhs), s));
    TRY(nrm.alloc(sizeof(R) * (size_t(n) + 2 * size_t(nrhs) + 1), s));
    R* rs = nrm.as<R>();
    R* cx = rs + n;
    R* cr = cx + nrhs;
    R* anrm = cr + nrhs;
    Info<TH> inf;
    TRY(inf.init(s));
    const dim3 gr(unsigned(ceildiv(n, 256)), unsigned(std::min<int64_t>(nrhs, 65535)));
    const dim3 ga(unsigned(ceildiv(n, 256)), unsigned(std::min<int64_t>(n, 65535)));
    // ||A||_inf
    crowsum_kernel<TH><<<unsigned(ceildiv(n, 256)), 256, 0, s>>>(n, n, A, lda, rs);
    rmax_kernel<R><<<1, 256, 0, s>>>(n, rs, anrm);
    count_launch();
    count_launch();
    R Anorm = 0;
    SLT_CUDA_TRY(cudaMemcpyAsync(&Anorm, anrm, sizeof(R), cudaMemcpyDeviceToHost, s));
    SLT_CUDA_TRY(cudaStreamSynchronize(s));
    const R cte = Anorm * tol;
    // low-precision factors
    tm.start("gesv_mixed::getrf_lo");
    cconvert_kernel<TH, TL><<<ga, 256, 0, s>>>(n, n, A, lda, Alo.as<TL>(), n);
    count_launch();
    slt_options olo = o;
    TRY(cgetrf_dev<TL>(n, n, Alo.as<TL>(), n, ipiv, olo, inf.d, s));
    tm.stop("gesv_mixed::getrf_lo");
    int64_t linfo = 0;
    TRY(inf.read(&linfo, s));
    std::vector<R> h(2 * size_t(nrhs));
    auto lo_solve = [&](const TH* Rin, int64_t ldr, TH* Y, int64_t ldy) -> int {
        cconvert_kernel<TH, TL><<<gr, 256, 0, s>>>(n, nrhs, Rin, ldr, Xlo.as<TL>(), n);
        count_launch();
        TRY(cgetrs_dev<TL>('N', n, nrhs, Alo.as<TL>(), n, ipiv, nb, Xlo.as<TL>(), n, s));
        cconvert_kernel<TL, TH><<<gr, 256, 0, s>>>(n, nrhs, Xlo.as<TL>(), n, Y, ldy);
        count_launch();
        return slt_from_cuda(cudaGetLastError());
    };
    auto residual = [&]() -> int {       // R = B - A X, then the column maxima of X and R
        caxpby_kernel<TH><<<gr, 256, 0, s>>>(n, nrhs, TH(1), B, ldb, TH(0), Rr.as<TH>(), n);
        count_launch();
        TRY(cgemm<TH>(0, 0, n, nrhs, n, TH(-1), A, lda, X, ldx, TH(1), Rr.as<TH>(), n, 0, s));
        for (int64_t c = 0; c < nrhs; ++c) {
            ccolmax_kernel<TH><<<1, 256, 0, s>>>(n, X + c * ldx, ldx, cx + c);
            ccolmax_kernel<TH><<<1, 256, 0, s>>>(n, Rr.as<TH>() + c * n, n, cr + c);
            count_launch();
            count_launch();
        }
        SLT_CUDA_TRY(cudaMemcpyAsync(h.data(), cx, sizeof(R) * 2 * size_t(nrhs), cudaMemcpyDeviceToHost, s));
        SLT_CUDA_TRY(cudaStreamSynchronize(s));
        return SLT_OK;
    };
    auto converged = [&]() {
        for (int64_t c = 0; c < nrhs; ++c)
            if (!(h[nrhs + c] <= h[c] * cte)) return false;
        return true;
    };
    bool conv = false;
    if (linfo != 0) {
        *iter = -3;
    }
    else {
        TRY(lo_solve(B, ldb, X, ldx));
        TRY(residual());
        if (converged()) { *iter = 0; conv = true; }
        for (int64_t it = 0; it < itermax && !conv; ++it) {
            TRY(lo_solve(Rr.as<TH>(), n, Rr.as<TH>(), n));
            caxpby_kernel<TH><<<gr, 256, 0, s>>>(n, nrhs, TH(1), Rr.as<TH>(), n, TH(1), X, ldx);
            count_launch();
            TRY(residual());
            if (converged()) { *iter = int(it + 1); conv = true; }
        }
    }
    *info = linfo;
    if (!conv) {
        if (linfo == 0) *iter = int(-itermax - 1);
        if (o.use_fallback) {
            // the FP64 fallback: A <- its factors, X from them
            Info<TH> f;
            TRY(f.init(s));
            tm.start("gesv_mixed::getrf_hi");
            TRY(cgetrf_dev<TH>(n, n, A, lda, ipiv, o, f.d, s));
            tm.stop("gesv_mixed::getrf_hi");
            TRY(f.read(info, s));
            if (*info == 0) {
                caxpby_kernel<TH><<<gr, 256, 0, s>>>(n, nrhs, TH(1), B, ldb, TH(0), X, ldx);
                count_launch();
                TRY(cgetrs_dev<TH>('N', n, nrhs, A, lda, ipiv, nb, X, ldx, s));
            }
        }
    }
    tm.stop("gesv_mixed");
    SLT_CUDA_TRY(cudaStreamSynchronize(s));
    return slt_from_cuda(cudaGetLastError());
}

template <typename T>
slt_options copts(const slt_options* o)
{
    slt_options r;
    if (o) r = *o;
    else slt_options_default(&r);
    return r;
}

template <typename T>
int getrf_entry(int64_t m, int64_t n, T* A, int64_t lda, int* ipiv, const slt_options* opts, cudaStream_t s,
                int64_t* info)
{
    Info<T> inf;
    TRY(inf.init(s));
    TRY(cgetrf_dev<T>(m, n, A, lda, ipiv, copts<T>(opts), inf.d, s));
    return inf.read(info, s);
}

template <typename T>
int getrs_entry(char trans, int64_t n, int64_t nrhs, const T* LU, int64_t lda, const int* ipiv, T* B,
                int64_t ldb, const slt_options* opts, cudaStream_t s)
{
    if (std::strchr("NnTtCc", trans) == nullptr || trans == 0) return SLT_ERR_ARG;
    const slt_options o = copts<T>(opts);
    TRY(cgetrs_dev<T>(trans, n, nrhs, LU, lda, ipiv, o.nb > 0 ? o.nb : 512, B, ldb, s));
    return slt_from_cuda(cudaStreamSynchronize(s));
}

template <typename T>
int gesv_entry(int64_t n, int64_t nrhs, T* A, int64_t lda, int* ipiv, T* B, int64_t ldb,
               const slt_options* opts, cudaStream_t s, int64_t* info)
{
    TRY(getrf_entry<T>(n, n, A, lda, ipiv, opts, s, info));
    if (*info != 0) return SLT_OK;          // SLATE skips the solve (src/gesv.cc:98-103)
    return getrs_entry<T>('N', n, nrhs, A, lda, ipiv, B, ldb, opts, s);
}

template <typename T>
int potrf_entry(int64_t n, T* A, int64_t lda, const slt_options* opts, cudaStream_t s, int64_t* info)
{
    Info<T> inf;
    TRY(inf.init(s));
    TRY(cpotrf_dev<T>(n, A, lda, copts<T>(opts), inf.d, s));
    return inf.read(info, s);
}

template <typename T>
int potrs_entry(int64_t n, int64_t nrhs, const T* L, int64_t lda, T* B, int64_t ldb, cudaStream_t s)
{
    TRY(cpotrs_dev<T>(n, nrhs, L, lda, B, ldb, s));
    return slt_from_cuda(cudaStreamSynchronize(s));
}

template <typename T>
int posv_entry(int64_t n, int64_t nrhs, T* A, int64_t lda, T* B, int64_t ldb, const slt_options* opts,
               cudaStream_t s, int64_t* info)
{
    TRY(potrf_entry<T>(n, A, lda, opts, s, info));
    if (*info != 0) return SLT_OK;
    return potrs_entry<T>(n, nrhs, A, lda, B, ldb, s);
}

} // namespace slt

using namespace slt;

#define SLT_COMPLEX_ENTRIES(P, T)                                                                           \
extern "C" int slt_##P##getrf_device(int64_t m, int64_t n, void* dA, int64_t lda, int* d_ipiv,              \
                                     const slt_options* opts, slt_stream_t stream, int64_t* info)           \
{ return getrf_entry<T>(m, n, static_cast<T*>(dA), lda, d_ipiv, opts, static_cast<cudaStream_t>(stream), info); } \
extern "C" int slt_##P##getrs_device(char trans, int64_t n, int64_t nrhs, const void* dLU, int64_t lda,      \
                                     const int* d_ipiv, void* dB, int64_t ldb, const slt_options* opts,     \
                                     slt_stream_t stream)                                                   \
{ return getrs_entry<T>(trans, n, nrhs, static_cast<const T*>(dLU), lda, d_ipiv, static_cast<T*>(dB), ldb,  \
                        opts, static_cast<cudaStream_t>(stream)); }                                         \
extern "C" int slt_##P##gesv_device(int64_t n, int64_t nrhs, void* dA, int64_t lda, int* d_ipiv, void* dB,  \
                                    int64_t ldb, const slt_options* opts, slt_stream_t stream, int64_t* info) \
{ return gesv_entry<T>(n, nrhs, static_cast<T*>(dA), lda, d_ipiv, static_cast<T*>(dB), ldb, opts,           \
                       static_cast<cudaStream_t>(stream), info); }                                          \
extern "C" int slt_##P##potrf_device(int64_t n, void* dA, int64_t lda, const slt_options* opts,             \
                                     slt_stream_t stream, int64_t* info)                                    \
{ return potrf_entry<T>(n, static_cast<T*>(dA), lda, opts, static_cast<cudaStream_t>(stream), info); }      \
extern "C" int slt_##P##potrs_device(int64_t n, int64_t nrhs, const void* dL, int64_t lda, void* dB,        \
                                     int64_t ldb, const slt_options* opts, slt_stream_t stream)             \
{ (void) opts; return potrs_entry<T>(n, nrhs, static_cast<const T*>(dL), lda, static_cast<T*>(dB), ldb,     \
                                     static_cast<cudaStream_t>(stream)); }                                  \
extern "C" int slt_##P##posv_device(int64_t n, int64_t nrhs, void* dA, int64_t lda, void* dB, int64_t ldb,  \
                                    const slt_options* opts, slt_stream_t stream, int64_t* info)            \
{ return posv_entry<T>(n, nrhs, static_cast<T*>(dA), lda, static_cast<T*>(dB), ldb, opts,                   \
                       static_cast<cudaStream_t>(stream), info); }

SLT_COMPLEX_ENTRIES(c, cfloat)
SLT_COMPLEX_ENTRIES(z, cdouble)

extern "C" int slt_zcgesv_device(int64_t n, int64_t nrhs, void* dA, int64_t lda, int* d_ipiv, const void* dB,
                                 int64_t ldb, void* dX, int64_t ldx, const slt_options* opts, slt_stream_t stream,
                                 int* iter, int64_t* info)
{
    slt_options o = copts<cdouble>(opts);
    int it = 0;
    int64_t inf = 0;
    const int rc = cgesv_mixed_dev<cdouble, cfloat>(n, nrhs, static_cast<cdouble*>(dA), lda, d_ipiv,
                                                    static_cast<const cdouble*>(dB), ldb, static_cast<cdouble*>(dX),
                                                    ldx, o, &it, &inf, static_cast<cudaStream_t>(stream));
    if (iter) *iter = it;
    if (info) *info = inf;
    return rc;
}

// ---------------------------------------------------------------------------
// Type-generic helpers of the host entry points (types: 0 float, 1 double,
// 2 complex<float>, 3 complex<double>).
namespace slt {

// B (n x m) = A^T (conj: A^H), 32 x 32 tiles through shared memory.
template <typename T, bool CONJ>
__global__ void xtranspose_kernel(int64_t m, int64_t n, const T* A, int64_t lda, T* B, int64_t ldb)
{
    __shared__ T tile[32][33];
    const int64_t i0 = int64_t(blockIdx.x) * 32, j0 = int64_t(blockIdx.y) * 32;
    const int tx = threadIdx.x % 32, ty = threadIdx.x / 32;       // 256 threads: 32 x 8
    for (int r = ty; r < 32; r += 8) {
        const int64_t i = i0 + tx, j = j0 + r;
        if (i < m && j < n) tile[r][tx] = A[i + j * lda];
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
        const int64_t j = j0 + tx, i = i0 + r;                    // B(j, i) = A(i, j)
        if (i < m && j < n) {
            const T v = tile[tx][r];
            B[j + i * ldb] = CONJ ? conj(v) : v;
        }
    }
}

// dst's lower (upper = 0) or upper (upper = 1) triangle <- src's.
template <typename T>
__global__ void xcopy_tri_kernel(int upper, int64_t n, const T* S, int64_t lds, T* D, int64_t ldd)
{
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int64_t j = blockIdx.y; j < n; j += gridDim.y)
        if (upper ? (i <= j) : (i >= j)) D[i + j * ldd] = S[i + j * lds];
}

template <typename T>
static int xtranspose_t(int64_t m, int64_t n, const void* A, int64_t lda, void* B, int64_t ldb, int cj, cudaStream_t s)
{
    if (m <= 0 || n <= 0) return SLT_OK;
    dim3 g(unsigned(ceildiv(m, 32)), unsigned(ceildiv(n, 32)));
    if (cj) xtranspose_kernel<T, true><<<g, 256, 0, s>>>(m, n, static_cast<const T*>(A), lda, static_cast<T*>(B), ldb);
    else xtranspose_kernel<T, false><<<g, 256, 0, s>>>(m, n, static_cast<const T*>(A), lda, static_cast<T*>(B), ldb);
    count_launch();
    return slt_from_cuda(cudaGetLastError());
}

template <typename T>
static int xcopy_tri_t(int upper, int64_t n, const void* S, int64_t lds, void* D, int64_t ldd, cudaStream_t s)
{
    if (n <= 0) return SLT_OK;
    dim3 g(unsigned(ceildiv(n, 256)), unsigned(std::min<int64_t>(n, 65535)));
    xcopy_tri_kernel<T><<<g, 256, 0, s>>>(upper, n, static_cast<const T*>(S), lds, static_cast<T*>(D), ldd);
    count_launch();
    return slt_from_cuda(cudaGetLastError());
}

} // namespace slt

extern "C" int slt_xtranspose(int type, int64_t m, int64_t n, const void* A, int64_t lda, void* B, int64_t ldb,
                              int conj_, slt_stream_t stream)
{
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    switch (type) {
    case 0: return xtranspose_t<float>(m, n, A, lda, B, ldb, 0, s);
    case 1: return xtranspose_t<double>(m, n, A, lda, B, ldb, 0, s);
    case 2: return xtranspose_t<cfloat>(m, n, A, lda, B, ldb, conj_, s);
    case 3: return xtranspose_t<cdouble>(m, n, A, lda, B, ldb, conj_, s);
    default: return SLT_ERR_ARG;
    }
}

extern "C" int slt_xcopy_tri(int type, int upper, int64_t n, const void* S, int64_t lds, void* D, int64_t ldd,
                             slt_stream_t stream)
{
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    switch (type) {
    case 0: return xcopy_tri_t<float>(upper, n, S, lds, D, ldd, s);
    case 1: return xcopy_tri_t<double>(upper, n, S, lds, D, ldd, s);
    case 2: return xcopy_tri_t<cfloat>(upper, n, S, lds, D, ldd, s);
    case 3: return xcopy_tri_t<cdouble>(upper, n, S, lds, D, ldd, s);
    default: return SLT_ERR_ARG;
    }
}
