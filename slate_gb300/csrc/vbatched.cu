// vbatched.cu -- variable-size batched LU and Cholesky solves.
//
// Thousands of independent systems A_i X_i = B_i of uneven size (n_i up to
// 2048, general or SPD) are factored and solved by one persistent launch:
// each CTA takes the next system from a work list sorted by decreasing cost,
// so the largest systems start first and the small ones fill the tail.  A CTA
// works on its system in place in global memory (the working set of one
// system is at most 32 MB and mostly L2-resident): a right-looking blocked
// factorisation with 32-column panels (partial pivoting with the lowest row
// index on ties for LU, lower Cholesky for SPD), a 64x64-tile register-
// blocked update of the trailing matrix, then forward/backward sweeps on up
// to eight right-hand sides at a time, staged in shared memory.
//
// The mixed variant factors an FP32 copy that the same CTA makes from the
// FP64 matrix while it takes the matrix's infinity norm, solves once, and
// then runs one FP64 refinement step -- residual, SLATE's stopping test
// (src/internal/internal_util.hh:121-138), FP32 correction -- per launch of
// vb_refine_kernel; a CUDA graph replays that launch itermax + 1 times and a
// system that has converged leaves each replay at once.
//
// SLATE has no batched solver; the per-system algorithm is its getrf/potrf +
// getrs/potrs (src/getrf.cc, src/potrf.cc), restated for one CTA.

#include "common.cuh"
#include "drivers.h"
#include "prof.h"

#include <algorithm>
#include <vector>

namespace slt {
namespace vb {

constexpr int NT = 256;       // threads per CTA
constexpr int PB = 32;        // panel width
constexpr int TS = 64;        // trailing-update tile
constexpr int TSP = TS + 1;   // padded smem row
constexpr int MAXR = 8;       // right-hand sides per solve pass
constexpr int MAXN = 2048;
constexpr unsigned FULL = 0xffffffffu;

struct Sys {
    double* A;      // FP64 matrix: factored in place (plain) or read only (mixed)
    double* B;      // right-hand sides (read)
    double* X;      // solution (written; may equal B)
    int* ipiv;      // LU: 1-based pivots
    float* lo;      // mixed: FP32 factor, leading dimension n
    int n, nrhs, kind, lda, ldb, ldx, id, pad;
};

__device__ __forceinline__ double tabs(double x) { return fabs(x); }
__device__ __forceinline__ float tabs(float x) { return fabsf(x); }

template <typename T>
__device__ __forceinline__ void argmax_merge(T& v, int& i, T v2, int i2)
{
    if (v2 > v || (v2 == v && i2 < i)) { v = v2; i = i2; }
}

// (max, lowest index on ties) over the CTA; every thread gets the result.
template <typename T>
__device__ void block_argmax(T& v, int& idx, T* sv, int* si)
{
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const T v2 = __shfl_xor_sync(FULL, v, o);
        const int i2 = __shfl_xor_sync(FULL, idx, o);
        argmax_merge(v, idx, v2, i2);
    }
    if ((threadIdx.x & 31) == 0) { sv[threadIdx.x >> 5] = v; si[threadIdx.x >> 5] = idx; }
    __syncthreads();
    v = sv[0];
    idx = si[0];
    #pragma unroll
    for (int k = 1; k < NT / 32; ++k) argmax_merge(v, idx, sv[k], si[k]);
    __syncthreads();
}

__device__ double block_max(double v, double* sv)
{
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(FULL, v, o));
    if ((threadIdx.x & 31) == 0) sv[threadIdx.x >> 5] = v;
    __syncthreads();
    v = sv[0];
    #pragma unroll
    for (int k = 1; k < NT / 32; ++k) v = fmax(v, sv[k]);
    __syncthreads();
    return v;
}

// C (m x nn) -= A (m x kk) * op(B), kk <= PB.  op(B)(q, c) = B[q + c ldb]
// (TRANS = false: the U12 row block) or B[c + q ldb] (TRANS = true: L21^T).
// LOWER: C starts on the diagonal and only its lower triangle is updated.
// Thread (tx, ty) of a 16 x 16 grid owns rows tx + 16 i and columns ty + 16 j
// of each 64 x 64 tile, so that C accesses are coalesced along rows.
template <typename T, bool TRANS, bool LOWER>
__device__ void tile_update(T* C, int ldc, const T* A, int lda, const T* B, int ldb, int m, int nn, int kk,
                            T* sA, T* sB)
{
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int mt = (m + TS - 1) / TS, nt = (nn + TS - 1) / TS;
    for (int t = 0; t < mt * nt; ++t) {
        const int bi = t % mt, bj = t / mt;
        if (LOWER && bi < bj) continue;
        const int r0 = bi * TS, c0 = bj * TS;
        for (int e = threadIdx.x; e < TS * PB; e += NT) {
            const int r = e % TS, q = e / TS;
            sA[q * TSP + r] = (r0 + r < m && q < kk) ? A[(r0 + r) + size_t(q) * lda] : T(0);
        }
        for (int e = threadIdx.x; e < TS * PB; e += NT) {
            int q, c;
            if (TRANS) { c = e % TS; q = e / TS; }
            else { q = e % PB; c = e / PB; }
            T v = T(0);
            if (c0 + c < nn && q < kk) v = TRANS ? B[(c0 + c) + size_t(q) * ldb] : B[q + size_t(c0 + c) * ldb];
            sB[q * TSP + c] = v;
        }
        __syncthreads();
        T acc[4][4];
        #pragma unroll
        for (int i = 0; i < 4; ++i)
            #pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
        for (int q = 0; q < kk; ++q) {
            T a[4], b[4];
            #pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = sA[q * TSP + tx + 16 * i];
            #pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = sB[q * TSP + ty + 16 * j];
            #pragma unroll
            for (int i = 0; i < 4; ++i)
                #pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
        #pragma unroll
        for (int i = 0; i < 4; ++i)
            #pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int r = r0 + tx + 16 * i, c = c0 + ty + 16 * j;
                if (r < m && c < nn && (!LOWER || r >= c)) C[r + size_t(c) * ldc] -= acc[i][j];
            }
        __syncthreads();
    }
}

template <typename T>
struct FactorSmem {
    T sA[PB * TSP];
    T sB[PB * TSP];
    T sL[PB * PB];
    T sv[NT / 32];
    int si[NT / 32];
};

// LU with partial pivoting of the n x n matrix M (leading dimension ld), in
// place; ipiv 1-based.  Returns SLATE's info (first exactly-zero pivot).
template <typename T>
__device__ int lu_factor(T* M, int n, int ld, int* ipiv, FactorSmem<T>& sm)
{
    int info = 0;
    for (int k = 0; k < n; k += PB) {
        const int kb = min(PB, n - k);
        for (int j = k; j < k + kb; ++j) {
            T best = T(-1);
            int bi = n;
            for (int i = j + threadIdx.x; i < n; i += NT) {
                const T v = tabs(M[i + size_t(j) * ld]);
                if (v > best) { best = v; bi = i; }
            }
            block_argmax(best, bi, sm.sv, sm.si);
            const int p = (bi < n) ? bi : j;
            if (threadIdx.x == 0) ipiv[j] = p + 1;
            if (p != j)
                for (int c = threadIdx.x; c < n; c += NT) {
                    const T t = M[j + size_t(c) * ld];
                    M[j + size_t(c) * ld] = M[p + size_t(c) * ld];
                    M[p + size_t(c) * ld] = t;
                }
            __syncthreads();
            const T piv = M[j + size_t(j) * ld];
            if (piv != T(0)) {
                if (tabs(piv) >= Real<T>::safe_min()) {
                    const T r = T(1) / piv;
                    for (int i = j + 1 + threadIdx.x; i < n; i += NT) M[i + size_t(j) * ld] *= r;
                }
                else {
                    for (int i = j + 1 + threadIdx.x; i < n; i += NT) M[i + size_t(j) * ld] /= piv;
                }
            }
            else if (info == 0) {
                info = j + 1;
            }
            __syncthreads();
            for (int i = j + 1 + threadIdx.x; i < n; i += NT) {
                const T l = M[i + size_t(j) * ld];
                for (int c = j + 1; c < k + kb; ++c) M[i + size_t(c) * ld] -= l * M[j + size_t(c) * ld];
            }
            __syncthreads();
        }
        const int rest = n - k - kb;
        if (rest > 0) {
            // U12 = L11^{-1} A12: L11 (unit lower) to smem, one column per thread
            for (int e = threadIdx.x; e < PB * PB; e += NT) {
                const int r = e % PB, c = e / PB;
                sm.sL[e] = (r < kb && c < kb) ? M[(k + r) + size_t(k + c) * ld] : T(0);
            }
            __syncthreads();
            for (int c = k + kb + threadIdx.x; c < n; c += NT) {
                T x[PB];
                #pragma unroll
                for (int q = 0; q < PB; ++q) x[q] = (q < kb) ? M[(k + q) + size_t(c) * ld] : T(0);
                #pragma unroll
                for (int r = 1; r < PB; ++r) {
                    T s = x[r];
                    #pragma unroll
                    for (int q = 0; q < r; ++q) s -= sm.sL[r + q * PB] * x[q];
                    x[r] = s;
                }
                #pragma unroll
                for (int q = 0; q < PB; ++q)
                    if (q < kb) M[(k + q) + size_t(c) * ld] = x[q];
            }
            __syncthreads();
            tile_update<T, false, false>(M + (k + kb) + size_t(k + kb) * ld, ld, M + (k + kb) + size_t(k) * ld, ld,
                                         M + k + size_t(k + kb) * ld, ld, rest, rest, kb, sm.sA, sm.sB);
        }
    }
    return info;
}

// Lower Cholesky of M in place.  Returns SLATE's info (first non-positive
// leading minor); the factorisation stops there.
template <typename T>
__device__ int chol_factor(T* M, int n, int ld, FactorSmem<T>& sm)
{
    for (int k = 0; k < n; k += PB) {
        const int kb = min(PB, n - k);
        for (int j = k; j < k + kb; ++j) {
            const T d = M[j + size_t(j) * ld];
            if (!(d > T(0))) return j + 1;
            const T s = sqrt(d);
            __syncthreads();
            if (threadIdx.x == 0) M[j + size_t(j) * ld] = s;
            const T r = T(1) / s;
            for (int i = j + 1 + threadIdx.x; i < n; i += NT) M[i + size_t(j) * ld] *= r;
            __syncthreads();
            for (int i = j + 1 + threadIdx.x; i < n; i += NT) {
                const T l = M[i + size_t(j) * ld];
                const int ce = min(k + kb - 1, i);
                for (int c = j + 1; c <= ce; ++c) M[i + size_t(c) * ld] -= l * M[c + size_t(j) * ld];
            }
            __syncthreads();
        }
        const int rest = n - k - kb;
        if (rest > 0) {
            tile_update<T, true, true>(M + (k + kb) + size_t(k + kb) * ld, ld, M + (k + kb) + size_t(k) * ld, ld,
                                       M + (k + kb) + size_t(k) * ld, ld, rest, rest, kb, sm.sA, sm.sB);
        }
    }
    return 0;
}

// Y (n x nr, column-major, leading dimension n, shared memory) <- A^{-1} Y
// with the factors in M.
template <typename T>
__device__ void lu_solve(const T* M, int n, int ld, const int* ipiv, T* Y, int nr)
{
    if (threadIdx.x < nr) {
        T* y = Y + threadIdx.x * n;
        for (int j = 0; j < n; ++j) {
            const int p = ipiv[j] - 1;
            if (p > j && p < n) { const T t = y[j]; y[j] = y[p]; y[p] = t; }
        }
    }
    __syncthreads();
    for (int j = 0; j < n - 1; ++j) {
        const int len = n - j - 1;
        for (int e = threadIdx.x; e < len * nr; e += NT) {
            const int i = j + 1 + e % len, q = e / len;
            Y[q * n + i] -= M[i + size_t(j) * ld] * Y[q * n + j];
        }
        __syncthreads();
    }
    for (int j = n - 1; j >= 0; --j) {
        if (threadIdx.x < nr) Y[threadIdx.x * n + j] /= M[j + size_t(j) * ld];
        __syncthreads();
        for (int e = threadIdx.x; e < j * nr; e += NT) {
            const int i = e % j, q = e / j;
            Y[q * n + i] -= M[i + size_t(j) * ld] * Y[q * n + j];
        }
        __syncthreads();
    }
}

template <typename T>
__device__ void chol_solve(const T* M, int n, int ld, T* Y, int nr)
{
    for (int j = 0; j < n; ++j) {
        if (threadIdx.x < nr) Y[threadIdx.x * n + j] /= M[j + size_t(j) * ld];
        __syncthreads();
        const int len = n - j - 1;
        for (int e = threadIdx.x; e < len * nr; e += NT) {
            const int i = j + 1 + e % len, q = e / len;
            Y[q * n + i] -= M[i + size_t(j) * ld] * Y[q * n + j];
        }
        __syncthreads();
    }
    for (int j = n - 1; j >= 0; --j) {
        if (threadIdx.x < nr) Y[threadIdx.x * n + j] /= M[j + size_t(j) * ld];
        __syncthreads();
        for (int e = threadIdx.x; e < j * nr; e += NT) {
            const int i = e % j, q = e / j;
            Y[q * n + i] -= M[j + size_t(i) * ld] * Y[q * n + j];
        }
        __syncthreads();
    }
}

__device__ __forceinline__ int next_system(int* counter, int* s_w)
{
    if (threadIdx.x == 0) *s_w = atomicAdd(counter, 1);
    __syncthreads();
    const int w = *s_w;
    __syncthreads();
    return w;
}

// Plain FP64: factor in place, then X = A^{-1} B (X may be B).
__global__ void __launch_bounds__(NT) vb_plain_kernel(const Sys* __restrict__ sys, int count, int* counter,
                                                      int* info)
{
    extern __shared__ __align__(16) unsigned char vb_smem[];
    __shared__ int s_w;
    auto& fs = *reinterpret_cast<FactorSmem<double>*>(vb_smem);
    double* Y = reinterpret_cast<double*>(vb_smem);
    for (;;) {
        const int w = next_system(counter, &s_w);
        if (w >= count) return;
        const Sys s = sys[w];
        if (s.n <= 0) {
            if (threadIdx.x == 0) info[s.id] = 0;
            continue;
        }
        const int inf = (s.kind == 0) ? lu_factor<double>(s.A, s.n, s.lda, s.ipiv, fs)
                                      : chol_factor<double>(s.A, s.n, s.lda, fs);
        __syncthreads();
        if (threadIdx.x == 0) info[s.id] = inf;
        if (inf != 0) continue;
        for (int c0 = 0; c0 < s.nrhs; c0 += MAXR) {
            const int nr = min(MAXR, s.nrhs - c0);
            for (int e = threadIdx.x; e < s.n * nr; e += NT) {
                const int i = e % s.n, q = e / s.n;
                Y[e] = s.B[i + size_t(c0 + q) * s.ldb];
            }
            __syncthreads();
            if (s.kind == 0) lu_solve<double>(s.A, s.n, s.lda, s.ipiv, Y, nr);
            else chol_solve<double>(s.A, s.n, s.lda, Y, nr);
            for (int e = threadIdx.x; e < s.n * nr; e += NT) {
                const int i = e % s.n, q = e / s.n;
                s.X[i + size_t(c0 + q) * s.ldx] = Y[e];
            }
            __syncthreads();
        }
    }
}

// ||A||_inf (SPD: of the symmetric matrix held in the lower triangle) and
// the FP32 copy lo = float(A) (SPD: lower triangle only).
__device__ double norm_and_cast(const Sys& s, double* sv)
{
    const int n = s.n;
    double mx = 0.0;
    for (int i = threadIdx.x; i < n; i += NT) {
        double acc = 0.0;
        if (s.kind == 0) {
            for (int j = 0; j < n; ++j) {
                const double a = s.A[i + size_t(j) * s.lda];
                s.lo[i + size_t(j) * n] = float(a);
                acc += fabs(a);
            }
        }
        else {
            for (int j = 0; j <= i; ++j) {
                const double a = s.A[i + size_t(j) * s.lda];
                s.lo[i + size_t(j) * n] = float(a);
                acc += fabs(a);
            }
            for (int j = i + 1; j < n; ++j) acc += fabs(s.A[j + size_t(i) * s.lda]);
        }
        mx = (acc > mx || acc != acc) ? acc : mx;
    }
    return block_max(mx, sv);
}

// Mixed, phase 1: norm + FP32 copy, FP32 factorisation, x0 = A_lo^{-1} b.
// iter[id] = 0 (refinement pending) or -3 (low-precision factor failed).
__global__ void __launch_bounds__(NT) vb_mixed_factor_kernel(const Sys* __restrict__ sys, int count, int* counter,
                                                             int* info, int* iter, int* state, double* anorm)
{
    extern __shared__ __align__(16) unsigned char vb_smem[];
    __shared__ int s_w;
    __shared__ double s_red[NT / 32];
    auto& fs = *reinterpret_cast<FactorSmem<float>*>(vb_smem);
    float* Y = reinterpret_cast<float*>(vb_smem);
    for (;;) {
        const int w = next_system(counter, &s_w);
        if (w >= count) return;
        const Sys s = sys[w];
        if (s.n <= 0) {
            if (threadIdx.x == 0) { info[s.id] = 0; iter[s.id] = 0; state[w] = 1; }
            continue;
        }
        const double an = norm_and_cast(s, s_red);
        __syncthreads();
        const int inf = (s.kind == 0) ? lu_factor<float>(s.lo, s.n, s.n, s.ipiv, fs)
                                      : chol_factor<float>(s.lo, s.n, s.n, fs);
        __syncthreads();
        if (threadIdx.x == 0) {
            info[s.id] = inf;
            iter[s.id] = inf ? -3 : 0;
            state[w] = inf ? 2 : 0;
            anorm[w] = an;
        }
        if (inf != 0) continue;
        const int nr = s.nrhs;     // <= MAXR (checked on the host)
        for (int e = threadIdx.x; e < s.n * nr; e += NT) {
            const int i = e % s.n, q = e / s.n;
            Y[e] = float(s.B[i + size_t(q) * s.ldb]);
        }
        __syncthreads();
        if (s.kind == 0) lu_solve<float>(s.lo, s.n, s.n, s.ipiv, Y, nr);
        else chol_solve<float>(s.lo, s.n, s.n, Y, nr);
        for (int e = threadIdx.x; e < s.n * nr; e += NT) {
            const int i = e % s.n, q = e / s.n;
            s.X[i + size_t(q) * s.ldx] = double(Y[e]);
        }
        __syncthreads();
    }
}

// R (n x NR, leading dimension n) = B - A X in FP64, one thread per row;
// SPD: the lower triangle, mirrored.
template <int NR>
__device__ void residual_rows(const Sys& s, double* R)
{
    const int n = s.n;
    for (int i = threadIdx.x; i < n; i += NT) {
        double acc[NR];
        #pragma unroll
        for (int q = 0; q < NR; ++q) acc[q] = s.B[i + size_t(q) * s.ldb];
        const int jl = (s.kind == 0) ? n : i + 1;
        for (int j = 0; j < jl; ++j) {
            const double a = s.A[i + size_t(j) * s.lda];
            #pragma unroll
            for (int q = 0; q < NR; ++q) acc[q] = fma(-a, s.X[j + size_t(q) * s.ldx], acc[q]);
        }
        if (s.kind != 0)
            for (int j = i + 1; j < n; ++j) {
                const double a = s.A[j + size_t(i) * s.lda];
                #pragma unroll
                for (int q = 0; q < NR; ++q) acc[q] = fma(-a, s.X[j + size_t(q) * s.ldx], acc[q]);
            }
        #pragma unroll
        for (int q = 0; q < NR; ++q) R[q * n + i] = acc[q];
    }
}

// Mixed, one refinement step `step` (0 .. itermax) over the active systems:
// R = B - A X in FP64, SLATE's test max|r_q| <= max|x_q| ||A|| eps sqrt(n)
// for every column q; converged -> iter = step; step == itermax -> iter =
// -(itermax + 1) and state 2 (FP64 fallback); else X += A_lo^{-1} R.
__global__ void __launch_bounds__(NT) vb_refine_kernel(const Sys* __restrict__ sys, int count, int* counters,
                                                       int step, int itermax, double tolerance, int* iter,
                                                       int* state, const double* anorm)
{
    extern __shared__ __align__(16) unsigned char vb_smem[];
    __shared__ int s_w;
    __shared__ double s_red[NT / 32];
    __shared__ int s_bad;
    double* R = reinterpret_cast<double*>(vb_smem);
    for (;;) {
        const int w = next_system(counters + step, &s_w);
        if (w >= count) return;
        if (state[w] != 0) continue;
        const Sys s = sys[w];
        const int n = s.n, nr = s.nrhs;
        switch (nr) {
            case 0: break;
            case 1: residual_rows<1>(s, R); break;
            case 2: residual_rows<2>(s, R); break;
            case 3: residual_rows<3>(s, R); break;
            case 4: residual_rows<4>(s, R); break;
            case 5: residual_rows<5>(s, R); break;
            case 6: residual_rows<6>(s, R); break;
            case 7: residual_rows<7>(s, R); break;
            default: residual_rows<8>(s, R); break;
        }
        if (threadIdx.x == 0) s_bad = 0;
        __syncthreads();
        const double tol = tolerance > 0 ? tolerance : 2.220446049250313e-16 * sqrt(double(n));
        const double cte = anorm[w] * tol;
        for (int q = 0; q < nr; ++q) {
            double xm = 0.0, rm = 0.0;
            for (int i = threadIdx.x; i < n; i += NT) {
                const double xv = fabs(s.X[i + size_t(q) * s.ldx]), rv = fabs(R[q * n + i]);
                xm = (xv > xm || xv != xv) ? xv : xm;
                rm = (rv > rm || rv != rv) ? rv : rm;
            }
            xm = block_max(xm, s_red);
            rm = block_max(rm, s_red);
            if (threadIdx.x == 0 && !(rm <= xm * cte)) s_bad = 1;
        }
        __syncthreads();
        const int bad = s_bad;
        if (!bad || step == itermax) {
            if (threadIdx.x == 0) {
                state[w] = bad ? 2 : 1;
                iter[s.id] = bad ? -(itermax + 1) : step;
            }
            __syncthreads();
            continue;
        }
        // correction in FP32.  R (double) -> Y (float) in place, 8 NT elements
        // at a time: the floats of chunk k land on the doubles of chunk k / 2,
        // which were read before the barrier.
        float* Y = reinterpret_cast<float*>(vb_smem);
        for (int base = 0; base < n * nr; base += 8 * NT) {
            double v[8];
            #pragma unroll
            for (int k = 0; k < 8; ++k) {
                const int e = base + threadIdx.x + NT * k;
                v[k] = e < n * nr ? R[e] : 0.0;
            }
            __syncthreads();
            #pragma unroll
            for (int k = 0; k < 8; ++k) {
                const int e = base + threadIdx.x + NT * k;
                if (e < n * nr) Y[e] = float(v[k]);
            }
            __syncthreads();
        }
        if (s.kind == 0) lu_solve<float>(s.lo, n, n, s.ipiv, Y, nr);
        else chol_solve<float>(s.lo, n, n, Y, nr);
        for (int e = threadIdx.x; e < n * nr; e += NT) {
            const int i = e % n, q = e / n;
            s.X[i + size_t(q) * s.ldx] += double(Y[e]);
        }
        __syncthreads();
    }
}

size_t factor_smem(bool dbl) { return dbl ? sizeof(FactorSmem<double>) : sizeof(FactorSmem<float>); }

} // namespace vb
} // namespace slt

using namespace slt;
using namespace slt::vb;

namespace {

struct HostSys {
    std::vector<int> kind, n, nrhs, lda, ldb, ldx;
    std::vector<double*> A, B, X;
    std::vector<int*> ipiv;
};

// Copies a device array of `batch` entries to the host (a null array reads
// as zeros / null pointers; validate() rejects what a system needs).
template <typename P>
int fetch(std::vector<P>& h, const P* d, int64_t batch, cudaStream_t s)
{
    h.assign(size_t(batch), P{});
    if (!d) return SLT_OK;
    SLT_CUDA_TRY(cudaMemcpyAsync(h.data(), d, sizeof(P) * size_t(batch), cudaMemcpyDeviceToHost, s));
    return SLT_OK;
}

// Largest-first work list (cost ~ n^3 for the factorisation + n^2 nrhs).
std::vector<int> work_order(const HostSys& h)
{
    std::vector<int> ord(h.n.size());
    for (size_t i = 0; i < ord.size(); ++i) ord[i] = int(i);
    auto cost = [&](int i) {
        const double n = h.n[i];
        return (h.kind[i] == 0 ? 2.0 / 3.0 : 1.0 / 3.0) * n * n * n + 2.0 * n * n * h.nrhs[i];
    };
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return cost(a) > cost(b); });
    return ord;
}

int validate(const HostSys& h, bool mixed, int* maxn, int* maxr)
{
    *maxn = 0;
    *maxr = 1;
    for (size_t i = 0; i < h.n.size(); ++i) {
        const int n = h.n[i], r = h.nrhs[i];
        if (n < 0 || r < 0 || (h.kind[i] != 0 && h.kind[i] != 1)) return SLT_ERR_ARG;
        if (n > MAXN || (mixed && r > MAXR)) return SLT_ERR_LIMIT;
        if (n == 0) continue;
        if (h.lda[i] < n || !h.A[i]) return SLT_ERR_ARG;
        if (r > 0 && (h.ldb[i] < n || !h.B[i])) return SLT_ERR_ARG;
        if (mixed && r > 0 && (h.ldx[i] < n || !h.X[i])) return SLT_ERR_ARG;
        if (h.kind[i] == 0 && !h.ipiv[i]) return SLT_ERR_ARG;
        *maxn = std::max(*maxn, n);
        *maxr = std::max(*maxr, std::min(r, MAXR));
    }
    return SLT_OK;
}

int grid_for(const void* kernel, size_t smem, int count)
{
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, NT, smem) != cudaSuccess || per < 1) {
        cudaGetLastError();
        per = 1;
    }
    return std::max(1, std::min(count, sms * per));
}

int set_smem(const void* kernel, size_t smem)
{
    return slt_from_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
}

int run_plain(const std::vector<Sys>& list, int* d_info, cudaStream_t s, size_t smem)
{
    if (list.empty()) return SLT_OK;
    const int count = int(list.size());
    DevBuf dsys, ctr;
    TRY(dsys.alloc(sizeof(Sys) * list.size(), s));
    TRY(ctr.alloc(sizeof(int), s));
    SLT_CUDA_TRY(cudaMemcpyAsync(dsys.p, list.data(), sizeof(Sys) * list.size(), cudaMemcpyHostToDevice, s));
    SLT_CUDA_TRY(cudaMemsetAsync(ctr.p, 0, sizeof(int), s));
    const void* k = reinterpret_cast<const void*>(&vb_plain_kernel);
    TRY(set_smem(k, smem));
    vb_plain_kernel<<<grid_for(k, smem, count), NT, smem, s>>>(dsys.as<Sys>(), count, ctr.as<int>(), d_info);
    count_launch();
    SLT_CUDA_TRY(cudaGetLastError());
    SLT_CUDA_TRY(cudaStreamSynchronize(s));   // list and buffers are released on return
    return SLT_OK;
}

int load(HostSys& h, int64_t batch, const int* d_kind, const int* d_n, const int* d_nrhs, double* const* d_A,
         const int* d_lda, int* const* d_ipiv, double* const* d_B, const int* d_ldb, double* const* d_X,
         const int* d_ldx, cudaStream_t s)
{
    TRY(fetch(h.kind, d_kind, batch, s));
    TRY(fetch(h.n, d_n, batch, s));
    TRY(fetch(h.nrhs, d_nrhs, batch, s));
    TRY(fetch(h.lda, d_lda, batch, s));
    TRY(fetch(h.ldb, d_ldb, batch, s));
    TRY(fetch(h.A, const_cast<double**>(d_A), batch, s));
    TRY(fetch(h.B, const_cast<double**>(d_B), batch, s));
    TRY(fetch(h.ipiv, const_cast<int**>(d_ipiv), batch, s));
    if (d_X) {
        TRY(fetch(h.X, const_cast<double**>(d_X), batch, s));
        TRY(fetch(h.ldx, d_ldx, batch, s));
    }
    else {
        h.X = h.B;
        h.ldx = h.ldb;
    }
    SLT_CUDA_TRY(cudaStreamSynchronize(s));
    return SLT_OK;
}

} // namespace

// Plain FP64 variable-size batched solve: system i is general (kind 0: LU
// with partial pivoting, ipiv[i] 1-based) or SPD (kind 1: lower Cholesky);
// A[i] is overwritten by its factors and B[i] by the solution; info[i] is
// SLATE's info.  Every argument array is a device array of `batch` entries.
extern "C" int slt_dsolve_vbatched(int64_t batch, const int* d_kind, const int* d_n, const int* d_nrhs,
                                   double* const* d_A, const int* d_lda, int* const* d_ipiv,
                                   double* const* d_B, const int* d_ldb, int* d_info, slt_stream_t sstream)
{
    cudaStream_t stream = static_cast<cudaStream_t>(sstream);
    if (batch < 0 || batch > (int64_t(1) << 30)) return SLT_ERR_ARG;
    if (batch == 0) return SLT_OK;
    if (!d_info) return SLT_ERR_ARG;
    HostSys h;
    TRY(load(h, batch, d_kind, d_n, d_nrhs, d_A, d_lda, d_ipiv, d_B, d_ldb, nullptr, nullptr, stream));
    int maxn = 0, maxr = 1;
    TRY(validate(h, false, &maxn, &maxr));
    std::vector<Sys> list;
    list.reserve(size_t(batch));
    for (int i : work_order(h))
        list.push_back(Sys{h.A[i], h.B[i], h.B[i], h.ipiv[i], nullptr, h.n[i], h.nrhs[i], h.kind[i],
                           std::max(1, h.lda[i]), std::max(1, h.ldb[i]), std::max(1, h.ldb[i]), i, 0});
    const size_t smem = std::max(factor_smem(true), sizeof(double) * size_t(std::max(1, maxn)) * size_t(maxr));
    return run_plain(list, d_info, stream, smem);
}

// Mixed variable-size batched solve: FP32 factors (LU or Cholesky per
// system), FP64 refinement to SLATE's stopping test, FP64 fallback for the
// systems that fail (their A[i] then holds the FP64 factors).  A[i], B[i] are
// left unchanged otherwise; X[i] receives the solution; iter[i] and info[i]
// follow slate::gesv_mixed (0 .. itermax, -3, -(itermax + 1)).  nrhs[i] <= 8.
extern "C" int slt_dsolve_mixed_vbatched(int64_t batch, const int* d_kind, const int* d_n, const int* d_nrhs,
                                         double* const* d_A, const int* d_lda, int* const* d_ipiv,
                                         double* const* d_B, const int* d_ldb, double* const* d_X,
                                         const int* d_ldx, int* d_iter, int* d_info, int64_t itermax,
                                         double tolerance, int use_fallback, slt_stream_t sstream)
{
    cudaStream_t stream = static_cast<cudaStream_t>(sstream);
    if (batch < 0 || batch > (int64_t(1) << 30) || itermax < 0 || itermax > 1000) return SLT_ERR_ARG;
    if (batch == 0) return SLT_OK;
    if (!d_info || !d_iter || !d_X || !d_ldx) return SLT_ERR_ARG;
    HostSys h;
    TRY(load(h, batch, d_kind, d_n, d_nrhs, d_A, d_lda, d_ipiv, d_B, d_ldb, d_X, d_ldx, stream));
    int maxn = 0, maxr = 1;
    TRY(validate(h, true, &maxn, &maxr));
    const std::vector<int> ord = work_order(h);
    size_t lo_words = 0;
    std::vector<size_t> off(static_cast<size_t>(batch));
    for (int i : ord) {
        off[size_t(i)] = lo_words;
        lo_words += (size_t(h.n[i]) * size_t(h.n[i]) + 3) & ~size_t(3);
    }
    DevBuf lo, dsys, ctr, st, an;
    const int count = int(batch);
    TRY(lo.alloc(sizeof(float) * std::max<size_t>(lo_words, 4), stream));
    std::vector<Sys> list;
    list.reserve(size_t(batch));
    for (int i : ord)
        list.push_back(Sys{h.A[i], h.B[i], h.X[i], h.ipiv[i], lo.as<float>() + off[size_t(i)], h.n[i], h.nrhs[i],
                           h.kind[i], std::max(1, h.lda[i]), std::max(1, h.ldb[i]), std::max(1, h.ldx[i]), i, 0});
    TRY(dsys.alloc(sizeof(Sys) * list.size(), stream));
    TRY(ctr.alloc(sizeof(int) * size_t(itermax + 2), stream));
    TRY(st.alloc(sizeof(int) * size_t(count), stream));
    TRY(an.alloc(sizeof(double) * size_t(count), stream));
    SLT_CUDA_TRY(cudaMemcpyAsync(dsys.p, list.data(), sizeof(Sys) * list.size(), cudaMemcpyHostToDevice, stream));
    SLT_CUDA_TRY(cudaMemsetAsync(ctr.p, 0, sizeof(int) * size_t(itermax + 2), stream));

    TimerSet tm(stream);
    tm.start("vbatched_mixed::factor_lo");
    // phase 1: norm + cast + FP32 factor + first solve
    const size_t smem_f = std::max(factor_smem(false), sizeof(float) * size_t(std::max(1, maxn)) * size_t(maxr));
    const void* kf = reinterpret_cast<const void*>(&vb_mixed_factor_kernel);
    TRY(set_smem(kf, smem_f));
    int* counters = ctr.as<int>();
    vb_mixed_factor_kernel<<<grid_for(kf, smem_f, count), NT, smem_f, stream>>>(
        dsys.as<Sys>(), count, counters + itermax + 1, d_info, d_iter, st.as<int>(), an.as<double>());
    count_launch();
    SLT_CUDA_TRY(cudaGetLastError());

    tm.stop("vbatched_mixed::factor_lo");
    tm.start("vbatched_mixed::refine");
    // phase 2: itermax + 1 refinement steps, captured once as a CUDA graph
    const size_t smem_r = sizeof(double) * size_t(std::max(1, maxn)) * size_t(maxr);
    const void* kr = reinterpret_cast<const void*>(&vb_refine_kernel);
    TRY(set_smem(kr, smem_r));
    const int gr = grid_for(kr, smem_r, count);
    cudaStream_t cs = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    SLT_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    int rc = SLT_OK;
    rc = slt_from_cuda(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    if (rc == SLT_OK) {
        for (int64_t step = 0; step <= itermax; ++step) {
            vb_refine_kernel<<<gr, NT, smem_r, cs>>>(dsys.as<Sys>(), count, counters, int(step), int(itermax),
                                                     tolerance, d_iter, st.as<int>(), an.as<double>());
            count_launch();
        }
        cudaError_t e = cudaStreamEndCapture(cs, &graph);
        if (e != cudaSuccess) rc = slt_from_cuda(e);
    }
    if (rc == SLT_OK) rc = slt_from_cuda(cudaGraphInstantiate(&exec, graph, 0));
    if (rc == SLT_OK) rc = slt_from_cuda(cudaGraphLaunch(exec, stream));
    tm.stop("vbatched_mixed::refine");
    if (rc == SLT_OK) rc = slt_from_cuda(cudaStreamSynchronize(stream));
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(cs);
    TRY(rc);

    // phase 3: FP64 fallback for the systems that failed (state 2)
    std::vector<int> hst(static_cast<size_t>(count));
    SLT_CUDA_TRY(cudaMemcpyAsync(hst.data(), st.p, sizeof(int) * size_t(count), cudaMemcpyDeviceToHost, stream));
    SLT_CUDA_TRY(cudaStreamSynchronize(stream));
    if (!use_fallback) return SLT_OK;
    std::vector<Sys> fb;
    for (int w = 0; w < count; ++w)
        if (hst[size_t(w)] == 2) {
            Sys s = list[size_t(w)];
            s.lo = nullptr;
            fb.push_back(s);
        }
    if (fb.empty()) return SLT_OK;
    tm.start("vbatched_mixed::fallback");
    struct StopAtExit { TimerSet& t; ~StopAtExit() { t.stop("vbatched_mixed::fallback"); } } stop_fb{tm};
    const size_t smem_p = std::max(factor_smem(true), sizeof(double) * size_t(std::max(1, maxn)) * size_t(maxr));
    return run_plain(fb, d_info, stream, smem_p);
}
