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
#include "vbatched_table.h"

#include <algorithm>
#include <cstdlib>
#include <string>
#include <vector>

namespace slt {
namespace vb {

constexpr int NT = 256;       // threads per CTA
constexpr int PBMAX = 32;     // widest panel (the tuning table picks 16 or 32 per system)
constexpr int TS = 64;        // trailing-update tile
constexpr int TSV = TS + 4;   // smem row of a trailing-update operand: 16-byte aligned rows
constexpr int MAXR = 8;       // right-hand sides per solve pass
constexpr int MAXN = 2048;
// In-panel updates: rows processed RG at a time and panel columns CH at a
// time, so that each batch of loads is issued before any of it is used.
template <typename T> struct PanelBatch;
template <> struct PanelBatch<float> { static constexpr int RG = 4, CH = 8; };
template <> struct PanelBatch<double> { static constexpr int RG = 2, CH = 8; };
constexpr int SWP = 4;           // row-swap elements per thread and batch
constexpr unsigned FULL = 0xffffffffu;

struct Sys {
    double* A;      // FP64 matrix: factored in place (plain) or read only (mixed)
    double* B;      // right-hand sides (read)
    double* X;      // solution (written; may equal B)
    int* ipiv;      // LU: 1-based pivots
    float* lo;      // mixed: FP32 factor, leading dimension n
    int n, nrhs, kind, lda, ldb, ldx, id, pb;   // pb: panel width (16 or 32)
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

// v = p[0 .. 3] from shared memory in one (float) or two (double) 16-byte loads;
// p is 16-byte aligned.
__device__ __forceinline__ void lds4(const float* p, float (&v)[4])
{
    const float4 t = *reinterpret_cast<const float4*>(p);
    v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
}
__device__ __forceinline__ void lds4(const double* p, double (&v)[4])
{
    const double2 t0 = *reinterpret_cast<const double2*>(p), t1 = *reinterpret_cast<const double2*>(p + 2);
    v[0] = t0.x; v[1] = t0.y; v[2] = t1.x; v[3] = t1.y;
}

// C (m x nn) -= A (m x kk) * op(B), kk <= PB.  op(B)(q, c) = B[q + c ldb]
// (TRANS = false: the U12 row block) or B[c + q ldb] (TRANS = true: L21^T).
// LOWER: C starts on the diagonal and only its lower triangle is updated.
// Thread (tx, ty) of a 16 x 16 grid owns rows 4 tx .. 4 tx + 3 and columns
// 4 ty .. 4 ty + 3 of each 64 x 64 tile and reads its four A and four B
// values per k-step with one vector load each from shared memory.
// FP32 (PIPE) is software-pipelined: the next tile's operands are fetched
// into registers and this tile's C is loaded before the FMAs, so that no
// global load is waited on right after it is issued.  FP64 is bound by its
// FMA pipe and keeps registers for a second CTA per SM instead: operands are
// fetched just before use, and C is read in one batch after the FMAs.
template <typename T, bool TRANS, bool LOWER, int PB>
__device__ void tile_update(T* C, int ldc, const T* A, int lda, const T* B, int ldb, int m, int nn, int kk,
                            T* sA, T* sB)
{
    constexpr int EPT = TS * PB / NT;      // operand elements per thread and tile
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int mt = (m + TS - 1) / TS, nt = (nn + TS - 1) / TS;
    const int ntiles = mt * nt;
    auto valid = [&](int t) { return !LOWER || (t % mt) >= (t / mt); };
    auto next = [&](int t) {
        do { ++t; } while (t < ntiles && !valid(t));
        return t;
    };
    T ra[EPT], rb[EPT];
    auto fetch = [&](int t) {
        const int r0 = (t % mt) * TS, c0 = (t / mt) * TS;
        #pragma unroll
        for (int u = 0; u < EPT; ++u) {
            const int e = threadIdx.x + u * NT;
            const int r = e % TS, q = e / TS;
            ra[u] = (r0 + r < m && q < kk) ? A[(r0 + r) + size_t(q) * lda] : T(0);
            int qb, c;
            if (TRANS) { c = e % TS; qb = e / TS; }
            else { qb = e % PB; c = e / PB; }
            rb[u] = (c0 + c < nn && qb < kk) ? (TRANS ? B[(c0 + c) + size_t(qb) * ldb] : B[qb + size_t(c0 + c) * ldb])
                                             : T(0);
        }
    };
    constexpr bool PIPE = sizeof(T) == 4;
    int t = 0;                               // tile (0, 0) is always valid
    if (PIPE && ntiles > 0) fetch(t);
    while (t < ntiles) {
        if (!PIPE) fetch(t);
        #pragma unroll
        for (int u = 0; u < EPT; ++u) {
            const int e = threadIdx.x + u * NT;
            sA[(e / TS) * TSV + e % TS] = ra[u];
            if (TRANS) sB[(e / TS) * TSV + e % TS] = rb[u];
            else sB[(e % PB) * TSV + e / PB] = rb[u];
        }
        __syncthreads();
        const int r0 = (t % mt) * TS, c0 = (t / mt) * TS;
        T cv[4][4];
        auto load_c = [&]() {
            #pragma unroll
            for (int i = 0; i < 4; ++i)
                #pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int r = r0 + 4 * tx + i, c = c0 + 4 * ty + j;
                    cv[i][j] = (r < m && c < nn && (!LOWER || r >= c)) ? C[r + size_t(c) * ldc] : T(0);
                }
        };
        if (PIPE) load_c();
        const int tn = next(t);
        if (PIPE && tn < ntiles) fetch(tn);
        T acc[4][4];
        #pragma unroll
        for (int i = 0; i < 4; ++i)
            #pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
        for (int q = 0; q < kk; ++q) {
            T a[4], b[4];
            lds4(sA + q * TSV + 4 * tx, a);
            lds4(sB + q * TSV + 4 * ty, b);
            #pragma unroll
            for (int i = 0; i < 4; ++i)
                #pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
        if (!PIPE) load_c();
        #pragma unroll
        for (int i = 0; i < 4; ++i)
            #pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int r = r0 + 4 * tx + i, c = c0 + 4 * ty + j;
                if (r < m && c < nn && (!LOWER || r >= c)) C[r + size_t(c) * ldc] = cv[i][j] - acc[i][j];
            }
        __syncthreads();
        t = tn;
    }
}

template <typename T>
struct alignas(16) FactorSmem {
    T sA[PBMAX * TSV];
    T sB[PBMAX * TSV];
    T sL[PBMAX * PBMAX];
    T sU[PBMAX];          // LU: panel part of the pivot row; Cholesky: panel part of column j
    T sv[NT / 32];
    int si[NT / 32];
};

// Column-by-column LU of the panel rows k .. n - 1, columns k .. k + kb - 1,
// held at Pn (element (i, c) of the panel at Pn[i + c pld]: in place in M, or
// a shared-memory copy).  Row interchanges reach the columns outside the
// panel in M, each column swapped by the one thread that owns it, so that they
// need no barrier; inside the panel threads 0 .. kb - 1 swap and stage the new
// pivot row in sm.sU.  Rows are updated RG at a time from batched loads, and
// the update of column j + 1 feeds the next pivot search.  Returns info.
template <typename T>
__device__ int lu_panel(T* M, int n, int ld, int k, int kb, int* ipiv, int info, FactorSmem<T>& sm, T* Pn, int pld)
{
    const int m = n - k;
    T best = T(-1);
    int bi = n;
    for (int ii = threadIdx.x; ii < m; ii += NT) {
        const T v = tabs(Pn[ii]);
        if (v > best) { best = v; bi = k + ii; }
    }
    constexpr int RG = PanelBatch<T>::RG, CH = PanelBatch<T>::CH;
    for (int jj = 0; jj < kb; ++jj) {
        const int j = k + jj;
        block_argmax(best, bi, sm.sv, sm.si);
        const int p = (bi < n) ? bi : j, pp = p - k;
        if (threadIdx.x == 0) ipiv[j] = p + 1;
        if (p != j)
            for (int t0 = threadIdx.x; t0 < n - kb; t0 += SWP * NT) {
                T av[SWP], bv[SWP];
                #pragma unroll
                for (int u = 0; u < SWP; ++u) {
                    const int t = min(t0 + u * NT, n - kb - 1);
                    const int c = t < k ? t : t + kb;
                    av[u] = M[j + size_t(c) * ld];
                    bv[u] = M[p + size_t(c) * ld];
                }
                #pragma unroll
                for (int u = 0; u < SWP; ++u) {
                    const int t = t0 + u * NT;
                    if (t < n - kb) {
                        const int c = t < k ? t : t + kb;
                        M[j + size_t(c) * ld] = bv[u];
                        M[p + size_t(c) * ld] = av[u];
                    }
                }
            }
        if (threadIdx.x < kb) {
            T* col = Pn + size_t(threadIdx.x) * pld;
            const T a = col[jj], b = col[pp];
            if (p != j) { col[jj] = b; col[pp] = a; }
            sm.sU[threadIdx.x] = b;
        }
        __syncthreads();
        const T piv = sm.sU[jj];
        if (piv == T(0) && info == 0) info = j + 1;
        const bool recip = tabs(piv) >= Real<T>::safe_min();
        const T r = recip ? T(1) / piv : T(0);
        // rows below: l = a_ij / piv, then a_ic -= l u_jc for the panel's columns c > j
        best = T(-1);
        bi = n;
        for (int i0 = jj + 1 + threadIdx.x; i0 < m; i0 += RG * NT) {
            T seg[RG][CH];
            T l[RG];
            #pragma unroll
            for (int g = 0; g < RG; ++g) {
                const int ii = min(i0 + g * NT, m - 1);
                #pragma unroll
                for (int q = 0; q < CH; ++q) seg[g][q] = Pn[ii + size_t(min(jj + q, kb - 1)) * pld];
            }
            #pragma unroll
            for (int g = 0; g < RG; ++g) {
                const int ii = i0 + g * NT;
                if (ii >= m) continue;
                l[g] = piv == T(0) ? seg[g][0] : (recip ? seg[g][0] * r : seg[g][0] / piv);
                Pn[ii + size_t(jj) * pld] = l[g];
                #pragma unroll
                for (int q = 1; q < CH; ++q)
                    if (jj + q < kb) {
                        seg[g][q] -= l[g] * sm.sU[jj + q];
                        Pn[ii + size_t(jj + q) * pld] = seg[g][q];
                    }
                if (jj + 1 < kb) {
                    const T v = tabs(seg[g][1]);
                    if (v > best) { best = v; bi = k + ii; }
                }
            }
            for (int c0 = jj + CH; c0 < kb; c0 += CH) {
                #pragma unroll
                for (int g = 0; g < RG; ++g) {
                    const int ii = min(i0 + g * NT, m - 1);
                    #pragma unroll
                    for (int q = 0; q < CH; ++q) seg[g][q] = Pn[ii + size_t(min(c0 + q, kb - 1)) * pld];
                }
                #pragma unroll
                for (int g = 0; g < RG; ++g) {
                    const int ii = i0 + g * NT;
                    #pragma unroll
                    for (int q = 0; q < CH; ++q)
                        if (ii < m && c0 + q < kb) {
                            seg[g][q] -= l[g] * sm.sU[c0 + q];
                            Pn[ii + size_t(c0 + q) * pld] = seg[g][q];
                        }
                }
            }
        }
        // the next block_argmax's barrier orders these updates before the
        // next interchange and before sU is rewritten
    }
    __syncthreads();
    return info;
}

// LU with partial pivoting of the n x n matrix M (leading dimension ld), in
// place; ipiv 1-based.  Returns SLATE's info (first exactly-zero pivot).
template <typename T, int PB>
__device__ int lu_factor(T* M, int n, int ld, int* ipiv, FactorSmem<T>& sm)
{
    int info = 0;
    for (int k = 0; k < n; k += PB) {
        const int kb = min(PB, n - k);
        info = lu_panel<T>(M, n, ld, k, kb, ipiv, info, sm, M + k + size_t(k) * ld, ld);
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
            tile_update<T, false, false, PB>(M + (k + kb) + size_t(k + kb) * ld, ld, M + (k + kb) + size_t(k) * ld, ld,
                                             M + k + size_t(k + kb) * ld, ld, rest, rest, kb, sm.sA, sm.sB);
        }
    }
    return info;
}

// Column-by-column Cholesky of the panel rows k .. n - 1, columns k .. k +
// kb - 1 at Pn (as for lu_panel); column j's panel rows are staged in sm.sU
// before it is scaled.  Returns 0 or the failing leading minor.
template <typename T>
__device__ int chol_panel(int n, int k, int kb, FactorSmem<T>& sm, T* Pn, int pld)
{
    const int m = n - k;
    constexpr int RG = PanelBatch<T>::RG, CH = PanelBatch<T>::CH;
    for (int jj = 0; jj < kb; ++jj) {
        if (threadIdx.x < kb - jj) sm.sU[threadIdx.x] = Pn[(jj + threadIdx.x) + size_t(jj) * pld];
        __syncthreads();
        const T d = sm.sU[0];
        if (!(d > T(0))) return k + jj + 1;
        const T sd = sqrt(d);
        const T r = T(1) / sd;
        if (threadIdx.x == 0) Pn[jj + size_t(jj) * pld] = sd;
        // rows below: l = a_ij / sqrt(d), then a_ic -= l l_cj for the panel's
        // columns j < c <= min(i, k + kb - 1)
        for (int i0 = jj + 1 + threadIdx.x; i0 < m; i0 += RG * NT) {
            T seg[RG][CH];
            T l[RG];
            #pragma unroll
            for (int g = 0; g < RG; ++g) {
                const int ii = min(i0 + g * NT, m - 1);
                #pragma unroll
                for (int q = 0; q < CH; ++q) seg[g][q] = Pn[ii + size_t(min(jj + q, kb - 1)) * pld];
            }
            #pragma unroll
            for (int g = 0; g < RG; ++g) {
                const int ii = i0 + g * NT;
                if (ii >= m) continue;
                const int ce = min(kb - 1, ii);      // last panel column of this row
                l[g] = seg[g][0] * r;
                Pn[ii + size_t(jj) * pld] = l[g];
                #pragma unroll
                for (int q = 1; q < CH; ++q)
                    if (jj + q <= ce) {
                        seg[g][q] -= l[g] * (sm.sU[q] * r);
                        Pn[ii + size_t(jj + q) * pld] = seg[g][q];
                    }
            }
            for (int c0 = jj + CH; c0 < kb; c0 += CH) {
                #pragma unroll
                for (int g = 0; g < RG; ++g) {
                    const int ii = min(i0 + g * NT, m - 1);
                    #pragma unroll
                    for (int q = 0; q < CH; ++q) seg[g][q] = Pn[ii + size_t(min(c0 + q, kb - 1)) * pld];
                }
                #pragma unroll
                for (int g = 0; g < RG; ++g) {
                    const int ii = i0 + g * NT;
                    const int ce = min(kb - 1, ii);
                    #pragma unroll
                    for (int q = 0; q < CH; ++q)
                        if (ii < m && c0 + q <= ce) {
                            seg[g][q] -= l[g] * (sm.sU[c0 + q - jj] * r);
                            Pn[ii + size_t(c0 + q) * pld] = seg[g][q];
                        }
                }
            }
        }
        __syncthreads();
    }
    return 0;
}

// Lower Cholesky of M in place.  Returns SLATE's info (first non-positive
// leading minor); the factorisation stops there.
template <typename T, int PB>
__device__ int chol_factor(T* M, int n, int ld, FactorSmem<T>& sm)
{
    for (int k = 0; k < n; k += PB) {
        const int kb = min(PB, n - k);
        const int f = chol_panel<T>(n, k, kb, sm, M + k + size_t(k) * ld, ld);
        if (f) return f;
        const int rest = n - k - kb;
        if (rest > 0)
            tile_update<T, true, true, PB>(M + (k + kb) + size_t(k + kb) * ld, ld, M + (k + kb) + size_t(k) * ld, ld,
                                           M + (k + kb) + size_t(k) * ld, ld, rest, rest, kb, sm.sA, sm.sB);
    }
    return 0;
}

// Factor with the panel width the tuning table chose for this system.
template <typename T>
__device__ int factor_sys(int kind, int pb, T* M, int n, int ld, int* ipiv, FactorSmem<T>& sm)
{
    if (kind == 0) return pb == 16 ? lu_factor<T, 16>(M, n, ld, ipiv, sm) : lu_factor<T, 32>(M, n, ld, ipiv, sm);
    return pb == 16 ? chol_factor<T, 16>(M, n, ld, sm) : chol_factor<T, 32>(M, n, ld, sm);
}

// Blocked triangular solves on Y (n x nr, column-major, leading dimension
// n, shared memory; nr <= MAXR).  Per block of SB rows, warp q solves the
// diagonal block for right-hand side q (lane r owns row r; shuffles, no
// barrier) from a shared tile, then every thread applies the block to the
// rows not yet solved, one row per thread, while the next diagonal block is
// staged: two barriers per block.
constexpr int SB = 32;
constexpr int SBP = SB + 1;
constexpr size_t kTileBytes = sizeof(double) * SB * SBP;   // solve tile at the start of shared memory

// op(T)(r, c) of the triangle stored in M: TRANS reads M(c, r).
template <typename T, bool TRANS>
__device__ __forceinline__ T tri_at(const T* M, int ld, int r, int c)
{
    return TRANS ? M[c + size_t(r) * ld] : M[r + size_t(c) * ld];
}

// tile(r, c) = op(M)(jb + r, jb + c) on the LOWER or upper triangle of the
// bs x bs diagonal block, zero elsewhere; reads are coalesced along memory.
template <typename T, bool TRANS, bool LOWER>
__device__ __forceinline__ void stage_tile(const T* M, int ld, int jb, int bs, T* tile)
{
    // element (lane, warp + 8u) of the tile in memory order: all loads first
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    constexpr int U = SB * SB / NT;
    T v[U];
    #pragma unroll
    for (int u = 0; u < U; ++u) {
        const int slow = w + (NT / 32) * u;
        const int r = TRANS ? slow : lane, c = TRANS ? lane : slow;
        const bool in = r < bs && c < bs && (LOWER ? c <= r : c >= r);
        v[u] = in ? tri_at<T, TRANS>(M, ld, jb + r, jb + c) : T(0);
    }
    #pragma unroll
    for (int u = 0; u < U; ++u) {
        const int slow = w + (NT / 32) * u;
        const int r = TRANS ? slow : lane, c = TRANS ? lane : slow;
        tile[r * SBP + c] = v[u];
    }
}

// Y rows [i0, i1) -= op(M)(rows, jb .. jb + bs) * Y(jb .. jb + bs, :)
template <typename T, bool TRANS>
__device__ __forceinline__ void block_gemv(const T* M, int ld, T* Y, int n, int nr, int i0, int i1, int jb, int bs)
{
    for (int i = i0 + threadIdx.x; i < i1; i += NT) {
        T acc[MAXR];
        #pragma unroll
        for (int q = 0; q < MAXR; ++q) acc[q] = T(0);
        for (int c = 0; c < bs; ++c) {
            const T m = tri_at<T, TRANS>(M, ld, i, jb + c);
            #pragma unroll
            for (int q = 0; q < MAXR; ++q)
                if (q < nr) acc[q] = fma(m, Y[q * n + jb + c], acc[q]);
        }
        #pragma unroll
        for (int q = 0; q < MAXR; ++q)
            if (q < nr) Y[q * n + i] -= acc[q];
    }
}

// Y <- L^{-1} Y, L = lower triangle of M; UNIT: unit diagonal.
template <typename T, bool UNIT>
__device__ void solve_lower(const T* M, int n, int ld, T* Y, int nr, T* tile)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    stage_tile<T, false, true>(M, ld, 0, min(SB, n), tile);
    __syncthreads();
    for (int jb = 0; jb < n; jb += SB) {
        const int bs = min(SB, n - jb);
        if (warp < nr) {
            T y = lane < bs ? Y[warp * n + jb + lane] : T(0);
            #pragma unroll
            for (int c = 0; c < SB; ++c) {
                if (!UNIT && lane == c && c < bs) y /= tile[lane * SBP + c];
                const T yc = __shfl_sync(FULL, y, c);
                if (lane > c) y -= tile[lane * SBP + c] * yc;
            }
            if (lane < bs) Y[warp * n + jb + lane] = y;
        }
        __syncthreads();
        block_gemv<T, false>(M, ld, Y, n, nr, jb + bs, n, jb, bs);
        if (jb + SB < n) stage_tile<T, false, true>(M, ld, jb + SB, min(SB, n - jb - SB), tile);
        __syncthreads();
    }
}

// Y <- U^{-1} Y with non-unit U = upper triangle of M (TRANS = false) or
// U = L^T for the lower triangle L of M (TRANS = true).
template <typename T, bool TRANS>
__device__ void solve_upper(const T* M, int n, int ld, T* Y, int nr, T* tile)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int jlast = ((n - 1) / SB) * SB;
    stage_tile<T, TRANS, false>(M, ld, jlast, n - jlast, tile);
    __syncthreads();
    for (int jb = jlast; jb >= 0; jb -= SB) {
        const int bs = min(SB, n - jb);
        if (warp < nr) {
            T y = lane < bs ? Y[warp * n + jb + lane] : T(0);
            #pragma unroll
            for (int c = SB - 1; c >= 0; --c) {
                if (lane == c && c < bs) y /= tile[lane * SBP + c];
                const T yc = __shfl_sync(FULL, y, c);
                if (lane < c) y -= tile[lane * SBP + c] * yc;
            }
            if (lane < bs) Y[warp * n + jb + lane] = y;
        }
        __syncthreads();
        block_gemv<T, TRANS>(M, ld, Y, n, nr, 0, jb, jb, bs);
        if (jb > 0) stage_tile<T, TRANS, false>(M, ld, jb - SB, SB, tile);
        __syncthreads();
    }
}

// Y <- A^{-1} Y with the LU factors in M (row interchanges ipiv, 1-based).
template <typename T>
__device__ void lu_solve(const T* M, int n, int ld, const int* ipiv, T* Y, int nr, T* tile)
{
    // row interchanges staged in the tile area (n <= MAXN ints fit), then
    // applied in order by one thread per right-hand side
    int* sp = reinterpret_cast<int*>(tile);
    staged_copy<MAXN / NT, NT>(n, [&](int j) { return ipiv[j]; }, [&](int j, int v) { sp[j] = v; });
    __syncthreads();
    if (threadIdx.x < nr) {
        T* y = Y + threadIdx.x * n;
        for (int j = 0; j < n; ++j) {
            const int p = sp[j] - 1;
            if (p > j && p < n) { const T t = y[j]; y[j] = y[p]; y[p] = t; }
        }
    }
    __syncthreads();
    solve_lower<T, true>(M, n, ld, Y, nr, tile);
    solve_upper<T, false>(M, n, ld, Y, nr, tile);
}

// Y <- A^{-1} Y with the lower Cholesky factor in M.
template <typename T>
__device__ void chol_solve(const T* M, int n, int ld, T* Y, int nr, T* tile)
{
    solve_lower<T, false>(M, n, ld, Y, nr, tile);
    solve_upper<T, true>(M, n, ld, Y, nr, tile);
}

__device__ __forceinline__ int next_system(int* counter, int* s_w)
{
    if (threadIdx.x == 0) *s_w = atomicAdd(counter, 1);
    __syncthreads();
    const int w = *s_w;
    __syncthreads();
    return w;
}

// Plain FP64: factor in place, then X = A^{-1} B (X may be B).  s.lo non-null: factor a copy placed
// there (as doubles) and leave A untouched.  iter non-null: iter[id] = 0
// (the mixed API's systems assigned to the FP64 tier).
__global__ void __launch_bounds__(NT, 2) vb_plain_kernel(const Sys* __restrict__ sys, int count, int* counter,
                                                      int* info, int* iter)
{
    extern __shared__ __align__(16) unsigned char vb_smem[];
    __shared__ int s_w;
    auto& fs = *reinterpret_cast<FactorSmem<double>*>(vb_smem);
    double* tile = reinterpret_cast<double*>(vb_smem);
    double* Y = reinterpret_cast<double*>(vb_smem + kTileBytes);
    for (;;) {
        const int w = next_system(counter, &s_w);
        if (w >= count) return;
        Sys s = sys[w];
        if (threadIdx.x == 0 && iter) iter[s.id] = 0;
        if (s.n <= 0) {
            if (threadIdx.x == 0) info[s.id] = 0;
            continue;
        }
        if (s.lo) {
            double* Wk = reinterpret_cast<double*>(s.lo);
            for (int64_t e = threadIdx.x; e < int64_t(s.n) * s.n; e += NT)
                Wk[e] = s.A[(e % s.n) + size_t(e / s.n) * s.lda];
            __syncthreads();
            s.A = Wk;
            s.lda = s.n;
        }
        const int inf = factor_sys<double>(s.kind, s.pb, s.A, s.n, s.lda, s.ipiv, fs);
        __syncthreads();
        if (threadIdx.x == 0) info[s.id] = inf;
        if (inf != 0) continue;
        for (int c0 = 0; c0 < s.nrhs; c0 += MAXR) {
            const int nr = min(MAXR, s.nrhs - c0);
            staged_copy<4, NT>(s.n * nr, [&](int e) { return s.B[e % s.n + size_t(c0 + e / s.n) * s.ldb]; },
                            [&](int e, double v) { Y[e] = v; });
            __syncthreads();
            if (s.kind == 0) lu_solve<double>(s.A, s.n, s.lda, s.ipiv, Y, nr, tile);
            else chol_solve<double>(s.A, s.n, s.lda, Y, nr, tile);
            for (int e = threadIdx.x; e < s.n * nr; e += NT)
                s.X[e % s.n + size_t(c0 + e / s.n) * s.ldx] = Y[e];
            __syncthreads();
        }
    }
}

// ||A||_inf (SPD: of the symmetric matrix held in the lower triangle) and
// the FP32 copy lo = float(A) (SPD: lower triangle only).
__device__ double norm_and_cast(const Sys& s, double* sv)
{
    constexpr int NB = 8;       // elements loaded per batch and thread
    const int n = s.n;
    double mx = 0.0;
    for (int i = threadIdx.x; i < n; i += NT) {
        double acc = 0.0;
        const int jl = s.kind == 0 ? n : i + 1;     // SPD: the lower triangle is cast
        for (int j0 = 0; j0 < jl; j0 += NB) {
            double a[NB];
            #pragma unroll
            for (int u = 0; u < NB; ++u)
                if (j0 + u < jl) a[u] = s.A[i + size_t(j0 + u) * s.lda];
            #pragma unroll
            for (int u = 0; u < NB; ++u)
                if (j0 + u < jl) {
                    s.lo[i + size_t(j0 + u) * n] = float(a[u]);
                    acc += fabs(a[u]);
                }
        }
        if (s.kind != 0)
            for (int j = i + 1; j < n; ++j) acc += fabs(s.A[j + size_t(i) * s.lda]);
        mx = (acc > mx || acc != acc) ? acc : mx;
    }
    return block_max(mx, sv);
}

// Mixed, phase 1: norm + FP32 copy, FP32 factorisation, x0 = A_lo^{-1} b.
// iter[id] = 0 (refinement pending) or -3 (low-precision factor failed).
__global__ void __launch_bounds__(NT, 2) vb_mixed_factor_kernel(const Sys* __restrict__ sys, int count, int* counter,
                                                             int* info, int* iter, int* state, double* anorm)
{
    extern __shared__ __align__(16) unsigned char vb_smem[];
    __shared__ int s_w;
    __shared__ double s_red[NT / 32];
    auto& fs = *reinterpret_cast<FactorSmem<float>*>(vb_smem);
    float* tile = reinterpret_cast<float*>(vb_smem);
    float* Y = reinterpret_cast<float*>(vb_smem + kTileBytes);
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
        const int inf = factor_sys<float>(s.kind, s.pb, s.lo, s.n, s.n, s.ipiv, fs);
        __syncthreads();
        if (threadIdx.x == 0) {
            info[s.id] = inf;
            iter[s.id] = inf ? -3 : 0;
            state[w] = inf ? 2 : 0;
            anorm[w] = an;
        }
        if (inf != 0) continue;
        const int nr = s.nrhs;     // <= MAXR (checked on the host)
        staged_copy<4, NT>(s.n * nr, [&](int e) { return float(s.B[e % s.n + size_t(e / s.n) * s.ldb]); },
                        [&](int e, float v) { Y[e] = v; });
        __syncthreads();
        if (s.kind == 0) lu_solve<float>(s.lo, s.n, s.n, s.ipiv, Y, nr, tile);
        else chol_solve<float>(s.lo, s.n, s.n, Y, nr, tile);
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
    float* tile = reinterpret_cast<float*>(vb_smem);
    double* R = reinterpret_cast<double*>(vb_smem + kTileBytes);
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
        __syncthreads();
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
        float* Y = reinterpret_cast<float*>(vb_smem + kTileBytes);
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
        if (s.kind == 0) lu_solve<float>(s.lo, n, n, s.ipiv, Y, nr, tile);
        else chol_solve<float>(s.lo, n, n, Y, nr, tile);
        staged_copy<4, NT>(n * nr, [&](int e) { return s.X[e % n + size_t(e / n) * s.ldx] + double(Y[e]); },
                        [&](int e, double v) { s.X[e % n + size_t(e / n) * s.ldx] = v; });
        __syncthreads();
    }
}

// Dynamic shared memory of the factor + solve kernels: the factorisation's
// staging, or the solve tile followed by the n x nr right-hand sides.
size_t solve_smem(bool dbl, int maxn, int maxr)
{
    const size_t es = dbl ? sizeof(double) : sizeof(float);
    const size_t f = dbl ? sizeof(FactorSmem<double>) : sizeof(FactorSmem<float>);
    const size_t y = kTileBytes + es * size_t(std::max(1, maxn)) * size_t(maxr);
    return std::max(f, y);
}

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

// The tuning table's entry for a system of size n, with overrides used by
// the tuner itself: SLT_VBATCHED_PB = 16 | 32, SLT_VBATCHED_TIER = fp32 | fp64.
VbTune tune_for(int n)
{
    VbTune t = kVbTable[sizeof(kVbTable) / sizeof(kVbTable[0]) - 1];
    for (const VbTune& e : kVbTable)
        if (n <= e.max_n) { t = e; break; }
    if (const char* v = std::getenv("SLT_VBATCHED_PB")) {
        const int pb = std::atoi(v);
        if (pb == 16 || pb == 32) { t.pb_fp64 = pb; t.pb_mixed = pb; }
    }
    if (const char* v = std::getenv("SLT_VBATCHED_TIER")) {
        if (std::string(v) == "fp64") t.mixed_tier = 0;
        if (std::string(v) == "fp32") t.mixed_tier = 1;
    }
    return t;
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

// Launches vb_plain_kernel over `list`; dsys and ctr receive the device
// copies and must outlive the launch.
int launch_plain(const std::vector<Sys>& list, int* d_info, int* d_iter, cudaStream_t s, size_t smem,
                 DevBuf& dsys, DevBuf& ctr)
{
    if (list.empty()) return SLT_OK;
    const int count = int(list.size());
    TRY(dsys.alloc(sizeof(Sys) * list.size(), s));
    TRY(ctr.alloc(sizeof(int), s));
    SLT_CUDA_TRY(cudaMemcpyAsync(dsys.p, list.data(), sizeof(Sys) * list.size(), cudaMemcpyHostToDevice, s));
    SLT_CUDA_TRY(cudaMemsetAsync(ctr.p, 0, sizeof(int), s));
    const void* k = reinterpret_cast<const void*>(&vb_plain_kernel);
    TRY(set_smem(k, smem));
    vb_plain_kernel<<<grid_for(k, smem, count), NT, smem, s>>>(dsys.as<Sys>(), count, ctr.as<int>(), d_info,
                                                              d_iter);
    count_launch();
    SLT_CUDA_TRY(cudaGetLastError());
    return SLT_OK;
}

int run_plain(const std::vector<Sys>& list, int* d_info, cudaStream_t s, size_t smem)
{
    DevBuf dsys, ctr;
    TRY(launch_plain(list, d_info, nullptr, s, smem, dsys, ctr));
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
                           std::max(1, h.lda[i]), std::max(1, h.ldb[i]), std::max(1, h.ldb[i]), i,
                           tune_for(h.n[i]).pb_fp64});
    const size_t smem = solve_smem(true, maxn, maxr);
    return run_plain(list, d_info, stream, smem);
}

// Mixed variable-size batched solve: FP32 factors (LU or Cholesky per
// system), FP64 refinement to SLATE's stopping test, FP64 fallback for the
// systems that fail (their A[i] then holds the FP64 factors).  A[i], B[i] are
// left unchanged otherwise; X[i] receives the solution; iter[i] and info[i]
// follow slate::gesv_mixed (0 .. itermax, -3, -(itermax + 1)).  nrhs[i] <= 8.
// Sizes whose tuning-table tier is FP64 skip the FP32 attempt: a copy of A[i]
// is factored in FP64 and solved into X[i] (iter[i] = 0; A[i], B[i] kept).
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
    // Per system, the table's tier: FP32 factor + FP64 refinement (n^2 floats
    // of workspace for the factor) or a direct FP64 solve of a copy (n^2
    // doubles), whichever measured faster for its size.
    size_t lo_words = 0;
    std::vector<size_t> off(static_cast<size_t>(batch));
    std::vector<VbTune> tune(static_cast<size_t>(batch));
    for (int i : ord) {
        tune[size_t(i)] = tune_for(h.n[i]);
        off[size_t(i)] = lo_words;
        const size_t words = size_t(h.n[i]) * size_t(h.n[i]) * (tune[size_t(i)].mixed_tier ? 1 : 2);
        lo_words += (words + 3) & ~size_t(3);
    }
    DevBuf lo, dsys, ctr, st, an, dsys64, ctr64;
    TRY(lo.alloc(sizeof(float) * std::max<size_t>(lo_words, 4), stream));
    std::vector<Sys> list, direct;
    list.reserve(size_t(batch));
    for (int i : ord) {
        const VbTune& t = tune[size_t(i)];
        const Sys sy{h.A[i], h.B[i], h.X[i], h.ipiv[i], lo.as<float>() + off[size_t(i)], h.n[i], h.nrhs[i],
                     h.kind[i], std::max(1, h.lda[i]), std::max(1, h.ldb[i]), std::max(1, h.ldx[i]), i,
                     t.mixed_tier ? t.pb_mixed : t.pb_fp64};
        (t.mixed_tier ? list : direct).push_back(sy);
    }
    const int count = int(list.size());

    TimerSet tm(stream);
    if (!direct.empty()) {
        tm.start("vbatched_mixed::direct_fp64");
        const size_t smem_p = solve_smem(true, maxn, maxr);
        TRY(launch_plain(direct, d_info, d_iter, stream, smem_p, dsys64, ctr64));
        tm.stop("vbatched_mixed::direct_fp64");
    }
    if (count == 0) {
        SLT_CUDA_TRY(cudaStreamSynchronize(stream));
        return SLT_OK;
    }
    TRY(dsys.alloc(sizeof(Sys) * list.size(), stream));
    TRY(ctr.alloc(sizeof(int) * size_t(itermax + 2), stream));
    TRY(st.alloc(sizeof(int) * size_t(count), stream));
    TRY(an.alloc(sizeof(double) * size_t(count), stream));
    SLT_CUDA_TRY(cudaMemcpyAsync(dsys.p, list.data(), sizeof(Sys) * list.size(), cudaMemcpyHostToDevice, stream));
    SLT_CUDA_TRY(cudaMemsetAsync(ctr.p, 0, sizeof(int) * size_t(itermax + 2), stream));

    tm.start("vbatched_mixed::factor_lo");
    // phase 1: norm + cast + FP32 factor + first solve
    const size_t smem_f = solve_smem(false, maxn, maxr);
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
    const size_t smem_r = kTileBytes + sizeof(double) * size_t(std::max(1, maxn)) * size_t(maxr);
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
            s.pb = tune[size_t(s.id)].pb_fp64;
            fb.push_back(s);
        }
    if (fb.empty()) return SLT_OK;
    tm.start("vbatched_mixed::fallback");
    struct StopAtExit { TimerSet& t; ~StopAtExit() { t.stop("vbatched_mixed::fallback"); } } stop_fb{tm};
    const size_t smem_p = solve_smem(true, maxn, maxr);
    return run_plain(fb, d_info, stream, smem_p);
}
