// chol_panel.cu -- Cholesky column panel in one cooperative launch.
//
// SLATE factors a column panel as potrf of the diagonal tile on the device
// queue (cuSOLVER, with a blocking info copy, src/internal/internal_potrf.cc:
// 56-81) followed by a batched trsm of the tiles below (src/potrf.cc:109-120).
// Here the whole nb-wide panel (rows r0..n-1, columns r0..r0+nb-1) is one
// cooperative persistent launch.  Block b owns a band of R rows (R a
// multiple of 64).  For each 64-column step k:
//   1. every block loads the published inverse of the factored 64 x 64
//      diagonal block (step 0: every block factors and inverts it itself);
//   2. every block solves its own rows below it, X = B L^{-T}, as one
//      register-tiled product with that inverse; the blocks owning rows of
//      the remaining panel columns ("head" rows, the update operand of
//      everyone) count themselves done in a per-step counter;
//   3. every block waits for that counter (a grid barrier at step 0 only) and
//      updates its rows in the remaining panel columns (rank-64 update);
//   4. the owner of the next diagonal block -- its only update tile is that
//      block -- factors it at once and publishes it (L11 in P, its inverse
//      and a failure word in the workspace, then a release of the step
//      number); the next step's blocks wait for exactly that.  With 64-row
//      blocks the owner skips step 3: it forms the block as D - X X^T from
//      its own solved rows, still in shared memory.
// No grid-wide barrier separates the steps: the critical path is the owner
// chain solve -> diagonal block update -> factor -> inverse.  Every wait is
// a bounded acquire spin (common.cuh), and the cooperative launch keeps all
// blocks resident, so every awaited block is running.

#include "common.cuh"
#include "prof.h"

namespace slt {

constexpr int kCpThreads = 256;
constexpr int kCpIB = 64;
constexpr int kCpSub = 16;
constexpr int kStage = kCpIB * kCpIB / kCpThreads;   // 64 x 64 tile elements per thread, loaded in one batch

// One warp: Cholesky of the bw x bw (bw <= 16) lower block S (row-major,
// row stride lds) in registers, lane r holding row r (rows bw .. 15 padded
// with the identity, which leaves the bw x bw factor unchanged); the factor
// is written back to S and the reciprocals of its diagonal to Rd[0 .. bw).
// Column j is scaled by 1 / sqrt(d) and broadcast through the 16-entry
// shared vector col.  The columns are unrolled by compile-time recursion so
// the row stays in registers.  Returns 0, or the 1-based column of the first
// non-positive pivot (S is then left as it was).
// sd = sqrt(d) and rd = 1 / sd.  FP32: the hardware reciprocal square root
// refined by one Newton-Raphson step, y <- y (3 - d y^2) / 2, which takes
// its ~2^-22 relative error below an ulp of the result (the division and
// square root chain of the IEEE forms is the panel's critical path).
// FP64: correctly rounded sqrt and division.
__device__ __forceinline__ void pivot_scale(float d, float& sd, float& rd)
{
    float y = rsqrtf(d);
    y = y * fmaf(-0.5f * d * y, y, 1.5f);
    rd = y;
    sd = d * y;
}
__device__ __forceinline__ void pivot_scale(double d, double& sd, double& rd)
{
    sd = sqrt(d);
    rd = 1.0 / sd;
}

template <int C, int N, typename T>
__device__ __forceinline__ void f16_update(T (&a)[N], const T aj, const T* col, int r)
{
    if constexpr (C < N) {
        a[C] = (r >= C) ? fma(-aj, col[C], a[C]) : a[C];
        f16_update<C + 1, N>(a, aj, col, r);
    }
}

template <int J, int N, typename T>
__device__ __forceinline__ void f16_columns(T (&a)[N], T* Rd, T* col, int r, int& fail)
{
    if constexpr (J < N) {
        const T d = __shfl_sync(0xffffffffu, a[J], J);
        if (!fail && !(d > T(0))) fail = J + 1;
        T sd, rd;
        pivot_scale(d, sd, rd);
        a[J] = (r == J) ? sd : a[J] * rd;
        if (r == J) Rd[J] = rd;
        if (r < N) col[r] = a[J];
        __syncwarp();
        f16_update<J + 1, N>(a, a[J], col, r);
        __syncwarp();
        f16_columns<J + 1, N>(a, Rd, col, r, fail);
    }
}

template <typename T>
__device__ int factor_16(T* S, int lds, int bw, T* Rd, T* col)
{
    const int r = threadIdx.x & 31;
    T a[kCpSub];
    #pragma unroll
    for (int c = 0; c < kCpSub; ++c)
        a[c] = (c > r) ? T(0) : (r < bw) ? S[r * lds + c] : (c == r) ? T(1) : T(0);
    int fail = 0;
    f16_columns<0, kCpSub>(a, Rd, col, r, fail);
    if (fail) return fail;
    if (r < bw) {
        #pragma unroll
        for (int cc = 0; cc < kCpSub; ++cc)
            if (cc <= r) S[r * lds + cc] = a[cc];
    }
    return 0;
}

// One warp: Inv (16 x 17, Inv[k * 17 + c] = L^{-1}(k, c), zero above the
// diagonal and outside bw) of the factor factor_16 left in S; lane c forms
// column c by forward substitution.
template <typename T>
__device__ void invert_16(const T* S, int lds, int bw, const T* Rd, T* Inv)
{
    const int c = threadIdx.x & 31;
    T x[kCpSub];
    #pragma unroll
    for (int k = 0; k < kCpSub; ++k) {
        T acc = (k == c) ? T(1) : T(0);
        #pragma unroll
        for (int p = 0; p < k; ++p) acc = fma(-S[k * lds + p], x[p], acc);
        x[k] = (k < bw && c < bw && k >= c) ? acc * Rd[k] : T(0);
    }
    if (c < kCpSub) {
        #pragma unroll
        for (int k = 0; k < kCpSub; ++k) Inv[k * (kCpSub + 1) + c] = x[k];
    }
}

template <typename T>
struct CholPanelArgs {
    int64_t m, nbk, ld, rows_per_block, info_offset;
    T* P;
    int* info;
    int* status;
    GridBarrier* bar;
    int* next_fail;     // 1 + the step whose diagonal block failed (its lookahead factor)
    unsigned* diag_ready;  // index of the last diagonal block published by the lookahead
    unsigned* head_done;   // per step: blocks that solved rows needed by the others' update
    T* dinv_ws;         // per step: the diagonal block's transposed inverse, [16][64][64]
    int vec;            // P 16-byte aligned and ld * sizeof(T) a multiple of 16: 4-vector access to P
};

// four consecutive elements of P (16-byte aligned), read through L2
__device__ __forceinline__ void ld4_cg(const float* p, float* v)
{
    const float4 x = __ldcg(reinterpret_cast<const float4*>(p));
    v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
}
__device__ __forceinline__ void ld4_cg(const double* p, double* v)
{
    const double2 x = __ldcg(reinterpret_cast<const double2*>(p));
    const double2 y = __ldcg(reinterpret_cast<const double2*>(p + 2));
    v[0] = x.x; v[1] = x.y; v[2] = y.x; v[3] = y.y;
}
__device__ __forceinline__ void st4(float* p, const float* v)
{
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void st4(double* p, const double* v)
{
    *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
    *reinterpret_cast<double2*>(p + 2) = make_double2(v[2], v[3]);
}
// four consecutive elements of a 16-byte aligned shared array
__device__ __forceinline__ void lds4(const float* p, float* v)
{
    const float4 x = *reinterpret_cast<const float4*>(p);
    v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
}
__device__ __forceinline__ void lds4(const double* p, double* v)
{
    const double2 x = *reinterpret_cast<const double2*>(p);
    const double2 y = *reinterpret_cast<const double2*>(p + 2);
    v[0] = x.x; v[1] = x.y; v[2] = y.x; v[3] = y.y;
}

constexpr int kCpLinv = kCpIB * kCpIB;                                 // transposed inverse of one diagonal block

// Bounded acquire spin of thread 0 until *p >= target; false on timeout or
// when another block has already failed (status set).
__device__ __forceinline__ bool wait_at_least(const unsigned* p, unsigned target, int* status)
{
    if (ld_acquire_u32(p) >= target) return true;
    const unsigned long long t0 = globaltimer();
    for (unsigned it = 1; ld_acquire_u32(p) < target; ++it) {
        if ((it & 63u) == 0 && (ld_volatile_i32(status) != 0 || globaltimer() - t0 > kWaitNs)) {
            atomicCAS(status, 0, SLT_ERR_TIMEOUT);
            return false;
        }
        __nanosleep(32);
    }
    return true;
}

// The 64 x 64 (kb x kb) diagonal block D (row-major in shared memory, row
// stride 65, lower triangle) factored in place by the whole CTA, in 16-column
// steps: warp 0 factors the 16 x 16 diagonal sub-block; then warps 1-7 solve
// the sub-block rows below it by forward substitution and update the rest of
// the block (their own 224-thread barrier).  At the end warps 0-3 invert the
// four sub-blocks in parallel into Dinv for the panel's row solves, so no
// inversion sits on the chain of sub-block steps.  Returns 0, or the 1-based column (within the
// block) of the first non-positive pivot; the same value in every thread.
__device__ __forceinline__ void bar_workers() { asm volatile("bar.sync 1, %0;" :: "n"(kCpThreads - 32) : "memory"); }

template <typename T>
__device__ int factor_diag_block(T* D, T* Dinv, int kb)
{
    __shared__ int s_f;
    __shared__ T s_rd[kCpIB / kCpSub][kCpSub];
    __shared__ T s_col[kCpSub];
    const int t = threadIdx.x;
    if (t == 0) s_f = 0;
    __syncthreads();
    for (int jb = 0, jbi = 0; jb < kb; jb += kCpSub, ++jbi) {
        const int bw = min(kCpSub, kb - jb);
        T* S = D + jb * (kCpIB + 1) + jb;
        if (t < 32) {
            const int fail = factor_16(S, kCpIB + 1, bw, s_rd[jbi], s_col);
            if (t == 0 && fail) s_f = jb + fail;
        }
        __syncthreads();
        if (s_f) break;
        const int below = kb - jb - bw;
        if (t >= 32 && below > 0) {
            const int w = t - 32;
            // rows i in [jb + bw, kb) of the sub-block column: X L^T = B, row by row
            if (w < below) {
                const int i = jb + bw + w;
                T* xi = D + i * (kCpIB + 1) + jb;
                T x[kCpSub];
                #pragma unroll
                for (int c = 0; c < kCpSub; ++c) {
                    T acc = (c < bw) ? xi[c] : T(0);
                    #pragma unroll
                    for (int p = 0; p < c; ++p) acc = fma(-x[p], S[c * (kCpIB + 1) + p], acc);
                    x[c] = (c < bw) ? acc * s_rd[jbi][c] : T(0);
                }
                #pragma unroll
                for (int c = 0; c < kCpSub; ++c)
                    if (c < bw) xi[c] = x[c];
            }
            bar_workers();
            // trailing update inside the block: D[i][c] -= sum_p D[i][jb+p] D[c][jb+p], jb+bw <= c <= i < kb
            // (bw = 16 whenever rows remain below).  4 x 4 output tiles on
            // and below the diagonal, one per worker thread; every element
            // sums its 16 products in order, as the one-element loop does.
            if (below % 4 == 0) {
                const int tb = below / 4;
                if (w < tb * (tb + 1) / 2) {
                    int ti = 0, tj = w;
                    while (tj > ti) { tj -= ti + 1; ++ti; }
                    const int i0 = jb + kCpSub + 4 * ti, c0 = jb + kCpSub + 4 * tj;
                    T acc[4][4];
                    #pragma unroll
                    for (int u = 0; u < 4; ++u)
                        #pragma unroll
                        for (int v = 0; v < 4; ++v) acc[u][v] = T(0);
                    #pragma unroll 2
                    for (int p = 0; p < kCpSub; ++p) {
                        T xi4[4], xc4[4];
                        #pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            xi4[u] = D[(i0 + u) * (kCpIB + 1) + jb + p];
                            xc4[u] = D[(c0 + u) * (kCpIB + 1) + jb + p];
                        }
                        #pragma unroll
                        for (int u = 0; u < 4; ++u)
                            #pragma unroll
                            for (int v = 0; v < 4; ++v) acc[u][v] = fma(xi4[u], xc4[v], acc[u][v]);
                    }
                    #pragma unroll
                    for (int u = 0; u < 4; ++u)
                        #pragma unroll
                        for (int v = 0; v < 4; ++v)
                            if (c0 + v <= i0 + u) D[(i0 + u) * (kCpIB + 1) + c0 + v] -= acc[u][v];
                }
            }
            else {
                for (int e = w; e < below * below; e += kCpThreads - 32) {
                    const int i = jb + bw + e % below, c = jb + bw + e / below;
                    if (c > i) continue;
                    T acc = T(0);
                    for (int p = 0; p < bw; ++p)
                        acc = fma(D[i * (kCpIB + 1) + jb + p], D[c * (kCpIB + 1) + jb + p], acc);
                    D[i * (kCpIB + 1) + c] -= acc;
                }
            }
        }
        __syncthreads();
    }
    // the sub-block inverses for the panel's row solves, one warp each, off
    // the chain of sub-block steps
    if (!s_f) {
        const int q = t >> 5;
        if (q * kCpSub < kb)
            invert_16(D + q * kCpSub * (kCpIB + 1) + q * kCpSub, kCpIB + 1, min(kCpSub, kb - q * kCpSub), s_rd[q],
                      Dinv + q * kCpSub * (kCpSub + 1));
    }
    __syncthreads();
    return s_f;
}

// The inverse of the factored kb x kb diagonal block L (D, row-major,
// stride 65), stored transposed: Lt[l * 68 + c] = L^{-1}(c, l), zero above
// the diagonal and outside kb.  The 16 x 16 diagonal blocks are the
// sub-block inverses Dinv; below them, by increasing distance d = I - J,
//     L^{-1}(I, J) = -Inv_I * sum_{K=J}^{I-1} L(I, K) L^{-1}(K, J)
// (16 x 16 blocks), the sums staged in Tmp (768 entries).  Every thread of
// the block takes part.
// One level d of build_linv_t: for the block pairs (I, J) = (J + d, J),
// Tmp = sum_{K=J}^{I-1} L(I, K) L^{-1}(K, J), then L^{-1}(I, J) = -Inv_I Tmp.
// Fixed trip counts (16 d products; Inv_I is zero above its diagonal) so the
// shared loads of every sum are issued ahead of its FMAs.
template <int DD, typename T>
__device__ __forceinline__ void linv_level(const T* D, const T* Dinv, T* Lt, T* Tmp, int nsub)
{
    const int npair = nsub - DD;
    if (npair <= 0) return;
    const int t = threadIdx.x;
    for (int e = t; e < npair * 256; e += kCpThreads) {
        const int J = e / 256, I = J + DD, i = (e % 256) / kCpSub, j = e % kCpSub;
        const T* drow = D + (kCpSub * I + i) * (kCpIB + 1) + kCpSub * J;
        const T* lcol = Lt + (kCpSub * J + j) * 68 + kCpSub * J;
        T acc = T(0);
        #pragma unroll
        for (int kk = 0; kk < kCpSub * DD; ++kk) acc = fma(drow[kk], lcol[kk], acc);
        Tmp[e] = acc;
    }
    __syncthreads();
    for (int e = t; e < npair * 256; e += kCpThreads) {
        const int J = e / 256, I = J + DD, i = (e % 256) / kCpSub, j = e % kCpSub;
        const T* inv = Dinv + I * kCpSub * (kCpSub + 1) + i * (kCpSub + 1);
        const T* tc = Tmp + J * 256 + j;
        T acc = T(0);
        #pragma unroll
        for (int mm = 0; mm < kCpSub; ++mm) acc = fma(inv[mm], tc[mm * kCpSub], acc);
        Lt[(kCpSub * J + j) * 68 + kCpSub * I + i] = -acc;
    }
    __syncthreads();
}

// The inverse of the factored kb x kb diagonal block L (D, row-major,
// stride 65), stored transposed: Lt[l * 68 + c] = L^{-1}(c, l), zero above
// the diagonal and outside kb.  The 16 x 16 diagonal blocks are the
// sub-block inverses Dinv (zero above their diagonals); below them, by
// increasing distance d = I - J,
//     L^{-1}(I, J) = -Inv_I * sum_{K=J}^{I-1} L(I, K) L^{-1}(K, J)
// (16 x 16 blocks), the sums staged in Tmp (768 entries).  Every thread of
// the block takes part.
template <typename T>
__device__ void build_linv_t(const T* D, const T* Dinv, T* Lt, T* Tmp, int kb)
{
    const int t = threadIdx.x;
    const int nsub = (kb + kCpSub - 1) / kCpSub;
    for (int e = t; e < kCpIB * kCpIB; e += kCpThreads) {
        const int l = e / kCpIB, c = e % kCpIB, q = c / kCpSub;
        T v = T(0);
        if (l / kCpSub == q && l <= c && c < kb)
            v = Dinv[q * kCpSub * (kCpSub + 1) + (c % kCpSub) * (kCpSub + 1) + l % kCpSub];
        Lt[l * 68 + c] = v;
    }
    __syncthreads();
    linv_level<1>(D, Dinv, Lt, Tmp, nsub);
    linv_level<2>(D, Dinv, Lt, Tmp, nsub);
    linv_level<3>(D, Dinv, Lt, Tmp, nsub);
}

template <typename T>
__global__ void __launch_bounds__(kCpThreads, 2)
chol_panel_kernel(CholPanelArgs<T> a)
{
    extern __shared__ __align__(16) unsigned char cp_smem_raw[];
    T* D = reinterpret_cast<T*>(cp_smem_raw);             // [64][65] diagonal block, D[i*65 + l] = L(i,l)
    T* Xs = D + kCpIB * (kCpIB + 1);                        // [64][68] solved rows, Xs[l*68 + i]
    T* Us = Xs + kCpIB * 68;                                // [64][68] inverse (transposed), then update operand
    T* Dinv = Us + kCpIB * 68;                              // [4][16][17] sub-block inverses
    __shared__ int s_fail, s_abort;
    const int G = gridDim.x, b = blockIdx.x, t = threadIdx.x;
    const int64_t ld = a.ld;
    T* P = a.P;
    const int64_t rb = int64_t(b) * a.rows_per_block;
    const int64_t re = min64(a.m, rb + a.rows_per_block);

    for (int64_t c0 = 0; c0 < a.nbk; c0 += kCpIB) {
        const int kb = int(min64(kCpIB, a.nbk - c0));
        // ---- 1. the inverse of the factored diagonal block in shared memory
        //      (Us, transposed).  First step: every block factors the block
        //      and inverts it itself (no earlier step could).  Later steps:
        //      its owner factored it during the previous step's update phase
        //      (below) and published L11 in P, the inverse and a failure word
        //      in the workspace; every block loads the inverse.
        const int k = int(c0 / kCpIB);
        // With 64-row blocks and a full 64-column next diagonal block, the
        // owner of that block owns exactly its rows, and its whole update is
        // D_next -= X X^T with X its own solved rows, formed in shared memory
        // below without waiting for the other head rows.  (A narrower next
        // block leaves owned rows below it in the panel: general path.)  The
        // old block goes to D (free while the rows are solved), fetched while
        // the owner waits for this step's diagonal block.
        const int64_t cnext = c0 + kb;
        const bool fast = cnext + kCpIB <= a.nbk && a.rows_per_block == kCpIB && cnext == rb;
        auto fetch_next_block = [&]() {
            const int kbn0 = int(min64(kCpIB, a.nbk - cnext));
            __syncthreads();          // the block's own update of this tile in the previous step
            staged_copy<kStage, kCpThreads>(kCpIB * kCpIB, [&](int e) {
                const int i = e % kCpIB, l = e / kCpIB;
                return (i < kbn0 && l < kbn0 && i >= l) ? __ldcg(&P[cnext + i + (cnext + l) * ld]) : T(0);
            }, [&](int e, T v) { D[(e % kCpIB) * (kCpIB + 1) + e / kCpIB] = v; });
        };
        if (fast && c0 > 0) fetch_next_block();
        if (c0 > 0) {
            if (t == 0) s_abort = wait_at_least(a.diag_ready, unsigned(k), a.status) ? 0 : 1;
            __syncthreads();
            if (s_abort) return;
            staged_copy<kStage, kCpThreads>(kCpLinv, [&](int e) {
                return __ldcg(&a.dinv_ws[size_t(k) * kCpLinv + e]);
            }, [&](int e, T v) { Us[(e / kCpIB) * 68 + e % kCpIB] = v; });
        }
        else {
            staged_copy<kStage, kCpThreads>(kCpIB * kCpIB, [&](int e) {
                const int i = e % kCpIB, l = e / kCpIB;
                return (i < kb && l < kb && i >= l) ? __ldcg(&P[c0 + i + (c0 + l) * ld]) : T(0);
            }, [&](int e, T v) { D[(e % kCpIB) * (kCpIB + 1) + e / kCpIB] = v; });
        }
        // next_fail holds 1 + the step whose diagonal block failed; the owner
        // of that block writes it during the step before, possibly before a
        // slower block has started that step, so only a failure of this
        // step's (or an earlier) block counts here
        if (t == 0) {
            const int nf = (c0 > 0) ? ld_volatile_i32(a.next_fail) : 0;
            s_fail = (nf != 0 && nf - 1 <= k) ? 1 : 0;
        }
        __syncthreads();
        if (c0 == 0) {
            const int f = factor_diag_block(D, Dinv, kb);
            if (t == 0 && f) {
                s_fail = 1;
                if (c0 >= rb && c0 < re) atomicCAS(a.info, 0, int(a.info_offset + c0 + f));
            }
            if (f == 0) build_linv_t(D, Dinv, Us, Xs, kb);
            // block 0 writes this factor back from D below; the owner of the
            // next block (never block 0) may now reuse D
            if (f == 0 && fast) fetch_next_block();
        }
        __syncthreads();
        const bool failed = s_fail != 0;
        // ---- 2. solve the owned rows below the block: X = B L^{-T}, 64 rows at
        //      a time, as one product with the inverse (Us) over 4 x 4
        //      register tiles (rows 4 tr + i, columns 4 tc + j; column c
        //      needs inverse rows l <= c).  The solved rows stay in Xs,
        //      [l][row] with stride 68 -- the layout of the update operand.
        if (!failed) {
            const int64_t r0 = max64(rb, c0 + kb);
            const int tr = t & 15, tc = t >> 4;
            for (int64_t rr = r0; rr < re; rr += kCpIB) {
                const int nr = int(min64(kCpIB, re - rr));
                __syncthreads();
                staged_copy<kStage, kCpThreads>(kCpIB * kCpIB, [&](int e) {
                    const int i = e % kCpIB, l = e / kCpIB;
                    return (i < nr && l < kb) ? __ldcg(&P[rr + i + (c0 + l) * ld]) : T(0);
                }, [&](int e, T v) { Xs[(e / kCpIB) * 68 + e % kCpIB] = v; });
                __syncthreads();
                T acc[4][4];
                #pragma unroll
                for (int i = 0; i < 4; ++i)
                    #pragma unroll
                    for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
                const int lmax = min(kb, 4 * tc + 4);
                #pragma unroll 4
                for (int l = 0; l < lmax; ++l) {
                    T xr[4], li[4];
                    lds4(Xs + l * 68 + 4 * tr, xr);
                    lds4(Us + l * 68 + 4 * tc, li);
                    #pragma unroll
                    for (int i = 0; i < 4; ++i)
                        #pragma unroll
                        for (int j = 0; j < 4; ++j) acc[i][j] = fma(xr[i], li[j], acc[i][j]);
                }
                __syncthreads();
                #pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const T v[4] = {acc[0][j], acc[1][j], acc[2][j], acc[3][j]};
                    st4(Xs + (4 * tc + j) * 68 + 4 * tr, v);
                }
                __syncthreads();
                for (int e = t; e < kCpIB * kCpIB; e += kCpThreads) {
                    int i = e % kCpIB, l = e / kCpIB;
                    if (i < nr && l < kb) P[rr + i + (c0 + l) * ld] = Xs[l * 68 + i];
                }
            }
        }
        // ---- rows [c0 + kb, nbk) are the update operand of every block: their
        //      owners announce them solved; the others wait for exactly those
        //      blocks (a grid barrier only at the first step, whose diagonal
        //      block every block read from P before its owner overwrites it).
        const int64_t cbeg = c0 + kb;
        const int64_t hend = min64(a.nbk, a.m);
        const int first_head = int(cbeg / a.rows_per_block);
        const int n_head = (cbeg < hend) ? int((hend - 1) / a.rows_per_block) - first_head + 1 : 0;
        const bool head = !failed && cbeg < hend && rb < hend && re > cbeg;
        __threadfence();
        __syncthreads();
        if (head && t == 0) atomicAdd(&a.head_done[k], 1u);
        if (c0 == 0) {
            if (!grid_sync(a.bar, unsigned(G), a.status)) return;
        }
        if (!failed && n_head > 0 && !fast) {
            if (t == 0) s_abort = wait_at_least(&a.head_done[k], unsigned(n_head), a.status) ? 0 : 1;
            __syncthreads();
            if (s_abort) return;
        }
        // every block has read the diagonal block: its owner writes the factor
        // back (later diagonal blocks were written by the lookahead below)
        if (c0 == 0 && c0 >= rb && c0 < re)
            for (int e = t; e < kCpIB * kCpIB; e += kCpThreads) {
                int i = e % kCpIB, l = e / kCpIB;
                if (i < kb && l < kb && i >= l) P[c0 + i + (c0 + l) * ld] = D[i * (kCpIB + 1) + l];
            }
        const bool owns_next = !failed && cbeg < a.nbk && cbeg >= rb && cbeg < re;
        // ---- 4. lookahead: the owner of the next diagonal block forms it as
        //      D - X X^T from its own solved rows X (the old block D fetched at
        //      the start of the step on the fast path, read from P here
        //      otherwise), factors and publishes it now, before its update of
        //      the other rows (section 3, which leaves that block's rows alone), while the
        //      other blocks are still updating.
        if (owns_next) {
            const int kbn = int(min64(kCpIB, a.nbk - cbeg));
            __syncthreads();
            if (!fast) {
                // the old block and the solved rows of the block's row tile
                staged_copy<kStage, kCpThreads>(kCpIB * kCpIB, [&](int e) {
                    const int i = e % kCpIB, l = e / kCpIB;
                    return (i < kbn && l < kbn && i >= l) ? __ldcg(&P[cbeg + i + (cbeg + l) * ld]) : T(0);
                }, [&](int e, T v) { D[(e % kCpIB) * (kCpIB + 1) + e / kCpIB] = v; });
                staged_copy<kStage, kCpThreads>(kCpIB * kCpIB, [&](int e) {
                    const int i = e % kCpIB, l = e / kCpIB;
                    return (i < kbn && l < kb) ? __ldcg(&P[cbeg + i + (c0 + l) * ld]) : T(0);
                }, [&](int e, T v) { Xs[(e / kCpIB) * 68 + e % kCpIB] = v; });
                __syncthreads();
            }
            {
                // D -= X X^T on the lower triangle, X = the solved rows in Xs
                // ([l][row], stride 68); the same FMA order as the update of
                // section 3, so the block is the one that update would make
                const int tr = t & 15, tc = t >> 4;      // rows 4 tr + i, columns 4 tc + j
                if (tc <= tr) {
                    T acc[4][4];
                    #pragma unroll
                    for (int i = 0; i < 4; ++i)
                        #pragma unroll
                        for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
                    #pragma unroll 4
                    for (int l = 0; l < kb; ++l) {
                        T xr[4], xc[4];
                        lds4(Xs + l * 68 + 4 * tr, xr);
                        lds4(Xs + l * 68 + 4 * tc, xc);
                        #pragma unroll
                        for (int i = 0; i < 4; ++i)
                            #pragma unroll
                            for (int j = 0; j < 4; ++j) acc[i][j] = fma(xr[i], xc[j], acc[i][j]);
                    }
                    #pragma unroll
                    for (int i = 0; i < 4; ++i)
                        #pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            const int row = 4 * tr + i, col = 4 * tc + j;
                            if (row < kbn && col <= row) D[row * (kCpIB + 1) + col] -= acc[i][j];
                        }
                }
            }
            __syncthreads();
            const int f = factor_diag_block(D, Dinv, kbn);
            if (f == 0) build_linv_t(D, Dinv, Us, Xs, kbn);
            for (int e = t; e < kCpIB * kCpIB; e += kCpThreads) {
                int i = e % kCpIB, l = e / kCpIB;
                if (i < kbn && l < kbn && i >= l) P[cbeg + i + (cbeg + l) * ld] = D[i * (kCpIB + 1) + l];
            }
            for (int e = t; e < kCpLinv; e += kCpThreads)
                a.dinv_ws[size_t(k + 1) * kCpLinv + e] = Us[(e / kCpIB) * 68 + e % kCpIB];
            if (t == 0 && f) {
                atomicCAS(a.info, 0, int(a.info_offset + cbeg + f));
                *reinterpret_cast<volatile int*>(a.next_fail) = k + 2;     // 1 + step k + 1
            }
            __threadfence();
            __syncthreads();
            if (t == 0) st_release_u32(a.diag_ready, unsigned(k + 1));
        }
        // ---- 3. rank-kb update of the owned rows in panel columns [c0+kb, nbk):
        //      per 64-row tile of the block (its solved rows staged once,
        //      [l][row], row stride 68) and per 64-column tile at or left of
        //      the tile's last row (operand [l][col]), 64 x 64 outputs with 4
        //      consecutive rows x 4 consecutive columns per thread: two
        //      4-vector shared loads per k step for 16 FMAs.  The old values
        //      of P are read before the product; whole tiles below the
        //      diagonal move as 4-vectors.
        if (cbeg < a.nbk && !failed && !fast) {
            T* X3 = Xs;                                  // [64][68]
            T* U3 = Us;                                  // [64][68]
            const int64_t r0 = max64(rb, cbeg);
            const int tr = t & 15, tc = t >> 4;          // rows 4 tr + i, columns 4 tc + j
            for (int64_t rr = r0; rr < re; rr += kCpIB) {
                const int nr = int(min64(kCpIB, re - rr));
                __syncthreads();
                // one row tile per block: the solve left exactly these rows in Xs,
                // unless section 4 used Xs since
                if (a.rows_per_block != kCpIB || owns_next)
                    staged_copy<kStage, kCpThreads>(kCpIB * kCpIB, [&](int e) {
                        const int i = e % kCpIB, l = e / kCpIB;
                        return (i < nr && l < kb) ? __ldcg(&P[rr + i + (c0 + l) * ld]) : T(0);
                    }, [&](int e, T v) { X3[(e / kCpIB) * 68 + e % kCpIB] = v; });
                // a column tile starting past the row tile's last row has no
                // lower-triangular entries here, nor have the tiles after it
                for (int64_t cb = cbeg; cb < a.nbk && cb < rr + nr; cb += kCpIB) {
                    // rows of the next diagonal block (factored in section 4) keep L11
                    const int keep = (owns_next && rr == cbeg && cb == cbeg) ? int(min64(kCpIB, a.nbk - cbeg)) : 0;
                    const int nc = int(min64(kCpIB, a.nbk - cb));
                    __syncthreads();
                    staged_copy<kStage, kCpThreads>(kCpIB * kCpIB, [&](int e) {
                        const int c = e % kCpIB, l = e / kCpIB;
                        return (c < nc && l < kb) ? __ldcg(&P[cb + c + (c0 + l) * ld]) : T(0);
                    }, [&](int e, T v) { U3[(e / kCpIB) * 68 + e % kCpIB] = v; });
                    const bool full = a.vec && nr == kCpIB && nc == kCpIB && rr >= cb + kCpIB;
                    T* Pt = P + rr + 4 * tr + (cb + 4 * tc) * ld;      // element (4 tr, 4 tc) of the tile
                    T old[4][4];                                        // [column j][row i]
                    if (full) {
                        #pragma unroll
                        for (int j = 0; j < 4; ++j) ld4_cg(Pt + j * ld, old[j]);
                    }
                    else {
                        #pragma unroll
                        for (int j = 0; j < 4; ++j)
                            #pragma unroll
                            for (int i = 0; i < 4; ++i) {
                                const int c = 4 * tc + j, ii = 4 * tr + i;
                                old[j][i] = (c < nc && ii < nr && rr + ii >= cb + c) ? __ldcg(Pt + i + j * ld) : T(0);
                            }
                    }
                    __syncthreads();
                    T acc[4][4];
                    #pragma unroll
                    for (int i = 0; i < 4; ++i)
                        #pragma unroll
                        for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
                    #pragma unroll 4
                    for (int l = 0; l < kb; ++l) {
                        T xr[4], uc[4];
                        lds4(X3 + l * 68 + 4 * tr, xr);
                        lds4(U3 + l * 68 + 4 * tc, uc);
                        #pragma unroll
                        for (int i = 0; i < 4; ++i)
                            #pragma unroll
                            for (int j = 0; j < 4; ++j) acc[i][j] = fma(xr[i], uc[j], acc[i][j]);
                    }
                    if (full) {
                        #pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            T v[4];
                            #pragma unroll
                            for (int i = 0; i < 4; ++i) v[i] = old[j][i] - acc[i][j];
                            st4(Pt + j * ld, v);
                        }
                    }
                    else {
                        #pragma unroll
                        for (int j = 0; j < 4; ++j)
                            #pragma unroll
                            for (int i = 0; i < 4; ++i) {
                                const int c = 4 * tc + j, ii = 4 * tr + i;
                                if (c < nc && ii < nr && ii >= keep && rr + ii >= cb + c) Pt[i + j * ld] = old[j][i] - acc[i][j];
                            }
                    }
                }
            }
        }
        if (failed) return;       // every block saw the same failing diagonal block
    }
}

template <typename T>
static int launch_chol_panel(int64_t m, int64_t nbk, T* P, int64_t ld, int* info, int64_t info_offset,
                             void* ws, int* status, cudaStream_t stream)
{
    if (m <= 0 || nbk <= 0) return SLT_OK;
    int dev = 0, sms = 0, coop = 0;
    SLT_CUDA_TRY(cudaGetDevice(&dev));
    SLT_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    SLT_CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (!coop) return SLT_ERR_NOT_SUPPORTED;
    sms = capped_sms(sms);
    const size_t smem = (size_t(kCpIB) * (kCpIB + 1) + size_t(2) * kCpIB * 68 +
                         size_t(kCpIB / kCpSub) * kCpSub * (kCpSub + 1)) * sizeof(T);
    SLT_SMEM_ONCE(chol_panel_kernel<T>, smem);
    int per_sm = 0;
    SLT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, chol_panel_kernel<T>, kCpThreads, smem));
    if (per_sm < 1) return SLT_ERR_NOT_SUPPORTED;
    const int64_t maxg = int64_t(sms) * per_sm;             // all blocks co-resident
    int64_t R = ceildiv(ceildiv(m, maxg), kCpIB) * kCpIB;     // multiple of 64
    int64_t G = ceildiv(m, R);
    if (nbk > 16 * kCpIB) return SLT_ERR_ARG;                // per-step words below
    // ws: barrier at 0, failure word at 256, diagonal-ready word at 260,
    // per-step head counters at 264, per-step sub-block inverses at 512
    char* w = static_cast<char*>(ws);
    GridBarrier* bar = reinterpret_cast<GridBarrier*>(w);
    int* next_fail = reinterpret_cast<int*>(w + 256);
    unsigned* diag_ready = reinterpret_cast<unsigned*>(w + 260);
    unsigned* head_done = reinterpret_cast<unsigned*>(w + 264);
    T* dinv_ws = reinterpret_cast<T*>(w + 512);
    SLT_CUDA_TRY(cudaMemsetAsync(ws, 0, 512, stream));
    const int vec = (reinterpret_cast<uintptr_t>(P) % 16 == 0) && ((ld * int64_t(sizeof(T))) % 16 == 0);
    CholPanelArgs<T> args{m, nbk, ld, R, info_offset, P, info, status, bar, next_fail, diag_ready, head_done,
                          dinv_ws, vec};
    void* kargs[] = { &args };
    const int pidx = prof_begin(SLT_PROF_POTRF, stream);
    SLT_CUDA_TRY(cudaLaunchCooperativeKernel((const void*) chol_panel_kernel<T>, dim3(unsigned(G)),
                                             dim3(kCpThreads), kargs, smem, stream));
    count_launch();
    prof_end(pidx, stream, double(m) * double(nbk) * double(nbk), 2.0 * sizeof(T) * double(m) * double(nbk));
    return SLT_OK;
}

} // namespace slt

using namespace slt;

// Device scratch of one panel launch: grid barrier, lookahead failure word
// and, per 64-column step, the diagonal block's transposed inverse.
extern "C" size_t slt_chol_panel_ws_bytes(void)
{
    return 512 + size_t(16) * kCpLinv * sizeof(double);
}

// Factor the Cholesky column panel with top-left P (the diagonal element),
// m rows (to the bottom of the matrix), nbk columns.  ws: slt_chol_panel_ws_bytes()
// bytes of device scratch.
extern "C" int slt_dchol_panel(int64_t m, int64_t nbk, double* P, int64_t ld, int* info, int64_t info_offset,
                               void* ws, int* status, cudaStream_t stream)
{ return launch_chol_panel<double>(m, nbk, P, ld, info, info_offset, ws, status, stream); }

extern "C" int slt_schol_panel(int64_t m, int64_t nbk, float* P, int64_t ld, int* info, int64_t info_offset,
                               void* ws, int* status, cudaStream_t stream)
{ return launch_chol_panel<float>(m, nbk, P, ld, info, info_offset, ws, status, stream); }
