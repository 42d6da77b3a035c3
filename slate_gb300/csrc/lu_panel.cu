// lu_panel.cu -- GPU LU panel factorization and row interchanges.
//
// Panel: replaces SLATE's host panel (internal::getrf_panel<HostTask>,
// src/internal/internal_getrf.cc:20-121, running tile::getrf,
// src/internal/Tile_getrf.hh:159-447), which SLATE runs on CPU threads even
// for Target::Devices (src/getrf.cc:95-97).  Same arithmetic per column:
// max-|a| search with the diagonal kept on ties, full-width row interchange,
// scaling by the reciprocal pivot when |pivot| >= safe_min (division
// otherwise), rank-1 update inside the ib-wide stripe; after each stripe a
// unit-lower trsm of the top block and a rank-ib update of the rest of the
// panel.
//
// GB300 design: one cooperative persistent launch per panel.  Block b owns a
// contiguous band of panel rows; each column costs one grid barrier: blocks
// publish their local pivot candidate (value, row, and the candidate row's
// stripe entries) to a double-buffered exchange area, every block then
// reduces the candidates identically, so no second barrier is needed.
// Barriers are bounded spin-waits (status word on timeout).
//
// Row interchanges outside the panel: SLATE issues one blas::swap per pivot
// row per tile (src/internal/internal_swap.cc:662-689).  Here a panel's
// interchanges are first folded into one gather plan (<= 2 nb row moves),
// then one launch moves every affected row of every column.

#include "common.cuh"
#include "prof.h"
#include <climits>

namespace slt {

constexpr int kPanelThreads = 256;
constexpr int kMaxPanelBlocks = 1024;
constexpr int kMaxIb = 64;
constexpr size_t kPanelStagedMax = 96 * 1024;   // dynamic shared memory of the staged panel

template <typename T>
struct PanelExchange {
    T cand_val[2][kMaxPanelBlocks];
    int cand_row[2][kMaxPanelBlocks];
    T cand_rowvals[2][kMaxPanelBlocks][kMaxIb];
    T diag_rowvals[2][kMaxIb];
};

template <typename T>
struct PanelArgs {
    int64_t prows, nbk, ib, ld, rows_per_block, info_offset;
    double threshold;   // SLATE's PivotThreshold: keep the diagonal when |a_jj| >= threshold * max
    T* P;
    int* ipiv;
    int* info;
    int* status;
    GridBarrier* bar;
    PanelExchange<T>* ex;
};

// (|v|, row) ordering: larger magnitude wins, ties go to the lower row.
template <typename T>
__device__ __forceinline__ bool better(T av, int row, T bv, int brow)
{
    return av > bv || (av == bv && row < brow);
}

template <typename T>
__device__ __forceinline__ void warp_argmax(T& av, T& v, int& row)
{
    #pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        T oav = __shfl_down_sync(0xffffffffu, av, off);
        T ov = __shfl_down_sync(0xffffffffu, v, off);
        int orow = __shfl_down_sync(0xffffffffu, row, off);
        if (better(oav, orow, av, row)) { av = oav; v = ov; row = orow; }
    }
}

// End of an ib-wide stripe (all its columns final): the interchanges of the
// stripe applied to the panel columns outside it, the unit-lower solve of the
// top block right of the stripe, and the rank-kb update of the owned rows
// below it.  Returns false when the kernel must stop (bounded wait failed).
template <typename T>
__device__ bool stripe_end(const PanelArgs<T>& a, int G, int b, int t, int64_t k0, int kb, int64_t rb,
                           int64_t re, const int* s_piv, T (*s_L)[kMaxIb + 1], T (*s_U)[32 + 1])
{
    const int64_t ld = a.ld;
    T* P = a.P;
    if (!grid_sync(a.bar, unsigned(G), a.status)) return false;
    {
        const int64_t nout = a.nbk - kb;
        for (int64_t q = int64_t(b) * kPanelThreads + t; q < nout; q += int64_t(G) * kPanelThreads) {
            const int64_t cc = (q < k0) ? q : q + kb;
            T* col = P + cc * ld;
            for (int jj = 0; jj < kb; ++jj) {
                int64_t r = k0 + jj, pr = s_piv[jj];
                if (pr != r) { T tmp = __ldcg(&col[r]); col[r] = __ldcg(&col[pr]); col[pr] = tmp; }
            }
            if (cc >= k0 + kb) {
                for (int r = 1; r < kb; ++r) {
                    T s = __ldcg(&col[k0 + r]);
                    for (int l = 0; l < r; ++l) s -= __ldcg(&P[k0 + r + (k0 + l) * ld]) * __ldcg(&col[k0 + l]);
                    col[k0 + r] = s;
                }
            }
        }
    }
    if (k0 + kb < a.nbk) {
        if (!grid_sync(a.bar, unsigned(G), a.status)) return false;
        // ---- rank-kb update of owned rows below the stripe
        const int64_t c0 = k0 + kb;
        const int64_t r0 = max(rb, k0 + kb);
        for (int64_t rr = r0; rr < re; rr += 32) {
            const int nr = int(min64(32, re - rr));
            __syncthreads();
            staged_copy<8, kPanelThreads>(32 * kb, [&](int e) {
                const int i = e % 32, l = e / 32;
                return (i < nr) ? __ldcg(&P[rr + i + (k0 + l) * ld]) : T(0);
            }, [&](int e, T v) { s_L[e % 32][e / 32] = v; });
            for (int64_t cb = c0; cb < a.nbk; cb += 32) {
                const int nc = int(min64(32, a.nbk - cb));
                __syncthreads();
                staged_copy<8, kPanelThreads>(kb * 32, [&](int e) {
                    const int l = e % kb, c = e / kb;
                    return (c < nc) ? __ldcg(&P[k0 + l + (cb + c) * ld]) : T(0);
                }, [&](int e, T v) { s_U[e % kb][e / kb] = v; });
                __syncthreads();
                // 32 x 32 outputs, 4 per thread
                const int i = t % 32;
                const int cg = t / 32;   // 0..7 -> columns cg, cg+8, cg+16, cg+24
                if (i < nr) {
                    #pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        int c = cg + 8 * q;
                        if (c < nc) {
                            T s = T(0);
                            for (int l = 0; l < kb; ++l) s = fma(s_L[i][l], s_U[l][c], s);
                            T* q2 = &P[rr + i + (cb + c) * ld];
                            *q2 = __ldcg(q2) - s;
                        }
                    }
                }
            }
            __syncthreads();
        }
        if (!grid_sync(a.bar, unsigned(G), a.status)) return false;
    }
    return true;
}

template <typename T>
__global__ void __launch_bounds__(kPanelThreads)
getrf_panel_kernel(PanelArgs<T> a)
{
    constexpr int NW = kPanelThreads / 32;
    const int G = gridDim.x;
    const int b = blockIdx.x;
    const int t = threadIdx.x;
    const int lane = t & 31, warp = t >> 5;
    const int64_t ld = a.ld;
    T* P = a.P;
    const int64_t rb = int64_t(b) * a.rows_per_block;
    const int64_t re = min(a.prows, rb + a.rows_per_block);
    const int64_t diag_len = min(a.prows, a.nbk);
    PanelExchange<T>* ex = a.ex;

    __shared__ T s_av[NW], s_v[NW];
    __shared__ int s_row[NW];
    __shared__ int s_piv[kMaxIb];
    __shared__ T s_u[kMaxIb];
    __shared__ T s_pval;
    __shared__ int s_p, s_wb;
    // staging for the in-panel rank-ib update
    __shared__ T s_L[32][kMaxIb + 1];
    __shared__ T s_U[kMaxIb][32 + 1];

    for (int64_t k0 = 0; k0 < diag_len; k0 += a.ib) {
        const int kb = int(min64(a.ib, diag_len - k0));
        for (int64_t j = k0; j < k0 + kb; ++j) {
            const int par = int(j & 1);
            // ---- local candidate
            T bav = T(-1), bv = T(0);
            int brow = INT_MAX;
            for (int64_t i = max(rb, j) + t; i < re; i += kPanelThreads) {
                T v = __ldcg(&P[i + j * ld]);
                T av = fabs(v);
                if (better(av, int(i), bav, brow)) { bav = av; bv = v; brow = int(i); }
            }
            warp_argmax(bav, bv, brow);
            if (lane == 0) { s_av[warp] = bav; s_v[warp] = bv; s_row[warp] = brow; }
            __syncthreads();
            if (warp == 0) {
                bav = lane < NW ? s_av[lane] : T(-1);
                bv = lane < NW ? s_v[lane] : T(0);
                brow = lane < NW ? s_row[lane] : INT_MAX;
                warp_argmax(bav, bv, brow);
                if (lane == 0) { s_av[0] = bav; s_v[0] = bv; s_row[0] = brow; }
            }
            __syncthreads();
            brow = s_row[0];
            if (t == 0) {
                ex->cand_val[par][b] = s_v[0];
                ex->cand_row[par][b] = (s_av[0] >= T(0)) ? brow : INT_MAX;
            }
            if (brow != INT_MAX && s_av[0] >= T(0))
                for (int c = t; c < kb; c += kPanelThreads)
                    ex->cand_rowvals[par][b][c] = __ldcg(&P[brow + (k0 + c) * ld]);
            if (j >= rb && j < re)
                for (int c = t; c < kb; c += kPanelThreads)
                    ex->diag_rowvals[par][c] = __ldcg(&P[j + (k0 + c) * ld]);
            __threadfence();
            if (!grid_sync(a.bar, unsigned(G), a.status)) return;

            // ---- global pivot: every block reduces the same candidates
            if (warp == 0) {
                T gav = T(-1), gv = T(0);
                int grow = INT_MAX, gwb = -1;
                for (int q = lane; q < G; q += 32) {
                    int r = ((volatile int*) ex->cand_row[par])[q];
                    T v = ((volatile T*) ex->cand_val[par])[q];
                    T av = (r == INT_MAX) ? T(-1) : fabs(v);
                    if (r != INT_MAX && better(av, r, gav, grow)) { gav = av; gv = v; grow = r; gwb = q; }
                }
                #pragma unroll
                for (int off = 16; off > 0; off >>= 1) {
                    T oav = __shfl_down_sync(0xffffffffu, gav, off);
                    T ov = __shfl_down_sync(0xffffffffu, gv, off);
                    int orow = __shfl_down_sync(0xffffffffu, grow, off);
                    int owb = __shfl_down_sync(0xffffffffu, gwb, off);
                    if (better(oav, orow, gav, grow)) { gav = oav; gv = ov; grow = orow; gwb = owb; }
                }
                if (lane == 0) {
                    if (grow == INT_MAX) {
                        // whole column NaN: keep the diagonal (SLATE's scan
                        // starts from it and '>' never accepts a NaN)
                        grow = int(j);
                        gwb = -1;
                        gv = __ldcg(&P[j + j * ld]);
                    }
                    else if (a.threshold < 1.0 && grow != int(j)) {
                        // threshold rule (Tile_getrf.hh:272-289): keep the diagonal
                        const T dv = ((volatile T*) ex->diag_rowvals[par])[j - k0];
                        if (fabs(dv) >= gav * T(a.threshold)) { grow = int(j); gwb = -1; gv = dv; }
                    }
                    s_p = grow;
                    s_wb = gwb;
                    s_pval = gv;
                    s_piv[j - k0] = grow;
                    if (b == 0) {
                        a.ipiv[j] = grow;
                        if (gv == T(0)) atomicCAS(a.info, 0, int(a.info_offset + j + 1));
                    }
                }
            }
            __syncthreads();
            const int64_t p = s_p;
            const int wb = s_wb;
            const T pval = s_pval;
            // new row j stripe entries (the pivot row), from the exchange area
            for (int c = t; c < kb; c += kPanelThreads) {
                T u = (wb >= 0) ? ((volatile T*) ex->cand_rowvals[par][wb])[c] : __ldcg(&P[j + (k0 + c) * ld]);
                s_u[c] = u;
            }
            __syncthreads();
            if (p != j) {
                if (j >= rb && j < re)
                    for (int c = t; c < kb; c += kPanelThreads) P[j + (k0 + c) * ld] = s_u[c];
                if (p >= rb && p < re)
                    for (int c = t; c < kb; c += kPanelThreads)
                        P[p + (k0 + c) * ld] = ((volatile T*) ex->diag_rowvals[par])[c];
            }
            __syncthreads();
            // ---- scale and rank-1 update of the owned rows below j
            const bool recip = fabs(pval) >= Real<T>::safe_min();
            const T rinv = T(1) / pval;
            const int jc = int(j - k0);
            for (int64_t i = max(rb, j + 1) + t; i < re; i += kPanelThreads) {
                T l = __ldcg(&P[i + j * ld]);
                if (recip) l *= rinv;
                else if (pval != T(0)) l /= pval;
                P[i + j * ld] = l;
                for (int c = jc + 1; c < kb; ++c) {
                    T* q = &P[i + (k0 + c) * ld];
                    *q = __ldcg(q) - l * s_u[c];
                }
            }
            __syncthreads();
        }

        if (!stripe_end(a, G, b, t, k0, kb, rb, re, s_piv, s_L, s_U)) return;
    }
}

// Staged variant, used when a block's rows of one stripe fit in shared memory
// (rows_per_block x ib elements).  Same arithmetic and the same choices as
// getrf_panel_kernel, with two changes on the per-column critical path:
//  * the block's rows of the current stripe live in shared memory for the
//    whole stripe (loaded once, written back at its end), so the search, the
//    scaling and the rank-1 update never wait on L2;
//  * the per-column grid barrier is replaced by a per-block sequence flag
//    published (release) with the block's candidate: every block waits
//    (acquire, bounded) until all flags reach the column's sequence number,
//    then reads the candidates -- one L2 round trip fewer than a
//    counter barrier followed by the reads.  Candidates stay double
//    buffered: a block can run at most one column ahead of the slowest.
template <typename T>
__global__ void __launch_bounds__(kPanelThreads)
getrf_panel2_kernel(PanelArgs<T> a, int* flags)
{
    constexpr int NW = kPanelThreads / 32;
    const int G = gridDim.x;
    const int b = blockIdx.x;
    const int t = threadIdx.x;
    const int lane = t & 31, warp = t >> 5;
    const int64_t ld = a.ld;
    T* P = a.P;
    const int64_t rb = int64_t(b) * a.rows_per_block;
    const int64_t re = min(a.prows, rb + a.rows_per_block);
    const int nrow = int(max64(0, re - rb));
    const int RP = int(a.rows_per_block);
    const int64_t diag_len = min(a.prows, a.nbk);
    PanelExchange<T>* ex = a.ex;

    extern __shared__ unsigned char p2_smem_raw[];
    T* S = reinterpret_cast<T*>(p2_smem_raw);          // S[c * RP + r]: owned row rb + r, stripe column c
    __shared__ T s_av[NW], s_v[NW];
    __shared__ int s_row[NW];
    __shared__ int s_piv[kMaxIb];
    __shared__ T s_u[kMaxIb];
    __shared__ T s_pval;
    __shared__ int s_p, s_wb, s_fail;
    __shared__ T s_L[32][kMaxIb + 1];
    __shared__ T s_U[kMaxIb][32 + 1];
    if (t == 0) s_fail = 0;
    int seq = 0;

    for (int64_t k0 = 0; k0 < diag_len; k0 += a.ib) {
        const int kb = int(min64(a.ib, diag_len - k0));
        __syncthreads();
        staged_copy<8, kPanelThreads>(nrow * kb, [&](int e) { return __ldcg(&P[rb + e % nrow + (k0 + e / nrow) * ld]); },
                                      [&](int e, T v) { S[(e / nrow) * RP + e % nrow] = v; });
        __syncthreads();
        for (int64_t j = k0; j < k0 + kb; ++j) {
            ++seq;
            const int par = seq & 1;
            const int jc = int(j - k0);
            // ---- local candidate from shared memory
            T bav = T(-1), bv = T(0);
            int brow = INT_MAX;
            for (int64_t i = max(rb, j) + t; i < re; i += kPanelThreads) {
                const T v = S[jc * RP + int(i - rb)];
                const T av = fabs(v);
                if (better(av, int(i), bav, brow)) { bav = av; bv = v; brow = int(i); }
            }
            warp_argmax(bav, bv, brow);
            if (lane == 0) { s_av[warp] = bav; s_v[warp] = bv; s_row[warp] = brow; }
            __syncthreads();
            if (warp == 0) {
                bav = lane < NW ? s_av[lane] : T(-1);
                bv = lane < NW ? s_v[lane] : T(0);
                brow = lane < NW ? s_row[lane] : INT_MAX;
                warp_argmax(bav, bv, brow);
                if (lane == 0) { s_av[0] = bav; s_v[0] = bv; s_row[0] = brow; }
            }
            __syncthreads();
            brow = s_row[0];
            const bool has = brow != INT_MAX && s_av[0] >= T(0);
            if (t == 0) {
                ex->cand_val[par][b] = s_v[0];
                ex->cand_row[par][b] = has ? brow : INT_MAX;
            }
            if (has)
                for (int c = t; c < kb; c += kPanelThreads)
                    ex->cand_rowvals[par][b][c] = S[c * RP + int(brow - rb)];
            if (j >= rb && j < re)
                for (int c = t; c < kb; c += kPanelThreads)
                    ex->diag_rowvals[par][c] = S[c * RP + int(j - rb)];
            __threadfence();
            __syncthreads();
            if (t == 0) st_release_u32(reinterpret_cast<unsigned*>(&flags[b]), unsigned(seq));

            // ---- wait for every block's candidate, then reduce them (warp 0)
            if (warp == 0) {
                bool ok = true;
                const unsigned long long t0 = globaltimer();
                for (int q = lane; q < G && ok; q += 32) {
                    for (unsigned it = 1; ld_acquire_u32(reinterpret_cast<const unsigned*>(&flags[q])) <
                                          unsigned(seq); ++it) {
                        if ((it & 63u) == 0 && (ld_volatile_i32(a.status) != 0 || globaltimer() - t0 > kWaitNs)) {
                            atomicCAS(a.status, 0, SLT_ERR_TIMEOUT);
                            ok = false;
                            break;
                        }
                    }
                }
                ok = __all_sync(0xffffffffu, ok);
                T gav = T(-1), gv = T(0);
                int grow = INT_MAX, gwb = -1;
                if (ok) {
                    for (int q = lane; q < G; q += 32) {
                        int r = ((volatile int*) ex->cand_row[par])[q];
                        T v = ((volatile T*) ex->cand_val[par])[q];
                        T av = (r == INT_MAX) ? T(-1) : fabs(v);
                        if (r != INT_MAX && better(av, r, gav, grow)) { gav = av; gv = v; grow = r; gwb = q; }
                    }
                }
                #pragma unroll
                for (int off = 16; off > 0; off >>= 1) {
                    T oav = __shfl_down_sync(0xffffffffu, gav, off);
                    T ov = __shfl_down_sync(0xffffffffu, gv, off);
                    int orow = __shfl_down_sync(0xffffffffu, grow, off);
                    int owb = __shfl_down_sync(0xffffffffu, gwb, off);
                    if (better(oav, orow, gav, grow)) { gav = oav; gv = ov; grow = orow; gwb = owb; }
                }
                if (lane == 0) {
                    if (!ok) s_fail = 1;
                    if (grow == INT_MAX) {
                        // whole column NaN: keep the diagonal (SLATE's scan
                        // starts from it and '>' never accepts a NaN)
                        grow = int(j);
                        gwb = -1;
                        gv = ((volatile T*) ex->diag_rowvals[par])[jc];
                    }
                    else if (a.threshold < 1.0 && grow != int(j)) {
                        // threshold rule (Tile_getrf.hh:272-289): keep the diagonal
                        const T dv = ((volatile T*) ex->diag_rowvals[par])[jc];
                        if (fabs(dv) >= gav * T(a.threshold)) { grow = int(j); gwb = -1; gv = dv; }
                    }
                    s_p = grow;
                    s_wb = gwb;
                    s_pval = gv;
                    s_piv[jc] = grow;
                    if (b == 0 && ok) {
                        a.ipiv[j] = grow;
                        if (gv == T(0)) atomicCAS(a.info, 0, int(a.info_offset + j + 1));
                    }
                }
            }
            __syncthreads();
            if (s_fail) return;
            const int64_t p = s_p;
            const int wb = s_wb;
            const T pval = s_pval;
            for (int c = t; c < kb; c += kPanelThreads)
                s_u[c] = (wb >= 0) ? ((volatile T*) ex->cand_rowvals[par][wb])[c]
                                   : ((volatile T*) ex->diag_rowvals[par])[c];
            __syncthreads();
            if (p != j) {
                if (j >= rb && j < re)
                    for (int c = t; c < kb; c += kPanelThreads) S[c * RP + int(j - rb)] = s_u[c];
                if (p >= rb && p < re)
                    for (int c = t; c < kb; c += kPanelThreads)
                        S[c * RP + int(p - rb)] = ((volatile T*) ex->diag_rowvals[par])[c];
            }
            __syncthreads();
            // ---- scale and rank-1 update of the owned rows below j
            const bool recip = fabs(pval) >= Real<T>::safe_min();
            const T rinv = T(1) / pval;
            for (int64_t i = max(rb, j + 1) + t; i < re; i += kPanelThreads) {
                const int r = int(i - rb);
                T l = S[jc * RP + r];
                if (recip) l *= rinv;
                else if (pval != T(0)) l /= pval;
                S[jc * RP + r] = l;
                for (int c = jc + 1; c < kb; ++c) S[c * RP + r] -= l * s_u[c];
            }
            __syncthreads();
        }
        // stripe final in shared memory: write it back
        for (int e = t; e < nrow * kb; e += kPanelThreads) {
            const int r = e % nrow, c = e / nrow;
            P[rb + r + (k0 + c) * ld] = S[c * RP + r];
        }
        __threadfence();
        if (!stripe_end(a, G, b, t, k0, kb, rb, re, s_piv, s_L, s_U)) return;
    }
}

// ---- swap plan: fold one panel's sequential interchanges into row moves.
// One thread; an open-addressing table in shared memory maps the absolute
// rows below the diagonal block to slots.
constexpr int kPlanHash = 4096;

__global__ void swap_plan_kernel(const int* __restrict__ ipiv, int len, int64_t r0, int* plan)
{
    __shared__ int h_key[kPlanHash];
    __shared__ int h_slot[kPlanHash];
    extern __shared__ int dyn[];
    int* cur = dyn;              // 2*len: original row held at slot
    int* slot_row = dyn + 2 * len;
    for (int i = threadIdx.x; i < kPlanHash; i += blockDim.x) h_key[i] = -1;
    for (int i = threadIdx.x; i < len; i += blockDim.x) {
        cur[i] = int(r0) + i;
        slot_row[i] = int(r0) + i;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    int nslots = len;
    for (int j = 0; j < len; ++j) {
        int p = ipiv[j];
        int sp;
        if (p < len) {
            sp = p;
        }
        else {
            int row = int(r0) + p;
            unsigned h = unsigned(row) * 2654435761u;
            int hidx = int(h >> 20) & (kPlanHash - 1);
            while (h_key[hidx] != -1 && h_key[hidx] != row) hidx = (hidx + 1) & (kPlanHash - 1);
            if (h_key[hidx] == -1) {
                h_key[hidx] = row;
                h_slot[hidx] = nslots;
                cur[nslots] = row;
                slot_row[nslots] = row;
                ++nslots;
            }
            sp = h_slot[hidx];
        }
        int tmp = cur[j]; cur[j] = cur[sp]; cur[sp] = tmp;
    }
    int cnt = 0;
    int* dst = plan + 1;
    int* src = plan + 1 + 2 * len;
    for (int s = 0; s < nslots; ++s) {
        if (cur[s] != slot_row[s]) {
            dst[cnt] = slot_row[s];
            src[cnt] = cur[s];
            ++cnt;
        }
    }
    plan[0] = cnt;
}

// Apply a plan to ncols columns: gather every source row first, then write.
template <typename T, int CB>
__global__ void __launch_bounds__(256)
laswp_plan_kernel(const int* __restrict__ plan, int maxcount, T* A, int64_t lda, int64_t ncols)
{
    extern __shared__ unsigned char smem_raw[];
    T* vals = reinterpret_cast<T*>(smem_raw);
    const int cnt = plan[0];
    if (cnt == 0) return;
    const int* dst = plan + 1;
    const int* src = plan + 1 + maxcount;
    const int64_t c0 = int64_t(blockIdx.x) * CB;
    const int nc = int(min64(CB, ncols - c0));
    for (int e = threadIdx.x; e < cnt * nc; e += blockDim.x) {
        int q = e % cnt, c = e / cnt;
        vals[c * cnt + q] = A[src[q] + (c0 + c) * lda];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < cnt * nc; e += blockDim.x) {
        int q = e % cnt, c = e / cnt;
        A[dst[q] + (c0 + c) * lda] = vals[c * cnt + q];
    }
}

// Compose all panels' interchanges into one permutation.  Thread i traces
// final position i backwards through the n interchanges (r <-> p_r, p_r >= r):
// O(n) work per thread, all threads reading the same pivot at the same time
// from a shared-memory chunk, so the whole composition is one short launch.
__global__ void __launch_bounds__(256)
perm_from_ipiv_kernel(const int* __restrict__ ipiv, int n, int nb, int* perm)
{
    constexpr int CH = 2048;
    __shared__ int s_p[CH];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int pos = i;
    for (int hi = n; hi > 0; hi -= CH) {
        const int lo = max(0, hi - CH);
        __syncthreads();
        for (int r = lo + threadIdx.x; r < hi; r += blockDim.x)
            s_p[r - lo] = (r / nb) * nb + ipiv[r];
        __syncthreads();
        for (int r = hi - 1; r >= lo; --r) {
            const int p = s_p[r - lo];
            if (pos == r) pos = p;
            else if (pos == p) pos = r;
        }
    }
    if (i < n) perm[i] = pos;
}

template <typename T>
__global__ void permute_rows_kernel(int forward, const int* __restrict__ perm, int64_t n, int64_t ncols,
                                    const T* __restrict__ X, int64_t ldx, T* __restrict__ Y, int64_t ldy)
{
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    int64_t c = blockIdx.y;
    if (i >= n || c >= ncols) return;
    if (forward) Y[i + c * ldy] = X[perm[i] + c * ldx];
    else Y[perm[i] + c * ldy] = X[i + c * ldx];
}

template <typename T>
static int launch_panel(int64_t prows, int64_t nbk, int64_t ib, T* P, int64_t ld, int* ipiv,
                        int* info, int64_t info_offset, double threshold, void* ws, int* status,
                        cudaStream_t stream)
{
    if (prows <= 0 || nbk <= 0) return SLT_OK;
    if (ib <= 0 || ib > kMaxIb) return SLT_ERR_ARG;
    int dev = 0, sms = 0, coop = 0;
    SLT_CUDA_TRY(cudaGetDevice(&dev));
    SLT_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    SLT_CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (!coop) return SLT_ERR_NOT_SUPPORTED;
    sms = capped_sms(sms);
    int per_sm = 0;
    SLT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, getrf_panel_kernel<T>,
                                                               kPanelThreads, 0));
    if (per_sm < 1) return SLT_ERR_NOT_SUPPORTED;
    int64_t maxg = std::min<int64_t>(int64_t(sms) * per_sm, int64_t(std::min(sms, kMaxPanelBlocks)));
    const int64_t min_rows = 128;
    int64_t G = std::max<int64_t>(1, std::min<int64_t>(maxg, ceildiv(prows, min_rows)));
    int64_t R = ceildiv(prows, G);
    G = ceildiv(prows, R);

    char* base = static_cast<char*>(ws);
    GridBarrier* bar = reinterpret_cast<GridBarrier*>(base);
    PanelExchange<T>* ex = reinterpret_cast<PanelExchange<T>*>(base + 256);
    SLT_CUDA_TRY(cudaMemsetAsync(bar, 0, sizeof(GridBarrier), stream));

    PanelArgs<T> args;
    args.prows = prows; args.nbk = nbk; args.ib = ib; args.ld = ld;
    args.rows_per_block = R; args.info_offset = info_offset;
    args.threshold = threshold;
    args.P = P; args.ipiv = ipiv; args.info = info; args.status = status;
    args.bar = bar; args.ex = ex;
    // staged variant when the block's stripe rows fit in shared memory
    const size_t staged = sizeof(T) * size_t(R) * size_t(ib);
    int* flags = reinterpret_cast<int*>(base + 256 + ((sizeof(PanelExchange<double>) + 255) & ~size_t(255)));
    const int pidx = prof_begin(SLT_PROF_PANEL, stream);
    if (staged <= kPanelStagedMax) {
        SLT_SMEM_ONCE(getrf_panel2_kernel<T>, kPanelStagedMax);
        int per2 = 0;
        SLT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per2, getrf_panel2_kernel<T>, kPanelThreads,
                                                                   staged));
        if (per2 >= 1 && int64_t(sms) * per2 >= G) {
            SLT_CUDA_TRY(cudaMemsetAsync(flags, 0, sizeof(int) * size_t(kMaxPanelBlocks), stream));
            void* kargs2[] = { &args, &flags };
            SLT_CUDA_TRY(cudaLaunchCooperativeKernel((const void*) getrf_panel2_kernel<T>, dim3(unsigned(G)),
                                                     dim3(kPanelThreads), kargs2, staged, stream));
            count_launch();
            const double nb_ = double(nbk), m_ = double(prows);
            prof_end(pidx, stream, m_ * nb_ * nb_ - nb_ * nb_ * nb_ / 3.0, 2.0 * m_ * nb_ * sizeof(T));
            return SLT_OK;
        }
    }
    void* kargs[] = { &args };
    SLT_CUDA_TRY(cudaLaunchCooperativeKernel((const void*) getrf_panel_kernel<T>, dim3(unsigned(G)),
                                             dim3(kPanelThreads), kargs, 0, stream));
    count_launch();
    {
        const double nb_ = double(nbk), m_ = double(prows);
        prof_end(pidx, stream, m_ * nb_ * nb_ - nb_ * nb_ * nb_ / 3.0, 2.0 * m_ * nb_ * sizeof(T));
    }
    return SLT_OK;
}

template <typename T>
static int launch_laswp(const int* plan, int64_t maxcount, T* A, int64_t lda, int64_t ncols,
                        cudaStream_t stream)
{
    if (ncols <= 0 || maxcount <= 0) return SLT_OK;
    constexpr int CB = 8;
    size_t smem = size_t(CB) * size_t(maxcount) * sizeof(T);
    if (smem > 200 * 1024) return SLT_ERR_ARG;
    if (smem > 48 * 1024)
        SLT_CUDA_TRY(cudaFuncSetAttribute(laswp_plan_kernel<T, CB>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    unsigned grid = unsigned(ceildiv(ncols, CB));
    const int pidx = prof_begin(SLT_PROF_LASWP, stream);
    laswp_plan_kernel<T, CB><<<grid, 256, smem, stream>>>(plan, int(maxcount), A, lda, ncols); slt::count_launch();
    prof_end(pidx, stream, 0.0, 2.0 * sizeof(T) * double(maxcount) * double(ncols));
    return slt_from_cuda(cudaGetLastError());
}

} // namespace slt

using namespace slt;

// Panel scratch: grid barrier (256 B), candidate exchange, per-block flags.
extern "C" size_t slt_getrf_panel_ws_bytes(int64_t prows, int64_t ib)
{
    (void) prows; (void) ib;
    return 256 + ((sizeof(PanelExchange<double>) + 255) & ~size_t(255)) + sizeof(int) * size_t(kMaxPanelBlocks);
}

extern "C" int slt_dgetrf_panel(int64_t prows, int64_t nbk, int64_t ib, double* P, int64_t ld,
                                int* ipiv, int* info, int64_t info_offset, double threshold, void* ws,
                                int* status, cudaStream_t stream)
{
    return launch_panel<double>(prows, nbk, ib, P, ld, ipiv, info, info_offset, threshold, ws, status, stream);
}

extern "C" int slt_sgetrf_panel(int64_t prows, int64_t nbk, int64_t ib, float* P, int64_t ld,
                                int* ipiv, int* info, int64_t info_offset, double threshold, void* ws,
                                int* status, cudaStream_t stream)
{
    return launch_panel<float>(prows, nbk, ib, P, ld, ipiv, info, info_offset, threshold, ws, status, stream);
}

extern "C" int slt_swap_plan(const int* ipiv, int64_t len, int64_t r0, int* plan, cudaStream_t stream)
{
    if (len <= 0) return SLT_OK;
    if (len > 1024) return SLT_ERR_ARG;
    size_t smem = size_t(4 * len) * sizeof(int);
    swap_plan_kernel<<<1, 256, smem, stream>>>(ipiv, int(len), r0, plan); slt::count_launch();
    return slt_from_cuda(cudaGetLastError());
}

extern "C" int slt_dlaswp_plan(const int* plan, int64_t maxcount, double* A, int64_t lda,
                               int64_t ncols, cudaStream_t stream)
{
    return launch_laswp<double>(plan, maxcount, A, lda, ncols, stream);
}

extern "C" int slt_slaswp_plan(const int* plan, int64_t maxcount, float* A, int64_t lda,
                               int64_t ncols, cudaStream_t stream)
{
    return launch_laswp<float>(plan, maxcount, A, lda, ncols, stream);
}

extern "C" int slt_perm_from_ipiv(const int* ipiv, int64_t n, int64_t nb, int* perm, cudaStream_t stream)
{
    if (n <= 0) return SLT_OK;
    perm_from_ipiv_kernel<<<unsigned(ceildiv(n, 256)), 256, 0, stream>>>(ipiv, int(n), int(nb), perm); slt::count_launch();
    return slt_from_cuda(cudaGetLastError());
}

extern "C" int slt_dpermute_rows(int forward, const int* perm, int64_t n, int64_t ncols,
                                 const double* X, int64_t ldx, double* Y, int64_t ldy, cudaStream_t stream)
{
    if (n <= 0 || ncols <= 0) return SLT_OK;
    dim3 grid(unsigned(ceildiv(n, 256)), unsigned(ncols));
    permute_rows_kernel<double><<<grid, 256, 0, stream>>>(forward, perm, n, ncols, X, ldx, Y, ldy); slt::count_launch();
    return slt_from_cuda(cudaGetLastError());
}

extern "C" int slt_spermute_rows(int forward, const int* perm, int64_t n, int64_t ncols,
                                 const float* X, int64_t ldx, float* Y, int64_t ldy, cudaStream_t stream)
{
    if (n <= 0 || ncols <= 0) return SLT_OK;
    dim3 grid(unsigned(ceildiv(n, 256)), unsigned(ncols));
    permute_rows_kernel<float><<<grid, 256, 0, stream>>>(forward, perm, n, ncols, X, ldx, Y, ldy); slt::count_launch();
    return slt_from_cuda(cudaGetLastError());
}
