// trsm.cu -- triangular solves and the diagonal-block Cholesky.
//
// Replaces SLATE's batched device trsm (internal::trsm<Devices>,
// src/internal/internal_trsm.cc:131-260: the LU row panel
// A(k,j) <- L(k,k)^{-1} A(k,j) and the Cholesky column panel
// A(i,k) <- A(i,k) L(k,k)^{-H}), the diagonal-block solves of getrs/potrs
// (internal::trsmA, src/internal/internal_trsmA.cc:332), and the device
// potrf of a diagonal tile that SLATE hands to cuSOLVER
// (src/internal/internal_potrf.cc:72-78).
//
// One kernel covers every case: solve op(T) X = B for a block of 32
// right-hand-side vectors held in shared memory; op(T) is effectively lower
// (forward sweep) or upper (backward sweep).  The right-side Cholesky panel
// solve B L^{-T} is the same forward sweep over the rows of B.
// Each 64-row block of X is first updated from the already-solved rows
// (256 threads, 8 outputs each), then solved against the 64 x 64 diagonal
// block staged in shared memory with 8 lanes per vector.

#include "common.cuh"
#include "prof.h"

namespace slt {

constexpr int kTrsmCols = 32;
constexpr int kTrsmDB = 64;

// FORWARD: op(T) lower.  TRANS: op(T)(r,l) = T(l,r).  RIGHT: the vectors are
// rows of B (B is m x kb, solved as X op(T)^T = B).
template <typename T, bool FORWARD, bool UNIT, bool TRANS, bool RIGHT>
__global__ void __launch_bounds__(256)
trsm_kernel(int kb, int64_t nvec, const T* __restrict__ Tm, int64_t ldt, T* B, int64_t ldb)
{
    extern __shared__ unsigned char smem_raw[];
    T* X = reinterpret_cast<T*>(smem_raw);                 // [kb][kTrsmCols]
    T* D = X + size_t(kb) * kTrsmCols;                     // [kTrsmDB][kTrsmDB + 1]
    const int t = threadIdx.x;
    const int64_t v0 = int64_t(blockIdx.x) * kTrsmCols;
    const int nv = int(min64(kTrsmCols, nvec - v0));

    auto opT = [&](int r, int l) -> T {
        return TRANS ? Tm[l + int64_t(r) * ldt] : Tm[r + int64_t(l) * ldt];
    };
    auto bidx = [&](int r, int c) -> int64_t {
        return RIGHT ? (v0 + c) + int64_t(r) * ldb : int64_t(r) + (v0 + c) * ldb;
    };

    staged_copy<16, 256>(kb * kTrsmCols, [&](int e) {
        const int r = RIGHT ? e / kTrsmCols : e % kb, c = RIGHT ? e % kTrsmCols : e / kb;
        return (c < nv) ? B[bidx(r, c)] : T(0);
    }, [&](int e, T v) {
        const int r = RIGHT ? e / kTrsmCols : e % kb, c = RIGHT ? e % kTrsmCols : e / kb;
        X[r * kTrsmCols + c] = v;
    });
    __syncthreads();

    const int nblk = (kb + kTrsmDB - 1) / kTrsmDB;
    for (int bi = 0; bi < nblk; ++bi) {
        const int blk = FORWARD ? bi : nblk - 1 - bi;
        const int rb = blk * kTrsmDB;
        const int re = min(kb, rb + kTrsmDB);
        const int nr = re - rb;
        // stage the diagonal block of op(T)
        staged_copy<kTrsmDB * kTrsmDB / 256, 256>(kTrsmDB * kTrsmDB, [&](int e) {
            const int i = e % kTrsmDB, l = e / kTrsmDB;
            return (i < nr && l < nr) ? opT(rb + i, rb + l) : T(0);
        }, [&](int e, T v) { D[(e % kTrsmDB) * (kTrsmDB + 1) + e / kTrsmDB] = v; });
        // update rows [rb, re) from the solved rows
        {
            const int i = t % kTrsmDB;
            const int cg = t / kTrsmDB;            // 4 groups of 8 vectors
            if (i < nr) {
                T acc[8];
                #pragma unroll
                for (int q = 0; q < 8; ++q) acc[q] = T(0);
                const int l0 = FORWARD ? 0 : re;
                const int l1 = FORWARD ? rb : kb;
                for (int l = l0; l < l1; ++l) {
                    T a = opT(rb + i, l);
                    #pragma unroll
                    for (int q = 0; q < 8; ++q) acc[q] = fma(a, X[l * kTrsmCols + cg * 8 + q], acc[q]);
                }
                #pragma unroll
                for (int q = 0; q < 8; ++q) X[(rb + i) * kTrsmCols + cg * 8 + q] -= acc[q];
            }
        }
        __syncthreads();
        // solve the diagonal block: 8 lanes per vector, 4 vectors per warp
        {
            const int c = t >> 3;          // vector 0..31
            const int q = t & 7;           // lane within group
            for (int s = 0; s < nr; ++s) {
                const int r = FORWARD ? s : nr - 1 - s;
                T part = T(0);
                if (FORWARD) {
                    for (int l = q; l < r; l += 8) part = fma(D[r * (kTrsmDB + 1) + l], X[(rb + l) * kTrsmCols + c], part);
                }
                else {
                    for (int l = r + 1 + q; l < nr; l += 8) part = fma(D[r * (kTrsmDB + 1) + l], X[(rb + l) * kTrsmCols + c], part);
                }
                part += __shfl_xor_sync(0xffffffffu, part, 4);
                part += __shfl_xor_sync(0xffffffffu, part, 2);
                part += __shfl_xor_sync(0xffffffffu, part, 1);
                if (q == 0) {
                    T x = X[(rb + r) * kTrsmCols + c] - part;
                    if (!UNIT) x = x / D[r * (kTrsmDB + 1) + r];
                    X[(rb + r) * kTrsmCols + c] = x;
                }
                __syncwarp();
            }
        }
        __syncthreads();
    }

    for (int e = t; e < kb * kTrsmCols; e += 256) {
        int r, c;
        if (RIGHT) { c = e % kTrsmCols; r = e / kTrsmCols; }
        else       { r = e % kb; c = e / kb; }
        if (c < nv) B[bidx(r, c)] = X[r * kTrsmCols + c];
    }
}

template <typename T, bool FORWARD, bool UNIT, bool TRANS, bool RIGHT>
static int launch_trsm(int64_t kb, int64_t nvec, const T* Tm, int64_t ldt, T* B, int64_t ldb,
                       cudaStream_t stream)
{
    if (kb <= 0 || nvec <= 0) return SLT_OK;
    if (kb > 1024) return SLT_ERR_ARG;
    size_t smem = (size_t(kb) * kTrsmCols + size_t(kTrsmDB) * (kTrsmDB + 1)) * sizeof(T);
    auto fn = trsm_kernel<T, FORWARD, UNIT, TRANS, RIGHT>;
    if (smem > 48 * 1024)
        SLT_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    unsigned grid = unsigned(ceildiv(nvec, kTrsmCols));
    const int pidx = prof_begin(SLT_PROF_TRSM, stream);
    fn<<<grid, 256, smem, stream>>>(int(kb), nvec, Tm, ldt, B, ldb); slt::count_launch();
    prof_end(pidx, stream, double(kb) * double(kb) * double(nvec), sizeof(T) * (double(kb) * kb / 2 + 2.0 * kb * nvec));
    return slt_from_cuda(cudaGetLastError());
}

// Cholesky of one kb x kb lower block (kb <= 128) in shared memory, one CTA.
template <typename T>
__global__ void __launch_bounds__(256)
potrf_small_kernel(int kb, T* A, int64_t lda, int* info, int64_t info_offset)
{
    extern __shared__ unsigned char smem_raw[];
    T* S = reinterpret_cast<T*>(smem_raw);     // [kb][kb+1], column l at S[l*(kb+1)]
    const int ld = kb + 1;
    const int t = threadIdx.x;
    __shared__ int s_fail;
    if (t == 0) s_fail = 0;
    for (int e = t; e < kb * kb; e += blockDim.x) {
        int i = e % kb, l = e / kb;
        if (i >= l) S[l * ld + i] = A[i + l * lda];
    }
    __syncthreads();
    for (int j = 0; j < kb; ++j) {
        T d = S[j * ld + j];
        bool bad = !(d > T(0));
        if (bad) {
            if (t == 0 && !s_fail) {
                s_fail = 1;
                atomicCAS(info, 0, int(info_offset + j + 1));
            }
        }
        T sd = sqrt(d);
        __syncthreads();
        if (s_fail) break;
        for (int i = j + 1 + t; i < kb; i += blockDim.x) S[j * ld + i] /= sd;
        if (t == 0) S[j * ld + j] = sd;
        __syncthreads();
        // trailing lower update: S(i,l) -= S(i,j) S(l,j), j < l <= i
        const int nt = kb - j - 1;
        for (int e = t; e < nt * nt; e += blockDim.x) {
            int i = j + 1 + e % nt, l = j + 1 + e / nt;
            if (i >= l) S[l * ld + i] -= S[j * ld + i] * S[j * ld + l];
        }
        __syncthreads();
    }
    for (int e = t; e < kb * kb; e += blockDim.x) {
        int i = e % kb, l = e / kb;
        if (i >= l) A[i + l * lda] = S[l * ld + i];
    }
}

template <typename T>
static int launch_potrf_small(int64_t kb, T* A, int64_t lda, int* info, int64_t info_offset,
                              cudaStream_t stream)
{
    if (kb <= 0) return SLT_OK;
    if (kb > 128) return SLT_ERR_ARG;
    size_t smem = size_t(kb) * (kb + 1) * sizeof(T);
    auto fn = potrf_small_kernel<T>;
    if (smem > 48 * 1024)
        SLT_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    const int pidx = prof_begin(SLT_PROF_POTRF, stream);
    fn<<<1, 256, smem, stream>>>(int(kb), A, lda, info, info_offset); slt::count_launch();
    prof_end(pidx, stream, double(kb) * kb * kb / 3.0, sizeof(T) * double(kb) * kb);
    return slt_from_cuda(cudaGetLastError());
}

} // namespace slt

using namespace slt;

extern "C" int slt_dtrsm_llnu(int64_t kb, int64_t n, const double* L, int64_t ldl, double* B,
                              int64_t ldb, cudaStream_t stream)
{ return launch_trsm<double, true, true, false, false>(kb, n, L, ldl, B, ldb, stream); }
extern "C" int slt_strsm_llnu(int64_t kb, int64_t n, const float* L, int64_t ldl, float* B,
                              int64_t ldb, cudaStream_t stream)
{ return launch_trsm<float, true, true, false, false>(kb, n, L, ldl, B, ldb, stream); }

extern "C" int slt_dtrsm_lunn(int64_t kb, int64_t n, const double* U, int64_t ldu, double* B,
                              int64_t ldb, cudaStream_t stream)
{ return launch_trsm<double, false, false, false, false>(kb, n, U, ldu, B, ldb, stream); }
extern "C" int slt_strsm_lunn(int64_t kb, int64_t n, const float* U, int64_t ldu, float* B,
                              int64_t ldb, cudaStream_t stream)
{ return launch_trsm<float, false, false, false, false>(kb, n, U, ldu, B, ldb, stream); }

extern "C" int slt_dtrsm_llnn(char trans, int64_t kb, int64_t n, const double* L, int64_t ldl,
                              double* B, int64_t ldb, cudaStream_t stream)
{
    if (trans == 'N') return launch_trsm<double, true, false, false, false>(kb, n, L, ldl, B, ldb, stream);
    if (trans == 'T') return launch_trsm<double, false, false, true, false>(kb, n, L, ldl, B, ldb, stream);
    return SLT_ERR_ARG;
}
extern "C" int slt_strsm_llnn(char trans, int64_t kb, int64_t n, const float* L, int64_t ldl,
                              float* B, int64_t ldb, cudaStream_t stream)
{
    if (trans == 'N') return launch_trsm<float, true, false, false, false>(kb, n, L, ldl, B, ldb, stream);
    if (trans == 'T') return launch_trsm<float, false, false, true, false>(kb, n, L, ldl, B, ldb, stream);
    return SLT_ERR_ARG;
}

extern "C" int slt_dtrsm_rltn(int64_t m, int64_t kb, const double* L, int64_t ldl, double* B,
                              int64_t ldb, cudaStream_t stream)
{ return launch_trsm<double, true, false, false, true>(kb, m, L, ldl, B, ldb, stream); }
extern "C" int slt_strsm_rltn(int64_t m, int64_t kb, const float* L, int64_t ldl, float* B,
                              int64_t ldb, cudaStream_t stream)
{ return launch_trsm<float, true, false, false, true>(kb, m, L, ldl, B, ldb, stream); }

// B (m x kb) <- B U^{-1}, U upper non-unit (the CALU panel's L21 = A21 U11^{-1},
// src/getrf_tntpiv.cc: internal::trsm Side::Right on the upper diagonal tile):
// the rows of B solved against op(T) = U^T, lower.
extern "C" int slt_dtrsm_runn(int64_t m, int64_t kb, const double* U, int64_t ldu, double* B,
                              int64_t ldb, cudaStream_t stream)
{ return launch_trsm<double, true, false, true, true>(kb, m, U, ldu, B, ldb, stream); }
extern "C" int slt_strsm_runn(int64_t m, int64_t kb, const float* U, int64_t ldu, float* B,
                              int64_t ldb, cudaStream_t stream)
{ return launch_trsm<float, true, false, true, true>(kb, m, U, ldu, B, ldb, stream); }

extern "C" int slt_dpotrf_small(int64_t kb, double* A, int64_t lda, int* info, int64_t info_offset,
                                cudaStream_t stream)
{ return launch_potrf_small<double>(kb, A, lda, info, info_offset, stream); }
extern "C" int slt_spotrf_small(int64_t kb, float* A, int64_t lda, int* info, int64_t info_offset,
                                cudaStream_t stream)
{ return launch_potrf_small<float>(kb, A, lda, info, info_offset, stream); }
