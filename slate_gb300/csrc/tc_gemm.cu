// tc_gemm.cu -- low-precision tensor-core trailing update on tcgen05 (sm_103a).
//
// The O(n^3) part of the mixed-precision factorisations: SLATE's trailing
// update (internal::gemm / internal::herk, src/internal/internal_gemm.cc:
// 354-518, src/internal/internal_herk.cc:350-540) runs in FP32 there
// (gesv_mixed<double,float>, src/gesv_mixed.cc:183).  Here the trailing matrix
// stays FP32 in HBM while the two panel operands are rounded to BF16 / FP16
// (or TF32) and multiplied on the 5th-generation tensor cores with FP32
// accumulation:
//
//     C (fp32, m x n) -= A (m x k) * op(B),  op(B) = B (k x n) or B^T.
//
// 1. pack_kernel: cast the operands to the tier's type, K-contiguous rows
//    ("K-major"), zero-padded to the tile grid.
// 2. tc_update_kernel: one 128 x BN output tile per CTA.  One thread issues
//    TMA loads (cp.async.bulk.tensor, 128B swizzle) into a ring of smem
//    stages guarded by mbarriers; one thread issues tcgen05.mma into a TMEM
//    accumulator and frees stages with tcgen05.commit; then all four warps
//    read the accumulator with tcgen05.ld (32 lanes x 32 columns per
//    instruction) and update C with coalesced column segments.
// FP8 (E4M3, kind::f8f6f4): each 128-row tile of A and of op(B)^T is scaled
// by a power of two s = 2^(8 - e), max|x| = m 2^e with m in [0.5, 1), so that
// its largest entry lands in [128, 256) below E4M3's 448; the epilogue
// multiplies the accumulator by 1 / (s_A s_B), exactly.  A K-tile is 128
// bytes of K in every tier (64 16-bit, 32 TF32 or 128 FP8 elements) and each
// MMA consumes 32 bytes of it, so the pipeline is the same for all kinds.
// Every mbarrier wait is bounded: on timeout the CTA records
// SLT_ERR_TIMEOUT, drains its own TMA copies (bounded), frees its TMEM and
// returns.

#include "common.cuh"
#include "prof.h"
#include "slate_gb300.h"
#include "tc_ptx.cuh"
#include "drivers.h"

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_fp8.h>

#include <mutex>

namespace slt {

constexpr int kTcBM = 128;
constexpr int kTcBN = 128;
constexpr int kTcStages = 4;
constexpr int kTcThreads = 128;

struct TcArgs {
    int64_t m, n, kpad;
    float* C;
    int64_t ldc;
    int lower;
    int* status;
    const float* inv_a;     // FP8: 1 / s per 128-row tile of A and of op(B)^T, else null
    const float* inv_b;
};

// elements of K in one 128-byte K tile for each kind
template <int KIND>
__host__ __device__ constexpr int kt_elems() { return KIND == 0 ? 64 : KIND == 2 ? 128 : 32; }

__device__ __forceinline__ float tile_factor(const TcArgs& a, int64_t row0, int64_t col0)
{
    return a.inv_a ? a.inv_a[row0 / kTcBM] * a.inv_b[col0 / kTcBN] : 1.f;
}

// KIND 0: 16-bit operands (BF16 or FP16 per fmt), KIND 1: TF32, KIND 2: FP8 E4M3.
template <int KIND>
__global__ void __launch_bounds__(kTcThreads, 1)
tc_update_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                 TcArgs a, uint32_t idesc)
{
    constexpr int BM = kTcBM, BN = kTcBN, S = kTcStages;
    constexpr int A_BYTES = BM * 128;   // 128 rows x 128 B (one swizzle atom of K)
    constexpr int B_BYTES = BN * 128;
    constexpr int STAGE = A_BYTES + B_BYTES;
    extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
    // 1024-byte aligned base for the swizzled tiles
    const uint32_t raw = smem_u32(tc_smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;
    unsigned char* gbase = tc_smem_raw + (base - raw);
    uint64_t* bars = reinterpret_cast<uint64_t*>(gbase + S * STAGE);   // full[S], empty[S], accum
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * S + 1);
    __shared__ int s_abort;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t row0 = int64_t(blockIdx.x) * BM;
    const int64_t col0 = int64_t(blockIdx.y) * BN;
    if (a.lower && row0 + BM - 1 < col0) return;       // tile strictly above the diagonal
    const int KT = int(a.kpad / kt_elems<KIND>());

    const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + S), accum = smem_u32(bars + 2 * S);
    if (threadIdx.x == 0) {
        s_abort = 0;
        for (int s = 0; s < S; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, 1);
        }
        mbar_init(accum, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 0) tmem_alloc(smem_u32(tmem_slot), BN);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t taddr = *tmem_slot;

    int issued = 0;   // TMA stages armed by the producer
    if (warp == 0 && lane == 0) {
        // ---- TMA producer
        for (int kt = 0; kt < KT; ++kt) {
            const int s = kt % S;
            const uint32_t par = ((kt / S) & 1) ^ 1;
            if (!mbar_wait(empty0 + 8 * s, par)) { atomicCAS(a.status, 0, SLT_ERR_TIMEOUT); s_abort = 1; break; }
            if (*(volatile int*) &s_abort) break;
            const uint32_t sa = base + s * STAGE, sb = sa + A_BYTES;
            mbar_expect_tx(full0 + 8 * s, STAGE);
            tma_load_2d(sa, &mapA, full0 + 8 * s, kt * kt_elems<KIND>(), int(row0));
            tma_load_2d(sb, &mapB, full0 + 8 * s, kt * kt_elems<KIND>(), int(col0));
            issued = kt + 1;
        }
    }
    else if (warp == 1 && lane == 0) {
        // ---- MMA issuer
        bool ok = true;
        for (int kt = 0; kt < KT; ++kt) {
            const int s = kt % S;
            const uint32_t par = (kt / S) & 1;
            if (!mbar_wait(full0 + 8 * s, par)) { atomicCAS(a.status, 0, SLT_ERR_TIMEOUT); ok = false; break; }
            if (*(volatile int*) &s_abort) { ok = false; break; }
            tc_fence_after();
            const uint32_t sa = base + s * STAGE, sb = sa + A_BYTES;
            const uint64_t da = sw128_desc(sa), db = sw128_desc(sb);
            #pragma unroll
            for (int k = 0; k < 4; ++k)   // 4 MMAs of K = 16 (16-bit), 8 (tf32) or 32 (fp8): 32 bytes each
                umma<KIND>(taddr, da + uint64_t(2 * k), db + uint64_t(2 * k), idesc, (kt | k) != 0 ? 1u : 0u);
            umma_commit(empty0 + 8 * s);
        }
        if (ok) umma_commit(accum);
        else s_abort = 1;
    }
    __syncwarp();

    // ---- epilogue: all four warps
    bool ready = mbar_wait(accum, 0);
    ready = __all_sync(0xffffffffu, ready);          // tcgen05.ld below is warp-collective
    if (!ready && lane == 0) atomicCAS(a.status, 0, SLT_ERR_TIMEOUT);
    tc_fence_after();
    if (ready) {
        const int64_t r = row0 + warp * 32 + lane;
        const float f = tile_factor(a, row0, col0);
        #pragma unroll 1
        for (int cc = 0; cc < BN; cc += 32) {
            float v[32];
            tmem_ld32(taddr + (uint32_t(warp * 32) << 16) + uint32_t(cc), v);
            if (r < a.m) {
                #pragma unroll
                for (int i = 0; i < 32; ++i) {
                    const int64_t c = col0 + cc + i;
                    if (c < a.n && !(a.lower && r < c)) {
                        float* p = a.C + r + c * a.ldc;
                        *p = *p - v[i] * f;
                    }
                }
            }
        }
    }
    // drain this CTA's own TMA copies if the pipeline was abandoned
    if (warp == 0 && lane == 0 && !ready) {
        for (int s = 0; s < S && s < issued; ++s) {
            const int last = s + ((issued - 1 - s) / S) * S;   // last armed phase of stage s
            mbar_wait(full0 + 8 * s, (last / S) & 1);
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(taddr, BN);
}

// Persistent, warp-specialised variant.  Warp 0: TMA producer; warp 1: MMA
// issuer (and TMEM owner); warps 2-5: epilogue, one TMEM lane quarter each.
// Two TMEM accumulators (2 x BN columns) let the epilogue of one tile overlap
// the MMAs of the next.  The epilogue stages -acc in shared memory and adds
// it to C with a TMA tensor reduce (cp.reduce.async.bulk.tensor .add), so the
// read-modify-write of C is done by the memory system with full overlap.
constexpr int kPThreads = 192;
constexpr int64_t kTcGroup = 8;        // column blocks per tile group of the persistent kernel
// The dynamic shared-memory limit set for tc_update_persistent<0> (one value
// for every launcher: the attribute is per kernel and device): a launch
// under an SM budget asks for all of it so no other CTA fits on its SMs.
constexpr size_t kTcExclusiveSmem = 200 * 1024;

__device__ __forceinline__ void tma_reduce_add_2d(const CUtensorMap* map, uint32_t src, int x, int y)
{
    asm volatile("cp.reduce.async.bulk.tensor.2d.global.shared::cta.add.tile.bulk_group [%0, {%2, %3}], [%1];"
                 :: "l"(reinterpret_cast<uint64_t>(map)), "r"(src), "r"(x), "r"(y) : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

__device__ __forceinline__ void bulk_wait_read_le1() { asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// BN: tile width, 128 or 256 (N of the MMA; two BN-column TMEM accumulators).
template <int KIND, int BN = kTcBN>
__global__ void __launch_bounds__(kPThreads, 1)
tc_update_persistent(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                     const __grid_constant__ CUtensorMap mapC, TcArgs a, uint32_t idesc)
{
    static_assert(BN == 128 || BN == 256, "tile width");
    constexpr int BM = kTcBM, S = kTcStages;
    constexpr int A_BYTES = BM * 128;
    constexpr int B_BYTES = BN * 128;
    constexpr int STAGE = A_BYTES + B_BYTES;
    constexpr int STG = 32 * 32 * 4;               // one 32 x 32 fp32 staging box
    extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
    const uint32_t raw = smem_u32(tc_smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;
    unsigned char* gbase = tc_smem_raw + (base - raw);
    float* stage_c = reinterpret_cast<float*>(gbase + S * STAGE);          // [4 warps][2][32*32]
    uint64_t* bars = reinterpret_cast<uint64_t*>(gbase + S * STAGE + 8 * STG);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * S + 4);
    __shared__ int s_abort;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t mt = ceildiv(a.m, BM), nt = ceildiv(a.n, BN);
    const int64_t ntiles = mt * nt;
    const int KT = int(a.kpad / kt_elems<KIND>());

    const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + S);
    const uint32_t tfull0 = smem_u32(bars + 2 * S), tempty0 = smem_u32(bars + 2 * S + 2);
    if (threadIdx.x == 0) {
        s_abort = 0;
        for (int s = 0; s < S; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(tfull0 + 8 * b, 1);
            mbar_init(tempty0 + 8 * b, 4);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 1) tmem_alloc(smem_u32(tmem_slot), 2 * BN);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t taddr = *tmem_slot;

    // Tile t -> (row block, column block) in groups of kTcGroup column
    // blocks: consecutive tiles walk the group's columns first, then its
    // rows, so the CTAs of one wave share a few A row blocks and a few B
    // column blocks in L2 instead of streaming every A row block again for
    // each column block.
    auto tile_rc = [&](int64_t t, int64_t& rb, int64_t& cb) {
        const int64_t per = kTcGroup * mt;
        const int64_t g = t / per, w = (nt - g * kTcGroup < kTcGroup) ? nt - g * kTcGroup : kTcGroup, q = t - g * per;
        cb = g * kTcGroup + q % w;
        rb = q / w;
    };
    auto skip = [&](int64_t t) {
        int64_t rb, cb;
        tile_rc(t, rb, cb);
        return a.lower && rb * BM + BM - 1 < cb * BN;
    };

    if (warp == 0) {
        if (lane == 0) {
            // ---- TMA producer
            long long it = 0;
            bool ok = true;
            for (int64_t t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
                if (skip(t)) continue;
                int64_t rb, cb;
                tile_rc(t, rb, cb);
                const int row0 = int(rb * BM), col0 = int(cb * BN);
                for (int kt = 0; kt < KT; ++kt, ++it) {
                    const int s = int(it % S);
                    const uint32_t par = uint32_t((it / S) & 1) ^ 1u;
                    if (!mbar_wait(empty0 + 8 * s, par) || *(volatile int*) &s_abort) {
                        atomicCAS(a.status, 0, SLT_ERR_TIMEOUT);
                        s_abort = 1;
                        ok = false;
                        break;
                    }
                    const uint32_t sa = base + s * STAGE, sb = sa + A_BYTES;
                    mbar_expect_tx(full0 + 8 * s, STAGE);
                    tma_load_2d(sa, &mapA, full0 + 8 * s, kt * kt_elems<KIND>(), row0);
                    tma_load_2d(sb, &mapB, full0 + 8 * s, kt * kt_elems<KIND>(), col0);
                }
            }
            // drain: the last armed phase of every stage must land before exit
            const long long issued = it;
            for (int s = 0; s < S && s < issued; ++s) {
                const long long last = s + ((issued - 1 - s) / S) * S;
                mbar_wait(full0 + 8 * s, uint32_t((last / S) & 1));
            }
        }
    }
    else if (warp == 1) {
        if (lane == 0) {
            // ---- MMA issuer
            long long it = 0;
            int lt = 0;
            for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
                if (skip(t)) continue;
                const int buf = lt & 1;
                const uint32_t upar = uint32_t((lt >> 1) & 1) ^ 1u;
                if (!mbar_wait(tempty0 + 8 * buf, upar) || *(volatile int*) &s_abort) {
                    atomicCAS(a.status, 0, SLT_ERR_TIMEOUT);
                    s_abort = 1;
                    break;
                }
                tc_fence_after();
                const uint32_t tacc = taddr + uint32_t(buf * BN);
                bool ok = true;
                for (int kt = 0; kt < KT; ++kt, ++it) {
                    const int s = int(it % S);
                    const uint32_t par = uint32_t((it / S) & 1);
                    if (!mbar_wait(full0 + 8 * s, par) || *(volatile int*) &s_abort) {
                        atomicCAS(a.status, 0, SLT_ERR_TIMEOUT);
                        s_abort = 1;
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t sa = base + s * STAGE, sb = sa + A_BYTES;
                    const uint64_t da = sw128_desc(sa), db = sw128_desc(sb);
                    #pragma unroll
                    for (int k = 0; k < 4; ++k)
                        umma<KIND>(tacc, da + uint64_t(2 * k), db + uint64_t(2 * k), idesc, (kt | k) != 0 ? 1u : 0u);
                    umma_commit(empty0 + 8 * s);
                }
                if (!ok) break;
                umma_commit(tfull0 + 8 * buf);
                ++lt;
            }
        }
    }
    else {
        // ---- epilogue warps 2..5: TMEM lane quarter q = warp % 4
        const int q = warp & 3;
        float* stg = stage_c + (warp - 2) * 2 * (32 * 32);
        int lt = 0, chunk = 0;
        bool prev_committed = true;     // did the previous chunk commit a bulk group?
        for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
            if (skip(t)) continue;
            const int buf = lt & 1;
            bool ready = mbar_wait(tfull0 + 8 * buf, uint32_t((lt >> 1) & 1));
            ready = __all_sync(0xffffffffu, ready) && !*(volatile int*) &s_abort;
            if (!ready) {
                if (lane == 0) { atomicCAS(a.status, 0, SLT_ERR_TIMEOUT); s_abort = 1; }
                break;
            }
            tc_fence_after();
            int64_t rbt, cbt;
            tile_rc(t, rbt, cbt);
            const int64_t row0 = rbt * BM, col0 = cbt * BN;
            const int64_t r = row0 + q * 32 + lane;
            const float f = tile_factor(a, row0, col0);
            #pragma unroll 1
            for (int cc = 0; cc < BN; cc += 32, ++chunk) {
                float v[32];
                tmem_ld32(taddr + (uint32_t(q * 32) << 16) + uint32_t(buf * BN + cc), v);
                float* sb = stg + (chunk & 1) * (32 * 32);
                // this buffer was last read by the group two chunks back: if the
                // previous chunk committed a group, allowing one pending group
                // leaves exactly that newer one in flight; otherwise wait for all
                if (lane == 0) {
                    if (prev_committed) bulk_wait_read_le1();
                    else asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
                }
                __syncwarp();
                #pragma unroll
                for (int i = 0; i < 32; ++i) {
                    const int64_t c = col0 + cc + i;
                    sb[i * 32 + lane] = (a.lower && r < c) ? 0.f : -(v[i] * f);
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                prev_committed = (row0 + q * 32 < a.m && col0 + cc < a.n);
                if (lane == 0 && prev_committed)
                    tma_reduce_add_2d(&mapC, smem_u32(sb), int(row0 + q * 32), int(col0 + cc));
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(tempty0 + 8 * buf);
            ++lt;
        }
        if (lane == 0) bulk_wait_all();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1) tmem_dealloc(taddr, 2 * BN);
}

// Cast + K-major packing: dst[r][c] (row stride kpad) = src element (r, c);
// TRANS: src is column-major rows x k (element (r, c) at src[r + c*ld]),
// else src "row" r is contiguous over c (element (r, c) at src[c + r*ld]).
// Zero fill up to rpad x kpad.
template <typename TO, bool TRANS>
__global__ void __launch_bounds__(256)
pack_kernel(int64_t rows, int64_t k, const float* __restrict__ src, int64_t ld, TO* __restrict__ dst,
            int64_t rpad, int64_t kpad)
{
    __shared__ float t[32][33];
    const int tx = threadIdx.x % 32, ty = threadIdx.x / 32;   // 32 x 8
    const int64_t r0 = int64_t(blockIdx.y) * 32, c0 = int64_t(blockIdx.x) * 32;
    if (TRANS) {
        for (int q = ty; q < 32; q += 8) {            // read column c0+q, rows r0+tx (coalesced)
            int64_t r = r0 + tx, c = c0 + q;
            t[q][tx] = (r < rows && c < k) ? src[r + c * ld] : 0.f;
        }
        __syncthreads();
        for (int q = ty; q < 32; q += 8) {            // write row r0+q, cols c0+tx (coalesced)
            int64_t r = r0 + q, c = c0 + tx;
            if (r < rpad && c < kpad) {
                float v = t[tx][q];
                if constexpr (sizeof(TO) == 4) {
                    uint32_t u;
                    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(u) : "f"(v));
                    dst[r * kpad + c] = __uint_as_float(u);
                }
                else {
                    dst[r * kpad + c] = TO(v);
                }
            }
        }
    }
    else {
        for (int q = ty; q < 32; q += 8) {
            int64_t r = r0 + q, c = c0 + tx;
            if (r < rpad && c < kpad) {
                float v = (r < rows && c < k) ? src[c + r * ld] : 0.f;
                if constexpr (sizeof(TO) == 4) {
                    uint32_t u;
                    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(u) : "f"(v));
                    dst[r * kpad + c] = __uint_as_float(u);
                }
                else {
                    dst[r * kpad + c] = TO(v);
                }
            }
        }
    }
}

// FP8 scales: one block per 128-row tile of an operand (element (r, c) at
// src[r + c ld] when TRANS, else src[c + r ld]); inv[t] = 1 / s[t].
template <bool TRANS>
__global__ void __launch_bounds__(256)
fp8_scale_kernel(int64_t rows, int64_t k, const float* __restrict__ src, int64_t ld, float* __restrict__ scale,
                 float* __restrict__ inv)
{
    __shared__ float red[8];
    const int64_t r0 = int64_t(blockIdx.x) * kTcBM;
    const int64_t nr = min64(kTcBM, rows - r0);
    float mx = 0.f;
    if (nr > 0)
        for (int64_t e = threadIdx.x; e < nr * k; e += 256) {
            const int64_t r = TRANS ? r0 + e % nr : r0 + e / k;
            const int64_t c = TRANS ? e / nr : e % k;
            const float v = fabsf(TRANS ? src[r + c * ld] : src[c + r * ld]);
            mx = v > mx ? v : mx;
        }
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < 8; ++w) mx = fmaxf(mx, red[w]);
        int e = 0;
        float sc = 1.f;
        if (mx > 0.f && isfinite(mx)) {
            frexpf(mx, &e);
            sc = ldexpf(1.f, 8 - e);
        }
        scale[blockIdx.x] = sc;
        inv[blockIdx.x] = 1.f / sc;
    }
}

// E4M3 K-major packing of s_t x (the tile's scale), as pack_kernel.
template <bool TRANS>
__global__ void __launch_bounds__(256)
pack_fp8_kernel(int64_t rows, int64_t k, const float* __restrict__ src, int64_t ld, uint8_t* __restrict__ dst,
                int64_t rpad, int64_t kpad, const float* __restrict__ scale)
{
    __shared__ float t[32][33];
    const int tx = threadIdx.x % 32, ty = threadIdx.x / 32;
    const int64_t r0 = int64_t(blockIdx.y) * 32, c0 = int64_t(blockIdx.x) * 32;
    const float sc = scale[r0 / kTcBM];               // 32-row blocks never straddle a 128-row tile
    if (TRANS) {
        for (int q = ty; q < 32; q += 8) {
            const int64_t r = r0 + tx, c = c0 + q;
            t[q][tx] = (r < rows && c < k) ? src[r + c * ld] : 0.f;
        }
        __syncthreads();
        for (int q = ty; q < 32; q += 8) {
            const int64_t r = r0 + q, c = c0 + tx;
            if (r < rpad && c < kpad) dst[r * kpad + c] = __nv_fp8_e4m3(t[tx][q] * sc).__x;
        }
    }
    else {
        for (int q = ty; q < 32; q += 8) {
            const int64_t r = r0 + q, c = c0 + tx;
            if (r < rpad && c < kpad) {
                const float v = (r < rows && c < k) ? src[c + r * ld] : 0.f;
                dst[r * kpad + c] = __nv_fp8_e4m3(v * sc).__x;
            }
        }
    }
}

// 3xTF32 packing: each K-major row holds three TF32 segments of kseg
// elements, [hi | hi | lo] for A (ROLE 0) and [hi | lo | hi] for op(B)^T
// (ROLE 1), hi = rna_tf32(x), lo = rna_tf32(x - hi), so that one TF32 GEMM
// over K' = 3 kseg accumulates A_hi B_hi + A_hi B_lo + A_lo B_hi: FP32 inputs
// to 22 bits, products exact, FP32 accumulation.
__device__ __forceinline__ float rna_tf32(float v)
{
    uint32_t u;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(u) : "f"(v));
    return __uint_as_float(u);
}

template <bool TRANS, int ROLE>
__global__ void __launch_bounds__(256)
pack3_kernel(int64_t rows, int64_t k, const float* __restrict__ src, int64_t ld, float* __restrict__ dst,
             int64_t rpad, int64_t kseg)
{
    __shared__ float t[32][33];
    const int tx = threadIdx.x % 32, ty = threadIdx.x / 32;
    const int64_t r0 = int64_t(blockIdx.y) * 32, c0 = int64_t(blockIdx.x) * 32;
    const int64_t kp = 3 * kseg;
    auto put = [&](int64_t r, int64_t c, float v) {
        const float hi = rna_tf32(v), lo = rna_tf32(v - hi);
        float* row = dst + r * kp;
        row[c] = ROLE == 0 ? hi : hi;
        row[kseg + c] = ROLE == 0 ? hi : lo;
        row[2 * kseg + c] = ROLE == 0 ? lo : hi;
    };
    if (TRANS) {
        for (int q = ty; q < 32; q += 8) {
            const int64_t r = r0 + tx, c = c0 + q;
            t[q][tx] = (r < rows && c < k) ? src[r + c * ld] : 0.f;
        }
        __syncthreads();
        for (int q = ty; q < 32; q += 8) {
            const int64_t r = r0 + q, c = c0 + tx;
            if (r < rpad && c < kseg) put(r, c, t[tx][q]);
        }
    }
    else {
        for (int q = ty; q < 32; q += 8) {
            const int64_t r = r0 + q, c = c0 + tx;
            if (r < rpad && c < kseg) put(r, c, (r < rows && c < k) ? src[c + r * ld] : 0.f);
        }
    }
}

// Rows [r0, m) x columns [c0, c1) of the column-major FP32 factor into the
// row-major 16-bit copy: dst[r * ldd + c] = round(src[r + c * lds]) for
// r >= c, zero above the diagonal.  32 x 32 tiles through shared memory
// (coalesced reads along rows, writes along columns).
// grid (ceil((c1 - c0) / 32), ceil((m - r0) / 32)), 256 threads.
template <typename TO>
__global__ void __launch_bounds__(256)
pack_rows_kernel(int64_t m, int64_t r0, int64_t c0, int64_t c1, const float* __restrict__ src, int64_t lds,
                 TO* __restrict__ dst, int64_t ldd)
{
    __shared__ float tl[32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int64_t rb = r0 + int64_t(blockIdx.y) * 32, cb = c0 + int64_t(blockIdx.x) * 32;
    for (int q = ty; q < 32; q += 8) {
        const int64_t row = rb + tx, col = cb + q;
        tl[q][tx] = (row < m && col < c1 && row >= col) ? src[row + col * lds] : 0.f;
    }
    __syncthreads();
    for (int q = ty; q < 32; q += 8) {
        const int64_t row = rb + q, col = cb + tx;
        if (row < m && col < c1) dst[row * ldd + col] = TO(tl[tx][q]);
    }
}

// ---------------------------------------------------------------------------
// Host side
static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
static std::once_flag g_encode_once;

static int get_encode()
{
    std::call_once(g_encode_once, [] {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &fn, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
        cudaGetLastError();
    });
    return g_encode ? SLT_OK : SLT_ERR_NOT_SUPPORTED;
}

// 2-D tiled map: inner dimension `inner` elements (contiguous), `outer` rows
// `stride_bytes` apart, box box_inner x box_outer.
int tma_map_2d(CUtensorMap* map, void* ptr, CUtensorMapDataType dt, int64_t inner, int64_t outer,
               int64_t stride_bytes, int box_inner, int box_outer, CUtensorMapSwizzle swz)
{
    if (get_encode()) return SLT_ERR_NOT_SUPPORTED;
    cuuint64_t dims[2] = {cuuint64_t(inner), cuuint64_t(outer)};
    cuuint64_t strides[1] = {cuuint64_t(stride_bytes)};
    cuuint32_t box[2] = {cuuint32_t(box_inner), cuuint32_t(box_outer)};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = g_encode(map, dt, 2, ptr, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, swz,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? SLT_OK : SLT_ERR_ARG;
}

// 2-D map over a packed operand: inner dim = kpad elements, outer = rpad rows,
// box = (128 bytes of K) x box_rows, 128B swizzle.
static int make_map(CUtensorMap* map, void* ptr, CUtensorMapDataType dt, int esize, int64_t kpad,
                    int64_t rpad, int box_rows)
{
    cuuint64_t dims[2] = {cuuint64_t(kpad), cuuint64_t(rpad)};
    cuuint64_t strides[1] = {cuuint64_t(kpad) * cuuint64_t(esize)};
    cuuint32_t box[2] = {cuuint32_t(128 / esize), cuuint32_t(box_rows)};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = g_encode(map, dt, 2, ptr, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? SLT_OK : SLT_ERR_ARG;
}

template <typename TO, bool TRANS>
static int launch_pack(int64_t rows, int64_t k, const float* src, int64_t ld, TO* dst, int64_t rpad,
                       int64_t kpad, cudaStream_t s)
{
    dim3 grid(unsigned(ceildiv(kpad, 32)), unsigned(ceildiv(rpad, 32)));
    pack_kernel<TO, TRANS><<<grid, 256, 0, s>>>(rows, k, src, ld, dst, rpad, kpad);
    count_launch();
    return slt_from_cuda(cudaGetLastError());
}

static size_t tc_smem_bytes()
{
    return size_t(kTcStages) * (kTcBM + kTcBN) * 128 + 1024 + 256;
}

static size_t tcp_smem_bytes(int bn = kTcBN)
{
    return size_t(kTcStages) * (kTcBM + bn) * 128 + 8 * 32 * 32 * 4 + 1024 + 256;
}

// fp32 column-major C: inner dim m (rows), outer n, box 32 x 32, no swizzle.
static int make_map_c(CUtensorMap* map, float* C, int64_t m, int64_t n, int64_t ldc)
{
    cuuint64_t dims[2] = {cuuint64_t(m), cuuint64_t(n)};
    cuuint64_t strides[1] = {cuuint64_t(ldc) * 4};
    cuuint32_t box[2] = {32, 32};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, C, dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                          CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? SLT_OK : SLT_ERR_ARG;
}

static int g_sms = 0;

// device status word for the tensor-core path (timeouts)
static int* g_tc_status = nullptr;

} // namespace slt

using namespace slt;

extern "C" size_t slt_tc_gemm_ws_bytes(int64_t m, int64_t n, int64_t k)
{
    int64_t kpad = ceildiv(k, 64) * 64;
    int64_t mp = ceildiv(m, kTcBM) * kTcBM, np = ceildiv(n, kTcBN) * kTcBN;
    return size_t(mp + np) * size_t(kpad) * 4 + 2048;
}

// C (fp32) -= A op(B), operands rounded to the tier's type.  transb 'N':
// B is k x n (column-major); 'T': B is n x k (C -= A B^T).  ws may be null
// (allocated from the stream-ordered pool).
extern "C" int slt_tc_gemm_update(int tier, char transb, int64_t m, int64_t n, int64_t k, const float* A,
                                  int64_t lda, const float* B, int64_t ldb, float* C, int64_t ldc, int lower,
                                  void* ws, size_t ws_bytes, cudaStream_t stream)
{
    if (m < 0 || n < 0 || k < 0 || (transb != 'N' && transb != 'T')) return SLT_ERR_ARG;
    if (tier != SLT_PREC_TF32 && tier != SLT_PREC_BF16 && tier != SLT_PREC_FP16 && tier != SLT_PREC_FP8 &&
        tier != SLT_PREC_TF32X3)
        return SLT_ERR_ARG;
    if (m == 0 || n == 0 || k == 0) return SLT_OK;
    int rc = get_encode();
    if (rc) return rc;
    if (!g_tc_status) {
        SLT_CUDA_TRY(cudaMalloc(&g_tc_status, sizeof(int)));
        SLT_CUDA_TRY(cudaMemset(g_tc_status, 0, sizeof(int)));
    }
    const bool x3 = tier == SLT_PREC_TF32X3;
    const bool tf32 = tier == SLT_PREC_TF32 || x3;
    const bool fp8 = tier == SLT_PREC_FP8;
    const int esize = tf32 ? 4 : fp8 ? 1 : 2;
    const int64_t kq = 128 / esize;                  // elements per 128-byte K tile
    const int64_t kseg = ceildiv(k, kq) * kq;        // one operand segment
    const int64_t kpad = x3 ? 3 * kseg : kseg;
    const int64_t mp = ceildiv(m, kTcBM) * kTcBM, np = ceildiv(n, kTcBN) * kTcBN;
    const int64_t mtl = mp / kTcBM, ntl = np / kTcBN;
    const size_t scale_bytes = fp8 ? sizeof(float) * 2 * size_t(mtl + ntl) + 256 : 0;
    const size_t need = size_t(mp + np) * size_t(kpad) * esize + 2048 + scale_bytes;
    DevBuf owned;          // the library's workspace pool (freed in stream order on return)
    if (!ws || ws_bytes < need) {
        TRY(owned.alloc(need, stream));
        ws = owned.p;
    }
    char* pa = static_cast<char*>(ws);
    char* pb = pa + ((size_t(mp) * kpad * esize + 1023) & ~size_t(1023));
    float* sA = reinterpret_cast<float*>(pb + ((size_t(np) * kpad * esize + 1023) & ~size_t(1023)));
    float* iA = sA + mtl;
    float* sB = iA + mtl;
    float* iB = sB + ntl;
    // pack operands
    if (x3) {
        dim3 ga(unsigned(ceildiv(kseg, 32)), unsigned(ceildiv(mp, 32)));
        dim3 gb(unsigned(ceildiv(kseg, 32)), unsigned(ceildiv(np, 32)));
        pack3_kernel<true, 0><<<ga, 256, 0, stream>>>(m, k, A, lda, reinterpret_cast<float*>(pa), mp, kseg);
        count_launch();
        if (transb == 'N')
            pack3_kernel<false, 1><<<gb, 256, 0, stream>>>(n, k, B, ldb, reinterpret_cast<float*>(pb), np, kseg);
        else
            pack3_kernel<true, 1><<<gb, 256, 0, stream>>>(n, k, B, ldb, reinterpret_cast<float*>(pb), np, kseg);
        count_launch();
        rc = slt_from_cuda(cudaGetLastError());
    }
    else if (fp8) {
        fp8_scale_kernel<true><<<unsigned(mtl), 256, 0, stream>>>(m, k, A, lda, sA, iA);
        count_launch();
        if (transb == 'N') fp8_scale_kernel<false><<<unsigned(ntl), 256, 0, stream>>>(n, k, B, ldb, sB, iB);
        else fp8_scale_kernel<true><<<unsigned(ntl), 256, 0, stream>>>(n, k, B, ldb, sB, iB);
        count_launch();
        dim3 ga(unsigned(ceildiv(kpad, 32)), unsigned(ceildiv(mp, 32)));
        dim3 gb(unsigned(ceildiv(kpad, 32)), unsigned(ceildiv(np, 32)));
        pack_fp8_kernel<true><<<ga, 256, 0, stream>>>(m, k, A, lda, reinterpret_cast<uint8_t*>(pa), mp, kpad, sA);
        count_launch();
        if (transb == 'N')
            pack_fp8_kernel<false><<<gb, 256, 0, stream>>>(n, k, B, ldb, reinterpret_cast<uint8_t*>(pb), np, kpad, sB);
        else
            pack_fp8_kernel<true><<<gb, 256, 0, stream>>>(n, k, B, ldb, reinterpret_cast<uint8_t*>(pb), np, kpad, sB);
        count_launch();
        rc = slt_from_cuda(cudaGetLastError());
    }
    else if (tier == SLT_PREC_BF16) {
        rc = launch_pack<__nv_bfloat16, true>(m, k, A, lda, reinterpret_cast<__nv_bfloat16*>(pa), mp, kpad, stream);
        if (!rc) rc = (transb == 'N')
            ? launch_pack<__nv_bfloat16, false>(n, k, B, ldb, reinterpret_cast<__nv_bfloat16*>(pb), np, kpad, stream)
            : launch_pack<__nv_bfloat16, true>(n, k, B, ldb, reinterpret_cast<__nv_bfloat16*>(pb), np, kpad, stream);
    }
    else if (tier == SLT_PREC_FP16) {
        rc = launch_pack<__half, true>(m, k, A, lda, reinterpret_cast<__half*>(pa), mp, kpad, stream);
        if (!rc) rc = (transb == 'N')
            ? launch_pack<__half, false>(n, k, B, ldb, reinterpret_cast<__half*>(pb), np, kpad, stream)
            : launch_pack<__half, true>(n, k, B, ldb, reinterpret_cast<__half*>(pb), np, kpad, stream);
    }
    else {
        rc = launch_pack<float, true>(m, k, A, lda, reinterpret_cast<float*>(pa), mp, kpad, stream);
        if (!rc) rc = (transb == 'N')
            ? launch_pack<float, false>(n, k, B, ldb, reinterpret_cast<float*>(pb), np, kpad, stream)
            : launch_pack<float, true>(n, k, B, ldb, reinterpret_cast<float*>(pb), np, kpad, stream);
    }
    if (!rc) {
        CUtensorMap mapA, mapB;
        CUtensorMapDataType dt = tier == SLT_PREC_BF16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16
                               : tier == SLT_PREC_FP16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16
                               : fp8                   ? CU_TENSOR_MAP_DATA_TYPE_UINT8
                                                       : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
        rc = make_map(&mapA, pa, dt, esize, kpad, mp, kTcBM);
        if (!rc) rc = make_map(&mapB, pb, dt, esize, kpad, np, kTcBN);
        if (!rc) {
            TcArgs args{m, n, kpad, C, ldc, lower, g_tc_status, fp8 ? iA : nullptr, fp8 ? iB : nullptr};
            const int pidx = prof_begin(SLT_PROF_GEMM_TC, stream);
            const bool tma_c = (reinterpret_cast<uintptr_t>(C) % 16 == 0) && (ldc % 4 == 0);
            CUtensorMap mapC;
            if (tma_c) rc = make_map_c(&mapC, C, m, n, ldc);
            if (rc) {
                // not reachable for aligned C; keep the status
            }
            else if (tma_c) {
                if (!g_sms) {
                    int dev = 0;
                    cudaGetDevice(&dev);
                    cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
                }
                const size_t psm = tcp_smem_bytes();
                const int64_t tiles = (mp / kTcBM) * (np / kTcBN);
                const unsigned grid1 = unsigned(std::min<int64_t>(tiles, capped_sms(g_sms)));
                if (tf32) {
                    SLT_SMEM_ONCE_INTO(rc, tc_update_persistent<1>, psm);
                    if (!rc) tc_update_persistent<1><<<grid1, kPThreads, psm, stream>>>(mapA, mapB, mapC, args, make_idesc(2, kTcBM, kTcBN));
                }
                else if (fp8) {
                    SLT_SMEM_ONCE_INTO(rc, tc_update_persistent<2>, psm);
                    if (!rc) tc_update_persistent<2><<<grid1, kPThreads, psm, stream>>>(mapA, mapB, mapC, args, make_idesc(0, kTcBM, kTcBN));
                }
                else {
                    SLT_SMEM_ONCE_INTO(rc, tc_update_persistent<0>, kTcExclusiveSmem);
                    const uint32_t fmt = tier == SLT_PREC_BF16 ? 1u : 0u;
                    if (!rc) tc_update_persistent<0><<<grid1, kPThreads, psm, stream>>>(mapA, mapB, mapC, args, make_idesc(fmt, kTcBM, kTcBN));
                }
            }
            else {
            const size_t smem = tc_smem_bytes();
            dim3 grid(unsigned(mp / kTcBM), unsigned(np / kTcBN));
            if (tf32) {
                SLT_SMEM_ONCE_INTO(rc, tc_update_kernel<1>, smem);
                if (!rc) tc_update_kernel<1><<<grid, kTcThreads, smem, stream>>>(mapA, mapB, args, make_idesc(2, kTcBM, kTcBN));
            }
            else if (fp8) {
                SLT_SMEM_ONCE_INTO(rc, tc_update_kernel<2>, smem);
                if (!rc) tc_update_kernel<2><<<grid, kTcThreads, smem, stream>>>(mapA, mapB, args, make_idesc(0, kTcBM, kTcBN));
            }
            else {
                SLT_SMEM_ONCE_INTO(rc, tc_update_kernel<0>, smem);
                const uint32_t fmt = tier == SLT_PREC_BF16 ? 1u : 0u;
                if (!rc) tc_update_kernel<0><<<grid, kTcThreads, smem, stream>>>(mapA, mapB, args, make_idesc(fmt, kTcBM, kTcBN));
            }
            }
            count_launch();
            if (!rc) rc = slt_from_cuda(cudaGetLastError());
            double mn = lower ? (double(m) * double(n) - (double(n) * double(n) - double(n)) / 2.0) : double(m) * double(n);
            prof_end(pidx, stream, 2.0 * mn * double(k), 8.0 * mn + double(esize) * double(kpad) * double(m + n));
        }
    }
    return rc;
}

// Status of the tensor-core path (SLT_ERR_TIMEOUT after an abandoned tile);
// reading clears it.
extern "C" int slt_tc_status(void)
{
    if (!g_tc_status) return SLT_OK;
    int h = 0;
    if (cudaMemcpy(&h, g_tc_status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return SLT_ERR_CUDA_BASE;
    if (h) cudaMemset(g_tc_status, 0, sizeof(int));
    return h;
}

// Rows [r0, m) x columns [c0, c1) of the lower FP32 factor L (column-major,
// leading dimension lds) into the row-major 16-bit copy L16 (row stride ldd
// elements; tier FP16 or BF16), zero above the diagonal.
extern "C" int slt_pack_rows16(int tier, int64_t m, int64_t r0, int64_t c0, int64_t c1, const float* src,
                               int64_t lds, void* dst, int64_t ldd, cudaStream_t stream)
{
    if (r0 >= m || c0 >= c1) return SLT_OK;
    dim3 grid(unsigned(ceildiv(c1 - c0, 32)), unsigned(ceildiv(m - r0, 32)));
    if (tier == SLT_PREC_FP16)
        pack_rows_kernel<__half><<<grid, 256, 0, stream>>>(m, r0, c0, c1, src, lds, static_cast<__half*>(dst), ldd);
    else if (tier == SLT_PREC_BF16)
        pack_rows_kernel<__nv_bfloat16><<<grid, 256, 0, stream>>>(m, r0, c0, c1, src, lds,
                                                                 static_cast<__nv_bfloat16*>(dst), ldd);
    else
        return SLT_ERR_ARG;
    count_launch();
    return slt_from_cuda(cudaGetLastError());
}

// C (fp32, m x n) -= A B^T on the tensor cores, A (m x kpad) and B (n x kpad)
// already in the tier's 16-bit type, K-major (row i of A at A16 + i lda16
// elements); kpad a multiple of 64, 16-byte aligned rows; C 16-byte aligned
// with ldc a multiple of 4.  lower: only C(i, j) with i >= j is updated.
extern "C" int slt_tc_gemm_packed(int tier, int64_t m, int64_t n, int64_t kpad, const void* A16, int64_t lda16,
                                  const void* B16, int64_t ldb16, float* C, int64_t ldc, int lower,
                                  cudaStream_t stream)
{
    if (tier != SLT_PREC_FP16 && tier != SLT_PREC_BF16) return SLT_ERR_ARG;
    if (m < 0 || n < 0 || kpad < 0) return SLT_ERR_ARG;
    if (m == 0 || n == 0 || kpad == 0) return SLT_OK;
    if (kpad % 64 || (lda16 * 2) % 16 || (ldb16 * 2) % 16 || reinterpret_cast<uintptr_t>(A16) % 16 ||
        reinterpret_cast<uintptr_t>(B16) % 16 || reinterpret_cast<uintptr_t>(C) % 16 || ldc % 4)
        return SLT_ERR_ARG;
    int rc = get_encode();
    if (rc) return rc;
    if (!g_tc_status) {
        SLT_CUDA_TRY(cudaMalloc(&g_tc_status, sizeof(int)));
        SLT_CUDA_TRY(cudaMemset(g_tc_status, 0, sizeof(int)));
    }
    const CUtensorMapDataType dt = tier == SLT_PREC_BF16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16
                                                         : CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
    CUtensorMap mapA, mapB, mapC;
    // 128 x 256 tiles: 48 KB of operands per 64-k stage for 4.2 MFLOP (128 x 128:
    // 32 KB for 2.1 MFLOP), so a third less shared-memory fill per flop
    constexpr int BN = 256;
    TRY(tma_map_2d(&mapA, const_cast<void*>(A16), dt, kpad, m, lda16 * 2, 64, kTcBM, CU_TENSOR_MAP_SWIZZLE_128B));
    TRY(tma_map_2d(&mapB, const_cast<void*>(B16), dt, kpad, n, ldb16 * 2, 64, BN, CU_TENSOR_MAP_SWIZZLE_128B));
    TRY(make_map_c(&mapC, C, m, n, ldc));
    if (!g_sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
    }
    TcArgs args{m, n, kpad, C, ldc, lower, g_tc_status, nullptr, nullptr};
    // ~225 KB of shared memory per CTA: one CTA per SM, and no other CTA of
    // this library fits beside it (what a launch under an SM budget needs)
    const size_t psm = tcp_smem_bytes(BN);
    SLT_SMEM_ONCE_INTO(rc, (tc_update_persistent<0, BN>), psm);
    if (rc) return rc;
    const int64_t tiles = ceildiv(m, kTcBM) * ceildiv(n, BN);
    const unsigned grid = unsigned(std::min<int64_t>(tiles, capped_sms(g_sms)));
    const int pidx = prof_begin(SLT_PROF_GEMM_TC, stream);
    tc_update_persistent<0, BN><<<grid, kPThreads, psm, stream>>>(mapA, mapB, mapC, args,
                                                                  make_idesc(tier == SLT_PREC_BF16 ? 1u : 0u, kTcBM, BN));
    count_launch();
    const double mn = lower ? (double(m) * double(n) - (double(n) * double(n) - double(n)) / 2.0) : double(m) * double(n);
    prof_end(pidx, stream, 2.0 * mn * double(kpad), 8.0 * mn + 2.0 * double(kpad) * double(m + n));
    return slt_from_cuda(cudaGetLastError());
}
