// digit_residual.cu -- the FP64 residual R = B - A X of the refinement loops
// on the BF16 tensor cores (tcgen05), for up to 16 right-hand sides.
//
// SLATE forms b - A x in double once per refinement step (gesv_mixed:
// src/gesv_mixed.cc:240-285, posv_mixed: src/posv_mixed.cc:230-290, and the
// Arnoldi products of gesv_mixed_gmres / posv_mixed_gmres,
// src/gesv_mixed_gmres.cc:250-330).  On GB300 FP64 arithmetic runs at about
// 1.2 TFLOP/s, so a 16-column product with A of order 65536 costs ~120 ms
// while one read of A costs 5 ms.  Here the product is formed on the tensor
// cores by splitting both operands into integer digits (the Ozaki scheme:
// Ozaki, Ogita, Oishi, Rump, Numer. Algorithms 59 (2012) 95-118; integer
// digits as in Ootomo, Ozaki, Yokota, IJHPCA 38 (2024)):
//
//  * row i of A is scaled by 2^-ea_i and column c of X by 2^-ex_c (powers of
//    two, exact) so that every |a'| and |x'| is below 1/2;
//  * a' is rounded to F = round(a' 2^56), |F| < 2^55, in int64 arithmetic on
//    the bits of the double, and F is split into eight balanced base-128
//    digits d_p in [-64, 64] (integers, exact in BF16):
//    a' = sum_{p<8} d_p 128^-(p+1) + r with |r| <= 2^-57;
//  * a' x' = sum_w S_w 128^-(w+2) with S_w = sum_k sum_{p+q=w} d_p d_q; the
//    weight classes w >= 8 lie below 2^-53 of the product scale and are
//    dropped, so 8 classes remain;
//  * the tensor cores form the class sums of one chunk of 1024 k in two FP32
//    accumulators (A planes 0-3 and 4-7), each taking at most four digit
//    pairs per class: every product is an integer of magnitude <= 2^12 and
//    every partial sum at most 1024 * 4 * 2^12 = 2^24, so FP32 accumulation
//    is exact in any order;
//  * per chunk the epilogue folds the class sums exactly into two int64
//    words, hi = sum_{w<4} S_w 2^(7(3-w)) and lo = sum_{w>=4} S_w 2^(7(7-w));
//    split-K segments add in int64 (exact), and the last kernel forms
//    r = (b - hi 2^(e-35)) - lo 2^(e-63), e = ea_i + ex_c.
//
// The computed A x differs from the exact one by at most about
// 2^-50 n max_k |a_ik| max_k |x_kc| (the dropped digits and classes), and
// typically by 2^-56 sqrt(n) of that scale: as accurate as an FP64 product.
//
// Layout in HBM.  The digit planes of A are bytes u = d + 64 in [0, 128],
// zero-padded (u = 64) to rows_pad = 128-multiple rows and ldk = 64-multiple
// columns: 8 n^2 bytes, the size of the FP64 matrix, written once per solve.
// They are stored as tiles of 128 rows x 64 k, the eight planes of one tile
// adjacent (64 KB), tiles of one row block in k order: a CTA streams its K
// segment as one contiguous run.  Within a plane tile row r holds its 64
// bytes at r * 64 with the 16-byte chunk j at position j ^ ((r >> 1) & 3)
// (the 64-byte swizzle, so that 32 threads reading 32 rows hit distinct
// banks).  The digits of X (per call) are 128 rows (plane q, column c at row
// 16 q + c) of ldk BF16.
//
// The MMA.  A CTA takes a 128-row block of A and a K segment.  Per 64 k, warp
// 0 loads the 64 KB byte tile of A with one bulk copy (three stages) and warp
// 10 the X digit tile (128 x 64 BF16, 128-byte swizzle) with TMA (two
// stages), each running ahead on its own ring.  Warps 6-9 (one TMEM lane
// quarter each; thread = row) turn the bytes into the BF16 digits
// in tensor memory: BF16 0x4300 | u is exactly 128 + u for every u in
// [0, 128] (u = 128 carries into the exponent: 0x4380 = 256), so one byte
// permute and one exact BF16x2 subtraction of 192 make two digits, stored
// with tcgen05.st.  Warp 1 issues,
// per 16 k and plane p, tcgen05.mma M128 N(128 - 16 p) K16 with A from
// tensor memory and B = X planes 0 .. 7 - p, accumulating class w = p + q
// into column 16 w + c of D_L (planes 0-3) or 16 (w - 4) + c of D_H (planes
// 4-7): the 36 digit products of weight <= 7 and no others, in two
// independent accumulator chains issued alternately.  The epilogue (warps
// 2-5) empties D once per 1024 k; the A operand has five 16-k stages.  Every
// mbarrier wait is bounded; on timeout the CTA records SLT_ERR_TIMEOUT,
// drains its own copies and MMAs, frees its TMEM and returns.

#include "common.cuh"
#include "drivers.h"
#include "prof.h"
#include "slate_gb300.h"
#include "tc_ptx.cuh"

#include <cuda.h>
#include <cuda_bf16.h>

#include <climits>

namespace slt {

constexpr int kDgPlanes = 8;          // digits per operand
constexpr int kDgBM = 128;            // rows of A per CTA (MMA M)
constexpr int kDgBK = 64;             // k per stage
constexpr int kDgChunk = 16;          // k-blocks per accumulator flush (1024 k)
constexpr int kDgUStages = 3;
constexpr int kDgXStages = 2;
constexpr int kDgThreads = 352;
constexpr int kDgCols = 16;           // right-hand sides per call
constexpr uint32_t kDgUPlane = kDgBM * kDgBK;          // 8 KB: one byte plane, 128 rows x 64 k
constexpr uint32_t kDgUStage = kDgPlanes * kDgUPlane;  // 64 KB
constexpr uint32_t kDgXStage = 128 * 128;              // 128 digit rows x 64 k BF16
// TMEM columns.  The accumulators are D_L (planes 0-3, classes 0-7: 128
// columns at 0) and D_H (planes 4-7, classes 4-7: 64 columns at 128): two
// independent accumulation chains, since consecutive MMAs into one
// accumulator run at one per ~130 clocks whatever N <= 128 is.  The A
// operand stages (16 k of 8 planes: 64 columns each) fill the other 320
// columns, so the operand warps run up to five stages ahead of the MMAs.
constexpr uint32_t kDgTmemH = 128;
constexpr uint32_t kDgTmemA = 192;
constexpr uint32_t kDgTmemAStage = 64;
constexpr int kDgAStagesT = 5;
constexpr int kDgASub = kDgBK / 16;                    // A operand stages per 64 k
static_assert(kDgTmemH + 64 <= kDgTmemA && kDgTmemA + kDgAStagesT * kDgTmemAStage <= 512,
              "D_L, D_H and the A operand stages fit the 512 TMEM columns");
static_assert(kDgAStagesT * kDgTmemAStage >= 2 * kDgTmemAStage, "at least two A operand stages");
static_assert(1024 + kDgUStages * kDgUStage + kDgXStages * kDgXStage + 256 + 1024 <= 232448,
              "stages, barriers and the static shared memory fit one CTA");
static_assert(kDgChunk * kDgBK * 4 * 64 * 64 <= (1 << 24), "FP32 class sums stay exact per chunk");
// Exponent keys.  key(v) = 0 for v = 0, 2047 for Inf / NaN, else
// max(biased exponent of v, 1); keys are monotone in |v|, and for the largest
// key K of a row, |v| < 2^(K - 1022) for every v of the row, so the scale
// exponent e = K - 1021 gives |v 2^-e| < 1/2.  Rows and columns keep the
// maximum key (atomicMax on a zeroed word).
constexpr int kDgBadKey = 2047;

__device__ __forceinline__ int dg_key(double v)
{
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v)) & 0x7fffffffffffffffull;
    if (b == 0) return 0;
    const int be = int(b >> 52);
    return be == 0 ? 1 : be;
}

__device__ __forceinline__ int dg_scale(int key) { return key == 0 ? 0 : key - 1021; }

// Maximum keys of the rows of A (general: over the whole row; sym, lower
// storage: over the stored part j <= i and, through the columns, over the
// part held in column i below the diagonal), kept with atomicMax on zeroed
// words.  Block: rows I0 .. I0 + 63 and four 64-column tiles from J0.
// grid (ceil(n / 256), ceil(n / 64)).
__global__ void __launch_bounds__(256)
dg_akeys_kernel(int64_t n, const double* __restrict__ A, int64_t lda, int sym, int* key)
{
    __shared__ int K[64][65];
    const int64_t I0 = int64_t(blockIdx.y) * 64;
    const int tx = threadIdx.x & 63, ty = threadIdx.x >> 6;
    int rmax = 0;
    for (int t = 0; t < 4; ++t) {
        const int64_t J0 = (int64_t(blockIdx.x) * 4 + t) * 64;
        if (J0 >= n || (sym && J0 > I0)) break;
        for (int kk = ty; kk < 64; kk += 4) {
            const int64_t i = I0 + tx, j = J0 + kk;
            K[tx][kk] = dg_key((i < n && j < n && !(sym && j > i)) ? A[i + j * lda] : 0.0);
        }
        __syncthreads();
        if (threadIdx.x < 64) {
            for (int c = 0; c < 64; ++c) rmax = max(rmax, K[threadIdx.x][c]);
        }
        else if (sym && threadIdx.x < 128) {
            const int c = threadIdx.x - 64;
            int cm = 0;
            for (int r = 0; r < 64; ++r) cm = max(cm, K[r][c]);
            if (cm && J0 + c < n) atomicMax(key + J0 + c, cm);
        }
        __syncthreads();
    }
    if (threadIdx.x < 64 && I0 + threadIdx.x < n && rmax) atomicMax(key + I0 + threadIdx.x, rmax);
}

// ||A||_inf from the split's exact row sums of |F| (F = round(a' 2^56), the
// fixed-point value of a' = a 2^-e of row i, e = dg_scale(key_i)), kept as
// two int64 words: sum |F| = h 2^28 + l.  Row sum = h 2^(e - 28) + l 2^(e - 56)
// (|a| and |F| 2^(e - 56) differ by at most 2^(e - 57)); NaN for a row holding
// Inf / NaN.  One block of 1024 threads.
__global__ void __launch_bounds__(1024)
dg_norm_kernel(int64_t n, const int* __restrict__ key, const unsigned long long* __restrict__ sh,
               const unsigned long long* __restrict__ sl, double* out)
{
    __shared__ double red[32];
    double m = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += 1024) {
        const int k = key[i];
        double v = 0.0;
        if (k == kDgBadKey) v = __longlong_as_double(0x7ff8000000000000ll);
        else if (k) v = ldexp(double(sh[i]), dg_scale(k) - 28) + ldexp(double(sl[i]), dg_scale(k) - 56);
        m = (v > m || v != v) ? v : m;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double y = __shfl_xor_sync(0xffffffffu, m, o);
        m = (y > m || y != y) ? y : m;
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < 32; ++w) m = (red[w] > m || red[w] != red[w]) ? red[w] : m;
        *out = m;
    }
}

// Maximum keys of the columns of an m x ncols column-major matrix.
// grid (ncols, segs), rps rows per segment.
__global__ void __launch_bounds__(256)
dg_colkeys_kernel(int64_t m, const double* __restrict__ X, int64_t ldx, int64_t rps, int* key)
{
    __shared__ int red[8];
    const int64_t c = blockIdx.x;
    const int64_t r0 = int64_t(blockIdx.y) * rps;
    const int64_t r1 = r0 + rps < m ? r0 + rps : m;
    int mx = 0;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += 256) mx = max(mx, dg_key(X[r + c * ldx]));
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < 8; ++w) mx = max(mx, red[w]);
        if (mx) atomicMax(key + c, mx);
    }
}

// F = round(v 2^(56 - e)), rounding half away from zero, for |v 2^-e| < 1/2:
// |F| < 2^55.  Integer arithmetic on the bits of v (FP64 instructions issue
// at a small fraction of the integer rate on this part).
__device__ __forceinline__ long long dg_fixed(double v, int e)
{
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v));
    const int be = int((b >> 52) & 0x7ff);
    long long m = static_cast<long long>(b & 0xFFFFFFFFFFFFFull);
    int x = -1074;                          // v = m 2^x
    if (be != 0) { m |= 1ll << 52; x = be - 1075; }
    const int sh = x - e + 56;
    long long F = 0;
    if (sh >= 0) F = m << sh;               // m 2^sh < 2^55, so sh < 55
    else if (sh > -64) F = (m + (1ll << (-sh - 1))) >> (-sh);
    return (b >> 63) ? -F : F;
}

// The eight balanced base-128 digits of F (d_0 most significant) as bytes
// u_p = d_p + 64: F = sum_p d_p 128^(7 - p), d_p in [-64, 63] for p >= 1 and
// d_0 in [-64, 64], so u_p in [0, 128].  With G = F + C7, C7 = 64 in each of
// the seven low base-128 places, u_p (p >= 1) is the 7-bit field of G and
// d_0 = G >> 49 -- taken with 32-bit shifts of G's two halves.  A key of 2047
// (Inf / NaN in the row or column) gives zero digits (u = 64); the
// reduction writes NaN for it.
constexpr long long kDgC7 = 0x1020408102040ll;

__device__ __forceinline__ long long dg_digit_bytes(double v, int key, uint32_t (&u)[kDgPlanes])
{
    const long long F = key == kDgBadKey ? 0 : dg_fixed(v, dg_scale(key));
    const long long G = F + kDgC7;
    const uint32_t lo = uint32_t(G), hi = uint32_t(static_cast<unsigned long long>(G) >> 32);
    u[7] = lo & 127u;
    u[6] = (lo >> 7) & 127u;
    u[5] = (lo >> 14) & 127u;
    u[4] = (lo >> 21) & 127u;
    u[3] = ((lo >> 28) | (hi << 4)) & 127u;
    u[2] = (hi >> 3) & 127u;
    u[1] = (hi >> 10) & 127u;
    u[0] = uint32_t((int(hi) >> 17) + 64);
    return F;
}

// Byte offset of (plane p, row i, k) in the tiled byte planes.
__device__ __forceinline__ int64_t dg_byte_at(int64_t i, int64_t k, int p, int64_t kbt)
{
    const int64_t tile = ((i >> 7) * kbt + (k >> 6)) * kDgPlanes + p;
    const int r = int(i & 127), j = int(k & 63);
    return tile * kDgUPlane + r * kDgBK + ((((j >> 4) ^ (r >> 1)) & 3) << 4) + (j & 15);
}

// Byte digit planes of A, kDgSplitTiles 64 x 64 blocks along k per CTA (rows
// I0.., k K0..); A column-major; with sym only its lower triangle is read
// (element (i, k), k > i, is A(k, i)).  Rows >= n and k >= n get the zero
// digit (u = 64).  With rsh / rsl (zeroed), also the exact row sums of |F|
// over k, as sum = rsh 2^28 + rsl (int64 atomics, order-free).
// grid (ceil(ldk / (64 kDgSplitTiles)), rows_pad / 64), 256 threads.
constexpr int kDgSplitTiles = 4;

__global__ void __launch_bounds__(256)
dg_split_a_kernel(int64_t n, const double* __restrict__ A, int64_t lda, int sym, const int* __restrict__ rexp,
                  uint8_t* planes, int64_t kbt, int64_t ldk, unsigned long long* rsh, unsigned long long* rsl)
{
    __shared__ double T[64][65];
    const int64_t I0 = int64_t(blockIdx.y) * 64;
    const int tx = threadIdx.x & 63, ty = threadIdx.x >> 6;
    const int kq = (threadIdx.x & 15) * 4;
    unsigned long long sh[4] = {0, 0, 0, 0}, sl[4] = {0, 0, 0, 0};   // rows r0 + 16 m
    for (int tile = 0; tile < kDgSplitTiles; ++tile) {
        const int64_t K0 = (int64_t(blockIdx.x) * kDgSplitTiles + tile) * 64;
        if (K0 >= ldk) break;
        if (tile) __syncthreads();                 // the previous block's reads of T
        if (sym && K0 > I0) {
            // strictly above the diagonal: element (i, k) = A(k, i), contiguous in k
            for (int ii = ty; ii < 64; ii += 4) {
                const int64_t i = I0 + ii, k = K0 + tx;
                T[ii][tx] = (i < n && k < n) ? A[k + i * lda] : 0.0;
            }
        }
        else {
            for (int kk = ty; kk < 64; kk += 4) {
                const int64_t i = I0 + tx, k = K0 + kk;
                T[tx][kk] = (i < n && k < n && !(sym && k > i)) ? A[i + k * lda] : 0.0;
            }
            if (sym && K0 == I0) {
                __syncthreads();
                for (int kk = ty; kk < 64; kk += 4)
                    if (kk > tx) T[tx][kk] = T[kk][tx];
            }
        }
        __syncthreads();
        #pragma unroll
        for (int m = 0; m < 4; ++m) {
            const int r = (threadIdx.x >> 4) + 16 * m;
            const int64_t i = I0 + r;
            const int key = i < n ? rexp[i] : 0;
            uint32_t w[kDgPlanes] = {0, 0, 0, 0, 0, 0, 0, 0};
            #pragma unroll
            for (int t = 0; t < 4; ++t) {
                uint32_t u[kDgPlanes];
                const long long F = dg_digit_bytes(T[r][kq + t], key, u);
                const unsigned long long a = static_cast<unsigned long long>(F < 0 ? -F : F);
                sh[m] += a >> 28;
                sl[m] += a & ((1ull << 28) - 1);
                #pragma unroll
                for (int p = 0; p < kDgPlanes; ++p) w[p] |= u[p] << (8 * t);
            }
            #pragma unroll
            for (int p = 0; p < kDgPlanes; ++p)
                *reinterpret_cast<uint32_t*>(planes + dg_byte_at(i, K0 + kq, p, kbt)) = w[p];
        }
    }
    if (rsh) {
        // the 16 threads of a row are 16 consecutive lanes
        #pragma unroll
        for (int m = 0; m < 4; ++m) {
            for (int o = 8; o > 0; o >>= 1) {
                sh[m] += __shfl_xor_sync(0xffffffffu, sh[m], o);
                sl[m] += __shfl_xor_sync(0xffffffffu, sl[m], o);
            }
            const int64_t i = I0 + (threadIdx.x >> 4) + 16 * m;
            if ((threadIdx.x & 15) == 0 && i < n && (sh[m] | sl[m])) {
                atomicAdd(rsh + i, sh[m]);
                atomicAdd(rsl + i, sl[m]);
            }
        }
    }
}

// Digits of X (n x nrhs, column-major) in BF16: plane q of column c at row
// 16 q + c of xd (128 rows of ldk), zeros for k >= n and c >= nrhs.
// grid (ldk / 1024, 16), 256 threads.
__global__ void __launch_bounds__(256)
dg_split_x_kernel(int64_t n, int nrhs, const double* __restrict__ X, int64_t ldx, const int* __restrict__ cexp,
                  __nv_bfloat16* xd, int64_t ldk)
{
    const int c = blockIdx.y;
    const int64_t k = (int64_t(blockIdx.x) * 256 + threadIdx.x) * 4;
    if (k >= ldk) return;
    const int key = c < nrhs ? cexp[c] : 0;
    int d[4][kDgPlanes];
    #pragma unroll
    for (int t = 0; t < 4; ++t) {
        const double v = (c < nrhs && k + t < n) ? X[k + t + int64_t(c) * ldx] : 0.0;
        uint32_t u[kDgPlanes];
        dg_digit_bytes(v, key, u);
        #pragma unroll
        for (int q = 0; q < kDgPlanes; ++q) d[t][q] = int(u[q]) - 64;
    }
    #pragma unroll
    for (int q = 0; q < kDgPlanes; ++q) {
        const __nv_bfloat162 a = __floats2bfloat162_rn(float(d[0][q]), float(d[1][q]));
        const __nv_bfloat162 b = __floats2bfloat162_rn(float(d[2][q]), float(d[3][q]));
        uint2 o;
        o.x = *reinterpret_cast<const uint32_t*>(&a);
        o.y = *reinterpret_cast<const uint32_t*>(&b);
        *reinterpret_cast<uint2*>(xd + int64_t(q * kDgCols + c) * ldk + k) = o;
    }
}

struct DgArgs {
    const uint8_t* planes;  // tiled byte planes
    int64_t rows_pad;       // rows of one A plane
    int rb;                 // 128-row blocks
    int kb_total;           // 64-k blocks
    int kb_per_seg;
    int segs;
    long long* part;        // [segs][2][16][rows_pad]: hi, lo
    int* status;
};

__device__ __forceinline__ void dg_fail(int* status, volatile int* abort_flag)
{
    atomicCAS(status, 0, SLT_ERR_TIMEOUT);
    *abort_flag = 1;
}

// The BF16 digits u - 64 of bytes 2j, 2j + 1 of w (j = 0, 1): the byte
// permute forms 128 + u, the subtraction of 192 (0x4340) is exact.
__device__ __forceinline__ uint32_t dg_bf16x2_sub192(uint32_t x)
{
    __nv_bfloat162 v = *reinterpret_cast<const __nv_bfloat162*>(&x);
    const uint32_t c = 0x43404340u;
    v = __hsub2(v, *reinterpret_cast<const __nv_bfloat162*>(&c));
    return *reinterpret_cast<const uint32_t*>(&v);
}

__device__ __forceinline__ void dg_expand(uint32_t w, uint32_t& o0, uint32_t& o1)
{
    o0 = dg_bf16x2_sub192(__byte_perm(w, 0x43434343u, 0x4140));
    o1 = dg_bf16x2_sub192(__byte_perm(w, 0x43434343u, 0x4342));
}

__global__ void __launch_bounds__(kDgThreads, 1)
dg_gemm_kernel(const __grid_constant__ CUtensorMap mapX, DgArgs a)
{
    constexpr int US = kDgUStages, XS = kDgXStages;
    extern __shared__ __align__(1024) unsigned char dg_smem_raw[];
    const uint32_t raw = smem_u32(dg_smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;
    unsigned char* gbase = dg_smem_raw + (base - raw);
    const uint32_t u0 = base, x0 = base + US * kDgUStage;
    uint64_t* bars = reinterpret_cast<uint64_t*>(gbase + US * kDgUStage + XS * kDgXStage);
    constexpr int AS = kDgAStagesT;
    // ufull[US] uempty[US] xfull[XS] xempty[XS] afull[AS] aempty[AS] tfull tempty fin
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * US + 2 * XS + 2 * AS + 3);
    __shared__ int s_abort;
    volatile int* abort_flag = &s_abort;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t ufull0 = smem_u32(bars), uempty0 = ufull0 + 8 * US;
    const uint32_t xfull0 = uempty0 + 8 * US, xempty0 = xfull0 + 8 * XS;
    const uint32_t afull0 = xempty0 + 8 * XS, aempty0 = afull0 + 8 * AS;
    const uint32_t tfull = aempty0 + 8 * AS, tempty = tfull + 8, fin = tempty + 8;
    const int64_t items = int64_t(a.rb) * a.segs;

    if (threadIdx.x == 0) {
        s_abort = 0;
        for (int s = 0; s < US; ++s) { mbar_init(ufull0 + 8 * s, 1); mbar_init(uempty0 + 8 * s, 4); }
        for (int s = 0; s < XS; ++s) { mbar_init(xfull0 + 8 * s, 1); mbar_init(xempty0 + 8 * s, 1); }
        for (int b = 0; b < AS; ++b) {
            mbar_init(afull0 + 8 * b, 4);
            mbar_init(aempty0 + 8 * b, 1);
        }
        mbar_init(tfull, 1);
        mbar_init(tempty, 4);
        mbar_init(fin, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) tmem_alloc(smem_u32(tmem_slot), 512);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t taddr = *tmem_slot;

    if (warp == 0 || warp == 10) {
        if (lane == 0) {
            // ---- producers: warp 0 streams the byte tiles of A (bulk copies),
            // warp 10 the X digit tiles (TMA), each as far ahead as its ring
            // allows
            const bool isx = warp == 10;
            const int NS = isx ? XS : US;
            const uint32_t full0 = isx ? xfull0 : ufull0, empty0 = isx ? xempty0 : uempty0;
            int st = 0;
            uint32_t ph = 0;
            long long issued = 0;
            bool ok = true;
            for (int64_t t = blockIdx.x; t < items && ok; t += gridDim.x) {
                const int row0 = int(t % a.rb) * kDgBM;
                const int seg = int(t / a.rb);
                const int kb0 = seg * a.kb_per_seg, kb1 = min(a.kb_total, kb0 + a.kb_per_seg);
                for (int kb = kb0; kb < kb1; ++kb) {
                    if (!mbar_wait(empty0 + 8 * st, ph ^ 1u) || *abort_flag) {
                        dg_fail(a.status, abort_flag);
                        ok = false;
                        break;
                    }
                    if (isx) {
                        mbar_expect_tx(full0 + 8 * st, kDgXStage);
                        tma_load_2d(x0 + st * kDgXStage, &mapX, full0 + 8 * st, kb * kDgBK, 0);
                    }
                    else {
                        mbar_expect_tx(full0 + 8 * st, kDgUStage);
                        bulk_load(u0 + st * kDgUStage,
                                  a.planes + (int64_t(row0 / kDgBM) * a.kb_total + kb) * int64_t(kDgUStage),
                                  kDgUStage, full0 + 8 * st);
                    }
                    ++issued;
                    if (++st == NS) { st = 0; ph ^= 1u; }
                }
            }
            // drain: the last armed phase of every stage lands before exit
            for (int s = 0; s < NS && s < issued; ++s) {
                const long long last = s + ((issued - 1 - s) / NS) * NS;
                mbar_wait(full0 + 8 * s, uint32_t((last / NS) & 1));
            }
        }
    }
    else if (warp == 1) {
        // ---- MMA issuer: the whole warp runs the loop (operands stay in
        // uniform registers), lane 0 issues the tcgen05 instructions
        const uint32_t lead = lane == 0 ? 1u : 0u;
        int as = 0, xs = 0;
        uint32_t aph = 0, xph = 0;
        long long lt = 0;
        bool ok = true;
        for (int64_t t = blockIdx.x; t < items && ok; t += gridDim.x) {
            const int seg = int(t / a.rb);
            const int kb0 = seg * a.kb_per_seg, kb1 = min(a.kb_total, kb0 + a.kb_per_seg);
            for (int kc = kb0; kc < kb1 && ok; kc += kDgChunk, ++lt) {
                ok = __all_sync(0xffffffffu, mbar_wait(tempty, uint32_t(lt & 1) ^ 1u) && !*abort_flag);
                if (!ok) break;
                tc_fence_after();
                const uint32_t tl = taddr;
                const int kend = min(kb1, kc + kDgChunk);
                for (int kb = kc; kb < kend && ok; ++kb) {
                    ok = __all_sync(0xffffffffu, mbar_wait(xfull0 + 8 * xs, xph) && !*abort_flag);
                    if (!ok) break;
                    tc_fence_after();
                    const uint64_t dx = sw128_desc(x0 + uint32_t(xs) * kDgXStage);
                    for (int h = 0; h < kDgASub; ++h) {
                        ok = __all_sync(0xffffffffu, mbar_wait(afull0 + 8 * as, aph) && !*abort_flag);
                        if (!ok) break;
                        tc_fence_after();
                        const uint32_t ta = taddr + kDgTmemA + uint32_t(as) * kDgTmemAStage;
                        const uint32_t first = (kb == kc && h == 0) ? 0u : 1u;
                        #pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            // plane j into D_L from column 16 j, plane j + 4 into D_H
                            // from column 16 j; B = X planes 0 .. 7 - p
                            umma_ta_w(tl + uint32_t(16 * j), ta + uint32_t(8 * j), dx + uint64_t(2 * h),
                                      make_idesc(1u, kDgBM, 128 - 16 * j), j == 0 ? first : 1u, lead);
                            umma_ta_w(taddr + kDgTmemH + uint32_t(16 * j), ta + uint32_t(8 * (j + 4)),
                                      dx + uint64_t(2 * h), make_idesc(1u, kDgBM, 64 - 16 * j),
                                      j == 0 ? first : 1u, lead);
                        }
                        umma_commit_w(aempty0 + 8 * as, lead);
                        if (++as == AS) { as = 0; aph ^= 1u; }
                    }
                    if (!ok) break;
                    umma_commit_w(xempty0 + 8 * xs, lead);
                    if (++xs == XS) { xs = 0; xph ^= 1u; }
                }
                if (!ok) break;
                umma_commit_w(tfull, lead);
            }
        }
        if (!ok && lane == 0) dg_fail(a.status, abort_flag);
        // every MMA issued above has completed before TMEM is freed
        umma_commit_w(fin, lead);
        if (lane == 0 && !mbar_wait(fin, 0u)) atomicCAS(a.status, 0, SLT_ERR_TIMEOUT);
        __syncwarp();
    }
    else if (warp >= 6) {
        // ---- operand warps 6..9: TMEM lanes 32 q .. 32 q + 31, q = warp % 4;
        // thread = row of the 128-row block
        const int q = warp & 3;
        const int row = q * 32 + lane;
        const uint32_t sw = uint32_t((row >> 1) & 3);          // 64-byte swizzle of the byte tiles
        const uint32_t tlane = taddr + (uint32_t(q * 32) << 16) + kDgTmemA;
        int us = 0, as = 0;
        uint32_t uph = 0, aph = 0;
        bool ok = true;
        for (int64_t t = blockIdx.x; t < items && ok; t += gridDim.x) {
            const int seg = int(t / a.rb);
            const int kb0 = seg * a.kb_per_seg, kb1 = min(a.kb_total, kb0 + a.kb_per_seg);
            for (int kb = kb0; kb < kb1 && ok; ++kb) {
                bool ready = mbar_wait(ufull0 + 8 * us, uph);
                ready = __all_sync(0xffffffffu, ready && !*abort_flag);
                if (!ready) {
                    if (lane == 0) dg_fail(a.status, abort_flag);
                    ok = false;
                    break;
                }
                const unsigned char* urow = gbase + us * kDgUStage + row * kDgBK;
                for (int h = 0; h < kDgASub; ++h) {
                    bool free_ = mbar_wait(aempty0 + 8 * as, aph ^ 1u);
                    free_ = __all_sync(0xffffffffu, free_ && !*abort_flag);
                    if (!free_) {
                        if (lane == 0) dg_fail(a.status, abort_flag);
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    #pragma unroll 4
                    for (int p = 0; p < kDgPlanes; ++p) {
                        const uint4 w = *reinterpret_cast<const uint4*>(urow + p * kDgUPlane +
                                                                        ((uint32_t(h) ^ sw) << 4));
                        uint32_t o[8];
                        dg_expand(w.x, o[0], o[1]);
                        dg_expand(w.y, o[2], o[3]);
                        dg_expand(w.z, o[4], o[5]);
                        dg_expand(w.w, o[6], o[7]);
                        tmem_st8(tlane + uint32_t(as) * kDgTmemAStage + uint32_t(8 * p), o);
                    }
                    tmem_st_wait();
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(afull0 + 8 * as);
                    if (++as == AS) { as = 0; aph ^= 1u; }
                }
                if (!ok) break;
                __syncwarp();
                if (lane == 0) mbar_arrive(uempty0 + 8 * us);
                if (++us == US) { us = 0; uph ^= 1u; }
            }
        }
    }
    else {
        // ---- epilogue warps 2..5: TMEM lanes 32 q .. 32 q + 31, q = warp % 4
        const int q = warp & 3;
        long long lt = 0;
        bool ok = true;
        for (int64_t t = blockIdx.x; t < items && ok; t += gridDim.x) {
            const int row0 = int(t % a.rb) * kDgBM;
            const int seg = int(t / a.rb);
            const int kb0 = seg * a.kb_per_seg, kb1 = min(a.kb_total, kb0 + a.kb_per_seg);
            long long hi[kDgCols], lo[kDgCols];
            #pragma unroll
            for (int c = 0; c < kDgCols; ++c) { hi[c] = 0; lo[c] = 0; }
            for (int kc = kb0; kc < kb1; kc += kDgChunk, ++lt) {
                bool ready = mbar_wait(tfull, uint32_t(lt & 1));
                ready = __all_sync(0xffffffffu, ready && !*abort_flag);
                if (!ready) {
                    if (lane == 0) dg_fail(a.status, abort_flag);
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t tq = taddr + (uint32_t(q * 32) << 16);
                #pragma unroll 1
                for (int g = 0; g < 6; ++g) {     // D_L classes 2h, 2h + 1 (g = h < 4), then D_H classes 4 .. 7
                    const int h = g < 4 ? g : g - 2;
                    float v[32];
                    tmem_ld32(tq + (g < 4 ? uint32_t(h * 32) : kDgTmemH + uint32_t((g - 4) * 32)), v);
                    // class w weighs 2^(7(3-w)) in hi (w < 4), 2^(7(7-w)) in lo
                    const long long m0 = (h & 1) ? (1ll << 7) : (1ll << 21);
                    const long long m1 = (h & 1) ? 1ll : (1ll << 14);
                    #pragma unroll
                    for (int c = 0; c < kDgCols; ++c) {
                        // |v| <= 2^24: exact in int32
                        const long long f = (long long) __float2int_rn(v[c]) * m0 +
                                            (long long) __float2int_rn(v[16 + c]) * m1;
                        if (h < 2) hi[c] += f;
                        else lo[c] += f;
                    }
                }
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(tempty);
            }
            if (!ok) break;
            const int64_t r = int64_t(row0) + q * 32 + lane;
            long long* ph = a.part + (int64_t(seg) * 2 * kDgCols) * a.rows_pad + r;
            #pragma unroll
            for (int c = 0; c < kDgCols; ++c) {
                ph[int64_t(c) * a.rows_pad] = hi[c];
                ph[int64_t(kDgCols + c) * a.rows_pad] = lo[c];
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1) tmem_dealloc(taddr, 512);
}

// R(i, c) = B(i, c) - sum over segments of (hi 2^(e-35) + lo 2^(e-63)),
// e = ea_i + ex_c; NaN where row i of A or column c of X holds Inf / NaN.
// grid (ceil(n / 256), nrhs).
__global__ void __launch_bounds__(256)
dg_reduce_kernel(int64_t n, int64_t rows_pad, int segs, const long long* __restrict__ part,
                 const int* __restrict__ rexp, const int* __restrict__ cexp, const double* __restrict__ B,
                 int64_t ldb, double* R, int64_t ldr)
{
    const int64_t i = int64_t(blockIdx.x) * 256 + threadIdx.x;
    const int c = blockIdx.y;
    if (i >= n) return;
    long long hi = 0, lo = 0;
    for (int s = 0; s < segs; ++s) {
        const long long* p = part + (int64_t(s) * 2 * kDgCols + c) * rows_pad + i;
        hi += p[0];
        lo += p[int64_t(kDgCols) * rows_pad];
    }
    double r;
    if (rexp[i] == kDgBadKey || cexp[c] == kDgBadKey) {
        r = __longlong_as_double(0x7ff8000000000000ll);
    }
    else {
        const int e = dg_scale(rexp[i]) + dg_scale(cexp[c]);
        const double yh = double(hi);
        // hi - yh is exact in int64 whenever |yh| < 2^62; fold it into lo
        if (fabs(yh) < 4.611686018427387904e18) lo += (hi - (long long) yh) * (1ll << 28);
        r = (B[i + c * ldb] - ldexp(yh, e - 35)) - ldexp(double(lo), e - 63);
    }
    R[i + c * ldr] = r;
}

static size_t dg_smem_bytes()
{
    return 1024 + size_t(kDgUStages) * kDgUStage + size_t(kDgXStages) * kDgXStage + 256;
}

// Split-K segments: the count that minimises waves x (k-blocks per item + 2).
static void dg_plan(int64_t rb, int64_t kb_total, int sms, int* segs, int* kps)
{
    double best = -1;
    *segs = 1;
    *kps = int(kb_total);
    for (int64_t s = 1; s <= std::min<int64_t>(kb_total, 64); ++s) {
        const int64_t k = ceildiv(kb_total, s);
        const int64_t se = ceildiv(kb_total, k);
        const int64_t waves = ceildiv(rb * se, int64_t(sms));
        const double cost = double(waves) * double(k + 2);
        if (best < 0 || cost < best) { best = cost; *segs = int(se); *kps = int(k); }
    }
}

size_t DigitMatrix::bytes_for(int64_t n)
{
    const int64_t ldk = ceildiv(n, kDgBK) * kDgBK, rp = ceildiv(n, kDgBM) * kDgBM;
    return size_t(kDgPlanes) * size_t(rp) * size_t(ldk);
}

void DigitMatrix::release()
{
    planes.reset();
    rexp.reset();
    cexp.reset();
    xplanes.reset();
    part.reset();
    status.reset();
    ready = false;
}

int DigitMatrix::prepare(int64_t n_, const double* A, int64_t lda, int sym, cudaStream_t s, double* d_norm)
{
    release();
    if (n_ <= 0 || lda < n_) return SLT_ERR_ARG;
    // grid rows (rows_pad / 64 <= 65535) and 32-bit TMA row coordinates
    if (n_ > (int64_t(1) << 22)) return SLT_ERR_NOT_SUPPORTED;
    n = n_;
    ldk = ceildiv(n, kDgBK) * kDgBK;
    rows_pad = ceildiv(n, kDgBM) * kDgBM;
    int dev = 0, nsm = 0;
    SLT_CUDA_TRY(cudaGetDevice(&dev));
    SLT_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    sms = capped_sms(nsm);
    dg_plan(rows_pad / kDgBM, ldk / kDgBK, sms, &segs, &kb_per_seg);
    TRY(planes.alloc(bytes_for(n), s));
    TRY(rexp.alloc(sizeof(int) * size_t(rows_pad), s));
    TRY(cexp.alloc(sizeof(int) * kDgCols, s));
    TRY(xplanes.alloc(size_t(kDgPlanes) * kDgCols * size_t(ldk) * 2, s));
    TRY(part.alloc(size_t(segs) * 2 * kDgCols * size_t(rows_pad) * sizeof(long long), s));
    TRY(status.alloc(sizeof(int), s));
    SLT_CUDA_TRY(cudaMemsetAsync(status.p, 0, sizeof(int), s));
    SLT_CUDA_TRY(cudaMemsetAsync(rexp.p, 0, sizeof(int) * size_t(rows_pad), s));

    // row keys: one pass over the stored part of A (integer work only)
    dg_akeys_kernel<<<dim3(unsigned(ceildiv(n, 256)), unsigned(ceildiv(n, 64))), 256, 0, s>>>(n, A, lda, sym,
                                                                                          rexp.as<int>());
    count_launch();
    // the split also sums |F| per row, for the infinity norm
    DevBuf rsh, rsl;
    if (d_norm) {
        TRY(rsh.alloc(sizeof(unsigned long long) * size_t(n), s));
        TRY(rsl.alloc(sizeof(unsigned long long) * size_t(n), s));
        SLT_CUDA_TRY(cudaMemsetAsync(rsh.p, 0, sizeof(unsigned long long) * size_t(n), s));
        SLT_CUDA_TRY(cudaMemsetAsync(rsl.p, 0, sizeof(unsigned long long) * size_t(n), s));
    }
    dg_split_a_kernel<<<dim3(unsigned(ceildiv(ldk, int64_t(64 * kDgSplitTiles))), unsigned(rows_pad / 64)), 256, 0, s>>>(
        n, A, lda, sym, rexp.as<int>(), planes.as<uint8_t>(), ldk / kDgBK, ldk,
        d_norm ? rsh.as<unsigned long long>() : nullptr, d_norm ? rsl.as<unsigned long long>() : nullptr);
    count_launch();
    if (d_norm) {
        dg_norm_kernel<<<1, 1024, 0, s>>>(n, rexp.as<int>(), rsh.as<unsigned long long>(),
                                           rsl.as<unsigned long long>(), d_norm);
        count_launch();
    }
    SLT_CUDA_TRY(cudaGetLastError());

    TRY(tma_map_2d(&mapX, xplanes.p, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, ldk, int64_t(kDgPlanes) * kDgCols,
                   ldk * 2, kDgBK, kDgPlanes * kDgCols, CU_TENSOR_MAP_SWIZZLE_128B));
    ready = true;
    return SLT_OK;
}

int DigitMatrix::residual(int64_t nrhs, const double* B, int64_t ldb, const double* X, int64_t ldx, double* R,
                          int64_t ldr, cudaStream_t s)
{
    if (!ready) return SLT_ERR_ARG;
    if (nrhs <= 0) return SLT_OK;
    if (nrhs > kDgCols || ldb < n || ldx < n || ldr < n) return SLT_ERR_ARG;
    static DeviceOnce once;
    TRY(once.run([] {
        return slt_from_cuda(cudaFuncSetAttribute(dg_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                  int(dg_smem_bytes())));
    }));
    SLT_CUDA_TRY(cudaMemsetAsync(cexp.p, 0, sizeof(int) * kDgCols, s));
    const int64_t rps = 16384;
    dg_colkeys_kernel<<<dim3(unsigned(nrhs), unsigned(ceildiv(n, rps))), 256, 0, s>>>(n, X, ldx, rps,
                                                                                    cexp.as<int>());
    count_launch();
    dg_split_x_kernel<<<dim3(unsigned(ceildiv(ldk, 1024)), kDgCols), 256, 0, s>>>(
        n, int(nrhs), X, ldx, cexp.as<int>(), xplanes.as<__nv_bfloat16>(), ldk);
    count_launch();

    DgArgs args{planes.as<uint8_t>(), rows_pad, int(rows_pad / kDgBM), int(ldk / kDgBK), kb_per_seg, segs, part.as<long long>(),
                status.as<int>()};
    const int64_t items = int64_t(args.rb) * segs;
    const unsigned grid = unsigned(std::min<int64_t>(items, sms));
    const int pidx = prof_begin(SLT_PROF_DIGIT, s);
    dg_gemm_kernel<<<grid, kDgThreads, dg_smem_bytes(), s>>>(mapX, args);
    count_launch();
    // algorithmic: 2 n^2 nrhs flops of the FP64 product; bytes: the digit planes of A
    prof_end(pidx, s, 2.0 * double(n) * double(n) * double(nrhs), double(bytes_for(n)));
    SLT_CUDA_TRY(cudaGetLastError());
    dg_reduce_kernel<<<dim3(unsigned(ceildiv(n, 256)), unsigned(nrhs)), 256, 0, s>>>(
        n, rows_pad, segs, part.as<long long>(), rexp.as<int>(), cexp.as<int>(), B, ldb, R, ldr);
    count_launch();
    return slt_from_cuda(cudaGetLastError());
}

int DigitMatrix::check_status(cudaStream_t s)
{
    if (!status.p) return SLT_OK;
    int h = 0;
    SLT_CUDA_TRY(cudaMemcpyAsync(&h, status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    SLT_CUDA_TRY(cudaStreamSynchronize(s));
    return h;
}

} // namespace slt

using namespace slt;

// One-shot digit residual (prepare, one product, status): R = B - A X for
// nrhs <= 16, A of order n (sym_lower: symmetric, lower storage); with
// d_norm (device, optional), also ||A||_inf from the split's exact integer
// row sums -- the norm the mixed solvers' stopping test uses.  The drivers
// keep the digit planes for a whole solve instead.
extern "C" int slt_dresidual_digits_norm(int64_t n, int64_t nrhs, const double* A, int64_t lda, int sym_lower,
                                         const double* B, int64_t ldb, const double* X, int64_t ldx, double* R,
                                         int64_t ldr, double* d_norm, cudaStream_t stream)
{
    if (n < 0 || nrhs < 0 || nrhs > kDgCols) return SLT_ERR_ARG;
    if (n == 0) return d_norm ? slt_from_cuda(cudaMemsetAsync(d_norm, 0, sizeof(double), stream)) : SLT_OK;
    if (nrhs == 0 && !d_norm) return SLT_OK;
    DigitMatrix dm;
    TRY(dm.prepare(n, A, lda, sym_lower, stream, d_norm));
    if (nrhs) TRY(dm.residual(nrhs, B, ldb, X, ldx, R, ldr, stream));
    return dm.check_status(stream);
}

extern "C" int slt_dresidual_digits(int64_t n, int64_t nrhs, const double* A, int64_t lda, int sym_lower,
                                    const double* B, int64_t ldb, const double* X, int64_t ldx, double* R,
                                    int64_t ldr, cudaStream_t stream)
{
    return slt_dresidual_digits_norm(n, nrhs, A, lda, sym_lower, B, ldb, X, ldx, R, ldr, nullptr, stream);
}
