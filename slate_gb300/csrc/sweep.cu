// sweep.cu -- one-launch triangular solves for few right-hand sides.
//
// Replaces the per-tile trsm + gemm sweeps of SLATE's getrs/potrs
// (work::trsmA, src/work/work_trsmA.cc:147-480; internal::trsmA/gemmA with a
// queue sync per call) by a single persistent kernel per sweep:
//
//   op(M) X = B,  op(M) lower (forward) or upper (backward), unit or not,
//   op(M) = M or M^T, X overwritten in place, nrhs <= 16.
//
// Row blocks of 64 are taken in solve order through an atomic ticket, so a
// block only ever waits for blocks that are already running.  The block
// with ticket p accumulates op(M)(i, j) x_j over the blocks solved two or
// more steps before it (tickets < p - 1), fetching the next tile into
// registers while it multiplies the current one, forms
// y_i = inv(op(M)_ii) (b_i - acc) before its predecessor has finished, and
// leaves only
//     x_i = y_i - W_i x_{i-1},   W_i = inv(op(M)_ii) op(M)(i, i-1)
// on the chain of dependent blocks (i - 1: the predecessor in solve order;
// W_i is formed beside the diagonal-block inverses before the sweep).
//
// Solved values travel between blocks through a mailbox of 64-bit words,
// 32 data bits and a 32-bit flag each (two words per double): one aligned
// 64-bit store is single-copy atomic, so a reader that sees the flag sees
// the data, and neither a fence nor a separate ready flag sits on the
// chain.  Readers poll with a bounded spin.  The mailbox is cleared before
// every launch.  The matrix is read once (HBM-bound); the critical path is
// one 64 x 64 matrix-vector product and one L2 round trip per block.  For
// up to 4 right-hand sides the four thread groups of a block split the 64
// columns of every product and add their partial sums in shared memory;
// for more, each group owns 4 right-hand sides.
//
// The FP32 kernel for 5 to 16 right-hand sides (sweep16_kernel, the block
// FGMRES preconditioner) runs in thread-block clusters (4 CTAs by default):
// a cluster takes consecutive blocks per ticket, and the chain input x_{i-1}
// and the last streamed block x_{i-2} reach a block through distributed
// shared memory from ranks r - 1 and r - 2 of its cluster (about 0.5 us
// against about 2 us through L2), through the mailbox across clusters.  The
// older solved blocks stream through the same cp.async ring as the matrix
// tiles, from a row-major copy released by per-block done flags.

#include "common.cuh"

#include <cstdlib>
#include "prof.h"

#include <type_traits>

namespace slt {

constexpr int kSwBS = 64;
constexpr int kSwRhs = 16;

template <typename T>
struct SweepSmem {
    T Ts[kSwBS][kSwBS + 1];    // off-diagonal tile, [col][row]
    T Ds[kSwBS][kSwBS + 1];    // inverse of the diagonal block, [row][col]
    T Ws[kSwBS][kSwBS + 1];    // W_i, [row][col]
    T xs[kSwBS][kSwRhs];       // solved block x_j
    T xi[kSwBS][kSwRhs];       // this block's right-hand side
    T red[4][kSwBS][4];        // partial sums of the four column groups
};

__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v)
{
    asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" :: "l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p)
{
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// Mailbox words: low half data, high half kMbFlag (the mailbox is zeroed
// before each launch, so a word carrying the flag was written by this launch).
constexpr unsigned long long kMbFlag = 0x5157ull << 32;

template <typename T> struct Mailbox;
template <> struct Mailbox<float> {
    static constexpr int kWords = 1;
    static __device__ __forceinline__ void put(unsigned long long* p, float v) {
        st_relaxed_u64(p, kMbFlag | __float_as_uint(v));
    }
    static __device__ __forceinline__ bool get(const unsigned long long* p, float& v) {
        const unsigned long long w = ld_relaxed_u64(p);
        v = __uint_as_float(unsigned(w));
        return (w & 0xffffffff00000000ull) == kMbFlag;
    }
};
template <> struct Mailbox<double> {
    static constexpr int kWords = 2;
    static __device__ __forceinline__ void put(unsigned long long* p, double v) {
        const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v));
        st_relaxed_u64(p, kMbFlag | (b & 0xffffffffull));
        st_relaxed_u64(p + 1, kMbFlag | (b >> 32));
    }
    static __device__ __forceinline__ bool get(const unsigned long long* p, double& v) {
        const unsigned long long w0 = ld_relaxed_u64(p), w1 = ld_relaxed_u64(p + 1);
        v = __longlong_as_double(static_cast<long long>((w1 << 32) | (w0 & 0xffffffffull)));
        return (w0 & 0xffffffff00000000ull) == kMbFlag && (w1 & 0xffffffff00000000ull) == kMbFlag;
    }
};

// a[0..3] += v * s[0..3], s 16-byte aligned in shared memory
__device__ __forceinline__ void axpy4(float v, const float* s, float* a)
{
    const float4 x = *reinterpret_cast<const float4*>(s);
    a[0] = fmaf(v, x.x, a[0]); a[1] = fmaf(v, x.y, a[1]); a[2] = fmaf(v, x.z, a[2]); a[3] = fmaf(v, x.w, a[3]);
}
__device__ __forceinline__ void axpy4(double v, const double* s, double* a)
{
    const double2 x = *reinterpret_cast<const double2*>(s);
    const double2 y = *reinterpret_cast<const double2*>(s + 2);
    a[0] = fma(v, x.x, a[0]); a[1] = fma(v, x.y, a[1]); a[2] = fma(v, y.x, a[2]); a[3] = fma(v, y.y, a[3]);
}

__device__ __forceinline__ uint64_t sw_globaltimer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// Inverse of every 64 x 64 diagonal block of op(M) (lower for FORWARD,
// upper otherwise), one block per CTA, 4 lanes per column.  Dinv[b] is
// row-major: Dinv[b][r][c].
template <typename T, bool FORWARD, bool UNIT, bool TRANS>
__global__ void __launch_bounds__(256)
trinv_kernel(int64_t n, const T* __restrict__ M, int64_t ldm, T* __restrict__ Dinv)
{
    extern __shared__ unsigned char ti_smem_raw[];
    T (*Ds)[kSwBS + 1] = reinterpret_cast<T (*)[kSwBS + 1]>(ti_smem_raw);
    T (*Xv)[kSwBS + 1] = Ds + kSwBS;       // Xv[r][c]: inverse being built, column c
    const int t = threadIdx.x;
    const int64_t i0 = int64_t(blockIdx.x) * kSwBS;
    const int ni = int(min64(kSwBS, n - i0));
    for (int e = t; e < kSwBS * kSwBS; e += 256) {
        int r, c;
        if (TRANS) { c = e % kSwBS; r = e / kSwBS; }
        else       { r = e % kSwBS; c = e / kSwBS; }
        T v;
        if (r < ni && c < ni) v = TRANS ? M[(i0 + c) + (i0 + r) * ldm] : M[(i0 + r) + (i0 + c) * ldm];
        else v = (r == c) ? T(1) : T(0);      // identity padding keeps the inverse well defined
        Ds[r][c] = v;
        Xv[r][c] = T(0);
    }
    __syncthreads();
    const int c = t >> 2, q = t & 3;          // column c, lane q of 4
    const T dcc = UNIT ? T(1) : Ds[c][c];
    if (q == 0) Xv[c][c] = T(1) / dcc;
    __syncwarp();
    // Every lane runs the same rows (warp-uniform trip count, so the shuffles
    // and __syncwarp below see all 32 lanes); rows outside the column's
    // triangle contribute nothing.
    for (int s = 1; s < kSwBS; ++s) {
        const int r = FORWARD ? s : kSwBS - 1 - s;
        const bool active = FORWARD ? (r > c) : (r < c);
        T part = T(0);
        if (active) {
            if (FORWARD) { for (int l = c + q; l < r; l += 4) part = fma(Ds[r][l], Xv[l][c], part); }
            else         { for (int l = r + 1 + q; l <= c; l += 4) part = fma(Ds[r][l], Xv[l][c], part); }
        }
        part += __shfl_xor_sync(0xffffffffu, part, 2);
        part += __shfl_xor_sync(0xffffffffu, part, 1);
        if (active && q == 0) Xv[r][c] = -part / (UNIT ? T(1) : Ds[r][r]);
        __syncwarp();
    }
    __syncthreads();
    T* out = Dinv + size_t(blockIdx.x) * kSwBS * kSwBS;
    for (int e = t; e < kSwBS * kSwBS; e += 256) out[e] = Xv[e / kSwBS][e % kSwBS];

    // W = inv(op(M)_ii) op(M)(i, j), j the block solved just before i
    const int64_t bj = FORWARD ? int64_t(blockIdx.x) - 1 : int64_t(blockIdx.x) + 1;
    if (bj < 0 || bj >= int64_t(gridDim.x)) return;
    const int64_t j0 = bj * kSwBS;
    const int nj = int(min64(kSwBS, n - j0));
    staged_copy<kSwBS * kSwBS / 256, 256>(kSwBS * kSwBS, [&](int e) {
        const int l = TRANS ? e / kSwBS : e % kSwBS, cc = TRANS ? e % kSwBS : e / kSwBS;
        return (l < ni && cc < nj) ? (TRANS ? M[(j0 + cc) + (i0 + l) * ldm] : M[(i0 + l) + (j0 + cc) * ldm]) : T(0);
    }, [&](int e, T v) {
        const int l = TRANS ? e / kSwBS : e % kSwBS, cc = TRANS ? e % kSwBS : e / kSwBS;
        Ds[l][cc] = v;
    });
    __syncthreads();
    const int wc = t % kSwBS, wr = t / kSwBS;    // column wc, rows wr, wr + 4, ...
    T w[kSwBS / 4];
    #pragma unroll
    for (int j = 0; j < kSwBS / 4; ++j) w[j] = T(0);
    for (int l = 0; l < kSwBS; ++l) {
        const T tl = Ds[l][wc];
        #pragma unroll
        for (int j = 0; j < kSwBS / 4; ++j) w[j] = fma(Xv[wr + 4 * j][l], tl, w[j]);
    }
    T* wout = Dinv + size_t(gridDim.x + blockIdx.x) * kSwBS * kSwBS;
    #pragma unroll
    for (int j = 0; j < kSwBS / 4; ++j) wout[(wr + 4 * j) * kSwBS + wc] = w[j];
}

// mb: mailbox, word ((q * npad + row) * kWords + h) for solved value
// (row, q), npad = 64 * ceil(n / 64).
template <typename T, bool FORWARD, bool UNIT, bool TRANS>
__global__ void __launch_bounds__(256)
sweep_kernel(int64_t n, int nrhs, const T* __restrict__ M, int64_t ldm, const T* __restrict__ Dinv,
             T* X, int64_t ldx, int* ticket, unsigned long long* mb, int* status)
{
    using MB = Mailbox<T>;
    extern __shared__ __align__(16) unsigned char sw_smem_raw[];
    SweepSmem<T>& sm = *reinterpret_cast<SweepSmem<T>*>(sw_smem_raw);
    __shared__ int s_p;
    constexpr int PER = kSwBS * kSwBS / 256;       // tile elements per thread
    constexpr int XPER = kSwBS * kSwRhs / 256;     // x_j elements per thread
    const int t = threadIdx.x;
    const int nblk = int(ceildiv(n, kSwBS));
    const int64_t npad = int64_t(nblk) * kSwBS;
    const int r = t % kSwBS, g = t / kSwBS;
    const bool split = nrhs <= 4;
    const int c0 = split ? 16 * g : 0, c1 = split ? c0 + 16 : kSwBS;   // columns of this thread's products
    const int qb = split ? 0 : 4 * g;                                  // its first right-hand side
    const T* Wall = Dinv + size_t(nblk) * kSwBS * kSwBS;

    auto opM = [&](int64_t rr, int64_t c) -> T {
        return TRANS ? __ldg(&M[c + rr * ldm]) : __ldg(&M[rr + c * ldm]);
    };
    auto mbox = [&](int64_t row, int q) { return mb + (q * npad + row) * MB::kWords; };
    // bounded poll of one mailbox value; false on timeout or error
    auto spin = [&](const unsigned long long* a, T& v) -> bool {
        if (MB::get(a, v)) return true;
        const uint64_t t0 = sw_globaltimer();
        for (unsigned it = 1; !MB::get(a, v); ++it) {
            if ((it & 255u) == 0 &&
                (ld_volatile_i32(status) != 0 || sw_globaltimer() - t0 > 2000000000ull)) {
                atomicCAS(status, 0, SLT_ERR_TIMEOUT);
                return false;
            }
        }
        return true;
    };

    for (;;) {
        if (t == 0) s_p = atomicAdd(ticket, 1);
        __syncthreads();
        const int p = s_p;
        if (p >= nblk) break;
        const int bi = FORWARD ? p : nblk - 1 - p;
        const int64_t i0 = int64_t(bi) * kSwBS;
        const int ni = int(min64(kSwBS, n - i0));

        // inverse of the diagonal block and W_i (row-major), this block's RHS
        {
            const T* dinv = Dinv + size_t(bi) * kSwBS * kSwBS;
            staged_copy<kSwBS * kSwBS / 256, 256>(kSwBS * kSwBS, [&](int e) { return dinv[e]; },
                                                  [&](int e, T v) { sm.Ds[e / kSwBS][e % kSwBS] = v; });
            if (p > 0) {
                const T* wsrc = Wall + size_t(bi) * kSwBS * kSwBS;
                staged_copy<kSwBS * kSwBS / 256, 256>(kSwBS * kSwBS, [&](int e) { return wsrc[e]; },
                                                      [&](int e, T v) { sm.Ws[e / kSwBS][e % kSwBS] = v; });
            }
        }
        staged_copy<kSwBS * kSwRhs / 256, 256>(kSwBS * kSwRhs, [&](int e) {
            const int rr = e % kSwBS, q = e / kSwBS;
            return (rr < ni && q < nrhs) ? X[i0 + rr + q * ldx] : T(0);
        }, [&](int e, T v) { sm.xi[e % kSwBS][e / kSwBS] = v; });

        T pre[PER], xv[XPER];
        bool xok[XPER];
        auto fetch_tile = [&](int k) {
            const int bj = FORWARD ? k : nblk - 1 - k;
            const int64_t j0 = int64_t(bj) * kSwBS;
            const int nj = int(min64(kSwBS, n - j0));
            #pragma unroll
            for (int u = 0; u < PER; ++u) {
                const int e = t + 256 * u;
                const int rr = TRANS ? e / kSwBS : e % kSwBS, c = TRANS ? e % kSwBS : e / kSwBS;
                pre[u] = (rr < ni && c < nj) ? opM(i0 + rr, j0 + c) : T(0);
            }
        };
        // one poll of x_k (block solved k-th); what is not there yet is finished by finish_x
        auto try_x = [&](int k) {
            const int bj = FORWARD ? k : nblk - 1 - k;
            const int64_t j0 = int64_t(bj) * kSwBS;
            const int nj = int(min64(kSwBS, n - j0));
            #pragma unroll
            for (int u = 0; u < XPER; ++u) {
                const int e = t + 256 * u, rr = e % kSwBS, q = e / kSwBS;
                if (rr < nj && q < nrhs) xok[u] = MB::get(mbox(j0 + rr, q), xv[u]);
                else { xv[u] = T(0); xok[u] = true; }
            }
        };
        auto finish_x = [&](int k) -> bool {
            const int64_t j0 = int64_t(FORWARD ? k : nblk - 1 - k) * kSwBS;
            bool ok = true;
            #pragma unroll
            for (int u = 0; u < XPER; ++u) {
                const int e = t + 256 * u, rr = e % kSwBS, q = e / kSwBS;
                if (!xok[u] && ok) ok = spin(mbox(j0 + rr, q), xv[u]);
            }
            return ok;
        };
        auto put_x = [&]() {
            #pragma unroll
            for (int u = 0; u < XPER; ++u) {
                const int e = t + 256 * u;
                sm.xs[e % kSwBS][e / kSwBS] = xv[u];
            }
        };
        auto put_tile = [&]() {
            #pragma unroll
            for (int u = 0; u < PER; ++u) {
                const int e = t + 256 * u;
                const int rr = TRANS ? e / kSwBS : e % kSwBS, c = TRANS ? e % kSwBS : e / kSwBS;
                sm.Ts[c][rr] = pre[u];
            }
        };

        // acc = sum over the blocks solved two or more steps earlier
        T acc[4] = {T(0), T(0), T(0), T(0)};
        const int K = p > 0 ? p - 1 : 0;
        if (K > 0) {
            fetch_tile(0);
            try_x(0);
            const bool ok = finish_x(0);
            put_tile();
            put_x();
            if (__syncthreads_or(!ok)) return;
        }
        else {
            __syncthreads();
        }
        for (int k = 0; k < K; ++k) {
            const bool more = k + 1 < K;
            if (more) {
                fetch_tile(k + 1);
                try_x(k + 1);
            }
            #pragma unroll 4
            for (int c = c0; c < c1; ++c) axpy4(sm.Ts[c][r], &sm.xs[c][qb], acc);
            __syncthreads();
            bool ok = true;
            if (more) {
                ok = finish_x(k + 1);
                put_tile();
                put_x();
            }
            if (__syncthreads_or(!ok)) return;
        }
        if (p > 0) try_x(p - 1);       // in flight while y_i is formed

        // z = b_i - acc (in xi)
        if (split) {
            #pragma unroll
            for (int u = 0; u < 4; ++u) sm.red[g][r][u] = acc[u];
            __syncthreads();
            sm.xi[r][g] -= (sm.red[0][r][g] + sm.red[1][r][g]) + (sm.red[2][r][g] + sm.red[3][r][g]);
        }
        else {
            #pragma unroll
            for (int u = 0; u < 4; ++u) sm.xi[r][qb + u] -= acc[u];
        }
        __syncthreads();

        // y_i = inv(op(M)_ii) z
        T y[4] = {T(0), T(0), T(0), T(0)};
        #pragma unroll 4
        for (int c = c0; c < c1; ++c) axpy4(sm.Ds[r][c], &sm.xi[c][qb], y);
        if (split) {
            #pragma unroll
            for (int u = 0; u < 4; ++u) sm.red[g][r][u] = y[u];
            __syncthreads();
            y[0] = (sm.red[0][r][g] + sm.red[1][r][g]) + (sm.red[2][r][g] + sm.red[3][r][g]);
        }

        // chain step: x_i = y_i - W_i x_{i-1}
        if (p > 0) {
            const bool ok = finish_x(p - 1);
            put_x();
            if (__syncthreads_or(!ok)) return;
            T v[4] = {T(0), T(0), T(0), T(0)};
            #pragma unroll 4
            for (int c = c0; c < c1; ++c) axpy4(sm.Ws[r][c], &sm.xs[c][qb], v);
            if (split) {
                #pragma unroll
                for (int u = 0; u < 4; ++u) sm.red[g][r][u] = v[u];
                __syncthreads();
                y[0] -= (sm.red[0][r][g] + sm.red[1][r][g]) + (sm.red[2][r][g] + sm.red[3][r][g]);
            }
            else {
                #pragma unroll
                for (int u = 0; u < 4; ++u) y[u] -= v[u];
            }
        }
        if (r < ni) {
            if (split) {
                if (g < nrhs) {
                    MB::put(mbox(i0 + r, g), y[0]);
                    X[i0 + r + g * ldx] = y[0];
                }
            }
            else {
                #pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (qb + u < nrhs) {
                        MB::put(mbox(i0 + r, qb + u), y[u]);
                        X[i0 + r + (qb + u) * ldx] = y[u];
                    }
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// FP32 sweep for 5 to 16 right-hand sides (the preconditioner of the block
// FGMRES).  Same ticket order, mailbox and chain step as sweep_kernel; the
// products with the blocks solved two or more steps earlier differ:
//  * every solved block also goes to a row-major copy xr (64 rows x 16
//    right-hand sides, 4 KB) followed by a release of its done flag; a block
//    acquires the flag of a solved block and copies its 4 KB with cp.async;
//  * the tiles and those solved blocks stream through a ring of kS16
//    shared-memory stages filled with cp.async (tiles zero-filled outside the
//    matrix), so kS16 - 1 tiles are in flight while one is multiplied, with
//    one barrier per tile; the mailbox serves only the chain step;
//  * thread t owns a 4 x 4 register tile -- 4 rows by 4 right-hand sides --
//    over one quarter (16 columns) of every tile: two 16-byte shared loads per
//    16 FMAs; the four quarters are added once per block row.
// Tile layout in a stage: [column][row] for op(M) = M (rows of a column
// contiguous, as in memory), [row][column] for op(M) = M^T; the thread's
// rows are 4 consecutive ones for M and 4 rows 16 apart for M^T, so that
// both layouts are read without bank conflicts.
constexpr int kS16 = 3;
constexpr int kSwLd = kSwBS + 4;       // stage row stride (floats), 16-byte rows

struct Sweep16Smem {
    float Ts[kS16][kSwBS][kSwLd];      // tile ring; the last block row's partial sums reuse it
    float Ds[kSwBS][kSwBS + 1];        // inverse of the diagonal block, [row][col]
    float Ws[kSwBS][kSwBS + 1];        // W_i, [row][col]
    float xs[kS16][kSwBS][kSwRhs];     // solved blocks x_k, [row][rhs]
    float xi[kSwBS][kSwRhs];           // this block's right-hand side
    float xin[kSwBS][kSwRhs];          // x_{i-1} of the chain step
    float xin2[kSwBS][kSwRhs];         // x_{i-2}, the last streamed block (from rank r - 2)
};

// Thread-block cluster helpers (sm_90+): rank and size, a full cluster
// barrier, shared-memory addresses of another CTA of the cluster (mapa),
// stores to them, and remote / cluster-scope mbarrier operations.
__device__ __forceinline__ uint32_t cluster_ctarank()
{
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t cluster_nctarank()
{
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ void cluster_sync_all()
{
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ uint32_t mapa_shared(uint32_t addr, uint32_t rank)
{
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
    return r;
}
__device__ __forceinline__ void st_cluster_u32(uint32_t addr, int v)
{
    asm volatile("st.shared::cluster.u32 [%0], %1;" :: "r"(addr), "r"(v) : "memory");
}
__device__ __forceinline__ void st_cluster_f4(uint32_t addr, float4 v)
{
    asm volatile("st.shared::cluster.v4.f32 [%0], {%1, %2, %3, %4};"
                 :: "r"(addr), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w) : "memory");
}
__device__ __forceinline__ void mbar_init_cta(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_remote(uint32_t bar_cluster_addr)
{
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" :: "r"(bar_cluster_addr) : "memory");
}
// Bounded wait (two seconds, or a failure recorded in status) for the phase
// with the given parity of a local mbarrier that CTAs of the cluster arrive on.
__device__ __forceinline__ bool mbar_wait_cluster(uint32_t bar, uint32_t parity, const int* status)
{
    auto try_once = [&]() -> bool {
        uint32_t ok;
        asm volatile("{\n\t.reg .pred P1;\n\t"
                     "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 P1, [%1], %2;\n\t"
                     "selp.b32 %0, 1, 0, P1;\n\t}"
                     : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
        return ok != 0;
    };
    if (try_once()) return true;
    const uint64_t t0 = sw_globaltimer();
    for (unsigned it = 1; !try_once(); ++it) {
        if ((it & 63u) == 0 && (ld_volatile_i32(status) != 0 || sw_globaltimer() - t0 > 2000000000ull)) {
            atomicCAS(const_cast<int*>(status), 0, SLT_ERR_TIMEOUT);
            return false;
        }
    }
    return true;
}

__device__ __forceinline__ void cp_async4(uint32_t dst, const void* src, bool valid)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;"
                 :: "r"(dst), "l"(src), "r"(valid ? 4 : 0) : "memory");
}
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" :: "r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ int ld_acquire_i32(const int* p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_i32(int* p, int v)
{
    asm volatile("st.release.gpu.global.b32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" :: "n"(N) : "memory"); }

template <bool FORWARD, bool UNIT, bool TRANS>
__global__ void __launch_bounds__(256, 2)
sweep16_kernel(int64_t n, int nrhs, const float* __restrict__ M, int64_t ldm, const float* __restrict__ Dinv,
               float* X, int64_t ldx, int* ticket, unsigned long long* mb, float* xr, int* done, int* status,
               int vec)
{
    using MB = Mailbox<float>;
    extern __shared__ __align__(16) unsigned char sw_smem_raw[];
    Sweep16Smem& sm = *reinterpret_cast<Sweep16Smem*>(sw_smem_raw);
    __shared__ int s_p, s_dead;
    __shared__ __align__(8) unsigned long long xin_bar[2];
    constexpr int XPER = kSwBS * kSwRhs / 256;
    const int t = threadIdx.x;
    const int nblk = int(ceildiv(n, kSwBS));
    const int64_t npad = int64_t(nblk) * kSwBS;
    const int r = t % kSwBS, g = t / kSwBS, qb = 4 * g;    // row / right-hand sides outside the products
    const int kq = t >> 6, tr = t & 15, tc = (t >> 4) & 3;  // product tile: column quarter, rows, rhs
    const float* Wall = Dinv + size_t(nblk) * kSwBS * kSwBS;

    auto mbox = [&](int64_t row, int q) { return mb + (q * npad + row) * MB::kWords; };
    auto spin = [&](const unsigned long long* a, float& v) -> bool {
        if (MB::get(a, v)) return true;
        const uint64_t t0 = sw_globaltimer();
        for (unsigned it = 1; !MB::get(a, v); ++it) {
            if ((it & 255u) == 0 &&
                (ld_volatile_i32(status) != 0 || sw_globaltimer() - t0 > 2000000000ull)) {
                atomicCAS(status, 0, SLT_ERR_TIMEOUT);
                return false;
            }
        }
        return true;
    };

    // cluster: rank crank of csize CTAs; the cluster takes csize consecutive
    // blocks per ticket, rank r the r-th, and hands x of each block to the
    // next rank through its shared memory (xin, xin_bar[0]) and to the rank
    // after it (xin2, xin_bar[1]: its last streamed block); the last two
    // ranks also write the mailbox, for the next cluster's ranks 0 and 1
    const uint32_t crank = cluster_ctarank(), csize = cluster_nctarank();
    const uint32_t bar_local = static_cast<uint32_t>(__cvta_generic_to_shared(&xin_bar[0]));
    const uint32_t bar2_local = static_cast<uint32_t>(__cvta_generic_to_shared(&xin_bar[1]));
    const uint32_t xin_local = static_cast<uint32_t>(__cvta_generic_to_shared(&sm.xin[r][qb]));
    const uint32_t xin2_local = static_cast<uint32_t>(__cvta_generic_to_shared(&sm.xin2[r][qb]));
    if (t == 0) {
        mbar_init_cta(bar_local, 256);
        mbar_init_cta(bar2_local, 256);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    uint32_t xph = 0, xph2 = 0;

    auto process = [&](const int p) -> bool {
        const int bi = FORWARD ? p : nblk - 1 - p;
        const int64_t i0 = int64_t(bi) * kSwBS;
        const int ni = int(min64(kSwBS, n - i0));

        {
            const float* dinv = Dinv + size_t(bi) * kSwBS * kSwBS;
            staged_copy<kSwBS * kSwBS / 256, 256>(kSwBS * kSwBS, [&](int e) { return dinv[e]; },
                                                  [&](int e, float v) { sm.Ds[e / kSwBS][e % kSwBS] = v; });
            if (p > 0) {
                const float* wsrc = Wall + size_t(bi) * kSwBS * kSwBS;
                staged_copy<kSwBS * kSwBS / 256, 256>(kSwBS * kSwBS, [&](int e) { return wsrc[e]; },
                                                      [&](int e, float v) { sm.Ws[e / kSwBS][e % kSwBS] = v; });
            }
        }
        staged_copy<kSwBS * kSwRhs / 256, 256>(kSwBS * kSwRhs, [&](int e) {
            const int rr = e % kSwBS, q = e / kSwBS;
            return (rr < ni && q < nrhs) ? X[i0 + rr + q * ldx] : 0.f;
        }, [&](int e, float v) { sm.xi[e % kSwBS][e / kSwBS] = v; });

        // tile of the k-th solved block into ring stage st
        auto issue_tile = [&](int k, int st) {
            const int bj = FORWARD ? k : nblk - 1 - k;
            const int64_t j0 = int64_t(bj) * kSwBS;
            const int nj = int(min64(kSwBS, n - j0));
            float* base = &sm.Ts[st][0][0];
            if (vec && ni == kSwBS && nj == kSwBS) {
                #pragma unroll
                for (int u = 0; u < kSwBS * kSwBS / (4 * 256); ++u) {
                    const int e = t + 256 * u;                 // 16-byte chunk: 4 consecutive rows (cols for TRANS)
                    const int a = (e % (kSwBS / 4)) * 4, b = e / (kSwBS / 4);
                    const float* src = TRANS ? &M[(j0 + a) + (i0 + b) * ldm] : &M[(i0 + a) + (j0 + b) * ldm];
                    cp_async16(static_cast<uint32_t>(__cvta_generic_to_shared(base + b * kSwLd + a)), src);
                }
            }
            else {
                #pragma unroll 4
                for (int u = 0; u < kSwBS * kSwBS / 256; ++u) {
                    const int e = t + 256 * u;
                    const int a = e % kSwBS, b = e / kSwBS;    // a: contiguous index in memory
                    const bool ok = TRANS ? (a < nj && b < ni) : (a < ni && b < nj);
                    const float* src = ok ? (TRANS ? &M[(j0 + a) + (i0 + b) * ldm] : &M[(i0 + a) + (j0 + b) * ldm]) : M;
                    cp_async4(static_cast<uint32_t>(__cvta_generic_to_shared(base + b * kSwLd + a)), src, ok);
                }
            }
        };
        float xv[XPER];
        bool xok[XPER];
        auto try_x = [&](int k) {
            const int64_t j0 = int64_t(FORWARD ? k : nblk - 1 - k) * kSwBS;
            const int nj = int(min64(kSwBS, n - j0));
            #pragma unroll
            for (int u = 0; u < XPER; ++u) {
                const int e = t + 256 * u, rr = e % kSwBS, q = e / kSwBS;
                if (rr < nj && q < nrhs) xok[u] = MB::get(mbox(j0 + rr, q), xv[u]);
                else { xv[u] = 0.f; xok[u] = true; }
            }
        };
        auto finish_x = [&](int k) -> bool {
            const int64_t j0 = int64_t(FORWARD ? k : nblk - 1 - k) * kSwBS;
            bool ok = true;
            #pragma unroll
            for (int u = 0; u < XPER; ++u) {
                const int e = t + 256 * u, rr = e % kSwBS, q = e / kSwBS;
                if (!xok[u] && ok) ok = spin(mbox(j0 + rr, q), xv[u]);
            }
            return ok;
        };
        auto put_x = [&](int st) {
            #pragma unroll
            for (int u = 0; u < XPER; ++u) {
                const int e = t + 256 * u;
                sm.xs[st][e % kSwBS][e / kSwBS] = xv[u];
            }
        };
        const int K = p > 0 ? p - 1 : 0;      // solved blocks streamed before the chain step
        // the k-th solved block into ring stage st: its tile of op(M) and, once
        // its done flag is seen, its 64 x 16 values from xr (thread t: row t / 4,
        // right-hand sides 4 (t % 4) ..).  Done flags are read 256 blocks at a
        // time (thread t the (k + t)-th): while all are set, no block waits on a
        // flag; at the solve front the block waits for the one flag it needs.
        // The last streamed block (k = K - 1, solved two steps before) gets
        // its values later, from rank r - 2 or the mailbox.  Called by every
        // thread with the same k; returns the same value to all.
        int known = 0;                          // blocks 0 .. known - 1 seen done
        auto issue = [&](int k, int st) -> bool {
            issue_tile(k, st);
            if (k == K - 1) return true;
            const int bj = FORWARD ? k : nblk - 1 - k;
            if (k >= known) {
                const int kk = min(k + t, K - 2);
                const int v = ld_acquire_i32(done + (FORWARD ? kk : nblk - 1 - kk));
                if (__syncthreads_and(v != 0)) {
                    known = min(K, k + 256);
                }
                else {
                    bool okw = true;
                    if (ld_acquire_i32(done + bj) == 0) {
                        const uint64_t t0 = sw_globaltimer();
                        for (unsigned it = 1; ld_acquire_i32(done + bj) == 0; ++it) {
                            if ((it & 255u) == 0 &&
                                (ld_volatile_i32(status) != 0 || sw_globaltimer() - t0 > 2000000000ull)) {
                                atomicCAS(status, 0, SLT_ERR_TIMEOUT);
                                okw = false;
                                break;
                            }
                        }
                    }
                    if (!__syncthreads_and(okw)) return false;
                    known = k + 1;
                }
            }
            cp_async16(static_cast<uint32_t>(__cvta_generic_to_shared(&sm.xs[st][t >> 2][4 * (t & 3)])),
                       xr + (int64_t(bj) * kSwBS + (t >> 2)) * kSwRhs + 4 * (t & 3));
            return true;
        };

        // acc = sum over the blocks solved two or more steps earlier
        float acc[4][4];
        #pragma unroll
        for (int i = 0; i < 4; ++i)
            #pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
        bool ok = true;
        #pragma unroll
        for (int st = 0; st < kS16 - 1; ++st) {
            if (st < K && ok) ok = issue(st, st);
            cp_async_commit();
        }
        const bool x2_mailbox = crank <= 1;    // x of the last streamed block: mailbox, else rank r - 2
        for (int k = 0; k < K; ++k) {
            const int st = k % kS16;
            if (k == K - 1 && x2_mailbox) try_x(k);
            cp_async_wait<kS16 - 2>();          // this thread's copies of block k
            if (__syncthreads_or(!ok)) { cp_async_wait<0>(); return false; }   // everyone's; stage (k - 1) free
            if (k + kS16 - 1 < K) ok = issue(k + kS16 - 1, (k + kS16 - 1) % kS16);
            cp_async_commit();
            if (k == K - 1) {
                bool okx;
                if (x2_mailbox) {
                    okx = finish_x(k);
                    #pragma unroll
                    for (int u = 0; u < XPER; ++u) {
                        const int e = t + 256 * u;
                        sm.xs[st][e % kSwBS][e / kSwBS] = xv[u];
                    }
                }
                else {
                    okx = mbar_wait_cluster(bar2_local, xph2, status);
                    xph2 ^= 1u;
                    *reinterpret_cast<float4*>(&sm.xs[st][t >> 2][4 * (t & 3)]) =
                        *reinterpret_cast<const float4*>(&sm.xin2[t >> 2][4 * (t & 3)]);
                }
                if (__syncthreads_or(!okx)) { cp_async_wait<0>(); return false; }
            }
            const float* Tt = &sm.Ts[st][0][0];
            if (!TRANS) {
                #pragma unroll 4
                for (int c = 16 * kq; c < 16 * kq + 16; ++c) {
                    const float4 a = *reinterpret_cast<const float4*>(Tt + c * kSwLd + 4 * tr);
                    const float4 x = *reinterpret_cast<const float4*>(&sm.xs[st][c][4 * tc]);
                    const float av[4] = {a.x, a.y, a.z, a.w}, xw[4] = {x.x, x.y, x.z, x.w};
                    #pragma unroll
                    for (int i = 0; i < 4; ++i)
                        #pragma unroll
                        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], xw[j], acc[i][j]);
                }
            }
            else {
                #pragma unroll
                for (int c = 16 * kq; c < 16 * kq + 16; c += 4) {
                    float av[4][4], xw[4][4];
                    #pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        const float4 a = *reinterpret_cast<const float4*>(Tt + (tr + 16 * i) * kSwLd + c);
                        av[i][0] = a.x; av[i][1] = a.y; av[i][2] = a.z; av[i][3] = a.w;
                    }
                    #pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const float4 x = *reinterpret_cast<const float4*>(&sm.xs[st][c + u][4 * tc]);
                        xw[u][0] = x.x; xw[u][1] = x.y; xw[u][2] = x.z; xw[u][3] = x.w;
                    }
                    #pragma unroll
                    for (int u = 0; u < 4; ++u)
                        #pragma unroll
                        for (int i = 0; i < 4; ++i)
                            #pragma unroll
                            for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i][u], xw[u][j], acc[i][j]);
                }
            }
        }
        if (__syncthreads_or(!ok)) { cp_async_wait<0>(); return false; }
        cp_async_wait<0>();
        const bool from_mailbox = crank == 0;   // else x_{p-1} comes from rank crank - 1
        if (p > 0 && from_mailbox) try_x(p - 1);       // in flight while y_i is formed

        // the four column quarters' partial sums, then z = b_i - acc (in xi)
        float (*red)[kSwBS][kSwRhs] = reinterpret_cast<float (*)[kSwBS][kSwRhs]>(&sm.Ts[0][0][0]);
        #pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int row = TRANS ? tr + 16 * i : 4 * tr + i;
            #pragma unroll
            for (int j = 0; j < 4; ++j) red[kq][row][4 * tc + j] = acc[i][j];
        }
        __syncthreads();
        #pragma unroll
        for (int u = 0; u < 4; ++u)
            sm.xi[r][qb + u] -= (red[0][r][qb + u] + red[1][r][qb + u]) + (red[2][r][qb + u] + red[3][r][qb + u]);
        __syncthreads();

        // y_i = inv(op(M)_ii) z
        float y[4] = {0.f, 0.f, 0.f, 0.f};
        #pragma unroll 4
        for (int c = 0; c < kSwBS; ++c) axpy4(sm.Ds[r][c], &sm.xi[c][qb], y);

        // chain step: x_i = y_i - W_i x_{i-1}
        if (p > 0) {
            bool okc = true;
            if (from_mailbox) {
                okc = finish_x(p - 1);
                #pragma unroll
                for (int u = 0; u < XPER; ++u) {
                    const int e = t + 256 * u;
                    sm.xin[e % kSwBS][e / kSwBS] = xv[u];
                }
            }
            else {
                okc = mbar_wait_cluster(bar_local, xph, status);
                xph ^= 1u;
            }
            if (__syncthreads_or(!okc)) return false;
            float v[4] = {0.f, 0.f, 0.f, 0.f};
            #pragma unroll 4
            for (int c = 0; c < kSwBS; ++c) axpy4(sm.Ws[r][c], &sm.xin[c][qb], v);
            #pragma unroll
            for (int u = 0; u < 4; ++u) y[u] -= v[u];
        }
        // x_i: to the next rank's shared memory (its chain step), else to the
        // mailbox (the next cluster's rank 0); to X; to the row-major copy
        // (zeros past n), then this block's done flag
        const float4 yv = r < ni ? make_float4(y[0], y[1], y[2], y[3]) : make_float4(0.f, 0.f, 0.f, 0.f);
        const bool to_next = crank + 1 < csize;
        if (to_next && p + 1 < nblk) {
            st_cluster_f4(mapa_shared(xin_local, crank + 1), yv);
            mbar_arrive_remote(mapa_shared(bar_local, crank + 1));
        }
        if (crank + 2 < csize && p + 2 < nblk) {
            st_cluster_f4(mapa_shared(xin2_local, crank + 2), yv);
            mbar_arrive_remote(mapa_shared(bar2_local, crank + 2));
        }
        const bool to_mailbox = crank + 2 >= csize;
        if (r < ni) {
            #pragma unroll
            for (int u = 0; u < 4; ++u)
                if (qb + u < nrhs) {
                    if (to_mailbox) MB::put(mbox(i0 + r, qb + u), y[u]);
                    X[i0 + r + (qb + u) * ldx] = y[u];
                }
        }
        *reinterpret_cast<float4*>(xr + (int64_t(bi) * kSwBS + r) * kSwRhs + qb) = yv;
        __threadfence();
        __syncthreads();
        if (t == 0) st_release_i32(done + bi, 1);
        return true;
    };

    for (;;) {
        // one ticket per cluster, taken by rank 0 and written to every rank
        cluster_sync_all();
        if (crank == 0 && t == 0) {
            const int cp = atomicAdd(ticket, 1);
            const int dead = ld_volatile_i32(status) != 0;
            for (uint32_t q = 0; q < csize; ++q) {
                st_cluster_u32(mapa_shared(static_cast<uint32_t>(__cvta_generic_to_shared(&s_p)), q), cp);
                st_cluster_u32(mapa_shared(static_cast<uint32_t>(__cvta_generic_to_shared(&s_dead)), q), dead);
            }
        }
        cluster_sync_all();
        const int p0 = s_p * int(csize);
        if (p0 >= nblk) break;
        const int p = p0 + int(crank);
        if (p < nblk && !s_dead) process(p);
    }
    // no shared-memory traffic of the cluster may target an exited CTA
    cluster_sync_all();
}

// CTAs per cluster of the FP32 16-right-hand-side sweep: SLT_SWEEP_CLUSTER
// (1, 2, 4 or 8) when set, else 4.
static int sweep_cluster_size()
{
    if (const char* e = std::getenv("SLT_SWEEP_CLUSTER")) {
        const int v = std::atoi(e);
        if (v == 1 || v == 2 || v == 4 || v == 8) return v;
    }
    return 4;
}

template <typename T, bool FORWARD, bool UNIT, bool TRANS>
static int launch_sweep(int64_t n, int64_t nrhs, const T* M, int64_t ldm, T* X, int64_t ldx, int* flags,
                        int* status, cudaStream_t s)
{
    if (n <= 0 || nrhs <= 0) return SLT_OK;
    if (nrhs > kSwRhs) return SLT_ERR_ARG;
    const int64_t nblk = ceildiv(n, kSwBS);
    const int64_t npad = nblk * kSwBS;
    // scratch layout: [ticket, pad to 256 B][mailbox: kSwRhs x npad x 2 words]
    // [Dinv: nblk x 64 x 64][W: nblk x 64 x 64] (sized for double)
    // [xr: npad x kSwRhs floats][done: nblk ints]
    unsigned long long* mb = reinterpret_cast<unsigned long long*>(reinterpret_cast<char*>(flags) + 256);
    T* Dinv = reinterpret_cast<T*>(reinterpret_cast<char*>(flags) + 256 + size_t(kSwRhs) * npad * 2 * 8);
    char* tail = reinterpret_cast<char*>(flags) + 256 + size_t(kSwRhs) * npad * 2 * 8 +
                 2 * size_t(nblk) * kSwBS * kSwBS * sizeof(double);
    float* xr = reinterpret_cast<float*>(tail);
    int* done = reinterpret_cast<int*>(tail + size_t(npad) * kSwRhs * sizeof(float));
    const size_t ti_smem = size_t(2) * kSwBS * (kSwBS + 1) * sizeof(T);
    SLT_SMEM_ONCE((trinv_kernel<T, FORWARD, UNIT, TRANS>), ti_smem);
    trinv_kernel<T, FORWARD, UNIT, TRANS><<<unsigned(nblk), 256, ti_smem, s>>>(n, M, ldm, Dinv);
    count_launch();
    SLT_CUDA_TRY(cudaGetLastError());
    // ticket and the first nrhs columns of the mailbox
    SLT_CUDA_TRY(cudaMemsetAsync(flags, 0, 256 + size_t(nrhs) * size_t(npad) * Mailbox<T>::kWords * 8, s));
    if (std::is_same<T, float>::value && nrhs > 4) {
        // 5 to 16 right-hand sides in FP32: the cp.async / register-tile variant
        // clusters of sweep_cluster_size() CTAs (consecutive blocks per cluster)
        auto fn16 = sweep16_kernel<FORWARD, UNIT, TRANS>;
        const size_t smem16 = sizeof(Sweep16Smem);
        SLT_SMEM_ONCE(fn16, smem16);
        const int vec = (reinterpret_cast<uintptr_t>(M) % 16 == 0) && ((ldm * int64_t(sizeof(T))) % 16 == 0);
        SLT_CUDA_TRY(cudaMemsetAsync(done, 0, size_t(nblk) * sizeof(int), s));
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute attr[1];
        cfg.blockDim = dim3(256);
        cfg.dynamicSmemBytes = smem16;
        cfg.stream = s;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        attr[0].id = cudaLaunchAttributeClusterDimension;
        int csize = sweep_cluster_size();
        int nclusters = 0;
        for (;; csize /= 2) {
            attr[0].val.clusterDim.x = unsigned(csize);
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.gridDim = dim3(unsigned(csize));
            SLT_CUDA_TRY(cudaOccupancyMaxActiveClusters(&nclusters, fn16, &cfg));
            if (nclusters > 0 || csize == 1) break;
        }
        if (nclusters <= 0) return SLT_ERR_NOT_SUPPORTED;
        const int64_t grid = std::min<int64_t>(ceildiv(nblk, int64_t(csize)), nclusters) * csize;
        cfg.gridDim = dim3(unsigned(grid));
        const int pidx = prof_begin(SLT_PROF_SWEEP, s);
        SLT_CUDA_TRY(cudaLaunchKernelEx(&cfg, fn16, n, int(nrhs), reinterpret_cast<const float*>(M), ldm,
                                        reinterpret_cast<const float*>(Dinv), reinterpret_cast<float*>(X), ldx,
                                        flags, mb, xr, done, status, vec));
        count_launch();
        prof_end(pidx, s, double(n) * double(n) * double(nrhs), sizeof(T) * (double(n) * double(n) / 2 + 2.0 * n * nrhs));
        return slt_from_cuda(cudaGetLastError());
    }
    auto fn = sweep_kernel<T, FORWARD, UNIT, TRANS>;
    const size_t smem = sizeof(SweepSmem<T>);
    SLT_SMEM_ONCE(fn, smem);
    int dev = 0, sms = 0, per = 0;
    SLT_CUDA_TRY(cudaGetDevice(&dev));
    SLT_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    SLT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, 256, smem));
    const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(nblk, int64_t(sms) * std::max(per, 1)));
    const int pidx = prof_begin(SLT_PROF_SWEEP, s);
    fn<<<unsigned(grid), 256, smem, s>>>(n, int(nrhs), M, ldm, Dinv, X, ldx, flags, mb, status);
    count_launch();
    prof_end(pidx, s, double(n) * double(n) * double(nrhs), sizeof(T) * (double(n) * double(n) / 2 + 2.0 * n * nrhs));
    return slt_from_cuda(cudaGetLastError());
}

} // namespace slt

using namespace slt;

// flags: device scratch of slt_sweep_flags_bytes(n) bytes; status: device int (timeouts).
// kind: 0 unit lower (L of LU), 1 upper non-unit (U of LU), 2 lower
// non-unit (L of Cholesky), 3 lower^T non-unit (L^T of Cholesky), 4 upper^T
// non-unit (U^T of LU), 5 unit lower^T (L^T of LU).
extern "C" int slt_dsweep(int kind, int64_t n, int64_t nrhs, const double* M, int64_t ldm, double* X,
                          int64_t ldx, int* flags, int* status, cudaStream_t s)
{
    switch (kind) {
        case 0: return launch_sweep<double, true, true, false>(n, nrhs, M, ldm, X, ldx, flags, status, s);
        case 1: return launch_sweep<double, false, false, false>(n, nrhs, M, ldm, X, ldx, flags, status, s);
        case 2: return launch_sweep<double, true, false, false>(n, nrhs, M, ldm, X, ldx, flags, status, s);
        case 3: return launch_sweep<double, false, false, true>(n, nrhs, M, ldm, X, ldx, flags, status, s);
        case 4: return launch_sweep<double, true, false, true>(n, nrhs, M, ldm, X, ldx, flags, status, s);
        case 5: return launch_sweep<double, false, true, true>(n, nrhs, M, ldm, X, ldx, flags, status, s);
        default: return SLT_ERR_ARG;
    }
}

extern "C" int slt_ssweep(int kind, int64_t n, int64_t nrhs, const float* M, int64_t ldm, float* X,
                          int64_t ldx, int* flags, int* status, cudaStream_t s)
{
    switch (kind) {
        case 0: return launch_sweep<float, true, true, false>(n, nrhs, M, ldm, X, ldx, flags, status, s);
        case 1: return launch_sweep<float, false, false, false>(n, nrhs, M, ldm, X, ldx, flags, status, s);
        case 2: return launch_sweep<float, true, false, false>(n, nrhs, M, ldm, X, ldx, flags, status, s);
        case 3: return launch_sweep<float, false, false, true>(n, nrhs, M, ldm, X, ldx, flags, status, s);
        case 4: return launch_sweep<float, true, false, true>(n, nrhs, M, ldm, X, ldx, flags, status, s);
        case 5: return launch_sweep<float, false, true, true>(n, nrhs, M, ldm, X, ldx, flags, status, s);
        default: return SLT_ERR_ARG;
    }
}

// Scratch of one sweep: ticket, mailbox of solved values, diagonal-block
// inverses and chain-step blocks W (sized for double).
extern "C" size_t slt_sweep_flags_bytes(int64_t n)
{
    const int64_t nblk = ceildiv(n, kSwBS);
    return 256 + size_t(kSwRhs) * size_t(nblk) * kSwBS * 2 * 8 + 2 * size_t(nblk) * kSwBS * kSwBS * sizeof(double) +
           size_t(nblk) * kSwBS * kSwRhs * sizeof(float) + size_t(nblk) * sizeof(int);
}

