// equil.cu -- equilibration of A before the low-precision cast, and the
// scaled FP64 <-> FP32 conversions that apply it.
//
// FP16 keeps 5 exponent bits (normal range 6.1e-5 .. 65504) and BF16 keeps
// only 8 mantissa bits, so an FP64 matrix whose rows or columns differ in
// scale by a few orders of magnitude loses its small entries, or overflows,
// once a trailing update casts a panel to 16 bits.  The mixed solvers
// therefore factor  A_s = R A C  (general; R, C diagonal) or  D A D  (SPD)
// and solve  A x = b  as  x = C A_s^{-1} (R b).  Every scale is a power of
// two, so scaling is exact in every precision and the FP64 residual of the
// refinement still uses the unscaled A.
//
// Scales follow LAPACK's dgeequb / dpoequb: r_i = 2^-e with e the exponent
// of max_j |a_ij| (so that max_j |r_i a_ij| is in [0.5, 1)), then
// c_j = 2^-e of max_i |r_i a_ij|; for SPD matrices d_i = 2^-ceil(e_i / 2)
// with e_i the exponent of a_ii, so that d_i^2 a_ii is in [0.25, 1).  A zero
// (or non-finite) row, column or diagonal keeps scale 1; the factorisation
// then reports it.

#include "common.cuh"
#include "prof.h"

namespace slt {

// 2^-e for x = m 2^e, m in [0.5, 1); 1 for x = 0, NaN or Inf.
__device__ __forceinline__ double pow2_inv_scale(double x)
{
    if (!(x > 0.0) || isinf(x)) return 1.0;
    int e;
    frexp(x, &e);
    return ldexp(1.0, -e);
}

// Row maxima of |A| (m x n): thread per row, 64 columns per block row of the
// grid, combined with an atomic max on the bit pattern (non-negative doubles
// order like their bits).
__global__ void rowmax_abs_kernel(int64_t m, int64_t n, const double* __restrict__ A, int64_t lda,
                                  unsigned long long* __restrict__ rmax)
{
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int64_t j0 = int64_t(blockIdx.y) * 64;
    const int64_t j1 = min64(n, j0 + 64);
    double mx = 0.0;
    for (int64_t j = j0; j < j1; ++j) {
        const double v = fabs(A[i + j * lda]);
        mx = v > mx ? v : mx;
    }
    if (mx > 0.0) atomicMax(&rmax[i], __double_as_longlong(mx));
}

__global__ void row_scale_kernel(int64_t m, unsigned long long* rmax_bits, double* r)
{
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < m) r[i] = pow2_inv_scale(__longlong_as_double(static_cast<long long>(rmax_bits[i])));
}

// Column scales c_j from max_i |r_i a_ij|: one block per column.
__global__ void col_scale_kernel(int64_t m, const double* __restrict__ A, int64_t lda,
                                 const double* __restrict__ r, double* __restrict__ c)
{
    __shared__ double red[32];
    const int64_t j = blockIdx.x;
    double mx = 0.0;
    for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
        const double v = fabs(r[i] * A[i + j * lda]);
        mx = v > mx ? v : mx;
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x < 32) {
        mx = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if (threadIdx.x == 0) c[j] = pow2_inv_scale(mx);
    }
}

__global__ void sym_scale_kernel(int64_t n, const double* __restrict__ A, int64_t lda, double* __restrict__ d)
{
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double a = A[i + i * lda];
    double s = 1.0;
    if (a > 0.0 && !isinf(a)) {
        int e;
        frexp(a, &e);
        s = ldexp(1.0, -((e + (e > 0 ? 1 : 0)) / 2));   // 2^-ceil(e/2)
    }
    d[i] = s;
}

// x 2^k without a floating-point multiply (the FP64 pipe is the slow one on
// this part): add k to the exponent field when x and the result are normal
// numbers; zeros, subnormals, Inf/NaN and out-of-range results take the
// multiply.
__device__ __forceinline__ double scale_pow2(double x, int k)
{
    const long long b = __double_as_longlong(x);
    const int e = int((b >> 52) & 0x7ff);
    if (e == 0 || e == 0x7ff || e + k <= 0 || e + k >= 0x7ff) return x * ldexp(1.0, k);
    return __longlong_as_double(b + (static_cast<long long>(k) << 52));
}

// k of a power-of-two scale 2^k (the scales above are exact powers of two)
__device__ __forceinline__ int pow2_exponent(double s)
{
    return int((__double_as_longlong(s) >> 52) & 0x7ff) - 1023;
}

// B = D(r_i * A_ij * c_j); SCALED = false: B = D(A) (r, c unused).  Each
// thread handles four rows of one column (1024 rows per block), so that every
// warp keeps four coalesced loads in flight.
// LOWER: only the lower triangle (i >= j) is read and written.
template <typename S, typename D, bool SCALED, bool LOWER = false>
__global__ void convert_scaled_kernel(int64_t m, int64_t n, const S* __restrict__ A, int64_t lda,
                                      const double* __restrict__ r, const double* __restrict__ c,
                                      D* __restrict__ B, int64_t ldb)
{
    const int64_t i0 = int64_t(blockIdx.x) * 1024 + threadIdx.x;
    const int64_t jend = LOWER ? min64(n, int64_t(blockIdx.x) * 1024 + 1024) : n;
    for (int64_t j = blockIdx.y; j < jend; j += gridDim.y) {
        const int kc = (SCALED && c) ? pow2_exponent(c[j]) : 0;
        S v[4];
        #pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int64_t i = i0 + 256 * k;
            v[k] = (i < m && (!LOWER || i >= j)) ? A[i + j * lda] : S(0);
        }
        #pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int64_t i = i0 + 256 * k;
            if (i < m && (!LOWER || i >= j)) {
                if (SCALED) B[i + j * ldb] = D(scale_pow2(double(v[k]), (r ? pow2_exponent(r[i]) : 0) + kc));
                else B[i + j * ldb] = D(v[k]);
            }
        }
    }
}

} // namespace slt

using namespace slt;

// Row and column scales of a general m x n matrix (dgeequb semantics, powers
// of two).  ws: m 8-byte words.
extern "C" int slt_dgeequ(int64_t m, int64_t n, const double* A, int64_t lda, double* r, double* c,
                          void* ws, cudaStream_t stream)
{
    if (m <= 0 || n <= 0) return SLT_OK;
    if (lda < m) return SLT_ERR_ARG;
    auto* bits = static_cast<unsigned long long*>(ws);
    SLT_CUDA_TRY(cudaMemsetAsync(bits, 0, sizeof(unsigned long long) * size_t(m), stream));
    dim3 g(unsigned(ceildiv(m, 256)), unsigned(ceildiv(n, 64)));
    rowmax_abs_kernel<<<g, 256, 0, stream>>>(m, n, A, lda, bits);
    count_launch();
    row_scale_kernel<<<unsigned(ceildiv(m, 256)), 256, 0, stream>>>(m, bits, r);
    count_launch();
    col_scale_kernel<<<unsigned(n), 256, 0, stream>>>(m, A, lda, r, c);
    count_launch();
    return slt_from_cuda(cudaGetLastError());
}

// Symmetric scales d_i = 2^-ceil(e_i/2) from the diagonal (dpoequb).
extern "C" int slt_dpoequ(int64_t n, const double* A, int64_t lda, double* d, cudaStream_t stream)
{
    if (n <= 0) return SLT_OK;
    if (lda < n) return SLT_ERR_ARG;
    sym_scale_kernel<<<unsigned(ceildiv(n, 256)), 256, 0, stream>>>(n, A, lda, d);
    count_launch();
    return slt_from_cuda(cudaGetLastError());
}

// B (float) = diag(r) A diag(c); r or c may be null.
extern "C" int slt_convert_d2s_scaled(int64_t m, int64_t n, const double* A, int64_t lda, const double* r,
                                      const double* c, float* B, int64_t ldb, cudaStream_t stream)
{
    if (m <= 0 || n <= 0) return SLT_OK;
    dim3 g(unsigned(ceildiv(m, 1024)), unsigned(std::min<int64_t>(n, 65535)));
    if (r || c) convert_scaled_kernel<double, float, true><<<g, 256, 0, stream>>>(m, n, A, lda, r, c, B, ldb);
    else convert_scaled_kernel<double, float, false><<<g, 256, 0, stream>>>(m, n, A, lda, r, c, B, ldb);
    count_launch();
    return slt_from_cuda(cudaGetLastError());
}

// The lower triangle of B (float, n x n) = diag(d) A diag(d) on the lower
// triangle of A; d may be null.  The strictly upper part of B is not written.
extern "C" int slt_convert_d2s_scaled_lower(int64_t n, const double* A, int64_t lda, const double* d, float* B,
                                            int64_t ldb, cudaStream_t stream)
{
    if (n <= 0) return SLT_OK;
    dim3 g(unsigned(ceildiv(n, 1024)), unsigned(std::min<int64_t>(n, 65535)));
    if (d) convert_scaled_kernel<double, float, true, true><<<g, 256, 0, stream>>>(n, n, A, lda, d, d, B, ldb);
    else convert_scaled_kernel<double, float, false, true><<<g, 256, 0, stream>>>(n, n, A, lda, d, d, B, ldb);
    count_launch();
    return slt_from_cuda(cudaGetLastError());
}

// Columns [j0, j1), rows [j0, n) of the same (the lower part of one block of
// columns): the streaming form of the cast above.
extern "C" int slt_convert_d2s_scaled_lower_cols(int64_t n, int64_t j0, int64_t j1, const double* A, int64_t lda,
                                                 const double* d, float* B, int64_t ldb, cudaStream_t stream)
{
    if (j0 >= j1 || j0 >= n) return SLT_OK;
    const int64_t m = n - j0, nc = j1 - j0;
    dim3 g(unsigned(ceildiv(m, 1024)), unsigned(std::min<int64_t>(nc, 65535)));
    const double* dd = d ? d + j0 : nullptr;
    if (d) convert_scaled_kernel<double, float, true, true><<<g, 256, 0, stream>>>(m, nc, A + j0 + j0 * lda, lda, dd, dd,
                                                                                B + j0 + j0 * ldb, ldb);
    else convert_scaled_kernel<double, float, false, true><<<g, 256, 0, stream>>>(m, nc, A + j0 + j0 * lda, lda, dd, dd,
                                                                                B + j0 + j0 * ldb, ldb);
    count_launch();
    return slt_from_cuda(cudaGetLastError());
}

// X (double) = diag(r) B; r may be null.
extern "C" int slt_convert_s2d_scaled(int64_t m, int64_t n, const float* B, int64_t ldb, const double* r,
                                      double* X, int64_t ldx, cudaStream_t stream)
{
    if (m <= 0 || n <= 0) return SLT_OK;
    dim3 g(unsigned(ceildiv(m, 1024)), unsigned(std::min<int64_t>(n, 65535)));
    if (r) convert_scaled_kernel<float, double, true><<<g, 256, 0, stream>>>(m, n, B, ldb, r, nullptr, X, ldx);
    else convert_scaled_kernel<float, double, false><<<g, 256, 0, stream>>>(m, n, B, ldb, r, nullptr, X, ldx);
    count_launch();
    return slt_from_cuda(cudaGetLastError());
}
