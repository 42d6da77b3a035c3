// arnoldi.cu -- the classical Gram-Schmidt steps (CGS2) of the block FGMRES,
// batched over the columns that are in an Arnoldi step.
//
// SLATE's gesv_mixed_gmres orthogonalises w against V(:, 0:j) twice with
// gemm (src/gesv_mixed_gmres.cc:300-330): h = V^T w, w -= V h, z = V^T w,
// w -= V z, then ||w||.  Each column of the block iteration has its own basis
// V_q (n x R1, column-major, slot q of the basis store), so the products are
// tall and skinny (n x (j + 1) with j + 1 <= 31): one launch per product and
// column would be a few hundred small launches per step, each a single
// reduction over n.  Here one launch covers every active column: the dot
// products are split over row segments into partial sums (fixed order, so
// the result is deterministic), and the update kernel first adds a column's
// partials, then subtracts V_q h from its rows; the second update also
// leaves the partial sums of squares for ||w||.

#include "common.cuh"
#include "prof.h"
#include "slate_gb300.h"

namespace slt {

constexpr int kCgsMaxR = 32;
constexpr int kCgsThreads = 256;

// Partial dot products of column i's new vector with V_q(:, 0:j):
// partial[(i * nseg + seg) * R1 + r].  With src (pass 0) the new vector is
// taken as -src(:, i) and written to V_q(:, j + 1) on the way.
__global__ void __launch_bounds__(kCgsThreads)
cgs_dots_kernel(int64_t n, double* V, int64_t R1, slt_cgs_cols c, const double* __restrict__ src,
                int64_t rps, double* partial)
{
    const int i = blockIdx.y, seg = blockIdx.x, nseg = gridDim.x;
    const int q = c.q[i], j = c.j[i];
    double* Vq = V + int64_t(q) * n * R1;
    double* v = Vq + int64_t(j + 1) * n;
    const double* s = src ? src + int64_t(i) * n : nullptr;
    double acc[kCgsMaxR];
    #pragma unroll
    for (int r = 0; r < kCgsMaxR; ++r) acc[r] = 0.0;
    const int64_t k0 = int64_t(seg) * rps;
    const int64_t k1 = k0 + rps < n ? k0 + rps : n;
    for (int64_t k = k0 + threadIdx.x; k < k1; k += kCgsThreads) {
        double vk;
        if (s) {
            vk = -s[k];
            v[k] = vk;
        }
        else {
            vk = v[k];
        }
        #pragma unroll
        for (int r = 0; r < kCgsMaxR; ++r)
            if (r <= j) acc[r] = fma(Vq[k + int64_t(r) * n], vk, acc[r]);
    }
    __shared__ double red[kCgsThreads / 32][kCgsMaxR];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    #pragma unroll
    for (int r = 0; r < kCgsMaxR; ++r) {
        double t = acc[r];
        #pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) red[warp][r] = t;
    }
    __syncthreads();
    if (threadIdx.x <= j) {
        double t = 0.0;
        for (int w = 0; w < kCgsThreads / 32; ++w) t += red[w][threadIdx.x];
        partial[(int64_t(i) * nseg + seg) * R1 + threadIdx.x] = t;
    }
}

// h = sum over segments of the partials (written to scal[q * SC + out + r]
// by the first block of the column), then V_q(:, j + 1) -= V_q(:, 0:j) h on
// this block's rows.  With sq, the block's partial sum of squares of the
// updated vector goes to sq[i * gridDim.x + blockIdx.x].
__global__ void __launch_bounds__(kCgsThreads)
cgs_update_kernel(int64_t n, double* V, int64_t R1, slt_cgs_cols c, int nseg, const double* __restrict__ partial,
                  double* scal, int64_t SC, int out, int64_t rps, double* sq)
{
    const int i = blockIdx.y;
    const int q = c.q[i], j = c.j[i];
    __shared__ double h[kCgsMaxR];
    __shared__ double red[kCgsThreads / 32];
    if (threadIdx.x <= j) {
        double t = 0.0;
        for (int s = 0; s < nseg; ++s) t += partial[(int64_t(i) * nseg + s) * R1 + threadIdx.x];
        h[threadIdx.x] = t;
        if (blockIdx.x == 0) scal[int64_t(q) * SC + out + threadIdx.x] = t;
    }
    __syncthreads();
    double* Vq = V + int64_t(q) * n * R1;
    double* v = Vq + int64_t(j + 1) * n;
    const int64_t k0 = int64_t(blockIdx.x) * rps;
    const int64_t k1 = k0 + rps < n ? k0 + rps : n;
    double ss = 0.0;
    for (int64_t k = k0 + threadIdx.x; k < k1; k += kCgsThreads) {
        double t = v[k];
        #pragma unroll
        for (int r = 0; r < kCgsMaxR; ++r)
            if (r <= j) t = fma(-Vq[k + int64_t(r) * n], h[r], t);
        v[k] = t;
        ss = fma(t, t, ss);
    }
    if (sq) {
        #pragma unroll
        for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = ss;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int w = 0; w < kCgsThreads / 32; ++w) t += red[w];
            sq[int64_t(i) * gridDim.x + blockIdx.x] = t;
        }
    }
}

// scal[q * SC + 3] = sqrt(sum of column i's partial sums of squares).
__global__ void cgs_norm_kernel(slt_cgs_cols c, int nblk, const double* __restrict__ sq, double* scal, int64_t SC)
{
    const int i = threadIdx.x;
    if (i >= c.na) return;
    double t = 0.0;
    for (int b = 0; b < nblk; ++b) t += sq[int64_t(i) * nblk + b];
    scal[int64_t(c.q[i]) * SC + 3] = sqrt(t);
}

static int cgs_segments(int64_t n, int na, int64_t* rps)
{
    // about four blocks per SM over all columns, at least 1024 rows a block
    int dev = 0, sms = 148;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaGetLastError();
    int64_t nseg = std::max<int64_t>(1, (4 * int64_t(sms) + na - 1) / std::max(na, 1));
    nseg = std::min<int64_t>(nseg, std::max<int64_t>(1, n / 1024));
    nseg = std::min<int64_t>(nseg, kSltCgsMaxSeg);
    *rps = ceildiv(n, nseg);
    return int(ceildiv(n, *rps));
}

} // namespace slt

using namespace slt;

extern "C" size_t slt_cgs_ws_bytes(int64_t R1)
{
    return size_t(kSltCgsMaxSeg) * kSltCgsMaxCols * size_t(R1 + 1) * sizeof(double) + 256;
}

// CGS2 of every column in c: V_q(:, j+1) = -W(:, i), then twice
// h = V_q(:, 0:j)^T v, v -= V_q(:, 0:j) h (h to scal[q SC + 4 ..] and
// scal[q SC + 4 + R1 ..]), and ||v|| to scal[q SC + 3].
extern "C" int slt_dcgs2(int64_t n, double* V, int64_t R1, const slt_cgs_cols* cols, const double* W, double* scal,
                         int64_t SC, void* ws, cudaStream_t stream)
{
    if (!cols || cols->na <= 0) return SLT_OK;
    if (cols->na > kSltCgsMaxCols || R1 > kCgsMaxR || n <= 0) return SLT_ERR_ARG;
    for (int i = 0; i < cols->na; ++i)
        if (cols->j[i] < 0 || cols->j[i] + 1 >= R1) return SLT_ERR_ARG;
    const slt_cgs_cols c = *cols;
    int64_t rps = 0;
    const int nseg = cgs_segments(n, c.na, &rps);
    double* partial = static_cast<double*>(ws);
    double* sq = partial + size_t(kSltCgsMaxSeg) * kSltCgsMaxCols * size_t(R1);
    const dim3 grid(unsigned(nseg), unsigned(c.na));
    for (int pass = 0; pass < 2; ++pass) {
        cgs_dots_kernel<<<grid, kCgsThreads, 0, stream>>>(n, V, R1, c, pass == 0 ? W : nullptr, rps, partial);
        count_launch();
        cgs_update_kernel<<<grid, kCgsThreads, 0, stream>>>(n, V, R1, c, nseg, partial, scal, SC,
                                                            int(4 + pass * R1), rps, pass == 1 ? sq : nullptr);
        count_launch();
    }
    cgs_norm_kernel<<<1, 32, 0, stream>>>(c, nseg, sq, scal, SC);
    count_launch();
    return slt_from_cuda(cudaGetLastError());
}
