// condest.cc -- reciprocal condition number estimates from the factors:
// slate::gecondest (src/gecondest.cc) and slate::pocondest (src/pocondest.cc).
//
// Both estimate ||A^{-1}|| in the 1-norm (or the infinity norm, as the 1-norm
// of A^{-T}) with Hager's method as refined by Higham (ACM TOMS 14, 1988,
// Algorithm 4.1; the estimator behind SLATE's internal::norm1est and LAPACK's
// xLACN2): at most five pairs of solves with A^{-1} and A^{-T}, each driven by
// the sign pattern / largest entry of the previous result, then one extra
// solve with an alternating vector as a safeguard.  The solves run on the
// device with the factors (getrs / potrs sweeps); the few n-vector
// operations between them run on the host.  rcond = 1 / (anorm * estimate).

#include "drivers.h"

#include <algorithm>
#include <cmath>
#include <vector>

using namespace slt;

namespace {

// Estimate of ||op1||_1 where op1 / op2 apply the inverse and its transpose
// to one device vector in place.
template <typename Op1, typename Op2>
int norm1_inverse_estimate(int64_t n, Op1 op1, Op2 op2, double* dv, cudaStream_t s, double* est_out)
{
    const size_t nn = static_cast<size_t>(n);
    std::vector<double> x(nn, 0.0), y(nn, 0.0), sgn(nn, 0.0);
    auto run = [&](auto& op, std::vector<double>& v) -> int {
        SLT_CUDA_TRY(cudaMemcpyAsync(dv, v.data(), sizeof(double) * size_t(n), cudaMemcpyHostToDevice, s));
        TRY(op(dv));
        SLT_CUDA_TRY(cudaMemcpyAsync(v.data(), dv, sizeof(double) * size_t(n), cudaMemcpyDeviceToHost, s));
        SLT_CUDA_TRY(cudaStreamSynchronize(s));
        return SLT_OK;
    };
    auto norm1 = [&](const std::vector<double>& v) {
        double a = 0.0;
        for (double e : v) a += std::fabs(e);
        return a;
    };
    auto argmax = [&](const std::vector<double>& v) {
        int64_t j = 0;
        for (int64_t i = 1; i < n; ++i)
            if (std::fabs(v[size_t(i)]) > std::fabs(v[size_t(j)])) j = i;
        return j;
    };
    // start from the uniform vector
    for (auto& e : x) e = 1.0 / double(n);
    y = x;
    TRY(run(op1, y));
    double est = norm1(y);
    if (n == 1) { *est_out = est; return SLT_OK; }
    for (int64_t i = 0; i < n; ++i) sgn[size_t(i)] = (y[size_t(i)] >= 0.0) ? 1.0 : -1.0;
    std::vector<double> z = sgn;
    TRY(run(op2, z));
    int64_t j = argmax(z);
    for (int iter = 2; iter <= 5; ++iter) {
        std::fill(x.begin(), x.end(), 0.0);
        x[size_t(j)] = 1.0;
        y = x;
        TRY(run(op1, y));
        const double est_old = est;
        est = norm1(y);
        bool same = true;
        for (int64_t i = 0; i < n && same; ++i)
            same = ((y[size_t(i)] >= 0.0) ? 1.0 : -1.0) == sgn[size_t(i)];
        if (same || est <= est_old) break;   // converged, or cycling
        for (int64_t i = 0; i < n; ++i) sgn[size_t(i)] = (y[size_t(i)] >= 0.0) ? 1.0 : -1.0;
        z = sgn;
        TRY(run(op2, z));
        const int64_t jlast = j;
        j = argmax(z);
        if (std::fabs(z[size_t(jlast)]) == std::fabs(z[size_t(j)])) break;
    }
    // safeguard: alternating vector with growing magnitude
    double alt = 1.0;
    for (int64_t i = 0; i < n; ++i) {
        x[size_t(i)] = alt * (1.0 + double(i) / double(n - 1));
        alt = -alt;
    }
    TRY(run(op1, x));
    const double temp = 2.0 * norm1(x) / (3.0 * double(n));
    *est_out = std::max(est, temp);
    return SLT_OK;
}

int finish_rcond(double anorm, double est, double* rcond)
{
    *rcond = (anorm > 0.0 && est > 0.0 && std::isfinite(est)) ? 1.0 / anorm / est : 0.0;
    return SLT_OK;
}

}  // namespace

// slate::gecondest: LU factors (getrf output, per-panel pivots), norm '1' or
// 'I' (SLATE's Norm::One / Norm::Inf), anorm = ||A|| in that norm.
extern "C" int slt_dgecondest_device(char norm, int64_t n, const double* dLU, int64_t lda, const int* d_ipiv,
                                     double anorm, double* rcond, const slt_options* opts, slt_stream_t stream)
{
    if (!rcond || n < 0 || lda < std::max<int64_t>(1, n)) return SLT_ERR_ARG;
    const bool one = (norm == '1' || norm == 'O' || norm == 'o');
    if (!one && norm != 'I' && norm != 'i') return SLT_ERR_ARG;
    *rcond = 0.0;
    if (n == 0) { *rcond = 1.0; return SLT_OK; }
    if (anorm == 0.0) return SLT_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    DevBuf v;
    TRY(v.alloc(sizeof(double) * size_t(n), s));
    auto solve_n = [&](double* x) { return slt_dgetrs_trans_device('N', n, 1, dLU, lda, d_ipiv, x, n, opts, s); };
    auto solve_t = [&](double* x) { return slt_dgetrs_trans_device('T', n, 1, dLU, lda, d_ipiv, x, n, opts, s); };
    double est = 0.0;
    if (one) TRY(norm1_inverse_estimate(n, solve_n, solve_t, v.as<double>(), s, &est));
    else TRY(norm1_inverse_estimate(n, solve_t, solve_n, v.as<double>(), s, &est));
    return finish_rcond(anorm, est, rcond);
}

// slate::pocondest: lower Cholesky factor (potrf output), norm '1' or 'I'
// (equal for a symmetric matrix), anorm = ||A||.
extern "C" int slt_dpocondest_device(char norm, int64_t n, const double* dL, int64_t lda, double anorm,
                                     double* rcond, const slt_options* opts, slt_stream_t stream)
{
    if (!rcond || n < 0 || lda < std::max<int64_t>(1, n)) return SLT_ERR_ARG;
    if (norm != '1' && norm != 'O' && norm != 'o' && norm != 'I' && norm != 'i') return SLT_ERR_ARG;
    *rcond = 0.0;
    if (n == 0) { *rcond = 1.0; return SLT_OK; }
    if (anorm == 0.0) return SLT_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    DevBuf v;
    TRY(v.alloc(sizeof(double) * size_t(n), s));
    auto solve = [&](double* x) { return slt_dpotrs_device(n, 1, dL, lda, x, n, opts, s); };
    double est = 0.0;
    TRY(norm1_inverse_estimate(n, solve, solve, v.as<double>(), s, &est));
    return finish_rcond(anorm, est, rcond);
}
