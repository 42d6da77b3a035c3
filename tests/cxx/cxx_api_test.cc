// Exercises the header-only C++ API (slate_gb300.hh) the way a SLATE caller
// would: build device matrices, gesv / posv / posv_mixed / getrf + getrs,
// check residuals on the host.  Prints "OK" and exits 0 on success.
#include "slate_gb300.hh"

#include <cuda_runtime.h>
#include <cmath>
#include <cstdio>
#include <vector>

namespace sg = slate_gb300;

static double lcg(uint64_t& s) { s = s * 6364136223846793005ull + 1442695040888963407ull; return double(s >> 11) / 9007199254740992.0 - 0.5; }

static double resid(const std::vector<double>& A, const std::vector<double>& X, const std::vector<double>& B, int n, int r)
{
    double worst = 0, an = 0, xn = 0;
    for (int j = 0; j < n; ++j) { double s = 0; for (int i = 0; i < n; ++i) s += std::fabs(A[i + j * n]); an = std::max(an, s); }
    for (int q = 0; q < r; ++q) {
        double rn = 0, xs = 0;
        for (int i = 0; i < n; ++i) {
            double v = B[i + q * n];
            for (int j = 0; j < n; ++j) v -= A[i + j * n] * X[j + q * n];
            rn += std::fabs(v);
            xs += std::fabs(X[i + q * n]);
        }
        worst = std::max(worst, rn); xn = std::max(xn, xs);
    }
    return worst / (n * an * xn);
}

int main()
{
    const int n = 300, r = 2, nb = 64;
    uint64_t seed = 7;
    std::vector<double> A(size_t(n) * n), S(size_t(n) * n), B(size_t(n) * r);
    for (auto& v : A) v = lcg(seed);
    for (auto& v : B) v = lcg(seed);
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
            double s = 0;
            for (int k = 0; k < n; ++k) s += A[i + k * n] * A[j + k * n];
            S[i + j * n] = s / n + (i == j ? 1.0 : 0.0);
        }
    double *dA, *dS, *dB, *dX;
    cudaMalloc(&dA, sizeof(double) * A.size()); cudaMalloc(&dS, sizeof(double) * S.size());
    cudaMalloc(&dB, sizeof(double) * B.size()); cudaMalloc(&dX, sizeof(double) * B.size());
    std::vector<double> X(B.size());
    const double eps = 2.220446049250313e-16;
    try {
        // gesv
        cudaMemcpy(dA, A.data(), sizeof(double) * A.size(), cudaMemcpyHostToDevice);
        cudaMemcpy(dB, B.data(), sizeof(double) * B.size(), cudaMemcpyHostToDevice);
        auto mA = sg::Matrix<double>::fromDevices(n, n, &dA, 1, n, nb);
        auto mB = sg::Matrix<double>::fromDevices(n, r, &dB, 1, n, nb);
        sg::Pivots piv;
        if (sg::gesv(mA, piv, mB, {{sg::Option::InnerBlocking, int64_t(32)}}) != 0) return 2;
        cudaMemcpy(X.data(), dB, sizeof(double) * X.size(), cudaMemcpyDeviceToHost);
        if (!(resid(A, X, B, n, r) <= 3 * eps)) { std::printf("gesv residual %g\n", resid(A, X, B, n, r)); return 3; }
        if (piv.size() != size_t((n + nb - 1) / nb)) return 4;
        // getrs with the returned pivots on the factors
        cudaMemcpy(dB, B.data(), sizeof(double) * B.size(), cudaMemcpyHostToDevice);
        sg::getrs(mA, piv, mB);
        cudaMemcpy(X.data(), dB, sizeof(double) * X.size(), cudaMemcpyDeviceToHost);
        if (!(resid(A, X, B, n, r) <= 3 * eps)) return 5;
        // posv and posv_mixed
        cudaMemcpy(dS, S.data(), sizeof(double) * S.size(), cudaMemcpyHostToDevice);
        cudaMemcpy(dB, B.data(), sizeof(double) * B.size(), cudaMemcpyHostToDevice);
        auto mS = sg::HermitianMatrix<double>::fromDevices(sg::Uplo::Lower, n, &dS, 1, n, nb);
        auto mX = sg::Matrix<double>::fromDevices(n, r, &dX, 1, n, nb);
        int iter = -99;
        if (sg::posv_mixed(mS, mB, mX, iter, {{sg::Option::MaxIterations, int64_t(30)}}) != 0 || iter < 0) return 6;
        cudaMemcpy(X.data(), dX, sizeof(double) * X.size(), cudaMemcpyDeviceToHost);
        if (!(resid(S, X, B, n, r) <= 3 * n * eps)) return 7;
        if (sg::posv(mS, mB) != 0) return 8;
        cudaMemcpy(X.data(), dB, sizeof(double) * X.size(), cudaMemcpyDeviceToHost);
        if (!(resid(S, X, B, n, r) <= 3 * eps)) return 9;
        // errors surface as exceptions
        bool threw = false;
        try { (void) sg::Matrix<double>::fromLAPACK(n, n, dA, n, nb, 2, 1); } catch (const sg::Exception&) { threw = true; }
        if (!threw) return 10;
    } catch (const std::exception& e) {
        std::printf("exception: %s\n", e.what());
        return 11;
    }
    std::printf("OK\n");
    return 0;
}
