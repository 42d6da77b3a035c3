// Exercises the tile storage of the header-only C++ API (slate_gb300.hh) the
// way SLATE callers build matrices: host-origin fromLAPACK, tile-by-tile
// insertLocalTiles on the host and on the device, user-owned tiles in
// separate allocations, MOSI state changes, complex and single precision,
// Upper Hermitian storage.  Every driver runs on the GPU.  Prints "OK" and
// exits 0 on success; a non-zero exit code names the failed check.
#include "slate_gb300.hh"

#include <cmath>
#include <complex>
#include <cstdio>
#include <vector>

namespace sg = slate_gb300;

template <typename T> static double mag(T v) { return std::abs(v); }
static double cj(double v) { return v; }
static float cj(float v) { return v; }
static std::complex<double> cj(std::complex<double> v) { return std::conj(v); }

static uint64_t g_seed = 11;
static double lcg() { g_seed = g_seed * 6364136223846793005ull + 1442695040888963407ull; return double(g_seed >> 11) / 9007199254740992.0 - 0.5; }
template <typename T> static T rnd();
template <> double rnd<double>() { return lcg(); }
template <> float rnd<float>() { return float(lcg()); }
template <> std::complex<double> rnd<std::complex<double>>() { double a = lcg(); return {a, lcg()}; }

// ||B - A X||_1 / (n ||A||_1 ||X||_1) over column-major host arrays
template <typename T>
static double resid(const std::vector<T>& A, const std::vector<T>& X, const std::vector<T>& B, int n, int r)
{
    double an = 0, xn = 0, rn = 0;
    for (int j = 0; j < n; ++j) { double s = 0; for (int i = 0; i < n; ++i) s += mag(A[i + j * n]); an = std::max(an, s); }
    for (int q = 0; q < r; ++q) {
        double rs = 0, xs = 0;
        for (int i = 0; i < n; ++i) {
            T v = B[i + q * n];
            for (int j = 0; j < n; ++j) v -= A[i + j * n] * X[j + q * n];
            rs += mag(v);
            xs += mag(X[i + q * n]);
        }
        rn = std::max(rn, rs); xn = std::max(xn, xs);
    }
    return rn / (n * an * xn);
}

template <typename T>
static std::vector<T> hpd(int n)
{
    std::vector<T> G(size_t(n) * n), S(size_t(n) * n);
    for (auto& v : G) v = rnd<T>();
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
            T s = T(0);
            for (int k = 0; k < n; ++k) s += G[i + k * n] * cj(G[j + k * n]);
            S[i + j * n] = s / T(double(n)) + (i == j ? T(1) : T(0));
        }
    return S;
}

// the host tiles of M as one column-major array
template <typename T>
static std::vector<T> gather(sg::BaseMatrix<T>& M, int device)
{
    std::vector<T> out(size_t(M.m()) * M.n());
    for (int64_t j = 0; j < M.nt(); ++j)
        for (int64_t i = 0; i < M.mt(); ++i) {
            M.tileGetForReading(i, j, sg::HostNum);
            auto t = M(i, j, sg::HostNum);
            for (int64_t jj = 0; jj < t.nb(); ++jj)
                for (int64_t ii = 0; ii < t.mb(); ++ii)
                    out[size_t(i * M.storage()->nb + ii) + size_t(j * M.storage()->nb + jj) * M.m()] = t(ii, jj);
        }
    (void) device;
    return out;
}

// fill M's tiles on `device` from a column-major host array
template <typename T>
static void scatter(sg::BaseMatrix<T>& M, const std::vector<T>& src, int device)
{
    const int64_t nb = M.storage()->nb;
    for (int64_t j = 0; j < M.nt(); ++j)
        for (int64_t i = 0; i < M.mt(); ++i) {
            auto t = M(i, j, device);
            sg::check(slt_memcpy2d(t.data(), size_t(t.stride()) * sizeof(T), src.data() + i * nb + j * nb * M.m(),
                                   size_t(M.m()) * sizeof(T), size_t(t.mb()) * sizeof(T), size_t(t.nb())));
            M.tileModified(i, j, device);
        }
}

int main()
{
    const int n = 300, r = 2, nb = 64;
    const double eps = 2.220446049250313e-16;
    try {
        std::vector<double> A(size_t(n) * n), B(size_t(n) * r);
        for (auto& v : A) v = rnd<double>();
        for (auto& v : B) v = rnd<double>();

        // 1. host memory, fromLAPACK: factors and solution come back to the host arrays
        {
            std::vector<double> a = A, b = B;
            auto mA = sg::Matrix<double>::fromLAPACK(n, n, a.data(), n, nb);
            auto mB = sg::Matrix<double>::fromLAPACK(n, r, b.data(), n, nb);
            sg::Pivots piv;
            if (sg::gesv(mA, piv, mB) != 0) return 10;
            if (!(resid(A, b, B, n, r) <= 3 * eps)) { std::printf("host gesv %g\n", resid(A, b, B, n, r)); return 11; }
            if (mA.tileState(0, 0, sg::HostNum) != sg::MOSI::Modified) return 12;
            // getrs from the host factors with the returned pivots
            std::vector<double> b2 = B;
            auto mB2 = sg::Matrix<double>::fromLAPACK(n, r, b2.data(), n, nb);
            sg::getrs(mA, piv, mB2);
            if (!(resid(A, b2, B, n, r) <= 3 * eps)) return 13;
        }
        // 2. tile by tile on the host (insertLocalTiles), filled element-wise
        {
            sg::Matrix<double> mA(n, n, nb, 1, 1), mB(n, r, nb, 1, 1);
            mA.insertLocalTiles(sg::Target::Host);
            mB.insertLocalTiles(sg::Target::HostTask);
            for (int64_t j = 0; j < mA.nt(); ++j)
                for (int64_t i = 0; i < mA.mt(); ++i) {
                    auto t = mA(i, j);
                    for (int64_t jj = 0; jj < t.nb(); ++jj)
                        for (int64_t ii = 0; ii < t.mb(); ++ii) t.at(ii, jj) = A[(i * nb + ii) + (j * nb + jj) * n];
                }
            scatter(mB, B, sg::HostNum);
            sg::Pivots piv;
            if (sg::gesv(mA, piv, mB) != 0) return 20;
            auto X = gather(mB, sg::HostNum);
            if (!(resid(A, X, B, n, r) <= 3 * eps)) return 21;
            auto E = mA.emptyLike();
            if (E.m() != n || E.n() != n || E.mt() != mA.mt() || E.tileExists(0, 0)) return 22;
        }
        // 3. tiles on the device (insertLocalTiles(Target::Devices)), Hermitian lower
        {
            auto S = hpd<double>(n);
            sg::HermitianMatrix<double> mS(sg::Uplo::Lower, n, nb, 1, 1);
            sg::Matrix<double> mB(n, r, nb, 1, 1);
            mS.insertLocalTiles(sg::Target::Devices);
            mB.insertLocalTiles(sg::Target::Devices);
            scatter(mS, S, 0);
            scatter(mB, B, 0);
            if (sg::posv(mS, mB) != 0) return 30;
            if (mB.tileState(0, 0, 0) != sg::MOSI::Modified) return 31;
            auto X = gather(mB, 0);             // device -> host workspace tiles
            if (!(resid(S, X, B, n, r) <= 3 * eps)) return 32;
            if (mB.tileState(0, 0, sg::HostNum) != sg::MOSI::Shared || mB.tileState(0, 0, 0) != sg::MOSI::Shared) return 33;
            mB.releaseWorkspace();
            if (mB.tileExists(0, 0, sg::HostNum) || !mB.tileExists(0, 0, 0)) return 34;
        }
        // 4. user-owned tiles in separate host allocations (tileInsert with data)
        {
            sg::Matrix<double> mA(n, n, nb, 1, 1), mB(n, r, nb, 1, 1);
            std::vector<std::vector<double>> store;
            for (int64_t j = 0; j < mA.nt(); ++j)
                for (int64_t i = 0; i < mA.mt(); ++i) {
                    const int64_t mb = mA.tileMb(i), tnb = mA.tileNb(j);
                    store.emplace_back(size_t(mb + 3) * tnb);          // ld = mb + 3
                    auto& v = store.back();
                    for (int64_t jj = 0; jj < tnb; ++jj)
                        for (int64_t ii = 0; ii < mb; ++ii) v[ii + jj * (mb + 3)] = A[(i * nb + ii) + (j * nb + jj) * n];
                    mA.tileInsert(i, j, sg::HostNum, v.data(), mb + 3);
                }
            mB.insertLocalTiles();
            scatter(mB, B, sg::HostNum);
            sg::Pivots piv;
            if (sg::gesv(mA, piv, mB) != 0) return 40;
            auto X = gather(mB, sg::HostNum);
            if (!(resid(A, X, B, n, r) <= 3 * eps)) return 41;
            // the user's tiles hold the factors: getrs with them solves again
            std::vector<double> b2 = B;
            auto mB2 = sg::Matrix<double>::fromLAPACK(n, r, b2.data(), n, nb);
            sg::getrs(mA, piv, mB2);
            if (!(resid(A, b2, B, n, r) <= 3 * eps)) return 42;
        }
        // 5. MOSI on a host-origin matrix
        {
            std::vector<double> a = A;
            auto mA = sg::Matrix<double>::fromLAPACK(n, n, a.data(), n, nb);
            mA.tileGetForWriting(1, 1, 0);
            if (mA.tileState(1, 1, 0) != sg::MOSI::Modified || mA.tileState(1, 1, sg::HostNum) != sg::MOSI::Invalid) return 50;
            std::vector<double> ones(size_t(nb) * nb, 1.0);
            auto t = mA(1, 1, 0);
            sg::check(slt_memcpy2d(t.data(), size_t(t.stride()) * 8, ones.data(), size_t(nb) * 8, size_t(nb) * 8, size_t(nb)));
            mA.tileUpdateOrigin(1, 1);
            if (a[nb + size_t(nb) * n] != 1.0 || mA.tileState(1, 1, sg::HostNum) != sg::MOSI::Shared) return 51;
        }
        // 6. complex<double>: host gesv, and posv with Upper storage (the lower triangle untouched)
        {
            using Z = std::complex<double>;
            std::vector<Z> Az(size_t(n) * n), Bz(size_t(n) * r);
            for (auto& v : Az) v = rnd<Z>();
            for (auto& v : Bz) v = rnd<Z>();
            std::vector<Z> a = Az, b = Bz;
            auto mA = sg::Matrix<Z>::fromLAPACK(n, n, a.data(), n, nb);
            auto mB = sg::Matrix<Z>::fromLAPACK(n, r, b.data(), n, nb);
            sg::Pivots piv;
            if (sg::gesv(mA, piv, mB) != 0) return 60;
            if (!(resid(Az, b, Bz, n, r) <= 3 * eps)) return 61;
            auto H = hpd<Z>(n);
            std::vector<Z> h = H;
            for (int j = 0; j < n; ++j)
                for (int i = j + 1; i < n; ++i) h[i + size_t(j) * n] = Z(7.0, 0.0);   // unreferenced marker
            std::vector<Z> b2 = Bz;
            auto mH = sg::HermitianMatrix<Z>::fromLAPACK(sg::Uplo::Upper, n, h.data(), n, nb);
            auto mB2 = sg::Matrix<Z>::fromLAPACK(n, r, b2.data(), n, nb);
            if (sg::posv(mH, mB2) != 0) return 62;
            if (!(resid(H, b2, Bz, n, r) <= 3 * eps)) return 63;
            for (int j = 0; j < n; ++j)
                for (int i = j + 1; i < n; ++i)
                    if (h[i + size_t(j) * n] != Z(7.0, 0.0)) return 64;
        }
        // 7. float Cholesky through the simplified API, tiles on the device
        {
            auto S = hpd<float>(n);
            std::vector<float> Bf(size_t(n) * r);
            for (auto& v : Bf) v = rnd<float>();
            sg::HermitianMatrix<float> mS(sg::Uplo::Lower, n, nb);
            sg::Matrix<float> mB(n, r, nb);
            mS.insertLocalTiles(sg::Target::Devices);
            mB.insertLocalTiles(sg::Target::Devices);
            scatter(mS, S, 0);
            scatter(mB, Bf, 0);
            sg::chol_solve(mS, mB);
            auto X = gather(mB, 0);
            if (!(resid(S, X, Bf, n, r) <= 50 * 1.1920929e-07)) return 70;
        }
    } catch (const std::exception& e) {
        std::printf("exception: %s\n", e.what());
        return 99;
    }
    std::printf("OK\n");
    return 0;
}
