// slate_gb300.hh -- SLATE's C++ driver API for the single-GPU solve path,
// header-only over the C ABI of libslate_gb300.so.
//
// Names, argument order and meaning follow include/slate/slate.hh:503-770
// (gesv, getrf, getrs, gesv_mixed, gesv_mixed_gmres, posv, potrf, potrs,
// posv_mixed, posv_mixed_gmres, gecondest, pocondest) and the simplified
// API include/slate/simplified_api.hh (lu_solve, lu_factor,
// lu_solve_using_factor, chol_solve, chol_factor, chol_solve_using_factor),
// with SLATE's Option keys (include/slate/enums.hh:453-490) and Pivot
// (include/slate/types.hh:84-117).  A C++ caller of SLATE on a 1 x 1 grid
// with Target::Devices changes `slate::` to `slate_gb300::` and creates its
// matrices with fromDevices on one device.
//
// Differences: matrices must be column-major arrays on the current CUDA
// device (Matrix::fromDevices with one device, or fromLAPACK on a device
// pointer), one tile size nb; errors throw slate_gb300::Exception carrying the
// library's status (SLATE throws slate::Exception); Upper HermitianMatrix
// goes through the LAPACK-style transpose in the device layer.
#pragma once

#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "slate_gb300.h"

namespace slate_gb300 {

class Exception : public std::runtime_error {
public:
    explicit Exception(int status)
        : std::runtime_error(std::string("slate_gb300: ") + slt_status_string(status)), status_(status) {}
    int status() const { return status_; }
private:
    int status_;
};

inline void check(int status) { if (status != 0) throw Exception(status); }

enum class Option {
    Lookahead, BlockSize, InnerBlocking, MaxPanelThreads, Tolerance, Target, MaxIterations,
    UseFallbackSolver, PivotThreshold, MethodLU, Depth,
    FactorPrecision, Refine, Equilibrate          // this library's additions
};
enum class Target : char { Host = 'H', HostTask = 'T', HostNest = 'N', HostBatch = 'B', Devices = 'D' };
enum class MethodLU : char { Auto = '*', PartialPiv = 'P', CALU = 'C', NoPiv = 'N' };
enum class Uplo : char { Lower = 'L', Upper = 'U' };
enum class Norm : char { One = '1', Inf = 'I' };

// The value of one option: SLATE's OptionValue holds an int64 or a double.
class OptionValue {
public:
    OptionValue(int64_t i) : i_(i), d_(double(i)) {}
    OptionValue(int i) : i_(i), d_(double(i)) {}
    OptionValue(double d) : i_(int64_t(d)), d_(d) {}
    OptionValue(bool b) : i_(b ? 1 : 0), d_(b ? 1.0 : 0.0) {}
    OptionValue(Target t) : i_(int64_t(t)), d_(double(int64_t(t))) {}
    OptionValue(MethodLU m) : i_(int64_t(m)), d_(double(int64_t(m))) {}
    int64_t i() const { return i_; }
    double d() const { return d_; }
private:
    int64_t i_;
    double d_;
};
using Options = std::map<Option, OptionValue>;

// Pivot of row k*nb + j: tile index relative to panel k and offset in that tile.
struct Pivot {
    int64_t tile_index = 0, element_offset = 0;
    Pivot() = default;
    Pivot(int64_t t, int64_t o) : tile_index(t), element_offset(o) {}
    int64_t tileIndex() const { return tile_index; }
    int64_t elementOffset() const { return element_offset; }
};
using Pivots = std::vector<std::vector<Pivot>>;

// A column-major device array with SLATE's tile size.
template <typename T>
class Matrix {
public:
    Matrix() = default;
    static Matrix fromDevices(int64_t m, int64_t n, T** Aarray, int num_devices, int64_t lda, int64_t nb,
                              int p = 1, int q = 1) {
        if (num_devices != 1 || p != 1 || q != 1) throw Exception(SLT_ERR_NOT_SUPPORTED);
        return Matrix(m, n, Aarray[0], lda, nb);
    }
    static Matrix fromLAPACK(int64_t m, int64_t n, T* A, int64_t lda, int64_t nb, int p = 1, int q = 1) {
        if (p != 1 || q != 1) throw Exception(SLT_ERR_NOT_SUPPORTED);
        return Matrix(m, n, A, lda, nb);
    }
    int64_t m() const { return m_; }
    int64_t n() const { return n_; }
    int64_t mt() const { return (m_ + nb_ - 1) / nb_; }
    int64_t nt() const { return (n_ + nb_ - 1) / nb_; }
    int64_t tileNb(int64_t) const { return nb_; }
    T* data() const { return data_; }
    int64_t stride() const { return ld_; }
protected:
    Matrix(int64_t m, int64_t n, T* A, int64_t lda, int64_t nb) : m_(m), n_(n), ld_(lda), nb_(nb), data_(A) {
        if (nb <= 0 || lda < (m > 1 ? m : 1)) throw Exception(SLT_ERR_ARG);
    }
    int64_t m_ = 0, n_ = 0, ld_ = 1, nb_ = 512;
    T* data_ = nullptr;
};

template <typename T>
class HermitianMatrix : public Matrix<T> {
public:
    HermitianMatrix() = default;
    static HermitianMatrix fromDevices(Uplo uplo, int64_t n, T** Aarray, int num_devices, int64_t lda,
                                       int64_t nb, int p = 1, int q = 1) {
        if (num_devices != 1 || p != 1 || q != 1) throw Exception(SLT_ERR_NOT_SUPPORTED);
        return HermitianMatrix(uplo, n, Aarray[0], lda, nb);
    }
    static HermitianMatrix fromLAPACK(Uplo uplo, int64_t n, T* A, int64_t lda, int64_t nb, int p = 1, int q = 1) {
        if (p != 1 || q != 1) throw Exception(SLT_ERR_NOT_SUPPORTED);
        return HermitianMatrix(uplo, n, A, lda, nb);
    }
    Uplo uplo() const { return uplo_; }
private:
    HermitianMatrix(Uplo uplo, int64_t n, T* A, int64_t lda, int64_t nb) : Matrix<T>(n, n, A, lda, nb), uplo_(uplo) {
        if (uplo != Uplo::Lower) throw Exception(SLT_ERR_NOT_SUPPORTED);   // device layer factors lower
    }
    Uplo uplo_ = Uplo::Lower;
};

namespace detail {

inline slt_options to_c(const Options& opts, int64_t nb)
{
    slt_options o;
    slt_options_default(&o);
    o.nb = nb;
    for (const auto& kv : opts) {
        switch (kv.first) {
            case Option::BlockSize:         break;              // the matrix's tile size rules, as in SLATE
            case Option::InnerBlocking:     o.ib = kv.second.i(); break;
            case Option::Lookahead:         o.lookahead = kv.second.i(); break;
            case Option::MaxIterations:     o.max_iterations = kv.second.i(); break;
            case Option::Tolerance:         o.tolerance = kv.second.d(); break;
            case Option::UseFallbackSolver: o.use_fallback = int(kv.second.i() != 0); break;
            case Option::PivotThreshold:    o.pivot_threshold = kv.second.d(); break;
            case Option::Depth:             o.depth = kv.second.i(); break;
            case Option::MethodLU:
                if (kv.second.i() == int64_t(MethodLU::NoPiv)) o.method_lu = 'N';
                if (kv.second.i() == int64_t(MethodLU::CALU)) o.method_lu = 'C';
                break;
            case Option::FactorPrecision:   o.factor_precision = int(kv.second.i()); break;
            case Option::Refine:            o.refine = int(kv.second.i()); break;
            case Option::Equilibrate:       o.equilibrate = int(kv.second.i()); break;
            default:                        break;              // Target, MaxPanelThreads: accepted
        }
    }
    return o;
}

// RAII device int array for the per-panel pivots
struct DeviceInts {
    int* p = nullptr;
    explicit DeviceInts(int64_t n);
    ~DeviceInts();
};

}  // namespace detail

// ---- LU ----------------------------------------------------------------------
// The pivot conversion needs the CUDA runtime; it lives in the library.
extern "C" int slt_ipiv_alloc(int64_t n, int** d);
extern "C" int slt_ipiv_free(int* d);
extern "C" int slt_ipiv_download(const int* d, int64_t n, int* h);
extern "C" int slt_ipiv_upload(const int* h, int64_t n, int* d);

inline detail::DeviceInts::DeviceInts(int64_t n) { check(slt_ipiv_alloc(n, &p)); }
inline detail::DeviceInts::~DeviceInts() { slt_ipiv_free(p); }

inline void pivots_from_device(const int* d, int64_t n, int64_t nb, Pivots& pivots)
{
    std::vector<int> h(size_t(n > 0 ? n : 1));
    if (n > 0) check(slt_ipiv_download(d, n, h.data()));
    pivots.assign(size_t((n + nb - 1) / nb), {});
    for (int64_t r = 0; r < n; ++r) pivots[size_t(r / nb)].push_back(Pivot(h[size_t(r)] / nb, h[size_t(r)] % nb));
}

inline void pivots_to_device(const Pivots& pivots, int64_t n, int64_t nb, int* d)
{
    std::vector<int> h(size_t(n > 0 ? n : 1), 0);
    for (int64_t r = 0; r < n; ++r) {
        const Pivot& pv = pivots.at(size_t(r / nb)).at(size_t(r % nb));
        h[size_t(r)] = int(pv.tile_index * nb + pv.element_offset);
    }
    if (n > 0) check(slt_ipiv_upload(h.data(), n, d));
}

inline int64_t getrf(Matrix<double>& A, Pivots& pivots, const Options& opts = Options())
{
    const int64_t mn = A.m() < A.n() ? A.m() : A.n();
    detail::DeviceInts piv(mn);
    slt_options o = detail::to_c(opts, A.tileNb(0));
    int64_t info = 0;
    check(slt_dgetrf_device(A.m(), A.n(), A.data(), A.stride(), piv.p, &o, nullptr, &info));
    pivots_from_device(piv.p, mn, A.tileNb(0), pivots);
    return info;
}

inline void getrs(Matrix<double>& A, Pivots& pivots, Matrix<double>& B, const Options& opts = Options())
{
    detail::DeviceInts piv(A.n());
    pivots_to_device(pivots, A.n(), A.tileNb(0), piv.p);
    slt_options o = detail::to_c(opts, A.tileNb(0));
    check(slt_dgetrs_device(A.n(), B.n(), A.data(), A.stride(), piv.p, B.data(), B.stride(), &o, nullptr));
}

inline int64_t gesv(Matrix<double>& A, Pivots& pivots, Matrix<double>& B, const Options& opts = Options())
{
    detail::DeviceInts piv(A.n());
    slt_options o = detail::to_c(opts, A.tileNb(0));
    int64_t info = 0;
    check(slt_dgesv_device(A.n(), B.n(), A.data(), A.stride(), piv.p, B.data(), B.stride(), &o, nullptr, &info));
    pivots_from_device(piv.p, A.n(), A.tileNb(0), pivots);
    return info;
}

inline int64_t gesv_mixed(Matrix<double>& A, Pivots& pivots, Matrix<double>& B, Matrix<double>& X, int& iter,
                          const Options& opts = Options())
{
    detail::DeviceInts piv(A.n());
    slt_options o = detail::to_c(opts, A.tileNb(0));
    int64_t info = 0;
    check(slt_dsgesv_device(A.n(), B.n(), A.data(), A.stride(), piv.p, B.data(), B.stride(), X.data(), X.stride(),
                            &o, nullptr, &iter, &info));
    pivots_from_device(piv.p, A.n(), A.tileNb(0), pivots);
    return info;
}

// slate::gesv_rbt (src/gesv_rbt.cc): random butterfly transform (Option::Depth,
// default 2), LU without pivoting, FP64 refinement; A receives the factors of
// the transformed matrix.  Returns info.
inline int64_t gesv_rbt(Matrix<double>& A, Matrix<double>& B, Matrix<double>& X, int& iter,
                        const Options& opts = Options())
{
    slt_options o = detail::to_c(opts, A.tileNb(0));
    int64_t info = 0;
    check(slt_dgesv_rbt_device(A.n(), B.n(), A.data(), A.stride(), B.data(), B.stride(), X.data(), X.stride(), &o,
                               nullptr, &iter, &info));
    return info;
}

inline int64_t gesv_mixed_gmres(Matrix<double>& A, Pivots& pivots, Matrix<double>& B, Matrix<double>& X,
                                int& iter, const Options& opts = Options())
{
    detail::DeviceInts piv(A.n());
    slt_options o = detail::to_c(opts, A.tileNb(0));
    int64_t info = 0;
    check(slt_dsgesv_gmres_device(A.n(), B.n(), A.data(), A.stride(), piv.p, B.data(), B.stride(), X.data(),
                                  X.stride(), &o, nullptr, &iter, &info));
    pivots_from_device(piv.p, A.n(), A.tileNb(0), pivots);
    return info;
}

inline double gecondest(Norm in_norm, Matrix<double>& A, double Anorm, const Options& opts = Options())
{
    slt_options o = detail::to_c(opts, A.tileNb(0));
    double rcond = 0.0;
    // the estimate does not depend on the row order: identity pivots
    detail::DeviceInts piv(A.n());
    Pivots id((size_t(A.n()) + size_t(A.tileNb(0)) - 1) / size_t(A.tileNb(0)));
    for (int64_t r = 0; r < A.n(); ++r) id[size_t(r / A.tileNb(0))].push_back(Pivot(0, r % A.tileNb(0)));
    pivots_to_device(id, A.n(), A.tileNb(0), piv.p);
    check(slt_dgecondest_device(char(in_norm), A.n(), A.data(), A.stride(), piv.p, Anorm, &rcond, &o, nullptr));
    return rcond;
}

// ---- Cholesky ----------------------------------------------------------------
inline int64_t potrf(HermitianMatrix<double>& A, const Options& opts = Options())
{
    slt_options o = detail::to_c(opts, A.tileNb(0));
    int64_t info = 0;
    check(slt_dpotrf_device(A.n(), A.data(), A.stride(), &o, nullptr, &info));
    return info;
}

inline void potrs(HermitianMatrix<double>& A, Matrix<double>& B, const Options& opts = Options())
{
    slt_options o = detail::to_c(opts, A.tileNb(0));
    check(slt_dpotrs_device(A.n(), B.n(), A.data(), A.stride(), B.data(), B.stride(), &o, nullptr));
}

inline int64_t posv(HermitianMatrix<double>& A, Matrix<double>& B, const Options& opts = Options())
{
    slt_options o = detail::to_c(opts, A.tileNb(0));
    int64_t info = 0;
    check(slt_dposv_device(A.n(), B.n(), A.data(), A.stride(), B.data(), B.stride(), &o, nullptr, &info));
    return info;
}

inline int64_t posv_mixed(HermitianMatrix<double>& A, Matrix<double>& B, Matrix<double>& X, int& iter,
                          const Options& opts = Options())
{
    slt_options o = detail::to_c(opts, A.tileNb(0));
    int64_t info = 0;
    check(slt_dsposv_device(A.n(), B.n(), A.data(), A.stride(), B.data(), B.stride(), X.data(), X.stride(), &o,
                            nullptr, &iter, &info));
    return info;
}

inline int64_t posv_mixed_gmres(HermitianMatrix<double>& A, Matrix<double>& B, Matrix<double>& X, int& iter,
                                const Options& opts = Options())
{
    slt_options o = detail::to_c(opts, A.tileNb(0));
    int64_t info = 0;
    check(slt_dsposv_gmres_device(A.n(), B.n(), A.data(), A.stride(), B.data(), B.stride(), X.data(), X.stride(),
                                  &o, nullptr, &iter, &info));
    return info;
}

inline double pocondest(Norm in_norm, HermitianMatrix<double>& A, double Anorm, const Options& opts = Options())
{
    slt_options o = detail::to_c(opts, A.tileNb(0));
    double rcond = 0.0;
    check(slt_dpocondest_device(char(in_norm), A.n(), A.data(), A.stride(), Anorm, &rcond, &o, nullptr));
    return rcond;
}

// ---- simplified API (include/slate/simplified_api.hh) -------------------------
inline void lu_solve(Matrix<double>& A, Matrix<double>& B, const Options& opts = Options())
{
    Pivots p;
    const int64_t info = gesv(A, p, B, opts);
    if (info != 0) throw Exception(SLT_ERR_ARG);
}
inline void lu_factor(Matrix<double>& A, Pivots& pivots, const Options& opts = Options())
{
    getrf(A, pivots, opts);
}
inline void lu_solve_using_factor(Matrix<double>& A, Pivots& pivots, Matrix<double>& B,
                                  const Options& opts = Options())
{
    getrs(A, pivots, B, opts);
}
inline void chol_solve(HermitianMatrix<double>& A, Matrix<double>& B, const Options& opts = Options())
{
    if (posv(A, B, opts) != 0) throw Exception(SLT_ERR_ARG);
}
inline void chol_factor(HermitianMatrix<double>& A, const Options& opts = Options())
{
    potrf(A, opts);
}
inline void chol_solve_using_factor(HermitianMatrix<double>& A, Matrix<double>& B, const Options& opts = Options())
{
    potrs(A, B, opts);
}

}  // namespace slate_gb300
