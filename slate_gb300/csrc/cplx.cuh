// cplx.cuh -- complex scalars of the c / z solve path.
//
// cplx<R> has the storage of C99 `R _Complex`, std::complex<R> and
// cuComplex (real then imaginary part, aligned to its size), so the caller's
// interleaved column-major arrays are used as they are.  The operations are
// the textbook ones; division scales by the larger component of the divisor
// (Smith's algorithm) to avoid overflow.  cabs1 = |re| + |im| is the pivot
// measure of SLATE's LU panel (include/slate/internal/util.hh, cabs1) and of
// LAPACK's izamax.
#pragma once

#include <cfloat>
#include <cmath>
#include <cuda_runtime.h>

namespace slt {

template <typename R>
struct alignas(2 * sizeof(R)) cplx {
    R re, im;
    __host__ __device__ constexpr cplx() : re(0), im(0) {}
    __host__ __device__ constexpr cplx(R r) : re(r), im(0) {}
    __host__ __device__ constexpr cplx(R r, R i) : re(r), im(i) {}
    __host__ __device__ cplx& operator+=(const cplx& b) { re += b.re; im += b.im; return *this; }
    __host__ __device__ cplx& operator-=(const cplx& b) { re -= b.re; im -= b.im; return *this; }
};

template <typename R> __host__ __device__ inline cplx<R> operator+(cplx<R> a, cplx<R> b) { return {a.re + b.re, a.im + b.im}; }
template <typename R> __host__ __device__ inline cplx<R> operator-(cplx<R> a, cplx<R> b) { return {a.re - b.re, a.im - b.im}; }
template <typename R> __host__ __device__ inline cplx<R> operator-(cplx<R> a) { return {-a.re, -a.im}; }
template <typename R> __host__ __device__ inline cplx<R> operator*(cplx<R> a, cplx<R> b)
{ return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
template <typename R> __host__ __device__ inline cplx<R> operator*(R s, cplx<R> a) { return {s * a.re, s * a.im}; }
template <typename R> __host__ __device__ inline bool operator==(cplx<R> a, cplx<R> b) { return a.re == b.re && a.im == b.im; }
template <typename R> __host__ __device__ inline bool operator!=(cplx<R> a, cplx<R> b) { return !(a == b); }
template <typename R> __host__ __device__ inline cplx<R> conj(cplx<R> a) { return {a.re, -a.im}; }
template <typename R> __host__ __device__ inline R real(cplx<R> a) { return a.re; }
template <typename R> __host__ __device__ inline R cabs1(cplx<R> a) { return fabs(a.re) + fabs(a.im); }
template <typename R> __host__ __device__ inline R cabs(cplx<R> a) { return hypot(a.re, a.im); }

// a * b + c with fused multiply-adds on the components.
template <typename R> __host__ __device__ inline cplx<R> fma(cplx<R> a, cplx<R> b, cplx<R> c)
{
    return {::fma(a.re, b.re, ::fma(-a.im, b.im, c.re)), ::fma(a.re, b.im, ::fma(a.im, b.re, c.im))};
}

// a / b, Smith's algorithm.
template <typename R> __host__ __device__ inline cplx<R> operator/(cplx<R> a, cplx<R> b)
{
    if (fabs(b.re) >= fabs(b.im)) {
        const R r = b.im / b.re, d = b.re + b.im * r;
        return {(a.re + a.im * r) / d, (a.im - a.re * r) / d};
    }
    const R r = b.re / b.im, d = b.im + b.re * r;
    return {(a.re * r + a.im) / d, (a.im * r - a.re) / d};
}

using cfloat = cplx<float>;
using cdouble = cplx<double>;

// Scalar traits shared by the real and complex kernels.
template <typename T> struct Scalar;
template <typename R> struct RealLimits;
template <> struct RealLimits<float>  { __host__ __device__ static constexpr float safe_min() { return FLT_MIN; } };
template <> struct RealLimits<double> { __host__ __device__ static constexpr double safe_min() { return DBL_MIN; } };
template <> struct Scalar<float>   : RealLimits<float>  { using real = float;  static constexpr bool complex = false; };
template <> struct Scalar<double>  : RealLimits<double> { using real = double; static constexpr bool complex = false; };
template <> struct Scalar<cfloat>  : RealLimits<float>  { using real = float;  static constexpr bool complex = true; };
template <> struct Scalar<cdouble> : RealLimits<double> { using real = double; static constexpr bool complex = true; };

__host__ __device__ inline float conj(float a) { return a; }
__host__ __device__ inline double conj(double a) { return a; }
__host__ __device__ inline float cabs1(float a) { return fabsf(a); }
__host__ __device__ inline double cabs1(double a) { return fabs(a); }
__host__ __device__ inline float cabs(float a) { return fabsf(a); }
__host__ __device__ inline double cabs(double a) { return fabs(a); }
__host__ __device__ inline float real(float a) { return a; }
__host__ __device__ inline double real(double a) { return a; }

} // namespace slt
