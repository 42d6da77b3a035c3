// Stand-in for the two BLAS++ type utilities that SLATE's matgen/random.cc
// uses (blas::real_type and blas::make_scalar).  BLAS++ is an empty submodule
// in the SLATE tree, so this header lets random.cc compile on its own, to
// produce reference Philox outputs for pinning the oracle's generator.
#ifndef ORACLE_REFSHIM_BLAS_HH
#define ORACLE_REFSHIM_BLAS_HH
#include <complex>
namespace blas {
template <typename T> struct real_type_s { using type = T; };
template <typename T> struct real_type_s<std::complex<T>> { using type = T; };
template <typename T> using real_type = typename real_type_s<T>::type;
template <typename T> inline T make_scalar(real_type<T> re, real_type<T> /*im*/) { return re; }
template <> inline std::complex<float> make_scalar<std::complex<float>>(float re, float im)
{ return std::complex<float>(re, im); }
template <> inline std::complex<double> make_scalar<std::complex<double>>(double re, double im)
{ return std::complex<double>(re, im); }
}
#endif
