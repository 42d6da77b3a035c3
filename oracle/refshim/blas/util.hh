// Empty stand-in: see ../blas.hh.
#ifndef ORACLE_REFSHIM_BLAS_UTIL_HH
#define ORACLE_REFSHIM_BLAS_UTIL_HH
#include "../blas.hh"
#endif
