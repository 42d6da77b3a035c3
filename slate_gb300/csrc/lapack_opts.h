// lapack_opts.h -- options of the LAPACK- and ScaLAPACK-compatible host
// entry points.
#pragma once

#include "slate_gb300.h"

namespace slt {

// The options the LAPACK-compatible entry points run with: the SLATE_LAPACK_*
// environment (SLATE_LAPACK_NB, default 512; SLATE_LAPACK_IB, default 32;
// SLATE_LAPACK_FACTOR_PRECISION; SLATE_LAPACK_REFINE), unless a LapackOptsScope is active on the
// calling thread.
slt_options lapack_opts();

// Makes lapack_opts() return `o` on this thread while the scope lives (the
// ScaLAPACK entry points use it to pass the descriptor's block size).
class LapackOptsScope {
public:
    explicit LapackOptsScope(const slt_options& o);
    ~LapackOptsScope();
    LapackOptsScope(const LapackOptsScope&) = delete;
    LapackOptsScope& operator=(const LapackOptsScope&) = delete;

private:
    const slt_options* prev_;
};

} // namespace slt
