// capi.cc -- the public C ABI (include/slate_gb300.h).
//
// LAPACK-compatible host entry points mirror SLATE's lapack_api/
// (lapack_gesv.cc, lapack_gesv_mixed.cc, lapack_getrf.cc, lapack_getrs.cc,
// lapack_posv.cc, lapack_potrf.cc): wrap the caller's column-major arrays,
// run the Target::Devices path on a 1 x 1 grid, and return LAPACK's 1-based
// ipiv (lapack_api/lapack_gesv.cc:90-100).

#include "drivers.h"
#include "lapack_opts.h"

#include <algorithm>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace slt {
double timer_value(const char* name);
void timers_clear();
}

extern "C" int slt_dtranspose(int64_t m, int64_t n, const double* A, int64_t lda, double* B, int64_t ldb,
                              cudaStream_t stream);

using namespace slt;

namespace {

slt_options resolve(const slt_options* o)
{
    slt_options r;
    slt_options_default(&r);
    if (o) r = *o;
    if (r.nb <= 0) r.nb = 512;
    if (r.ib <= 0) r.ib = 32;
    if (r.max_iterations < 0) r.max_iterations = 30;
    return r;
}

cudaStream_t as_stream(slt_stream_t s) { return static_cast<cudaStream_t>(s); }

struct Status {
    DevBuf buf;
    FactorCtx fc;
    int init(cudaStream_t s) {
        int rc = buf.alloc(2 * sizeof(int), s);
        if (rc) return rc;
        SLT_CUDA_TRY(cudaMemsetAsync(buf.p, 0, 2 * sizeof(int), s));
        fc.d_info = buf.as<int>();
        fc.d_status = buf.as<int>() + 1;
        return SLT_OK;
    }
};

int64_t env_int(const char* name, int64_t dflt)
{
    const char* v = std::getenv(name);
    if (!v) return dflt;
    int64_t x = std::strtoll(v, nullptr, 0);
    return x != 0 ? x : dflt;
}

thread_local const slt_options* t_opts_override = nullptr;

// Host <-> device helpers for the LAPACK entry points.
template <typename T>
int to_device(const T* h, int64_t m, int64_t n, int64_t ld, DevBuf& d, cudaStream_t s)
{
    int rc = d.alloc(sizeof(T) * size_t(std::max<int64_t>(m, 1)) * size_t(std::max<int64_t>(n, 1)), s);
    if (rc) return rc;
    if (m > 0 && n > 0)
        SLT_CUDA_TRY(cudaMemcpy2DAsync(d.p, size_t(m) * sizeof(T), h, size_t(ld) * sizeof(T),
                                       size_t(m) * sizeof(T), size_t(n), cudaMemcpyHostToDevice, s));
    return SLT_OK;
}

template <typename T>
int to_host(const DevBuf& d, T* h, int64_t m, int64_t n, int64_t ld, cudaStream_t s)
{
    if (m > 0 && n > 0)
        SLT_CUDA_TRY(cudaMemcpy2DAsync(h, size_t(ld) * sizeof(T), d.p, size_t(m) * sizeof(T),
                                       size_t(m) * sizeof(T), size_t(n), cudaMemcpyDeviceToHost, s));
    return SLT_OK;
}

// The referenced triangle of an n x n column-major array (lower: rows
// j0 .. n of columns j0 .. j0 + 511; upper: rows 0 .. j0 + 511), one 2-D copy
// per 512-column block: half the bytes of the whole array.  The diagonal
// blocks travel whole; the drivers leave their other triangle as it is, so
// copying the result back restores the caller's values there.
template <typename T>
int tri_copy(bool lower, int64_t n, const T* src, int64_t lds, T* dst, int64_t ldd, cudaMemcpyKind kind,
             cudaStream_t s)
{
    constexpr int64_t kB = 512;
    for (int64_t j0 = 0; j0 < n; j0 += kB) {
        const int64_t w = std::min(kB, n - j0);
        const int64_t r0 = lower ? j0 : 0;
        const int64_t rows = lower ? n - j0 : j0 + w;
        SLT_CUDA_TRY(cudaMemcpy2DAsync(dst + r0 + j0 * ldd, size_t(ldd) * sizeof(T), src + r0 + j0 * lds,
                                       size_t(lds) * sizeof(T), size_t(rows) * sizeof(T), size_t(w), kind, s));
    }
    return SLT_OK;
}

// Per-panel relative pivots -> LAPACK 1-based global ipiv, and back.
void ipiv_to_lapack(const std::vector<int>& rel, int64_t nb, int* ipiv, int64_t cnt)
{
    for (int64_t r = 0; r < cnt; ++r) ipiv[r] = int((r / nb) * nb + rel[r] + 1);
}

void ipiv_from_lapack(const int* ipiv, int64_t nb, std::vector<int>& rel, int64_t cnt)
{
    rel.resize(cnt);
    for (int64_t r = 0; r < cnt; ++r) rel[r] = int(ipiv[r] - 1 - (r / nb) * nb);
}

struct LapackStream {
    cudaStream_t s = nullptr;
    LapackStream() { if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) s = nullptr; }
    ~LapackStream() { if (s) cudaStreamDestroy(s); }
};

cudaStream_t lapack_stream()
{
    static thread_local LapackStream ls;
    return ls.s;
}

// Second stream of the LAPACK entry points: host-to-device copies of A that
// the solve consumes while they are still arriving.
cudaStream_t lapack_copy_stream()
{
    static thread_local LapackStream ls;
    return ls.s;
}

// The lower triangle of the host array a (n x n, leading dimension lda) into
// the device array d (leading dimension n) on the copy stream cs, in the
// order the left-looking factor reads it: all 512 x 512 diagonal blocks
// first (the equilibration scales need the diagonal), then the columns
// below them block by block, one event each.  The copies are enqueued by a
// worker thread: cudaMemcpy2DAsync blocks the enqueuing thread once the
// driver's copy queue is full, which would hold back the enqueue of the
// solve itself until most of A had arrived.  The driver's stream waits
// through arr (whose recorded() blocks until the event it is about to wait
// for has been recorded).  cs first waits for `ready` (d allocated on s).
struct StreamedLower {
    static constexpr int64_t kB = 512;
    std::vector<cudaEvent_t> ev;
    cudaEvent_t ev_diag = nullptr, ev_ready = nullptr;
    InputArrival arr;
    cudaStream_t s_ = nullptr;
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv;
    int64_t done = -2;          // last recorded event: -2 none, -1 the diagonal's, b block b
    int err = SLT_OK;

    ~StreamedLower() {
        // whatever happened, the compute stream (which frees d) waits for the copies
        if (worker.joinable()) worker.join();
        if (s_ && done >= 0) cudaStreamWaitEvent(s_, ev[size_t(done)], 0);
        for (cudaEvent_t e : ev) cudaEventDestroy(e);
        if (ev_diag) cudaEventDestroy(ev_diag);
        if (ev_ready) cudaEventDestroy(ev_ready);
    }
    void publish(int64_t k, int rc) {
        std::lock_guard<std::mutex> lk(mu);
        if (rc) err = rc;
        else done = k;
        cv.notify_all();
    }
    int start(int64_t n, const double* a, int64_t lda, double* d, cudaStream_t s, cudaStream_t cs, bool whole) {
        const int64_t nblk = (n + kB - 1) / kB;
        int dev = 0;
        SLT_CUDA_TRY(cudaGetDevice(&dev));
        SLT_CUDA_TRY(cudaEventCreateWithFlags(&ev_ready, cudaEventDisableTiming));
        SLT_CUDA_TRY(cudaEventCreateWithFlags(&ev_diag, cudaEventDisableTiming));
        ev.assign(size_t(nblk), nullptr);
        for (auto& e : ev) SLT_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        SLT_CUDA_TRY(cudaEventRecord(ev_ready, s));
        arr.ev_diag = ev_diag;
        arr.ev = ev.data();
        arr.nev = nblk;
        arr.blk = kB;
        arr.recorded = [this](int64_t k) -> int {
            std::unique_lock<std::mutex> lk(mu);
            cv.wait(lk, [&] { return err != SLT_OK || done >= k; });
            return err;
        };
        s_ = s;
        worker = std::thread([=]() {
            int rc = slt_from_cuda(cudaSetDevice(dev));
            if (!rc) rc = slt_from_cuda(cudaStreamWaitEvent(cs, ev_ready, 0));
            for (int64_t j0 = 0; j0 < n && !rc; j0 += kB) {
                const int64_t w = std::min(kB, n - j0);
                rc = slt_from_cuda(cudaMemcpy2DAsync(d + j0 + j0 * n, size_t(n) * 8, a + j0 + j0 * lda, size_t(lda) * 8,
                                                     size_t(w) * 8, size_t(w), cudaMemcpyHostToDevice, cs));
            }
            if (!rc) rc = slt_from_cuda(cudaEventRecord(ev_diag, cs));
            publish(-1, rc);
            for (int64_t j0 = 0, b = 0; j0 < n && !rc; j0 += kB, ++b) {
                const int64_t w = std::min(kB, n - j0), r0 = j0 + w;
                if (whole && lda == n)          // the whole block column: one contiguous copy
                    rc = slt_from_cuda(cudaMemcpyAsync(d + j0 * n, a + j0 * lda, size_t(n) * size_t(w) * 8,
                                                       cudaMemcpyHostToDevice, cs));
                else if (r0 < n)
                    rc = slt_from_cuda(cudaMemcpy2DAsync(d + r0 + j0 * n, size_t(n) * 8, a + r0 + j0 * lda,
                                                         size_t(lda) * 8, size_t(n - r0) * 8, size_t(w),
                                                         cudaMemcpyHostToDevice, cs));
                if (!rc) rc = slt_from_cuda(cudaEventRecord(ev[size_t(b)], cs));
                publish(b, rc);
            }
        });
        return SLT_OK;
    }
    // the compute stream waits for every copy (before d is freed or reused)
    int join(cudaStream_t s) {
        if (worker.joinable()) worker.join();
        if (err) return err;
        return arr.wait_all(s);
    }
};

template <typename T>
int getrf_device_impl(int64_t m, int64_t n, T* dA, int64_t lda, int* d_ipiv, const slt_options* opts,
                      slt_stream_t stream, int64_t* info)
{
    cudaStream_t s = as_stream(stream);
    slt_options o = resolve(opts);
    Status st;
    int rc = st.init(s);
    if (rc) return rc;
    rc = getrf_dev<T>(m, n, dA, lda, d_ipiv, o, st.fc, s);
    if (rc) return rc;
    return finish_factor(st.fc, info, s);
}

} // namespace

namespace slt {

slt_options lapack_opts()
{
    if (t_opts_override) return *t_opts_override;
    slt_options o;
    slt_options_default(&o);
    o.nb = env_int("SLATE_LAPACK_NB", 512);
    o.ib = std::min<int64_t>(env_int("SLATE_LAPACK_IB", 32), o.nb);
    if (const char* p = std::getenv("SLATE_LAPACK_FACTOR_PRECISION")) {
        std::string v(p);
        if (v == "fp32") o.factor_precision = SLT_PREC_FP32;
        else if (v == "tf32") o.factor_precision = SLT_PREC_TF32;
        else if (v == "bf16") o.factor_precision = SLT_PREC_BF16;
        else if (v == "fp16") o.factor_precision = SLT_PREC_FP16;
        else if (v == "fp8") o.factor_precision = SLT_PREC_FP8;
        else if (v == "tf32x3") o.factor_precision = SLT_PREC_TF32X3;
    }
    if (const char* p = std::getenv("SLATE_LAPACK_REFINE")) {
        std::string v(p);
        if (v == "ir") o.refine = SLT_REFINE_IR;
        else if (v == "gmres") o.refine = SLT_REFINE_GMRES;
        else if (v == "ir+gmres") o.refine = SLT_REFINE_IR_GMRES;
    }
    return o;
}

LapackOptsScope::LapackOptsScope(const slt_options& o) : prev_(t_opts_override) { t_opts_override = &o; }
LapackOptsScope::~LapackOptsScope() { t_opts_override = prev_; }

} // namespace slt

extern "C" {

void slt_options_default(slt_options* o)
{
    if (!o) return;
    o->nb = 512;
    o->ib = 32;
    o->lookahead = 1;
    o->max_iterations = 30;
    o->tolerance = 0.0;
    o->use_fallback = 1;
    o->pivot_threshold = 1.0;
    o->factor_precision = SLT_PREC_FP32;
    o->gemm_engine = 0;
    o->refine = SLT_REFINE_IR;
    o->residual_engine = 0;
    o->equilibrate = -1;
    o->lo_retry = -1;
    o->depth = 2;
    o->method_lu = 'P';
}

const char* slt_status_string(int st)
{
    switch (st) {
        case SLT_OK: return "success";
        case SLT_ERR_ARG: return "invalid argument";
        case SLT_ERR_TIMEOUT: return "a bounded device wait timed out";
        case SLT_ERR_NOMEM: return "device allocation failed";
        case SLT_ERR_NOT_SUPPORTED: return "not supported on this device or configuration";
        case SLT_ERR_NO_DEVICE: return "no CUDA device";
        case SLT_ERR_LIMIT: return "size exceeds a fixed limit";
        default:
            if (st >= SLT_ERR_CUDA_BASE) return cudaGetErrorString(cudaError_t(st - SLT_ERR_CUDA_BASE));
            return "unknown status";
    }
}

const char* slt_version(void) { return "slate_gb300 0.1 (sm_103a)"; }

double slt_timer(const char* name) { return timer_value(name); }

int slt_dgetrf_device(int64_t m, int64_t n, double* dA, int64_t lda, int* d_ipiv,
                      const slt_options* opts, slt_stream_t stream, int64_t* info)
{ return getrf_device_impl<double>(m, n, dA, lda, d_ipiv, opts, stream, info); }

int slt_sgetrf_device(int64_t m, int64_t n, float* dA, int64_t lda, int* d_ipiv,
                      const slt_options* opts, slt_stream_t stream, int64_t* info)
{ return getrf_device_impl<float>(m, n, dA, lda, d_ipiv, opts, stream, info); }

int slt_dgetrs_device(int64_t n, int64_t nrhs, const double* dLU, int64_t lda, const int* d_ipiv,
                      double* dB, int64_t ldb, const slt_options* opts, slt_stream_t stream)
{
    cudaStream_t s = as_stream(stream);
    slt_options o = resolve(opts);
    Status st;
    int rc = st.init(s);
    if (rc) return rc;
    rc = getrs_dev<double>(n, nrhs, dLU, lda, d_ipiv, o.nb, dB, ldb, st.fc.d_status, s);
    if (rc) return rc;
    return finish_factor(st.fc, nullptr, s);
}

int slt_dgetrs_trans_device(char trans, int64_t n, int64_t nrhs, const double* dLU, int64_t lda,
                            const int* d_ipiv, double* dB, int64_t ldb, const slt_options* opts,
                            slt_stream_t stream)
{
    if (trans == 'N' || trans == 'n') return slt_dgetrs_device(n, nrhs, dLU, lda, d_ipiv, dB, ldb, opts, stream);
    if (trans != 'T' && trans != 't' && trans != 'C' && trans != 'c') return SLT_ERR_ARG;
    cudaStream_t s = as_stream(stream);
    slt_options o = resolve(opts);
    Status st;
    int rc = st.init(s);
    if (rc) return rc;
    rc = getrs_trans_dev<double>(n, nrhs, dLU, lda, d_ipiv, o.nb, dB, ldb, st.fc.d_status, s);
    if (rc) return rc;
    return finish_factor(st.fc, nullptr, s);
}

int slt_sgetrs_device(int64_t n, int64_t nrhs, const float* dLU, int64_t lda, const int* d_ipiv,
                      float* dB, int64_t ldb, const slt_options* opts, slt_stream_t stream)
{
    cudaStream_t s = as_stream(stream);
    slt_options o = resolve(opts);
    Status st;
    int rc = st.init(s);
    if (rc) return rc;
    rc = getrs_dev<float>(n, nrhs, dLU, lda, d_ipiv, o.nb, dB, ldb, st.fc.d_status, s);
    if (rc) return rc;
    return finish_factor(st.fc, nullptr, s);
}

int slt_dgesv_device(int64_t n, int64_t nrhs, double* dA, int64_t lda, int* d_ipiv, double* dB,
                     int64_t ldb, const slt_options* opts, slt_stream_t stream, int64_t* info)
{
    cudaStream_t s = as_stream(stream);
    slt_options o = resolve(opts);
    TimerSet tm(s);
    tm.start("gesv");
    tm.start("gesv::getrf");
    Status st;
    int rc = st.init(s);
    if (rc) return rc;
    rc = getrf_dev<double>(n, n, dA, lda, d_ipiv, o, st.fc, s);
    if (rc) return rc;
    tm.stop("gesv::getrf");
    rc = finish_factor(st.fc, info, s);
    if (rc) return rc;
    tm.start("gesv::getrs");
    if (*info == 0) {
        rc = getrs_dev<double>(n, nrhs, dA, lda, d_ipiv, o.nb, dB, ldb, st.fc.d_status, s);
        if (rc) return rc;
    }
    tm.stop("gesv::getrs");
    tm.stop("gesv");
    return finish_factor(st.fc, nullptr, s);
}

int slt_dpotrf_device(int64_t n, double* dA, int64_t lda, const slt_options* opts, slt_stream_t stream,
                      int64_t* info)
{
    cudaStream_t s = as_stream(stream);
    slt_options o = resolve(opts);
    Status st;
    int rc = st.init(s);
    if (rc) return rc;
    rc = potrf_dev<double>(n, dA, lda, o, st.fc, s);
    if (rc) return rc;
    return finish_factor(st.fc, info, s);
}

int slt_spotrf_device(int64_t n, float* dA, int64_t lda, const slt_options* opts, slt_stream_t stream,
                      int64_t* info)
{
    cudaStream_t s = as_stream(stream);
    slt_options o = resolve(opts);
    Status st;
    int rc = st.init(s);
    if (rc) return rc;
    rc = potrf_dev<float>(n, dA, lda, o, st.fc, s);
    if (rc) return rc;
    return finish_factor(st.fc, info, s);
}

int slt_dpotrs_device(int64_t n, int64_t nrhs, const double* dL, int64_t lda, double* dB, int64_t ldb,
                      const slt_options* opts, slt_stream_t stream)
{
    cudaStream_t s = as_stream(stream);
    slt_options o = resolve(opts);
    Status st;
    int rc = st.init(s);
    if (rc) return rc;
    rc = potrs_dev<double>(n, nrhs, dL, lda, o.nb, dB, ldb, st.fc.d_status, s);
    if (rc) return rc;
    return finish_factor(st.fc, nullptr, s);
}

int slt_dposv_device(int64_t n, int64_t nrhs, double* dA, int64_t lda, double* dB, int64_t ldb,
                     const slt_options* opts, slt_stream_t stream, int64_t* info)
{
    cudaStream_t s = as_stream(stream);
    slt_options o = resolve(opts);
    TimerSet tm(s);
    tm.start("posv");
    Status st;
    int rc = st.init(s);
    if (rc) return rc;
    tm.start("posv::potrf");
    rc = potrf_dev<double>(n, dA, lda, o, st.fc, s);
    if (rc) return rc;
    tm.stop("posv::potrf");
    rc = finish_factor(st.fc, info, s);
    if (rc) return rc;
    tm.start("posv::potrs");
    if (*info == 0) {
        rc = potrs_dev<double>(n, nrhs, dA, lda, o.nb, dB, ldb, st.fc.d_status, s);
        if (rc) return rc;
    }
    tm.stop("posv::potrs");
    tm.stop("posv");
    return finish_factor(st.fc, nullptr, s);
}

int slt_dgesv_rbt_device(int64_t n, int64_t nrhs, double* dA, int64_t lda, const double* dB, int64_t ldb,
                         double* dX, int64_t ldx, const slt_options* opts, slt_stream_t stream, int* iter,
                         int64_t* info)
{
    slt_options o = resolve(opts);
    int it = 0;
    int64_t inf = 0;
    const int rc = gesv_rbt_dev(n, nrhs, dA, lda, dB, ldb, dX, ldx, o, &it, &inf, as_stream(stream));
    if (iter) *iter = it;
    if (info) *info = inf;
    return rc;
}

int slt_dsgesv_device(int64_t n, int64_t nrhs, double* dA, int64_t lda, int* d_ipiv, const double* dB,
                      int64_t ldb, double* dX, int64_t ldx, const slt_options* opts, slt_stream_t stream,
                      int* iter, int64_t* info)
{
    slt_options o = resolve(opts);
    if (o.refine == SLT_REFINE_GMRES)
        return gesv_mixed_gmres_dev(0, n, nrhs, dA, lda, d_ipiv, dB, ldb, dX, ldx, o, iter, info,
                                    as_stream(stream));
    return gesv_mixed_dev(0, n, nrhs, dA, lda, d_ipiv, dB, ldb, dX, ldx, o, iter, info, as_stream(stream));
}

int slt_dsgesv_gmres_device(int64_t n, int64_t nrhs, double* dA, int64_t lda, int* d_ipiv,
                            const double* dB, int64_t ldb, double* dX, int64_t ldx,
                            const slt_options* opts, slt_stream_t stream, int* iter, int64_t* info)
{
    slt_options o = resolve(opts);
    return gesv_mixed_gmres_dev(0, n, nrhs, dA, lda, d_ipiv, dB, ldb, dX, ldx, o, iter, info,
                                as_stream(stream));
}

int slt_dsposv_device(int64_t n, int64_t nrhs, double* dA, int64_t lda, const double* dB, int64_t ldb,
                      double* dX, int64_t ldx, const slt_options* opts, slt_stream_t stream, int* iter,
                      int64_t* info)
{
    slt_options o = resolve(opts);
    if (o.refine == SLT_REFINE_GMRES)
        return gesv_mixed_gmres_dev(1, n, nrhs, dA, lda, nullptr, dB, ldb, dX, ldx, o, iter, info,
                                    as_stream(stream));
    return gesv_mixed_dev(1, n, nrhs, dA, lda, nullptr, dB, ldb, dX, ldx, o, iter, info, as_stream(stream));
}

int slt_dsposv_gmres_device(int64_t n, int64_t nrhs, double* dA, int64_t lda, const double* dB,
                            int64_t ldb, double* dX, int64_t ldx, const slt_options* opts,
                            slt_stream_t stream, int* iter, int64_t* info)
{
    slt_options o = resolve(opts);
    return gesv_mixed_gmres_dev(1, n, nrhs, dA, lda, nullptr, dB, ldb, dX, ldx, o, iter, info,
                                as_stream(stream));
}

int slt_sgetrs_trans_device(char trans, int64_t n, int64_t nrhs, const float* dLU, int64_t lda, const int* d_ipiv,
                            float* dB, int64_t ldb, const slt_options* opts, slt_stream_t stream)
{
    if (trans == 'N' || trans == 'n') return slt_sgetrs_device(n, nrhs, dLU, lda, d_ipiv, dB, ldb, opts, stream);
    if (trans != 'T' && trans != 't' && trans != 'C' && trans != 'c') return SLT_ERR_ARG;
    cudaStream_t s = as_stream(stream);
    slt_options o = resolve(opts);
    Status st;
    int rc = st.init(s);
    if (rc) return rc;
    rc = getrs_trans_dev<float>(n, nrhs, dLU, lda, d_ipiv, o.nb > 0 ? o.nb : 512, dB, ldb, st.fc.d_status, s);
    if (rc) return rc;
    return finish_factor(st.fc, nullptr, s);
}

int slt_spotrs_device(int64_t n, int64_t nrhs, const float* dL, int64_t lda, float* dB, int64_t ldb,
                      const slt_options* opts, slt_stream_t stream)
{
    cudaStream_t s = as_stream(stream);
    slt_options o = resolve(opts);
    Status st;
    int rc = st.init(s);
    if (rc) return rc;
    rc = potrs_dev<float>(n, nrhs, dL, lda, o.nb, dB, ldb, st.fc.d_status, s);
    if (rc) return rc;
    return finish_factor(st.fc, nullptr, s);
}

int slt_sposv_device(int64_t n, int64_t nrhs, float* dA, int64_t lda, float* dB, int64_t ldb,
                     const slt_options* opts, slt_stream_t stream, int64_t* info)
{
    int rc = slt_spotrf_device(n, dA, lda, opts, stream, info);
    if (rc || *info != 0) return rc;       // SLATE skips the solve when info != 0 (src/posv.cc:85-91)
    return slt_spotrs_device(n, nrhs, dA, lda, dB, ldb, opts, stream);
}

// ---- memory helpers of the header-only C++ API (tile storage of
// Matrix::insertLocalTiles, workspace tiles, copies between tile instances)
int slt_device_malloc(size_t bytes, void** p)
{
    if (!p) return SLT_ERR_ARG;
    *p = nullptr;
    const cudaError_t e = cudaMalloc(p, bytes > 0 ? bytes : 16);
    if (e != cudaSuccess) { cudaGetLastError(); *p = nullptr; return SLT_ERR_NOMEM; }
    return SLT_OK;
}

int slt_device_free(void* p) { return p ? slt_from_cuda(cudaFree(p)) : SLT_OK; }

int slt_memcpy2d(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, size_t height)
{
    if (width == 0 || height == 0) return SLT_OK;
    return slt_from_cuda(cudaMemcpy2D(dst, dpitch, src, spitch, width, height, cudaMemcpyDefault));
}

int slt_is_device_pointer(const void* p)
{
    cudaPointerAttributes a;
    if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

int slt_dgenerate_device(int dist, int64_t seed, int64_t m, int64_t n, int64_t ioff, int64_t joff,
                         double* dA, int64_t lda, slt_stream_t stream)
{
    cudaStream_t s = as_stream(stream);
    int rc = slt_dgenerate(dist, seed, m, n, ioff, joff, dA, lda, s);
    if (rc) return rc;
    return slt_from_cuda(cudaStreamSynchronize(s));
}

// ---------------------------------------------------------------------------
// LAPACK-compatible entry points.

static void lapack_gesv_impl(int n, int nrhs, double* a, int lda, int* ipiv, double* b, int ldb, int* info)
{
    *info = 0;
    if (n < 0) { *info = -1; return; }
    if (nrhs < 0) { *info = -2; return; }
    if (lda < std::max(1, n)) { *info = -4; return; }
    if (ldb < std::max(1, n)) { *info = -7; return; }
    if (n == 0) return;
    cudaStream_t s = lapack_stream();
    slt_options o = lapack_opts();
    DevBuf dA, dB, dP;
    if (to_device(a, n, n, lda, dA, s) || to_device(b, n, nrhs, ldb, dB, s) ||
        dP.alloc(sizeof(int) * size_t(n), s)) { *info = -100; return; }
    int64_t inf = 0;
    int rc = slt_dgesv_device(n, nrhs, dA.as<double>(), n, dP.as<int>(), dB.as<double>(), n, &o, s, &inf);
    if (rc) { *info = -1000 + rc; return; }
    std::vector<int> rel(n);
    if (to_host(dA, a, n, n, lda, s) || to_host(dB, b, n, nrhs, ldb, s) ||
        cudaMemcpyAsync(rel.data(), dP.p, sizeof(int) * size_t(n), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) { *info = -100; return; }
    ipiv_to_lapack(rel, o.nb, ipiv, n);
    *info = int(inf);
}

void slate_dgesv(const int* n, const int* nrhs, double* a, const int* lda, int* ipiv, double* b,
                 const int* ldb, int* info)
{ lapack_gesv_impl(*n, *nrhs, a, *lda, ipiv, b, *ldb, info); }
void slate_dgesv_(const int* n, const int* nrhs, double* a, const int* lda, int* ipiv, double* b,
                  const int* ldb, int* info)
{ lapack_gesv_impl(*n, *nrhs, a, *lda, ipiv, b, *ldb, info); }

static void lapack_sgesv_impl(int n, int nrhs, float* a, int lda, int* ipiv, float* b, int ldb, int* info)
{
    *info = 0;
    if (n < 0) { *info = -1; return; }
    if (nrhs < 0) { *info = -2; return; }
    if (lda < std::max(1, n)) { *info = -4; return; }
    if (ldb < std::max(1, n)) { *info = -7; return; }
    if (n == 0) return;
    cudaStream_t s = lapack_stream();
    slt_options o = lapack_opts();
    DevBuf dA, dB, dP;
    if (to_device(a, n, n, lda, dA, s) || to_device(b, n, nrhs, ldb, dB, s) ||
        dP.alloc(sizeof(int) * size_t(n), s)) { *info = -100; return; }
    int64_t inf = 0;
    int rc = slt_sgetrf_device(n, n, dA.as<float>(), n, dP.as<int>(), &o, s, &inf);
    if (rc) { *info = -1000 + rc; return; }
    if (inf == 0) {
        rc = slt_sgetrs_device(n, nrhs, dA.as<float>(), n, dP.as<int>(), dB.as<float>(), n, &o, s);
        if (rc) { *info = -1000 + rc; return; }
    }
    std::vector<int> rel(n);
    if (to_host(dA, a, n, n, lda, s) || to_host(dB, b, n, nrhs, ldb, s) ||
        cudaMemcpyAsync(rel.data(), dP.p, sizeof(int) * size_t(n), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) { *info = -100; return; }
    ipiv_to_lapack(rel, o.nb, ipiv, n);
    *info = int(inf);
}

void slate_sgesv(const int* n, const int* nrhs, float* a, const int* lda, int* ipiv, float* b,
                 const int* ldb, int* info)
{ lapack_sgesv_impl(*n, *nrhs, a, *lda, ipiv, b, *ldb, info); }
void slate_sgesv_(const int* n, const int* nrhs, float* a, const int* lda, int* ipiv, float* b,
                  const int* ldb, int* info)
{ lapack_sgesv_impl(*n, *nrhs, a, *lda, ipiv, b, *ldb, info); }

} // extern "C"

template <typename T>
static void lapack_getrf_impl(int m, int n, T* a, int lda, int* ipiv, int* info)
{
    *info = 0;
    if (m < 0) { *info = -1; return; }
    if (n < 0) { *info = -2; return; }
    if (lda < std::max(1, m)) { *info = -4; return; }
    if (m == 0 || n == 0) return;
    cudaStream_t s = lapack_stream();
    slt_options o = lapack_opts();
    const int mn = std::min(m, n);
    DevBuf dA, dP;
    if (to_device(a, m, n, lda, dA, s) || dP.alloc(sizeof(int) * size_t(mn), s)) { *info = -100; return; }
    int64_t inf = 0;
    int rc = getrf_device_impl<T>(m, n, dA.as<T>(), m, dP.as<int>(), &o, s, &inf);
    if (rc) { *info = -1000 + rc; return; }
    std::vector<int> rel(mn);
    if (to_host(dA, a, m, n, lda, s) ||
        cudaMemcpyAsync(rel.data(), dP.p, sizeof(int) * size_t(mn), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) { *info = -100; return; }
    ipiv_to_lapack(rel, o.nb, ipiv, mn);
    *info = int(inf);
}

extern "C" {

void slate_dgetrf(const int* m, const int* n, double* a, const int* lda, int* ipiv, int* info)
{ lapack_getrf_impl<double>(*m, *n, a, *lda, ipiv, info); }
void slate_dgetrf_(const int* m, const int* n, double* a, const int* lda, int* ipiv, int* info)
{ lapack_getrf_impl<double>(*m, *n, a, *lda, ipiv, info); }
void slate_sgetrf(const int* m, const int* n, float* a, const int* lda, int* ipiv, int* info)
{ lapack_getrf_impl<float>(*m, *n, a, *lda, ipiv, info); }
void slate_sgetrf_(const int* m, const int* n, float* a, const int* lda, int* ipiv, int* info)
{ lapack_getrf_impl<float>(*m, *n, a, *lda, ipiv, info); }

static void lapack_getrs_impl(char trans, int n, int nrhs, double* a, int lda, int* ipiv, double* b, int ldb,
                              int* info)
{
    *info = 0;
    if (std::strchr("NnTtCc", trans) == nullptr || trans == 0) { *info = -1; return; }
    if (n < 0) { *info = -2; return; }
    if (nrhs < 0) { *info = -3; return; }
    if (lda < std::max(1, n)) { *info = -5; return; }
    if (ldb < std::max(1, n)) { *info = -8; return; }
    if (n == 0 || nrhs == 0) return;
    cudaStream_t s = lapack_stream();
    slt_options o = lapack_opts();
    std::vector<int> rel;
    ipiv_from_lapack(ipiv, o.nb, rel, n);
    DevBuf dA, dB, dP;
    if (to_device(a, n, n, lda, dA, s) || to_device(b, n, nrhs, ldb, dB, s) ||
        to_device(rel.data(), n, 1, n, dP, s)) { *info = -100; return; }
    int rc = slt_dgetrs_trans_device(trans, n, nrhs, dA.as<double>(), n, dP.as<int>(), dB.as<double>(), n, &o, s);
    if (rc) { *info = -1000 + rc; return; }
    if (to_host(dB, b, n, nrhs, ldb, s) || cudaStreamSynchronize(s) != cudaSuccess) { *info = -100; return; }
}

void slate_dgetrs(const char* trans, const int* n, const int* nrhs, double* a, const int* lda, int* ipiv,
                  double* b, const int* ldb, int* info)
{ lapack_getrs_impl(*trans, *n, *nrhs, a, *lda, ipiv, b, *ldb, info); }
void slate_dgetrs_(const char* trans, const int* n, const int* nrhs, double* a, const int* lda, int* ipiv,
                   double* b, const int* ldb, int* info)
{ lapack_getrs_impl(*trans, *n, *nrhs, a, *lda, ipiv, b, *ldb, info); }

static void lapack_dsgesv_impl(int n, int nrhs, double* a, int lda, int* ipiv, double* b, int ldb,
                               double* x, int ldx, int* iter, int* info)
{
    *info = 0;
    *iter = 0;
    if (n < 0) { *info = -1; return; }
    if (nrhs < 0) { *info = -2; return; }
    if (lda < std::max(1, n)) { *info = -4; return; }
    if (ldb < std::max(1, n)) { *info = -7; return; }
    if (ldx < std::max(1, n)) { *info = -9; return; }
    if (n == 0) return;
    cudaStream_t s = lapack_stream();
    slt_options o = lapack_opts();
    DevBuf dA, dB, dX, dP;
    if (to_device(a, n, n, lda, dA, s) || to_device(b, n, nrhs, ldb, dB, s) ||
        dX.alloc(sizeof(double) * size_t(n) * size_t(std::max(nrhs, 1)), s) ||
        dP.alloc(sizeof(int) * size_t(n), s)) { *info = -100; return; }
    int64_t inf = 0;
    int it = 0;
    int rc = slt_dsgesv_device(n, nrhs, dA.as<double>(), n, dP.as<int>(), dB.as<double>(), n,
                               dX.as<double>(), n, &o, s, &it, &inf);
    if (rc) { *info = -1000 + rc; return; }
    std::vector<int> rel(n);
    if (to_host(dX, x, n, nrhs, ldx, s) || to_host(dA, a, n, n, lda, s) ||
        cudaMemcpyAsync(rel.data(), dP.p, sizeof(int) * size_t(n), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) { *info = -100; return; }
    ipiv_to_lapack(rel, o.nb, ipiv, n);
    *iter = it;
    *info = int(inf);
}

void slate_dsgesv(const int* n, const int* nrhs, double* a, const int* lda, int* ipiv, double* b,
                  const int* ldb, double* x, const int* ldx, double* work, float* swork, int* iter, int* info)
{ (void) work; (void) swork; lapack_dsgesv_impl(*n, *nrhs, a, *lda, ipiv, b, *ldb, x, *ldx, iter, info); }
void slate_dsgesv_(const int* n, const int* nrhs, double* a, const int* lda, int* ipiv, double* b,
                   const int* ldb, double* x, const int* ldx, double* work, float* swork, int* iter, int* info)
{ (void) work; (void) swork; lapack_dsgesv_impl(*n, *nrhs, a, *lda, ipiv, b, *ldb, x, *ldx, iter, info); }

// posv / potrf with uplo: an upper-stored matrix is transposed on the device
// into lower storage (SLATE: A = conj_transpose(A), src/potrf.cc:45-47) and
// the factor is transposed back.
static int lower_view(char uplo, int64_t n, DevBuf& dA, DevBuf& tmp, cudaStream_t s)
{
    if (uplo == 'L' || uplo == 'l') return SLT_OK;
    int rc = tmp.alloc(sizeof(double) * size_t(n) * size_t(n), s);
    if (rc) return rc;
    rc = slt_dtranspose(n, n, dA.as<double>(), n, tmp.as<double>(), n, s);
    if (rc) return rc;
    std::swap(dA.p, tmp.p);
    return SLT_OK;
}

static void lapack_potrf_impl(char uplo, int n, double* a, int lda, int* info, int nrhs, double* b, int ldb)
{
    *info = 0;
    bool up = (uplo == 'U' || uplo == 'u');
    if (!up && uplo != 'L' && uplo != 'l') { *info = -1; return; }
    if (n < 0) { *info = -2; return; }
    if (nrhs < 0) { *info = -3; return; }
    if (lda < std::max(1, n)) { *info = b ? -5 : -4; return; }
    if (b && ldb < std::max(1, n)) { *info = -7; return; }
    if (n == 0) return;
    cudaStream_t s = lapack_stream();
    slt_options o = lapack_opts();
    DevBuf dA, dB, tmp;
    // only the referenced triangle crosses the link, both ways
    if (dA.alloc(sizeof(double) * size_t(n) * size_t(n), s) ||
        tri_copy<double>(!up, n, a, lda, dA.as<double>(), n, cudaMemcpyHostToDevice, s)) { *info = -100; return; }
    if (b && to_device(b, n, nrhs, ldb, dB, s)) { *info = -100; return; }
    if (lower_view(uplo, n, dA, tmp, s)) { *info = -100; return; }
    int64_t inf = 0;
    int rc = b ? slt_dposv_device(n, nrhs, dA.as<double>(), n, dB.as<double>(), n, &o, s, &inf)
               : slt_dpotrf_device(n, dA.as<double>(), n, &o, s, &inf);
    if (rc) { *info = -1000 + rc; return; }
    if (up) {
        rc = slt_dtranspose(n, n, dA.as<double>(), n, tmp.as<double>(), n, s);
        if (rc) { *info = -1000 + rc; return; }
        std::swap(dA.p, tmp.p);
    }
    if (tri_copy<double>(!up, n, dA.as<double>(), n, a, lda, cudaMemcpyDeviceToHost, s) ||
        (b && to_host(dB, b, n, nrhs, ldb, s)) || cudaStreamSynchronize(s) != cudaSuccess) { *info = -100; return; }
    *info = int(inf);
}

static void lapack_dsposv_impl(char uplo, int n, int nrhs, double* a, int lda, double* b, int ldb,
                               double* x, int ldx, int* iter, int* info)
{
    *info = 0;
    *iter = 0;
    bool up = (uplo == 'U' || uplo == 'u');
    if (!up && uplo != 'L' && uplo != 'l') { *info = -1; return; }
    if (n < 0) { *info = -2; return; }
    if (nrhs < 0) { *info = -3; return; }
    if (lda < std::max(1, n)) { *info = -5; return; }
    if (ldb < std::max(1, n)) { *info = -7; return; }
    if (ldx < std::max(1, n)) { *info = -9; return; }
    if (n == 0) return;
    cudaStream_t s = lapack_stream();
    slt_options o = lapack_opts();
    DevBuf dA, dB, dX, tmp;
    // phase timers of the host entry point (slt_timer("dsposv::h2d") etc.):
    // with streaming, h2d covers the work issued before the solve and the
    // copies of A overlap the solve's factorisation
    TimerSet tm(s);
    tm.start("dsposv::h2d");
    StreamedLower sl;
    // SLATE_LAPACK_STREAM: 0 copy A first, 1 (default) stream the lower
    // triangle by 512-column blocks, 2 stream whole block columns (one
    // contiguous copy each when lda == n: twice the bytes, plain 1-D copies)
    const char* se = std::getenv("SLATE_LAPACK_STREAM");
    const int smode = se ? std::atoi(se) : 1;
    const bool stream_a = !up && smode != 0;
    // B first: a copy queued on the compute stream behind A's blocks on the
    // copy engine would hold the solve back until all of A had arrived.
    // Only the referenced triangle of A crosses the link.
    if (to_device(b, n, nrhs, ldb, dB, s) ||
        dX.alloc(sizeof(double) * size_t(n) * size_t(std::max(nrhs, 1)), s) ||
        dA.alloc(sizeof(double) * size_t(n) * size_t(n), s) ||
        (stream_a ? sl.start(n, a, lda, dA.as<double>(), s, lapack_copy_stream(), smode == 2)
                  : tri_copy<double>(!up, n, a, lda, dA.as<double>(), n, cudaMemcpyHostToDevice, s))) {
        *info = -100;
        return;
    }
    if (lower_view(uplo, n, dA, tmp, s)) { *info = -100; return; }
    tm.stop("dsposv::h2d");
    int64_t inf = 0;
    int it = 0;
    tm.start("dsposv::solve");
    int rc;
    {
        InputArrivalScope scope(stream_a ? &sl.arr : nullptr);
        rc = slt_dsposv_device(n, nrhs, dA.as<double>(), n, dB.as<double>(), n, dX.as<double>(), n, &o, s,
                               &it, &inf);
    }
    if (stream_a && !rc) rc = sl.join(s);
    if (rc) { *info = -1000 + rc; return; }
    tm.stop("dsposv::solve");
    tm.start("dsposv::d2h");
    if (to_host(dX, x, n, nrhs, ldx, s)) { *info = -100; return; }
    tm.stop("dsposv::d2h");
    if (cudaStreamSynchronize(s) != cudaSuccess) { *info = -100; return; }
    if (it < 0) {
        // the FP64 fallback ran: A holds its Cholesky factor (referenced triangle)
        if (up) {
            rc = slt_dtranspose(n, n, dA.as<double>(), n, tmp.as<double>(), n, s);
            if (rc) { *info = -1000 + rc; return; }
            std::swap(dA.p, tmp.p);
        }
        if (tri_copy<double>(!up, n, dA.as<double>(), n, a, lda, cudaMemcpyDeviceToHost, s) ||
            cudaStreamSynchronize(s) != cudaSuccess) { *info = -100; return; }
    }
    *iter = it;
    *info = int(inf);
}

void slate_dsposv(const char* uplo, const int* n, const int* nrhs, double* a, const int* lda, double* b,
                  const int* ldb, double* x, const int* ldx, double* work, float* swork, int* iter, int* info)
{ (void) work; (void) swork; lapack_dsposv_impl(*uplo, *n, *nrhs, a, *lda, b, *ldb, x, *ldx, iter, info); }
void slate_dsposv_(const char* uplo, const int* n, const int* nrhs, double* a, const int* lda, double* b,
                   const int* ldb, double* x, const int* ldx, double* work, float* swork, int* iter, int* info)
{ (void) work; (void) swork; lapack_dsposv_impl(*uplo, *n, *nrhs, a, *lda, b, *ldb, x, *ldx, iter, info); }

void slate_dposv(const char* uplo, const int* n, const int* nrhs, double* a, const int* lda, double* b,
                 const int* ldb, int* info)
{ lapack_potrf_impl(*uplo, *n, a, *lda, info, *nrhs, b, *ldb); }
void slate_dposv_(const char* uplo, const int* n, const int* nrhs, double* a, const int* lda, double* b,
                  const int* ldb, int* info)
{ lapack_potrf_impl(*uplo, *n, a, *lda, info, *nrhs, b, *ldb); }
void slate_dpotrf(const char* uplo, const int* n, double* a, const int* lda, int* info)
{ lapack_potrf_impl(*uplo, *n, a, *lda, info, 0, nullptr, 1); }
void slate_dpotrf_(const char* uplo, const int* n, double* a, const int* lda, int* info)
{ lapack_potrf_impl(*uplo, *n, a, *lda, info, 0, nullptr, 1); }

} // extern "C"
