// drivers.cc -- C++ host drivers of the LU / Cholesky solve path.
//
// The drivers issue stream-ordered launches of the kernel layer
// (slt_kernels.h) and never synchronise inside a factorisation; the only
// host reads are the ones SLATE's own algorithms need (norms and stopping
// tests of the refinement loops, the Givens rotations of GMRES, info).

#include "drivers.h"
#include "driver_table.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <mutex>
#include <string>
#include <utility>
#include <functional>
#include <vector>

namespace slt {

// ---------------------------------------------------------------------------
// Timers: the slate::timers keys of the reference drivers, measured with CUDA
// events on the driver's stream and resolved when the call ends.
static thread_local std::map<std::string, double> t_timers;

TimerSet::~TimerSet()
{
    for (auto& kv : open) cudaEventDestroy(kv.second);
    if (spans.empty()) return;
    cudaStreamSynchronize(s);
    std::map<std::string, double> acc;
    for (auto& sp : spans) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, sp.a, sp.b) == cudaSuccess) acc[sp.key] += ms * 1e-3;
        cudaEventDestroy(sp.a);
        cudaEventDestroy(sp.b);
    }
    cudaGetLastError();
    for (auto& kv : acc) t_timers[kv.first] = kv.second;
}

bool plain_alloc()
{
    static const bool plain = [] {
        const char* e = std::getenv("SLT_WORKSPACE_POOL");
        return e && std::atoi(e) == 0;
    }();
    return plain;
}

static thread_local const InputArrival* t_arrival = nullptr;
const InputArrival* input_arrival() { return t_arrival; }
InputArrivalScope::InputArrivalScope(const InputArrival* a) { t_arrival = a; }
InputArrivalScope::~InputArrivalScope() { t_arrival = nullptr; }

double timer_value(const char* name)
{
    auto it = t_timers.find(name);
    return it == t_timers.end() ? -1.0 : it->second;
}

void timers_clear() { t_timers.clear(); }


// ---------------------------------------------------------------------------
// Workspace pool: one per device, release threshold "never", so that the
// physical memory of a call's workspace stays mapped for the next call.
static std::mutex g_pool_mtx;
static cudaMemPool_t g_pools[64] = {};

cudaMemPool_t workspace_pool()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) { cudaGetLastError(); return nullptr; }
    std::lock_guard<std::mutex> lk(g_pool_mtx);
    if (!g_pools[dev]) {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.handleTypes = cudaMemHandleTypeNone;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool = nullptr;
        if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) { cudaGetLastError(); return nullptr; }
        uint64_t keep = ~uint64_t(0);
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        cudaGetLastError();
        g_pools[dev] = pool;
    }
    return g_pools[dev];
}

} // namespace slt

// Returns the memory the library's workspace pool holds on the current device
// (for callers that need it back between solves).
extern "C" int slt_release_workspace(void)
{
    cudaMemPool_t pool = slt::workspace_pool();
    if (!pool) return SLT_OK;
    SLT_CUDA_TRY(cudaDeviceSynchronize());
    SLT_CUDA_TRY(cudaMemPoolTrimTo(pool, 0));
    return SLT_OK;
}

namespace slt {

// ---------------------------------------------------------------------------
// Type dispatch onto the kernel layer.
static int k_gemm(char tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A, int64_t lda,
                  const double* B, int64_t ldb, double beta, double* C, int64_t ldc, int lower,
                  const slt_options& o, cudaStream_t s)
{ return slt_dgemm(tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, lower, o.gemm_engine, s); }

static int k_gemm(char tb, int64_t m, int64_t n, int64_t k, float alpha, const float* A, int64_t lda,
                  const float* B, int64_t ldb, float beta, float* C, int64_t ldc, int lower,
                  const slt_options& o, cudaStream_t s)
{
    int tier = o.factor_precision;
    if ((tier == SLT_PREC_TF32 || tier == SLT_PREC_BF16 || tier == SLT_PREC_FP16 || tier == SLT_PREC_FP8 ||
         tier == SLT_PREC_TF32X3) &&
        alpha == -1.f
        && beta == 1.f && k >= 16 && m >= 128 && n >= 128)
        return slt_tc_gemm_update(tier, tb, m, n, k, A, lda, B, ldb, C, ldc, lower, nullptr, 0, s);
    return slt_sgemm(tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, lower, s);
}

static int k_panel(int64_t prows, int64_t nbk, int64_t ib, double thr, double* P, int64_t ld, int* ipiv, int* info,
                   int64_t off, void* ws, int* status, cudaStream_t s)
{ return slt_dgetrf_panel(prows, nbk, ib, P, ld, ipiv, info, off, thr, ws, status, s); }
static int k_panel(int64_t prows, int64_t nbk, int64_t ib, double thr, float* P, int64_t ld, int* ipiv, int* info,
                   int64_t off, void* ws, int* status, cudaStream_t s)
{ return slt_sgetrf_panel(prows, nbk, ib, P, ld, ipiv, info, off, thr, ws, status, s); }

static int k_laswp(const int* plan, int64_t maxc, double* A, int64_t lda, int64_t nc, cudaStream_t s)
{ return slt_dlaswp_plan(plan, maxc, A, lda, nc, s); }
static int k_laswp(const int* plan, int64_t maxc, float* A, int64_t lda, int64_t nc, cudaStream_t s)
{ return slt_slaswp_plan(plan, maxc, A, lda, nc, s); }

static int k_trsm_llnu(int64_t kb, int64_t n, const double* L, int64_t ldl, double* B, int64_t ldb, cudaStream_t s)
{ return slt_dtrsm_llnu(kb, n, L, ldl, B, ldb, s); }
static int k_trsm_llnu(int64_t kb, int64_t n, const float* L, int64_t ldl, float* B, int64_t ldb, cudaStream_t s)
{ return slt_strsm_llnu(kb, n, L, ldl, B, ldb, s); }
static int k_trsm_lunn(int64_t kb, int64_t n, const double* U, int64_t ldu, double* B, int64_t ldb, cudaStream_t s)
{ return slt_dtrsm_lunn(kb, n, U, ldu, B, ldb, s); }
static int k_trsm_lunn(int64_t kb, int64_t n, const float* U, int64_t ldu, float* B, int64_t ldb, cudaStream_t s)
{ return slt_strsm_lunn(kb, n, U, ldu, B, ldb, s); }
static int k_trsm_llnn(char tr, int64_t kb, int64_t n, const double* L, int64_t ldl, double* B, int64_t ldb, cudaStream_t s)
{ return slt_dtrsm_llnn(tr, kb, n, L, ldl, B, ldb, s); }
static int k_trsm_llnn(char tr, int64_t kb, int64_t n, const float* L, int64_t ldl, float* B, int64_t ldb, cudaStream_t s)
{ return slt_strsm_llnn(tr, kb, n, L, ldl, B, ldb, s); }
static int k_trsm_runn(int64_t m, int64_t kb, const double* U, int64_t ldu, double* B, int64_t ldb, cudaStream_t s)
{ return slt_dtrsm_runn(m, kb, U, ldu, B, ldb, s); }
static int k_trsm_runn(int64_t m, int64_t kb, const float* U, int64_t ldu, float* B, int64_t ldb, cudaStream_t s)
{ return slt_strsm_runn(m, kb, U, ldu, B, ldb, s); }
static int k_trsm_rltn(int64_t m, int64_t kb, const double* L, int64_t ldl, double* B, int64_t ldb, cudaStream_t s)
{ return slt_dtrsm_rltn(m, kb, L, ldl, B, ldb, s); }
static int k_trsm_rltn(int64_t m, int64_t kb, const float* L, int64_t ldl, float* B, int64_t ldb, cudaStream_t s)
{ return slt_strsm_rltn(m, kb, L, ldl, B, ldb, s); }
static int k_potrf_small(int64_t kb, double* A, int64_t lda, int* info, int64_t off, cudaStream_t s)
{ return slt_dpotrf_small(kb, A, lda, info, off, s); }
static int k_potrf_small(int64_t kb, float* A, int64_t lda, int* info, int64_t off, cudaStream_t s)
{ return slt_spotrf_small(kb, A, lda, info, off, s); }

static int k_skinny(int64_t m, int64_t nrhs, int64_t k, double alpha, const double* A, int64_t lda,
                    const double* X, int64_t ldx, double beta, double* C, int64_t ldc, void* ws, cudaStream_t s)
{ return slt_dgemm_skinny(m, nrhs, k, alpha, A, lda, 0, X, ldx, beta, C, ldc, ws, s); }
static int k_skinny(int64_t m, int64_t nrhs, int64_t k, float alpha, const float* A, int64_t lda,
                    const float* X, int64_t ldx, float beta, float* C, int64_t ldc, void*, cudaStream_t s)
{ return slt_sgemm_skinny(m, nrhs, k, alpha, A, lda, X, ldx, beta, C, ldc, s); }
static int k_skinny_t(int64_t m, int64_t nrhs, int64_t kk, double alpha, const double* A, int64_t lda,
                      const double* X, int64_t ldx, double beta, double* C, int64_t ldc, cudaStream_t s)
{ return slt_dgemm_skinny_t(m, nrhs, kk, alpha, A, lda, X, ldx, beta, C, ldc, s); }
static int k_skinny_t(int64_t m, int64_t nrhs, int64_t kk, float alpha, const float* A, int64_t lda,
                      const float* X, int64_t ldx, float beta, float* C, int64_t ldc, cudaStream_t s)
{ return slt_sgemm_skinny_t(m, nrhs, kk, alpha, A, lda, X, ldx, beta, C, ldc, s); }
static int k_permute(int fwd, const int* perm, int64_t n, int64_t nc, const double* X, int64_t ldx,
                     double* Y, int64_t ldy, cudaStream_t s)
{ return slt_dpermute_rows(fwd, perm, n, nc, X, ldx, Y, ldy, s); }
static int k_permute(int fwd, const int* perm, int64_t n, int64_t nc, const float* X, int64_t ldx,
                     float* Y, int64_t ldy, cudaStream_t s)
{ return slt_spermute_rows(fwd, perm, n, nc, X, ldx, Y, ldy, s); }

static int64_t eff_nb(const slt_options& o) { return o.nb > 0 ? o.nb : 512; }
static int64_t eff_ib(const slt_options& o, int64_t nb)
{
    int64_t ib = o.ib > 0 ? o.ib : 32;
    return std::max<int64_t>(1, std::min<int64_t>(std::min<int64_t>(ib, 64), nb));
}

int finish_factor(FactorCtx& fc, int64_t* info, cudaStream_t s)
{
    int h[2] = {0, 0};
    if (fc.d_info) SLT_CUDA_TRY(cudaMemcpyAsync(&h[0], fc.d_info, sizeof(int), cudaMemcpyDeviceToHost, s));
    if (fc.d_status) SLT_CUDA_TRY(cudaMemcpyAsync(&h[1], fc.d_status, sizeof(int), cudaMemcpyDeviceToHost, s));
    SLT_CUDA_TRY(cudaStreamSynchronize(s));
    if (info) *info = h[0];
    return h[1] != 0 ? h[1] : SLT_OK;
}

// ---------------------------------------------------------------------------
// Lookahead (Option::Lookahead, src/getrf.cc:39,120-135, src/potrf.cc:41-61):
// after the panel of step k, the next block column is updated first, on the
// caller's stream, and the rest of the trailing matrix on a second,
// lower-priority stream, so that the panel of step k+1 runs while the update
// of step k is still going.  The two get disjoint shares of the SMs: the
// panel launches take `panel_sms` SMs, the trailing update the rest
// (slt_set_sm_cap).  Events order the streams:
//   panel k+1       after  lookahead update k       (same stream)
//   swaps / lookahead update k+1   after  rest update k   (ev_rest)
//   rest update k   after  panel k and the U12 solve of step k (ev_row)
// The autotuned choices (driver_table.h) for a factorisation of order n:
// kind 0 getrf, 1 potrf; cls 0 FP64, 1 FP32 SIMT, 2 tensor cores.
static const DriverTune& driver_tune(int kind, int cls, int64_t n)
{
    const DriverTune* last = nullptr;
    for (const DriverTune& t : kDriverTable) {
        if (t.kind != kind || t.cls != cls) continue;
        last = &t;
        if (n <= t.max_n) return t;
    }
    static const DriverTune none{kind, cls, 0, 0, 1};
    return last ? *last : none;
}

template <typename T>
static int update_class(const slt_options& o)
{
    if (sizeof(T) == 8) return 0;
    const int p = o.factor_precision;
    return (p == SLT_PREC_TF32 || p == SLT_PREC_BF16 || p == SLT_PREC_FP16 || p == SLT_PREC_FP8 ||
            p == SLT_PREC_TF32X3) ? 2 : 1;
}

// SMs given to the panel while an update runs beside it: SLT_LOOKAHEAD_PANEL_SMS
// when set (the tuner's override; 0 turns the overlap off), else the table's.
static int lookahead_panel_sms(const DriverTune& t, int sms)
{
    if (const char* e = std::getenv("SLT_LOOKAHEAD_PANEL_SMS")) return std::atoi(e);
    return std::min(t.panel_sms, sms);
}

// Panels per deferred trailing update of potrf (1: update after every
// panel): SLT_UPDATE_DEPTH when set (the tuner's override), else the table's.
static int64_t update_depth(const DriverTune& t)
{
    if (const char* e = std::getenv("SLT_UPDATE_DEPTH")) return std::max(1, std::atoi(e));
    return std::max(1, t.depth);
}

struct Lookahead {
    bool on = false;
    cudaStream_t s = nullptr, su = nullptr;
    cudaEvent_t ev_row = nullptr, ev_rest = nullptr;
    int sms = 0, panel_sms = 0;
    bool rest_pending = false;

    int init(const slt_options& o, const DriverTune& tune, int64_t n, int64_t nb, cudaStream_t stream) {
        s = stream;
        const int64_t depth = o.lookahead;
        if (depth <= 0 || n <= 2 * nb) return SLT_OK;
        int dev = 0;
        SLT_CUDA_TRY(cudaGetDevice(&dev));
        SLT_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        panel_sms = lookahead_panel_sms(tune, sms);
        if (panel_sms <= 0 || panel_sms >= sms) return SLT_OK;
        int lo = 0, hi = 0;
        SLT_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        SLT_CUDA_TRY(cudaStreamCreateWithPriority(&su, cudaStreamNonBlocking, lo));
        SLT_CUDA_TRY(cudaEventCreateWithFlags(&ev_row, cudaEventDisableTiming));
        SLT_CUDA_TRY(cudaEventCreateWithFlags(&ev_rest, cudaEventDisableTiming));
        on = true;
        return SLT_OK;
    }
    // the caller's stream waits for the last rest update
    int join() {
        if (!on || !rest_pending) return SLT_OK;
        SLT_CUDA_TRY(cudaStreamWaitEvent(s, ev_rest, 0));
        rest_pending = false;
        return SLT_OK;
    }
    ~Lookahead() {
        if (su) { join(); cudaStreamDestroy(su); }
        if (ev_row) cudaEventDestroy(ev_row);
        if (ev_rest) cudaEventDestroy(ev_rest);
    }
};

// Scoped SM budget for the launches issued on this thread.
struct SmCap {
    int prev;
    explicit SmCap(int sms) : prev(slt_set_sm_cap(sms)) {}
    ~SmCap() { slt_set_sm_cap(prev); }
};

// ---------------------------------------------------------------------------
// LU: right-looking, one cooperative panel launch per block column, then the
// panel's interchanges on both sides, the U12 solve and the trailing GEMM
// (impl::getrf, src/getrf.cc:22-244).  MethodLU::NoPiv is the panel's
// threshold rule with threshold 0.  MethodLU::CALU follows SLATE's device path
// on a 1 x 1 grid (src/getrf_tntpiv.cc, internal_getrf_tntpiv.cc:120-172): the
// tournament has one participant, which factors the whole local panel with
// partial pivoting, so the pivots are the partial-pivoting panel's; the
// diagonal block keeps that factorisation and L21 is recomputed from the
// original panel rows, permuted by the pivots, as A21 U11^{-1}.
template <typename T>
int getrf_dev(int64_t m, int64_t n, T* A, int64_t lda, int* ipiv, const slt_options& o,
              FactorCtx& fc, cudaStream_t s)
{
    if (m < 0 || n < 0 || lda < std::max<int64_t>(1, m)) return SLT_ERR_ARG;
    const int64_t nb = eff_nb(o);
    const int64_t ib = eff_ib(o, nb);
    const int64_t mn = std::min(m, n);
    if (mn == 0) return SLT_OK;
    if (nb > 1024) return SLT_ERR_ARG;
    const bool calu = o.method_lu == 'C' || o.method_lu == 'c';
    const bool nopiv = o.method_lu == 'N' || o.method_lu == 'n';
    DevBuf pws, plan, W, plan0;
    TRY(pws.alloc(slt_getrf_panel_ws_bytes(m, ib), s));
    TRY(plan.alloc(sizeof(int) * size_t(1 + 4 * nb), s));
    if (calu) {
        TRY(W.alloc(sizeof(T) * size_t(m) * size_t(std::min(nb, n)), s));
        TRY(plan0.alloc(sizeof(int) * size_t(1 + 4 * nb), s));
    }
    const DriverTune& tune = driver_tune(0, update_class<T>(o), std::min(m, n));
    slt_options ot = o;
    if (ot.gemm_engine == 0) ot.gemm_engine = tune.engine;
    Lookahead la;
    TRY(la.init(o, tune, std::min(m, n), nb, s));
    for (int64_t r0 = 0; r0 < mn; r0 += nb) {
        const int64_t nbk = std::min(nb, n - r0);
        const int64_t prows = m - r0;
        const int64_t diag = std::min(prows, nbk);
        T* P = A + r0 + r0 * lda;
        double thr = (o.pivot_threshold >= 0.0 && o.pivot_threshold <= 1.0) ? o.pivot_threshold : 1.0;
        if (nopiv) thr = 0.0;
        if (calu)
            SLT_CUDA_TRY(cudaMemcpy2DAsync(W.p, sizeof(T) * size_t(prows), P, sizeof(T) * size_t(lda),
                                           sizeof(T) * size_t(prows), size_t(nbk), cudaMemcpyDeviceToDevice, s));
        {
            // the panel shares the GPU with the previous step's rest update
            SmCap cap(la.rest_pending ? la.panel_sms : 0);
            TRY(k_panel(prows, nbk, ib, thr, P, lda, ipiv + r0, fc.d_info, r0, pws.p, fc.d_status, s));
        }
        TRY(slt_swap_plan(ipiv + r0, diag, r0, plan.as<int>(), s));
        if (calu && prows > diag) {
            // W <- the panel's interchanges applied to the original panel;
            // L21 = W21 U11^{-1}
            TRY(slt_swap_plan(ipiv + r0, diag, 0, plan0.as<int>(), s));
            TRY(k_laswp(plan0.as<int>(), 2 * diag, W.as<T>(), prows, diag, s));
            SLT_CUDA_TRY(cudaMemcpy2DAsync(P + diag, sizeof(T) * size_t(lda), W.as<T>() + diag,
                                           sizeof(T) * size_t(prows), sizeof(T) * size_t(prows - diag),
                                           size_t(diag), cudaMemcpyDeviceToDevice, s));
            TRY(k_trsm_runn(prows - diag, diag, P, lda, P + diag, lda, s));
        }
        const int64_t c1 = r0 + nbk;
        // the interchanges touch every column to the right: the previous
        // rest update must be done with them
        TRY(la.join());
        TRY(k_laswp(plan.as<int>(), 2 * diag, A + c1 * lda, lda, n - c1, s));
        TRY(k_laswp(plan.as<int>(), 2 * diag, A, lda, r0, s));
        if (c1 < n) {
            TRY(k_trsm_llnu(diag, n - c1, P, lda, A + r0 + c1 * lda, lda, s));
            if (r0 + diag < m) {
                const int64_t rows = m - r0 - diag;
                const T* L21 = A + (r0 + diag) + r0 * lda;
                if (!la.on || n - c1 <= nb) {
                    TRY(k_gemm('N', rows, n - c1, diag, T(-1), L21, lda, A + r0 + c1 * lda, lda, T(1),
                               A + (r0 + diag) + c1 * lda, lda, 0, ot, s));
                }
                else {
                    // rest of the trailing matrix on the second stream
                    const int64_t c2 = c1 + nb;
                    SLT_CUDA_TRY(cudaEventRecord(la.ev_row, s));
                    SLT_CUDA_TRY(cudaStreamWaitEvent(la.su, la.ev_row, 0));
                    {
                        SmCap cap(la.sms - la.panel_sms);
                        TRY(k_gemm('N', rows, n - c2, diag, T(-1), L21, lda, A + r0 + c2 * lda, lda, T(1),
                                   A + (r0 + diag) + c2 * lda, lda, 0, ot, la.su));
                    }
                    SLT_CUDA_TRY(cudaEventRecord(la.ev_rest, la.su));
                    la.rest_pending = true;
                    // lookahead: the next block column first, on the caller's stream
                    TRY(k_gemm('N', rows, nb, diag, T(-1), L21, lda, A + r0 + c1 * lda, lda, T(1),
                               A + (r0 + diag) + c1 * lda, lda, 0, ot, s));
                }
            }
        }
    }
    return la.join();
}

// getrs NoTrans: W = P B, forward sweep with unit L, backward with U
// (src/getrs.cc:66-117; work::trsmA, src/work/work_trsmA.cc:147-480), each
// sweep one persistent launch.
static int k_sweep(int kind, int64_t n, int64_t nrhs, const double* M, int64_t ldm, double* X, int64_t ldx,
                   int* flags, int* status, cudaStream_t s)
{ return slt_dsweep(kind, n, nrhs, M, ldm, X, ldx, flags, status, s); }
static int k_sweep(int kind, int64_t n, int64_t nrhs, const float* M, int64_t ldm, float* X, int64_t ldx,
                   int* flags, int* status, cudaStream_t s)
{ return slt_ssweep(kind, n, nrhs, M, ldm, X, ldx, flags, status, s); }

template <typename T>
int getrs_dev(int64_t n, int64_t nrhs, const T* LU, int64_t lda, const int* ipiv, int64_t nb,
              T* B, int64_t ldb, int* d_status, cudaStream_t s)
{
    if (n < 0 || nrhs < 0) return SLT_ERR_ARG;
    if (n == 0 || nrhs == 0) return SLT_OK;
    DevBuf perm, W, flags;
    TRY(perm.alloc(sizeof(int) * size_t(n), s));
    TRY(W.alloc(sizeof(T) * size_t(n) * size_t(std::min<int64_t>(nrhs, 16)), s));
    TRY(flags.alloc(slt_sweep_flags_bytes(n), s));
    TRY(slt_perm_from_ipiv(ipiv, n, nb, perm.as<int>(), s));
    T* w = W.as<T>();
    for (int64_t c0 = 0; c0 < nrhs; c0 += 16) {
        const int64_t nc = std::min<int64_t>(16, nrhs - c0);
        TRY(k_permute(1, perm.as<int>(), n, nc, B + c0 * ldb, ldb, w, n, s));
        TRY(k_sweep(0, n, nc, LU, lda, w, n, flags.as<int>(), d_status, s));
        TRY(k_sweep(1, n, nc, LU, lda, w, n, flags.as<int>(), d_status, s));
        SLT_CUDA_TRY(cudaMemcpy2DAsync(B + c0 * ldb, size_t(ldb) * sizeof(T), w, size_t(n) * sizeof(T),
                                       size_t(n) * sizeof(T), size_t(nc), cudaMemcpyDeviceToDevice, s));
    }
    return SLT_OK;
}

// getrs Trans (src/getrs.cc:66-117 with Op::Trans): A^T X = B with
// P A = L U is U^T L^T P X = B: a forward sweep with U^T, a backward sweep
// with L^T, then the inverse row permutation.
template <typename T>
int getrs_trans_dev(int64_t n, int64_t nrhs, const T* LU, int64_t lda, const int* ipiv, int64_t nb,
                    T* B, int64_t ldb, int* d_status, cudaStream_t s)
{
    if (n < 0 || nrhs < 0) return SLT_ERR_ARG;
    if (n == 0 || nrhs == 0) return SLT_OK;
    DevBuf perm, W, flags;
    TRY(perm.alloc(sizeof(int) * size_t(n), s));
    TRY(W.alloc(sizeof(T) * size_t(n) * size_t(std::min<int64_t>(nrhs, 16)), s));
    TRY(flags.alloc(slt_sweep_flags_bytes(n), s));
    TRY(slt_perm_from_ipiv(ipiv, n, nb, perm.as<int>(), s));
    T* w = W.as<T>();
    for (int64_t c0 = 0; c0 < nrhs; c0 += 16) {
        const int64_t nc = std::min<int64_t>(16, nrhs - c0);
        SLT_CUDA_TRY(cudaMemcpy2DAsync(w, size_t(n) * sizeof(T), B + c0 * ldb, size_t(ldb) * sizeof(T),
                                       size_t(n) * sizeof(T), size_t(nc), cudaMemcpyDeviceToDevice, s));
        TRY(k_sweep(4, n, nc, LU, lda, w, n, flags.as<int>(), d_status, s));
        TRY(k_sweep(5, n, nc, LU, lda, w, n, flags.as<int>(), d_status, s));
        TRY(k_permute(0, perm.as<int>(), n, nc, w, n, B + c0 * ldb, ldb, s));
    }
    return SLT_OK;
}

// Cholesky, lower: block columns of nb; inside a block column, 64-wide
// steps of small potrf + solve of everything below + update of the rest of
// the block column; then the herk-shaped trailing update
// (impl::potrf, src/potrf.cc:22-210).
static int k_chol_panel(int64_t m, int64_t nbk, double* P, int64_t ld, int* info, int64_t off, void* ws,
                        int* status, cudaStream_t s)
{ return slt_dchol_panel(m, nbk, P, ld, info, off, ws, status, s); }
static int k_chol_panel(int64_t m, int64_t nbk, float* P, int64_t ld, int* info, int64_t off, void* ws,
                        int* status, cudaStream_t s)
{ return slt_schol_panel(m, nbk, P, ld, info, off, ws, status, s); }

template <typename T>
int potrf_dev(int64_t n, T* A, int64_t lda, const slt_options& o, FactorCtx& fc, cudaStream_t s)
{
    if (n < 0 || lda < std::max<int64_t>(1, n)) return SLT_ERR_ARG;
    const int64_t nb = eff_nb(o);
    DevBuf bar;
    TRY(bar.alloc(slt_chol_panel_ws_bytes(), s));
    const DriverTune& tune = driver_tune(1, update_class<T>(o), n);
    slt_options ot = o;
    if (ot.gemm_engine == 0) ot.gemm_engine = tune.engine;
    Lookahead la;
    TRY(la.init(o, tune, n, nb, s));
    const int64_t depth = update_depth(tune);
    if (!la.on && depth > 1) {
        // Deferred trailing update: the panels of a block of `depth` panels
        // are factored one after the other, each block column first brought
        // up to date with the block's earlier panels (a GEMM with k = the
        // columns factored so far in the block), and the rest of the
        // trailing matrix takes one update with k = depth * nb.  Same
        // factor L; the trailing matrix is read and written once per block
        // instead of once per panel.
        for (int64_t r0 = 0; r0 < n; r0 += depth * nb) {
            const int64_t sb = std::min(depth * nb, n - r0);
            for (int64_t c = r0; c < r0 + sb; c += nb) {
                const int64_t kb = std::min(nb, n - c);
                if (c > r0)
                    TRY(k_gemm('T', n - c, kb, c - r0, T(-1), A + c + r0 * lda, lda, A + c + r0 * lda, lda, T(1),
                               A + c + c * lda, lda, 1, ot, s));
                TRY(k_chol_panel(n - c, kb, A + c + c * lda, lda, fc.d_info, c, bar.p, fc.d_status, s));
            }
            const int64_t t0 = r0 + sb;
            if (t0 >= n) break;
            const T* L = A + t0 + r0 * lda;
            TRY(k_gemm('T', n - t0, n - t0, sb, T(-1), L, lda, L, lda, T(1), A + t0 + t0 * lda, lda, 1, ot, s));
        }
        return SLT_OK;
    }
    for (int64_t r0 = 0; r0 < n; r0 += nb) {
        const int64_t kb = std::min(nb, n - r0);
        {
            // the whole column panel (diagonal block and everything below) in
            // one launch, beside the previous step's rest update
            SmCap cap(la.rest_pending ? la.panel_sms : 0);
            TRY(k_chol_panel(n - r0, kb, A + r0 + r0 * lda, lda, fc.d_info, r0, bar.p, fc.d_status, s));
        }
        const int64_t t0 = r0 + kb;
        if (t0 >= n) break;
        const T* L = A + t0 + r0 * lda;
        if (!la.on || n - t0 <= nb) {
            TRY(la.join());
            TRY(k_gemm('T', n - t0, n - t0, kb, T(-1), L, lda, L, lda, T(1), A + t0 + t0 * lda, lda, 1, ot, s));
            continue;
        }
        // rest of the trailing matrix (columns t0 + nb ...) on the second stream
        const int64_t t2 = t0 + nb;
        SLT_CUDA_TRY(cudaEventRecord(la.ev_row, s));
        // the previous rest update wrote block column t0: it must be done
        // before the lookahead update below
        TRY(la.join());
        SLT_CUDA_TRY(cudaStreamWaitEvent(la.su, la.ev_row, 0));
        {
            SmCap cap(la.sms - la.panel_sms);
            TRY(k_gemm('T', n - t2, n - t2, kb, T(-1), A + t2 + r0 * lda, lda, A + t2 + r0 * lda, lda, T(1),
                       A + t2 + t2 * lda, lda, 1, ot, la.su));
        }
        SLT_CUDA_TRY(cudaEventRecord(la.ev_rest, la.su));
        la.rest_pending = true;
        // lookahead: block column t0 (rows t0 .. n), lower part of its diagonal tile
        TRY(k_gemm('T', n - t0, nb, kb, T(-1), L, lda, L, lda, T(1), A + t0 + t0 * lda, lda, 1, ot, s));
    }
    return la.join();
}

// Left-looking Cholesky by blocks of S columns for the 16-bit tensor-core
// tiers (FP16, BF16), S a multiple of 64: before block [s0, s1) is factored,
// its columns (rows s0 .. n) take the whole contribution of columns 0 .. s0
// in one tensor-core update with k = s0, read from a row-major 16-bit copy of
// the factor (L16); inside the block, each nb-column panel is brought up to
// date with the block's earlier panels (again from L16), factored by the
// panel kernel, and its rows below it added to L16.  Same factor as the
// right-looking order (the same operand roundings, FP32 sums grouped
// differently), but the trailing matrix is read and written once in all,
// every column is packed once instead of at every update, and block s needs
// only columns s0 .. s1 of A -- which lets the caller stream A in while
// earlier blocks are being factored (prologue(s0, s1, stream) runs first on
// each block).
// Width of the left-looking factor's SIMT panels: SLT_LL_PANEL_WIDTH when
// set (a multiple of 64 dividing nb), else 256 when it divides nb, else nb.
// The block's earlier panels reach each panel through the tensor-core
// update, so a narrower panel moves the intra-block update work from the
// SIMT panel to tcgen05 (n = 65536, nb = 512: 138.5 ms factor at width 512,
// 130.3 ms at 256, 136.7 ms at 128).
static int64_t potrf_ll_panel_width(const slt_options& o)
{
    const int64_t nb = eff_nb(o);
    if (const char* e = std::getenv("SLT_LL_PANEL_WIDTH")) {
        const int64_t w = std::atoll(e);
        if (w >= 64 && w % 64 == 0 && nb % w == 0) return w;
    }
    return nb % 256 == 0 ? 256 : nb;
}

static int potrf_ll_tc(int64_t n, float* A, int64_t lda, const slt_options& o, int64_t S, FactorCtx& fc,
                       cudaStream_t s, const std::function<int(int64_t, int64_t, cudaStream_t)>& prologue,
                       int panel_sms)
{
    const int64_t nb = potrf_ll_panel_width(o);
    const int tier = o.factor_precision;
    DevBuf bar, L16;
    TRY(bar.alloc(slt_chol_panel_ws_bytes(), s));
    const int64_t kld = (n + 63) / 64 * 64;
    TRY(L16.alloc(size_t(n) * size_t(kld) * 2, s));
    char* L16b = L16.as<char>();
    auto rows16 = [&](int64_t r, int64_t k) { return L16b + (size_t(r) * size_t(kld) + size_t(k)) * 2; };
    // the panels of one block, each brought up to date with the block's
    // earlier panels from L16 and added to L16 (rows below it) once factored
    auto panels = [&](int64_t s0, int64_t s1) -> int {
        for (int64_t c = s0; c < s1; c += nb) {
            const int64_t kb = std::min(nb, s1 - c);
            if (c > s0)
                TRY(slt_tc_gemm_packed(tier, n - c, kb, c - s0, rows16(c, s0), kld, rows16(c, s0), kld,
                                       A + c + c * lda, lda, 1, s));
            TRY(k_chol_panel(n - c, kb, A + c + c * lda, lda, fc.d_info, c, bar.p, fc.d_status, s));
            if (c + kb < n) TRY(slt_pack_rows16(tier, n, c + kb, c, c + kb, A, lda, L16b, kld, s));
        }
        return SLT_OK;
    };
    int dev = 0, sms = 0;
    SLT_CUDA_TRY(cudaGetDevice(&dev));
    SLT_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int64_t nblk = (n + S - 1) / S;
    if (panel_sms <= 0 || panel_sms >= sms || nblk <= 2) {
        for (int64_t s0 = 0; s0 < n; s0 += S) {
            const int64_t s1 = std::min(n, s0 + S);
            if (prologue) TRY(prologue(s0, s1, s));
            if (s0 > 0)
                TRY(slt_tc_gemm_packed(tier, n - s0, s1 - s0, s0, rows16(s0, 0), kld, rows16(s0, 0), kld,
                                       A + s0 + s0 * lda, lda, 1, s));
            TRY(panels(s0, s1));
        }
        return SLT_OK;
    }
    // Overlap: block b's update splits into the part from blocks 0 .. b-2
    // (k = (b-1) S, "big") and the part from block b-1 (k = S, "small").
    // The big part of block b+1 needs nothing of block b, so it runs on a
    // second, lower-priority stream on sms - panel_sms SMs while block b's
    // panels run on panel_sms SMs; the small part follows on the caller's
    // stream once block b-1 is packed.  Events order the two streams:
    //   cast + big(b+1)      after  pack(b-1)         (ev_issue)
    //   small(b+1), panels   after  cast + big(b+1)   (ev_big)
    int lo = 0, hi = 0;
    SLT_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    struct Res {
        cudaStream_t su = nullptr;
        cudaEvent_t ev_issue = nullptr, ev_big = nullptr;
        ~Res() {
            if (su) cudaStreamDestroy(su);
            if (ev_issue) cudaEventDestroy(ev_issue);
            if (ev_big) cudaEventDestroy(ev_big);
        }
    } r;
    SLT_CUDA_TRY(cudaStreamCreateWithPriority(&r.su, cudaStreamNonBlocking, lo));
    SLT_CUDA_TRY(cudaEventCreateWithFlags(&r.ev_issue, cudaEventDisableTiming));
    SLT_CUDA_TRY(cudaEventCreateWithFlags(&r.ev_big, cudaEventDisableTiming));
    int rc = SLT_OK;
    bool big_pending = false;
    if (prologue) rc = prologue(0, std::min(n, S), s);
    for (int64_t b = 0; b < nblk && !rc; ++b) {
        const int64_t s0 = b * S, s1 = std::min(n, s0 + S);
        if (b >= 1) {
            if ((rc = slt_from_cuda(cudaStreamWaitEvent(s, r.ev_big, 0)))) break;
            big_pending = false;
            // small part: block b-1's columns (k from s0 - S to s0)
            if ((rc = slt_tc_gemm_packed(tier, n - s0, s1 - s0, S, rows16(s0, s0 - S), kld, rows16(s0, s0 - S), kld,
                                         A + s0 + s0 * lda, lda, 1, s)))
                break;
        }
        const bool side = b + 1 < nblk;
        if (side) {
            const int64_t t0 = s1, t1 = std::min(n, t0 + S);
            if ((rc = slt_from_cuda(cudaEventRecord(r.ev_issue, s)))) break;
            if ((rc = slt_from_cuda(cudaStreamWaitEvent(r.su, r.ev_issue, 0)))) break;
            if (prologue && (rc = prologue(t0, t1, r.su))) break;
            if (b >= 1) {
                SmCap cap(sms - panel_sms);
                if ((rc = slt_tc_gemm_packed(tier, n - t0, t1 - t0, s0, rows16(t0, 0), kld, rows16(t0, 0), kld,
                                             A + t0 + t0 * lda, lda, 1, r.su)))
                    break;
            }
            if ((rc = slt_from_cuda(cudaEventRecord(r.ev_big, r.su)))) break;
            big_pending = true;
        }
        {
            SmCap cap(side && b >= 1 ? panel_sms : 0);
            rc = panels(s0, s1);
        }
    }
    // nothing of the side stream may outlive the call
    if (big_pending) {
        const int jr = slt_from_cuda(cudaStreamWaitEvent(s, r.ev_big, 0));
        if (!rc) rc = jr;
    }
    return rc;
}

// SMs of the left-looking factor's panels while the next block's big
// update runs beside them: SLT_LL_PANEL_SMS when set (0: no overlap).
static int potrf_ll_panel_sms(int64_t n)
{
    (void) n;
    if (const char* e = std::getenv("SLT_LL_PANEL_SMS")) return std::atoi(e);
    return 0;
}

// The left-looking form applies to FP16 / BF16 factors when the size
// bucket defers its updates (depth > 1) and nb is a multiple of 64;
// SLT_POTRF_LL=0 turns it off, =1 forces it.  Returns the block width S, or
// 0 for the right-looking driver.
static int64_t potrf_ll_width(int64_t n, const slt_options& o)
{
    const int p = o.factor_precision;
    if (p != SLT_PREC_FP16 && p != SLT_PREC_BF16) return 0;
    const int64_t nb = eff_nb(o);
    if (nb % 64 != 0) return 0;
    const DriverTune& t = driver_tune(1, 2, n);
    int64_t depth = update_depth(t);
    if (const char* e = std::getenv("SLT_POTRF_LL")) {
        if (std::atoi(e) == 0) return 0;
        depth = std::max<int64_t>(depth, 2);
    }
    else if (depth <= 1 || t.panel_sms > 0) {
        return 0;
    }
    return depth * nb;
}

// potrs lower: forward with L, backward with L^T (src/potrs.cc:55-78).
template <typename T>
int potrs_dev(int64_t n, int64_t nrhs, const T* L, int64_t lda, int64_t nb, T* B, int64_t ldb,
              int* d_status, cudaStream_t s)
{
    (void) nb;
    if (n < 0 || nrhs < 0) return SLT_ERR_ARG;
    if (n == 0 || nrhs == 0) return SLT_OK;
    DevBuf flags;
    TRY(flags.alloc(slt_sweep_flags_bytes(n), s));
    for (int64_t c0 = 0; c0 < nrhs; c0 += 16) {
        const int64_t nc = std::min<int64_t>(16, nrhs - c0);
        T* b = B + c0 * ldb;
        TRY(k_sweep(2, n, nc, L, lda, b, ldb, flags.as<int>(), d_status, s));
        TRY(k_sweep(3, n, nc, L, lda, b, ldb, flags.as<int>(), d_status, s));
    }
    return SLT_OK;
}

template int getrf_dev<double>(int64_t, int64_t, double*, int64_t, int*, const slt_options&, FactorCtx&, cudaStream_t);
template int getrf_dev<float>(int64_t, int64_t, float*, int64_t, int*, const slt_options&, FactorCtx&, cudaStream_t);
template int getrs_dev<double>(int64_t, int64_t, const double*, int64_t, const int*, int64_t, double*, int64_t, int*, cudaStream_t);
template int getrs_dev<float>(int64_t, int64_t, const float*, int64_t, const int*, int64_t, float*, int64_t, int*, cudaStream_t);
template int getrs_trans_dev<double>(int64_t, int64_t, const double*, int64_t, const int*, int64_t, double*, int64_t, int*, cudaStream_t);
template int getrs_trans_dev<float>(int64_t, int64_t, const float*, int64_t, const int*, int64_t, float*, int64_t, int*, cudaStream_t);
template int potrf_dev<double>(int64_t, double*, int64_t, const slt_options&, FactorCtx&, cudaStream_t);
template int potrf_dev<float>(int64_t, float*, int64_t, const slt_options&, FactorCtx&, cudaStream_t);
template int potrs_dev<double>(int64_t, int64_t, const double*, int64_t, int64_t, double*, int64_t, int*, cudaStream_t);
template int potrs_dev<float>(int64_t, int64_t, const float*, int64_t, int64_t, float*, int64_t, int*, cudaStream_t);

// ---------------------------------------------------------------------------
// Mixed precision.
namespace {

// Equilibration is on by default only for the 16- and 8-bit tiers, whose
// operand range or mantissa a badly scaled matrix can exceed; FP32 and TF32
// keep SLATE's unscaled cast (src/gesv_mixed.cc:196-199).
bool low_tier(int p) { return p == SLT_PREC_BF16 || p == SLT_PREC_FP16 || p == SLT_PREC_FP8; }

bool equilibrate_on(const slt_options& o)
{
    if (o.equilibrate >= 0) return o.equilibrate != 0;
    return low_tier(o.factor_precision);
}

// The low-precision factorisation the mixed solvers refine with: FP32
// storage of A_s = diag(r) A diag(c) (r = c = 1 without equilibration), the
// O(n^3) update in the tier's arithmetic.  solve() applies
// A^{-1} = diag(c) A_s^{-1} diag(r).
struct LoFactor {
    int chol;
    int64_t n, nb;
    slt_options o;
    DevBuf A;          // float n x n, leading dimension ld (a multiple of 32 so the
                       // tensor-core update can address it with TMA)
    int* ipiv;
    int64_t ld = 0;
    int* status = nullptr;
    DevBuf scales;     // r (n), c (n), row-maximum words (n)
    const double* r = nullptr;
    const double* c = nullptr;
    double sigma = 0.0;  // diagonal shift of a 16-bit Cholesky factor (0: none)

    int factor(const double* Ahi, int64_t lda, FactorCtx& fc, int64_t* info, cudaStream_t s) {
        ld = ((n + 31) / 32) * 32;
        TRY(A.alloc(sizeof(float) * size_t(ld) * size_t(n), s));
        const InputArrival* arr = input_arrival();
        if (arr) TRY(arr->wait_diag(s));
        // only the Cholesky factor below streams its columns in
        if (arr && !(chol && potrf_ll_width(n, o) > 0)) TRY(arr->wait_all(s));
        if (equilibrate_on(o)) {
            TRY(scales.alloc(sizeof(double) * 3 * size_t(n), s));
            double* rr = scales.as<double>();
            if (chol) {
                TRY(slt_dpoequ(n, Ahi, lda, rr, s));
                r = c = rr;
            }
            else {
                TRY(slt_dgeequ(n, n, Ahi, lda, rr, rr + n, rr + 2 * n, s));
                r = rr;
                c = rr + n;
            }
        }
        status = fc.d_status;
        if (!chol) {
            TRY(slt_convert_d2s_scaled(n, n, Ahi, lda, r, c, A.as<float>(), ld, s));
            TRY(getrf_dev<float>(n, n, A.as<float>(), ld, ipiv, o, fc, s));
            return finish_factor(fc, info, s);
        }
        // Cholesky in a 16-bit tier: a matrix with lambda_min below the
        // tier's rounding error breaks down in low precision although it is
        // SPD in FP64.  Factor A_s + sigma I instead, sigma = c u_tier with
        // c = 1, 8, 64 (A_s has diagonal in [0.25, 1) after equilibration),
        // and let the FP64 refinement correct for the shift.
        const bool shift = low_tier(o.factor_precision);
        const double u = o.factor_precision == SLT_PREC_BF16 ? 0x1p-8
                       : o.factor_precision == SLT_PREC_FP8  ? 0x1p-4 : 0x1p-11;
        const int64_t S = potrf_ll_width(n, o);
        for (int attempt = 0;; ++attempt) {
            if (attempt == 0 && S > 0) {
                // left-looking: each block of columns is cast (lower part) just
                // before it is needed, after its columns have arrived
                const double* dr = r;
                float* Af = A.as<float>();
                const int64_t ldf = ld;
                TRY(potrf_ll_tc(n, Af, ld, o, S, fc, s, [&](int64_t s0, int64_t s1, cudaStream_t cs) -> int {
                    if (arr) TRY(arr->wait_cols(s1, cs));
                    return slt_convert_d2s_scaled_lower_cols(n, s0, s1, Ahi, lda, dr, Af, ldf, cs);
                }, potrf_ll_panel_sms(n)));
            }
            else {
                // the factor reads and writes the lower triangle only
                TRY(slt_convert_d2s_scaled_lower(n, Ahi, lda, r, A.as<float>(), ld, s));
                if (attempt > 0) {
                    sigma = u * double(int64_t(1) << (3 * (attempt - 1)));
                    TRY(slt_sshift_diag(n, float(sigma), A.as<float>(), ld, s));
                    SLT_CUDA_TRY(cudaMemsetAsync(fc.d_info, 0, sizeof(int), s));
                }
                if (S > 0) TRY(potrf_ll_tc(n, A.as<float>(), ld, o, S, fc, s, nullptr, potrf_ll_panel_sms(n)));
                else TRY(potrf_dev<float>(n, A.as<float>(), ld, o, fc, s));
            }
            TRY(finish_factor(fc, info, s));
            if (*info == 0 || !shift || attempt == 3) return SLT_OK;
        }
    }
    // X (double) <- A^{-1} R (double), through FP32.  R and X may alias.
    int solve(int64_t nrhs, const double* R, int64_t ldr, double* X, int64_t ldx, float* wlo, cudaStream_t s) {
        TRY(slt_convert_d2s_scaled(n, nrhs, R, ldr, r, nullptr, wlo, n, s));
        if (chol) TRY(potrs_dev<float>(n, nrhs, A.as<float>(), ld, nb, wlo, n, status, s));
        else TRY(getrs_dev<float>(n, nrhs, A.as<float>(), ld, ipiv, nb, wlo, n, status, s));
        return slt_convert_s2d_scaled(n, nrhs, wlo, n, c, X, ldx, s);
    }
};

int read_doubles(const double* d, double* h, int64_t cnt, cudaStream_t s)
{
    SLT_CUDA_TRY(cudaMemcpyAsync(h, d, sizeof(double) * size_t(cnt), cudaMemcpyDeviceToHost, s));
    SLT_CUDA_TRY(cudaStreamSynchronize(s));
    return SLT_OK;
}

bool converged(const double* cr, const double* cx, int64_t k, double cte)
{
    for (int64_t i = 0; i < k; ++i)
        if (!(cr[i] <= cx[i] * cte)) return false;
    return true;
}

// The FP64 products of one refinement solve, R = B - A X for at most 16
// columns per call (SLATE's gemm / hemm in double, src/gesv_mixed.cc:262,
// src/posv_mixed.cc:271): FP64 FMA (slt_dresidual), or FP64-accurate digit
// products on the tensor cores (DigitMatrix, split from A on first use and
// kept for the solve).  engine (Options.residual_engine): 0 auto -- the
// tensor cores for products of >= 4 columns at n >= 2048, where they beat
// the FP64 units even counting the split --, 1 FP64, 2 tensor cores.  When
// the digit planes cannot be allocated the FP64 path runs.
struct Residual {
    int64_t n;
    const double* A;
    int64_t lda;
    int sym;
    int engine;
    DevBuf ws;
    DigitMatrix dm;
    bool dm_failed = false;

    Residual(int64_t n_, const double* A_, int64_t lda_, int sym_, int engine_)
        : n(n_), A(A_), lda(lda_), sym(sym_), engine(engine_) {}

    bool use_digits(int64_t nc) const {
        if (engine == 1 || dm_failed) return false;
        if (engine == 2) return true;
        return nc >= 4 && n >= 2048;
    }

    int compute(int64_t nc, const double* B, int64_t ldb, const double* X, int64_t ldx, double* R, int64_t ldr,
                cudaStream_t s) {
        if (nc <= 0) return SLT_OK;
        if (use_digits(nc)) {
            if (!dm.ready) {
                const int rc = dm.prepare(n, A, lda, sym, s);
                if (rc == SLT_ERR_NOMEM || rc == SLT_ERR_NOT_SUPPORTED) {
                    dm.release();
                    dm_failed = true;
                }
                else if (rc) return rc;
            }
            if (dm.ready) return dm.residual(nc, B, ldb, X, ldx, R, ldr, s);
        }
        if (!ws.p) TRY(ws.alloc(slt_residual_ws_bytes(n, 16), s));
        return slt_dresidual(n, nc, A, lda, sym, B, ldb, X, ldx, R, ldr, ws.p, s);
    }

    // ||A||_inf to d_out: from the digit split's pass over A when the
    // tensor-core products will run (the planes are prepared here, once), else
    // the FP64 norm kernel (ws: slt_norm_ws_bytes(n) bytes).  nc: the columns
    // of the first products.
    int norm_inf(double* d_out, void* nws, int64_t nc, cudaStream_t s) {
        if (use_digits(nc) && !dm.ready) {
            const int rc = dm.prepare(n, A, lda, sym, s, d_out);
            if (rc == SLT_OK) return SLT_OK;
            if (rc != SLT_ERR_NOMEM && rc != SLT_ERR_NOT_SUPPORTED) return rc;
            dm.release();
            dm_failed = true;
        }
        return slt_dnorm_inf(n, n, A, lda, sym, d_out, nws, s);
    }

    // the bounded-wait status of the tensor-core products (synchronises)
    int status(cudaStream_t s) { return dm.ready ? dm.check_status(s) : SLT_OK; }
};

// Right-preconditioned FGMRES(restart) (src/gesv_mixed_gmres.cc:225-395),
// run for up to 16 right-hand sides in lockstep.  Every column is its own
// instance of SLATE's single-right-hand-side iteration -- CGS2 Arnoldi in
// FP64 on the GPU, the low-precision factors as preconditioner, Givens
// rotations and the small triangular solve on the host -- with its own
// restart cycles and stopping test.  What the columns share is the traffic:
// each tick applies the preconditioner to every column that is in an
// Arnoldi step with one sweep pair over the factors, and forms every
// product A w (Arnoldi step) and residual b - A x (start of a restart cycle)
// with one pass over A, instead of one pass per column.  Starts from the x it
// is given.
struct FgmresBlock {
    static constexpr int64_t kMaxCols = 16;
    int chol;
    int64_t n;
    const double* A;
    int64_t lda;
    LoFactor& lo;
    double cte;
    Residual& res;
    int64_t restart = 0, R1 = 1, SC = 0;
    DevBuf nws, scal, V, W, Z, Bg, Rg, Wlo, cgsws;
    std::vector<double> hs;

    struct Col {
        int64_t c = 0;             // column of B and X
        int st = 0;                // 0: start of a restart cycle, 1: Arnoldi step, 2: done
        int64_t iiter = 0, j = 0;
        double cx = 0, ares = 0;
        bool conv = false, stopped = false;
        int citer = 0;
        std::vector<double> H, S, gc, gs, y;
    };

    FgmresBlock(int chol_, int64_t n_, const double* A_, int64_t lda_, LoFactor& lo_, double cte_, Residual& res_)
        : chol(chol_), n(n_), A(A_), lda(lda_), lo(lo_), cte(cte_), res(res_) {}

    int init(int64_t itermax, int64_t nb, cudaStream_t s) {
        restart = std::max<int64_t>(0, std::min<int64_t>(std::min<int64_t>(30, itermax), std::min(nb, n) - 1));
        R1 = restart + 1;
        SC = 4 + 3 * R1;           // per column: cx, cr, ares, nrm | h | z | y
        const size_t nn = size_t(n);
        TRY(nws.alloc(std::max(slt_norm_ws_bytes(n), slt_residual_ws_bytes(n, 1)), s));
        TRY(scal.alloc(sizeof(double) * size_t(SC * kMaxCols), s));
        TRY(V.alloc(sizeof(double) * nn * size_t(R1 * kMaxCols), s));
        TRY(W.alloc(sizeof(double) * nn * size_t(R1 * kMaxCols), s));
        TRY(Z.alloc(sizeof(double) * nn * size_t(kMaxCols), s));
        TRY(Bg.alloc(sizeof(double) * nn * size_t(kMaxCols), s));
        TRY(Rg.alloc(sizeof(double) * nn * size_t(kMaxCols), s));
        hs.assign(size_t(SC * kMaxCols), 0.0);
        TRY(cgsws.alloc(slt_cgs_ws_bytes(R1), s));
        return Wlo.alloc(sizeof(float) * nn * size_t(kMaxCols), s);
    }

    double* Vc(int64_t q) const { return V.as<double>() + size_t(q) * size_t(n) * size_t(R1); }
    double* Wc(int64_t q) const { return W.as<double>() + size_t(q) * size_t(n) * size_t(R1); }
    double* Sc(int64_t q) const { return scal.as<double>() + q * SC; }

    static int copy_col(const double* src, double* dst, int64_t n, cudaStream_t s) {
        SLT_CUDA_TRY(cudaMemcpyAsync(dst, src, sizeof(double) * size_t(n), cudaMemcpyDeviceToDevice, s));
        return SLT_OK;
    }

    // End of a restart cycle: x += W(:, 1:j) H(0:j-1, 0:j-1)^{-1} S(0:j-1).
    int cycle_end(Col& cl, int64_t q, double* X, int64_t ldx, cudaStream_t s) {
        const int64_t j = cl.j;
        if (j > 0) {
            cl.y.assign(cl.S.begin(), cl.S.begin() + j);
            for (int64_t rr = j - 1; rr >= 0; --rr) {
                double sum = cl.y[rr];
                for (int64_t cc = rr + 1; cc < j; ++cc) sum -= cl.H[rr + cc * R1] * cl.y[cc];
                cl.y[rr] = sum / cl.H[rr + rr * R1];
            }
            double* dy = Sc(q) + 4 + 2 * R1;
            SLT_CUDA_TRY(cudaMemcpyAsync(dy, cl.y.data(), sizeof(double) * size_t(j), cudaMemcpyHostToDevice, s));
            TRY(slt_dgemm_skinny(n, 1, j, 1.0, Wc(q) + n, n, 0, dy, R1, 1.0, X + cl.c * ldx, ldx, nws.p, s));
        }
        cl.st = 0;
        return SLT_OK;
    }

    // The loop condition of the Arnoldi steps; false ends the restart cycle.
    bool keep_going(const Col& cl, int64_t itermax) const {
        return cl.j < restart && cl.iiter < itermax && !(cl.ares <= cl.cx * cte);
    }

    // R(:, 0:k) = Bg(:, 0:k) - A Z(:, 0:k), in chunks of 16 columns.
    int products(int64_t k, cudaStream_t s) {
        return res.compute(k, Bg.as<double>(), n, Z.as<double>(), n, Rg.as<double>(), n, s);
    }

    // Runs the columns cols[0..k) (k <= 16) until each one's stopping test
    // holds or it has spent itermax Arnoldi steps.  used[i]: the steps column
    // cols[i] took; conv[i]: whether its test held.  SLATE's loop tests the
    // true residual only at the top of a restart cycle, so a cycle that ends
    // on the budget is never tested; final_check (used by the IR -> GMRES-IR
    // chain, which is not SLATE's driver) tests it once more.
    int run(const int64_t* cols, int64_t k, const double* B, int64_t ldb, double* X, int64_t ldx,
            int64_t itermax, int* used, bool* conv, cudaStream_t s, bool final_check = false) {
        std::vector<Col> cl(k);
        for (int64_t q = 0; q < k; ++q) {
            cl[q].c = cols[q];
            cl[q].H.assign(size_t(R1 * R1), 0.0);
            cl[q].S.assign(R1, 0.0);
            cl[q].gc.assign(R1, 0.0);
            cl[q].gs.assign(R1, 0.0);
        }
        double* z = Z.as<double>();
        double* bg = Bg.as<double>();
        double* rg = Rg.as<double>();
        std::vector<int64_t> arn, st;
        for (;;) {
            arn.clear();
            st.clear();
            for (int64_t q = 0; q < k; ++q) {
                if (cl[q].st == 0 && !(cl[q].iiter < itermax)) cl[q].st = 2;   // budget spent
                if (cl[q].st == 1) arn.push_back(q);
                else if (cl[q].st == 0) st.push_back(q);
            }
            if (arn.empty() && st.empty()) break;
            const int64_t na = int64_t(arn.size()), ns = int64_t(st.size());
            // preconditioner: w = M^{-1} v_j for every column in an Arnoldi step
            for (int64_t i = 0; i < na; ++i) {
                const Col& c = cl[arn[i]];
                TRY(copy_col(Vc(arn[i]) + c.j * n, z + i * n, n, s));
            }
            if (na) {
                TRY(lo.solve(na, z, n, z, n, Wlo.as<float>(), s));
                for (int64_t i = 0; i < na; ++i)
                    TRY(copy_col(z + i * n, Wc(arn[i]) + (cl[arn[i]].j + 1) * n, n, s));
                SLT_CUDA_TRY(cudaMemsetAsync(bg, 0, sizeof(double) * size_t(n) * size_t(na), s));
            }
            // one pass over A: -A w (Arnoldi steps) and b - A x (cycle starts)
            for (int64_t i = 0; i < ns; ++i) {
                const Col& c = cl[st[i]];
                TRY(copy_col(X + c.c * ldx, z + (na + i) * n, n, s));
                TRY(copy_col(B + c.c * ldb, bg + (na + i) * n, n, s));
            }
            TRY(products(na + ns, s));
            if (na) {
                // CGS2 of every Arnoldi column in one set of launches:
                // v_{j+1} = -(A w), orthogonalised twice against v_0 .. v_j
                slt_cgs_cols cc{};
                cc.na = int(na);
                for (int64_t i = 0; i < na; ++i) {
                    cc.q[i] = int(arn[i]);
                    cc.j[i] = int(cl[arn[i]].j);
                }
                TRY(slt_dcgs2(n, V.as<double>(), R1, &cc, rg, scal.as<double>(), SC, cgsws.p, s));
            }
            for (int64_t i = 0; i < ns; ++i) {
                const int64_t q = st[i];
                TRY(copy_col(rg + (na + i) * n, Vc(q), n, s));
                TRY(slt_dcolmax(n, 1, X + cl[q].c * ldx, ldx, Sc(q), s));
                TRY(slt_dcolmax(n, 1, Vc(q), n, Sc(q) + 1, s));
                TRY(slt_dnrm2(n, Vc(q), Sc(q) + 2, s));
            }
            TRY(read_doubles(scal.as<double>(), hs.data(), k * SC, s));
            // host side of every column
            for (int64_t i = 0; i < ns; ++i) {
                const int64_t q = st[i];
                Col& c = cl[q];
                const double* h = hs.data() + q * SC;
                c.cx = h[0];
                const double cr = h[1];
                if (cr <= c.cx * cte) { c.citer = int(c.iiter); c.conv = true; c.stopped = true; c.st = 2; continue; }
                c.ares = h[2];
                if (c.ares == 0) { c.citer = int(c.iiter); c.stopped = true; c.st = 2; continue; }
                TRY(slt_dgeadd(n, 1, 1.0 / c.ares, Vc(q), n, 0.0, Vc(q), n, s));
                c.S.assign(R1, 0.0);
                c.S[0] = c.ares;
                c.j = 0;
                c.st = 1;
                if (!keep_going(c, itermax)) TRY(cycle_end(c, q, X, ldx, s));
            }
            for (int64_t i = 0; i < na; ++i) {
                const int64_t q = arn[i];
                Col& c = cl[q];
                const int64_t j = c.j;
                const double* h = hs.data() + q * SC;
                const double nrm = h[3];
                TRY(slt_dgeadd(n, 1, 1.0 / nrm, Vc(q) + (j + 1) * n, n, 0.0, Vc(q) + (j + 1) * n, n, s));
                double* hj = c.H.data() + j * R1;
                for (int64_t r = 0; r <= j; ++r) hj[r] = h[4 + r] + h[4 + R1 + r];
                hj[j + 1] = nrm;
                auto rot = [](double* xx, double* yy, double cc, double ss) {
                    double tx = cc * *xx + ss * *yy;
                    double ty = cc * *yy - ss * *xx;
                    *xx = tx; *yy = ty;
                };
                for (int64_t r = 0; r < j; ++r) rot(&hj[r], &hj[r + 1], c.gc[r], c.gs[r]);
                {
                    double a = hj[j], bb = hj[j + 1];
                    double roe = std::fabs(a) > std::fabs(bb) ? a : bb;
                    double scale = std::fabs(a) + std::fabs(bb);
                    if (scale == 0) { c.gc[j] = 1; c.gs[j] = 0; }
                    else {
                        double rr = scale * std::sqrt((a / scale) * (a / scale) + (bb / scale) * (bb / scale));
                        rr = std::copysign(1.0, roe) * rr;
                        c.gc[j] = a / rr; c.gs[j] = bb / rr;
                    }
                }
                rot(&hj[j], &hj[j + 1], c.gc[j], c.gs[j]);
                rot(&c.S[j], &c.S[j + 1], c.gc[j], c.gs[j]);
                c.ares = std::fabs(c.S[j + 1]);
                c.j = j + 1;
                c.iiter += 1;
                if (!keep_going(c, itermax)) TRY(cycle_end(c, q, X, ldx, s));
            }
        }
        if (final_check) {
            // columns that ended on the budget: test the true residual once more
            int64_t nf = 0;
            std::vector<int64_t> fq;
            for (int64_t q = 0; q < k; ++q)
                if (!cl[q].stopped) {
                    TRY(copy_col(X + cl[q].c * ldx, z + nf * n, n, s));
                    TRY(copy_col(B + cl[q].c * ldb, bg + nf * n, n, s));
                    fq.push_back(q);
                    ++nf;
                }
            if (nf) {
                TRY(products(nf, s));
                for (int64_t i = 0; i < nf; ++i) {
                    TRY(slt_dcolmax(n, 1, X + cl[fq[i]].c * ldx, ldx, Sc(fq[i]), s));
                    TRY(slt_dcolmax(n, 1, rg + i * n, n, Sc(fq[i]) + 1, s));
                }
                TRY(read_doubles(scal.as<double>(), hs.data(), k * SC, s));
                for (int64_t i = 0; i < nf; ++i) {
                    const double* h = hs.data() + fq[i] * SC;
                    if (h[1] <= h[0] * cte) cl[fq[i]].conv = true;
                }
            }
        }
        for (int64_t q = 0; q < k; ++q) {
            used[q] = cl[q].stopped ? cl[q].citer : int(cl[q].iiter);
            conv[q] = cl[q].conv;
        }
        return SLT_OK;
    }
};

int fallback_fp64(int chol, int64_t n, int64_t nrhs, double* A, int64_t lda, int* ipiv,
                  const double* B, int64_t ldb, double* X, int64_t ldx, const slt_options& o,
                  int64_t* info, TimerSet& tm, const char* pfx, cudaStream_t s)
{
    DevBuf st;
    TRY(st.alloc(2 * sizeof(int), s));
    SLT_CUDA_TRY(cudaMemsetAsync(st.p, 0, 2 * sizeof(int), s));
    FactorCtx fc{st.as<int>(), st.as<int>() + 1};
    slt_options o64 = o;
    o64.factor_precision = SLT_PREC_FP64;
    tm.start(std::string(pfx) + (chol ? "::potrf_hi" : "::getrf_hi"));
    if (chol) TRY(potrf_dev<double>(n, A, lda, o64, fc, s));
    else TRY(getrf_dev<double>(n, n, A, lda, ipiv, o64, fc, s));
    tm.stop(std::string(pfx) + (chol ? "::potrf_hi" : "::getrf_hi"));
    TRY(finish_factor(fc, info, s));
    if (*info == 0) {
        tm.start(std::string(pfx) + (chol ? "::potrs_hi" : "::getrs_hi"));
        TRY(slt_dcopy2d(n, nrhs, B, ldb, X, ldx, s));
        if (chol) TRY(potrs_dev<double>(n, nrhs, A, lda, eff_nb(o), X, ldx, fc.d_status, s));
        else TRY(getrs_dev<double>(n, nrhs, A, lda, ipiv, eff_nb(o), X, ldx, fc.d_status, s));
        tm.stop(std::string(pfx) + (chol ? "::potrs_hi" : "::getrs_hi"));
    }
    return SLT_OK;
}

} // namespace

// gesv_mixed / posv_mixed (src/gesv_mixed.cc:105-289, src/posv_mixed.cc:105-320).
// With o.refine == SLT_REFINE_IR_GMRES the IR loop stops early once a
// column's residual max-norm falls by less than half in one step, and every
// column still unconverged continues with FGMRES-IR from its current x on the
// remaining iteration budget; *iter then counts IR steps plus the largest
// number of Arnoldi steps any column took.
static int gesv_mixed_once(int chol, int64_t n, int64_t nrhs, double* A, int64_t lda, int* ipiv,
                           const double* B, int64_t ldb, double* X, int64_t ldx, const slt_options& o,
                           int* iter, int64_t* info, cudaStream_t s, bool stop_early = false)
{
    if (n < 0 || nrhs < 0 || lda < std::max<int64_t>(1, n)) return SLT_ERR_ARG;
    *iter = 0;
    *info = 0;
    if (n == 0 || nrhs == 0) return SLT_OK;
    const char* pfx = chol ? "posv_mixed" : "gesv_mixed";
    TimerSet tm(s);
    tm.start(pfx);
    const double eps = std::numeric_limits<double>::epsilon();
    const double tol = o.tolerance > 0 ? o.tolerance : eps * std::sqrt(double(n));
    const int64_t itermax = o.max_iterations;
    const int64_t nb = eff_nb(o);
    const bool chain = o.refine == SLT_REFINE_IR_GMRES;

    DevBuf nws, scal, R, Wlo, st, col;
    TRY(nws.alloc(slt_norm_ws_bytes(n), s));
    TRY(scal.alloc(sizeof(double) * 4, s));
    TRY(R.alloc(sizeof(double) * size_t(n) * size_t(nrhs), s));
    TRY(Wlo.alloc(sizeof(float) * size_t(n) * size_t(nrhs), s));
    TRY(st.alloc(2 * sizeof(int), s));
    TRY(col.alloc(sizeof(double) * 2 * size_t(nrhs), s));
    SLT_CUDA_TRY(cudaMemsetAsync(st.p, 0, 2 * sizeof(int), s));
    FactorCtx fc{st.as<int>(), st.as<int>() + 1};

    LoFactor lo{chol, n, nb, o, {}, ipiv};
    if (lo.o.factor_precision == SLT_PREC_FP64) lo.o.factor_precision = SLT_PREC_FP32;
    int64_t linfo = 0;
    tm.start(std::string(pfx) + (chol ? "::potrf_lo" : "::getrf_lo"));
    TRY(lo.factor(A, lda, fc, &linfo, s));
    tm.stop(std::string(pfx) + (chol ? "::potrf_lo" : "::getrf_lo"));

    // ||A||_inf for the stopping test, after the factor (A may still have been
    // arriving from the host while it ran; the factor waited for all of it)
    double Anorm = 0;
    if (const InputArrival* arr = input_arrival()) TRY(arr->wait_all(s));
    Residual res(n, A, lda, chol, o.residual_engine);
    // (no planes when the factor failed: no product will run)
    TRY(res.norm_inf(scal.as<double>(), nws.p, linfo ? 0 : std::min<int64_t>(nrhs, 16), s));
    TRY(read_doubles(scal.as<double>(), &Anorm, 1, s));
    const double cte = Anorm * tol;
    bool conv = false;
    std::vector<double> h(2 * nrhs);
    double* dcx = col.as<double>();
    double* dcr = dcx + nrhs;
    const int64_t rhs_chunks = (nrhs + 15) / 16;
    auto residual = [&]() -> int {
        tm.start(std::string(pfx) + (chol ? "::hemm_hi" : "::gemm_hi"));
        for (int64_t c = 0; c < rhs_chunks; ++c) {
            int64_t c0 = c * 16, nc = std::min<int64_t>(16, nrhs - c0);
            TRY(res.compute(nc, B + c0 * ldb, ldb, X + c0 * ldx, ldx, R.as<double>() + c0 * n, n, s));
        }
        tm.stop(std::string(pfx) + (chol ? "::hemm_hi" : "::gemm_hi"));
        TRY(slt_dcolmax(n, nrhs, X, ldx, dcx, s));
        TRY(slt_dcolmax(n, nrhs, R.as<double>(), n, dcr, s));
        return read_doubles(dcx, h.data(), 2 * nrhs, s);
    };
    int64_t ir_steps = 0;
    bool stalled = false;
    if (linfo != 0) {
        *iter = -3;
    }
    else {
        tm.start(std::string(pfx) + (chol ? "::potrs_lo" : "::getrs_lo"));
        TRY(lo.solve(nrhs, B, ldb, X, ldx, Wlo.as<float>(), s));
        tm.stop(std::string(pfx) + (chol ? "::potrs_lo" : "::getrs_lo"));
        TRY(residual());
        if (converged(h.data() + nrhs, h.data(), nrhs, cte)) { *iter = 0; conv = true; }
        std::vector<double> prev(nrhs);
        for (int64_t it = 0; it < itermax && !conv && !stalled; ++it) {
            std::copy(h.begin() + nrhs, h.end(), prev.begin());
            TRY(lo.solve(nrhs, R.as<double>(), n, R.as<double>(), n, Wlo.as<float>(), s));
            TRY(slt_dgeadd(n, nrhs, 1.0, R.as<double>(), n, 1.0, X, ldx, s));
            TRY(residual());
            ir_steps = it + 1;
            if (converged(h.data() + nrhs, h.data(), nrhs, cte)) { *iter = int(it + 1); conv = true; }
            else if (chain) {
                for (int64_t c = 0; c < nrhs; ++c)
                    if (!(h[nrhs + c] <= h[c] * cte) && !(h[nrhs + c] <= 0.5 * prev[c])) stalled = true;
            }
        }
        if (!conv && chain && itermax - ir_steps > 0) {
            // GMRES-IR on the stalled columns, preconditioned by the same factors
            tm.start(std::string(pfx) + "::gmres");
            FgmresBlock g(chol, n, A, lda, lo, cte, res);
            TRY(g.init(itermax - ir_steps, nb, s));
            std::vector<int64_t> todo;
            for (int64_t c = 0; c < nrhs; ++c)
                if (!(h[nrhs + c] <= h[c] * cte)) todo.push_back(c);
            bool all = true;
            int worst = 0;
            for (size_t g0 = 0; g0 < todo.size(); g0 += FgmresBlock::kMaxCols) {
                const int64_t k = std::min<int64_t>(FgmresBlock::kMaxCols, int64_t(todo.size() - g0));
                int used[FgmresBlock::kMaxCols];
                bool cc[FgmresBlock::kMaxCols];
                TRY(g.run(todo.data() + g0, k, B, ldb, X, ldx, itermax - ir_steps, used, cc, s, true));
                for (int64_t q = 0; q < k; ++q) {
                    all = all && cc[q];
                    worst = std::max(worst, used[q]);
                }
                if (!all && stop_early) break;
            }
            tm.stop(std::string(pfx) + "::gmres");
            if (all) { conv = true; *iter = int(ir_steps + worst); }
        }
    }
    *info = linfo;
    TRY(res.status(s));
    res.dm.release();
    if (!conv) {
        if (linfo == 0) *iter = int(-itermax - 1);
        if (o.use_fallback)
            TRY(fallback_fp64(chol, n, nrhs, A, lda, ipiv, B, ldb, X, ldx, o, info, tm, pfx, s));
    }
    tm.stop(pfx);
    return finish_factor(fc, nullptr, s);   // bounded-wait status of every launch above
}

// gesv_rbt (src/gesv_rbt.cc:100-230): A' = W_U^T A W_V with depth-d random
// butterflies (rbt.cu), LU of A' without pivoting, X = W_V A'^{-1} W_U^T B,
// then FP64 iterative refinement against the original A to SLATE's stopping
// test; not converged after itermax steps -> iter = -(itermax + 1) and, with
// use_fallback, X from partial-pivoting gesv of A.  On return A holds the
// factors of A' (or, after the fallback, A itself, as SLATE restores it).
// The random diagonals come from the Philox stream (seeds 42 and 42 + mt,
// SLATE's rbt_seed and seed + mt).
int gesv_rbt_dev(int64_t n, int64_t nrhs, double* A, int64_t lda, const double* B, int64_t ldb, double* X,
                 int64_t ldx, const slt_options& o, int* iter, int64_t* info, cudaStream_t s)
{
    if (n < 0 || nrhs < 0 || lda < std::max<int64_t>(1, n) || ldb < std::max<int64_t>(1, n) ||
        ldx < std::max<int64_t>(1, n))
        return SLT_ERR_ARG;
    *iter = 0;
    *info = 0;
    if (n == 0 || nrhs == 0) return SLT_OK;
    TimerSet tm(s);
    tm.start("gesv_rbt");
    const double eps = std::numeric_limits<double>::epsilon();
    const double tol = o.tolerance > 0 ? o.tolerance : eps * std::sqrt(double(n));
    const int64_t itermax = o.max_iterations;
    const int64_t nb = eff_nb(o);
    const int64_t d = o.depth >= 0 ? o.depth : 2;
    const int64_t mt = (n + nb - 1) / nb;

    DevBuf uv, Acp, R, nws, scal, col, st, piv;
    TRY(uv.alloc(sizeof(double) * 2 * size_t(n), s));
    double* u = uv.as<double>();
    double* v = u + n;
    TRY(slt_drbt_diag_device(n, 42, u, s));
    TRY(slt_drbt_diag_device(n, 42 + mt, v, s));
    TRY(st.alloc(2 * sizeof(int), s));
    SLT_CUDA_TRY(cudaMemsetAsync(st.p, 0, 2 * sizeof(int), s));
    FactorCtx fc{st.as<int>(), st.as<int>() + 1};
    TRY(piv.alloc(sizeof(int) * size_t(n), s));

    double cte = 0;
    if (itermax > 0) {
        TRY(Acp.alloc(sizeof(double) * size_t(n) * size_t(n), s));
        TRY(R.alloc(sizeof(double) * size_t(n) * size_t(nrhs), s));
        TRY(nws.alloc(std::max(slt_norm_ws_bytes(n), slt_residual_ws_bytes(n, std::min<int64_t>(nrhs, 16))), s));
        TRY(scal.alloc(sizeof(double) * 4, s));
        TRY(col.alloc(sizeof(double) * 2 * size_t(nrhs), s));
        TRY(slt_dcopy2d(n, n, A, lda, Acp.as<double>(), n, s));
        double Anorm = 0;
        TRY(slt_dnorm_inf(n, n, A, lda, 0, scal.as<double>(), nws.p, s));
        TRY(read_doubles(scal.as<double>(), &Anorm, 1, s));
        cte = Anorm * tol;
    }
    TRY(slt_dcopy2d(n, nrhs, B, ldb, X, ldx, s));

    // factor A' without pivoting (the panel's threshold rule with threshold 0)
    slt_options onp = o;
    onp.pivot_threshold = 0.0;
    onp.factor_precision = SLT_PREC_FP64;
    tm.start("gesv_rbt::gerbt");
    TRY(slt_dgerbt2_device(n, A, lda, u, v, d, nb, s));
    tm.stop("gesv_rbt::gerbt");
    tm.start("gesv_rbt::getrf_nopiv");
    TRY(getrf_dev<double>(n, n, A, lda, piv.as<int>(), onp, fc, s));
    tm.stop("gesv_rbt::getrf_nopiv");
    int64_t finfo = 0;
    TRY(finish_factor(fc, &finfo, s));
    // X = W_V A'^{-1} W_U^T X, one right-hand-side block
    auto rbt_solve = [&](double* Y, int64_t ldy) -> int {
        TRY(slt_dgerbt1_device('T', n, nrhs, Y, ldy, u, d, nb, s));
        TRY(getrs_dev<double>(n, nrhs, A, lda, piv.as<int>(), nb, Y, ldy, fc.d_status, s));
        return slt_dgerbt1_device('N', n, nrhs, Y, ldy, v, d, nb, s);
    };
    bool conv = false;
    if (finfo == 0) {
        tm.start("gesv_rbt::getrs_nopiv");
        TRY(rbt_solve(X, ldx));
        tm.stop("gesv_rbt::getrs_nopiv");
    }
    if (itermax == 0) {
        *info = finfo;
        tm.stop("gesv_rbt");
        return finish_factor(fc, nullptr, s);
    }
    std::vector<double> h(2 * size_t(nrhs));
    double* dcx = col.as<double>();
    double* dcr = dcx + nrhs;
    auto residual = [&]() -> int {
        for (int64_t c0 = 0; c0 < nrhs; c0 += 16) {
            const int64_t nc = std::min<int64_t>(16, nrhs - c0);
            TRY(slt_dresidual(n, nc, Acp.as<double>(), n, 0, B + c0 * ldb, ldb, X + c0 * ldx, ldx,
                              R.as<double>() + c0 * n, n, nws.p, s));
        }
        TRY(slt_dcolmax(n, nrhs, X, ldx, dcx, s));
        TRY(slt_dcolmax(n, nrhs, R.as<double>(), n, dcr, s));
        return read_doubles(dcx, h.data(), 2 * nrhs, s);
    };
    if (finfo == 0) {
        tm.start("gesv_rbt::refine");
        TRY(residual());
        if (converged(h.data() + nrhs, h.data(), nrhs, cte)) { *iter = 0; conv = true; }
        for (int64_t it = 0; it < itermax && !conv; ++it) {
            TRY(rbt_solve(R.as<double>(), n));
            TRY(slt_dgeadd(n, nrhs, 1.0, R.as<double>(), n, 1.0, X, ldx, s));
            TRY(residual());
            if (converged(h.data() + nrhs, h.data(), nrhs, cte)) { *iter = int(it + 1); conv = true; }
        }
        tm.stop("gesv_rbt::refine");
    }
    *info = 0;
    if (!conv) {
        *iter = int(-itermax - 1);
        if (o.use_fallback) {
            // A <- original; X from partial-pivoting gesv of the copy
            TRY(slt_dcopy2d(n, n, Acp.as<double>(), n, A, lda, s));
            slt_options o64 = o;
            o64.factor_precision = SLT_PREC_FP64;
            TRY(fallback_fp64(0, n, nrhs, Acp.as<double>(), n, piv.as<int>(), B, ldb, X, ldx, o64, info, tm,
                              "gesv_rbt", s));
        }
        else {
            *info = finfo;
        }
    }
    tm.stop("gesv_rbt");
    return finish_factor(fc, nullptr, s);
}

// gesv_mixed_gmres / posv_mixed_gmres (src/gesv_mixed_gmres.cc:110-410,
// src/posv_mixed_gmres.cc:109-436): FGMRES(restart) preconditioned by the
// low-precision factors, CGS2 Arnoldi in FP64, Givens rotations on the
// host.  Each right-hand side is an independent instance sharing the
// factorisation.
static int gesv_mixed_gmres_once(int chol, int64_t n, int64_t nrhs, double* A, int64_t lda, int* ipiv,
                                 const double* B, int64_t ldb, double* X, int64_t ldx,
                                 const slt_options& o, int* iter, int64_t* info, cudaStream_t s,
                                 bool stop_early = false)
{
    if (n < 0 || nrhs < 0 || lda < std::max<int64_t>(1, n)) return SLT_ERR_ARG;
    *iter = 0;
    *info = 0;
    if (n == 0 || nrhs == 0) return SLT_OK;
    const char* pfx = chol ? "posv_mixed_gmres" : "gesv_mixed_gmres";
    TimerSet tm(s);
    tm.start(pfx);
    const double eps = std::numeric_limits<double>::epsilon();
    const double tol = o.tolerance > 0 ? o.tolerance : eps * std::sqrt(double(n));
    const int64_t itermax = o.max_iterations;
    const int64_t nb = eff_nb(o);

    DevBuf nws, scal, st, Wlo;
    TRY(nws.alloc(slt_norm_ws_bytes(n), s));
    TRY(scal.alloc(sizeof(double) * 4, s));
    TRY(st.alloc(2 * sizeof(int), s));
    TRY(Wlo.alloc(sizeof(float) * size_t(n) * size_t(nrhs), s));
    SLT_CUDA_TRY(cudaMemsetAsync(st.p, 0, 2 * sizeof(int), s));
    FactorCtx fc{st.as<int>(), st.as<int>() + 1};

    LoFactor lo{chol, n, nb, o, {}, ipiv};
    if (lo.o.factor_precision == SLT_PREC_FP64) lo.o.factor_precision = SLT_PREC_FP32;
    int64_t linfo = 0;
    tm.start(std::string(pfx) + (chol ? "::potrf_lo" : "::getrf_lo"));
    TRY(lo.factor(A, lda, fc, &linfo, s));
    tm.stop(std::string(pfx) + (chol ? "::potrf_lo" : "::getrf_lo"));

    // ||A||_inf for the stopping test, after the factor (A may still have been
    // arriving from the host while it ran; the factor waited for all of it)
    double Anorm = 0;
    if (const InputArrival* arr = input_arrival()) TRY(arr->wait_all(s));
    Residual res(n, A, lda, chol, o.residual_engine);
    // (no planes when the factor failed: no product will run)
    TRY(res.norm_inf(scal.as<double>(), nws.p, linfo ? 0 : std::min<int64_t>(nrhs, 16), s));
    TRY(read_doubles(scal.as<double>(), &Anorm, 1, s));
    const double cte = Anorm * tol;
    *info = linfo;
    bool all_conv = true;
    int worst_iter = 0;
    if (linfo != 0) {
        *iter = -3;
        all_conv = false;
    }
    else {
        FgmresBlock g(chol, n, A, lda, lo, cte, res);
        TRY(g.init(itermax, nb, s));
        tm.start(std::string(pfx) + (chol ? "::potrs_lo" : "::getrs_lo"));
        TRY(lo.solve(nrhs, B, ldb, X, ldx, Wlo.as<float>(), s));
        tm.stop(std::string(pfx) + (chol ? "::potrs_lo" : "::getrs_lo"));
        std::vector<int64_t> cols(nrhs);
        for (int64_t c = 0; c < nrhs; ++c) cols[c] = c;
        bool stop = false;
        for (int64_t g0 = 0; g0 < nrhs && !stop; g0 += FgmresBlock::kMaxCols) {
            const int64_t k = std::min<int64_t>(FgmresBlock::kMaxCols, nrhs - g0);
            int used[FgmresBlock::kMaxCols];
            bool cc[FgmresBlock::kMaxCols];
            TRY(g.run(cols.data() + g0, k, B, ldb, X, ldx, itermax, used, cc, s));
            for (int64_t q = 0; q < k; ++q) {
                const int64_t c = g0 + q;
                int citer = used[q];
                if (!cc[q]) { all_conv = false; citer = int(-itermax - 1); }
                // a first attempt that the FP32 retry will redo: one failed column decides it
                if (!cc[q] && stop_early) { worst_iter = citer; stop = true; break; }
                worst_iter = (c == 0) ? citer : (citer < 0 || worst_iter < 0 ? std::min(worst_iter, citer)
                                                                            : std::max(worst_iter, citer));
            }
        }
        *iter = worst_iter;
    }
    TRY(res.status(s));
    res.dm.release();
    if (!all_conv) {
        if (linfo == 0 && *iter >= 0) *iter = int(-itermax - 1);
        if (o.use_fallback)
            TRY(fallback_fp64(chol, n, nrhs, A, lda, ipiv, B, ldb, X, ldx, o, info, tm, pfx, s));
    }
    tm.stop(pfx);
    return finish_factor(fc, nullptr, s);   // bounded-wait status of every launch above
}

// A 16- or 8-bit factorisation that breaks down (info > 0 even after the diagonal
// shifts) or whose refinement does not converge is retried once with an
// FP32 factorisation before SLATE's FP64 fallback: the retry costs one FP32
// factorisation, the FP64 fallback an FP64 one, an order of magnitude more
// on this part.  A is unchanged between the two attempts (the first runs
// without the fallback).  o.lo_retry: -1 auto (on for BF16 / FP16 / FP8), 0, 1.
static bool ladder_on(const slt_options& o)
{
    const bool low = low_tier(o.factor_precision) || o.factor_precision == SLT_PREC_TF32;
    return low && (o.lo_retry < 0 ? (o.factor_precision != SLT_PREC_TF32) : o.lo_retry != 0);
}

template <typename F>
static int with_ladder(F once, const slt_options& o, const char* key, int* iter, int64_t* info)
{
    if (!ladder_on(o)) return once(o, false);
    slt_options o1 = o;
    o1.use_fallback = 0;
    TRY(once(o1, true));
    if (*iter >= 0) return SLT_OK;
    slt_options o2 = o;
    o2.factor_precision = SLT_PREC_FP32;
    const int rc = once(o2, false);
    t_timers[key] = 1.0;          // marks that the FP32 retry ran
    (void) info;
    return rc;
}

int gesv_mixed_dev(int chol, int64_t n, int64_t nrhs, double* A, int64_t lda, int* ipiv,
                   const double* B, int64_t ldb, double* X, int64_t ldx, const slt_options& o,
                   int* iter, int64_t* info, cudaStream_t s)
{
    t_timers.erase(chol ? "posv_mixed::retry_fp32" : "gesv_mixed::retry_fp32");
    return with_ladder([&](const slt_options& oo, bool first) {
        return gesv_mixed_once(chol, n, nrhs, A, lda, ipiv, B, ldb, X, ldx, oo, iter, info, s, first);
    }, o, chol ? "posv_mixed::retry_fp32" : "gesv_mixed::retry_fp32", iter, info);
}

int gesv_mixed_gmres_dev(int chol, int64_t n, int64_t nrhs, double* A, int64_t lda, int* ipiv,
                         const double* B, int64_t ldb, double* X, int64_t ldx,
                         const slt_options& o, int* iter, int64_t* info, cudaStream_t s)
{
    t_timers.erase(chol ? "posv_mixed_gmres::retry_fp32" : "gesv_mixed_gmres::retry_fp32");
    return with_ladder([&](const slt_options& oo, bool first) {
        return gesv_mixed_gmres_once(chol, n, nrhs, A, lda, ipiv, B, ldb, X, ldx, oo, iter, info, s, first);
    }, o, chol ? "posv_mixed_gmres::retry_fp32" : "gesv_mixed_gmres::retry_fp32", iter, info);
}

} // namespace slt
