// drivers.h -- C++ host drivers of the LU / Cholesky solve path (internal).
#pragma once

#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

#include "slt_kernels.h"
#include "slate_gb300.h"
#include "status.h"

#include <algorithm>
#include <functional>
#include <map>
#include <string>
#include <vector>

extern "C" {
int slt_dgemm_skinny(int64_t m, int64_t nrhs, int64_t k, double alpha, const double* A, int64_t lda,
                     int sym_lower, const double* X, int64_t ldx, double beta, double* C, int64_t ldc,
                     void* ws, cudaStream_t stream);
int slt_sgemm_skinny(int64_t m, int64_t nrhs, int64_t k, float alpha, const float* A, int64_t lda,
                     const float* X, int64_t ldx, float beta, float* C, int64_t ldc, cudaStream_t stream);
int slt_dgemm_skinny_t(int64_t m, int64_t nrhs, int64_t kk, double alpha, const double* A, int64_t lda,
                       const double* X, int64_t ldx, double beta, double* C, int64_t ldc,
                       cudaStream_t stream);
int slt_sgemm_skinny_t(int64_t m, int64_t nrhs, int64_t kk, float alpha, const float* A, int64_t lda,
                       const float* X, int64_t ldx, float beta, float* C, int64_t ldc,
                       cudaStream_t stream);
int slt_dsweep(int kind, int64_t n, int64_t nrhs, const double* M, int64_t ldm, double* X, int64_t ldx,
               int* flags, int* status, cudaStream_t s);
int slt_ssweep(int kind, int64_t n, int64_t nrhs, const float* M, int64_t ldm, float* X, int64_t ldx,
               int* flags, int* status, cudaStream_t s);
size_t slt_sweep_flags_bytes(int64_t n);
size_t slt_chol_panel_ws_bytes(void);
int slt_dchol_panel(int64_t m, int64_t nbk, double* P, int64_t ld, int* info, int64_t info_offset, void* ws,
                    int* status, cudaStream_t stream);
int slt_schol_panel(int64_t m, int64_t nbk, float* P, int64_t ld, int* info, int64_t info_offset, void* ws,
                    int* status, cudaStream_t stream);
int slt_dnrm2(int64_t n, const double* x, double* out, cudaStream_t stream);
int slt_dscal(int64_t n, const double* num, const double* den, double* x, cudaStream_t stream);
}

namespace slt {

// The library's stream-ordered memory pool on the current device (created on
// first use).  Unlike the device's default pool it keeps freed memory
// reserved between driver calls, so a repeated solve does not map its
// workspace afresh each time; slt_release_workspace() hands it back.
cudaMemPool_t workspace_pool();

// SLT_WORKSPACE_POOL=0: workspace from cudaMalloc / cudaFree instead of the
// stream-ordered pool (slower: every free synchronises the device).  For
// tools that replay kernels and must save and restore the memory they touch.
bool plain_alloc();

// Device workspace owned by one driver call (stream-ordered, from the
// library's pool).
struct DevBuf {
    void* p = nullptr;
    cudaStream_t s = nullptr;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { free_now(); }
    int alloc(size_t bytes, cudaStream_t stream) {
        s = stream;
        if (bytes == 0) bytes = 16;
        cudaError_t e;
        if (plain_alloc()) {
            e = cudaMalloc(&p, bytes);
        }
        else {
            cudaMemPool_t pool = workspace_pool();
            e = pool ? cudaMallocFromPoolAsync(&p, bytes, pool, stream) : cudaMallocAsync(&p, bytes, stream);
        }
        if (e != cudaSuccess) { p = nullptr; cudaGetLastError(); return SLT_ERR_NOMEM; }
        return SLT_OK;
    }
    void free_now() {
        if (!p) return;
        if (plain_alloc()) cudaFree(p);       // synchronises the device
        else cudaFreeAsync(p, s);
        p = nullptr;
    }
    template <typename T> T* as() const { return static_cast<T*>(p); }
    void reset() { free_now(); }
};

// A of order n split once into the byte digit planes of the tensor-core
// residual (digit_residual.cu); residual() then forms R = B - A X for up to
// 16 right-hand sides per call with FP64 accuracy.  The planes take 8 n^2
// bytes (bytes_for); A must not change while they are in use.
struct DigitMatrix {
    int64_t n = 0, ldk = 0, rows_pad = 0;
    int segs = 1, kb_per_seg = 0, sms = 0;
    bool ready = false;
    DevBuf planes, rexp, cexp, xplanes, part, status;
    CUtensorMap mapX;
    DigitMatrix() = default;
    DigitMatrix(const DigitMatrix&) = delete;
    DigitMatrix& operator=(const DigitMatrix&) = delete;
    // d_norm (device, optional): also ||A||_inf, from the same pass over A
    int prepare(int64_t n, const double* A, int64_t lda, int sym_lower, cudaStream_t s, double* d_norm = nullptr);
    int residual(int64_t nrhs, const double* B, int64_t ldb, const double* X, int64_t ldx, double* R,
                 int64_t ldr, cudaStream_t s);
    // SLT_OK, or SLT_ERR_TIMEOUT when a bounded wait of a product ran out
    // (synchronises the stream)
    int check_status(cudaStream_t s);
    void release();
    static size_t bytes_for(int64_t n);
};

// Timers: the slate::timers keys of the reference drivers, measured with CUDA
// events on the driver's stream and resolved when the call ends.
struct TimerSet {
    struct Span { std::string key; cudaEvent_t a, b; };
    std::vector<Span> spans;
    std::map<std::string, cudaEvent_t> open;
    cudaStream_t s;
    explicit TimerSet(cudaStream_t st) : s(st) {}
    void start(const std::string& key) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) { cudaGetLastError(); return; }
        cudaEventRecord(e, s);
        open[key] = e;
    }
    void stop(const std::string& key) {
        auto it = open.find(key);
        if (it == open.end()) return;
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) { cudaGetLastError(); return; }
        cudaEventRecord(e, s);
        spans.push_back({key, it->second, e});
        open.erase(it);
    }
    ~TimerSet();
};


// Columns of A still arriving from the host while a driver runs (set by the
// LAPACK entry points around one call, on the calling thread): the driver's
// stream waits for ev[j / blk] before it reads columns of block j, and for
// ev_diag before it reads the diagonal.  The events are recorded in column
// order on one copy stream.
// The events may be recorded by another host thread: recorded(b) (when
// set) blocks until event b (-1: the diagonal's) has been recorded, so that
// the stream wait below waits for that recording and is not a no-op, and
// returns non-zero if the producer failed.
struct InputArrival {
    cudaEvent_t ev_diag = nullptr;
    const cudaEvent_t* ev = nullptr;
    int64_t nev = 0, blk = 1;
    std::function<int(int64_t)> recorded;
    int wait_diag(cudaStream_t s) const {
        if (!ev_diag) return SLT_OK;
        if (recorded) TRY(recorded(-1));
        return slt_from_cuda(cudaStreamWaitEvent(s, ev_diag, 0));
    }
    // columns [0, j1)
    int wait_cols(int64_t j1, cudaStream_t s) const {
        if (!ev || nev <= 0 || j1 <= 0) return SLT_OK;
        const int64_t b = std::min<int64_t>(nev - 1, (j1 - 1) / blk);
        if (recorded) TRY(recorded(b));
        return slt_from_cuda(cudaStreamWaitEvent(s, ev[b], 0));
    }
    int wait_all(cudaStream_t s) const { return ev && nev > 0 ? wait_cols(nev * blk, s) : SLT_OK; }
};
// The calling thread's arrivals (null: A is complete when the driver starts).
const InputArrival* input_arrival();
// Sets the calling thread's arrivals for its lifetime.
struct InputArrivalScope {
    explicit InputArrivalScope(const InputArrival* a);
    ~InputArrivalScope();
};

struct FactorCtx {
    int* d_info = nullptr;      // first failing column (1-based), 0 = ok
    int* d_status = nullptr;    // SLT_ERR_TIMEOUT from a bounded wait
};

template <typename T>
int getrf_dev(int64_t m, int64_t n, T* A, int64_t lda, int* ipiv, const slt_options& o,
              FactorCtx& fc, cudaStream_t s);
template <typename T>
int getrs_dev(int64_t n, int64_t nrhs, const T* LU, int64_t lda, const int* ipiv, int64_t nb,
              T* B, int64_t ldb, int* d_status, cudaStream_t s);
template <typename T>
int getrs_trans_dev(int64_t n, int64_t nrhs, const T* LU, int64_t lda, const int* ipiv, int64_t nb,
              T* B, int64_t ldb, int* d_status, cudaStream_t s);
template <typename T>
int potrf_dev(int64_t n, T* A, int64_t lda, const slt_options& o, FactorCtx& fc, cudaStream_t s);
template <typename T>
int potrs_dev(int64_t n, int64_t nrhs, const T* L, int64_t lda, int64_t nb, T* B, int64_t ldb,
              int* d_status, cudaStream_t s);

int gesv_mixed_dev(int chol, int64_t n, int64_t nrhs, double* A, int64_t lda, int* ipiv,
                   const double* B, int64_t ldb, double* X, int64_t ldx, const slt_options& o,
                   int* iter, int64_t* info, cudaStream_t s);
int gesv_mixed_gmres_dev(int chol, int64_t n, int64_t nrhs, double* A, int64_t lda, int* ipiv,
                         const double* B, int64_t ldb, double* X, int64_t ldx,
                         const slt_options& o, int* iter, int64_t* info, cudaStream_t s);

int gesv_rbt_dev(int64_t n, int64_t nrhs, double* A, int64_t lda, const double* B, int64_t ldb, double* X,
                 int64_t ldx, const slt_options& o, int* iter, int64_t* info, cudaStream_t s);

// Read the factorisation status words; returns an slt status (timeout wins).
int finish_factor(FactorCtx& fc, int64_t* info, cudaStream_t s);

} // namespace slt
