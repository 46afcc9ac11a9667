// Batches of uneven RREFs solved concurrently: float64 / complex128 matrices,
// and 64-bit residues (a prime per matrix, up to 2^64 - 59).
//
// linac's callers reduce one matrix per cuda_row_reduce call
// (linac/pycuda_row_reduce.py:18-151).  The float path is latency-bound per
// matrix: the exhaustive panel waits on one grid barrier per column, and the
// mixed-precision refinement reads its convergence statistics back to the
// host once per iteration.  The 64-bit F_p path of a matrix of a few thousand
// columns is bound by its candidate panels (one 8-CTA cluster each) and
// fills only part of the GPU.  Here a pool of host worker threads, each with
// its own non-blocking stream, takes the batch's matrices from a shared
// counter and solves them with the single-matrix path, so that one solve's
// barriers, panels and host round trips overlap the other solves' kernels on
// the GPU.  Each worker copies its matrix into a stream-ordered work buffer
// (the batch's inputs are not modified), solves into the caller's output and
// records the solve's mixed-precision report (float batches).
#include <algorithm>
#include <atomic>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"
#include "rref_internal.cuh"

namespace lnc {

double mixed_error_estimate();

namespace {

struct FloatBatchShared {
    int device = 0;
    int dtype = 0;
    double tol = 1e-9;
    int flags = 0;
    const lnc_batch_matrix* mats = nullptr;
    lnc_mixed_result* reports = nullptr;
    int64_t count = 0;
    std::atomic<int64_t> next{0};
    std::atomic<bool> failed{false};
    std::mutex mu;
    int status = LNC_OK;
    std::string message;
};

void record_failure(FloatBatchShared* S, int rc, int64_t i) {
    std::lock_guard<std::mutex> g(S->mu);
    if (S->status == LNC_OK) {
        S->status = rc;
        S->message = "batch, matrix " + std::to_string((long long)i) + ": " + lnc_last_error();
    }
    S->failed.store(true);
}

void worker(FloatBatchShared* S) {
    cudaSetDevice(S->device);
    cudaStream_t s = nullptr;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        set_error("batch: stream creation failed");
        record_failure(S, LNC_ERR_CUDA, -1);
        return;
    }
    const size_t elt = dtype_size(S->dtype);
    for (;;) {
        if (S->failed.load()) break;
        const int64_t i = S->next.fetch_add(1);
        if (i >= S->count) break;
        const lnc_batch_matrix& M = S->mats[i];
        if (M.m == 0 || M.n == 0) {
            if (M.dev_rank) cudaMemsetAsync(M.dev_rank, 0, sizeof(int64_t), s);
            if (S->reports) S->reports[i] = lnc_mixed_result{0, 0, 0.0};
            continue;
        }
        void* work = nullptr;
        cudaError_t e = cudaMallocAsync(&work, elt * (size_t)M.m * (size_t)M.n, s);
        if (e != cudaSuccess) {
            cudaGetLastError();
            set_error("batch: work buffer of a %lld x %lld matrix: %s", (long long)M.m, (long long)M.n,
                      cudaGetErrorString(e));
            record_failure(S, LNC_ERR_OOM, i);
            break;
        }
        int rc = LNC_OK;
        e = cudaMemcpy2DAsync(work, elt * M.n, M.dev_in, elt * M.ld_in, elt * M.n, M.m, cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) rc = cuda_status(e, "batch: input copy");
        const uint64_t p = (S->dtype == LNC_U32 || S->dtype == LNC_U64) ? M.p : 0;
        if (!rc)
            rc = rref_device_dispatch(S->dtype, M.m, M.n, p, S->tol, work, M.n, M.dev_out, M.ld_out,
                                      M.dev_pivot_cols, M.dev_rank, s, S->flags);
        cudaFreeAsync(work, s);
        if (rc) {
            record_failure(S, rc, i);
            break;
        }
        if (S->reports) {
            lnc_mixed_result r{0, 0, 0.0};
            if (S->flags & LNC_FLAG_MIXED) {
                double corr = 0.0;
                mixed_report(&r.iterations, &corr, &r.redone_fp64);
                r.error_estimate = mixed_error_estimate();
            }
            S->reports[i] = r;
        }
    }
    if (cudaStreamSynchronize(s) != cudaSuccess) {
        cudaGetLastError();
        set_error("batch: stream synchronisation failed");
        record_failure(S, LNC_ERR_CUDA, -1);
    }
    cudaStreamDestroy(s);
}

}  // namespace
}  // namespace lnc

namespace lnc {

// Validate, then solve every matrix of the batch on `workers` concurrent
// streams (synchronous).  F_p batches (LNC_U32 / LNC_U64) take each matrix's
// prime from its descriptor.
int concurrent_batch(int dtype, const lnc_batch_matrix* mats, int64_t count, double tol, int flags, int workers,
                     lnc_mixed_result* reports) {
    const bool modp = dtype == LNC_U32 || dtype == LNC_U64;
    if (count < 0 || (count > 0 && !mats)) { set_error("batch: null matrix list"); return LNC_ERR_INVALID; }
    for (int64_t i = 0; i < count; ++i) {
        const lnc_batch_matrix& M = mats[i];
        int rc = validate_rref_args(dtype, M.m, M.n, modp ? M.p : 0, M.ld_in);
        if (!rc && M.ld_out < M.n) { set_error("output leading dimension < n"); rc = LNC_ERR_INVALID; }
        if (!rc && M.m > 0 && M.n > 0 && (!M.dev_in || !M.dev_out)) { set_error("null buffer"); rc = LNC_ERR_INVALID; }
        if (rc) {
            set_error("batch, matrix %lld: %s", (long long)i, lnc_last_error());
            return rc;
        }
    }
    if (count == 0) return LNC_OK;
    FloatBatchShared S;
    if (cudaGetDevice(&S.device) != cudaSuccess) { cudaGetLastError(); set_error("no CUDA device"); return LNC_ERR_NO_DEVICE; }
    S.dtype = dtype;
    S.tol = tol > 0 ? tol : 1e-9;
    S.flags = flags & ~LNC_FLAG_DEFER_FALLBACK;
    S.mats = mats;
    S.reports = reports;
    S.count = count;
    const int W = (int)std::max<int64_t>(1, std::min<int64_t>(workers > 0 ? workers : 16, count));
    std::vector<std::thread> pool;
    pool.reserve((size_t)W);
    for (int w = 0; w < W; ++w) pool.emplace_back(worker, &S);
    for (auto& t : pool) t.join();
    if (S.status != LNC_OK) {
        set_error("%s", S.message.c_str());
        return S.status;
    }
    return LNC_OK;
}

}  // namespace lnc

using namespace lnc;

extern "C" int lnc_rref_float_batch(int dtype, const lnc_batch_matrix* mats, int64_t count, double tol, int flags,
                                    int workers, lnc_mixed_result* reports) {
    if (dtype != LNC_F64 && dtype != LNC_C128) {
        set_error("float batch: dtype must be LNC_F64 or LNC_C128");
        return LNC_ERR_INVALID;
    }
    return concurrent_batch(dtype, mats, count, tol, flags, workers, reports);
}
