// C ABI of liblinac_gb300 (declared in include/linac_gb300.h) and the shared
// host-side helpers: error messages, launch counting, kernel timing, device
// properties and the per-thread library stream.
#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <unistd.h>
#include <vector>

#include "common.cuh"
#include "rref_internal.cuh"

namespace lnc {

static thread_local std::string t_last_error;
static std::atomic<int64_t> g_launches{0};

void set_error(const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    t_last_error = buf;
}

int cuda_status(cudaError_t e, const char* what) {
    set_error("%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
    if (e == cudaErrorMemoryAllocation) return LNC_ERR_OOM;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return LNC_ERR_NO_DEVICE;
    return LNC_ERR_CUDA;
}

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

// ---- kernel timing ---------------------------------------------------------
static std::mutex g_timing_mu;
static bool g_timing_enabled = false;
struct PendingTiming {
    cudaEvent_t start, stop;
    double work;
};
static std::vector<PendingTiming> g_timing_pending[KC_COUNT];
static double g_timing_work[KC_COUNT];
static std::vector<cudaEvent_t> g_event_pool;
static int64_t g_timing_launches[KC_COUNT];
static double g_timing_ms[KC_COUNT];

static cudaEvent_t pool_event() {
    if (!g_event_pool.empty()) {
        cudaEvent_t e = g_event_pool.back();
        g_event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

ScopedKernelTimer::ScopedKernelTimer(int kc, cudaStream_t s, double w) : kclass(kc), stream(s), work(w) {
    std::lock_guard<std::mutex> g(g_timing_mu);
    if (!g_timing_enabled) return;
    start = pool_event();
    stop = pool_event();
    if (start) cudaEventRecord(start, stream);
}

ScopedKernelTimer::~ScopedKernelTimer() {
    if (!start) return;
    std::lock_guard<std::mutex> g(g_timing_mu);
    cudaEventRecord(stop, stream);
    g_timing_pending[kclass].push_back({start, stop, work});
}

static void timing_drain_locked() {
    for (int k = 0; k < KC_COUNT; ++k) {
        for (auto& pr : g_timing_pending[k]) {
            cudaEventSynchronize(pr.stop);
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, pr.start, pr.stop) == cudaSuccess) {
                g_timing_ms[k] += ms;
                g_timing_launches[k] += 1;
                g_timing_work[k] += pr.work;
            }
            g_event_pool.push_back(pr.start);
            g_event_pool.push_back(pr.stop);
        }
        g_timing_pending[k].clear();
    }
}

// ---- device properties -----------------------------------------------------
static std::mutex g_dev_mu;
static DeviceInfo g_dev_cache[64];

int device_info(DeviceInfo* out) {
    int dev = 0;
    LNC_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) { set_error("device index out of range"); return LNC_ERR_INVALID; }
    std::lock_guard<std::mutex> g(g_dev_mu);
    DeviceInfo& d = g_dev_cache[dev];
    if (d.device != dev) {
        cudaDeviceProp prop;
        LNC_CUDA(cudaGetDeviceProperties(&prop, dev));
        d.sms = prop.multiProcessorCount;
        d.smem_optin = (int)prop.sharedMemPerBlockOptin;
        d.cc_major = prop.major;
        d.cc_minor = prop.minor;
        int coop = 0;
        LNC_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
        d.coop = coop != 0;
        // keep freed stream-ordered allocations cached in the pool
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            uint64_t thr = ~0ull;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
        }
        d.device = dev;
    }
    *out = d;
    return LNC_OK;
}

static std::mutex g_smem_mu;
static std::vector<std::pair<const void*, int>> g_smem_done;  // (kernel, device) pairs already raised

int allow_dynamic_smem(const void* kernel, size_t need) {
    DeviceInfo di;
    int rc = device_info(&di);
    if (rc) return rc;
    std::lock_guard<std::mutex> g(g_smem_mu);
    for (const auto& kd : g_smem_done)
        if (kd.first == kernel && kd.second == di.device) {
            return need <= (size_t)di.smem_optin ? LNC_OK
                                                  : (set_error("kernel needs %zu bytes of shared memory", need),
                                                     LNC_ERR_UNSUPPORTED);
        }
    cudaFuncAttributes fa;
    LNC_CUDA(cudaFuncGetAttributes(&fa, kernel));
    const size_t cap = (size_t)di.smem_optin - fa.sharedSizeBytes;
    if (need > cap) {
        set_error("kernel needs %zu bytes of dynamic shared memory; the device allows %zu", need, cap);
        return LNC_ERR_UNSUPPORTED;
    }
    LNC_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cap));
    g_smem_done.emplace_back(kernel, di.device);
    return LNC_OK;
}

// Per-thread library stream (non-blocking), created on first use per device.
static thread_local cudaStream_t t_streams[64] = {nullptr};
static int library_stream(cudaStream_t* s) {
    int dev = 0;
    LNC_CUDA(cudaGetDevice(&dev));
    if (!t_streams[dev]) LNC_CUDA(cudaStreamCreateWithFlags(&t_streams[dev], cudaStreamNonBlocking));
    *s = t_streams[dev];
    return LNC_OK;
}

// ---- first touch of pageable host destinations -----------------------------
// A device-to-host copy into pageable memory that has never been written (a
// fresh numpy or malloc array) maps the destination one page at a time inside
// the copy: measured at about 1 s per GB on a Grace host, ten times the whole
// solve of a 20,000^2 matrix.  HostPrefault writes one zero per page of the
// destination rows from a few host threads while the GPU works; the copy then
// lands in mapped pages.  Pinned / registered memory and small buffers are
// left alone, and so is a destination that overlaps the input [src, src +
// src_bytes) (an in-place call: its pages are mapped, and the input must not
// be overwritten before it is copied).  join() must return before the copy
// into the buffer is queued.
class HostPrefault {
  public:
    HostPrefault(void* base, size_t row_bytes, size_t pitch, int64_t rows, const void* src, size_t src_bytes) {
        const size_t span = rows > 0 ? pitch * (size_t)(rows - 1) + row_bytes : 0;
        if (!base || span < ((size_t)64 << 20)) return;
        const uintptr_t b0 = (uintptr_t)base, s0 = (uintptr_t)src;
        if (src && b0 < s0 + src_bytes && s0 < b0 + span) return;
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, base) != cudaSuccess) {
            cudaGetLastError();
            return;
        }
        if (a.type != cudaMemoryTypeUnregistered) return;
        long pg = sysconf(_SC_PAGESIZE);
        const size_t page = pg > 0 ? (size_t)pg : 4096;
        unsigned hc = std::thread::hardware_concurrency();
        const bool contiguous = pitch == row_bytes || rows == 1;
        const int64_t nt = std::max<int64_t>(
            1, std::min<int64_t>({(int64_t)(hc ? hc / 2 : 4), 8, contiguous ? (int64_t)8 : rows}));
        for (int64_t t = 0; t < nt; ++t) {
            try {
            threads_.emplace_back([=]() {
                volatile unsigned char* b = (volatile unsigned char*)base;
                auto touch = [&](size_t lo, size_t hi) {  // one write per page of [lo, hi)
                    for (size_t x = lo; x < hi; x = (x / page + 1) * page) b[x] = 0;
                };
                if (contiguous) {
                    const size_t chunk = (span + nt - 1) / nt;
                    const size_t lo = chunk * t, hi = std::min(span, lo + chunk);
                    if (lo < hi) touch(lo, hi);
                } else {
                    for (int64_t r = t; r < rows; r += nt) touch(pitch * (size_t)r, pitch * (size_t)r + row_bytes);
                }
            });
            } catch (...) {  // no thread to spare: the pages left are mapped by the copy itself
                break;
            }
        }
    }
    void join() {
        for (auto& th : threads_) th.join();
        threads_.clear();
    }
    ~HostPrefault() { join(); }

  private:
    std::vector<std::thread> threads_;
};

// ---- modulus validation ----------------------------------------------------
static uint64_t mulmod_u64(uint64_t a, uint64_t b, uint64_t m) {
    return (uint64_t)(((unsigned __int128)a * b) % m);
}
static uint64_t powmod_u64(uint64_t a, uint64_t e, uint64_t m) {
    uint64_t r = 1 % m;
    a %= m;
    while (e) {
        if (e & 1) r = mulmod_u64(r, a, m);
        a = mulmod_u64(a, a, m);
        e >>= 1;
    }
    return r;
}
bool is_prime_u64(uint64_t n) {
    if (n < 2) return false;
    static const uint64_t bases[] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
    for (uint64_t q : bases) {
        if (n % q == 0) return n == q;
    }
    uint64_t d = n - 1;
    int s = 0;
    while ((d & 1) == 0) { d >>= 1; ++s; }
    for (uint64_t a : bases) {
        uint64_t x = powmod_u64(a, d, n);
        if (x == 1 || x == n - 1) continue;
        bool comp = true;
        for (int i = 1; i < s; ++i) {
            x = mulmod_u64(x, x, n);
            if (x == n - 1) { comp = false; break; }
        }
        if (comp) return false;
    }
    return true;
}

size_t dtype_size(int dtype) {
    switch (dtype) {
        case LNC_U32: return 4;
        case LNC_U64: return 8;
        case LNC_F64: return 8;
        case LNC_C128: return 16;
        default: return 0;
    }
}

int validate_rref_args(int dtype, int64_t m, int64_t n, uint64_t p, int64_t ld) {
    if (dtype_size(dtype) == 0) { set_error("unknown dtype %d", dtype); return LNC_ERR_INVALID; }
    if (m < 0 || n < 0) { set_error("negative shape (%lld, %lld)", (long long)m, (long long)n); return LNC_ERR_INVALID; }
    if (ld < n) { set_error("leading dimension %lld < n = %lld", (long long)ld, (long long)n); return LNC_ERR_INVALID; }
    if (m > INT32_MAX) { set_error("too many rows (%lld)", (long long)m); return LNC_ERR_UNSUPPORTED; }
    if (dtype == LNC_U32 || dtype == LNC_U64) {
        if (dtype == LNC_U32 && p > 0xFFFFFFFFull) { set_error("p = %llu does not fit 32-bit residues", (unsigned long long)p); return LNC_ERR_INVALID; }
        if (!is_prime_u64(p)) {
            set_error("Inverse mod %llu does not exist in general. Are you sure %llu is prime?",
                      (unsigned long long)p, (unsigned long long)p);
            return LNC_ERR_NOT_PRIME;
        }
    }
    return LNC_OK;
}

int check_loader_indices(const uint32_t* lind, int64_t n_cols, int64_t degree, int64_t basis_len) {
    const int64_t count = n_cols * degree;
    for (int64_t i = 0; i < count; ++i) {
        if ((int64_t)lind[i] >= basis_len) {
            set_error("loader: lindices[%lld, %lld] = %u refers past the end of a bases row (length %lld)",
                      (long long)(i / degree), (long long)(i % degree), lind[i], (long long)basis_len);
            return LNC_ERR_INVALID;
        }
    }
    return LNC_OK;
}

int load_matrix_dispatch(int dtype, int64_t n_rows, int64_t n_cols, int64_t basis_len, int64_t degree,
                         uint64_t p, const void* bases, const uint32_t* lind, void* out, int64_t ldo,
                         cudaStream_t s);

struct BatchPlan;
int batch_plan_create(const lnc_batch_matrix* mats, int64_t count, int tpc, int smax, cudaStream_t s,
                      BatchPlan** out);
int batch_run(BatchPlan* P, cudaStream_t s);
int batch_finish(BatchPlan* P, cudaStream_t s, int64_t* n_redo);
void batch_destroy(BatchPlan* P);
size_t batch_plan_bytes(BatchPlan* P);
struct BatchGroup;
int batch_group_create(BatchPlan* const* plans, int64_t count, BatchGroup** out);
int batch_group_run(BatchGroup* G, cudaStream_t s);
void batch_group_destroy(BatchGroup* G);

}  // namespace lnc

using namespace lnc;

extern "C" {

const char* lnc_version(void) { return "linac_gb300 0.1.0 (sm_103a)"; }

const char* lnc_last_error(void) { return t_last_error.c_str(); }

int lnc_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

int lnc_set_device(int device) {
    LNC_CUDA(cudaSetDevice(device));
    return LNC_OK;
}

int lnc_device_info(int* sms, size_t* free_bytes, size_t* total_bytes) {
    DeviceInfo di;
    int rc = device_info(&di);
    if (rc) return rc;
    if (sms) *sms = di.sms;
    size_t f = 0, t = 0;
    LNC_CUDA(cudaMemGetInfo(&f, &t));
    if (free_bytes) *free_bytes = f;
    if (total_bytes) *total_bytes = t;
    return LNC_OK;
}

int64_t lnc_launch_count(void) { return g_launches.load(); }

int lnc_malloc(void** p, size_t bytes) {
    if (!p) return LNC_ERR_INVALID;
    *p = nullptr;
    if (bytes == 0) return LNC_OK;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
        return LNC_ERR_OOM;
    }
    return LNC_OK;
}
int lnc_free(void* p) { LNC_CUDA(cudaFree(p)); return LNC_OK; }
int lnc_malloc_host(void** p, size_t bytes) {
    if (!p) return LNC_ERR_INVALID;
    *p = nullptr;
    if (bytes == 0) return LNC_OK;
    cudaError_t e = cudaMallocHost(p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("cudaMallocHost(%zu): %s", bytes, cudaGetErrorString(e));
        return LNC_ERR_OOM;
    }
    return LNC_OK;
}
int lnc_free_host(void* p) { LNC_CUDA(cudaFreeHost(p)); return LNC_OK; }
int lnc_memcpy_h2d(void* dst, const void* src, size_t bytes, void* stream) {
    LNC_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, (cudaStream_t)stream));
    return LNC_OK;
}
int lnc_memcpy_d2h(void* dst, const void* src, size_t bytes, void* stream) {
    LNC_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    return LNC_OK;
}
int lnc_memcpy_d2d(void* dst, const void* src, size_t bytes, void* stream) {
    LNC_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
    return LNC_OK;
}
int lnc_memset(void* p, int value, size_t bytes, void* stream) {
    LNC_CUDA(cudaMemsetAsync(p, value, bytes, (cudaStream_t)stream));
    return LNC_OK;
}
int lnc_stream_create(void** s) {
    cudaStream_t st;
    LNC_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    *s = (void*)st;
    return LNC_OK;
}
int lnc_stream_destroy(void* s) { LNC_CUDA(cudaStreamDestroy((cudaStream_t)s)); return LNC_OK; }
int lnc_stream_synchronize(void* s) { LNC_CUDA(cudaStreamSynchronize((cudaStream_t)s)); return LNC_OK; }
int lnc_device_synchronize(void) { LNC_CUDA(cudaDeviceSynchronize()); return LNC_OK; }
int lnc_event_create(void** e) {
    cudaEvent_t ev;
    LNC_CUDA(cudaEventCreate(&ev));
    *e = (void*)ev;
    return LNC_OK;
}
int lnc_event_destroy(void* e) { LNC_CUDA(cudaEventDestroy((cudaEvent_t)e)); return LNC_OK; }
int lnc_event_record(void* e, void* s) { LNC_CUDA(cudaEventRecord((cudaEvent_t)e, (cudaStream_t)s)); return LNC_OK; }
int lnc_stream_wait_event(void* s, void* e) {
    LNC_CUDA(cudaStreamWaitEvent((cudaStream_t)s, (cudaEvent_t)e, 0));
    return LNC_OK;
}
int lnc_event_elapsed_ms(void* a, void* b, float* ms) {
    LNC_CUDA(cudaEventSynchronize((cudaEvent_t)b));
    LNC_CUDA(cudaEventElapsedTime(ms, (cudaEvent_t)a, (cudaEvent_t)b));
    return LNC_OK;
}

int lnc_mixed_report(int* iterations, double* last_correction, int* redone_fp64) {
    return mixed_report(iterations, last_correction, redone_fp64);
}

int lnc_mixed_error_estimate(double* error_estimate) {
    if (!error_estimate) { set_error("null argument"); return LNC_ERR_INVALID; }
    *error_estimate = mixed_error_estimate();
    return LNC_OK;
}

int lnc_device_status(void) {
    LNC_CUDA(cudaDeviceSynchronize());
    int st = 0;
    int rc = rref_read_and_clear_status(&st);
    if (rc) return rc;
    if (st == LNC_ERR_INVALID) {
        set_error("a loader index referred past the end of a bases row (those columns were written as 0)");
        return st;
    }
    if (st != 0) {
        set_error("a bounded device-side wait timed out (status %d)", st);
        return st;
    }
    return LNC_OK;
}

int lnc_kernel_timing_enable(int enable) {
    std::lock_guard<std::mutex> g(g_timing_mu);
    g_timing_enabled = enable != 0;
    return LNC_OK;
}

int lnc_kernel_timing_reset(void) {
    std::lock_guard<std::mutex> g(g_timing_mu);
    timing_drain_locked();
    for (int k = 0; k < KC_COUNT; ++k) { g_timing_ms[k] = 0.0; g_timing_launches[k] = 0; g_timing_work[k] = 0.0; }
    return LNC_OK;
}

int lnc_kernel_timing_read(int kc, int64_t* launches, double* total_ms) {
    if (kc < 0 || kc >= KC_COUNT) { set_error("unknown kernel class %d", kc); return LNC_ERR_INVALID; }
    std::lock_guard<std::mutex> g(g_timing_mu);
    timing_drain_locked();
    if (launches) *launches = g_timing_launches[kc];
    if (total_ms) *total_ms = g_timing_ms[kc];
    return LNC_OK;
}

int lnc_kernel_timing_work(int kc, double* work) {
    if (kc < 0 || kc >= KC_COUNT) { set_error("unknown kernel class %d", kc); return LNC_ERR_INVALID; }
    std::lock_guard<std::mutex> g(g_timing_mu);
    timing_drain_locked();
    if (work) *work = g_timing_work[kc];
    return LNC_OK;
}

int lnc_rref_device(int dtype, int64_t m, int64_t n, uint64_t p, double tol, void* work, int64_t ldw,
                    void* out, int64_t ldo, int64_t* dev_piv, int64_t* dev_rank, void* stream, int flags) {
    int rc = validate_rref_args(dtype, m, n, p, ldw);
    if (rc) return rc;
    if (ldo < n) { set_error("output leading dimension %lld < n", (long long)ldo); return LNC_ERR_INVALID; }
    cudaStream_t s = (cudaStream_t)stream;
    if (m == 0 || n == 0) {
        if (dev_rank) LNC_CUDA(cudaMemsetAsync(dev_rank, 0, sizeof(int64_t), s));
        if (dev_piv && std::min(m, n) > 0) LNC_CUDA(cudaMemsetAsync(dev_piv, 0xff, sizeof(int64_t) * std::min(m, n), s));
        return LNC_OK;
    }
    return rref_device_dispatch(dtype, m, n, p, tol, work, ldw, out, ldo, dev_piv, dev_rank, s, flags);
}

int lnc_rref_host(int dtype, int64_t m, int64_t n, uint64_t p, double tol, const void* host_in,
                  int64_t ld, void* host_out, int64_t ld_out, int64_t* piv, int64_t* rank, int flags) {
    int rc = validate_rref_args(dtype, m, n, p, ld);
    if (rc) return rc;
    if (ld_out < n) { set_error("output leading dimension %lld < n", (long long)ld_out); return LNC_ERR_INVALID; }
    const int64_t kmax = std::min(m, n);
    if (m == 0 || n == 0) {
        if (rank) *rank = 0;
        return LNC_OK;
    }
    cudaStream_t s;
    rc = library_stream(&s);
    if (rc) return rc;
    const size_t elt = dtype_size(dtype);
    const size_t bytes = elt * (size_t)m * (size_t)n;
    void *dwork = nullptr, *dout = nullptr, *dsmall = nullptr;
    cudaError_t e = cudaMallocAsync(&dwork, bytes, s);
    if (e == cudaSuccess) e = cudaMallocAsync(&dout, bytes, s);
    if (e == cudaSuccess) e = cudaMallocAsync(&dsmall, sizeof(int64_t) * (size_t)(kmax + 1), s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        if (dwork) cudaFreeAsync(dwork, s);
        if (dout) cudaFreeAsync(dout, s);
        set_error("device allocation for a %lld x %lld matrix failed: %s", (long long)m, (long long)n,
                  cudaGetErrorString(e));
        return LNC_ERR_OOM;
    }
    int64_t* dpiv = (int64_t*)dsmall;
    int64_t* drank = dpiv + kmax;
    HostPrefault prefault(host_out, elt * n, elt * ld_out, m, host_in, elt * ((size_t)ld * (size_t)(m - 1) + (size_t)n));
    e = cudaMemcpy2DAsync(dwork, elt * n, host_in, elt * ld, elt * n, m, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) rc = cuda_status(e, "host-to-device copy");
    if (!rc) rc = rref_device_dispatch(dtype, m, n, p, tol, dwork, n, dout, n, dpiv, drank, s, flags);
    prefault.join();
    if (!rc) {
        e = cudaMemcpy2DAsync(host_out, elt * ld_out, dout, elt * n, elt * n, m, cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) rc = cuda_status(e, "device-to-host copy");
    }
    std::vector<int64_t> small((size_t)kmax + 1);
    if (!rc) {
        e = cudaMemcpyAsync(small.data(), dsmall, sizeof(int64_t) * (size_t)(kmax + 1), cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) rc = cuda_status(e, "device-to-host copy");
    }
    cudaFreeAsync(dwork, s);
    cudaFreeAsync(dout, s);
    cudaFreeAsync(dsmall, s);
    e = cudaStreamSynchronize(s);
    if (!rc && e != cudaSuccess) rc = cuda_status(e, "rref");
    if (!rc) {
        int st = 0;
        rc = rref_read_and_clear_status(&st);
        if (!rc && st != 0) {
            set_error("a bounded device-side wait timed out during the RREF (status %d)", st);
            rc = st;
        }
    }
    if (!rc) {
        if (piv) memcpy(piv, small.data(), sizeof(int64_t) * (size_t)kmax);
        if (rank) *rank = small[(size_t)kmax];
    }
    return rc;
}

int lnc_load_matrix_device(int dtype, int64_t n_rows, int64_t n_cols, int64_t basis_len, int64_t degree,
                           uint64_t p, const void* bases, const uint32_t* lind, void* out, int64_t ldo,
                           void* stream) {
    if (dtype_size(dtype) == 0) { set_error("unknown dtype %d", dtype); return LNC_ERR_INVALID; }
    if (n_rows < 0 || n_cols < 0 || ldo < n_cols) { set_error("loader: bad shape"); return LNC_ERR_INVALID; }
    return load_matrix_dispatch(dtype, n_rows, n_cols, basis_len, degree, p, bases, lind, out, ldo,
                                (cudaStream_t)stream);
}

int lnc_load_matrix_host(int dtype, int64_t n_rows, int64_t n_cols, int64_t basis_len, int64_t degree,
                         uint64_t p, const void* hbases, const uint32_t* hlind, void* hout) {
    const size_t elt = dtype_size(dtype);
    if (elt == 0) { set_error("unknown dtype %d", dtype); return LNC_ERR_INVALID; }
    if (n_rows < 0 || n_cols < 0 || basis_len < 0 || degree < 0) { set_error("loader: bad shape"); return LNC_ERR_INVALID; }
    if (n_rows == 0 || n_cols == 0) return LNC_OK;
    if (degree < 1 || basis_len < 1) { set_error("loader: degree and basis length must be >= 1"); return LNC_ERR_INVALID; }
    int rc = check_loader_indices(hlind, n_cols, degree, basis_len);
    if (rc) return rc;
    cudaStream_t s;
    rc = library_stream(&s);
    if (rc) return rc;
    const size_t bb = elt * (size_t)n_rows * (size_t)basis_len;
    const size_t lb = sizeof(uint32_t) * (size_t)n_cols * (size_t)degree;
    const size_t ob = elt * (size_t)n_rows * (size_t)n_cols;
    void *db = nullptr, *dl = nullptr, *dout = nullptr;
    cudaError_t e = cudaMallocAsync(&db, bb ? bb : 16, s);
    if (e == cudaSuccess) e = cudaMallocAsync(&dl, lb ? lb : 16, s);
    if (e == cudaSuccess) e = cudaMallocAsync(&dout, ob, s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        if (db) cudaFreeAsync(db, s);
        if (dl) cudaFreeAsync(dl, s);
        set_error("loader: device allocation failed: %s", cudaGetErrorString(e));
        return LNC_ERR_OOM;
    }
    HostPrefault prefault(hout, ob, ob, 1, hbases, bb);
    if (bb) e = cudaMemcpyAsync(db, hbases, bb, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && lb) e = cudaMemcpyAsync(dl, hlind, lb, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) rc = cuda_status(e, "loader host-to-device copy");
    if (!rc) rc = load_matrix_dispatch(dtype, n_rows, n_cols, basis_len, degree, p, db, (const uint32_t*)dl, dout,
                                       n_cols, s);
    prefault.join();
    if (!rc) {
        e = cudaMemcpyAsync(hout, dout, ob, cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) rc = cuda_status(e, "loader device-to-host copy");
    }
    cudaFreeAsync(db, s);
    cudaFreeAsync(dl, s);
    cudaFreeAsync(dout, s);
    e = cudaStreamSynchronize(s);
    if (!rc && e != cudaSuccess) rc = cuda_status(e, "loader");
    return rc;
}

int lnc_batch_plan_create(int dtype, const lnc_batch_matrix* mats, int64_t count, int tiles_per_cta, int cand_rows,
                          void* stream, void** plan) {
    if (dtype != LNC_U32) { set_error("the batched RREF serves 32-bit residues (LNC_U32)"); return LNC_ERR_UNSUPPORTED; }
    if (!mats || !plan) { set_error("null argument"); return LNC_ERR_INVALID; }
    BatchPlan* P = nullptr;
    int rc = batch_plan_create(mats, count, tiles_per_cta, cand_rows, (cudaStream_t)stream, &P);
    *plan = rc ? nullptr : (void*)P;
    return rc;
}

int lnc_batch_plan_run(void* plan, void* stream) {
    if (!plan) { set_error("null plan"); return LNC_ERR_INVALID; }
    return batch_run((BatchPlan*)plan, (cudaStream_t)stream);
}

int lnc_batch_plan_finish(void* plan, void* stream, int64_t* n_redo) {
    if (!plan) { set_error("null plan"); return LNC_ERR_INVALID; }
    return batch_finish((BatchPlan*)plan, (cudaStream_t)stream, n_redo);
}

int64_t lnc_batch_plan_bytes(void* plan) { return (int64_t)batch_plan_bytes((BatchPlan*)plan); }

int lnc_batch_plan_destroy(void* plan) {
    batch_destroy((BatchPlan*)plan);
    return LNC_OK;
}

int lnc_batch_group_create(void* const* plans, int64_t count, void** group) {
    if (!plans || !group) { set_error("null argument"); return LNC_ERR_INVALID; }
    BatchGroup* G = nullptr;
    int rc = batch_group_create((BatchPlan* const*)plans, count, &G);
    *group = rc ? nullptr : (void*)G;
    return rc;
}

int lnc_batch_group_run(void* group, void* stream) {
    if (!group) { set_error("null plan group"); return LNC_ERR_INVALID; }
    return batch_group_run((BatchGroup*)group, (cudaStream_t)stream);
}

int lnc_batch_group_destroy(void* group) {
    batch_group_destroy((BatchGroup*)group);
    return LNC_OK;
}

int lnc_rref_batch_device(int dtype, const lnc_batch_matrix* mats, int64_t count, void* stream, int flags) {
    if (dtype == LNC_U64) {
        // no captured plan for 64-bit residues: the single-matrix path on concurrent worker streams,
        // after the work already queued on `stream` (which may be producing the inputs)
        if (stream) LNC_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
        return concurrent_batch(LNC_U64, mats, count, 0.0, flags & ~(LNC_FLAG_MIXED | LNC_FLAG_NO_SCALING), 0,
                                nullptr);
    }
    void* plan = nullptr;
    int rc = lnc_batch_plan_create(dtype, mats, count, 0, 0, stream, &plan);
    if (rc) return rc;
    rc = lnc_batch_plan_run(plan, stream);
    if (!rc) rc = lnc_batch_plan_finish(plan, stream, nullptr);
    lnc_batch_plan_destroy(plan);
    return rc;
}

}  // extern "C"
