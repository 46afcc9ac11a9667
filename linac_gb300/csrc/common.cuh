// Shared definitions for the linac_gb300 CUDA library (sm_103a).
#pragma once

#include <cstdint>
#include <cstddef>
#include <cuda_runtime.h>

#include "linac_gb300.h"

namespace lnc {

// ---------------------------------------------------------------------------
// error plumbing: every entry point returns an LNC_* status and leaves a
// message retrievable through lnc_last_error().
// ---------------------------------------------------------------------------
void set_error(const char* fmt, ...);
int cuda_status(cudaError_t e, const char* what);

#define LNC_CUDA(call)                                                        \
    do {                                                                      \
        cudaError_t _e = (call);                                              \
        if (_e != cudaSuccess) return ::lnc::cuda_status(_e, #call);          \
    } while (0)

#define LNC_CHECK_LAUNCH(name)                                                \
    do {                                                                      \
        cudaError_t _e = cudaGetLastError();                                  \
        if (_e != cudaSuccess) return ::lnc::cuda_status(_e, name);           \
        ::lnc::count_launch();                                                \
    } while (0)

void count_launch();

// Kernel classes whose launches can be timed with CUDA events (see
// lnc_kernel_timing_*); the dominant kernel of each path has its own class.
enum KernelClass : int {
    KC_PANEL = 0,
    KC_TRAILING = 1,
    KC_LOADER = 2,
    KC_GATHER = 3,
    KC_BATCH = 4,
    KC_COUNT = 5
};

// Records CUDA events around one launch of a kernel class (when timing is
// enabled) together with the launch's algorithmic work (units chosen per
// class: field multiply-adds for the trailing update, bytes for the others).
struct ScopedKernelTimer {
    ScopedKernelTimer(int kclass, cudaStream_t s, double work = 0.0);
    ~ScopedKernelTimer();
    int kclass;
    cudaStream_t stream;
    double work;
    cudaEvent_t start = nullptr, stop = nullptr;
};

// Per-device properties cached at first use.
struct DeviceInfo {
    int device = -1;
    int sms = 0;
    int smem_optin = 0;      // max dynamic shared memory per block (bytes)
    int cc_major = 0, cc_minor = 0;
    bool coop = false;
};
int device_info(DeviceInfo* out);

// Raise a kernel's dynamic shared-memory limit to everything the device allows
// beside its static shared memory (once per kernel and device), and check that
// `need` bytes fit.  The limit is a property of the kernel, shared by all host
// threads: setting it to each launch's own size would let a concurrent launch
// with a larger size on another thread fail.
int allow_dynamic_smem(const void* kernel, size_t need);

size_t dtype_size(int dtype);
bool is_prime_u64(uint64_t n);
int validate_rref_args(int dtype, int64_t m, int64_t n, uint64_t p, int64_t ld);
// LNC_ERR_INVALID (with a message) when a host index list refers past the
// end of a bases row.
int check_loader_indices(const uint32_t* host_lindices, int64_t n_cols, int64_t degree, int64_t basis_len);

constexpr int kMaxPanel = 128;           // widest panel (columns)
constexpr int kPanelThreads = 256;

}  // namespace lnc
