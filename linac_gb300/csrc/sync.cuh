// Bounded device-side synchronisation helpers.
//
// Every spin-wait in this library has a time limit: when it runs out the
// waiting CTA records LNC_ERR_TIMEOUT in the call's error word and in the
// module's status word, stops waiting and returns, so that the host sees an
// error status instead of a hung GPU.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace lnc {

// ~2 s at the GB300 maximum SM clock (2.07 GHz); an ordinary barrier wait is
// a few microseconds.
constexpr long long kSpinLimitCycles = 4000000000ll;

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ int ld_volatile_i32(const int* p) {
    return *(const volatile int*)p;
}

__device__ __forceinline__ unsigned atom_add_release_u32(unsigned* p, unsigned v) {
    unsigned old;
    asm volatile("atom.add.release.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

struct GridBarrier {
    unsigned* count;   // arrival word: bit 31 flips once per completed barrier (starts at 0)
    unsigned* gen;     // unused (kept for the layout of the callers' scratch)
    int* err;          // call-wide error word (0 = ok)
    int* status;       // module status word read by lnc_device_status()
};

// Grid-wide barrier for a cooperative launch (all CTAs co-resident).  One
// atomic per CTA: CTA 0 adds 2^31 - (G - 1), every other CTA adds 1, so the
// word's low bits return to 0 and bit 31 flips exactly when the last CTA
// arrives; each CTA polls for the flip of the bit it saw.  Returns false
// (uniformly within the CTA) when the wait timed out or another CTA reported
// an error; the caller must then return.
__device__ __forceinline__ bool grid_sync(const GridBarrier& b) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        const unsigned nblocks = gridDim.x * gridDim.y * gridDim.z;
        const bool first = (blockIdx.x | blockIdx.y | blockIdx.z) == 0;
        __threadfence();  // the CTA's writes (ordered before thread 0 by __syncthreads) precede the arrival
        const unsigned old = atom_add_release_u32(b.count, first ? (0x80000000u - (nblocks - 1)) : 1u);
        const long long t0 = clock64();
        unsigned spins = 0;
        while (((old ^ ld_acquire_u32(b.count)) & 0x80000000u) == 0) {
            if ((++spins & 63u) == 0) {
                if (ld_volatile_i32(b.err) != 0) { ok = 0; break; }
                if (clock64() - t0 > kSpinLimitCycles) {
                    atomicExch(b.err, -5);
                    atomicExch(b.status, -5);
                    ok = 0;
                    break;
                }
            }
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

}  // namespace lnc
