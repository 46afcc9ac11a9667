// Seeded synthetic residues on the device (benchmark and test inputs): entry
// i of a fill is a SplitMix64 hash of (seed, i) mapped to [0, p) by a
// 64 x 64 -> high-64 multiply (bias below 2^-32 for p < 2^32).
#include "common.cuh"

namespace lnc {

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

template <class T>
__global__ void fill_uniform_kernel(T* out, int64_t count, uint64_t p, uint64_t seed) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count;
         i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t h = splitmix64(seed * 0xD1B54A32D192ED03ull + (uint64_t)i);
        out[i] = (T)__umul64hi(h, p);
    }
}

int fill_uniform_dispatch(void* dev, int64_t count, uint64_t p, uint64_t seed, int dtype, cudaStream_t s) {
    if (count <= 0) return LNC_OK;
    if (p < 1) { set_error("fill: p must be positive"); return LNC_ERR_INVALID; }
    const int grid = (int)std::min<int64_t>((count + 255) / 256, 152 * 32);
    if (dtype == LNC_U32) {
        if (p > 0xFFFFFFFFull + 1) { set_error("fill: p too large for uint32"); return LNC_ERR_INVALID; }
        fill_uniform_kernel<uint32_t><<<grid, 256, 0, s>>>((uint32_t*)dev, count, p, seed);
    } else if (dtype == LNC_U64) {
        fill_uniform_kernel<uint64_t><<<grid, 256, 0, s>>>((uint64_t*)dev, count, p, seed);
    } else {
        set_error("fill: dtype must be LNC_U32 or LNC_U64");
        return LNC_ERR_INVALID;
    }
    LNC_CHECK_LAUNCH("fill_uniform_kernel");
    return LNC_OK;
}

}  // namespace lnc

extern "C" int lnc_fill_uniform_modp(void* dev_ptr, int64_t count, uint64_t p, uint64_t seed, int dtype,
                                     void* stream) {
    return lnc::fill_uniform_dispatch(dev_ptr, count, p, seed, dtype, (cudaStream_t)stream);
}
