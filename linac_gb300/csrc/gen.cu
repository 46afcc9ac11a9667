// Seeded synthetic residues on the device (benchmark and test inputs): entry
// i of a fill is a SplitMix64 hash of (seed, i) mapped to [0, p) by a
// 64 x 64 -> high-64 multiply (bias below 2^-32 for p < 2^32).
//
// Also the 64-bit-residue product C = A B mod p used to certify solves of
// augmented systems [A | B] (A X = B mod p) and to build inputs on the device.
#include "common.cuh"
#include "field.cuh"

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

// C = A B mod p for 64-bit residues (odd p): 16 x 16 output tiles, 16-deep
// slices of A and B staged in shared memory, B converted to Montgomery form
// on load so that one Montgomery product per term gives a b mod p.  A SIMT
// kernel: its use (certificates, narrow right-hand sides) is small next to
// the elimination.
constexpr int kMatTile = 16;
__global__ void __launch_bounds__(kMatTile * kMatTile) matmul_u64_kernel(FieldU64 f, const uint64_t* A, int64_t lda,
                                                                         const uint64_t* B, int64_t ldb, uint64_t* C,
                                                                         int64_t ldc, int64_t m, int64_t k, int64_t n) {
    __shared__ uint64_t As[kMatTile][kMatTile + 1];
    __shared__ uint64_t Bs[kMatTile][kMatTile + 1];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int64_t row = (int64_t)blockIdx.y * kMatTile + ty;
    const int64_t col = (int64_t)blockIdx.x * kMatTile + tx;
    uint64_t acc = 0;
    for (int64_t t0 = 0; t0 < k; t0 += kMatTile) {
        const int64_t ta = t0 + tx, tb = t0 + ty;
        As[ty][tx] = (row < m && ta < k) ? f.reduce_input(A[row * lda + ta]) : 0ull;
        Bs[ty][tx] = (tb < k && col < n) ? f.to_mont(f.reduce_input(B[tb * ldb + col])) : 0ull;
        __syncthreads();
#pragma unroll
        for (int u = 0; u < kMatTile; ++u) acc = f.add(acc, f.montmul(As[ty][u], Bs[u][tx]));
        __syncthreads();
    }
    if (row < m && col < n) C[row * ldc + col] = acc;
}

int matmul_modp_u64(uint64_t p, int64_t m, int64_t k, int64_t n, const uint64_t* A, int64_t lda, const uint64_t* B,
                    int64_t ldb, uint64_t* C, int64_t ldc, cudaStream_t s) {
    if (m <= 0 || n <= 0) return LNC_OK;
    if ((p & 1) == 0 || p < 3) { set_error("matmul: 64-bit residues need an odd p > 2"); return LNC_ERR_INVALID; }
    const int64_t gy = (m + kMatTile - 1) / kMatTile, gx = (n + kMatTile - 1) / kMatTile;
    if (gy > 65535) { set_error("matmul: at most %d rows", 65535 * kMatTile); return LNC_ERR_UNSUPPORTED; }
    if (gx > INT32_MAX) { set_error("matmul: too many columns"); return LNC_ERR_UNSUPPORTED; }
    matmul_u64_kernel<<<dim3((unsigned)gx, (unsigned)gy), dim3(kMatTile, kMatTile), 0, s>>>(
        FieldU64::make(p), A, lda, B, ldb, C, ldc, m, k, n);
    LNC_CHECK_LAUNCH("matmul_u64_kernel");
    return LNC_OK;
}

}  // namespace lnc

extern "C" int lnc_fill_uniform_modp(void* dev_ptr, int64_t count, uint64_t p, uint64_t seed, int dtype,
                                     void* stream) {
    return lnc::fill_uniform_dispatch(dev_ptr, count, p, seed, dtype, (cudaStream_t)stream);
}
