// Canonical null-space basis from an RREF, on the device.
//
// linac builds the kernel on the host from the RREF with zero rows dropped
// (linac/linear_algebra_tools.py:54-63): with pivot columns Pc (one per row)
// and the other columns Nc, the basis has one column per non-pivot column j,
//     K[Pc[t], j] = R[t, Nc[j]],   K[Nc[i], j] = -[i == j],
// so that R K = 0.  Here the RREF stays on the device (for example straight
// from lnc_rref_device), the column classification is one CTA's scan over the
// n columns, and the basis is written in the RREF's element type: -1 is p - 1
// over F_p, -1.0 over the reals and complex numbers.
#include <algorithm>

#include "common.cuh"
#include "field.cuh"

namespace lnc {
namespace {

// colmap[c] = t for pivot column c = pivots[t], else -1 - (index of c among the non-pivot columns)
static __global__ void __launch_bounds__(1024) classify_columns_kernel(int64_t r, int64_t n, const int64_t* pivots,
                                                                       int32_t* colmap, int32_t* nonpiv) {
    __shared__ int s_warp[32];
    __shared__ int s_base, s_total;
    for (int64_t c = threadIdx.x; c < n; c += blockDim.x) colmap[c] = INT32_MIN;
    __syncthreads();
    for (int64_t t = threadIdx.x; t < r; t += blockDim.x) colmap[pivots[t]] = (int32_t)t;
    if (threadIdx.x == 0) s_base = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int64_t c0 = 0; c0 < n; c0 += blockDim.x) {
        const int64_t c = c0 + threadIdx.x;
        const int flag = (c < n) && colmap[c] == INT32_MIN;
        const unsigned ballot = __ballot_sync(0xffffffffu, flag);
        if (lane == 0) s_warp[warp] = __popc(ballot);
        __syncthreads();
        if (threadIdx.x == 0) {
            int acc = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
                const int v = s_warp[w];
                s_warp[w] = acc;
                acc += v;
            }
            s_total = acc;
        }
        __syncthreads();
        if (flag) {
            const int j = s_base + s_warp[warp] + __popc(ballot & ((1u << lane) - 1u));
            colmap[c] = -1 - j;
            nonpiv[j] = (int32_t)c;
        }
        __syncthreads();
        if (threadIdx.x == 0) s_base += s_total;
        __syncthreads();
    }
}

template <class T>
static __global__ void canonical_kernel_fill(int64_t n, int64_t q, const T* R, int64_t ldr, const int32_t* colmap,
                                             const int32_t* nonpiv, T* K, int64_t ldk, T minus_one, T zero) {
    for (int64_t row = blockIdx.y; row < n; row += gridDim.y) {
        const int32_t cm = colmap[row];
        T* dst = K + row * ldk;
        for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < q; j += (int64_t)gridDim.x * blockDim.x) {
            if (cm >= 0) dst[j] = R[(int64_t)cm * ldr + nonpiv[j]];
            else dst[j] = (-1 - cm == j) ? minus_one : zero;
        }
    }
}

template <class T>
int canonical_kernel_typed(int64_t r, int64_t n, const T* R, int64_t ldr, const int64_t* pivots, T* K, int64_t ldk,
                           T minus_one, T zero, cudaStream_t s) {
    const int64_t q = n - r;
    if (q <= 0) return LNC_OK;
    void* scratch = nullptr;
    cudaError_t e = cudaMallocAsync(&scratch, sizeof(int32_t) * (size_t)(2 * n + 2), s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("canonical kernel scratch: %s", cudaGetErrorString(e));
        return LNC_ERR_OOM;
    }
    int32_t* colmap = (int32_t*)scratch;
    int32_t* nonpiv = colmap + n + 1;
    classify_columns_kernel<<<1, 1024, 0, s>>>(r, n, pivots, colmap, nonpiv);
    LNC_CHECK_LAUNCH("classify_columns_kernel");
    dim3 grid((unsigned)std::max<int64_t>(1, std::min<int64_t>((q + 255) / 256, 16)),
              (unsigned)std::min<int64_t>(n, 65535));
    canonical_kernel_fill<T><<<grid, 256, 0, s>>>(n, q, R, ldr, colmap, nonpiv, K, ldk, minus_one, zero);
    LNC_CHECK_LAUNCH("canonical_kernel_fill");
    cudaFreeAsync(scratch, s);
    return LNC_OK;
}

}  // namespace
}  // namespace lnc

using namespace lnc;

extern "C" int lnc_canonical_kernel_device(int dtype, int64_t r, int64_t n, uint64_t p, const void* dev_rref,
                                           int64_t ld_rref, const int64_t* dev_pivot_cols, void* dev_out,
                                           int64_t ld_out, void* stream) {
    if (dtype_size(dtype) == 0) { set_error("unknown dtype %d", dtype); return LNC_ERR_INVALID; }
    if (r < 0 || n < 0 || r > n || ld_rref < n || ld_out < n - r) {
        set_error("canonical kernel: bad shape (r %lld, n %lld)", (long long)r, (long long)n);
        return LNC_ERR_INVALID;
    }
    // F_p: -1 is written as p - 1 in the element type (p = 2^32 for uint32, 0 for uint64 give the
    // all-ones word, which no residue equals: callers without p use it as a marker)
    if ((dtype == LNC_U32 && (p == 1 || p > 0x100000000ull)) || (dtype == LNC_U64 && p == 1)) {
        set_error("canonical kernel: bad modulus");
        return LNC_ERR_INVALID;
    }
    cudaStream_t s = (cudaStream_t)stream;
    switch (dtype) {
        case LNC_U32:
            return canonical_kernel_typed<uint32_t>(r, n, (const uint32_t*)dev_rref, ld_rref, dev_pivot_cols,
                                                    (uint32_t*)dev_out, ld_out, (uint32_t)(p - 1), 0u, s);
        case LNC_U64:
            return canonical_kernel_typed<uint64_t>(r, n, (const uint64_t*)dev_rref, ld_rref, dev_pivot_cols,
                                                    (uint64_t*)dev_out, ld_out, p - 1, 0ull, s);
        case LNC_F64:
            return canonical_kernel_typed<double>(r, n, (const double*)dev_rref, ld_rref, dev_pivot_cols,
                                                  (double*)dev_out, ld_out, -1.0, 0.0, s);
        default: {
            c128 m1, z;
            m1.x = -1.0; m1.y = 0.0;
            z.x = 0.0; z.y = 0.0;
            return canonical_kernel_typed<c128>(r, n, (const c128*)dev_rref, ld_rref, dev_pivot_cols, (c128*)dev_out,
                                                ld_out, m1, z, s);
        }
    }
}
