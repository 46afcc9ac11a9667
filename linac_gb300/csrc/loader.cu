// Monomial matrix loader: out[r, c] = prod_t bases[r, lindices[c, t]].
//
// linac's LoadMatrix (linac/matrix_loader.cu:88-112) runs one block per row,
// stages that row's basis values in shared memory and re-reads / re-writes the
// global output element once per factor, with a wide `%` per product.  Here a
// CTA covers 8 rows x 256 columns: the 256 columns' index lists and the 8 basis
// rows are staged in shared memory once, every thread keeps its 8 running
// products in registers (Montgomery form for F_p, so one multiply-reduce per
// factor), and each output element is written exactly once, coalesced.
//
// Semantics follow the reference: the product is folded left to right, each
// product reduced mod p; a single factor is copied unreduced (as the reference
// GPU kernel and its CPU fallback both do).  Real / complex products use
// round-to-nearest multiplies without contraction, so they are bit-identical
// to the Python left fold of linac's CPU path (pycuda_matrix_loader.py:225).
#include <algorithm>

#include "common.cuh"
#include "field.cuh"

namespace lnc {

// Montgomery arithmetic with R = 2^32 for odd p < 2^31.
struct LoadMont32 {
    using T = uint32_t;
    using W = uint32_t;
    uint32_t p, pinv, r2;
    static LoadMont32 make(uint64_t prime) {
        LoadMont32 o;
        o.p = (uint32_t)prime;
        uint32_t x = o.p;
        for (int i = 0; i < 5; ++i) x *= 2u - o.p * x;
        o.pinv = 0u - x;
        o.r2 = (uint32_t)((((unsigned __int128)1) << 64) % prime);
        return o;
    }
    __device__ __forceinline__ uint32_t redc(uint64_t t) const {
        uint32_t m = (uint32_t)t * pinv;
        uint64_t u = (t + (uint64_t)m * p) >> 32;
        return (uint32_t)(u >= p ? u - p : u);
    }
    __device__ __forceinline__ W to_work(T x) const { return redc((uint64_t)x * r2); }
    __device__ __forceinline__ W mul(W a, W b) const { return redc((uint64_t)a * b); }
    __device__ __forceinline__ T from_work(W a) const { return redc((uint64_t)a); }
};

// Generic 32-bit modulus (even p): Barrett on the 64-bit product.
struct LoadBarrett32 {
    using T = uint32_t;
    using W = uint32_t;
    uint32_t p;
    uint64_t mu;
    static LoadBarrett32 make(uint64_t prime) { LoadBarrett32 o; o.p = (uint32_t)prime; o.mu = ~0ull / prime; return o; }
    __device__ __forceinline__ uint32_t red(uint64_t x) const {
        uint64_t q = __umul64hi(x, mu);
        uint64_t r = x - q * (uint64_t)p;
        r = r >= p ? r - p : r;
        r = r >= p ? r - p : r;
        return (uint32_t)r;
    }
    __device__ __forceinline__ W to_work(T x) const { return red(x); }
    __device__ __forceinline__ W mul(W a, W b) const { return red((uint64_t)a * b); }
    __device__ __forceinline__ T from_work(W a) const { return a; }
};

// 64-bit residues, odd p: Montgomery with R = 2^64 (FieldU64).
struct LoadMont64 {
    using T = uint64_t;
    using W = uint64_t;
    FieldU64 f;
    static LoadMont64 make(uint64_t prime) { LoadMont64 o; o.f = FieldU64::make(prime); return o; }
    // x * R^2 < 2^64 * p = p R, so REDC accepts unreduced inputs
    __device__ __forceinline__ W to_work(T x) const { return f.montmul(x, f.r2); }
    __device__ __forceinline__ W mul(W a, W b) const { return f.montmul(a, b); }
    __device__ __forceinline__ T from_work(W a) const { return f.from_mont(a); }
};

// 64-bit, even modulus: 128-bit remainder.
struct LoadWide64 {
    using T = uint64_t;
    using W = uint64_t;
    uint64_t p;
    static LoadWide64 make(uint64_t prime) { LoadWide64 o; o.p = prime; return o; }
    __device__ __forceinline__ W to_work(T x) const { return x % p; }
    __device__ __forceinline__ W mul(W a, W b) const {
        return (uint64_t)(((unsigned __int128)a * b) % p);
    }
    __device__ __forceinline__ T from_work(W a) const { return a; }
};

struct LoadF64 {
    using T = double;
    using W = double;
    static LoadF64 make(uint64_t) { return LoadF64{}; }
    __device__ __forceinline__ W to_work(T x) const { return x; }
    __device__ __forceinline__ W mul(W a, W b) const { return __dmul_rn(a, b); }
    __device__ __forceinline__ T from_work(W a) const { return a; }
};

struct LoadC128 {
    using T = c128;
    using W = c128;
    static LoadC128 make(uint64_t) { return LoadC128{}; }
    __device__ __forceinline__ W to_work(T x) const { return x; }
    // (a.x b.x - a.y b.y) + (a.x b.y + a.y b.x) i, each product rounded
    __device__ __forceinline__ W mul(W a, W b) const {
        W r;
        r.x = __dsub_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y));
        r.y = __dadd_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x));
        return r;
    }
    __device__ __forceinline__ T from_work(W a) const { return a; }
};

constexpr int kLoadRows = 8;
constexpr int kLoadCols = 256;

template <class Ops>
__global__ void __launch_bounds__(kLoadCols) load_matrix_kernel(Ops ops, const typename Ops::T* bases,
                                                               int64_t n_rows, int64_t basis_len,
                                                               const uint32_t* lind, int64_t n_cols,
                                                               int degree, typename Ops::T* out,
                                                               int64_t ldo) {
    using T = typename Ops::T;
    using W = typename Ops::W;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    W* bs = (W*)smem_raw;                                         // [kLoadRows][basis_len]
    uint32_t* ls = (uint32_t*)(bs + (size_t)kLoadRows * basis_len);  // [degree][kLoadCols]
    const int64_t r0 = (int64_t)blockIdx.y * kLoadRows;
    const int64_t c0 = (int64_t)blockIdx.x * kLoadCols;
    const int nr = (int)(n_rows - r0 < kLoadRows ? n_rows - r0 : kLoadRows);
    const int nc = (int)(n_cols - c0 < kLoadCols ? n_cols - c0 : kLoadCols);

    for (int64_t i = threadIdx.x; i < (int64_t)nr * basis_len; i += blockDim.x) {
        const int r = (int)(i / basis_len);
        const int64_t v = i - (int64_t)r * basis_len;
        bs[(size_t)r * basis_len + v] = ops.to_work(bases[(r0 + r) * basis_len + v]);
    }
    for (int64_t i = threadIdx.x; i < (int64_t)nc * degree; i += blockDim.x) {
        const int c = (int)(i / degree), t = (int)(i - (int64_t)c * degree);
        uint32_t ix = lind[(c0 + c) * degree + t];
        ls[(size_t)t * kLoadCols + c] = ix < basis_len ? ix : 0u;  // out-of-range index -> column 0
    }
    __syncthreads();
    const int c = threadIdx.x;
    if (c >= nc) return;
    if (degree == 1) {
        // a single factor is copied as given
        const uint32_t ix = ls[c];
        for (int r = 0; r < nr; ++r) out[(r0 + r) * ldo + c0 + c] = bases[(r0 + r) * basis_len + ix];
        return;  // degree is uniform across the grid: no thread reaches a barrier after this
    }
    W acc[kLoadRows];
    {
        const uint32_t ix = ls[c];
#pragma unroll
        for (int r = 0; r < kLoadRows; ++r)
            if (r < nr) acc[r] = bs[(size_t)r * basis_len + ix];
    }
    for (int t = 1; t < degree; ++t) {
        const uint32_t ix = ls[(size_t)t * kLoadCols + c];
#pragma unroll
        for (int r = 0; r < kLoadRows; ++r)
            if (r < nr) acc[r] = ops.mul(acc[r], bs[(size_t)r * basis_len + ix]);
    }
#pragma unroll
    for (int r = 0; r < kLoadRows; ++r)
        if (r < nr) out[(r0 + r) * ldo + c0 + c] = ops.from_work(acc[r]);
}

template <class Ops>
static int launch_loader(const Ops& ops, int64_t n_rows, int64_t n_cols, int64_t basis_len, int64_t degree,
                         const void* bases, const uint32_t* lind, void* out, int64_t ldo, cudaStream_t s) {
    using T = typename Ops::T;
    using W = typename Ops::W;
    const size_t smem = sizeof(W) * (size_t)kLoadRows * basis_len + sizeof(uint32_t) * (size_t)degree * kLoadCols;
    DeviceInfo di;
    int rc = device_info(&di);
    if (rc) return rc;
    if (smem > (size_t)di.smem_optin) {
        set_error("loader: basis length %lld x degree %lld exceeds shared memory", (long long)basis_len,
                  (long long)degree);
        return LNC_ERR_UNSUPPORTED;
    }
    auto kern = load_matrix_kernel<Ops>;
    LNC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t gy = (n_rows + kLoadRows - 1) / kLoadRows;
    const int64_t gx = (n_cols + kLoadCols - 1) / kLoadCols;
    if (gy > 65535 || gx > 2147483647ll) { set_error("loader: matrix too large"); return LNC_ERR_UNSUPPORTED; }
    ScopedKernelTimer kt(KC_LOADER, s,
                         (double)sizeof(T) * ((double)n_rows * n_cols + (double)n_rows * basis_len) +
                             4.0 * (double)n_cols * degree);
    kern<<<dim3((unsigned)gx, (unsigned)gy), kLoadCols, smem, s>>>(ops, (const T*)bases, n_rows, basis_len, lind,
                                                                   n_cols, (int)degree, (T*)out, ldo);
    LNC_CHECK_LAUNCH("load_matrix_kernel");
    return LNC_OK;
}

int load_matrix_dispatch(int dtype, int64_t n_rows, int64_t n_cols, int64_t basis_len, int64_t degree,
                         uint64_t p, const void* bases, const uint32_t* lind, void* out, int64_t ldo,
                         cudaStream_t s) {
    if (n_rows == 0 || n_cols == 0) return LNC_OK;
    if (degree < 1 || basis_len < 1) { set_error("loader: degree and basis length must be >= 1"); return LNC_ERR_INVALID; }
    switch (dtype) {
        case LNC_U32:
            if (p < 2 || p >= (1ull << 32)) { set_error("loader: uint32 needs 2 <= p < 2^32"); return LNC_ERR_INVALID; }
            if ((p & 1) && p < (1ull << 31))
                return launch_loader(LoadMont32::make(p), n_rows, n_cols, basis_len, degree, bases, lind, out, ldo, s);
            return launch_loader(LoadBarrett32::make(p), n_rows, n_cols, basis_len, degree, bases, lind, out, ldo, s);
        case LNC_U64:
            if (p < 2) { set_error("loader: p must be >= 2"); return LNC_ERR_INVALID; }
            if (p & 1) return launch_loader(LoadMont64::make(p), n_rows, n_cols, basis_len, degree, bases, lind, out, ldo, s);
            return launch_loader(LoadWide64::make(p), n_rows, n_cols, basis_len, degree, bases, lind, out, ldo, s);
        case LNC_F64:
            return launch_loader(LoadF64::make(0), n_rows, n_cols, basis_len, degree, bases, lind, out, ldo, s);
        case LNC_C128:
            return launch_loader(LoadC128::make(0), n_rows, n_cols, basis_len, degree, bases, lind, out, ldo, s);
        default:
            set_error("loader: unknown dtype %d", dtype);
            return LNC_ERR_INVALID;
    }
}

}  // namespace lnc
