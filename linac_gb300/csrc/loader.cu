// Monomial matrix loader: out[r, c] = prod_t bases[r, lindices[c, t]].
//
// linac's LoadMatrix (linac/matrix_loader.cu:88-112) runs one block per row,
// stages that row's basis values in shared memory and re-reads / re-writes the
// global output element once per factor, with a wide `%` per product.  Here a
// CTA owns a band of rows and walks a strip of 256-column blocks: the band's
// basis values are staged in shared memory once per CTA (as multipliers ready
// for the CTA's arithmetic), each column block's index lists are copied in
// with one coalesced sweep, every thread keeps its band's running products in
// registers, and each output element is written exactly once, coalesced.
//
// F_p with p < 2^31 (the served stream's moduli): a product of residues mod p
// does not depend on how it is associated, so the band stages every pair
// product b_i b_j (with its Shoup constant floor(b_i b_j 2^32 / p)) and a
// column of d factors takes ceil(d/2) - 1 pair / single multiplications
// instead of d - 1.  Each is a lazy Shoup product -- q = hi32(a b'),
// r = a b - q p in 32-bit arithmetic, r in [0, 2p) for any a < 2^32 -- three
// integer multiplies, one final correction.  Other moduli and the reals /
// complex numbers multiply factor by factor (Montgomery for odd 64-bit p,
// Barrett for 2^31 <= p < 2^32, exact IEEE products folded left to right).
//
// Semantics follow the reference: the product is folded left to right, each
// product reduced mod p (any association gives the same residue); a single
// factor is copied unreduced (as the reference GPU kernel and its CPU fallback
// both do).  Real / complex products use round-to-nearest multiplies without
// contraction, so they are bit-identical to the Python left fold of linac's
// CPU path (pycuda_matrix_loader.py:225).  An index past the end of a bases
// row is an error: the host entry rejects it before launching; on the device
// entry the kernel writes 0 for that column and raises the library's device
// status word to LNC_ERR_INVALID (read by lnc_device_status).
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

constexpr int kLoadCols = 256;      // columns per block (one per thread)
constexpr int kLoadStripBlocks = 8;  // column blocks a CTA walks (staging amortised over them)

int* rref_status_symbol_address();

__device__ __forceinline__ void raise_invalid(int* status) {
    if (status) atomicCAS(status, 0, LNC_ERR_INVALID);
}

// Factor by factor, for every element type: the band's basis values in the
// arithmetic's working form, [basis_len][ROWS + 1] (the pad spreads the rows
// of different indices over the banks).
template <class Ops, int ROWS>
__global__ void __launch_bounds__(kLoadCols) load_matrix_kernel(Ops ops, const typename Ops::T* bases,
                                                               int n_rows, int basis_len, const uint32_t* lind,
                                                               int64_t n_cols, int degree, typename Ops::T* out,
                                                               int64_t ldo, int* status) {
    using T = typename Ops::T;
    using W = typename Ops::W;
    constexpr int RP = ROWS + 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    W* bs = (W*)smem_raw;                                    // [basis_len][RP]
    uint32_t* ls = (uint32_t*)(bs + (size_t)basis_len * RP);  // [kLoadCols * degree], row-major per column
    const int r0 = blockIdx.y * ROWS;
    const int nr = min(ROWS, n_rows - r0);
    for (int i = threadIdx.x; i < nr * basis_len; i += blockDim.x) {
        const int r = i / basis_len, v = i - r * basis_len;
        bs[v * RP + r] = ops.to_work(bases[(int64_t)(r0 + r) * basis_len + v]);
    }
    const int64_t blocks = (n_cols + kLoadCols - 1) / kLoadCols;
    for (int64_t blk = (int64_t)blockIdx.x * kLoadStripBlocks;
         blk < ::min((int64_t)blocks, ((int64_t)blockIdx.x + 1) * kLoadStripBlocks); ++blk) {
        const int64_t c0 = blk * kLoadCols;
        const int nc = (int)::min((int64_t)kLoadCols, n_cols - c0);
        __syncthreads();  // previous block's indices consumed (and the band staged, on the first pass)
        for (int i = threadIdx.x; i < nc * degree; i += blockDim.x) ls[i] = lind[c0 * degree + i];
        __syncthreads();
        const int c = threadIdx.x;
        if (c >= nc) continue;
        const uint32_t* li = ls + c * degree;
        T* dst = out + (int64_t)r0 * ldo + c0 + c;
        bool bad = false;
        for (int t = 0; t < degree; ++t) bad |= li[t] >= (uint32_t)basis_len;
        if (bad) {
            raise_invalid(status);
            for (int r = 0; r < nr; ++r) dst[(int64_t)r * ldo] = T{};
            continue;
        }
        if (degree == 1) {  // a single factor is copied as given
            for (int r = 0; r < nr; ++r) dst[(int64_t)r * ldo] = bases[(int64_t)(r0 + r) * basis_len + li[0]];
            continue;
        }
        W acc[ROWS];
        {
            const W* b = bs + li[0] * RP;
#pragma unroll
            for (int r = 0; r < ROWS; ++r) acc[r] = b[r];
        }
        for (int t = 1; t < degree; ++t) {
            const W* b = bs + li[t] * RP;
#pragma unroll
            for (int r = 0; r < ROWS; ++r) acc[r] = ops.mul(acc[r], b[r]);
        }
#pragma unroll
        for (int r = 0; r < ROWS; ++r)
            if (r < nr) dst[(int64_t)r * ldo] = ops.from_work(acc[r]);
    }
}

// F_p, p < 2^31: pair products with Shoup constants, [basis_len^2][ROWS + 1]
// entries (x = b_i b_j mod p, y = floor(x 2^32 / p)); the pair (i, j) sits at
// i * basis_len + j, both orders staged, and the single factors b_i (with
// their constants) follow at basis_len^2 + i.
struct ShoupPairs {
    uint32_t p;
    uint64_t mu;  // floor((2^64 - 1) / p)
    static ShoupPairs make(uint64_t prime) { ShoupPairs o; o.p = (uint32_t)prime; o.mu = ~0ull / prime; return o; }
    __device__ __forceinline__ uint32_t reduce(uint64_t x) const {  // x mod p (Barrett)
        uint64_t q = __umul64hi(x, mu);
        uint64_t r = x - q * (uint64_t)p;
        r = r >= p ? r - p : r;
        return (uint32_t)(r >= p ? r - p : r);
    }
    // x < p  ->  (x, floor(x 2^32 / p))
    __device__ __forceinline__ uint2 with_constant(uint32_t x) const {
        const uint64_t num = (uint64_t)x << 32;
        uint64_t q = __umul64hi(num, mu);
        uint64_t r = num - q * (uint64_t)p;
        while (r >= p) { r -= p; ++q; }
        return make_uint2(x, (uint32_t)q);
    }
    // a * m.x mod p, lazily: the result lies in [0, 2p) for any a < 2^32
    __device__ __forceinline__ uint32_t mul(uint32_t a, uint2 m) const {
        const uint32_t q = __umulhi(a, m.y);
        return a * m.x - q * p;
    }
};

template <int ROWS>
__global__ void __launch_bounds__(kLoadCols) load_pairs_kernel(ShoupPairs ops, const uint32_t* bases, int n_rows,
                                                              int basis_len, const uint32_t* lind, int64_t n_cols,
                                                              int degree, uint32_t* out, int64_t ldo, int* status) {
    constexpr int RP = ROWS + 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int L = basis_len, L2 = basis_len * basis_len;
    uint2* ps = (uint2*)smem_raw;                            // [(L^2 + L)][RP]
    uint32_t* ls = (uint32_t*)(ps + (size_t)(L2 + L) * RP);  // [kLoadCols * degree]
    uint32_t* raw = ls + kLoadCols * degree;                 // [ROWS][L] band values mod p
    const int r0 = blockIdx.y * ROWS;
    const int nr = min(ROWS, n_rows - r0);
    for (int i = threadIdx.x; i < ROWS * L; i += blockDim.x) {
        const int r = i / L, v = i - r * L;
        raw[i] = r < nr ? ops.reduce(bases[(int64_t)(r0 + r) * L + v]) : 0u;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < (L2 + L) * ROWS; i += blockDim.x) {
        const int e = i / ROWS, r = i - e * ROWS;
        uint32_t x;
        if (e < L2) {
            const int a = e / L, b = e - a * L;
            x = ops.reduce((uint64_t)raw[r * L + a] * raw[r * L + b]);
        } else {
            x = raw[r * L + (e - L2)];
        }
        ps[e * RP + r] = ops.with_constant(x);
    }
    const int64_t blocks = (n_cols + kLoadCols - 1) / kLoadCols;
    for (int64_t blk = (int64_t)blockIdx.x * kLoadStripBlocks;
         blk < ::min((int64_t)blocks, ((int64_t)blockIdx.x + 1) * kLoadStripBlocks); ++blk) {
        const int64_t c0 = blk * kLoadCols;
        const int nc = (int)::min((int64_t)kLoadCols, n_cols - c0);
        __syncthreads();
        for (int i = threadIdx.x; i < nc * degree; i += blockDim.x) ls[i] = lind[c0 * degree + i];
        __syncthreads();
        const int c = threadIdx.x;
        if (c >= nc) continue;
        const uint32_t* li = ls + c * degree;
        uint32_t* dst = out + (int64_t)r0 * ldo + c0 + c;
        bool bad = false;
        for (int t = 0; t < degree; ++t) bad |= li[t] >= (uint32_t)L;
        if (bad) {
            raise_invalid(status);
            for (int r = 0; r < nr; ++r) dst[(int64_t)r * ldo] = 0u;
            continue;
        }
        if (degree == 1) {  // a single factor is copied as given
            for (int r = 0; r < nr; ++r) dst[(int64_t)r * ldo] = bases[(int64_t)(r0 + r) * L + li[0]];
            continue;
        }
        uint32_t acc[ROWS];
        {
            const uint2* m = ps + (li[0] * L + li[1]) * RP;
#pragma unroll
            for (int r = 0; r < ROWS; ++r) acc[r] = m[r].x;
        }
        int t = 2;
        for (; t + 1 < degree; t += 2) {
            const uint2* m = ps + (li[t] * L + li[t + 1]) * RP;
#pragma unroll
            for (int r = 0; r < ROWS; ++r) acc[r] = ops.mul(acc[r], m[r]);
        }
        if (t < degree) {
            const uint2* m = ps + (L2 + li[t]) * RP;
#pragma unroll
            for (int r = 0; r < ROWS; ++r) acc[r] = ops.mul(acc[r], m[r]);
        }
#pragma unroll
        for (int r = 0; r < ROWS; ++r)
            if (r < nr) dst[(int64_t)r * ldo] = acc[r] >= ops.p ? acc[r] - ops.p : acc[r];
    }
}

static int loader_grid(int64_t n_rows, int64_t n_cols, int rows, dim3* grid) {
    const int64_t gy = (n_rows + rows - 1) / rows;
    const int64_t blocks = (n_cols + kLoadCols - 1) / kLoadCols;
    const int64_t gx = (blocks + kLoadStripBlocks - 1) / kLoadStripBlocks;
    if (gy > 65535 || gx > 2147483647ll || n_rows > INT32_MAX) {
        set_error("loader: matrix too large");
        return LNC_ERR_UNSUPPORTED;
    }
    *grid = dim3((unsigned)gx, (unsigned)gy);
    return LNC_OK;
}

static double loader_bytes(size_t elt, int64_t n_rows, int64_t n_cols, int64_t basis_len, int64_t degree) {
    return (double)elt * ((double)n_rows * n_cols + (double)n_rows * basis_len) + 4.0 * (double)n_cols * degree;
}

template <class Ops, int ROWS>
static int launch_loader(const Ops& ops, int64_t n_rows, int64_t n_cols, int64_t basis_len, int64_t degree,
                         const void* bases, const uint32_t* lind, void* out, int64_t ldo, int* status,
                         cudaStream_t s) {
    using T = typename Ops::T;
    using W = typename Ops::W;
    const size_t smem = sizeof(W) * (size_t)basis_len * (ROWS + 1) + sizeof(uint32_t) * (size_t)degree * kLoadCols;
    DeviceInfo di;
    int rc = device_info(&di);
    if (rc) return rc;
    if (smem > (size_t)di.smem_optin || basis_len > INT32_MAX || degree > INT32_MAX) {
        set_error("loader: basis length %lld x degree %lld exceeds shared memory", (long long)basis_len,
                  (long long)degree);
        return LNC_ERR_UNSUPPORTED;
    }
    auto kern = load_matrix_kernel<Ops, ROWS>;
    rc = allow_dynamic_smem((const void*)kern, smem);
    if (rc) return rc;
    dim3 grid;
    rc = loader_grid(n_rows, n_cols, ROWS, &grid);
    if (rc) return rc;
    ScopedKernelTimer kt(KC_LOADER, s, loader_bytes(sizeof(T), n_rows, n_cols, basis_len, degree));
    kern<<<grid, kLoadCols, smem, s>>>(ops, (const T*)bases, (int)n_rows, (int)basis_len, lind, n_cols, (int)degree,
                                       (T*)out, ldo, status);
    LNC_CHECK_LAUNCH("load_matrix_kernel");
    return LNC_OK;
}

constexpr int kPairRows = 32;

static size_t pairs_smem(int64_t basis_len, int64_t degree) {
    return sizeof(uint2) * (size_t)(basis_len * basis_len + basis_len) * (kPairRows + 1) +
           sizeof(uint32_t) * ((size_t)degree * kLoadCols + (size_t)kPairRows * basis_len);
}

static int launch_pairs(uint64_t p, int64_t n_rows, int64_t n_cols, int64_t basis_len, int64_t degree,
                        const void* bases, const uint32_t* lind, void* out, int64_t ldo, int* status, cudaStream_t s) {
    const size_t smem = pairs_smem(basis_len, degree);
    auto kern = load_pairs_kernel<kPairRows>;
    int rc = allow_dynamic_smem((const void*)kern, smem);
    if (rc) return rc;
    dim3 grid;
    rc = loader_grid(n_rows, n_cols, kPairRows, &grid);
    if (rc) return rc;
    ScopedKernelTimer kt(KC_LOADER, s, loader_bytes(4, n_rows, n_cols, basis_len, degree));
    kern<<<grid, kLoadCols, smem, s>>>(ShoupPairs::make(p), (const uint32_t*)bases, (int)n_rows, (int)basis_len, lind,
                                       n_cols, (int)degree, (uint32_t*)out, ldo, status);
    LNC_CHECK_LAUNCH("load_pairs_kernel");
    return LNC_OK;
}

int load_matrix_dispatch(int dtype, int64_t n_rows, int64_t n_cols, int64_t basis_len, int64_t degree,
                         uint64_t p, const void* bases, const uint32_t* lind, void* out, int64_t ldo,
                         cudaStream_t s) {
    if (n_rows == 0 || n_cols == 0) return LNC_OK;
    if (degree < 1 || basis_len < 1) { set_error("loader: degree and basis length must be >= 1"); return LNC_ERR_INVALID; }
    int* status = rref_status_symbol_address();
    switch (dtype) {
        case LNC_U32: {
            if (p < 2 || p >= (1ull << 32)) { set_error("loader: uint32 needs 2 <= p < 2^32"); return LNC_ERR_INVALID; }
            DeviceInfo di;
            int rc = device_info(&di);
            if (rc) return rc;
            if (p < (1ull << 31) && degree >= 2 && pairs_smem(basis_len, degree) <= (size_t)std::min(di.smem_optin, 96 << 10))
                return launch_pairs(p, n_rows, n_cols, basis_len, degree, bases, lind, out, ldo, status, s);
            if ((p & 1) && p < (1ull << 31))
                return launch_loader<LoadMont32, 32>(LoadMont32::make(p), n_rows, n_cols, basis_len, degree, bases,
                                                     lind, out, ldo, status, s);
            return launch_loader<LoadBarrett32, 32>(LoadBarrett32::make(p), n_rows, n_cols, basis_len, degree, bases,
                                                    lind, out, ldo, status, s);
        }
        case LNC_U64:
            if (p < 2) { set_error("loader: p must be >= 2"); return LNC_ERR_INVALID; }
            if (p & 1)
                return launch_loader<LoadMont64, 16>(LoadMont64::make(p), n_rows, n_cols, basis_len, degree, bases,
                                                     lind, out, ldo, status, s);
            return launch_loader<LoadWide64, 16>(LoadWide64::make(p), n_rows, n_cols, basis_len, degree, bases, lind,
                                                 out, ldo, status, s);
        case LNC_F64:
            return launch_loader<LoadF64, 8>(LoadF64::make(0), n_rows, n_cols, basis_len, degree, bases, lind, out,
                                              ldo, status, s);
        case LNC_C128:
            return launch_loader<LoadC128, 8>(LoadC128::make(0), n_rows, n_cols, basis_len, degree, bases, lind, out,
                                              ldo, status, s);
        default:
            set_error("loader: unknown dtype %d", dtype);
            return LNC_ERR_INVALID;
    }
}

}  // namespace lnc
