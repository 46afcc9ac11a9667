// Mixed-precision float path: fixed-point tensor-core trailing update and the
// FP64 kernels of the iterative refinement.
//
// Trailing update  A[:, T] += E * A[P, T]  (float64 / complex128).  Every
// row of E and every column of B = A[P, T] is scaled by a power of two so that
// its largest entry lies below 2^31, rounded to an integer (31 bits plus
// sign), and split into four balanced base-256 digits in [-128, 128], exact in
// BF16.  The limb GEMM of the F_p path (tc_kernels.cuh) multiplies the digits
// on the tensor cores with FP32 accumulation; every digit-group sum is an
// integer below 2^24 in magnitude, hence exact, so the contraction of the
// rounded operands is exact and is rounded once to FP64 in the epilogue
// (then scaled back and added to A).  The only error is the rounding of E and
// B to 31-bit fixed point relative to their row / column maxima: a 2^-31
// relative contraction instead of FP64's 2^-53.  The FP64 panels, pivot choice
// and threshold are those of the FP64 path; the refinement below restores
// FP64 accuracy of the non-pivot columns.
//
// Complex128 is realified: GEMM rows 2r and 2r + 1 of E are [Re E_r, -Im E_r]
// and [Im E_r, Re E_r] (contraction depth 2k <= 128, so the panel width is at
// most 64), B's rows are [Re B; Im B], and the epilogue writes the real and
// imaginary parts of output row r.
//
// Refinement (rref.cu drives it): with the RREF R of the eliminated matrix,
// pivot columns Pc and non-pivot columns Nc, the residual of the non-pivot
// columns is  Res = A_s Z,  Z[Pc[t], j] = -R[t, Nc[j]],  Z[Nc[j], j] = 1
// (A_s the row-scaled input), and the correction is M Res, M the product of
// the panel transforms of the elimination (stored E and pivot rows per
// panel); R[t, Nc[j]] += (M Res)[piv_row[t], j].
#include <cuda_bf16.h>

#include "tc_kernels.cuh"

namespace lnc {

int tc_make_map_bf16(CUtensorMap* map, void* base, uint64_t inner, uint64_t outer, uint32_t box_inner,
                     uint32_t box_outer);

namespace fx {

using tc::BM;
using tc::BN;
using tc::B_ROWS;
using tc::KMAX;
using tc::LIMBS;

__host__ __device__ inline int m_pad_of(int64_t rows) { return (int)((rows + BM - 1) / BM * BM); }
__host__ __device__ inline int n_tiles_of(int64_t n) { return (int)((n + BN - 1) / BN); }

// x * 2^(31 - e) rounded (|x| < 2^e) -> four balanced base-256 digits (the top one in [-128, 128])
__device__ __forceinline__ void split_fixed(double x, int e, __nv_bfloat16 (&d)[LIMBS]) {
    long long v = llrint(scalbn(x, 31 - e));
#pragma unroll
    for (int i = 0; i < LIMBS - 1; ++i) {
        const int di = (int)(((v + 128) & 255) - 128);
        d[i] = __int2bfloat16_rn(di);
        v = (v - di) >> 8;  // exact: v - di is a multiple of 256
    }
    d[LIMBS - 1] = __int2bfloat16_rn((int)v);
}

__device__ __forceinline__ int exponent_above(double mx) {  // smallest e with mx < 2^e (0 for 0)
    int e = 0;
    if (mx > 0.0) frexp(mx, &e);
    return e;
}

template <bool CPLX>
__device__ __forceinline__ double e_entry(const void* E, int64_t ldE, int64_t R, int t, int k) {
    if constexpr (!CPLX) {
        return t < k ? ((const double*)E)[R * ldE + t] : 0.0;
    } else {
        // GEMM row 2r: [Re, -Im], 2r + 1: [Im, Re] of source row r
        const int64_t r = R >> 1;
        const int part = (int)(R & 1);
        if (t >= 2 * k) return 0.0;
        const double* src = (const double*)E + 2 * (r * ldE + (t < k ? t : t - k));
        if (t < k) return part ? src[1] : src[0];
        return part ? src[0] : -src[1];
    }
}

// digit planes of E (one warp per GEMM row) and the row scales 2^(e_r - 31)
template <bool CPLX>
static __global__ void __launch_bounds__(256) fx_split_e_kernel(const void* E, int64_t ldE, int64_t rows,
                                                                int m_pad, const int32_t* k_ptr,
                                                                __nv_bfloat16* EL, double* rscale) {
    const int k = *k_ptr;
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t R = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); R < m_pad; R += warps) {
        double x[KMAX / 32];
        double mx = 0.0;
#pragma unroll
        for (int j = 0; j < KMAX / 32; ++j) {
            x[j] = (R < rows) ? e_entry<CPLX>(E, ldE, R, lane + 32 * j, k) : 0.0;
            mx = fmax(mx, fabs(x[j]));
        }
        for (int o = 16; o; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        const int e = exponent_above(mx);
        if (lane == 0 && R < rows) rscale[R] = scalbn(1.0, e - 31);
#pragma unroll
        for (int j = 0; j < KMAX / 32; ++j) {
            __nv_bfloat16 d[LIMBS];
            split_fixed(x[j], e, d);
#pragma unroll
            for (int i = 0; i < LIMBS; ++i) EL[((size_t)i * m_pad + R) * KMAX + lane + 32 * j] = d[i];
        }
    }
}

// pivot rows of the trailing block (zeroed in C) -> stacked digit tiles of B
// and the column scales 2^(f_c - 31); one CTA per 32-column tile
template <bool CPLX>
static __global__ void __launch_bounds__(256) fx_gather_split_b_kernel(void* C, int64_t ldc, int64_t N,
                                                                       const int32_t* rows,
                                                                       const int32_t* k_ptr,
                                                                       __nv_bfloat16* BS, double* cscale,
                                                                       int32_t* kk_out) {
    __shared__ double s[KMAX][BN + 1];
    __shared__ int s_e[BN];
    const int k = *k_ptr;
    const int kk = CPLX ? 2 * k : k;
    if (blockIdx.x == 0 && threadIdx.x == 0 && kk_out) *kk_out = kk;
    if (k == 0) return;
    const int64_t c0 = (int64_t)blockIdx.x * BN;
    for (int idx = threadIdx.x; idx < KMAX * BN; idx += blockDim.x) {
        const int t = idx / BN, cc = idx % BN;
        if (CPLX ? (t >= k) : false) continue;  // complex: rows t < k fill s[t] and s[t + k]
        double v = 0.0, w = 0.0;
        if (t < k && c0 + cc < N) {
            if constexpr (CPLX) {
                double* src = (double*)C + 2 * ((int64_t)rows[t] * ldc + c0 + cc);
                v = src[0];
                w = src[1];
                src[0] = 0.0;
                src[1] = 0.0;
            } else {
                double* src = (double*)C + (int64_t)rows[t] * ldc + c0 + cc;
                v = *src;
                *src = 0.0;
            }
        }
        s[t][cc] = v;
        if constexpr (CPLX) s[t + k][cc] = w;
    }
    if constexpr (CPLX) {
        for (int idx = threadIdx.x; idx < KMAX * BN; idx += blockDim.x) {
            const int t = idx / BN, cc = idx % BN;
            if (t >= 2 * k) s[t][cc] = 0.0;
        }
    }
    __syncthreads();
    if (threadIdx.x < BN) {
        const int cc = threadIdx.x;
        double mx = 0.0;
        for (int t = 0; t < kk; ++t) mx = fmax(mx, fabs(s[t][cc]));
        const int e = exponent_above(mx);
        s_e[cc] = e;
        if (c0 + cc < N) cscale[c0 + cc] = scalbn(1.0, e - 31);
    }
    __syncthreads();
    __nv_bfloat16* dst = BS + (size_t)blockIdx.x * B_ROWS * KMAX;
    for (int idx = threadIdx.x; idx < BN * KMAX; idx += blockDim.x) {
        const int cc = idx / KMAX, t = idx % KMAX;
        __nv_bfloat16 d[LIMBS];
        split_fixed(s[t][cc], s_e[cc], d);
#pragma unroll
        for (int i = 0; i < LIMBS; ++i) dst[((size_t)i * BN + cc) * KMAX + t] = d[i];
    }
}

}  // namespace fx

// scratch of the fixed-point trailing update: digit planes of E (4 x m_pad x
// 128), digit tiles of B, row / column scales, the contraction depth word
size_t trailing_fx_scratch(int64_t m, int64_t n, bool cplx) {
    const int64_t rows = cplx ? 2 * m : m;
    const size_t el = (size_t)tc::LIMBS * fx::m_pad_of(rows) * tc::KMAX * 2;
    const size_t bs = (size_t)fx::n_tiles_of(n) * tc::B_ROWS * tc::KMAX * 2;
    return 1024 + (el + 1023) / 1024 * 1024 + (bs + 1023) / 1024 * 1024 + 8 * (size_t)fx::m_pad_of(rows) +
           8 * (size_t)(n + 32) + 256;
}

template <class F>
int trailing_update_fx(const TrailingCtx<F>& t, cudaStream_t s) {
    constexpr bool CPLX = F::kDtype == LNC_C128;
    using namespace tc;
    const int64_t rows = CPLX ? 2 * t.m : t.m;
    const int m_pad = fx::m_pad_of(rows);
    const int n_tiles = fx::n_tiles_of(t.N);
    unsigned char* base = (unsigned char*)(((uintptr_t)t.fx + 1023) & ~(uintptr_t)1023);
    const size_t el = (size_t)LIMBS * m_pad * KMAX * 2;
    __nv_bfloat16* EL = (__nv_bfloat16*)base;
    __nv_bfloat16* BS = (__nv_bfloat16*)(base + (el + 1023) / 1024 * 1024);
    const size_t bs_max = (size_t)fx::n_tiles_of(t.n) * B_ROWS * KMAX * 2;
    double* rscale = (double*)((unsigned char*)BS + (bs_max + 1023) / 1024 * 1024);
    double* cscale = rscale + m_pad;
    int32_t* kk = (int32_t*)(cscale + t.n + 32);
    {
        const int grid = (int)std::min<int64_t>((m_pad + 7) / 8, 4096);
        fx::fx_split_e_kernel<CPLX><<<grid, 256, 0, s>>>(t.E, t.ldE, rows, m_pad, t.panel_k, EL, rscale);
        LNC_CHECK_LAUNCH("fx_split_e_kernel");
    }
    fx::fx_gather_split_b_kernel<CPLX><<<n_tiles, 256, 0, s>>>((void*)(t.A + t.j1), t.lda, t.N, t.panel_rows,
                                                               t.panel_k, BS, cscale, kk);
    LNC_CHECK_LAUNCH("fx_gather_split_b_kernel");
    CUtensorMap mapA, mapB;
    int rc = tc_make_map_bf16(&mapA, EL, KMAX, (uint64_t)LIMBS * m_pad, KC, BM);
    if (!rc) rc = tc_make_map_bf16(&mapB, BS, KMAX, (uint64_t)n_tiles * B_ROWS, KC, B_ROWS);
    if (rc) return rc;
    TcParams P{};
    P.C = nullptr;
    P.ldc = t.lda;
    P.m = rows;
    P.N = t.N;
    P.m_pad = m_pad;
    P.n_tiles = n_tiles;
    P.panel_k = kk;
    P.overwrite = 0;
    P.err = t.err;
    P.status = t.status;
    P.Cd = (double*)(t.A + t.j1);
    P.rscale = rscale;
    P.cscale = cscale;
    P.tpc = limb_tiles_per_cta(n_tiles, m_pad / BM);
    constexpr int EPI = CPLX ? EPI_C128 : EPI_F64;
    auto kern = limb_gemm_kernel<EPI>;
    LNC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES));
    dim3 grid((unsigned)((n_tiles + P.tpc - 1) / P.tpc), (unsigned)(m_pad / BM));
    if (grid.y > 65535) { set_error("trailing update: too many row blocks"); return LNC_ERR_UNSUPPORTED; }
    ScopedKernelTimer kt(KC_TRAILING, s, (double)t.m * (double)t.N * (double)t.b * (CPLX ? 4.0 : 1.0));
    kern<<<grid, THREADS, SMEM_BYTES, s>>>(mapA, mapB, P);
    LNC_CHECK_LAUNCH("limb_gemm_kernel (fixed point)");
    return LNC_OK;
}

template int trailing_update_fx<FieldF64>(const TrailingCtx<FieldF64>&, cudaStream_t);
template int trailing_update_fx<FieldC128>(const TrailingCtx<FieldC128>&, cudaStream_t);

// ----------------------------------------------------------------------------
// refinement kernels (FP64)
// ----------------------------------------------------------------------------
namespace fx {

template <class T> struct Ar;
template <> struct Ar<double> {
    static __device__ __forceinline__ double zero() { return 0.0; }
    static __device__ __forceinline__ double fma_(double a, double b, double c) { return fma(a, b, c); }
    static __device__ __forceinline__ double add(double a, double b) { return a + b; }
    static __device__ __forceinline__ double neg(double a) { return -a; }
    static __device__ __forceinline__ double absv(double a) { return fabs(a); }
    static __device__ __forceinline__ double one() { return 1.0; }
};
template <> struct Ar<c128> {
    static __device__ __forceinline__ c128 mk(double x, double y) { c128 r; r.x = x; r.y = y; return r; }
    static __device__ __forceinline__ c128 zero() { return mk(0.0, 0.0); }
    static __device__ __forceinline__ c128 fma_(c128 a, c128 b, c128 c) {
        return mk(fma(a.x, b.x, fma(-a.y, b.y, c.x)), fma(a.x, b.y, fma(a.y, b.x, c.y)));
    }
    static __device__ __forceinline__ c128 add(c128 a, c128 b) { return mk(a.x + b.x, a.y + b.y); }
    static __device__ __forceinline__ c128 neg(c128 a) { return mk(-a.x, -a.y); }
    static __device__ __forceinline__ double absv(c128 a) { return hypot(a.x, a.y); }
    static __device__ __forceinline__ c128 one() { return mk(1.0, 0.0); }
};

// C[:m, :q] += A[:m, :K] B[:K, :q] for narrow q: a CTA owns 32 rows x 16
// columns and streams K in chunks of 32 through shared memory; K is *k_ptr
// when k_ptr is given.
template <class T>
static __global__ void __launch_bounds__(256) narrow_gemm_kernel(int64_t m, int q, int64_t K, const int32_t* k_ptr,
                                                                 const T* A, int64_t lda, const T* B, int64_t ldb,
                                                                 T* C, int64_t ldc) {
    constexpr int RB = 32, CB = 16, KB = 32;
    __shared__ T As[RB][KB + 1];
    __shared__ T Bs[KB][CB];
    const int64_t kk = k_ptr ? (int64_t)*k_ptr : K;
    const int64_t r0 = (int64_t)blockIdx.x * RB;
    const int c0 = blockIdx.y * CB;
    const int tr = threadIdx.x >> 3, tc2 = (threadIdx.x & 7) * 2;
    T acc0 = Ar<T>::zero(), acc1 = Ar<T>::zero();
    for (int64_t k0 = 0; k0 < kk; k0 += KB) {
        for (int idx = threadIdx.x; idx < RB * KB; idx += blockDim.x) {
            const int r = idx / KB, c = idx % KB;
            As[r][c] = (r0 + r < m && k0 + c < kk) ? A[(r0 + r) * lda + k0 + c] : Ar<T>::zero();
        }
        for (int idx = threadIdx.x; idx < KB * CB; idx += blockDim.x) {
            const int r = idx / CB, c = idx % CB;
            Bs[r][c] = (k0 + r < kk && c0 + c < q) ? B[(k0 + r) * ldb + c0 + c] : Ar<T>::zero();
        }
        __syncthreads();
#pragma unroll 8
        for (int t = 0; t < KB; ++t) {
            const T a = As[tr][t];
            acc0 = Ar<T>::fma_(a, Bs[t][tc2], acc0);
            acc1 = Ar<T>::fma_(a, Bs[t][tc2 + 1], acc1);
        }
        __syncthreads();
    }
    const int64_t r = r0 + tr;
    if (r < m) {
        if (c0 + tc2 < q) C[r * ldc + c0 + tc2] = Ar<T>::add(C[r * ldc + c0 + tc2], acc0);
        if (c0 + tc2 + 1 < q) C[r * ldc + c0 + tc2 + 1] = Ar<T>::add(C[r * ldc + c0 + tc2 + 1], acc1);
    }
}

// Z[c, j] = -R[colmap[c], Nc[j]] for a pivot column c, [c == Nc[j]] otherwise
template <class T>
static __global__ void build_z_kernel(int64_t n, int q, const int32_t* colmap, const int32_t* Nc, const T* R,
                                      int64_t ldr, T* Z) {
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n * q;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = idx / q;
        const int j = (int)(idx % q);
        const int t = colmap[c];
        Z[idx] = t >= 0 ? Ar<T>::neg(R[(int64_t)t * ldr + Nc[j]]) : (c == Nc[j] ? Ar<T>::one() : Ar<T>::zero());
    }
}

// R[t, Nc[j]] += D[piv_row[t], j]; stats[0] = max |correction|, stats[1] = max |R[t, Nc[j]]|
// (non-negative doubles compare like their bit patterns)
template <class T>
static __global__ void apply_correction_kernel(int64_t rank, int q, const int32_t* piv_row, const int32_t* Nc,
                                               const T* D, T* R, int64_t ldr, unsigned long long* stats,
                                               int apply) {
    double mc = 0.0, mv = 0.0;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < rank * q;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t t = idx / q;
        const int j = (int)(idx % q);
        const T corr = D[(int64_t)piv_row[t] * q + j];
        T* y = R + t * ldr + Nc[j];
        if (apply) *y = Ar<T>::add(*y, corr);
        mc = fmax(mc, Ar<T>::absv(corr));
        mv = fmax(mv, Ar<T>::absv(*y));
    }
    for (int o = 16; o; o >>= 1) {
        mc = fmax(mc, __shfl_xor_sync(0xffffffffu, mc, o));
        mv = fmax(mv, __shfl_xor_sync(0xffffffffu, mv, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(stats + 0, (unsigned long long)__double_as_longlong(mc));
        atomicMax(stats + 1, (unsigned long long)__double_as_longlong(mv));
    }
}

}  // namespace fx

template <class T>
int refine_narrow_gemm(int64_t m, int q, int64_t K, const int32_t* k_ptr, const T* A, int64_t lda, const T* B,
                       int64_t ldb, T* C, int64_t ldc, cudaStream_t s) {
    if (m <= 0 || q <= 0) return LNC_OK;
    dim3 grid((unsigned)((m + 31) / 32), (unsigned)((q + 15) / 16));
    if (grid.y > 65535) { set_error("refinement: too many columns"); return LNC_ERR_UNSUPPORTED; }
    fx::narrow_gemm_kernel<T><<<grid, 256, 0, s>>>(m, q, K, k_ptr, A, lda, B, ldb, C, ldc);
    LNC_CHECK_LAUNCH("narrow_gemm_kernel");
    return LNC_OK;
}

template <class T>
int refine_build_z(int64_t n, int q, const int32_t* colmap, const int32_t* Nc, const T* R, int64_t ldr, T* Z,
                   cudaStream_t s) {
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((n * q + 255) / 256, 4096));
    fx::build_z_kernel<T><<<grid, 256, 0, s>>>(n, q, colmap, Nc, R, ldr, Z);
    LNC_CHECK_LAUNCH("build_z_kernel");
    return LNC_OK;
}

template <class T>
int refine_apply(int64_t rank, int q, const int32_t* piv_row, const int32_t* Nc, const T* D, T* R, int64_t ldr,
                 unsigned long long* stats, cudaStream_t s, bool apply) {
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((rank * q + 255) / 256, 4096));
    fx::apply_correction_kernel<T><<<grid, 256, 0, s>>>(rank, q, piv_row, Nc, D, R, ldr, stats, apply ? 1 : 0);
    LNC_CHECK_LAUNCH("apply_correction_kernel");
    return LNC_OK;
}

template int refine_narrow_gemm<double>(int64_t, int, int64_t, const int32_t*, const double*, int64_t, const double*,
                                        int64_t, double*, int64_t, cudaStream_t);
template int refine_narrow_gemm<c128>(int64_t, int, int64_t, const int32_t*, const c128*, int64_t, const c128*,
                                      int64_t, c128*, int64_t, cudaStream_t);
template int refine_build_z<double>(int64_t, int, const int32_t*, const int32_t*, const double*, int64_t, double*,
                                    cudaStream_t);
template int refine_build_z<c128>(int64_t, int, const int32_t*, const int32_t*, const c128*, int64_t, c128*,
                                  cudaStream_t);
template int refine_apply<double>(int64_t, int, const int32_t*, const int32_t*, const double*, double*, int64_t,
                                  unsigned long long*, cudaStream_t, bool);
template int refine_apply<c128>(int64_t, int, const int32_t*, const int32_t*, const c128*, c128*, int64_t,
                                unsigned long long*, cudaStream_t, bool);

}  // namespace lnc
