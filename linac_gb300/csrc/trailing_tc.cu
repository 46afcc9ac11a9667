// Exact F_p trailing update on the tcgen05 tensor cores (32-bit residues).
//
//   C[:, T] <- C[:, T] + E * B   (mod p),  E: m x K transform, B: K x N pivot rows
//
// The reference has no counterpart for this step: linac eliminates one column
// at a time with a 64-bit `%` per element (linac/row_reduce.cu:107-114,
// 138-196).  Here the whole panel (K = 128 pivots) is applied in one
// contraction, exactly, on the BF16 tensor cores:
//
//  * every residue x (centred to (-p/2, p/2)) is split into four balanced
//    base-256 digits x = sum_i d_i 256^i, d_i in [-128, 128]; integers of that
//    size are exact in BF16;
//  * a digit product is at most 2^14 in magnitude, and the four products that
//    share a weight 256^s (s = i + j) summed over K = 128 stay below 2^23, so
//    every FP32 accumulation in TMEM is an exact integer;
//  * the epilogue converts the seven group sums D_s to integers, forms
//    sum_s D_s * (256^s mod p) in 64-bit, reduces it mod p (Barrett) and adds
//    it to the old residue.
//
// Layout: the four E digit planes are K-major (row = matrix row, 128 digits),
// the B digits are stacked per 64-column output tile as 4 x 64 K-major rows, so
// one UMMA (M = 128, N = 256, K = 16) multiplies digit plane i of E with all
// four digit planes of B and lands in TMEM columns [64 i, 64 i + 256): the
// column block s = i + j accumulates exactly the weight-256^s products.
//
// Kernel: one CTA per 128-row block and up to 8 consecutive 64-column tiles;
// warp 0 issues TMA loads (E digits once, B digits double-buffered), warp 1
// issues the UMMAs and owns the TMEM allocation, warps 2-5 drain TMEM, combine,
// write C and re-zero their TMEM lanes for the next tile.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include <cuda.h>
#include <cuda_bf16.h>

#include "rref_internal.cuh"
#include "tc_ptx.cuh"

namespace lnc {
namespace tc {

constexpr int BM = 128;                 // tile rows (TMEM lanes)
constexpr int BN = 32;                  // output columns per tile
constexpr int LIMBS = 4;                // base-256 digits per residue
constexpr int KMAX = 128;               // contraction depth (panel width)
constexpr int KC = 64;                  // K per stage: one 128-byte swizzle row of BF16
constexpr int NKC = KMAX / KC;          // 2
constexpr int GROUPS = 2 * LIMBS - 1;   // 7 weights 256^0 .. 256^6
constexpr int B_ROWS = LIMBS * BN;      // 128 stacked digit rows per output tile (UMMA N)
constexpr int STAGES = 4;
constexpr int TILES_PER_CTA = 16;
constexpr int EPI_WARPS = 8;            // two per TMEM lane quarter, 16 columns each
constexpr int THREADS = 64 + 32 * EPI_WARPS;
constexpr uint32_t TMEM_COLS = 512;
constexpr uint32_t ACC_STRIDE = 256;    // two accumulators of GROUPS * BN = 224 columns
constexpr uint32_t A_TILE_BYTES = BM * KC * 2;      // 16 KB
constexpr uint32_t B_TILE_BYTES = B_ROWS * KC * 2;  // 16 KB
constexpr uint32_t A_BYTES = LIMBS * NKC * A_TILE_BYTES;  // 128 KB
constexpr uint32_t SMEM_BYTES = A_BYTES + STAGES * B_TILE_BYTES + 1024 /*barriers*/ + 1024 /*align*/;
// exact float -> int for |x| < 2^22: x + 1.5 * 2^23 has unit spacing
constexpr float MAGIC_F = 12582912.0f;
constexpr int32_t MAGIC_I = 0x4B400000;

struct TcParams {
    uint32_t* C;            // trailing block base: A + j1
    int64_t ldc;
    int64_t m;
    int64_t N;
    int m_pad;              // rows per digit plane in the E operand
    int n_tiles;            // 64-column tiles covering N
    const int32_t* panel_k;
    FieldU32 f;
    int32_t w[GROUPS];      // 256^s mod p, centred
    uint64_t off;           // multiple of p >= 2^59 (makes the 64-bit sum non-negative)
    int overwrite;          // 1: C <- E * B (C is not read), 0: C <- C + E * B
    uint32_t pinv;          // -p^-1 mod 2^32 (Montgomery reduction of the epilogue sum)
    int* err;
    int* status;
};

__device__ __forceinline__ void split_digits(uint32_t x, uint32_t p, uint32_t half, __nv_bfloat16 (&d)[LIMBS]) {
    int32_t v = (x > half) ? (int32_t)((int64_t)x - (int64_t)p) : (int32_t)x;
#pragma unroll
    for (int i = 0; i < LIMBS - 1; ++i) {
        const int32_t di = ((v + 128) & 255) - 128;
        d[i] = __float2bfloat16_rn((float)di);
        v = (v - di) >> 8;
    }
    d[LIMBS - 1] = __float2bfloat16_rn((float)v);  // |v| <= 128
}

// E (m x ldE residues, columns >= k are zero) -> four K-major digit planes of
// m_pad x 128 BF16.
__global__ void split_e_kernel(const uint32_t* E, int64_t ldE, int b, int64_t m, int m_pad, uint32_t p,
                               const int32_t* panel_k, __nv_bfloat16* EL) {
    const int k = *panel_k;
    if (k == 0) return;
    const uint32_t half = p >> 1;
    const size_t plane = (size_t)m_pad * KMAX;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < (int64_t)m_pad * KMAX;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = idx / KMAX;
        const int t = (int)(idx - r * KMAX);
        uint32_t x = (r < m && t < k && t < b) ? E[r * ldE + t] : 0u;
        __nv_bfloat16 d[LIMBS];
        split_digits(x, p, half, d);
#pragma unroll
        for (int i = 0; i < LIMBS; ++i) EL[i * plane + idx] = d[i];
    }
}

// Pivot rows of the trailing block -> stacked digit rows (one CTA per 64-column
// tile), zeroing those rows in C.
__global__ void __launch_bounds__(256) gather_split_b_kernel(uint32_t* C, int64_t ldc, int64_t N,
                                                             const int32_t* panel_rows, const int32_t* panel_k,
                                                             uint32_t p, __nv_bfloat16* BS, int zero_src) {
    __shared__ uint32_t s[KMAX][BN + 1];
    const int k = *panel_k;
    if (k == 0) return;
    const int tile = blockIdx.x;
    const int64_t c0 = (int64_t)tile * BN;
    const uint32_t half = p >> 1;
    for (int idx = threadIdx.x; idx < KMAX * BN; idx += blockDim.x) {
        const int t = idx / BN, cc = idx % BN;
        uint32_t v = 0;
        if (t < k && c0 + cc < N) {
            uint32_t* src = C + (int64_t)(panel_rows ? panel_rows[t] : t) * ldc + c0 + cc;
            v = *src;
            if (zero_src) *src = 0u;
        }
        s[t][cc] = v;
    }
    __syncthreads();
    // row (i, cc) of this tile's stacked block holds digit i of column cc for t = 0..127
    __nv_bfloat16* dst = BS + (size_t)tile * B_ROWS * KMAX;
    for (int idx = threadIdx.x; idx < BN * KMAX; idx += blockDim.x) {
        const int cc = idx / KMAX, t = idx % KMAX;
        __nv_bfloat16 d[LIMBS];
        split_digits(s[t][cc], p, half, d);
#pragma unroll
        for (int i = 0; i < LIMBS; ++i) dst[((size_t)i * BN + cc) * KMAX + t] = d[i];
    }
}

__device__ __forceinline__ void flag_error(const TcParams& P, volatile int* cta_err) {
    *cta_err = 1;
    atomicExch(P.err, LNC_ERR_TIMEOUT);
    atomicExch(P.status, LNC_ERR_TIMEOUT);
}

// v mod p for the epilogue sum v < 2^60: Montgomery (v 2^-32; the weights
// already carry the factor 2^32) when 2^30 <= p < 2^31, else Barrett.
template <bool REDC>
__device__ __forceinline__ uint32_t reduce_sum(const FieldU32& f, uint32_t pinv, uint64_t v) {
    if constexpr (REDC) {
        const uint32_t lo = (uint32_t)v;
        const uint32_t u = (uint32_t)(v >> 32) + __umulhi(lo * pinv, f.p) + (lo != 0u ? 1u : 0u);  // < 2p
        return min(u, u - f.p);
    } else {
        return f.reduce64(v);
    }
}

// REDC: 2^30 <= p < 2^31, the weights carry an extra factor 2^32 and the
// 64-bit sum is reduced by one Montgomery step; otherwise Barrett.
template <bool REDC>
__global__ void __launch_bounds__(THREADS, 1)
    limb_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                     const TcParams P) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // 1024-byte alignment for the 128-byte swizzle atoms
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char* sA = smem;                         // [LIMBS][NKC][BM x KC]
    unsigned char* sB = smem + A_BYTES;               // [STAGES][B_ROWS x KC]
    uint64_t* bars = (uint64_t*)(sB + STAGES * B_TILE_BYTES);
    uint64_t* a_full = bars + 0;
    uint64_t* b_full = bars + 1;                  // [STAGES]
    uint64_t* b_empty = bars + 1 + STAGES;        // [STAGES]
    uint64_t* acc_full = bars + 1 + 2 * STAGES;   // [2]
    uint64_t* acc_empty = bars + 3 + 2 * STAGES;  // [2]
    uint64_t* drain = bars + 5 + 2 * STAGES;
    uint32_t* s_tmem = (uint32_t*)(bars + 6 + 2 * STAGES);
    __shared__ volatile int s_err;

    const int k = *P.panel_k;  // written by an earlier kernel: identical in every thread
    if (k == 0) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int rb = blockIdx.y;
    const int t0 = blockIdx.x * TILES_PER_CTA;
    const int t1 = min(P.n_tiles, t0 + TILES_PER_CTA);
    const int ntiles = t1 - t0;
    const int nkc = (k > KC) ? 2 : 1;  // skip the second K chunk when it is all zero

    if (threadIdx.x == 0) {
        s_err = (ld_volatile_i32(P.err) != 0) ? 1 : 0;  // an earlier kernel of this call failed
        ptx::mbar_init(a_full, 1);
        for (int s = 0; s < STAGES; ++s) {
            ptx::mbar_init(&b_full[s], 1);
            ptx::mbar_init(&b_empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            ptx::mbar_init(&acc_full[b], 1);
            ptx::mbar_init(&acc_empty[b], EPI_WARPS);
        }
        ptx::mbar_init(drain, 1);
        ptx::fence_mbar_init();
    }
    if (warp == 1) {
        ptx::tmem_alloc(s_tmem, TMEM_COLS);
        ptx::tmem_relinquish();
    }
    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    const uint32_t tmem = *s_tmem;

    if (warp == 0) {
        // ------------------------------------------------------------ producer
        if (lane == 0) {
            ptx::prefetch_tmap(&tmA);
            ptx::prefetch_tmap(&tmB);
            ptx::mbar_expect_tx(a_full, LIMBS * nkc * A_TILE_BYTES);
            for (int i = 0; i < LIMBS; ++i)
                for (int kc = 0; kc < nkc; ++kc)
                    ptx::tma_load_2d(sA + (i * NKC + kc) * A_TILE_BYTES, &tmA, a_full, kc * KC,
                                     i * P.m_pad + rb * BM);
            int it = 0;
            int issued_round[STAGES];
            for (int st = 0; st < STAGES; ++st) issued_round[st] = -1;
            for (int t = 0; t < ntiles && !s_err; ++t) {
                for (int kc = 0; kc < nkc; ++kc, ++it) {
                    const int st = it % STAGES, round = it / STAGES;
                    if (!ptx::mbar_wait(&b_empty[st], (round & 1) ^ 1, &s_err)) { flag_error(P, &s_err); break; }
                    ptx::mbar_expect_tx(&b_full[st], B_TILE_BYTES);
                    ptx::tma_load_2d(sB + st * B_TILE_BYTES, &tmB, &b_full[st], kc * KC, (t0 + t) * B_ROWS);
                    issued_round[st] = round;
                }
            }
            // never leave with copies in flight: wait (bounded) for every load issued
            const long long lim = kSpinLimitCycles / 4;
            ptx::mbar_wait_nocancel(a_full, 0, lim);
            for (int st = 0; st < STAGES; ++st)
                if (issued_round[st] >= 0) ptx::mbar_wait_nocancel(&b_full[st], issued_round[st] & 1, lim);
        }
    } else if (warp == 1) {
        // ------------------------------------------------------------ MMA issuer
        if (lane == 0) {
            constexpr uint32_t idesc = ptx::umma_idesc_bf16(BM, B_ROWS);
            const uint32_t a_base = ptx::smem_u32(sA);
            const uint32_t b_base = ptx::smem_u32(sB);
            bool ok = ptx::mbar_wait(a_full, 0, &s_err);
            if (!ok) flag_error(P, &s_err);
            int it = 0;
            for (int t = 0; t < ntiles && ok; ++t) {
                const int buf = t & 1;
                if (!ptx::mbar_wait(&acc_empty[buf], (t >> 1) & 1, &s_err)) { flag_error(P, &s_err); break; }
                ptx::tc_fence_after();
                const uint32_t dbase = tmem + ACC_STRIDE * buf;
                for (int kc = 0; kc < nkc && ok; ++kc, ++it) {
                    const int st = it % STAGES, round = it / STAGES;
                    if (!ptx::mbar_wait(&b_full[st], round & 1, &s_err)) { flag_error(P, &s_err); ok = false; break; }
                    ptx::tc_fence_after();
#pragma unroll
                    for (int ks = 0; ks < KC / 16; ++ks) {
                        const uint64_t bdesc = ptx::umma_desc_sw128(b_base + st * B_TILE_BYTES + ks * 32);
#pragma unroll
                        for (int i = 0; i < LIMBS; ++i) {
                            const uint64_t adesc =
                                ptx::umma_desc_sw128(a_base + (i * NKC + kc) * A_TILE_BYTES + ks * 32);
                            ptx::umma_bf16(dbase + (uint32_t)(BN * i), adesc, bdesc, idesc, 1u);
                        }
                    }
                    ptx::umma_commit(&b_empty[st]);  // stage reusable once these UMMAs finish
                }
                if (ok) ptx::umma_commit(&acc_full[buf]);
            }
            // all issued UMMAs complete before the TMEM is released
            ptx::umma_commit(drain);
            ptx::mbar_wait_nocancel(drain, 0, kSpinLimitCycles / 4);
        }
    } else {
        // ------------------------------------------------------------ epilogue
        const int ew = warp - 2;            // 0 .. EPI_WARPS-1
        const int q = warp & 3;             // TMEM lane quarter this warp may access
        const int half = ew >> 2;           // which 16 of the tile's 32 columns
        const int64_t row = (int64_t)rb * BM + q * 32 + lane;
        const uint32_t t_lane = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(16 * half);
        const FieldU32 f = P.f;
        const bool row_ok = row < P.m;
        // zero both accumulators (this warp's lanes and columns)
        for (int b = 0; b < 2; ++b) {
            for (int g = 0; g < GROUPS; ++g) ptx::tmem_st16_zero(t_lane + ACC_STRIDE * b + BN * g);
        }
        ptx::tmem_st_wait();
        ptx::tc_fence_before();
        __syncwarp();
        if (lane == 0) {
            ptx::mbar_arrive(&acc_empty[0]);
            ptx::mbar_arrive(&acc_empty[1]);
        }
        int64_t wsum = 0;  // sum of the weights: removes the magic offset in one step
#pragma unroll
        for (int g = 0; g < GROUPS; ++g) wsum += P.w[g];
        const uint64_t bias = P.off - (uint64_t)((int64_t)MAGIC_I * wsum);
        for (int t = 0; t < ntiles; ++t) {
            const int buf = t & 1;
            const int64_t col0 = (int64_t)(t0 + t) * BN + 16 * half;
            uint32_t* crow = P.C + (row_ok ? row : 0) * P.ldc + col0;
            const int ncols = (int)((P.N - col0) < 16 ? (P.N - col0) : 16);
            const bool vec = row_ok && ncols == 16 && ((((uintptr_t)crow) & 15) == 0);
            uint32_t old[16];
            if (P.overwrite) {
#pragma unroll
                for (int c = 0; c < 16; ++c) old[c] = 0u;
            } else if (vec) {
#pragma unroll
                for (int c = 0; c < 16; c += 4) {
                    const uint4 v = *(const uint4*)(crow + c);
                    old[c] = v.x; old[c + 1] = v.y; old[c + 2] = v.z; old[c + 3] = v.w;
                }
            } else {
#pragma unroll
                for (int c = 0; c < 16; ++c) old[c] = (row_ok && c < ncols) ? crow[c] : 0u;
            }
            const bool got = ptx::mbar_wait(&acc_full[buf], (t >> 1) & 1, &s_err);
            if (!__all_sync(0xffffffffu, got)) {  // warp-uniform before the aligned TMEM loads
                if (lane == 0) flag_error(P, &s_err);
                break;
            }
            ptx::tc_fence_after();
            uint32_t d[GROUPS][16];
#pragma unroll
            for (int g = 0; g < GROUPS; ++g) ptx::tmem_ld16(t_lane + ACC_STRIDE * buf + BN * g, d[g]);
            ptx::tmem_ld_wait();
            // accumulator drained: re-zero it and hand it back to the MMA warp
#pragma unroll
            for (int g = 0; g < GROUPS; ++g) ptx::tmem_st16_zero(t_lane + ACC_STRIDE * buf + BN * g);
            ptx::tmem_st_wait();
            ptx::tc_fence_before();
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(&acc_empty[buf]);
            // exact conversion: for |x| <= 2^22, x + 1.5 * 2^23 is exact and its bit pattern minus
            // 0x4B400000 is x (full-rate FADD instead of the quarter-rate F2I).  Groups 0, 1, 5, 6 hold
            // at most two digit products per step and stay within 2^22 for any input; groups 2-4 are
            // checked.  The weighted sum is formed modulo 2^64; its true value lies in [0, 2^60].
            float mx = 0.f;
#pragma unroll
            for (int g = 2; g <= 4; ++g)
#pragma unroll
                for (int c = 0; c < 16; ++c) mx = fmaxf(mx, fabsf(__uint_as_float(d[g][c])));
            const bool fast = mx <= 4194304.0f;
            uint32_t res[16];
            if (__all_sync(0xffffffffu, fast)) {
#pragma unroll
                for (int c = 0; c < 16; ++c) {
                    uint64_t v = (uint64_t)bias;
#pragma unroll
                    for (int g = 0; g < GROUPS; ++g) {
                        const int32_t y = (int32_t)__float_as_uint(__fadd_rn(__uint_as_float(d[g][c]), MAGIC_F));
                        v += (uint64_t)((int64_t)y * (int64_t)P.w[g]);
                    }
                    res[c] = f.add(old[c], reduce_sum<REDC>(f, P.pinv, v));
                }
            } else {
#pragma unroll
                for (int c = 0; c < 16; ++c) {
                    uint64_t v = P.off;
#pragma unroll
                    for (int g = 0; g < GROUPS; ++g)
                        v += (uint64_t)((int64_t)__float2int_rn(__uint_as_float(d[g][c])) * (int64_t)P.w[g]);
                    res[c] = f.add(old[c], reduce_sum<REDC>(f, P.pinv, v));
                }
            }
            if (vec) {
#pragma unroll
                for (int c = 0; c < 16; c += 4)
                    *(uint4*)(crow + c) = make_uint4(res[c], res[c + 1], res[c + 2], res[c + 3]);
            } else if (row_ok) {
#pragma unroll
                for (int c = 0; c < 16; ++c)
                    if (c < ncols) crow[c] = res[c];
            }
        }
    }
    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    if (warp == 1) ptx::tmem_dealloc(tmem, TMEM_COLS);
}

// ----------------------------------------------------------------------------
// host side
// ----------------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static std::mutex g_mu;
static EncodeTiledFn g_encode = nullptr;
static int g_avail = -1;

static EncodeTiledFn encode_fn() {
    std::lock_guard<std::mutex> g(g_mu);
    if (!g_encode) {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_encode = (EncodeTiledFn)fn;
        else
            cudaGetLastError();
    }
    return g_encode;
}

static int make_map(CUtensorMap* map, void* base, uint64_t inner, uint64_t outer, uint32_t box_inner,
                    uint32_t box_outer) {
    EncodeTiledFn enc = encode_fn();
    if (!enc) { set_error("cuTensorMapEncodeTiled is not available"); return LNC_ERR_UNSUPPORTED; }
    cuuint64_t dims[2] = {inner, outer};
    cuuint64_t strides[1] = {inner * 2};
    cuuint32_t box[2] = {box_inner, box_outer};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
        return LNC_ERR_CUDA;
    }
    return LNC_OK;
}

static int m_pad_of(int64_t m) { return (int)((m + BM - 1) / BM * BM); }
static int n_tiles_of(int64_t n) { return (int)((n + BN - 1) / BN); }

}  // namespace tc

bool trailing_tc_u32_available() {
    using namespace tc;
    if (g_avail >= 0) return g_avail == 1;
    int ok = 0;
    const char* env = getenv("LNC_DISABLE_TC");
    if (!(env && env[0] == '1')) {
        DeviceInfo di;
        if (device_info(&di) == LNC_OK && di.cc_major == 10 && di.smem_optin >= (int)SMEM_BYTES &&
            encode_fn() != nullptr)
            ok = 1;
    }
    g_avail = ok;
    return ok == 1;
}

size_t trailing_tc_u32_scratch(int64_t m, int64_t n, int /*b*/) {
    using namespace tc;
    return tc_el_bytes(m) + tc_bs_bytes(n) + 1024;
}

size_t tc_el_bytes(int64_t m) {
    using namespace tc;
    return ((size_t)LIMBS * m_pad_of(m) * KMAX * 2 + 1023) / 1024 * 1024;
}
size_t tc_bs_bytes(int64_t n) {
    using namespace tc;
    return ((size_t)n_tiles_of(n) * B_ROWS * KMAX * 2 + 1023) / 1024 * 1024;
}
int tc_m_pad(int64_t m) { return tc::m_pad_of(m); }

int tc_split_e(const uint32_t* E, int64_t ldE, int b, int64_t m, uint32_t p, const int32_t* k_ptr, void* EL,
               cudaStream_t s) {
    using namespace tc;
    const int m_pad = m_pad_of(m);
    const int64_t total = (int64_t)m_pad * KMAX;
    const int grid = (int)std::min<int64_t>((total + 255) / 256, 4096);
    split_e_kernel<<<grid, 256, 0, s>>>(E, ldE, b, m, m_pad, p, k_ptr, (__nv_bfloat16*)EL);
    LNC_CHECK_LAUNCH("split_e_kernel");
    return LNC_OK;
}

int tc_gather_split_b(uint32_t* C, int64_t ldc, int64_t N, const int32_t* rows, const int32_t* k_ptr, uint32_t p,
                      void* BS, bool zero_src, cudaStream_t s) {
    using namespace tc;
    gather_split_b_kernel<<<n_tiles_of(N), 256, 0, s>>>(C, ldc, N, rows, k_ptr, p, (__nv_bfloat16*)BS,
                                                        zero_src ? 1 : 0);
    LNC_CHECK_LAUNCH("gather_split_b_kernel");
    return LNC_OK;
}

int tc_limb_gemm(const FieldU32& f, uint32_t* C, int64_t ldc, int64_t m, int64_t N, const int32_t* k_ptr,
                 bool overwrite, const void* EL, const void* BS, int64_t n_map, int* err, int* status,
                 cudaStream_t s, bool count_work) {
    using namespace tc;
    const int m_pad = m_pad_of(m);
    const int n_tiles = n_tiles_of(N);
    CUtensorMap mapA, mapB;
    int rc = make_map(&mapA, const_cast<void*>(EL), KMAX, (uint64_t)LIMBS * m_pad, KC, BM);
    if (rc) return rc;
    rc = make_map(&mapB, const_cast<void*>(BS), KMAX, (uint64_t)n_tiles_of(n_map) * B_ROWS, KC, B_ROWS);
    if (rc) return rc;
    const uint32_t p = f.p;
    TcParams P;
    P.C = C;
    P.ldc = ldc;
    P.m = m;
    P.N = N;
    P.m_pad = m_pad;
    P.n_tiles = n_tiles;
    P.panel_k = k_ptr;
    P.f = f;
    const bool redc = (p & 1u) && p >= (1u << 30) && p < (1u << 31);
    uint64_t w = redc ? (((uint64_t)1 << 32) % p) : (1 % p);  // 2^32 folded in for the Montgomery step
    for (int sgrp = 0; sgrp < GROUPS; ++sgrp) {
        P.w[sgrp] = (w > p / 2) ? (int32_t)((int64_t)w - (int64_t)p) : (int32_t)w;
        w = (w * 256) % p;
    }
    P.off = ((((uint64_t)1 << 59) + p - 1) / p) * p;
    P.overwrite = overwrite ? 1 : 0;
    {
        uint32_t x = p;
        for (int i = 0; i < 5; ++i) x *= 2u - p * x;
        P.pinv = 0u - x;
    }
    P.err = err;
    P.status = status;
    auto kern = redc ? limb_gemm_kernel<true> : limb_gemm_kernel<false>;
    LNC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES));
    dim3 grid((unsigned)((n_tiles + TILES_PER_CTA - 1) / TILES_PER_CTA), (unsigned)(m_pad / BM));
    if (grid.y > 65535) { set_error("trailing update: too many row blocks"); return LNC_ERR_UNSUPPORTED; }
    ScopedKernelTimer kt(KC_TRAILING, s, count_work ? (double)m * (double)N * (double)KMAX : 0.0);
    kern<<<grid, THREADS, SMEM_BYTES, s>>>(mapA, mapB, P);
    LNC_CHECK_LAUNCH("limb_gemm_kernel");
    return LNC_OK;
}

int trailing_update_tc_u32(const TrailingCtx<FieldU32>& t, cudaStream_t s) {
    unsigned char* base = (unsigned char*)(((uintptr_t)t.extra + 1023) & ~(uintptr_t)1023);
    void* EL = base;
    void* BS = base + tc_el_bytes(t.m);
    const uint32_t p = t.f.p;
    int rc = tc_split_e(t.E, t.ldE, t.b, t.m, p, t.panel_k, EL, s);
    if (rc) return rc;
    rc = tc_gather_split_b(t.A + t.j1, t.lda, t.N, t.panel_rows, t.panel_k, p, BS, true, s);
    if (rc) return rc;
    return tc_limb_gemm(t.f, t.A + t.j1, t.lda, t.m, t.N, t.panel_k, false, EL, BS, t.n, t.err, t.status, s,
                        !t.predicated);
}

}  // namespace lnc
