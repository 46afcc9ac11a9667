// Tensor-core limb GEMM for 64-bit residues (device code of trailing_tc64.cu).
//
// Same scheme as the 32-bit kernel (tc_kernels.cuh), sized for residues below
// 2^64: a centred residue (|v| < 2^63) is split into eight balanced base-256
// digits in [-128, 128], exact in BF16.  The panel is 64 columns wide (K = 64),
// so every digit-group sum (at most 8 digit pairs x 2^14 x 64 = 2^23) is an
// integer exact in FP32.  One UMMA  M=128, N=128, K=16  multiplies a digit
// plane of E by the eight stacked digit planes of a 16-column tile of B, so
// A_i B_j lands in accumulator columns 16(i+j) .. 16(i+j)+15: 15 weight groups
// s = i + j, two accumulators of 240 columns in TMEM.  The epilogue forms
// T = sum_s y_s w_s with w_s = 2^(8 s) 2^64 mod p (centred), |T| < 2^91,
// exactly in 128 bits, adds a multiple of p to make it non-negative and
// reduces it with one Montgomery step (T < p 2^64 since p > 2^32):
// sum_s y_s 2^(8 s) mod p.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>

#include "rref_internal.cuh"
#include "tc_ptx.cuh"

namespace lnc {
namespace tc64 {

constexpr int BM = 128;                 // tile rows (TMEM lanes)
constexpr int BN = 16;                  // output columns per tile
constexpr int LIMBS = 8;                // base-256 digits per residue
constexpr int KMAX = 64;                // contraction depth (panel width)
constexpr int KC = 64;                  // one 128-byte swizzle row of BF16
constexpr int GROUPS = 2 * LIMBS - 1;   // 15 weights
constexpr int B_ROWS = LIMBS * BN;      // 128 stacked digit rows per tile (UMMA N)
constexpr int STAGES = 4;
constexpr int TILES_PER_CTA = 16;
constexpr int EPI_WARPS = 8;            // two per TMEM lane quarter, 8 columns each
constexpr int THREADS = 64 + 32 * EPI_WARPS;
constexpr uint32_t TMEM_COLS = 512;
constexpr uint32_t ACC_STRIDE = 256;    // two accumulators of GROUPS * BN = 240 columns
constexpr uint32_t A_TILE_BYTES = BM * KC * 2;      // 16 KB
constexpr uint32_t B_TILE_BYTES = B_ROWS * KC * 2;  // 16 KB
constexpr uint32_t A_BYTES = LIMBS * A_TILE_BYTES;  // 128 KB
constexpr uint32_t SMEM_BYTES = A_BYTES + STAGES * B_TILE_BYTES + 1024 + 1024;
constexpr float MAGIC_F = 12582912.0f;  // exact float -> int for |x| <= 2^22
constexpr int32_t MAGIC_I = 0x4B400000;

struct Params64 {
    uint64_t* C;            // trailing block base: A + j1
    int64_t ldc, m, N;
    int overwrite;          // 1: C <- E B (C is not read), 0: C <- C + E B
    int m_pad;              // rows per digit plane of E
    int n_tiles;            // 16-column tiles covering N
    const int32_t* panel_k;
    FieldU64 f;
    int64_t w[GROUPS];      // 2^(8 s) 2^64 mod p, centred
    uint64_t off_lo, off_hi;  // multiple of p >= 2^91 (makes the sum non-negative)
    int* err;
    int* status;
    int tpc = TILES_PER_CTA;  // 16-column tiles per CTA (grid.x covers n_tiles / tpc)
};

__device__ __forceinline__ void split_digits64(uint64_t x, uint64_t p, __nv_bfloat16 (&d)[LIMBS]) {
    int64_t v = (x > (p >> 1)) ? (int64_t)(x - p) : (int64_t)x;  // |v| < 2^63
#pragma unroll
    for (int i = 0; i < LIMBS - 1; ++i) {
        // v = 256 q + r, 0 <= r < 256: digit r (r < 128) or r - 256 with a carry into q
        // (no intermediate leaves int64, also for |v| near 2^63)
        const int r = (int)(v & 255);
        const int di = r < 128 ? r : r - 256;
        d[i] = __float2bfloat16_rn((float)di);
        v = (v >> 8) + (r < 128 ? 0 : 1);
    }
    d[LIMBS - 1] = __float2bfloat16_rn((float)v);  // |v| <= 128
}

// E (m x ldE residues, first k columns) -> eight K-major digit planes of m_pad x 64
static __global__ void __launch_bounds__(256) split_e64_kernel(const uint64_t* E, int64_t ldE, int64_t m, int m_pad,
                                                               uint64_t p, const int32_t* panel_k,
                                                               __nv_bfloat16* EL) {
    const int k = *panel_k;
    if (k == 0) return;
    const size_t plane = (size_t)m_pad * KMAX;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < (int64_t)m_pad * KMAX;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = idx / KMAX;
        const int t = (int)(idx - r * KMAX);
        const uint64_t x = (r < m && t < k) ? E[r * ldE + t] : 0ull;
        __nv_bfloat16 d[LIMBS];
        split_digits64(x, p, d);
#pragma unroll
        for (int i = 0; i < LIMBS; ++i) EL[i * plane + idx] = d[i];
    }
}

// G operand of E = G X for the candidate panel: G[o, t] = -A[o, j0 + cols[t]]
// for rows that are not pivot rows of this panel, G[prow_t, :] = e_t; eight
// K-major digit planes of m_pad x 64
static __global__ void __launch_bounds__(256) split_g64_kernel(const uint64_t* A, int64_t lda, int64_t m, int m_pad,
                                                               int64_t j0, uint64_t p, const int32_t* panel_k,
                                                               const int32_t* panel_cols, const int32_t* panel_mark,
                                                               int gen, __nv_bfloat16* EL) {
    const int k = *panel_k;
    if (k == 0) return;
    const size_t plane = (size_t)m_pad * KMAX;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < (int64_t)m_pad * KMAX;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = idx / KMAX;
        const int t = (int)(idx - r * KMAX);
        uint64_t v = 0;
        if (r < m && t < k) {
            const int mk = panel_mark[r];
            if ((mk >> 8) == gen) {
                v = ((mk & 255) - 1 == t) ? 1ull : 0ull;
            } else {
                const uint64_t x = A[r * lda + j0 + panel_cols[t]];
                v = x ? p - x : 0ull;
            }
        }
        __nv_bfloat16 d[LIMBS];
        split_digits64(v, p, d);
#pragma unroll
        for (int i = 0; i < LIMBS; ++i) EL[i * plane + idx] = d[i];
    }
}

// pivot rows of the trailing block (zeroed in C) -> stacked digit tiles of B,
// one CTA per 16-column tile
// (rows == nullptr: rows 0 .. k-1; zero_src: zero the gathered rows in C)
static __global__ void __launch_bounds__(256) gather_split_b64_kernel(uint64_t* C, int64_t ldc, int64_t N,
                                                                      const int32_t* rows, const int32_t* panel_k,
                                                                      uint64_t p, __nv_bfloat16* BS, int zero_src) {
    __shared__ uint64_t s[KMAX][BN + 1];
    const int k = *panel_k;
    if (k == 0) return;
    const int64_t c0 = (int64_t)blockIdx.x * BN;
    constexpr int PER = KMAX * BN / 256;  // entries per thread (blockDim.x == 256)
    uint64_t v[PER];
#pragma unroll
    for (int j = 0; j < PER; ++j) {  // every load issued before any is used
        const int idx = threadIdx.x + 256 * j;
        const int t = idx / BN, cc = idx % BN;
        v[j] = (t < k && c0 + cc < N) ? C[(int64_t)(rows ? rows[t] : t) * ldc + c0 + cc] : 0ull;
    }
#pragma unroll
    for (int j = 0; j < PER; ++j) {
        const int idx = threadIdx.x + 256 * j;
        s[idx / BN][idx % BN] = v[j];
    }
    __syncthreads();
    if (zero_src) {  // after the loads have returned
#pragma unroll
        for (int j = 0; j < PER; ++j) {
            const int idx = threadIdx.x + 256 * j;
            const int t = idx / BN, cc = idx % BN;
            if (t < k && c0 + cc < N) C[(int64_t)(rows ? rows[t] : t) * ldc + c0 + cc] = 0ull;
        }
    }
    __nv_bfloat16* dst = BS + (size_t)blockIdx.x * B_ROWS * KMAX;
    for (int idx = threadIdx.x; idx < BN * KMAX; idx += blockDim.x) {
        const int cc = idx / KMAX, t = idx % KMAX;
        __nv_bfloat16 d[LIMBS];
        split_digits64(s[t][cc], p, d);
#pragma unroll
        for (int i = 0; i < LIMBS; ++i) dst[((size_t)i * BN + cc) * KMAX + t] = d[i];
    }
}

__device__ __forceinline__ void flag_error64(const Params64& P, volatile int* cta_err) {
    *cta_err = 1;
    atomicExch(P.err, LNC_ERR_TIMEOUT);
    atomicExch(P.status, LNC_ERR_TIMEOUT);
}

// C[rows of block blockIdx.y, tiles [blockIdx.x * TILES_PER_CTA, ...)] += E B (mod p)
// One output column's group sums: b_g = y_g + 0x4B400000 (the bit pattern of the magic-number
// conversion, or F2I plus the same constant) times the low and high 32-bit halves of w_g, added
// modulo 2^64 to the start values a0, a1.
template <bool FAST>
__device__ __forceinline__ void group_sums(const uint32_t (&d)[GROUPS][8], int c, const Params64& P, uint64_t& a0,
                                           uint64_t& a1) {
#pragma unroll
    for (int g = 0; g < GROUPS; ++g) {
        const uint32_t b = FAST ? __float_as_uint(__fadd_rn(__uint_as_float(d[g][c]), MAGIC_F))
                                : (uint32_t)(__float2int_rn(__uint_as_float(d[g][c])) + MAGIC_I);
        a0 += (uint64_t)b * (uint32_t)P.w[g];
        a1 += (uint64_t)((int64_t)b * (int64_t)(int32_t)(P.w[g] >> 32));
    }
}

static __global__ void __launch_bounds__(THREADS, 1)
    limb64_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                       const __grid_constant__ Params64 P) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char* sA = smem;                         // [LIMBS][BM x KC]
    unsigned char* sB = smem + A_BYTES;               // [STAGES][B_ROWS x KC]
    uint64_t* bars = (uint64_t*)(sB + STAGES * B_TILE_BYTES);
    uint64_t* a_full = bars + 0;
    uint64_t* b_full = bars + 1;
    uint64_t* b_empty = bars + 1 + STAGES;
    uint64_t* acc_full = bars + 1 + 2 * STAGES;
    uint64_t* acc_empty = bars + 3 + 2 * STAGES;
    uint64_t* drain = bars + 5 + 2 * STAGES;
    uint32_t* s_tmem = (uint32_t*)(bars + 6 + 2 * STAGES);
    __shared__ volatile int s_err;

    const int k = *P.panel_k;  // written by an earlier kernel: identical in every thread
    const int rb = blockIdx.y;
    const int t0 = blockIdx.x * P.tpc;
    const int t1 = min(P.n_tiles, t0 + P.tpc);
    if (k == 0 || t1 <= t0) return;
    const int ntiles = t1 - t0;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        s_err = (ld_volatile_i32(P.err) != 0) ? 1 : 0;
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
        // warp-wide loops, elected lanes issue (see elect_one in tc_ptx.cuh)
        const bool leader = ptx::elect_one();
        if (leader) {
            ptx::prefetch_tmap(&tmA);
            ptx::prefetch_tmap(&tmB);
            ptx::mbar_expect_tx(a_full, LIMBS * A_TILE_BYTES);
            for (int i = 0; i < LIMBS; ++i)
                ptx::tma_load_2d(sA + i * A_TILE_BYTES, &tmA, a_full, 0, i * P.m_pad + rb * BM);
        }
        int issued_round[STAGES];
        for (int st = 0; st < STAGES; ++st) issued_round[st] = -1;
        for (int t = 0; t < ntiles; ++t) {
            if (__any_sync(0xffffffffu, s_err != 0)) break;
            const int st = t % STAGES, round = t / STAGES;
            if (!__all_sync(0xffffffffu, ptx::mbar_wait(&b_empty[st], (round & 1) ^ 1, &s_err))) {
                if (leader) flag_error64(P, &s_err);
                break;
            }
            if (leader) {
                ptx::mbar_expect_tx(&b_full[st], B_TILE_BYTES);
                ptx::tma_load_2d(sB + st * B_TILE_BYTES, &tmB, &b_full[st], 0, (t0 + t) * B_ROWS);
            }
            issued_round[st] = round;
            __syncwarp();
        }
        if (leader) {
            const long long lim = kSpinLimitCycles / 4;
            ptx::mbar_wait_nocancel(a_full, 0, lim);
            for (int st = 0; st < STAGES; ++st)
                if (issued_round[st] >= 0) ptx::mbar_wait_nocancel(&b_full[st], issued_round[st] & 1, lim);
        }
        __syncwarp();
    } else if (warp == 1) {
        // ------------------------------------------------------------ MMA issuer
        const bool leader = ptx::elect_one();
        constexpr uint32_t idesc = ptx::umma_idesc_bf16(BM, B_ROWS);
        const uint64_t adesc0 = ptx::umma_desc_sw128(ptx::smem_u32(sA));  // K steps move the address field
        const uint64_t bdesc0 = ptx::umma_desc_sw128(ptx::smem_u32(sB));
        bool ok = __all_sync(0xffffffffu, ptx::mbar_wait(a_full, 0, &s_err));
        if (!ok && leader) flag_error64(P, &s_err);
        const int ksteps = (k + 15) / 16;  // K steps beyond k are all zero (and skipped)
        for (int t = 0; t < ntiles && ok; ++t) {
            const int buf = t & 1;
            const int st = t % STAGES, round = t / STAGES;
            if (!__all_sync(0xffffffffu, ptx::mbar_wait(&acc_empty[buf], (t >> 1) & 1, &s_err)) ||
                !__all_sync(0xffffffffu, ptx::mbar_wait(&b_full[st], round & 1, &s_err))) {
                if (leader) flag_error64(P, &s_err);
                break;
            }
            ptx::tc_fence_after();
            const uint32_t dbase = tmem + ACC_STRIDE * buf;
            for (int ks = 0; ks < ksteps; ++ks) {
                const uint64_t bdesc = bdesc0 + (uint64_t)((st * B_TILE_BYTES + ks * 32) >> 4);
#pragma unroll
                for (int i = 0; i < LIMBS; ++i) {
                    const uint64_t adesc = adesc0 + (uint64_t)((i * A_TILE_BYTES + ks * 32) >> 4);
                    if (leader) ptx::umma_bf16(dbase + (uint32_t)(BN * i), adesc, bdesc, idesc, 1u);
                }
            }
            if (leader) {
                ptx::umma_commit(&b_empty[st]);
                ptx::umma_commit(&acc_full[buf]);
            }
            __syncwarp();
        }
        if (leader) {
            ptx::umma_commit(drain);
            ptx::mbar_wait_nocancel(drain, 0, kSpinLimitCycles / 4);
        }
        __syncwarp();
    } else {
        // ------------------------------------------------------------ epilogue
        const int ew = warp - 2;
        const int q = warp & 3;             // TMEM lane quarter this warp may access
        const int half = ew >> 2;           // which 8 of the tile's 16 columns
        const int64_t row = (int64_t)rb * BM + q * 32 + lane;
        const uint32_t t_lane = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(8 * half);
        const FieldU64 f = P.f;
        const bool row_ok = row < P.m;
        // zero both accumulators (this warp's lanes and columns): the digit planes' UMMAs
        // overlap in the accumulator, so every one of them accumulates
        for (int b = 0; b < 2; ++b)
            for (int g = 0; g < GROUPS; ++g) ptx::tmem_st8_zero(t_lane + ACC_STRIDE * b + BN * g);
        ptx::tmem_st_wait();
        ptx::tc_fence_before();
        __syncwarp();
        if (lane == 0) {
            ptx::mbar_arrive(&acc_empty[0]);
            ptx::mbar_arrive(&acc_empty[1]);
        }
        // w_s = wh_s 2^32 + wl_s (wl_s unsigned): T = off + A0 + A1 2^32 with A0 = sum_s y_s wl_s and
        // A1 = sum_s y_s wh_s, both below 2^59 in magnitude.  The groups enter as b_s = y_s + 0x4B400000
        // (the bit pattern of the magic-number conversion); the sums of b_s wl_s and b_s wh_s are formed
        // modulo 2^64 from starting values -0x4B400000 sum wl and -0x4B400000 sum wh, which leaves A0
        // and A1 exactly (as signed 64-bit values) at the end.
        // (the weights stay in the kernel's parameter space: operands of the multiply-adds, no registers)
        uint64_t swl = 0, swh = 0;
#pragma unroll
        for (int g = 0; g < GROUPS; ++g) {
            swl += (uint32_t)P.w[g];
            swh += (uint64_t)(int64_t)(int32_t)(P.w[g] >> 32);
        }
        const uint64_t a0_init = 0ull - (uint64_t)MAGIC_I * swl;
        const uint64_t a1_init = 0ull - (uint64_t)MAGIC_I * swh;
        for (int t = 0; t < ntiles; ++t) {
            const int buf = t & 1;
            const int64_t col0 = (int64_t)(t0 + t) * BN + 8 * half;
            uint64_t* crow = P.C + (row_ok ? row : 0) * P.ldc + col0;
            const int ncols = (int)((P.N - col0) < 8 ? (P.N - col0) : 8);
            const bool vec = row_ok && ncols == 8 && ((((uintptr_t)crow) & 15) == 0);
            uint64_t old[8];
            if (P.overwrite) {
#pragma unroll
                for (int c = 0; c < 8; ++c) old[c] = 0ull;
            } else if (vec) {
#pragma unroll
                for (int c = 0; c < 8; c += 2) {
                    const ulonglong2 v = *(const ulonglong2*)(crow + c);
                    old[c] = v.x;
                    old[c + 1] = v.y;
                }
            } else {
#pragma unroll
                for (int c = 0; c < 8; ++c) old[c] = (row_ok && c < ncols) ? crow[c] : 0ull;
            }
            const bool got = ptx::mbar_wait(&acc_full[buf], (t >> 1) & 1, &s_err);
            if (!__all_sync(0xffffffffu, got)) {
                if (lane == 0) flag_error64(P, &s_err);
                break;
            }
            ptx::tc_fence_after();
            uint32_t d[GROUPS][8];
#pragma unroll
            for (int g = 0; g < GROUPS; ++g) ptx::tmem_ld8(t_lane + ACC_STRIDE * buf + BN * g, d[g]);
            ptx::tmem_ld_wait();
#pragma unroll
            for (int g = 0; g < GROUPS; ++g) ptx::tmem_st8_zero(t_lane + ACC_STRIDE * buf + BN * g);
            ptx::tmem_st_wait();
            ptx::tc_fence_before();
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(&acc_empty[buf]);
            // groups 0-3 and 11-14 sum at most four digit products per K step (<= 2^22 for K = 64):
            // the magic-number conversion is exact for them; groups 4-10 are checked
            float mx = 0.f;
#pragma unroll
            for (int g = 4; g <= 10; ++g)
#pragma unroll
                for (int c = 0; c < 8; ++c) mx = fmaxf(mx, fabsf(__uint_as_float(d[g][c])));
            const bool fast = __all_sync(0xffffffffu, mx <= 4194304.0f);
            // the rest of an output column once its two partial sums are formed (modulo 2^64)
            auto finish = [&](int c, uint64_t a0, uint64_t a1) {
                const unsigned __int128 T = (((unsigned __int128)P.off_hi << 64) | P.off_lo) +
                                            (unsigned __int128)((__int128)(int64_t)a0 + ((__int128)(int64_t)a1 << 32));
                old[c] = f.add(old[c], f.redc((uint64_t)T, (uint64_t)(T >> 64)));
                if (c & 1) {  // store each finished pair of columns
                    if (vec) {
                        *(ulonglong2*)(crow + c - 1) = make_ulonglong2(old[c - 1], old[c]);
                    } else if (row_ok) {
                        if (c - 1 < ncols) crow[c - 1] = old[c - 1];
                        if (c < ncols) crow[c] = old[c];
                    }
                }
            };
            // one conversion or the other for the whole warp (a uniform branch, not a select per group)
            if (fast) {
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    uint64_t a0 = a0_init, a1 = a1_init;
                    group_sums<true>(d, c, P, a0, a1);
                    finish(c, a0, a1);
                }
            } else {
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    uint64_t a0 = a0_init, a1 = a1_init;
                    group_sums<false>(d, c, P, a0, a1);
                    finish(c, a0, a1);
                }
            }
        }
    }
    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    if (warp == 1) ptx::tmem_dealloc(tmem, TMEM_COLS);
}

}  // namespace tc64
}  // namespace lnc
