// Tensor-core limb GEMM kernels (device code shared by trailing_tc.cu and
// batch.cu).  See trailing_tc.cu for the method.
#pragma once

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
// epilogue kinds: residues mod p (Barrett or one Montgomery step), or the
// fixed-point contraction of the float path (real, or complex realified with
// GEMM rows 2r / 2r + 1 the real / imaginary parts of output row r)
constexpr int EPI_BARRETT = 0, EPI_REDC = 1, EPI_F64 = 2, EPI_C128 = 3;
// exact float -> int for |x| < 2^22: x + 1.5 * 2^23 has unit spacing
constexpr float MAGIC_F = 12582912.0f;
constexpr int32_t MAGIC_I = 0x4B400000;

// What one CTA of the limb GEMM computes: rows [rb*128, rb*128+128) and
// 32-column tiles [t0, t1) of  C (+)= E * B  for one matrix.
struct LimbJob {
    uint32_t* C;
    int64_t ldc, m, N;
    int rb, t0, t1;
    int a_row0, a_plane;  // digit plane i of E, row r: tensor row a_row0 + i * a_plane + r
    int b_row0;           // tile t of B: tensor rows b_row0 + t * B_ROWS ...
    int k;                // contraction depth actually used (pivots of the panel)
    int overwrite;
    int redc;
    FieldU32 f;
    uint32_t pinv;
    const int32_t* w;
    uint64_t off;
    int* err;
    int* status;
    // float epilogue: C is double (Cd, ldc in elements of the output type),
    // value = sum of digit products * rscale[row] * cscale[column]
    double* Cd;
    const double* rscale;
    const double* cscale;
};

// Epilogue constants of the limb contraction for a prime p < 2^32 (host side).
// The epilogue forms v = off + sum_s D_s w_s (w_s = 256^s R mod p, centred,
// so |w_s| <= p / 2) in 64-bit arithmetic and reduces it mod p.
//  * odd p < 2^31: R = 2^32 mod p and one Montgomery step (v 2^-32 mod p),
//    valid for 0 <= v < 2^32 p.  The digit-group sums (paired or not) weigh
//    at most 2.52 * 2^30 in magnitude in total, so |sum| <= 1.26 * 2^30 p and
//    off = 1.5 * 2^30 p keeps v inside [0.24, 2.76] * 2^30 p;
//  * p = 2 and 2^31 <= p < 2^32: R = 1 and Barrett; |sum| < 1.26 * 2^61 and
//    off is the first multiple of p at or above 2^62.
struct LimbConstants {
    int redc;
    int32_t w[GROUPS];
    uint64_t off;
    uint32_t pinv;  // -p^-1 mod 2^32
};
static inline LimbConstants limb_constants(uint32_t p) {
    LimbConstants c;
    c.redc = ((p & 1u) && p < (1u << 31)) ? 1 : 0;
    uint64_t w = c.redc ? (((uint64_t)1 << 32) % p) : (1 % p);
    for (int g = 0; g < GROUPS; ++g) {
        c.w[g] = (w > p / 2) ? (int32_t)((int64_t)w - (int64_t)p) : (int32_t)w;
        w = (w * 256) % p;
    }
    c.off = c.redc ? (((uint64_t)p * 3) << 29) : (((((uint64_t)1 << 62) + p - 1) / p) * p);
    uint32_t x = p;
    for (int i = 0; i < 5; ++i) x *= 2u - p * x;
    c.pinv = 0u - x;
    return c;
}

struct TcParams {
    uint32_t* C;            // trailing block base: A + j1
    int64_t ldc;
    int64_t m;
    int64_t N;
    int m_pad;              // rows per digit plane in the E operand
    int n_tiles;            // 64-column tiles covering N
    const int32_t* panel_k;
    FieldU32 f;
    int32_t w[GROUPS];      // 256^s R mod p, centred (limb_constants)
    uint64_t off;           // multiple of p keeping the 64-bit epilogue sum in range (limb_constants)
    int overwrite;          // 1: C <- E * B (C is not read), 0: C <- C + E * B
    uint32_t pinv;          // -p^-1 mod 2^32 (Montgomery reduction of the epilogue sum)
    int redc;
    int* err;
    int* status;
    double* Cd;             // float epilogue (see LimbJob)
    const double* rscale;
    const double* cscale;
    int tpc = TILES_PER_CTA;  // 32-column tiles per CTA (grid.x covers n_tiles / tpc)
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
__device__ __forceinline__ void split_e_body(const uint32_t* E, int64_t ldE, int b, int64_t m, int m_pad,
                                             uint32_t p, const int32_t* panel_k, __nv_bfloat16* EL) {
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

static __global__ void split_e_kernel(const uint32_t* E, int64_t ldE, int b, int64_t m, int m_pad, uint32_t p,
                                      const int32_t* panel_k, __nv_bfloat16* EL) {
    split_e_body(E, ldE, b, m, m_pad, p, panel_k, EL);
}

// Pivot rows of the trailing block -> stacked digit rows (one 256-thread CTA
// per 32-column tile), zeroing those rows in C.  Warp w reads rows w, w + 8,
// ... (128 contiguous bytes each); all 16 loads of a thread are issued before
// any is used, so a tile costs about one memory round trip.
__device__ __forceinline__ void gather_split_b_body(int tile, uint32_t* C, int64_t ldc, int64_t N,
                                                    const int32_t* panel_rows, const int32_t* panel_k, uint32_t p,
                                                    __nv_bfloat16* BS, int zero_src) {
    constexpr int RPW = KMAX / 8;  // rows per warp (8 warps)
    __shared__ uint32_t s[KMAX][BN + 1];
    const int k = *panel_k;
    if (k == 0) return;
    const int64_t c0 = (int64_t)tile * BN;
    const uint32_t half = p >> 1;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool col_ok = c0 + lane < N;
    uint32_t* base = C + c0 + lane;
    // row indices staged in shared memory: the loads of C below then depend
    // on nothing the stores to C could alias
    __shared__ int s_rows[KMAX];
    if (threadIdx.x < KMAX)
        s_rows[threadIdx.x] = ((int)threadIdx.x < k) ? (panel_rows ? panel_rows[threadIdx.x] : (int)threadIdx.x) : -1;
    __syncthreads();
    uint32_t v[RPW];
#pragma unroll
    for (int r = 0; r < RPW; ++r) {
        const int row = s_rows[w + 8 * r];
        v[r] = (row >= 0 && col_ok) ? base[(int64_t)row * ldc] : 0u;
    }
#pragma unroll
    for (int r = 0; r < RPW; ++r) s[w + 8 * r][lane] = v[r];
    __syncthreads();
    // the rows are zeroed only after every load has returned (a store right behind a load of the
    // same address holds the thread until that load completes, serialising the 16 round trips)
    if (zero_src) {
#pragma unroll
        for (int r = 0; r < RPW; ++r) {
            const int row = s_rows[w + 8 * r];
            if (row >= 0 && col_ok) base[(int64_t)row * ldc] = 0u;
        }
    }
    // row (i, cc) of this tile's stacked block holds digit i of column cc for t = 0..127
    // (two consecutive t per thread: 4-byte stores, 128 contiguous bytes per warp)
    __nv_bfloat16* dst = BS + (size_t)tile * B_ROWS * KMAX;
    for (int idx = threadIdx.x; idx < BN * KMAX / 2; idx += blockDim.x) {
        const int cc = idx / (KMAX / 2), t = 2 * (idx % (KMAX / 2));
        __nv_bfloat16 d0[LIMBS], d1[LIMBS];
        split_digits(s[t][cc], p, half, d0);
        split_digits(s[t + 1][cc], p, half, d1);
#pragma unroll
        for (int i = 0; i < LIMBS; ++i)
            *reinterpret_cast<__nv_bfloat162*>(dst + ((size_t)i * BN + cc) * KMAX + t) = __halves2bfloat162(d0[i], d1[i]);
    }
}

static __global__ void __launch_bounds__(256, 6) gather_split_b_kernel(uint32_t* C, int64_t ldc, int64_t N,
                                                                    const int32_t* panel_rows,
                                                                    const int32_t* panel_k, uint32_t p,
                                                                    __nv_bfloat16* BS, int zero_src) {
    gather_split_b_body(blockIdx.x, C, ldc, N, panel_rows, panel_k, p, BS, zero_src);
}

__device__ __forceinline__ void flag_error(const LimbJob& P, volatile int* cta_err) {
    *cta_err = 1;
    atomicExch(P.err, LNC_ERR_TIMEOUT);
    atomicExch(P.status, LNC_ERR_TIMEOUT);
}

// v mod p for the epilogue sum: Montgomery (v 2^-32, valid for 0 <= v < 2^32
// p; the weights already carry the factor 2^32) for odd p < 2^31, else
// Barrett (any 64-bit v).  Montgomery: with m = v pinv mod 2^32, v + m p is a
// multiple of 2^32 below 2^33 p <= 2^64, and (v + m p) / 2^32 < 2p.
template <bool REDC>
__device__ __forceinline__ uint32_t reduce_sum(const FieldU32& f, uint32_t pinv, uint64_t v) {
    if (REDC) {
        const uint32_t m = (uint32_t)v * pinv;
        const uint32_t u = (uint32_t)(((uint64_t)m * f.p + v) >> 32);  // < 2p
        return min(u, u - f.p);
    } else {
        return f.reduce64(v);
    }
}
// old + r mod p for residues old, r < p (p < 2^31 when REDC: no 64-bit sum)
template <bool REDC>
__device__ __forceinline__ uint32_t add_residue(const FieldU32& f, uint32_t old, uint32_t r) {
    if (REDC) {
        const uint32_t s = old + r;
        return min(s, s - f.p);
    } else {
        return f.add(old, r);
    }
}

// One CTA of the limb GEMM (see the file comment).  REDC (J.redc): odd p <
// 2^31, the weights carry an extra factor 2^32 and the 64-bit digit sum is
// reduced by one Montgomery step; otherwise Barrett (limb_constants).
// Exact value of the digit-product sum of one output element (float
// epilogue): the seven group sums are integers below 2^24 in magnitude, so
// hi (groups 3..6) and lo (groups 0..2) are exact in int64 and the result
// hi * 2^24 + lo is rounded once.
__device__ __forceinline__ double fx_digit_value(const int32_t (&y)[GROUPS]) {
    const int64_t hi = (int64_t)y[3] + ((int64_t)y[4] << 8) + ((int64_t)y[5] << 16) + ((int64_t)y[6] << 24);
    const int64_t lo = (int64_t)y[0] + ((int64_t)y[1] << 8) + ((int64_t)y[2] << 16);
    return fma((double)hi, 16777216.0, (double)lo);
}

// mbarrier wait of the producer / MMA warp: warp-uniform by a vote when the whole warp runs the loop
template <bool WIDE>
__device__ __forceinline__ bool issuer_wait(uint64_t* bar, uint32_t parity, volatile int* cta_err) {
    const bool got = ptx::mbar_wait(bar, parity, cta_err);
    return WIDE ? __all_sync(0xffffffffu, got) : got;
}

template <int EPI>
__device__ __forceinline__ void limb_cta(const LimbJob& P, const CUtensorMap* tmA, const CUtensorMap* tmB) {
    constexpr bool REDC = EPI == EPI_REDC;
    constexpr bool WIDE = EPI != EPI_BARRETT;  // producer / MMA loops run by the whole warp
    constexpr bool FLOAT = EPI == EPI_F64 || EPI == EPI_C128;
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

    const int k = P.k;
    if (k == 0 || P.t1 <= P.t0) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int rb = P.rb;
    const int t0 = P.t0;
    const int ntiles = P.t1 - P.t0;
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

    if (warp == 0 && (WIDE || lane == 0)) {
        // ------------------------------------------------------------ producer
        // warp-wide loop (WIDE), the elected lane issues the copies (as for the MMA issuer)
        const bool leader = WIDE ? ptx::elect_one() : true;
        if (leader) {
            ptx::prefetch_tmap(tmA);
            ptx::prefetch_tmap(tmB);
            ptx::mbar_expect_tx(a_full, LIMBS * nkc * A_TILE_BYTES);
            for (int i = 0; i < LIMBS; ++i)
                for (int kc = 0; kc < nkc; ++kc)
                    ptx::tma_load_2d(sA + (i * NKC + kc) * A_TILE_BYTES, tmA, a_full, kc * KC,
                                     P.a_row0 + i * P.a_plane + rb * BM);
        }
        int it = 0;
        int issued_round[STAGES];
        for (int st = 0; st < STAGES; ++st) issued_round[st] = -1;
        bool go = true;
        for (int t = 0; t < ntiles && go; ++t) {
            if (WIDE ? __any_sync(0xffffffffu, s_err != 0) : (s_err != 0)) break;
            for (int kc = 0; kc < nkc; ++kc, ++it) {
                const int st = it % STAGES, round = it / STAGES;
                if (!issuer_wait<WIDE>(&b_empty[st], (round & 1) ^ 1, &s_err)) {
                    if (leader) flag_error(P, &s_err);
                    go = false;
                    break;
                }
                if (leader) {
                    ptx::mbar_expect_tx(&b_full[st], B_TILE_BYTES);
                    ptx::tma_load_2d(sB + st * B_TILE_BYTES, tmB, &b_full[st], kc * KC, P.b_row0 + (t0 + t) * B_ROWS);
                }
                issued_round[st] = round;
                if (WIDE) __syncwarp();
            }
        }
        // never leave with copies in flight: wait (bounded) for every load issued
        if (leader) {
            const long long lim = kSpinLimitCycles / 4;
            ptx::mbar_wait_nocancel(a_full, 0, lim);
            for (int st = 0; st < STAGES; ++st)
                if (issued_round[st] >= 0) ptx::mbar_wait_nocancel(&b_full[st], issued_round[st] & 1, lim);
        }
        if (WIDE) __syncwarp();
    } else if (warp == 1 && (WIDE || lane == 0)) {
        // ------------------------------------------------------------ MMA issuer
        // WIDE: the whole warp runs the loop, so the descriptor arithmetic stays warp-uniform; the
        // elected lane issues the UMMAs and their commits, and every wait is decided by a warp vote
        // (without it, integer work on this SM sub-partition slows the UMMA stream).  The Barrett
        // epilogue, whose heavier combine bounds the kernel, runs faster with lane 0 alone.
        const bool leader = WIDE ? ptx::elect_one() : true;
        constexpr uint32_t idesc = ptx::umma_idesc_bf16(BM, B_ROWS);
        // descriptors of the ring / plane bases; a K step or a stage moves only the start-address
        // field (address / 16, 14 bits: shared-memory offsets never carry out of it)
        const uint64_t adesc0 = ptx::umma_desc_sw128(ptx::smem_u32(sA));
        const uint64_t bdesc0 = ptx::umma_desc_sw128(ptx::smem_u32(sB));
        bool ok = issuer_wait<WIDE>(a_full, 0, &s_err);
        if (!ok && leader) flag_error(P, &s_err);
        int it = 0;
        for (int t = 0; t < ntiles && ok; ++t) {
            const int buf = t & 1;
            if (!issuer_wait<WIDE>(&acc_empty[buf], (t >> 1) & 1, &s_err)) {
                if (leader) flag_error(P, &s_err);
                break;
            }
            ptx::tc_fence_after();
            const uint32_t dbase = tmem + ACC_STRIDE * buf;
            for (int kc = 0; kc < nkc && ok; ++kc, ++it) {
                const int st = it % STAGES, round = it / STAGES;
                if (!issuer_wait<WIDE>(&b_full[st], round & 1, &s_err)) {
                    if (leader) flag_error(P, &s_err);
                    ok = false;
                    break;
                }
                ptx::tc_fence_after();
#pragma unroll
                for (int ks = 0; ks < KC / 16; ++ks) {
                    const uint64_t bdesc = bdesc0 + (uint64_t)((st * B_TILE_BYTES + ks * 32) >> 4);
#pragma unroll
                    for (int i = 0; i < LIMBS; ++i) {
                        const uint64_t adesc = adesc0 + (uint64_t)(((i * NKC + kc) * A_TILE_BYTES + ks * 32) >> 4);
                        if (leader) ptx::umma_bf16(dbase + (uint32_t)(BN * i), adesc, bdesc, idesc, 1u);
                    }
                }
                if (leader) ptx::umma_commit(&b_empty[st]);  // stage reusable once these UMMAs finish
                if (WIDE) __syncwarp();
            }
            if (ok && leader) ptx::umma_commit(&acc_full[buf]);
            if (WIDE) __syncwarp();
        }
        // all issued UMMAs complete before the TMEM is released
        if (leader) {
            ptx::umma_commit(drain);
            ptx::mbar_wait_nocancel(drain, 0, kSpinLimitCycles / 4);
        }
        if (WIDE) __syncwarp();
    } else if (warp >= 2) {
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
        int32_t w[GROUPS];  // weights in registers (P.w may alias nothing, but the compiler cannot tell)
#pragma unroll
        for (int g = 0; g < GROUPS; ++g) w[g] = FLOAT ? 0 : P.w[g];
        // integer fast path: groups (0, 1), (2, 3) and (5, 6) are paired before weighting,
        // z = y_g + 256 y_{g+1} (w_{g+1} = 256 w_g mod p), from one shift-add of their conversion bits;
        // the first group of a pair is converted negated (sign bit set), which leaves z + KPAIR in
        // int32 range
        constexpr int32_t KPAIR = 0x0B400000;  // (257 * MAGIC_I + 2^31) mod 2^32
        const uint64_t bias3 = P.off - (uint64_t)((int64_t)KPAIR * ((int64_t)w[0] + w[2] + w[5])) -
                               (uint64_t)((int64_t)MAGIC_I * (int64_t)w[4]);
        if constexpr (FLOAT) {
            // output element (row, col): F64 -> Cd[row * ldc + col];  C128 -> part (row & 1) of
            // Cd[(row >> 1) * ldc + col] (complex elements, viewed as pairs of doubles)
            const int64_t orow = (EPI == EPI_C128) ? (row >> 1) : row;
            const int64_t estride = (EPI == EPI_C128) ? 2 : 1;
            double* cbase = P.Cd + ((row_ok ? orow : 0) * P.ldc) * estride + ((EPI == EPI_C128) ? (row & 1) : 0);
            const double rs = row_ok ? P.rscale[row] : 0.0;
            for (int t = 0; t < ntiles; ++t) {
                const int buf = t & 1;
                const int64_t col0 = (int64_t)(t0 + t) * BN + 16 * half;
                const int ncols = (int)((P.N - col0) < 16 ? (P.N - col0) : 16);
                double* crow = cbase + col0 * estride;
                double old[16], cs[16];
#pragma unroll
                for (int c = 0; c < 16; ++c) {
                    const bool ok = row_ok && c < ncols;
                    old[c] = (ok && !P.overwrite) ? crow[c * estride] : 0.0;
                    cs[c] = (c < ncols) ? P.cscale[col0 + c] : 0.0;
                }
                const bool got = ptx::mbar_wait(&acc_full[buf], (t >> 1) & 1, &s_err);
                if (!__all_sync(0xffffffffu, got)) {
                    if (lane == 0) flag_error(P, &s_err);
                    break;
                }
                ptx::tc_fence_after();
                uint32_t d[GROUPS][16];
#pragma unroll
                for (int g = 0; g < GROUPS; ++g) ptx::tmem_ld16(t_lane + ACC_STRIDE * buf + BN * g, d[g]);
                ptx::tmem_ld_wait();
#pragma unroll
                for (int g = 0; g < GROUPS; ++g) ptx::tmem_st16_zero(t_lane + ACC_STRIDE * buf + BN * g);
                ptx::tmem_st_wait();
                ptx::tc_fence_before();
                __syncwarp();
                if (lane == 0) ptx::mbar_arrive(&acc_empty[buf]);
                // group sums are exact integers: magic-number conversion where |x| <= 2^22
                // (groups 0, 1, 5, 6 always; 2-4 checked), F2I otherwise
                float mx = 0.f;
#pragma unroll
                for (int g = 2; g <= 4; ++g)
#pragma unroll
                    for (int c = 0; c < 16; ++c) mx = fmaxf(mx, fabsf(__uint_as_float(d[g][c])));
                const bool fast = __all_sync(0xffffffffu, mx <= 4194304.0f);
                // one conversion or the other for the whole warp (a uniform branch, not a select per group)
                if (fast) {
#pragma unroll
                    for (int c = 0; c < 16; ++c) {
                        int32_t y[GROUPS];
#pragma unroll
                        for (int g = 0; g < GROUPS; ++g)
                            y[g] = (int32_t)__float_as_uint(__fadd_rn(__uint_as_float(d[g][c]), MAGIC_F)) - MAGIC_I;
                        const double v = fx_digit_value(y);
                        if (row_ok && c < ncols) crow[c * estride] = old[c] + (v * rs) * cs[c];
                    }
                } else {
#pragma unroll
                    for (int c = 0; c < 16; ++c) {
                        int32_t y[GROUPS];
#pragma unroll
                        for (int g = 0; g < GROUPS; ++g) y[g] = __float2int_rn(__uint_as_float(d[g][c]));
                        const double v = fx_digit_value(y);
                        if (row_ok && c < ncols) crow[c * estride] = old[c] + (v * rs) * cs[c];
                    }
                }
            }
        } else {
            // C's old values are loaded one tile ahead, so their memory latency overlaps the
            // previous tile's combine instead of stalling the accumulator hand-back
            auto tile_at = [&](int t, uint32_t*& crow, int& ncols, bool& vec) {
                const int64_t col0 = (int64_t)(t0 + t) * BN + 16 * half;
                crow = P.C + (row_ok ? row : 0) * P.ldc + col0;
                ncols = (int)((P.N - col0) < 16 ? (P.N - col0) : 16);
                vec = row_ok && ncols == 16 && ((((uintptr_t)crow) & 15) == 0);
            };
            auto load_old = [&](int t, uint32_t (&o)[16]) {
                uint32_t* crow;
                int ncols;
                bool vec;
                tile_at(t, crow, ncols, vec);
                if (P.overwrite) {
#pragma unroll
                    for (int c = 0; c < 16; ++c) o[c] = 0u;
                } else if (vec) {
#pragma unroll
                    for (int c = 0; c < 16; c += 4) {
                        const uint4 v = *(const uint4*)(crow + c);
                        o[c] = v.x; o[c + 1] = v.y; o[c + 2] = v.z; o[c + 3] = v.w;
                    }
                } else {
#pragma unroll
                    for (int c = 0; c < 16; ++c) o[c] = (row_ok && c < ncols) ? crow[c] : 0u;
                }
            };
            uint32_t oldn[16];
            if (ntiles > 0) load_old(0, oldn);
            for (int t = 0; t < ntiles; ++t) {
                const int buf = t & 1;
                uint32_t* crow;
                int ncols;
                bool vec;
                tile_at(t, crow, ncols, vec);
                uint32_t old[16];
#pragma unroll
                for (int c = 0; c < 16; ++c) old[c] = oldn[c];
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
                if (t + 1 < ntiles) load_old(t + 1, oldn);
                // exact conversion: for |x| <= 2^22, x + 1.5 * 2^23 is exact and its bit pattern minus
                // 0x4B400000 is x (full-rate FADD instead of the quarter-rate F2I).  Digits 0-2 lie in
                // [-128, 127] and the top digit in [-64, 64] for p < 2^31 ([-128, 128] otherwise), so
                // groups 0, 1, 5, 6 stay within 2^22 for any input, group 4 too for p < 2^31; groups
                // 2, 3 (and 4 for p >= 2^31) are checked.  The weighted sum is formed modulo 2^64.
                float mx = 0.f;
#pragma unroll
                for (int g = 2; g <= (REDC ? 3 : 4); ++g)
#pragma unroll
                    for (int c = 0; c < 16; ++c) mx = fmaxf(mx, fabsf(__uint_as_float(d[g][c])));
                const bool fast = mx <= 4194304.0f;
                if (__all_sync(0xffffffffu, fast)) {
                    // |y_0|, |y_6| <= 2^21, |y_1|, |y_5| <= 2^22, |y_2|, |y_3|, |y_4| <= 2^22 here:
                    // |z_01|, |z_23| <= 2^30 + 2^22, |z_56| <= 2^29 + 2^22; four 64-bit multiply-adds
#pragma unroll
                    for (int c = 0; c < 16; ++c) {
                        const uint32_t b0n = __float_as_uint(__fadd_rn(-__uint_as_float(d[0][c]), -MAGIC_F));
                        const uint32_t b1 = __float_as_uint(__fadd_rn(__uint_as_float(d[1][c]), MAGIC_F));
                        const uint32_t b2n = __float_as_uint(__fadd_rn(-__uint_as_float(d[2][c]), -MAGIC_F));
                        const uint32_t b3 = __float_as_uint(__fadd_rn(__uint_as_float(d[3][c]), MAGIC_F));
                        const int32_t b4 = (int32_t)__float_as_uint(__fadd_rn(__uint_as_float(d[4][c]), MAGIC_F));
                        const uint32_t b5n = __float_as_uint(__fadd_rn(-__uint_as_float(d[5][c]), -MAGIC_F));
                        const uint32_t b6 = __float_as_uint(__fadd_rn(__uint_as_float(d[6][c]), MAGIC_F));
                        const int32_t z01 = (int32_t)((b1 << 8) + b0n);  // z_01 + KPAIR
                        const int32_t z23 = (int32_t)((b3 << 8) + b2n);  // z_23 + KPAIR
                        const int32_t z56 = (int32_t)((b6 << 8) + b5n);  // z_56 + KPAIR
                        uint64_t v = bias3 + (uint64_t)((int64_t)z01 * (int64_t)w[0]);
                        v += (uint64_t)((int64_t)z23 * (int64_t)w[2]);
                        v += (uint64_t)((int64_t)b4 * (int64_t)w[4]);  // y_4 + MAGIC_I
                        v += (uint64_t)((int64_t)z56 * (int64_t)w[5]);
                        old[c] = add_residue<REDC>(f, old[c], reduce_sum<REDC>(f, P.pinv, v));
                    }
                } else {
#pragma unroll
                    for (int c = 0; c < 16; ++c) {
                        uint64_t v = P.off;
#pragma unroll
                        for (int g = 0; g < GROUPS; ++g)
                            v += (uint64_t)((int64_t)__float2int_rn(__uint_as_float(d[g][c])) * (int64_t)w[g]);
                        old[c] = add_residue<REDC>(f, old[c], reduce_sum<REDC>(f, P.pinv, v));
                    }
                }
                if (vec) {
#pragma unroll
                    for (int c = 0; c < 16; c += 4)
                        *(uint4*)(crow + c) = make_uint4(old[c], old[c + 1], old[c + 2], old[c + 3]);
                } else if (row_ok) {
#pragma unroll
                    for (int c = 0; c < 16; ++c)
                        if (c < ncols) crow[c] = old[c];
                }
            }
        }
    }
    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    if (warp == 1) ptx::tmem_dealloc(tmem, TMEM_COLS);
}

template <int EPI>
static __global__ void __launch_bounds__(THREADS, 1)
    limb_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                     const __grid_constant__ TcParams P) {
    LimbJob J;
    J.C = P.C;
    J.ldc = P.ldc;
    J.m = P.m;
    J.N = P.N;
    J.rb = blockIdx.y;
    J.t0 = blockIdx.x * P.tpc;
    J.t1 = min(P.n_tiles, J.t0 + P.tpc);
    J.a_row0 = 0;
    J.a_plane = P.m_pad;
    J.b_row0 = 0;
    J.k = *P.panel_k;  // written by an earlier kernel: identical in every thread
    J.overwrite = P.overwrite;
    J.redc = P.redc;
    J.f = P.f;
    J.pinv = P.pinv;
    J.w = P.w;
    J.off = P.off;
    J.err = P.err;
    J.status = P.status;
    J.Cd = P.Cd;
    J.rscale = P.rscale;
    J.cscale = P.cscale;
    limb_cta<EPI>(J, &tmA, &tmB);
}

}  // namespace tc
}  // namespace lnc
