// Exact F_p trailing update on the tcgen05 tensor cores (32-bit residues).
//
//   C[:, T] <- C[:, T] + E * B   (mod p),  E: m x K transform, B: K x N pivot rows
//
// The reference has no counterpart for this step: linac eliminates one column
// at a time with a 64-bit `%` per element (linac/row_reduce.cu:107-114,
// 138-196).  Here the whole panel (K = 128 pivots) is applied in one
// contraction, exactly, on the BF16 tensor cores:
//
//  * every residue x (centred to (-p/2, p/2]) is split into four balanced
//    base-256 digits x = sum_i d_i 256^i, |d_i| <= 128; integers of that size
//    are exact in BF16;
//  * a digit product is at most 2^14 in magnitude, and the products that
//    share a weight 256^s (s = i + j) summed over K = 128 stay below 2^23, so
//    every FP32 accumulation in TMEM is an exact integer;
//  * the epilogue converts the seven group sums D_s to integers (x + 1.5 2^23
//    where |x| <= 2^22, F2I otherwise), forms sum_s D_s (256^s mod p) in
//    64-bit (groups (0, 1), (2, 3) and (5, 6) paired first by a shift-add), reduces
//    it mod p (one Montgomery step for odd p < 2^31, the weights carrying the
//    factor 2^32; Barrett otherwise) and adds it to the old residue.
//
// Layout: the four E digit planes are K-major (row = matrix row, 128 digits),
// the B digits are stacked per 32-column output tile as 4 x 32 K-major rows, so
// one UMMA (M = 128, N = 128, K = 16) multiplies digit plane i of E with all
// four digit planes of B and lands in TMEM columns [32 i, 32 i + 128): the
// column block s = i + j accumulates exactly the weight-256^s products.
//
// Kernel (tc_kernels.cuh): one CTA per 128-row block and a run of consecutive
// 32-column tiles (chosen to fill whole waves of the GPU); warp 0 issues the
// TMA loads (E digits once, B digits through a 4-stage ring), warp 1 issues
// the UMMAs (each warp runs its loop as a whole, one elected lane issuing)
// and owns the TMEM allocation (two accumulators of 7 x 32 columns,
// so the epilogue of one tile overlaps the UMMAs of the next), warps 2-9
// (two per TMEM lane quarter, 16 columns each) drain TMEM, re-zero it,
// combine and write C.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>
#include <algorithm>

#include <cuda.h>
#include <cuda_bf16.h>

#include "tc_kernels.cuh"

namespace lnc {
namespace tc {
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

}  // namespace tc

int tc_make_map_bf16(CUtensorMap* map, void* base, uint64_t inner, uint64_t outer, uint32_t box_inner,
                     uint32_t box_outer) {
    return tc::make_map(map, base, inner, outer, box_inner, box_outer);
}

namespace tc {

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

int limb_tiles_per_cta(int n_tiles, int row_blocks) {
    DeviceInfo di;
    const int sms = (device_info(&di) == LNC_OK && di.sms > 0) ? di.sms : 148;
    int best = 16;
    double best_cost = 1e300;
    for (int t = 4; t <= 48; ++t) {
        const long long ctas = (long long)row_blocks * ((n_tiles + t - 1) / t);
        const long long waves = (ctas + sms - 1) / sms;
        const double c = (double)waves * ((double)std::min(t, n_tiles) + 0.6);
        if (c < best_cost - 1e-9) {
            best_cost = c;
            best = t;
        }
    }
    return best;
}

int tc_split_e(const uint32_t* E, int64_t ldE, int b, int64_t m, uint32_t p, const int32_t* k_ptr, void* EL,
               cudaStream_t s, int max_grid) {
    using namespace tc;
    const int m_pad = m_pad_of(m);
    const int64_t total = (int64_t)m_pad * KMAX;
    const int grid = (int)std::min<int64_t>((total + 255) / 256, max_grid > 0 ? max_grid : 4096);
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
                 cudaStream_t s, bool count_work, int tiles_per_cta) {
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
    const LimbConstants lc = limb_constants(p);
    const bool redc = lc.redc != 0;
    for (int sgrp = 0; sgrp < GROUPS; ++sgrp) P.w[sgrp] = lc.w[sgrp];
    P.off = lc.off;
    P.overwrite = overwrite ? 1 : 0;
    P.pinv = lc.pinv;
    P.err = err;
    P.status = status;
    P.redc = redc ? 1 : 0;
    P.tpc = tiles_per_cta > 0 ? tiles_per_cta : limb_tiles_per_cta(n_tiles, m_pad / BM);
    auto kern = redc ? limb_gemm_kernel<EPI_REDC> : limb_gemm_kernel<EPI_BARRETT>;
    LNC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES));
    dim3 grid((unsigned)((n_tiles + P.tpc - 1) / P.tpc), (unsigned)(m_pad / BM));
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
    // a predicated update (a fallback that usually finds nothing) launches few CTAs, one per row
    // block for the contraction: they read the pivot count and exit
    int rc = tc_split_e(t.E, t.ldE, t.b, t.m, p, t.panel_k, EL, s, t.predicated ? 152 : 0);
    if (rc) return rc;
    rc = tc_gather_split_b(t.A + t.j1, t.lda, t.N, t.panel_rows, t.panel_k, p, BS, true, s);
    if (rc) return rc;
    return tc_limb_gemm(t.f, t.A + t.j1, t.lda, t.m, t.N, t.panel_k, false, EL, BS, t.n, t.err, t.status, s,
                        !t.predicated, t.predicated ? (1 << 20) : 0);
}

// C = A B mod p (32-bit residues, any sizes): the limb GEMM applied to
// 128-deep slices of the contraction, the first slice overwriting C.
int matmul_modp_u64(uint64_t p, int64_t m, int64_t k, int64_t n, const uint64_t* A, int64_t lda, const uint64_t* B,
                    int64_t ldb, uint64_t* C, int64_t ldc, cudaStream_t s);

int tc_matmul_modp(uint32_t p, int64_t m, int64_t k, int64_t n, const uint32_t* A, int64_t lda,
                   const uint32_t* B, int64_t ldb, uint32_t* C, int64_t ldc, cudaStream_t s) {
    using namespace tc;
    if (m <= 0 || n <= 0) return LNC_OK;
    if (k <= 0) {
        LNC_CUDA(cudaMemset2DAsync(C, 4 * ldc, 0, 4 * n, m, s));
        return LNC_OK;
    }
    if (!trailing_tc_u32_available()) { set_error("tensor-core path unavailable"); return LNC_ERR_UNSUPPORTED; }
    const FieldU32 f = FieldU32::make(p);
    const int64_t chunks = (k + KMAX - 1) / KMAX;
    const size_t el = tc_el_bytes(m), bs = tc_bs_bytes(n);
    void* scratch = nullptr;
    cudaError_t e = cudaMallocAsync(&scratch, el + bs + 1024 + 256 + sizeof(int32_t) * chunks + 16, s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("matmul scratch: %s", cudaGetErrorString(e));
        return LNC_ERR_OOM;
    }
    unsigned char* base = (unsigned char*)(((uintptr_t)scratch + 1023) & ~(uintptr_t)1023);
    void* EL = base;
    void* BS = base + el;
    int32_t* ks = (int32_t*)(base + el + bs);
    int* words = (int*)(ks + chunks);
    std::vector<int32_t> hk((size_t)chunks);
    for (int64_t c = 0; c < chunks; ++c) hk[(size_t)c] = (int32_t)std::min<int64_t>(KMAX, k - c * KMAX);
    int rc = LNC_OK;
    e = cudaMemcpyAsync(ks, hk.data(), sizeof(int32_t) * chunks, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(words, 0, 8, s);
    if (e != cudaSuccess) rc = cuda_status(e, "matmul setup");
    if (!rc) e = cudaStreamSynchronize(s);  // the chunk sizes live in pageable host memory
    for (int64_t c = 0; c < chunks && !rc; ++c) {
        rc = tc_split_e(A + c * KMAX, lda, KMAX, m, p, ks + c, EL, s);
        if (!rc) rc = tc_gather_split_b(const_cast<uint32_t*>(B) + c * KMAX * ldb, ldb, n, nullptr, ks + c, p, BS,
                                        false, s);
        if (!rc) rc = tc_limb_gemm(f, C, ldc, m, n, ks + c, c == 0, EL, BS, n, words, words + 1, s);
    }
    cudaFreeAsync(scratch, s);
    return rc;
}

}  // namespace lnc

extern "C" int lnc_matmul_modp_device(int dtype, int64_t m, int64_t k, int64_t n, uint64_t p, const void* A,
                                      int64_t lda, const void* B, int64_t ldb, void* C, int64_t ldc, void* stream) {
    using namespace lnc;
    if (m < 0 || k < 0 || n < 0) { set_error("matmul: negative shape"); return LNC_ERR_INVALID; }
    if (lda < k || ldb < n || ldc < n) { set_error("matmul: leading dimension too small"); return LNC_ERR_INVALID; }
    if (dtype == LNC_U64) {
        if (k == 0) {
            if (m > 0 && n > 0) LNC_CUDA(cudaMemset2DAsync(C, 8 * ldc, 0, 8 * n, m, (cudaStream_t)stream));
            return LNC_OK;
        }
        return matmul_modp_u64(p, m, k, n, (const uint64_t*)A, lda, (const uint64_t*)B, ldb, (uint64_t*)C, ldc,
                               (cudaStream_t)stream);
    }
    if (dtype != LNC_U32) { set_error("matmul: LNC_U32 or LNC_U64"); return LNC_ERR_UNSUPPORTED; }
    if (p < 2 || p > 0xFFFFFFFFull) { set_error("matmul: 2 <= p < 2^32"); return LNC_ERR_INVALID; }
    return tc_matmul_modp((uint32_t)p, m, k, n, (const uint32_t*)A, lda, (const uint32_t*)B, ldb, (uint32_t*)C, ldc,
                          (cudaStream_t)stream);
}
