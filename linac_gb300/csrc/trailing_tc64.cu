// Tensor-core trailing update for 64-bit residues (host side of
// tc64_kernels.cuh): digit split of E, gather + digit split of the pivot rows
// (zeroed in A), and the limb GEMM  A[:, T] += E A[P, T] (mod p).
#include <cuda.h>

#include "tc64_kernels.cuh"

namespace lnc {

int tc_make_map_bf16(CUtensorMap* map, void* base, uint64_t inner, uint64_t outer, uint32_t box_inner,
                     uint32_t box_outer);

namespace {
int m_pad64(int64_t m) { return (int)((m + tc64::BM - 1) / tc64::BM * tc64::BM); }
int n_tiles64(int64_t n) { return (int)((n + tc64::BN - 1) / tc64::BN); }
size_t el64_bytes(int64_t m) { return ((size_t)tc64::LIMBS * m_pad64(m) * tc64::KMAX * 2 + 1023) / 1024 * 1024; }
size_t bs64_bytes(int64_t n) {
    return ((size_t)n_tiles64(n) * tc64::B_ROWS * tc64::KMAX * 2 + 1023) / 1024 * 1024;
}
}  // namespace

bool trailing_tc_u64_available() {
    DeviceInfo di;
    return trailing_tc_u32_available() && device_info(&di) == LNC_OK && di.smem_optin >= (int)tc64::SMEM_BYTES;
}

size_t trailing_tc_u64_scratch(int64_t m, int64_t n) { return el64_bytes(m) + bs64_bytes(n) + 1024; }

// ---- pieces shared by the trailing update and the candidate-panel path
int tc64_split_e(const uint64_t* E, int64_t ldE, int64_t m, uint64_t p, const int32_t* k_ptr, void* EL,
                 cudaStream_t s, int max_grid) {
    using namespace tc64;
    const int m_pad = m_pad64(m);
    const int grid = (int)std::min<int64_t>(((int64_t)m_pad * KMAX + 255) / 256, max_grid > 0 ? max_grid : 8192);
    split_e64_kernel<<<grid, 256, 0, s>>>(E, ldE, m, m_pad, p, k_ptr, (__nv_bfloat16*)EL);
    LNC_CHECK_LAUNCH("split_e64_kernel");
    return LNC_OK;
}

int tc64_split_g(const uint64_t* A, int64_t lda, int64_t m, int64_t j0, uint64_t p, const int32_t* k_ptr,
                 const int32_t* panel_cols, const int32_t* panel_mark, int gen, void* EL, cudaStream_t s) {
    using namespace tc64;
    const int m_pad = m_pad64(m);
    const int grid = (int)std::min<int64_t>(((int64_t)m_pad * KMAX + 255) / 256, 8192);
    split_g64_kernel<<<grid, 256, 0, s>>>(A, lda, m, m_pad, j0, p, k_ptr, panel_cols, panel_mark, gen,
                                          (__nv_bfloat16*)EL);
    LNC_CHECK_LAUNCH("split_g64_kernel");
    return LNC_OK;
}

int tc64_gather_split_b(uint64_t* C, int64_t ldc, int64_t N, const int32_t* rows, const int32_t* k_ptr, uint64_t p,
                        void* BS, bool zero_src, cudaStream_t s) {
    tc64::gather_split_b64_kernel<<<n_tiles64(N), 256, 0, s>>>(C, ldc, N, rows, k_ptr, p, (__nv_bfloat16*)BS,
                                                              zero_src ? 1 : 0);
    LNC_CHECK_LAUNCH("gather_split_b64_kernel");
    return LNC_OK;
}

int tc64_limb_gemm(const FieldU64& f, uint64_t* C, int64_t ldc, int64_t m, int64_t N, const int32_t* k_ptr,
                   bool overwrite, const void* EL, const void* BS, int* err, int* status, cudaStream_t s,
                   bool count_work, int kwork, int tiles_per_cta) {
    using namespace tc64;
    const uint64_t p = f.p;
    const int m_pad = m_pad64(m);
    const int n_tiles = n_tiles64(N);
    CUtensorMap mapA, mapB;
    int rc = tc_make_map_bf16(&mapA, const_cast<void*>(EL), KMAX, (uint64_t)LIMBS * m_pad, KC, BM);
    if (!rc) rc = tc_make_map_bf16(&mapB, const_cast<void*>(BS), KMAX, (uint64_t)n_tiles * B_ROWS, KC, B_ROWS);
    if (rc) return rc;
    Params64 P{};
    P.C = C;
    P.ldc = ldc;
    P.m = m;
    P.N = N;
    P.overwrite = overwrite ? 1 : 0;
    P.m_pad = m_pad;
    P.n_tiles = n_tiles;
    P.panel_k = k_ptr;
    P.f = f;
    {
        // w_s = 2^(8 s) 2^64 mod p (centred): one Montgomery step of the weighted sum gives sum y_s 2^(8 s)
        unsigned __int128 x = (((unsigned __int128)1) << 64) % p;
        for (int g = 0; g < GROUPS; ++g) {
            const uint64_t xv = (uint64_t)x;
            P.w[g] = (xv > p / 2) ? -(int64_t)(p - xv) : (int64_t)xv;
            x = (x * 256) % p;
        }
        const unsigned __int128 two91 = ((unsigned __int128)1) << 91;
        const unsigned __int128 off = ((two91 + p - 1) / p) * p;
        P.off_lo = (uint64_t)off;
        P.off_hi = (uint64_t)(off >> 64);
    }
    P.err = err;
    P.status = status;
    P.tpc = tiles_per_cta > 0 ? tiles_per_cta : limb_tiles_per_cta(n_tiles, m_pad / BM);
    LNC_CUDA(cudaFuncSetAttribute(limb64_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES));
    dim3 grid((unsigned)((n_tiles + P.tpc - 1) / P.tpc), (unsigned)(m_pad / BM));
    if (grid.y > 65535) { set_error("trailing update: too many row blocks"); return LNC_ERR_UNSUPPORTED; }
    ScopedKernelTimer kt(KC_TRAILING, s, count_work ? (double)m * (double)N * (double)kwork : 0.0);
    limb64_gemm_kernel<<<grid, THREADS, SMEM_BYTES, s>>>(mapA, mapB, P);
    LNC_CHECK_LAUNCH("limb64_gemm_kernel");
    return LNC_OK;
}

int trailing_update_tc_u64(const TrailingCtx<FieldU64>& t, cudaStream_t s) {
    using namespace tc64;
    if (t.b > KMAX) { set_error("64-bit tensor-core update needs panels of at most %d columns", KMAX); return LNC_ERR_INVALID; }
    unsigned char* base = (unsigned char*)(((uintptr_t)t.extra + 1023) & ~(uintptr_t)1023);
    void* EL = base;
    void* BS = base + el64_bytes(t.m);
    // a predicated update (a fallback that usually finds nothing) launches few CTAs, one per row
    // block for the contraction: they read the pivot count and exit
    int rc = tc64_split_e(t.E, t.ldE, t.m, t.f.p, t.panel_k, EL, s, t.predicated ? 152 : 0);
    if (!rc) rc = tc64_gather_split_b(t.A + t.j1, t.lda, t.N, t.panel_rows, t.panel_k, t.f.p, BS, true, s);
    if (!rc) rc = tc64_limb_gemm(t.f, t.A + t.j1, t.lda, t.m, t.N, t.panel_k, false, EL, BS, t.err, t.status, s,
                                 !t.predicated, t.b, t.predicated ? (1 << 20) : 0);
    return rc;
}

size_t tc64_el_bytes(int64_t m) { return el64_bytes(m); }
size_t tc64_bs_bytes(int64_t n) { return bs64_bytes(n); }

void* tc64_bs_base(void* extra, int64_t m) {
    unsigned char* base = (unsigned char*)(((uintptr_t)extra + 1023) & ~(uintptr_t)1023);
    return base + el64_bytes(m);
}

}  // namespace lnc
