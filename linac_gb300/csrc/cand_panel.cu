// Fast F_p panel: Gauss-Jordan on a candidate block in one CTA.
//
// Over a field any non-zero entry is a valid pivot and the RREF is unique, so
// the pivots of a 128-column panel need not be searched over all m rows at
// once (the grid-wide search of panel_kernel costs one grid barrier per
// column).  This kernel takes the first `smax` (<= 256) rows that are not yet
// pivot rows, loads their panel block into shared memory and runs Gauss-Jordan
// on it in one CTA (barriers are __syncthreads only), choosing in each column
// the first candidate row with a non-zero entry.  Eliminated pivot columns keep
// the transform in place, so the block's pivot rows end with
//     X = A[P, Q]^-1        (k x k, in their pivot columns).
// The panel is then applied to every row by two tensor-core contractions (see
// rref.cu, rref_run_u32_fast):  E = G X  with G_o = -A[o, Q] (G = e_t for pivot
// row t), and  A[:, j0:] += E A[P, j0:]  with the pivot rows zeroed first.
//
// If the block missed a pivot (a panel column whose only non-zero entries lie
// in rows outside the block), the check kernel below finds a non-zero entry in
// a non-pivot panel column of a remaining row after the update, and the driver
// re-runs that panel with the exhaustive grid-wide panel kernel; results are
// exact either way.
//
// Field arithmetic: Montgomery multiplication with R = 2^32 for odd p (any
// 32-bit prime), Barrett for p = 2; inverses by Fermat's little theorem in the
// Montgomery domain.
#include <cstdint>

#include <cuda_bf16.h>

#include "cand_cluster.cuh"

namespace lnc {

template <class Arith, class W, int PW, int CL>
static __global__ void __launch_bounds__(kCandClusterThreads, 1)
    cand_cluster_kernel(const __grid_constant__ CandArgs a) {
    cand_cluster_body<Arith, W, PW, CL>(a);
}

// CTAs of the cluster panel: 8 by default; LNC_CAND_CLUSTER=4 selects four, =0 the one-CTA panel.
static int cluster_panel_ctas() {
    static int ctas = -1;
    if (ctas < 0) {
        const char* env = getenv("LNC_CAND_CLUSTER");
        ctas = (env && env[0] == '0') ? 0 : (env && env[0] == '4') ? 4 : 8;
    }
    return ctas;
}

template <class Arith, class W, int PW, int CL>
static int launch_cand_cluster(const CandArgs& a, double elt, cudaStream_t s) {
    auto kern = cand_cluster_kernel<Arith, W, PW, CL>;
    const size_t smem = cand_cluster_smem<W, PW, CL>(a.smax);
    int rc = allow_dynamic_smem((const void*)kern, smem);
    if (rc) return rc;
    ScopedKernelTimer kt(KC_PANEL, s, 2.0 * a.smax * a.bw * elt);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(CL, 1, 1);
    cfg.blockDim = dim3(kCandClusterThreads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CL;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    LNC_CUDA(cudaLaunchKernelEx(&cfg, kern, a));
    LNC_CHECK_LAUNCH("cand_cluster_kernel");
    return LNC_OK;
}

template <class Arith>
static int launch_cand_typed(const CandArgs& a, size_t smem, cudaStream_t s) {
    int rc = allow_dynamic_smem((const void*)cand_panel_kernel<Arith>, smem);
    if (rc) return rc;
    ScopedKernelTimer kt(KC_PANEL, s, 2.0 * a.smax * a.bw * 4.0);
    cand_panel_kernel<Arith><<<1, kCandThreads, smem, s>>>(a);
    LNC_CHECK_LAUNCH("cand_panel_kernel");
    return LNC_OK;
}

int launch_cand_panel(const CandArgs& a, cudaStream_t s) {
    const int cl = cluster_panel_ctas();
    if (cl == 8) {
        if (!(a.M.p & 1u)) return launch_cand_cluster<ArithTwo, uint32_t, kMaxPanel, 8>(a, 4.0, s);
        if (a.M.p < (1u << 31)) return launch_cand_cluster<ArithSmall, uint32_t, kMaxPanel, 8>(a, 4.0, s);
        return launch_cand_cluster<ArithMont, uint32_t, kMaxPanel, 8>(a, 4.0, s);
    }
    if (cl == 4) {
        if (!(a.M.p & 1u)) return launch_cand_cluster<ArithTwo, uint32_t, kMaxPanel, 4>(a, 4.0, s);
        if (a.M.p < (1u << 31)) return launch_cand_cluster<ArithSmall, uint32_t, kMaxPanel, 4>(a, 4.0, s);
        return launch_cand_cluster<ArithMont, uint32_t, kMaxPanel, 4>(a, 4.0, s);
    }
    const size_t smem = (size_t)(a.smax | 1) * kMaxPanel * 4 + 2 * kMaxPanel * 4 + 256 * 4;
    if (!(a.M.p & 1u)) return launch_cand_typed<ArithTwo>(a, smem, s);
    if (a.M.p < (1u << 31)) return launch_cand_typed<ArithSmall>(a, smem, s);
    return launch_cand_typed<ArithMont>(a, smem, s);
}

int launch_cand_panel64(const CandArgs& a, cudaStream_t s) {
    const int cl = cluster_panel_ctas();
    if (cl == 8) return launch_cand_cluster<Arith64, uint64_t, kPanelU64, 8>(a, 8.0, s);
    if (cl == 4) return launch_cand_cluster<Arith64, uint64_t, kPanelU64, 4>(a, 8.0, s);
    const size_t smem = cand_smem<uint64_t, kPanelU64>(a.smax);
    auto kern = cand_panel_kernel<Arith64, uint64_t, kPanelU64>;
    int rc = allow_dynamic_smem((const void*)kern, smem);
    if (rc) return rc;
    ScopedKernelTimer kt(KC_PANEL, s, 2.0 * a.smax * a.bw * 8.0);
    kern<<<1, kCandThreads, smem, s>>>(a);
    LNC_CHECK_LAUNCH("cand_panel_kernel (64-bit)");
    return LNC_OK;
}

int launch_check_missed64(const uint64_t* A, int64_t lda, int64_t m, int64_t j0, int bw, const uint8_t* row_used,
                          const uint32_t* pivmask, int* missed, cudaStream_t s) {
    const int64_t warps = std::min<int64_t>(m, 152 * 64);
    const int grid = (int)std::max<int64_t>(1, (warps * 32 + 255) / 256);
    check_missed_kernel<uint64_t><<<grid, 256, 0, s>>>(A, lda, m, j0, bw, row_used, pivmask, missed);
    LNC_CHECK_LAUNCH("check_missed_kernel (64-bit)");
    return LNC_OK;
}

int launch_split_g(const uint32_t* A, int64_t lda, int64_t m, int64_t j0, uint32_t p, const int32_t* panel_k,
                   const int32_t* panel_cols, const int32_t* panel_mark, int gen, void* EL, cudaStream_t s) {
    const int m_pad = tc_m_pad(m);
    const int64_t total = (int64_t)m_pad * kMaxPanel;
    const int grid = (int)std::min<int64_t>((total + 255) / 256, 4096);
    split_g_kernel<<<grid, 256, 0, s>>>(A, lda, m, m_pad, j0, p, panel_k, panel_cols, panel_mark, gen,
                                        (__nv_bfloat16*)EL);
    LNC_CHECK_LAUNCH("split_g_kernel");
    return LNC_OK;
}

int launch_check_missed(const uint32_t* A, int64_t lda, int64_t m, int64_t j0, int bw, const uint8_t* row_used,
                        const uint32_t* pivmask, int* missed, cudaStream_t s) {
    const int64_t warps = std::min<int64_t>(m, 152 * 64);
    const int grid = (int)std::max<int64_t>(1, (warps * 32 + 255) / 256);
    check_missed_kernel<<<grid, 256, 0, s>>>(A, lda, m, j0, bw, row_used, pivmask, missed);
    LNC_CHECK_LAUNCH("check_missed_kernel");
    return LNC_OK;
}

}  // namespace lnc
