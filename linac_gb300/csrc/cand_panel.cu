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

#include "rref_internal.cuh"

namespace lnc {

struct Mont32 {
    uint32_t p, pinv, r2;  // pinv = -p^-1 mod 2^32, r2 = 2^64 mod p
    uint64_t mu;           // Barrett constant (p = 2 path)
    __device__ Mont32(const decltype(CandArgs::M)& c) : p(c.p), pinv(c.pinv), r2(c.r2), mu(c.mu) {}
    __device__ __forceinline__ uint32_t mont(uint64_t t) const {
        const uint32_t m = (uint32_t)t * pinv;
        const uint64_t mp = (uint64_t)m * p;
        // (t + m p) / 2^32: the low words cancel, carry iff low(t) != 0
        const uint64_t u = (t >> 32) + (mp >> 32) + (((uint32_t)t != 0u) ? 1ull : 0ull);
        return (uint32_t)(u >= p ? u - p : u);
    }
    __device__ __forceinline__ uint32_t montmul(uint32_t a, uint32_t b) const { return mont((uint64_t)a * b); }
    __device__ __forceinline__ uint32_t to_mont(uint32_t a) const { return montmul(a, r2); }
    __device__ __forceinline__ uint32_t from_mont(uint32_t a) const { return mont((uint64_t)a); }
    __device__ __forceinline__ uint32_t barrett(uint64_t x) const {
        uint64_t q = __umul64hi(x, mu);
        uint64_t r = x - q * (uint64_t)p;
        r = (r >= p) ? r - p : r;
        r = (r >= p) ? r - p : r;
        return (uint32_t)r;
    }
    __device__ __forceinline__ uint32_t sub(uint32_t a, uint32_t b) const { return a >= b ? a - b : a + (p - b); }
};

template <bool MONT>
__device__ __forceinline__ uint32_t cp_inverse(const Mont32& M, uint32_t a) {
    if constexpr (MONT) {
        uint32_t x = M.to_mont(a), r = M.to_mont(1u);
        uint64_t e = (uint64_t)M.p - 2;
        while (e) {
            if (e & 1) r = M.montmul(r, x);
            x = M.montmul(x, x);
            e >>= 1;
        }
        return M.from_mont(r);
    } else {
        return 1u;  // p = 2: the only non-zero residue is its own inverse
    }
}

// block-wide exclusive scan of a 0/1 flag (blockDim.x <= 1024); returns the
// prefix, writes the total to *total (shared)
__device__ __forceinline__ int block_scan_flag(int flag, int* s_warp, int* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned ballot = __ballot_sync(0xffffffffu, flag);
    const int in_warp = __popc(ballot & ((1u << lane) - 1u));
    if (lane == 0) s_warp[warp] = __popc(ballot);
    __syncthreads();
    if (threadIdx.x == 0) {
        int acc = 0;
        const int nw = (blockDim.x + 31) >> 5;
        for (int w = 0; w < nw; ++w) {
            const int v = s_warp[w];
            s_warp[w] = acc;
            acc += v;
        }
        *total = acc;
    }
    __syncthreads();
    const int r = s_warp[warp] + in_warp;
    __syncthreads();
    return r;
}

template <bool MONT>
__global__ void __launch_bounds__(kCandThreads, 1) cand_panel_kernel(CandArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int bw = a.bw;
    uint32_t* tile = (uint32_t*)smem_raw;                 // [smax][bw]
    uint32_t* nprM = tile + (size_t)a.smax * bw;          // [kMaxPanel]
    uint32_t* fcol = nprM + kMaxPanel;                    // [256]
    __shared__ int s_cand[256];
    __shared__ uint8_t s_isp[256];
    __shared__ int s_pr[kMaxPanel], s_pc[kMaxPanel];
    __shared__ int s_warp[32];
    __shared__ int s_n, s_total, s_next, s_min;
    __shared__ uint32_t s_inv;
    const Mont32 M = a.M;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int NW = kCandThreads / 32;

    if (tid == 0) {
        *a.missed = 0;
        s_next = *a.next_row;
    }
    // ---- candidate rows: keep the old ones that are still eligible, refill in row order
    {
        const int n0 = *a.cand_n;
        int r = -1, keep = 0;
        if (tid < n0) {
            r = a.cand[tid];
            keep = !a.row_used[r];
        }
        const int pos = block_scan_flag(keep, s_warp, &s_total);
        if (keep) s_cand[pos] = r;
        if (tid == 0) s_n = s_total;
        __syncthreads();
    }
    while (s_n < a.smax && s_next < a.m) {
        const int base = s_next;
        const int r = base + tid;
        const int e = (r < a.m) ? !a.row_used[r] : 0;
        const int pos = block_scan_flag(e, s_warp, &s_total);
        const int need = a.smax - s_n;
        if (e && pos < need) s_cand[s_n + pos] = r;
        if (e && pos == need - 1) s_next = r + 1;  // filled: resume after the last row taken
        __syncthreads();
        if (tid == 0) {
            if (s_total < need) {
                s_n += s_total;
                s_next = min((int64_t)base + (int64_t)blockDim.x, a.m);
            } else {
                s_n += need;
            }
        }
        __syncthreads();
    }
    const int n = s_n;
    // ---- load the candidate block
    for (int i = warp; i < n; i += NW) {
        const uint32_t* src = a.A + (int64_t)s_cand[i] * a.lda + a.j0;
        for (int c = lane; c < bw; c += 32) tile[(size_t)i * bw + c] = src[c];
    }
    for (int i = tid; i < 256; i += blockDim.x) s_isp[i] = 0;
    __syncthreads();

    // ---- Gauss-Jordan on the block, transform kept in the pivot columns
    int k = 0;
    for (int c = 0; c < bw; ++c) {
        if (tid == 0) s_min = 0x7fffffff;
        __syncthreads();
        if (tid < n && !s_isp[tid] && tile[(size_t)tid * bw + c] != 0u) atomicMin(&s_min, tid);
        __syncthreads();
        const int pi = s_min;
        if (pi == 0x7fffffff) continue;  // no pivot in this column among the candidates
        if (tid < n) fcol[tid] = tile[(size_t)tid * bw + c];
        if (tid == 0) s_inv = cp_inverse<MONT>(M, tile[(size_t)pi * bw + c]);
        __syncthreads();
        const uint32_t inv = s_inv;
        for (int cc = tid; cc < bw; cc += blockDim.x) {
            uint32_t v;
            if constexpr (MONT) {
                v = (cc == c) ? inv : M.montmul(M.to_mont(tile[(size_t)pi * bw + cc]), inv);
                nprM[cc] = M.to_mont(v);
            } else {
                v = (cc == c) ? inv : M.barrett((uint64_t)tile[(size_t)pi * bw + cc] * inv);
                nprM[cc] = v;
            }
            tile[(size_t)pi * bw + cc] = v;
        }
        __syncthreads();
        for (int i = warp; i < n; i += NW) {
            if (i == pi) continue;
            const uint32_t f = fcol[i];
            if (f == 0u) continue;
            uint32_t* row = tile + (size_t)i * bw;
            for (int cc = lane; cc < bw; cc += 32) {
                const uint32_t x = (cc == c) ? 0u : row[cc];
                uint32_t prod;
                if constexpr (MONT) prod = M.montmul(f, nprM[cc]);
                else prod = M.barrett((uint64_t)f * nprM[cc]);
                row[cc] = M.sub(x, prod);
            }
        }
        if (tid == 0) {
            s_pr[k] = pi;
            s_pc[k] = c;
            s_isp[pi] = 1;
        }
        ++k;
        __syncthreads();
    }

    // ---- outputs
    const int64_t rank0 = *a.rank;
    for (int idx = tid; idx < kMaxPanel * kMaxPanel; idx += blockDim.x) {
        const int t = idx / kMaxPanel, u = idx % kMaxPanel;
        a.X[idx] = (t < k && u < k) ? tile[(size_t)s_pr[t] * bw + s_pc[u]] : 0u;
    }
    for (int t = tid; t < k; t += blockDim.x) {
        const int r = s_cand[s_pr[t]];
        a.panel_rows[t] = r;
        a.panel_cols[t] = s_pc[t];
        a.piv_row[rank0 + t] = r;
        a.piv_col[rank0 + t] = a.j0 + s_pc[t];
        a.row_used[r] = 1;
        a.panel_mark[r] = (a.gen << 8) | (t + 1);
    }
    if (tid < 4) {
        uint32_t mask = 0u;
        for (int t = 0; t < k; ++t)
            if ((s_pc[t] >> 5) == tid) mask |= 1u << (s_pc[t] & 31);
        a.pivmask[tid] = mask;
    }
    {
        const int keep = (tid < n) ? !s_isp[tid] : 0;
        const int pos = block_scan_flag(keep, s_warp, &s_total);
        if (keep) a.cand[pos] = s_cand[tid];
        if (tid == 0) {
            *a.cand_n = s_total;
            *a.next_row = s_next;
            *a.panel_k = k;
            *a.rank = rank0 + k;
        }
    }
}

// G operand of E = G X, as four K-major digit planes: G[o, t] = -A[o, j0 + c_t]
// for rows that are not pivot rows of this panel, G[prow_t, :] = e_t.
__device__ __forceinline__ void split4(uint32_t x, uint32_t p, __nv_bfloat16 (&d)[4]) {
    int32_t v = (x > (p >> 1)) ? (int32_t)((int64_t)x - (int64_t)p) : (int32_t)x;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const int32_t di = ((v + 128) & 255) - 128;
        d[i] = __float2bfloat16_rn((float)di);
        v = (v - di) >> 8;
    }
    d[3] = __float2bfloat16_rn((float)v);
}

__global__ void split_g_kernel(const uint32_t* A, int64_t lda, int64_t m, int m_pad, int64_t j0, uint32_t p,
                               const int32_t* panel_k, const int32_t* panel_cols, const int32_t* panel_mark,
                               int gen, __nv_bfloat16* EL) {
    const int k = *panel_k;
    if (k == 0) return;
    const size_t plane = (size_t)m_pad * kMaxPanel;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < (int64_t)m_pad * kMaxPanel;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = idx / kMaxPanel;
        const int t = (int)(idx - r * kMaxPanel);
        uint32_t v = 0u;
        if (r < m && t < k) {
            const int mk = panel_mark[r];
            if ((mk >> 8) == gen) {
                v = ((mk & 255) - 1 == t) ? 1u : 0u;
            } else {
                const uint32_t x = A[r * lda + j0 + panel_cols[t]];
                v = x ? p - x : 0u;
            }
        }
        __nv_bfloat16 d[4];
        split4(v, p, d);
#pragma unroll
        for (int i = 0; i < 4; ++i) EL[i * plane + idx] = d[i];
    }
}

// After the update every remaining (non-pivot) row must be zero in the
// panel's non-pivot columns; a non-zero entry means the candidate block missed
// a pivot.
__global__ void check_missed_kernel(const uint32_t* A, int64_t lda, int64_t m, int64_t j0, int bw,
                                    const uint8_t* row_used, const uint32_t* pivmask, int* missed) {
    __shared__ uint32_t s_mask[4];
    if (threadIdx.x < 4) s_mask[threadIdx.x] = pivmask[threadIdx.x];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t wid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    int bad = 0;
    for (int64_t r = wid; r < m; r += nw) {
        if (row_used[r]) continue;
        const uint32_t* row = A + r * lda + j0;
        for (int c = lane; c < bw; c += 32)
            if (!((s_mask[c >> 5] >> (c & 31)) & 1u) && row[c] != 0u) bad = 1;
    }
    if (__any_sync(0xffffffffu, bad) && lane == 0) atomicExch(missed, 1);
}

int launch_cand_panel(const CandArgs& a, cudaStream_t s) {
    const size_t smem = (size_t)a.smax * a.bw * 4 + kMaxPanel * 4 + 256 * 4;
    void* args[] = {(void*)&a};
    if (a.M.p & 1u) {
        LNC_CUDA(cudaFuncSetAttribute(cand_panel_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        ScopedKernelTimer kt(KC_PANEL, s, 2.0 * a.smax * a.bw * 4.0);
        cand_panel_kernel<true><<<1, kCandThreads, smem, s>>>(a);
    } else {
        LNC_CUDA(cudaFuncSetAttribute(cand_panel_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        ScopedKernelTimer kt(KC_PANEL, s, 2.0 * a.smax * a.bw * 4.0);
        cand_panel_kernel<false><<<1, kCandThreads, smem, s>>>(a);
    }
    (void)args;
    LNC_CHECK_LAUNCH("cand_panel_kernel");
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
