// Incremental RREF: append rows to an existing RREF over F_p (32-bit residues).
//
// linac's grow-and-retry caller (linac/vector_spaces/over_function_fields.py:74-101)
// re-reduces an ever larger matrix from scratch.  Given the RREF R (r x n,
// pivot columns Pc) of the rows so far and k new rows N, the RREF of the
// stacked matrix is obtained from
//   1. N' = N - N[:, Pc] R           (the new rows reduced by the old pivots;
//                                     N'[:, Pc] = 0)
//   2. S  = RREF(N')                 (s new pivots Qc, disjoint from Pc)
//   3. R' = R - R[:, Qc] S           (old rows cleared in the new pivot columns)
//   4. rows of R' and S merged by pivot column,
// with the two products on the tensor-core limb GEMM (k r n + r s n
// multiply-adds instead of a full re-reduction) and step 2 a k-row RREF.
#include <algorithm>

#include "common.cuh"
#include "rref_internal.cuh"

namespace lnc {

int tc_matmul_modp(uint32_t p, int64_t m, int64_t k, int64_t n, const uint32_t* A, int64_t lda, const uint32_t* B,
                   int64_t ldb, uint32_t* C, int64_t ldc, cudaStream_t s);

namespace {

// G[i, t] = -X[i, cols[t]] mod p   (rows x nc)
static __global__ void gather_neg_cols_kernel(const uint32_t* X, int64_t ldx, int64_t rows, const int64_t* cols,
                                              int64_t nc, uint32_t p, uint32_t* G) {
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < rows * nc;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = idx / nc, t = idx % nc;
        const uint32_t v = X[i * ldx + cols[t]];
        G[idx] = v ? p - v : 0u;
    }
}

// Y[i, :] = (Y[i, :] + Z[i, :]) mod p
static __global__ void add_rows_kernel(uint32_t* Y, int64_t ldy, const uint32_t* Z, int64_t ldz, int64_t rows,
                                       int64_t n, uint32_t p) {
    for (int64_t i = blockIdx.y; i < rows; i += gridDim.y)
        for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
            const uint32_t a = Y[i * ldy + c], b = Z[i * ldz + c];
            const uint32_t sum = a + b;  // < 2^32 for p < 2^31; otherwise compare
            Y[i * ldy + c] = (sum < a || sum >= p) ? sum - p : sum;
        }
}

// merge the rows of R' (pivots pr[0..r)) and S (pivots ps[0..s)) by pivot column into out
static __global__ void merge_rows_kernel(const uint32_t* R, int64_t ldr, const int64_t* pr, int64_t r, const uint32_t* S,
                                         int64_t lds, const int64_t* ps, const int64_t* s_ptr, uint32_t* out,
                                         int64_t ldo, int64_t rows_out, int64_t n, int64_t* out_piv,
                                         int64_t* out_rank) {
    const int64_t s = *s_ptr;
    for (int64_t row = blockIdx.y; row < rows_out; row += gridDim.y) {
        // which source row lands at `row`: rank of its pivot among both lists
        const uint32_t* src = nullptr;
        int64_t pc = -1;
        if (row < r + s) {
            // binary search: the number of R pivots before position `row`
            int64_t lo = 0, hi = r;  // find t in [0, r]: t + #(ps < pr[t]) ... merge by counting
            // position of R row t = t + lower_bound(ps, pr[t]); of S row u = u + lower_bound(pr, ps[u])
            while (lo < hi) {  // largest t with pos(t) <= row
                const int64_t mid = (lo + hi) / 2;
                int64_t a = 0, b = s;
                while (a < b) { const int64_t c = (a + b) / 2; if (ps[c] < pr[mid]) a = c + 1; else b = c; }
                if (mid + a <= row) lo = mid + 1; else hi = mid;
            }
            // lo = number of R rows placed at positions <= row
            const int64_t u = row - lo;  // S rows before or at row
            if (lo > 0) {
                const int64_t t = lo - 1;
                int64_t a = 0, b = s;
                while (a < b) { const int64_t c = (a + b) / 2; if (ps[c] < pr[t]) a = c + 1; else b = c; }
                if (t + a == row) { src = R + t * ldr; pc = pr[t]; }
            }
            if (!src) { src = S + u * lds; pc = ps[u]; }
        }
        for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
            out[row * ldo + c] = src ? src[c] : 0u;
        if (blockIdx.x == 0 && threadIdx.x == 0 && out_piv && row < r + s) out_piv[row] = pc;
    }
    if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && out_rank) *out_rank = r + s;
}

size_t al256(size_t x) { return (x + 255) / 256 * 256; }

}  // namespace
}  // namespace lnc

using namespace lnc;

extern "C" int lnc_rref_append_device(int dtype, int64_t r, int64_t k, int64_t n, uint64_t p, void* dev_rref,
                                      int64_t ld_rref, const int64_t* dev_pivot_cols, const void* dev_new,
                                      int64_t ld_new, void* dev_out, int64_t ld_out, int64_t* dev_out_pivot_cols,
                                      int64_t* dev_out_rank, void* stream) {
    if (dtype != LNC_U32) { set_error("appending rows is implemented for 32-bit residues"); return LNC_ERR_UNSUPPORTED; }
    int rc = validate_rref_args(dtype, k, n, p, ld_new);
    if (rc) return rc;
    if (r < 0 || r > n || (r > 0 && ld_rref < n) || ld_out < n) { set_error("append: bad shape"); return LNC_ERR_INVALID; }
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t pp = (uint32_t)p;
    const int64_t rows_out = r + k;
    if (n == 0 || rows_out == 0) {
        if (dev_out_rank) LNC_CUDA(cudaMemsetAsync(dev_out_rank, 0, sizeof(int64_t), s));
        return LNC_OK;
    }
    const int64_t kmax = std::max<int64_t>(std::min(k, n), 1);
    const size_t w_b = al256(sizeof(uint32_t) * (size_t)k * n);
    const size_t g_b = al256(sizeof(uint32_t) * (size_t)std::max<int64_t>(k, r) * std::max<int64_t>(std::max<int64_t>(r, kmax), 1));
    const size_t c_b = al256(sizeof(uint32_t) * (size_t)std::max<int64_t>(k, r) * n);
    unsigned char* blk = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&blk, 2 * w_b + g_b + c_b + al256(8 * kmax) + 256, s);
    if (e != cudaSuccess) { cudaGetLastError(); set_error("append scratch: %s", cudaGetErrorString(e)); return LNC_ERR_OOM; }
    uint32_t* W = (uint32_t*)blk;               // N' (k x n)
    uint32_t* S = (uint32_t*)(blk + w_b);       // RREF(N') (k x n)
    uint32_t* G = (uint32_t*)(blk + 2 * w_b);   // gathered, negated columns
    uint32_t* C = (uint32_t*)(blk + 2 * w_b + g_b);
    int64_t* ps = (int64_t*)(blk + 2 * w_b + g_b + c_b);
    int64_t* srank = (int64_t*)(blk + 2 * w_b + g_b + c_b + al256(8 * kmax));
    auto done = [&](int code) { cudaFreeAsync(blk, s); return code; };
    // 1. N' = N - N[:, Pc] R
    if (k > 0) {
        LNC_CUDA(cudaMemcpy2DAsync(W, 4 * n, dev_new, 4 * ld_new, 4 * n, k, cudaMemcpyDeviceToDevice, s));
        if (r > 0) {
            gather_neg_cols_kernel<<<(unsigned)std::min<int64_t>((k * r + 255) / 256, 4096), 256, 0, s>>>(
                (const uint32_t*)dev_new, ld_new, k, dev_pivot_cols, r, pp, G);
            LNC_CHECK_LAUNCH("gather_neg_cols_kernel");
            rc = tc_matmul_modp(pp, k, r, n, G, r, (const uint32_t*)dev_rref, ld_rref, C, n, s);
            if (rc) return done(rc);
            dim3 g((unsigned)std::min<int64_t>((n + 255) / 256, 64), (unsigned)std::min<int64_t>(k, 65535));
            add_rows_kernel<<<g, 256, 0, s>>>(W, n, C, n, k, n, pp);
            LNC_CHECK_LAUNCH("add_rows_kernel");
        }
        // 2. S = RREF(N')
        rc = rref_device_dispatch(LNC_U32, k, n, p, 0.0, W, n, S, n, ps, srank, s, 0);
        if (rc) return done(rc);
    } else {
        LNC_CUDA(cudaMemsetAsync(srank, 0, 8, s));
    }
    int64_t sh = 0;
    LNC_CUDA(cudaMemcpyAsync(&sh, srank, 8, cudaMemcpyDeviceToHost, s));
    LNC_CUDA(cudaStreamSynchronize(s));
    // 3. R' = R - R[:, Qc] S   (in place in the caller's R)
    if (sh > 0 && r > 0) {
        gather_neg_cols_kernel<<<(unsigned)std::min<int64_t>((r * sh + 255) / 256, 4096), 256, 0, s>>>(
            (const uint32_t*)dev_rref, ld_rref, r, ps, sh, pp, G);
        LNC_CHECK_LAUNCH("gather_neg_cols_kernel");
        rc = tc_matmul_modp(pp, r, sh, n, G, sh, S, n, C, n, s);
        if (rc) return done(rc);
        dim3 g((unsigned)std::min<int64_t>((n + 255) / 256, 64), (unsigned)std::min<int64_t>(r, 65535));
        add_rows_kernel<<<g, 256, 0, s>>>((uint32_t*)dev_rref, ld_rref, C, n, r, n, pp);
        LNC_CHECK_LAUNCH("add_rows_kernel");
    }
    // 4. merge by pivot column
    {
        dim3 g((unsigned)std::min<int64_t>((n + 255) / 256, 16), (unsigned)std::min<int64_t>(rows_out, 65535));
        merge_rows_kernel<<<g, 256, 0, s>>>((const uint32_t*)dev_rref, ld_rref, dev_pivot_cols, r, S, n, ps, srank,
                                             (uint32_t*)dev_out, ld_out, rows_out, n, dev_out_pivot_cols, dev_out_rank);
        LNC_CHECK_LAUNCH("merge_rows_kernel");
    }
    return done(LNC_OK);
}
