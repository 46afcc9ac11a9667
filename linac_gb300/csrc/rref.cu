// Dense reduced row-echelon form on one GPU: blocked right-looking
// Gauss-Jordan with a cooperative panel kernel and a trailing update.
//
// The reference (linac/pycuda_row_reduce.py:94-131 driving
// linac/row_reduce.cu:273-430) runs an unblocked loop from Python, 6-7 kernel
// launches per column, each column touching the whole m x (n - j) trailing
// matrix.  This driver processes `b` columns per panel:
//
//  1. panel_kernel (cooperative, one CTA per SM, panel rows held in shared
//     memory): for each panel column, every CTA proposes its best eligible
//     row (largest residue / |a|, as in row_reduce.cu:287-393), one bounded
//     grid barrier exchanges the proposals, and every CTA eliminates its own
//     rows with the normalised winner (row_reduce.cu:117-196).  Eliminated
//     pivot columns keep the Gauss-Jordan transform in place ("E"), so that
//     after the panel   A[:, T] <- A[:, T] (pivot rows zeroed) + E * A[P, T]
//     applies the whole panel to the trailing columns T in one contraction.
//  2. gather_pivot_rows: copies the k pivot rows' trailing part to a dense
//     operand and zeroes them in A.
//  3. trailing update: the contraction above (tensor-core limb GEMM for
//     32-bit residues, see trailing_tc.cu; a SIMT kernel here for the other
//     fields and as the reference implementation for tests).
//  4. gather_rref_rows: rows are never swapped in memory; pivot rows are
//     tracked in a list and gathered into RREF order once at the end.
//
// The RREF over a field is unique, so the pivot order does not change the
// F_p result; it is bit-identical to linac's CPU row_reduce.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "field.cuh"
#include "sync.cuh"
#include "rref_internal.cuh"

namespace lnc {

__device__ int g_rref_status = 0;

int rref_read_and_clear_status(int* status) {
    int v = 0, zero = 0;
    LNC_CUDA(cudaMemcpyFromSymbol(&v, g_rref_status, sizeof(int)));
    LNC_CUDA(cudaMemcpyToSymbol(g_rref_status, &zero, sizeof(int)));
    *status = v;
    return LNC_OK;
}

int* rref_status_symbol_address() {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_rref_status) != cudaSuccess) return nullptr;
    return (int*)p;
}

// ----------------------------------------------------------------------------
// key helpers
// ----------------------------------------------------------------------------
template <class F> struct KeyNone;
template <> struct KeyNone<FieldU32> { static __device__ __forceinline__ uint64_t v() { return 0ull; } };
template <> struct KeyNone<FieldU64> { static __device__ __forceinline__ uint64_t v() { return 0ull; } };
template <> struct KeyNone<FieldF64> { static __device__ __forceinline__ double v() { return -1.0; } };
template <> struct KeyNone<FieldC128> { static __device__ __forceinline__ double v() { return -1.0; } };

template <class K>
__device__ __forceinline__ bool better(K ka, int64_t ra, K kb, int64_t rb) {
    return ka > kb || (ka == kb && ra < rb);
}

template <class T>
__device__ __forceinline__ T ldcg(const T* p) { return __ldcg(p); }

// a value of lane `src` of the warp, for the field element types
__device__ __forceinline__ uint32_t shfl_value(uint32_t v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ uint64_t shfl_value(uint64_t v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ double shfl_value(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ c128 shfl_value(c128 v, int src) {
    v.x = __shfl_sync(0xffffffffu, v.x, src);
    v.y = __shfl_sync(0xffffffffu, v.y, src);
    return v;
}
template <>
__device__ __forceinline__ c128 ldcg<c128>(const c128* p) {
    double2 v = __ldcg((const double2*)p);
    c128 r; r.x = v.x; r.y = v.y; return r;
}

// ----------------------------------------------------------------------------
// 0. input preparation
// ----------------------------------------------------------------------------
template <class F>
__global__ void reduce_input_kernel(F f, typename F::T* A, int64_t lda, int64_t m, int64_t n) {
    for (int64_t r = blockIdx.y; r < m; r += gridDim.y) {
        typename F::T* row = A + r * lda;
        for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
             c += (int64_t)gridDim.x * blockDim.x)
            row[c] = f.reduce_input(row[c]);
    }
}

// Row pre-scaling of the float path (linac/row_reduce.cu:201-270): each row
// divided by its largest |a|.  A zero row is left as is (the reference would
// divide by zero and fill the row with NaN).
template <class F>
__global__ void row_scale_kernel(F f, typename F::T* A, int64_t lda, int64_t m, int64_t n) {
    __shared__ double s_part[32];
    for (int64_t r = blockIdx.x; r < m; r += gridDim.x) {
        typename F::T* row = A + r * lda;
        double mx = 0.0;
        for (int64_t c = threadIdx.x; c < n; c += blockDim.x) mx = fmax(mx, (double)f.key(row[c]));
        for (int o = 16; o; o >>= 1) mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
        if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = mx;
        __syncthreads();
        if (threadIdx.x < 32) {
            double v = threadIdx.x < (blockDim.x >> 5) ? s_part[threadIdx.x] : 0.0;
            for (int o = 16; o; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
            if (threadIdx.x == 0) s_part[0] = v;
        }
        __syncthreads();
        double s = s_part[0];
        __syncthreads();
        if (s > 0.0) {
            for (int64_t c = threadIdx.x; c < n; c += blockDim.x) row[c] = scale_real(row[c], s);
        }
    }
}

// ----------------------------------------------------------------------------
// 1. panel kernel
// ----------------------------------------------------------------------------
template <class F>
__global__ void __launch_bounds__(kPanelThreads, 1) panel_kernel(PanelArgs<F> a) {
    using T = typename F::T;
    using Key = typename F::Key;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const F f = a.f;
    const int G = gridDim.x;
    const int bw = a.bw;
    const int RP = a.rows_per_cta;
    const int64_t r0 = (int64_t)blockIdx.x * RP;
    const int64_t r1 = min(a.m, r0 + RP);
    const int R = (int)max((int64_t)0, r1 - r0);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int NW = kPanelThreads / 32;

    T* tile = (T*)smem_raw;                // [RP][bw]
    T* prow = tile + (size_t)RP * bw;      // [bw]
    T* fcol = prow + bw;                   // [RP]
    int* ispiv = (int*)(fcol + RP);        // [bw]
    uint8_t* used = (uint8_t*)(ispiv + bw);  // [RP]

    __shared__ int64_t s_prows[kMaxPanel];
    __shared__ int s_pcols[kMaxPanel];
    __shared__ Key s_wkey[NW];
    __shared__ int64_t s_wrow[NW];
    __shared__ int64_t s_win_row;
    __shared__ int s_win_ok;

    if (ld_volatile_i32(a.bar.err) != 0) return;
    if (a.run_if != nullptr && ld_volatile_i32(a.run_if) == 0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) *a.panel_k = 0;
        return;
    }
    const int64_t rank0 = *a.rank;

    for (int r = warp; r < R; r += NW) {
        const T* src = a.A + (r0 + r) * a.lda + a.j0;
        for (int c = lane; c < bw; c += 32) tile[(size_t)r * bw + c] = src[c];
        if (lane == 0) used[r] = a.row_used[r0 + r];
    }
    for (int c = threadIdx.x; c < bw; c += blockDim.x) ispiv[c] = -1;
    __syncthreads();

    int k = 0;
    for (int c = 0; c < bw; ++c) {
        if (rank0 + k >= a.m) break;  // every row is a pivot row already
        const int par = c & 1;
        // -- local proposal: best eligible row of this CTA for column c (warps reduce their rows,
        //    warp 0 combines the warps and publishes the candidate row); own rows' column c to fcol
        Key bk = KeyNone<F>::v();
        int64_t br = INT64_MAX;
        for (int r = threadIdx.x; r < R; r += blockDim.x) {
            const T v = tile[(size_t)r * bw + c];
            fcol[r] = v;
            if (!used[r]) {
                Key kk = f.key(v);
                if (better(kk, r0 + r, bk, br)) { bk = kk; br = r0 + r; }
            }
        }
        for (int o = 16; o; o >>= 1) {
            Key ok = __shfl_down_sync(0xffffffffu, bk, o);
            int64_t orow = __shfl_down_sync(0xffffffffu, br, o);
            if (better(ok, orow, bk, br)) { bk = ok; br = orow; }
        }
        if (lane == 0) { s_wkey[warp] = bk; s_wrow[warp] = br; }
        __syncthreads();
        if (warp == 0) {
            bk = (lane < NW) ? s_wkey[lane] : KeyNone<F>::v();
            br = (lane < NW) ? s_wrow[lane] : INT64_MAX;
            for (int o = 16; o; o >>= 1) {
                Key ok = __shfl_xor_sync(0xffffffffu, bk, o);
                int64_t orow = __shfl_xor_sync(0xffffffffu, br, o);
                if (better(ok, orow, bk, br)) { bk = ok; br = orow; }
            }
            if (lane == 0) {
                a.cand_key[par * G + blockIdx.x] = bk;
                a.cand_row[par * G + blockIdx.x] = br;
            }
            if (br != INT64_MAX) {
                const int rl = (int)(br - r0);
                T* dst = a.cand_vals + ((size_t)par * G + blockIdx.x) * a.b;
                for (int cc = lane; cc < bw; cc += 32) dst[cc] = tile[(size_t)rl * bw + cc];
            }
        }
        // -- exchange
        if (!grid_sync(a.bar)) return;
        // -- winner over all CTAs (warp 0; identical in every CTA) and its row, normalised, in prow
        if (warp == 0) {
            Key wk = KeyNone<F>::v();
            int64_t wr = INT64_MAX;
            int wb = -1;
            // all proposals in one round of independent loads (G <= 32 * GL CTAs)
            constexpr int GL = 8;
            int64_t rrs[GL];
            Key kks[GL];
#pragma unroll
            for (int j = 0; j < GL; ++j) {
                const int g = lane + 32 * j;
                rrs[j] = (g < G) ? ldcg(a.cand_row + par * G + g) : INT64_MAX;
                kks[j] = (g < G) ? ldcg(a.cand_key + par * G + g) : KeyNone<F>::v();
            }
#pragma unroll
            for (int j = 0; j < GL; ++j)
                if (rrs[j] != INT64_MAX && better(kks[j], rrs[j], wk, wr)) { wk = kks[j]; wr = rrs[j]; wb = lane + 32 * j; }
            for (int o = 16; o; o >>= 1) {
                Key ok = __shfl_xor_sync(0xffffffffu, wk, o);
                int64_t orow = __shfl_xor_sync(0xffffffffu, wr, o);
                int ob = __shfl_xor_sync(0xffffffffu, wb, o);
                if (better(ok, orow, wk, wr)) { wk = ok; wr = orow; wb = ob; }
            }
            const bool ok = (wr != INT64_MAX) && f.is_pivot(wk);
            if (ok) {
                // the winner's row in one round of loads (kMaxPanel / 32 per lane), its pivot
                // from the lane holding column c, the inverse in every lane
                const T* src = a.cand_vals + ((size_t)par * G + wb) * a.b;
                constexpr int PL = kMaxPanel / 32;
                T v[PL];
#pragma unroll
                for (int j = 0; j < PL; ++j) {
                    const int cc = lane + 32 * j;
                    v[j] = (cc < bw) ? ldcg(src + cc) : f.zero();
                }
                T piv = f.zero();
#pragma unroll
                for (int j = 0; j < PL; ++j)
                    if (j == (c >> 5)) piv = v[j];
                piv = shfl_value(piv, c & 31);
                const T pinv = f.inv(piv);
#pragma unroll
                for (int j = 0; j < PL; ++j) {
                    const int cc = lane + 32 * j;
                    if (cc < bw) prow[cc] = (cc == c) ? pinv : f.scale(v[j], piv, pinv);
                }
            }
            if (lane == 0) {
                s_win_row = wr;
                s_win_ok = ok ? 1 : 0;
                if constexpr (F::kDtype >= 3) {
                    if (a.uncertain && wr != INT64_MAX && wk > a.band_lo && wk <= a.band_hi) atomicExch(a.uncertain, 1);
                }
            }
        }
        __syncthreads();
        if (!s_win_ok) continue;  // column c has no pivot (uniform decision)
        const int64_t wrow = s_win_row;
        // -- eliminate own rows (Gauss-Jordan, above and below), keeping the
        //    transform in column c
        for (int r = warp; r < R; r += NW) {
            T* row = tile + (size_t)r * bw;
            if (r0 + r == wrow) {
                for (int cc = lane; cc < bw; cc += 32) row[cc] = prow[cc];
                if (lane == 0) used[r] = 1;
            } else {
                const T fv = fcol[r];
                if (f.nonzero(fv)) {
                    for (int cc = lane; cc < bw; cc += 32) {
                        T x = (cc == c) ? f.zero() : row[cc];
                        row[cc] = f.sub(x, f.mul(fv, prow[cc]));
                    }
                }
            }
        }
        if (threadIdx.x == 0) {
            s_pcols[k] = c;
            s_prows[k] = wrow;
            ispiv[c] = k;
        }
        ++k;
        __syncthreads();
    }

    // -- write back: pivot columns become unit vectors, the transform goes to E
    if (k > 0) {
        for (int r = warp; r < R; r += NW) {
            const int64_t gr = r0 + r;
            T* dst = a.A + gr * a.lda + a.j0;
            const T* row = tile + (size_t)r * bw;
            for (int cc = lane; cc < bw; cc += 32) {
                const int t = ispiv[cc];
                if (t >= 0) dst[cc] = (gr == s_prows[t]) ? f.one() : f.zero();
                else dst[cc] = row[cc];
            }
            if (lane == 0) a.row_used[gr] = used[r];
        }
    }
    if (a.E != nullptr) {
        for (int r = warp; r < R; r += NW) {
            const int64_t gr = r0 + r;
            T* e = a.E + gr * a.ldE;
            const T* row = tile + (size_t)r * bw;
            for (int t = lane; t < a.b; t += 32) e[t] = (t < k) ? row[s_pcols[t]] : f.zero();
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        for (int t = 0; t < k; ++t) {
            a.piv_row[rank0 + t] = (int32_t)s_prows[t];
            a.piv_col[rank0 + t] = a.j0 + s_pcols[t];
            a.panel_rows[t] = (int32_t)s_prows[t];
        }
        *a.panel_k = k;
        *a.rank = rank0 + k;
    }
}

// ----------------------------------------------------------------------------
// 2. pivot-row gather for the trailing update
// ----------------------------------------------------------------------------
template <class F>
__global__ void gather_pivot_rows_kernel(F f, typename F::T* A, int64_t lda, int64_t j1, int64_t N,
                                         const int32_t* panel_rows, const int32_t* panel_k,
                                         typename F::T* Bm, int64_t ldb) {
    const int t = blockIdx.y;
    const int k = *panel_k;
    if (t >= k) return;
    const int64_t row = panel_rows[t];
    typename F::T* src = A + row * lda + j1;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < N;
         c += (int64_t)gridDim.x * blockDim.x) {
        Bm[t * ldb + c] = GemmOps<F>::prep_b(f, src[c]);
        src[c] = f.zero();
    }
}

// ----------------------------------------------------------------------------
// 3. SIMT trailing update:  A[:, j1:j1+N] += E[:, :k] * Bm[:k, :]
// ----------------------------------------------------------------------------
template <class F, int BK, int LAZY>
__global__ void __launch_bounds__(256) trailing_simt_kernel(F f, typename F::T* A, int64_t lda,
                                                            int64_t m, int64_t j1, int64_t N,
                                                            const typename F::T* E, int64_t ldE,
                                                            const typename F::T* Bm, int64_t ldb,
                                                            const int32_t* panel_k) {
    using T = typename F::T;
    using Ops = GemmOps<F>;
    using Acc = typename Ops::Acc;
    constexpr int BM = 64, BN = 128;
    __shared__ T Es[BM][BK + 1];
    __shared__ T Bs[BK][BN];
    const int k = *panel_k;
    if (k == 0) return;
    const int64_t bm0 = (int64_t)blockIdx.y * BM;
    const int64_t bn0 = (int64_t)blockIdx.x * BN;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    Acc acc[4][8];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = Ops::acc_zero(f);

    for (int kk = 0; kk < k; kk += BK) {
        for (int idx = threadIdx.x; idx < BM * BK; idx += blockDim.x) {
            const int r = idx / BK, t = idx % BK;
            const int64_t row = bm0 + r;
            Es[r][t] = (row < m && kk + t < k) ? E[row * ldE + kk + t] : f.zero();
        }
        for (int idx = threadIdx.x; idx < BK * BN; idx += blockDim.x) {
            const int t = idx / BN, cc = idx % BN;
            Bs[t][cc] = (kk + t < k && bn0 + cc < N) ? Bm[(int64_t)(kk + t) * ldb + bn0 + cc]
                                                    : Ops::b_zero(f);
        }
        __syncthreads();
#pragma unroll
        for (int t0 = 0; t0 < BK; t0 += LAZY) {
#pragma unroll
            for (int t = t0; t < t0 + LAZY; ++t) {
                T av[4], bv[8];
#pragma unroll
                for (int i = 0; i < 4; ++i) av[i] = Es[ty * 4 + i][t];
#pragma unroll
                for (int j = 0; j < 8; ++j) bv[j] = Bs[t][tx + 16 * j];
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 8; ++j) acc[i][j] = Ops::mac(f, acc[i][j], av[i], bv[j]);
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j) acc[i][j] = Ops::fold(f, acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int64_t row = bm0 + ty * 4 + i;
        if (row >= m) continue;
        T* dst = A + row * lda + j1;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int64_t col = bn0 + tx + 16 * j;
            if (col < N) dst[col] = Ops::finish(f, acc[i][j], dst[col]);
        }
    }
}

// ----------------------------------------------------------------------------
// 4. final gather into RREF row order
// ----------------------------------------------------------------------------
template <class T>
__global__ void gather_rref_rows_kernel(const T* A, int64_t lda, T* out, int64_t ldo, int64_t m,
                                        int64_t n, const int32_t* piv_row, const int64_t* rank_p,
                                        T zero) {
    const int64_t rank = *rank_p;
    for (int64_t r = blockIdx.y; r < m; r += gridDim.y) {
        T* dst = out + r * ldo;
        if (r < rank) {
            const T* src = A + (int64_t)piv_row[r] * lda;
            for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
                 c += (int64_t)gridDim.x * blockDim.x)
                dst[c] = src[c];
        } else {
            for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
                 c += (int64_t)gridDim.x * blockDim.x)
                dst[c] = zero;
        }
    }
}

__global__ void copy_pivots_kernel(const int64_t* piv_col, const int64_t* rank_p, int64_t cap,
                                   int64_t* out_piv, int64_t* out_rank) {
    const int64_t rank = *rank_p;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < cap;
         i += (int64_t)gridDim.x * blockDim.x)
        if (out_piv) out_piv[i] = (i < rank) ? piv_col[i] : -1;
    if (blockIdx.x == 0 && threadIdx.x == 0 && out_rank) *out_rank = rank;
}

__global__ void publish_status_kernel(const int* err, int* status) {
    if (*err != 0) atomicExch(status, *err);
}

// deferred-fallback solves: the rank output carries the outcome
__global__ void publish_deferred_kernel(const int* err, const int* missed_any, int64_t* dev_rank) {
    if (*err != 0) *dev_rank = -2;
    else if (missed_any && *missed_any) *dev_rank = -1;
}

// ----------------------------------------------------------------------------
// host driver
// ----------------------------------------------------------------------------
static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

template <class F>
static size_t panel_smem_bytes(int rows_per_cta, int bw) {
    using T = typename F::T;
    return (size_t)rows_per_cta * bw * sizeof(T) + (size_t)bw * sizeof(T) +
           (size_t)rows_per_cta * sizeof(T) + (size_t)bw * sizeof(int) + (size_t)rows_per_cta + 16;
}

template <class F>
int plan_rref(int64_t m, int64_t n, RrefPlan* plan) {
    DeviceInfo di;
    int rc = device_info(&di);
    if (rc) return rc;
    if (!di.coop) { set_error("device does not support cooperative launches"); return LNC_ERR_UNSUPPORTED; }
    int G = (int)std::min<int64_t>(di.sms, m);
    if constexpr (F::kDtype >= 3) {
        // float panels: at least 32 rows per CTA.  Fewer CTAs make the per-column grid barrier
        // cheaper and leave SMs to the panels of concurrent solves (a batch of 64 float systems,
        // n ~ U[256, 4096], 16 workers: 67 -> 80 solves/s); a 5000-row panel is unchanged
        G = (int)std::max<int64_t>(1, std::min<int64_t>(G, (m + 31) / 32));
    }
    int R = (int)((m + G - 1) / G);
    G = (int)((m + R - 1) / R);
    const size_t budget = (size_t)di.smem_optin - 8 * 1024;  // static smem headroom
    int b = 0;
    for (int cand : {128, 112, 96, 80, 64, 48, 32, 16}) {
        if (panel_smem_bytes<F>(R, cand) <= budget) { b = cand; break; }
    }
    if (b == 0) {
        set_error("matrix too tall for the panel kernel: %lld rows", (long long)m);
        return LNC_ERR_UNSUPPORTED;
    }
    if constexpr (F::kDtype == 2) {  // 64-bit residues: the tensor-core update takes 64-column panels
        if (trailing_tc_u64_available()) b = std::min(b, kMaxPanelU64Tc);
    }
    // look-ahead pays once a trailing update outlasts a candidate panel: matrices of >= 2^22 entries
    // with at least three panels, on the tensor-core path
    bool la = false;
    if constexpr (F::kDtype == 1) la = b == kMaxPanel && trailing_tc_u32_available();
    if constexpr (F::kDtype == 2) la = b == kPanelU64 && trailing_tc_u64_available();
    plan->lookahead_ok = la;
    plan->lookahead = la && m * n >= ((int64_t)1 << 22) && n > 2 * (int64_t)b;
    plan->G = G;
    plan->rows_per_cta = R;
    plan->b = b;
    plan->smem = panel_smem_bytes<F>(R, std::min<int64_t>(b, n));
    return LNC_OK;
}

// scratch of the candidate-panel path (32-bit residues)
static size_t fast_extra_scratch(int64_t m, int64_t n) {
    return align_up(sizeof(uint32_t) * kMaxPanel * kMaxPanel, 256)  // X
           + align_up(sizeof(int32_t) * 256, 256)                     // candidate rows
           + 256                                                      // cand_n, next_row, missed, pivmask
           + align_up(sizeof(int32_t) * kMaxPanel, 256)               // panel_cols
           + align_up(sizeof(int32_t) * (size_t)m, 256)               // panel_mark
           + align_up(sizeof(int32_t) * (size_t)std::max<int64_t>(n, 1), 256);  // column -> pivot row
}

// Look-ahead of the candidate-panel path.  While the caller's stream applies
// panel q to the columns beyond panel q + 1, a second stream (highest
// priority, so its one-CTA panel takes the first SM that frees up) runs panel
// q + 1: candidate block, E = G X and the digit split of E.  That needs its
// own G digits, a second E digit buffer (panel q's is still being read), its
// own X digits and a second pivot-count word; the exhaustive fallback of a
// panel that missed a pivot gets its own transform, pivot rows, count and
// digit scratch, because its correction of the far columns runs after the
// fork, next to panel q + 1.
template <class F>
static size_t lookahead_scratch(int64_t m, int64_t n, const RrefPlan& pl) {
    using T = typename F::T;
    constexpr bool U64 = F::kDtype == 2;
    constexpr int PW = U64 ? kPanelU64 : kMaxPanel;
    const size_t el = U64 ? tc64_el_bytes(m) : tc_el_bytes(m);
    const size_t bsx = U64 ? tc64_bs_bytes(PW) : tc_bs_bytes(PW);
    return 2 * (el + 1024) + bsx + 1024                      // G digits, second E digits, X digits
           + align_up(sizeof(T) * (size_t)m * PW, 256)       // fallback transform
           + align_up(sizeof(int32_t) * PW, 256) + 256       // fallback pivot rows; pivot counts
           + trailing_extra_scratch<F>(m, n, pl) + 256;      // fallback digit scratch
}

struct LookaheadStreams {
    int dev = -1;
    cudaStream_t main = nullptr;
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
};
static std::mutex g_la_mu;
static std::vector<LookaheadStreams> g_la;

// The side stream and fork / join events of a caller's stream, created on first
// use and kept for the process (calls on one stream come from one thread at a time).
static int lookahead_streams(cudaStream_t main, LookaheadStreams* out) {
    int dev = 0;
    LNC_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> g(g_la_mu);
    for (const auto& x : g_la)
        if (x.dev == dev && x.main == main) { *out = x; return LNC_OK; }
    LookaheadStreams x;
    x.dev = dev;
    x.main = main;
    int lo = 0, hi = 0;
    LNC_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    LNC_CUDA(cudaStreamCreateWithPriority(&x.side, cudaStreamNonBlocking, hi));
    LNC_CUDA(cudaEventCreateWithFlags(&x.fork, cudaEventDisableTiming));
    LNC_CUDA(cudaEventCreateWithFlags(&x.join, cudaEventDisableTiming));
    g_la.push_back(x);
    *out = x;
    return LNC_OK;
}

// Pivots may be found out of column order when a candidate panel is redone by
// the exhaustive panel: order the (row, column) lists by column (one CTA).
__global__ void __launch_bounds__(1024) sort_pivots_kernel(int32_t* piv_row, int64_t* piv_col, const int64_t* rank_p,
                                                           int64_t n, int32_t* col_row) {
    __shared__ int s_warp[32];
    __shared__ int s_base, s_total;
    const int64_t rank = *rank_p;
    for (int64_t c = threadIdx.x; c < n; c += blockDim.x) col_row[c] = -1;
    __syncthreads();
    for (int64_t i = threadIdx.x; i < rank; i += blockDim.x) col_row[piv_col[i]] = piv_row[i];
    if (threadIdx.x == 0) s_base = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int64_t c0 = 0; c0 < n; c0 += blockDim.x) {
        const int64_t c = c0 + threadIdx.x;
        const int32_t r = (c < n) ? col_row[c] : -1;
        const int flag = r >= 0;
        const unsigned ballot = __ballot_sync(0xffffffffu, flag);
        if (lane == 0) s_warp[warp] = __popc(ballot);
        __syncthreads();
        if (threadIdx.x == 0) {
            int acc = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
                const int v = s_warp[w];
                s_warp[w] = acc;
                acc += v;
            }
            s_total = acc;
        }
        __syncthreads();
        const int pos = s_base + s_warp[warp] + __popc(ballot & ((1u << lane) - 1u));
        if (flag) {
            piv_row[pos] = r;
            piv_col[pos] = c;
        }
        __syncthreads();
        if (threadIdx.x == 0) s_base += s_total;
        __syncthreads();
    }
}

template <class F>
size_t rref_scratch_bytes(int64_t m, int64_t n, const RrefPlan& pl) {
    using T = typename F::T;
    const int64_t kmax = std::min(m, n);
    size_t s = 0;
    s += align_up((size_t)m, 256);                              // row_used
    s += align_up(sizeof(int32_t) * (size_t)std::max<int64_t>(kmax, 1), 256);  // piv_row
    s += align_up(sizeof(int64_t) * (size_t)std::max<int64_t>(kmax, 1), 256);  // piv_col
    s += 256;                                                   // scalars
    s += align_up(sizeof(int32_t) * kMaxPanel, 256);            // panel_rows
    s += align_up(sizeof(typename F::Key) * 2 * pl.G, 256);     // cand_key
    s += align_up(sizeof(int64_t) * 2 * pl.G, 256);             // cand_row
    s += align_up(sizeof(T) * 2 * (size_t)pl.G * pl.b, 256);    // cand_vals
    s += align_up(sizeof(T) * (size_t)m * pl.b, 256);           // E
    s += align_up(sizeof(T) * (size_t)pl.b * (size_t)std::max<int64_t>(n, 1), 256);  // Bm
    s += trailing_extra_scratch<F>(m, n, pl);
    if constexpr (F::kDtype == 1 || F::kDtype == 2) {
        s += fast_extra_scratch(m, n);
        if (pl.lookahead) s += lookahead_scratch<F>(m, n, pl);
    }
    return s;
}

// Extra state of a mixed-precision float solve: the row-scaled input kept
// for the refinement residuals, every panel's transform (E columns and pivot
// rows, which define the elimination's product of transforms M), the
// fixed-point update scratch and the uncertain-rank-decision flag.
template <class T>
struct MixedCtx {
    T* As = nullptr;           // m x n
    T* E_all = nullptr;        // m x ldE, panel q in columns [q b, q b + b)
    int64_t ldE = 0;
    int32_t* P_all = nullptr;  // pivot rows of panel q at [q b, q b + b)
    int32_t* K_all = nullptr;  // pivots of panel q
    void* fx = nullptr;
    int* uncertain = nullptr;
};

template <class F>
int rref_run(const F& f, typename F::T* A, int64_t m, int64_t n, int64_t lda, typename F::T* out,
             int64_t ldo, int64_t* dev_piv, int64_t* dev_rank, cudaStream_t s, int flags,
             void* scratch, size_t scratch_bytes, const RrefPlan& pl,
             MixedCtx<typename F::T>* mx = nullptr) {
    using T = typename F::T;
    const int64_t kmax = std::min(m, n);
    // carve scratch
    unsigned char* p = (unsigned char*)scratch;
    auto take = [&](size_t bytes) { void* r = p; p += align_up(bytes, 256); return r; };
    uint8_t* row_used = (uint8_t*)take((size_t)m);
    int32_t* piv_row = (int32_t*)take(sizeof(int32_t) * (size_t)std::max<int64_t>(kmax, 1));
    int64_t* piv_col = (int64_t*)take(sizeof(int64_t) * (size_t)std::max<int64_t>(kmax, 1));
    unsigned char* scal = (unsigned char*)take(256);
    int64_t* rank = (int64_t*)scal;
    int32_t* panel_k = (int32_t*)(scal + 8);
    unsigned* bar_count = (unsigned*)(scal + 16);
    unsigned* bar_gen = (unsigned*)(scal + 20);
    int* err = (int*)(scal + 24);
    int32_t* panel_rows = (int32_t*)take(sizeof(int32_t) * kMaxPanel);
    typename F::Key* cand_key = (typename F::Key*)take(sizeof(typename F::Key) * 2 * pl.G);
    int64_t* cand_row = (int64_t*)take(sizeof(int64_t) * 2 * pl.G);
    T* cand_vals = (T*)take(sizeof(T) * 2 * (size_t)pl.G * pl.b);
    T* E = (T*)take(sizeof(T) * (size_t)m * pl.b);
    T* Bm = (T*)take(sizeof(T) * (size_t)pl.b * (size_t)std::max<int64_t>(n, 1));
    void* extra = (void*)p;
    if ((size_t)(p - (unsigned char*)scratch) > scratch_bytes) {
        set_error("internal: scratch layout overflow");
        return LNC_ERR_INVALID;
    }
    int* status = rref_status_symbol_address();
    if (!status) { set_error("cannot resolve the status word"); return LNC_ERR_CUDA; }

    LNC_CUDA(cudaMemsetAsync(row_used, 0, (size_t)m, s));
    LNC_CUDA(cudaMemsetAsync(scal, 0, 256, s));

    // input preparation
    {
        dim3 grid((unsigned)std::min<int64_t>((n + 255) / 256, 64), (unsigned)std::min<int64_t>(m, 65535));
        if constexpr (F::kDtype == 1 || F::kDtype == 2) {
            reduce_input_kernel<F><<<grid, 256, 0, s>>>(f, A, lda, m, n);
            LNC_CHECK_LAUNCH("reduce_input_kernel");
        } else {
            if (!(flags & LNC_FLAG_NO_SCALING)) {
                row_scale_kernel<F><<<(unsigned)std::min<int64_t>(m, 65535), 256, 0, s>>>(f, A, lda, m, n);
                LNC_CHECK_LAUNCH("row_scale_kernel");
            }
            if (mx)
                LNC_CUDA(cudaMemcpy2DAsync(mx->As, sizeof(T) * n, A, sizeof(T) * lda, sizeof(T) * n, m,
                                           cudaMemcpyDeviceToDevice, s));
        }
    }

    auto kpanel = panel_kernel<F>;
    const size_t smem_max = panel_smem_bytes<F>(pl.rows_per_cta, pl.b);
    {
        int rc0 = allow_dynamic_smem((const void*)kpanel, smem_max);
        if (rc0) return rc0;
    }

    TrailingCtx<F> tctx;
    tctx.f = f;
    tctx.m = m;
    tctx.n = n;
    tctx.A = A;
    tctx.lda = lda;
    tctx.E = E;
    tctx.ldE = pl.b;
    tctx.Bm = Bm;
    tctx.panel_k = panel_k;
    tctx.panel_rows = panel_rows;
    tctx.err = err;
    tctx.status = status;
    tctx.extra = extra;
    tctx.b = pl.b;
    tctx.force_simt = (flags & LNC_FLAG_SIMT_TRAILING) != 0;
    if (mx) tctx.fx = mx->fx;

    auto make_panel_args = [&](int64_t j0, int bw, bool with_e, const int* run_if) {
        PanelArgs<F> pa;
        pa.f = f;
        pa.A = A;
        pa.lda = lda;
        pa.m = m;
        pa.j0 = j0;
        pa.bw = bw;
        pa.b = pl.b;
        pa.row_used = row_used;
        pa.rank = rank;
        pa.piv_row = piv_row;
        pa.piv_col = piv_col;
        pa.panel_k = panel_k;
        pa.panel_rows = panel_rows;
        pa.E = with_e ? E : nullptr;
        pa.ldE = pl.b;
        pa.cand_key = cand_key;
        pa.cand_row = cand_row;
        pa.cand_vals = cand_vals;
        pa.bar.count = bar_count;
        pa.bar.gen = bar_gen;
        pa.bar.err = err;
        pa.bar.status = status;
        pa.rows_per_cta = pl.rows_per_cta;
        pa.run_if = run_if;
        return pa;
    };
    auto launch_panel = [&](PanelArgs<F>& pa) -> int {
        ScopedKernelTimer kt(KC_PANEL, s, pa.run_if ? 0.0 : 2.0 * (double)m * pa.bw * sizeof(T));
        void* args[] = {&pa};
        const size_t smem = panel_smem_bytes<F>(pl.rows_per_cta, pa.bw);
        LNC_CUDA(cudaLaunchCooperativeKernel((const void*)kpanel, dim3(pl.G), dim3(kPanelThreads), args, smem, s));
        LNC_CHECK_LAUNCH("panel_kernel");
        return LNC_OK;
    };

    bool fast = false;
    const bool defer = (flags & LNC_FLAG_DEFER_FALLBACK) != 0;
    int* defer_missed = nullptr;
    if constexpr (F::kDtype == 1) {
        fast = !(flags & (LNC_FLAG_SIMT_TRAILING | LNC_FLAG_ROBUST_PANEL)) && pl.b == kMaxPanel &&
               trailing_tc_u32_available();
    }
    if constexpr (F::kDtype == 2) {
        fast = !(flags & (LNC_FLAG_SIMT_TRAILING | LNC_FLAG_ROBUST_PANEL)) && pl.b == kPanelU64 &&
               trailing_tc_u64_available();
    }
    if (fast) {
        if constexpr (F::kDtype == 1 || F::kDtype == 2) {
            constexpr bool U64 = F::kDtype == 2;
            constexpr int PW = U64 ? kPanelU64 : kMaxPanel;  // panel width (contraction depth)
            // ---------------- candidate-block panels + tensor-core updates
            unsigned char* fx = (unsigned char*)extra + trailing_extra_scratch<F>(m, n, pl);
            fx = (unsigned char*)(((uintptr_t)fx + 255) & ~(uintptr_t)255);
            auto takef = [&](size_t bytes) { void* r = fx; fx += align_up(bytes, 256); return r; };
            T* Xbuf = (T*)takef(sizeof(T) * PW * PW);
            int32_t* cand = (int32_t*)takef(sizeof(int32_t) * 256);
            unsigned char* fscal = (unsigned char*)takef(256);
            int32_t* cand_n = (int32_t*)fscal;
            int32_t* next_row = (int32_t*)(fscal + 4);
            int* missed = (int*)(fscal + 8);
            int* missed_any = (int*)(fscal + 12);  // sticky miss flag of a deferred-fallback solve
            uint32_t* pivmask = (uint32_t*)(fscal + 16);
            defer_missed = missed_any;
            int32_t* panel_cols = (int32_t*)takef(sizeof(int32_t) * kMaxPanel);
            int32_t* panel_mark = (int32_t*)takef(sizeof(int32_t) * (size_t)m);
            int32_t* col_row = (int32_t*)takef(sizeof(int32_t) * (size_t)std::max<int64_t>(n, 1));
            if ((size_t)(fx - (unsigned char*)scratch) > scratch_bytes) {
                set_error("internal: scratch layout overflow (fast path)");
                return LNC_ERR_INVALID;
            }
            LNC_CUDA(cudaMemsetAsync(fscal, 0, 256, s));
            LNC_CUDA(cudaMemsetAsync(panel_mark, 0, sizeof(int32_t) * (size_t)m, s));
            unsigned char* tcb = (unsigned char*)(((uintptr_t)extra + 1023) & ~(uintptr_t)1023);
            void* EL = tcb;
            void* BS = U64 ? tc64_bs_base(extra, m) : (void*)(tcb + tc_el_bytes(m));
            CandArgs ca;
            ca.A = A;
            ca.lda = lda;
            ca.m = m;
            ca.smax = kCandRows;
            ca.row_used = row_used;
            ca.cand = cand;
            ca.cand_n = cand_n;
            ca.next_row = next_row;
            ca.rank = rank;
            ca.piv_row = piv_row;
            ca.piv_col = piv_col;
            ca.panel_k = panel_k;
            ca.panel_rows = panel_rows;
            ca.panel_cols = panel_cols;
            ca.panel_mark = panel_mark;
            ca.X = Xbuf;
            ca.pivmask = pivmask;
            ca.missed = missed;
            if constexpr (U64) {
                ca.f64 = f;
            } else {
                const uint32_t pp = f.p;
                uint32_t x = pp;
                for (int i = 0; i < 5; ++i) x *= 2u - pp * x;
                ca.M.p = pp;
                ca.M.pinv = 0u - x;
                ca.M.r2 = (uint32_t)((((unsigned __int128)1) << 64) % pp);
                ca.M.mu = f.mu;
            }
            // ---- look-ahead buffers (without look-ahead they alias the single-stream ones)
            const bool la = pl.lookahead && !(flags & LNC_FLAG_NO_LOOKAHEAD);
            LookaheadStreams ls;
            void* ELG = EL;            // G digits of E = G X
            void* ELE[2] = {EL, EL};   // E digits of panels q even / odd
            void* BSX = BS;            // X digits
            int32_t* pk[2] = {panel_k, panel_k};
            T* Efb = E;                // exhaustive fallback: transform, pivot rows, count, digit scratch
            int32_t* prow_fb = panel_rows;
            int32_t* pk_fb = panel_k;
            void* fb_extra = extra;
            if (la) {
                int rc0 = lookahead_streams(s, &ls);
                if (rc0) return rc0;
                const size_t el = U64 ? tc64_el_bytes(m) : tc_el_bytes(m);
                const size_t bsx = U64 ? tc64_bs_bytes(PW) : tc_bs_bytes(PW);
                auto take1k = [&](size_t bytes) {
                    fx = (unsigned char*)(((uintptr_t)fx + 1023) & ~(uintptr_t)1023);
                    void* r = fx;
                    fx += bytes;
                    return r;
                };
                ELG = take1k(el);
                ELE[1] = take1k(el);
                BSX = take1k(bsx);
                fx = (unsigned char*)(((uintptr_t)fx + 255) & ~(uintptr_t)255);
                Efb = (T*)takef(sizeof(T) * (size_t)m * PW);
                prow_fb = (int32_t*)takef(sizeof(int32_t) * PW);
                int32_t* ks = (int32_t*)takef(256);
                pk[1] = ks;
                pk_fb = ks + 1;
                fb_extra = takef(trailing_extra_scratch<F>(m, n, pl));
                if ((size_t)(fx - (unsigned char*)scratch) > scratch_bytes) {
                    set_error("internal: scratch layout overflow (look-ahead)");
                    return LNC_ERR_INVALID;
                }
            }
            TrailingCtx<F> tfb = tctx;  // correction of a redone panel
            tfb.E = Efb;
            tfb.panel_k = pk_fb;
            tfb.panel_rows = prow_fb;
            tfb.extra = fb_extra;
            tfb.predicated = true;

            // panel q on stream st: candidate block, G and X digits, E = G X, E digits
            auto panel_chain = [&](int64_t pj0, int q, cudaStream_t st) -> int {
                ca.j0 = pj0;
                ca.bw = (int)std::min<int64_t>(PW, n - pj0);
                ca.gen = q + 1;
                ca.panel_k = pk[q & 1];
                const int32_t* kq = pk[q & 1];
                int rc = LNC_OK;
                if constexpr (U64) {
                    rc = launch_cand_panel64(ca, st);
                    if (!rc) rc = tc64_split_g(A, lda, m, pj0, f.p, kq, panel_cols, panel_mark, q + 1, ELG, st);
                    if (!rc) rc = tc64_gather_split_b(Xbuf, PW, PW, nullptr, kq, f.p, BSX, false, st);
                    if (!rc) rc = tc64_limb_gemm(f, E, PW, m, PW, kq, true, ELG, BSX, err, status, st, true, PW);
                    if (!rc) rc = tc64_split_e(E, PW, m, f.p, kq, ELE[q & 1], st);
                } else {
                    rc = launch_cand_panel(ca, st);
                    if (!rc) rc = launch_split_g(A, lda, m, pj0, f.p, kq, panel_cols, panel_mark, q + 1, ELG, st);
                    if (!rc) rc = tc_gather_split_b(Xbuf, kMaxPanel, kMaxPanel, nullptr, kq, f.p, BSX, false, st);
                    if (!rc) rc = tc_limb_gemm(f, E, kMaxPanel, m, kMaxPanel, kq, true, ELG, BSX, kMaxPanel, err,
                                               status, st);
                    if (!rc) rc = tc_split_e(E, kMaxPanel, kMaxPanel, m, f.p, kq, ELE[q & 1], st);
                }
                return rc;
            };
            // C[:, c0:c0+N) += E B for the columns of B's digit tiles from column offset off
            auto apply = [&](int q, int64_t c0, int64_t N, int64_t off, int tpc, cudaStream_t st) -> int {
                const int32_t* kq = pk[q & 1];
                if constexpr (U64) {
                    void* B = (unsigned char*)BS + tc64_bs_bytes(off);
                    return tc64_limb_gemm(f, A + c0, lda, m, N, kq, false, ELE[q & 1], B, err, status, st, true, PW,
                                          tpc);
                } else {
                    void* B = (unsigned char*)BS + tc_bs_bytes(off);
                    return tc_limb_gemm(f, A + c0, lda, m, N, kq, false, ELE[q & 1], B, N, err, status, st, true,
                                        tpc);
                }
            };

            int rc = panel_chain(0, 0, s);
            if (rc) return rc;
            int q = 0;
            for (int64_t j0 = 0; j0 < n; j0 += PW, ++q) {
                const int bw = (int)std::min<int64_t>(PW, n - j0);
                const int64_t j1 = j0 + bw;
                // columns updated before the fork: this panel's and the next one's (all of them without look-ahead)
                const int64_t j2 = la ? std::min<int64_t>(j1 + PW, n) : n;
                const int32_t* kq = pk[q & 1];
                int* miss = defer ? missed_any : missed;
                // A[:, j0:] += E A[P, j0:]  (pivot rows gathered and zeroed first)
                if constexpr (U64) {
                    rc = tc64_gather_split_b(A + j0, lda, n - j0, panel_rows, kq, f.p, BS, true, s);
                } else {
                    rc = tc_gather_split_b(A + j0, lda, n - j0, panel_rows, kq, f.p, BS, true, s);
                }
                if (!rc) rc = apply(q, j0, j2 - j0, 0, la ? 2 : 0, s);
                if (!rc) {
                    if constexpr (U64) rc = launch_check_missed64(A, lda, m, j0, bw, row_used, pivmask, miss, s);
                    else rc = launch_check_missed(A, lda, m, j0, bw, row_used, pivmask, miss, s);
                }
                if (rc) return rc;
                if (!defer) {
                    // redo the panel exhaustively when the candidate block missed a pivot
                    PanelArgs<F> pa = make_panel_args(j0, bw, j1 < n, missed);
                    pa.E = Efb;
                    pa.panel_k = pk_fb;
                    pa.panel_rows = prow_fb;
                    rc = launch_panel(pa);
                    if (!rc && j1 < n) {
                        tfb.j1 = j1;
                        tfb.N = j2 - j1;
                        tfb.ldb = tfb.N;
                        rc = trailing_update<F>(tfb, s);
                    }
                    if (rc) return rc;
                }
                if (j1 >= n) break;
                if (!la) {
                    rc = panel_chain(j1, q + 1, s);
                    if (rc) return rc;
                    continue;
                }
                // fork: panel q + 1 on the side stream, columns [j2, n) of panel q here
                LNC_CUDA(cudaEventRecord(ls.fork, s));
                LNC_CUDA(cudaStreamWaitEvent(ls.side, ls.fork, 0));
                rc = panel_chain(j1, q + 1, ls.side);
                const cudaError_t ej = cudaEventRecord(ls.join, ls.side);
                if (!rc && j2 < n) {
                    // 16 tiles per CTA, not the wave-fitted count: many short CTAs free SMs for the
                    // side stream's cluster more often than a grid of exactly filled waves
                    rc = apply(q, j2, n - j2, j2 - j0, 16, s);
                    if (!rc && !defer) {
                        tfb.j1 = j2;
                        tfb.N = n - j2;
                        tfb.ldb = tfb.N;
                        rc = trailing_update<F>(tfb, s);
                    }
                }
                // join (also on failure, so a capture never ends with the side stream's work unjoined)
                const cudaError_t ew = (ej == cudaSuccess) ? cudaStreamWaitEvent(s, ls.join, 0) : ej;
                if (rc) return rc;
                if (ew != cudaSuccess) return cuda_status(ew, "look-ahead join");
            }
            sort_pivots_kernel<<<1, 1024, 0, s>>>(piv_row, piv_col, rank, n, col_row);
            LNC_CHECK_LAUNCH("sort_pivots_kernel");
        }
    } else {
        for (int64_t j0 = 0; j0 < n; j0 += pl.b) {
            const int bw = (int)std::min<int64_t>(pl.b, n - j0);
            const int64_t j1 = j0 + bw;
            const int64_t N = n - j1;
            PanelArgs<F> pa = make_panel_args(j0, bw, N > 0 || mx != nullptr, nullptr);
            if constexpr (F::kDtype >= 3) {
                if (mx) {  // keep every panel's transform for the refinement
                    const int64_t q = j0 / pl.b;
                    pa.E = mx->E_all + q * pl.b;
                    pa.ldE = mx->ldE;
                    pa.panel_k = mx->K_all + q;
                    pa.panel_rows = mx->P_all + q * pl.b;
                    pa.uncertain = mx->uncertain;
                    pa.band_lo = 1e-3 * f.tol;
                    pa.band_hi = 1e5 * f.tol;  // well above the fixed-point updates' noise
                    tctx.E = pa.E;
                    tctx.ldE = pa.ldE;
                    tctx.panel_k = pa.panel_k;
                    tctx.panel_rows = pa.panel_rows;
                }
            }
            int rc = launch_panel(pa);
            if (rc) return rc;
            if (N > 0) {
                tctx.j1 = j1;
                tctx.N = N;
                tctx.ldb = N;
                rc = trailing_update<F>(tctx, s);
                if (rc) return rc;
            }
        }
    }
    {
        ScopedKernelTimer kt(KC_GATHER, s, 2.0 * (double)m * (double)n * sizeof(T));
        dim3 grid((unsigned)std::min<int64_t>((n + 255) / 256, 16), (unsigned)std::min<int64_t>(m, 65535));
        T zero;
        memset(&zero, 0, sizeof(T));
        gather_rref_rows_kernel<T><<<grid, 256, 0, s>>>(A, lda, out, ldo, m, n, piv_row, rank, zero);
        LNC_CHECK_LAUNCH("gather_rref_rows_kernel");
    }
    if (dev_piv || dev_rank) {
        copy_pivots_kernel<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>((kmax + 255) / 256, 1024)), 256, 0, s>>>(
            piv_col, rank, kmax, dev_piv, dev_rank);
        LNC_CHECK_LAUNCH("copy_pivots_kernel");
    }
    publish_status_kernel<<<1, 1, 0, s>>>(err, status);
    LNC_CHECK_LAUNCH("publish_status_kernel");
    if (defer && dev_rank) {
        publish_deferred_kernel<<<1, 1, 0, s>>>(err, defer_missed, dev_rank);
        LNC_CHECK_LAUNCH("publish_deferred_kernel");
    }
    return LNC_OK;
}

// ----------------------------------------------------------------------------
// SIMT trailing update dispatch (the tensor-core path lives in trailing_tc.cu)
// ----------------------------------------------------------------------------
template <class F>
int trailing_update_simt(const TrailingCtx<F>& t, cudaStream_t s) {
    {
        dim3 g((unsigned)std::min<int64_t>((t.N + 255) / 256, 1024), (unsigned)t.b);
        gather_pivot_rows_kernel<F><<<g, 256, 0, s>>>(t.f, t.A, t.lda, t.j1, t.N, t.panel_rows, t.panel_k,
                                                     const_cast<typename F::T*>(t.Bm), t.ldb);
        LNC_CHECK_LAUNCH("gather_pivot_rows_kernel");
    }
    dim3 grid((unsigned)((t.N + 127) / 128), (unsigned)((t.m + 63) / 64));
    if (grid.y > 65535) { set_error("trailing update: too many row tiles"); return LNC_ERR_UNSUPPORTED; }
    ScopedKernelTimer kt(KC_TRAILING, s, (double)t.m * (double)t.N * (double)t.b);
    if constexpr (F::kDtype == 1) {
        if (t.f.p < (1u << 31))
            trailing_simt_kernel<F, 32, 4><<<grid, 256, 0, s>>>(t.f, t.A, t.lda, t.m, t.j1, t.N, t.E, t.ldE, t.Bm, t.ldb, t.panel_k);
        else
            trailing_simt_kernel<F, 32, 1><<<grid, 256, 0, s>>>(t.f, t.A, t.lda, t.m, t.j1, t.N, t.E, t.ldE, t.Bm, t.ldb, t.panel_k);
    } else if constexpr (F::kDtype == 4) {
        trailing_simt_kernel<F, 8, 1><<<grid, 256, 0, s>>>(t.f, t.A, t.lda, t.m, t.j1, t.N, t.E, t.ldE, t.Bm, t.ldb, t.panel_k);
    } else {
        trailing_simt_kernel<F, 16, 1><<<grid, 256, 0, s>>>(t.f, t.A, t.lda, t.m, t.j1, t.N, t.E, t.ldE, t.Bm, t.ldb, t.panel_k);
    }
    LNC_CHECK_LAUNCH("trailing_simt_kernel");
    return LNC_OK;
}

template int trailing_update_simt<FieldU32>(const TrailingCtx<FieldU32>&, cudaStream_t);
template int trailing_update_simt<FieldU64>(const TrailingCtx<FieldU64>&, cudaStream_t);
template int trailing_update_simt<FieldF64>(const TrailingCtx<FieldF64>&, cudaStream_t);
template int trailing_update_simt<FieldC128>(const TrailingCtx<FieldC128>&, cudaStream_t);

// ----------------------------------------------------------------------------
// public entry (dtype dispatch, scratch allocation)
// ----------------------------------------------------------------------------
template <class F>
static int rref_device_typed(const F& f, void* work, int64_t ldw, void* out, int64_t ldo, int64_t m,
                             int64_t n, int64_t* dev_piv, int64_t* dev_rank, cudaStream_t s, int flags) {
    using T = typename F::T;
    RrefPlan pl;
    int rc = plan_rref<F>(m, n, &pl);
    if (rc) return rc;
    if ((flags & LNC_FLAG_LOOKAHEAD) && pl.lookahead_ok && n > 2 * (int64_t)pl.b) pl.lookahead = true;
    size_t sb = rref_scratch_bytes<F>(m, n, pl);
    const bool in_place = (out == work);
    if (in_place) sb += align_up(sizeof(T) * (size_t)m * (size_t)n, 256);
    void* scratch = nullptr;
    cudaError_t e = cudaMallocAsync(&scratch, sb, s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("device scratch allocation of %zu bytes failed: %s", sb, cudaGetErrorString(e));
        return LNC_ERR_OOM;
    }
    T* out_t = (T*)out;
    int64_t ldo_t = ldo;
    T* tmp = nullptr;
    if (in_place) {
        tmp = (T*)((unsigned char*)scratch + rref_scratch_bytes<F>(m, n, pl));
        out_t = tmp;
        ldo_t = n;
    }
    rc = rref_run<F>(f, (T*)work, m, n, ldw, out_t, ldo_t, dev_piv, dev_rank, s, flags, scratch,
                     rref_scratch_bytes<F>(m, n, pl), pl);
    if (rc == LNC_OK && in_place) {
        e = cudaMemcpy2DAsync(out, sizeof(T) * ldo, tmp, sizeof(T) * n, sizeof(T) * n, m,
                              cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) rc = cuda_status(e, "cudaMemcpy2DAsync");
    }
    cudaFreeAsync(scratch, s);
    return rc;
}

// ----------------------------------------------------------------------------
// mixed-precision float solve: fixed-point tensor-core elimination, then FP64
// refinement of the non-pivot columns (see trailing_fx.cu)
// ----------------------------------------------------------------------------
struct MixedReport {
    int iterations = 0;
    double last_correction = 0.0;
    int redone = 0;
    double error_estimate = 0.0;  // -1 when the solve was redone in FP64 (not estimated)
};
static thread_local MixedReport t_mixed;

template <class F>
static int rref_mixed_typed(const F& f, void* work, int64_t ldw, void* out, int64_t ldo, int64_t m, int64_t n,
                            int64_t* dev_piv, int64_t* dev_rank, cudaStream_t s, int flags) {
    using T = typename F::T;
    constexpr bool CPLX = F::kDtype == LNC_C128;
    t_mixed = MixedReport();
    RrefPlan pl;
    int rc = plan_rref<F>(m, n, &pl);
    if (rc) return rc;
    if (CPLX && pl.b > 64) {  // realified contraction depth 2b <= 128
        pl.b = 64;
        pl.smem = panel_smem_bytes<F>(pl.rows_per_cta, (int)std::min<int64_t>(pl.b, n));
    }
    if (flags & LNC_FLAG_NO_SCALING) { set_error("mixed precision needs the row scaling"); return LNC_ERR_INVALID; }
    const int64_t panels = (n + pl.b - 1) / pl.b;
    const int64_t kmax = std::min(m, n);
    const size_t sb = rref_scratch_bytes<F>(m, n, pl);
    const size_t as_b = align_up(sizeof(T) * (size_t)m * n, 256);
    const size_t e_b = align_up(sizeof(T) * (size_t)m * panels * pl.b, 256);
    const size_t p_b = align_up(sizeof(int32_t) * (size_t)panels * pl.b, 256);
    const size_t k_b = align_up(sizeof(int32_t) * (size_t)panels, 256);
    const size_t fx_b = align_up(trailing_fx_scratch(m, n, CPLX), 256);
    const size_t out_b = align_up(sizeof(T) * (size_t)m * n, 256);  // out of place result
    const size_t total = sb + as_b + e_b + p_b + k_b + fx_b + out_b + 256;
    unsigned char* blk = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&blk, total, s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("mixed-precision scratch of %zu bytes: %s", total, cudaGetErrorString(e));
        return LNC_ERR_OOM;
    }
    unsigned char* q = blk + sb;
    MixedCtx<T> mx;
    mx.As = (T*)q; q += as_b;
    mx.E_all = (T*)q; q += e_b;
    mx.ldE = panels * pl.b;
    mx.P_all = (int32_t*)q; q += p_b;
    mx.K_all = (int32_t*)q; q += k_b;
    mx.fx = q; q += fx_b;
    T* R = (T*)q; q += out_b;
    mx.uncertain = (int*)q;
    auto fail = [&](int code) { cudaFreeAsync(blk, s); return code; };
    LNC_CUDA(cudaMemsetAsync(mx.uncertain, 0, 256, s));
    LNC_CUDA(cudaMemsetAsync(mx.K_all, 0, sizeof(int32_t) * panels, s));
    const int run_flags = flags & ~(LNC_FLAG_MIXED | LNC_FLAG_DEFER_FALLBACK);
    rc = rref_run<F>(f, (T*)work, m, n, ldw, R, n, nullptr, nullptr, s, run_flags, blk, sb, pl, &mx);
    if (rc) return fail(rc);
    // pivots of the mixed elimination (scratch layout of rref_run: row_used, piv_row, piv_col, scalars)
    unsigned char* sp = blk;
    sp += align_up((size_t)m, 256);
    int32_t* piv_row = (int32_t*)sp;
    sp += align_up(sizeof(int32_t) * (size_t)std::max<int64_t>(kmax, 1), 256);
    int64_t* piv_col = (int64_t*)sp;
    sp += align_up(sizeof(int64_t) * (size_t)std::max<int64_t>(kmax, 1), 256);
    int64_t* rank_d = (int64_t*)sp;
    int64_t rank = 0;
    int unc = 0;
    LNC_CUDA(cudaMemcpyAsync(&rank, rank_d, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    LNC_CUDA(cudaMemcpyAsync(&unc, mx.uncertain, sizeof(int), cudaMemcpyDeviceToHost, s));
    LNC_CUDA(cudaStreamSynchronize(s));
    if (unc) {
        // a rank decision within reach of the reduced precision: redo in FP64 from the scaled input
        t_mixed.redone = 1;
        t_mixed.error_estimate = -1.0;
        LNC_CUDA(cudaMemcpy2DAsync(work, sizeof(T) * ldw, mx.As, sizeof(T) * n, sizeof(T) * n, m,
                                   cudaMemcpyDeviceToDevice, s));
        rc = rref_run<F>(f, (T*)work, m, n, ldw, R, n, nullptr, nullptr, s, run_flags | LNC_FLAG_NO_SCALING, blk,
                         sb, pl);
        if (rc) return fail(rc);
        LNC_CUDA(cudaMemcpyAsync(&rank, rank_d, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        LNC_CUDA(cudaStreamSynchronize(s));
    } else if (rank > 0 && rank < n) {
        // ---- FP64 refinement of the non-pivot columns
        const int qn = (int)(n - rank);
        std::vector<int64_t> pc((size_t)rank);
        LNC_CUDA(cudaMemcpy(pc.data(), piv_col, sizeof(int64_t) * rank, cudaMemcpyDeviceToHost));
        std::vector<int32_t> colmap((size_t)n, -1), nc;
        nc.reserve((size_t)qn);
        for (int64_t t = 0; t < rank; ++t) colmap[(size_t)pc[(size_t)t]] = (int32_t)t;
        for (int64_t c = 0; c < n; ++c)
            if (colmap[(size_t)c] < 0) nc.push_back((int32_t)c);
        const size_t z_b = align_up(sizeof(T) * (size_t)n * qn, 256);
        const size_t r_b = align_up(sizeof(T) * (size_t)m * qn, 256);
        const size_t g_b = align_up(sizeof(T) * (size_t)pl.b * qn, 256);
        const size_t i_b = align_up(sizeof(int32_t) * (size_t)(n + qn), 256);
        unsigned char* rb = nullptr;
        e = cudaMallocAsync((void**)&rb, z_b + r_b + g_b + i_b + 256, s);
        if (e != cudaSuccess) {
            cudaGetLastError();
            set_error("refinement scratch: %s", cudaGetErrorString(e));
            return fail(LNC_ERR_OOM);
        }
        T* Z = (T*)rb;
        T* Res = (T*)(rb + z_b);
        T* Bg = (T*)(rb + z_b + r_b);
        int32_t* d_colmap = (int32_t*)(rb + z_b + r_b + g_b);
        int32_t* d_nc = d_colmap + n;
        unsigned long long* stats = (unsigned long long*)(rb + z_b + r_b + g_b + i_b);
        LNC_CUDA(cudaMemcpyAsync(d_colmap, colmap.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, s));
        LNC_CUDA(cudaMemcpyAsync(d_nc, nc.data(), sizeof(int32_t) * qn, cudaMemcpyHostToDevice, s));
        // one correction: Res = A_s Z (the FP64 residual of the current result), Res <- M Res
        // through the stored panel transforms, then R += Res on the refined entries (or, with
        // apply = false, only the max-norms of the correction and of the entries are measured)
        auto correction = [&](bool apply, double* corr, double* ymax) -> int {
            int r2 = refine_build_z<T>(n, qn, d_colmap, d_nc, R, n, Z, s);
            if (!r2) {
                cudaError_t e2 = cudaMemsetAsync(Res, 0, sizeof(T) * (size_t)m * qn, s);
                if (e2 != cudaSuccess) return cuda_status(e2, "cudaMemsetAsync");
                r2 = refine_narrow_gemm<T>(m, qn, n, nullptr, mx.As, n, Z, qn, Res, qn, s);
            }
            for (int64_t pq = 0; pq < panels && !r2; ++pq) {  // Res <- M Res, panel by panel
                dim3 g((unsigned)std::max<int64_t>(1, std::min<int64_t>((qn + 255) / 256, 64)), (unsigned)pl.b);
                gather_pivot_rows_kernel<F><<<g, 256, 0, s>>>(f, Res, qn, 0, qn, mx.P_all + pq * pl.b,
                                                              mx.K_all + pq, Bg, qn);
                LNC_CHECK_LAUNCH("gather_pivot_rows_kernel (refinement)");
                r2 = refine_narrow_gemm<T>(m, qn, pl.b, mx.K_all + pq, mx.E_all + pq * pl.b, mx.ldE, Bg, qn, Res, qn,
                                           s);
            }
            if (r2) return r2;
            LNC_CUDA(cudaMemsetAsync(stats, 0, 16, s));
            r2 = refine_apply<T>(rank, qn, piv_row, d_nc, Res, R, n, stats, s, apply);
            if (r2) return r2;
            unsigned long long hs[2];
            LNC_CUDA(cudaMemcpyAsync(hs, stats, 16, cudaMemcpyDeviceToHost, s));
            LNC_CUDA(cudaStreamSynchronize(s));
            memcpy(corr, &hs[0], 8);
            memcpy(ymax, &hs[1], 8);
            return LNC_OK;
        };
        double prev = INFINITY;
        for (int it = 0; it < 10 && !rc; ++it) {
            double corr = 0.0, ymax = 0.0;
            rc = correction(true, &corr, &ymax);
            if (rc) break;
            t_mixed.iterations = it + 1;
            t_mixed.last_correction = ymax > 0 ? corr / ymax : corr;
            if (corr <= 4.0 * 1.1102230246251565e-16 * ymax || corr >= 0.5 * prev) break;
            prev = corr;
        }
        if (!rc) {  // a-posteriori estimate of the remaining error: one further correction, not applied
            double corr = 0.0, ymax = 0.0;
            rc = correction(false, &corr, &ymax);
            t_mixed.error_estimate = ymax > 0 ? corr / ymax : corr;
        }
        cudaFreeAsync(rb, s);
        if (rc) return fail(rc);
    }
    // outputs: the result (refined), pivots and rank
    LNC_CUDA(cudaMemcpy2DAsync(out, sizeof(T) * ldo, R, sizeof(T) * n, sizeof(T) * n, m, cudaMemcpyDeviceToDevice,
                               s));
    if (dev_piv || dev_rank) {
        copy_pivots_kernel<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>((kmax + 255) / 256, 1024)), 256, 0,
                             s>>>(piv_col, rank_d, kmax, dev_piv, dev_rank);
        LNC_CHECK_LAUNCH("copy_pivots_kernel");
    }
    cudaFreeAsync(blk, s);
    return LNC_OK;
}

int mixed_report(int* iterations, double* last_correction, int* redone) {
    if (iterations) *iterations = t_mixed.iterations;
    if (last_correction) *last_correction = t_mixed.last_correction;
    if (redone) *redone = t_mixed.redone;
    return LNC_OK;
}

double mixed_error_estimate() { return t_mixed.error_estimate; }

// device scratch one (out-of-place) solve allocates, 0 when the shape is not supported
size_t rref_device_scratch(int dtype, int64_t m, int64_t n) {
    RrefPlan pl;
    switch (dtype) {
        case LNC_U32: return plan_rref<FieldU32>(m, n, &pl) ? 0 : rref_scratch_bytes<FieldU32>(m, n, pl);
        case LNC_U64: return plan_rref<FieldU64>(m, n, &pl) ? 0 : rref_scratch_bytes<FieldU64>(m, n, pl);
        case LNC_F64: return plan_rref<FieldF64>(m, n, &pl) ? 0 : rref_scratch_bytes<FieldF64>(m, n, pl);
        case LNC_C128: return plan_rref<FieldC128>(m, n, &pl) ? 0 : rref_scratch_bytes<FieldC128>(m, n, pl);
        default: return 0;
    }
}

int rref_device_dispatch(int dtype, int64_t m, int64_t n, uint64_t p, double tol, void* work,
                         int64_t ldw, void* out, int64_t ldo, int64_t* dev_piv, int64_t* dev_rank,
                         cudaStream_t s, int flags) {
    switch (dtype) {
        case LNC_U32: return rref_device_typed(FieldU32::make(p), work, ldw, out, ldo, m, n, dev_piv, dev_rank, s, flags);
        case LNC_U64: return rref_device_typed(FieldU64::make(p), work, ldw, out, ldo, m, n, dev_piv, dev_rank, s, flags);
        case LNC_F64:
            if (flags & LNC_FLAG_MIXED)
                return rref_mixed_typed(FieldF64::make(tol), work, ldw, out, ldo, m, n, dev_piv, dev_rank, s, flags);
            return rref_device_typed(FieldF64::make(tol), work, ldw, out, ldo, m, n, dev_piv, dev_rank, s, flags);
        case LNC_C128:
            if (flags & LNC_FLAG_MIXED)
                return rref_mixed_typed(FieldC128::make(tol), work, ldw, out, ldo, m, n, dev_piv, dev_rank, s, flags);
            return rref_device_typed(FieldC128::make(tol), work, ldw, out, ldo, m, n, dev_piv, dev_rank, s, flags);
        default: set_error("unknown dtype %d", dtype); return LNC_ERR_INVALID;
    }
}

// ----------------------------------------------------------------------------
// No-allocation variant: the same RREF with its scratch in a fixed, file-scope
// device array instead of stream-ordered allocations.
//
// Some callers cannot allocate device memory at the time they need an RREF:
// a host framework that has reserved all of HBM for its own pool allocator
// up front (so cudaMalloc / cudaMallocAsync fail or steal from it), or a
// latency-critical serving thread that must never wait on an allocator.  For
// them the scratch lives in g_noalloc_scratch, a 16 MiB array that every GPU
// loading this library holds until the process exits.  Requests whose
// scratch does not fit are rejected up front with LNC_ERR_INVALID.
//
// The array's name in host code is only a host-side stand-in; the device
// address is obtained once per device with cudaGetSymbolAddress, on that
// device's first call of lnc_rref_device_noalloc (so make that first call
// before any stream capture), and kept for the life of the process: like the
// library's other per-device state it does not survive cudaDeviceReset.  All
// calls share the array and it keeps the previous call's contents; rref_run
// clears everything that must start at zero.  Calls that overlap on the GPU
// (concurrent streams, or devices not yet synchronised between calls) race on
// the array.  Input and output must not overlap at all: the final row gather
// reads the work matrix while it writes the output.
// ----------------------------------------------------------------------------
constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

static std::mutex g_noalloc_mu;
static void* g_noalloc_ptr[64] = {};

static int noalloc_scratch(void** out) {
    int dev = 0;
    LNC_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) { set_error("device index out of range"); return LNC_ERR_INVALID; }
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(no-allocation scratch)");
        g_noalloc_ptr[dev] = ptr;
    }
    *out = g_noalloc_ptr[dev];
    return LNC_OK;
}

// [a, a + bytes_a) and [b, b + bytes_b) share at least one byte
static bool ranges_overlap(const void* a, size_t bytes_a, const void* b, size_t bytes_b) {
    const uintptr_t a0 = (uintptr_t)a, b0 = (uintptr_t)b;
    return a0 < b0 + bytes_b && b0 < a0 + bytes_a;
}

template <class F>
static int rref_noalloc_typed(const F& f, void* work, int64_t ldw, void* out, int64_t ldo, int64_t m, int64_t n,
                              int64_t* dev_piv, int64_t* dev_rank, cudaStream_t s, int flags) {
    using T = typename F::T;
    RrefPlan pl;
    int rc = plan_rref<F>(m, n, &pl);
    if (rc) return rc;
    pl.lookahead = false;  // one stream: the fixed scratch holds no look-ahead buffers
    const size_t need = rref_scratch_bytes<F>(m, n, pl);
    if (need > kNoAllocScratchBytes) {
        set_error("a %lld x %lld RREF needs %zu bytes of scratch; the fixed no-allocation scratch holds %zu",
                  (long long)m, (long long)n, need, kNoAllocScratchBytes);
        return LNC_ERR_INVALID;
    }
    const size_t work_bytes = sizeof(T) * ((size_t)ldw * (size_t)(m - 1) + (size_t)n);
    const size_t out_bytes = sizeof(T) * ((size_t)ldo * (size_t)(m - 1) + (size_t)n);
    if (ranges_overlap(work, work_bytes, out, out_bytes)) {
        set_error("the no-allocation RREF needs input and output buffers that do not overlap");
        return LNC_ERR_INVALID;
    }
    void* scratch = nullptr;
    rc = noalloc_scratch(&scratch);
    if (rc) return rc;
    return rref_run<F>(f, (T*)work, m, n, ldw, (T*)out, ldo, dev_piv, dev_rank, s, flags, scratch, need, pl);
}

int rref_device_noalloc_dispatch(int dtype, int64_t m, int64_t n, uint64_t p, double tol, void* work,
                                 int64_t ldw, void* out, int64_t ldo, int64_t* dev_piv, int64_t* dev_rank,
                                 cudaStream_t s, int flags) {
    switch (dtype) {
        case LNC_U32: return rref_noalloc_typed(FieldU32::make(p), work, ldw, out, ldo, m, n, dev_piv, dev_rank, s, flags);
        case LNC_U64: return rref_noalloc_typed(FieldU64::make(p), work, ldw, out, ldo, m, n, dev_piv, dev_rank, s, flags);
        case LNC_F64: return rref_noalloc_typed(FieldF64::make(tol), work, ldw, out, ldo, m, n, dev_piv, dev_rank, s, flags);
        case LNC_C128: return rref_noalloc_typed(FieldC128::make(tol), work, ldw, out, ldo, m, n, dev_piv, dev_rank, s, flags);
        default: set_error("unknown dtype %d", dtype); return LNC_ERR_INVALID;
    }
}

}  // namespace lnc

extern "C" int lnc_rref_device_noalloc(int dtype, int64_t m, int64_t n, uint64_t p, double tol, void* dev_work,
                                       int64_t ld_work, void* dev_out, int64_t ld_out, int64_t* dev_pivot_cols,
                                       int64_t* dev_rank, void* stream, int flags) {
    using namespace lnc;
    int rc = validate_rref_args(dtype, m, n, p, ld_work);
    if (rc) return rc;
    if (flags & LNC_FLAG_MIXED) { set_error("mixed precision allocates: not available without allocation"); return LNC_ERR_UNSUPPORTED; }
    if (ld_out < n) { set_error("output leading dimension %lld < n", (long long)ld_out); return LNC_ERR_INVALID; }
    if (m == 0 || n == 0) {
        set_error("the no-allocation RREF needs a non-empty matrix");
        return LNC_ERR_INVALID;
    }
    return rref_device_noalloc_dispatch(dtype, m, n, p, tol, dev_work, ld_work, dev_out, ld_out, dev_pivot_cols,
                                        dev_rank, (cudaStream_t)stream, flags);
}
