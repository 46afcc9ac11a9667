// Batched RREF of many uneven matrices over F_p (32-bit residues, a prime per
// matrix) on the tensor-core path, captured as one CUDA graph.
//
// linac has no batched entry point: its callers (vector spaces, the iterative
// solver, linac/vector_spaces/over_function_fields.py:74-101,
// linac/linear_system_solver.py:41-45) call cuda_row_reduce once per matrix,
// each call a fresh JIT, two synchronous copies and 7 launches per column.
//
// Here a plan covers the whole batch:
//  * one scratch arena; all matrices' E-digit planes share one tensor and all
//    B-digit tiles another (per-matrix row offsets), so two TMA descriptors
//    serve every GEMM of the batch;
//  * panel step q (columns [128 q, 128 q + 128) of every matrix that has them):
//    one candidate-panel CTA per matrix, batched digit splits, and the two
//    limb contractions E = G X and A[:, j0:] += E A[P, j0:] as work lists whose
//    CTAs find their (matrix, row block, tile range) by binary search over a
//    per-step prefix array;
//  * the launches of all steps are captured once into a CUDA graph; a run of
//    the batch is a single graph launch;
//  * a matrix whose candidate panels missed a pivot (only structured inputs do)
//    is flagged on the device and redone afterwards by the exhaustive
//    single-matrix path from its untouched input.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "cand_kernels.cuh"
#include "tc_kernels.cuh"

namespace lnc {

struct BatchMat {
    uint32_t* A;  // working copy (n columns per row)
    int64_t m, n;
    const uint32_t* in;
    int64_t ldi;
    uint32_t* out;
    int64_t ldo;
    int64_t* out_piv;
    int64_t* out_rank;
    uint32_t p, pinv, r2;
    uint64_t mu;
    int redc;
    int32_t w[tc::GROUPS];
    uint64_t off;
    uint8_t* row_used;
    int32_t* piv_row;
    int64_t* piv_col;
    int64_t* rank;
    int32_t* panel_k;
    int32_t* panel_rows;
    int32_t* panel_cols;
    int32_t* panel_mark;
    uint32_t* X;
    uint32_t* E;
    int32_t* cand;
    int32_t* cand_n;
    int32_t* next_row;
    int* missed;
    int* missed_any;
    uint32_t* pivmask;
    int32_t* col_row;
    int el_row0, m_pad, bs_row0, bs_tiles;
    int bx_row0;  // digit rows of X (the first contraction's B operand)
};

// ---------------------------------------------------------------------------
// batched kernels: blockIdx.y (or blockIdx.x for one-CTA-per-matrix kernels)
// selects the matrix; the bodies are the single-matrix ones
// ---------------------------------------------------------------------------
static __global__ void batch_prepare_kernel(const BatchMat* mats) {
    const BatchMat& M = mats[blockIdx.y];
    for (int64_t r = blockIdx.x; r < M.m; r += gridDim.x) {
        const uint32_t* src = M.in + r * M.ldi;
        uint32_t* dst = M.A + r * M.n;
        for (int64_t c = threadIdx.x; c < M.n; c += blockDim.x) {
            const uint32_t x = src[c];
            dst[c] = x >= M.p ? x % M.p : x;
        }
    }
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < M.m; r += (int64_t)gridDim.x * blockDim.x) {
        M.row_used[r] = 0;
        M.panel_mark[r] = 0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *M.rank = 0;
        *M.cand_n = 0;
        *M.next_row = 0;
        *M.missed = 0;
        *M.missed_any = 0;
        *M.panel_k = 0;
    }
}

static __device__ __forceinline__ CandArgs batch_cand_args(const BatchMat& M, int step, int smax) {
    CandArgs a;
    a.A = M.A;
    a.lda = M.n;
    a.m = M.m;
    a.j0 = (int64_t)step * kMaxPanel;
    a.bw = (int)((M.n - a.j0) < kMaxPanel ? (M.n - a.j0) : kMaxPanel);
    a.smax = smax;
    a.row_used = M.row_used;
    a.cand = M.cand;
    a.cand_n = M.cand_n;
    a.next_row = M.next_row;
    a.rank = M.rank;
    a.piv_row = M.piv_row;
    a.piv_col = M.piv_col;
    a.panel_k = M.panel_k;
    a.panel_rows = M.panel_rows;
    a.panel_cols = M.panel_cols;
    a.panel_mark = M.panel_mark;
    a.gen = step + 1;
    a.X = M.X;
    a.pivmask = M.pivmask;
    a.missed = M.missed;
    a.M.p = M.p;
    a.M.pinv = M.pinv;
    a.M.r2 = M.r2;
    a.M.mu = M.mu;
    return a;
}

// arithmetic class of a prime: 0 = p is 2, 1 = odd p < 2^31, 2 = odd p >= 2^31
__host__ __device__ __forceinline__ int arith_class(uint32_t p) { return !(p & 1u) ? 0 : (p < (1u << 31) ? 1 : 2); }

// one instantiation per arithmetic class (few registers: two CTAs per SM);
// the host launches the classes present in the batch
template <class Arith, int CLS>
static __global__ void __launch_bounds__(kCandThreads, 2)
    batch_cand_kernel(const BatchMat* mats, const int* active, int step, int smax) {
    const BatchMat& M = mats[active[blockIdx.x]];
    if (arith_class(M.p) != CLS) return;
    const CandArgs a = batch_cand_args(M, step, smax);
    cand_body<Arith>(a);
}

// per-step kernels: `active` lists the matrices that still have columns at this step
static __global__ void batch_split_g_kernel(const BatchMat* mats, const int* active, int step, __nv_bfloat16* EL) {
    const BatchMat& M = mats[active[blockIdx.y]];
    const int64_t j0 = (int64_t)step * kMaxPanel;
    split_g_body(M.A, M.n, M.m, M.m_pad, j0, M.p, M.panel_k, M.panel_cols, M.panel_mark, step + 1,
                 EL + (size_t)M.el_row0 * tc::KMAX);
}

static __global__ void batch_split_e_kernel(const BatchMat* mats, const int* active, __nv_bfloat16* EL) {
    const BatchMat& M = mats[active[blockIdx.y]];
    tc::split_e_body(M.E, tc::KMAX, tc::KMAX, M.m, M.m_pad, M.p, M.panel_k, EL + (size_t)M.el_row0 * tc::KMAX);
}

// Digit tiles of both contractions' B operands, one 32-column tile per CTA
// (work list item (matrix, l): l < 4 is tile l of X, else tile l - 4 of the
// pivot rows of A[:, j0:], which are zeroed in A).  X's tiles have their
// own rows (bx_row0) so both kinds run in one launch.
static __global__ void __launch_bounds__(256, 6) batch_gather_b_kernel(const BatchMat* mats, const int2* items,
                                                                       int step, __nv_bfloat16* BS) {
    const int2 it = items[blockIdx.x];
    const BatchMat& M = mats[it.x];
    const int l = it.y;
    constexpr int XT = kMaxPanel / tc::BN;
    if (l < XT) {
        tc::gather_split_b_body(l, M.X, kMaxPanel, kMaxPanel, nullptr, M.panel_k, M.p,
                                BS + (size_t)M.bx_row0 * tc::KMAX, 0);
    } else {
        const int64_t j0 = (int64_t)step * kMaxPanel;
        tc::gather_split_b_body(l - XT, M.A + j0, M.n, M.n - j0, M.panel_rows, M.panel_k, M.p,
                                BS + (size_t)M.bs_row0 * tc::KMAX, 1);
    }
}

static __global__ void __launch_bounds__(tc::THREADS, 1)
    batch_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                      const BatchMat* mats, const int2* items, int step, int kind, int tpc, int* err,
                      int* status) {
    const int2 it = items[blockIdx.x];  // (matrix, item of that matrix)
    const BatchMat& M = mats[it.x];
    const int64_t j0 = (int64_t)step * kMaxPanel;
    const int l = it.y;
    const int64_t N = (kind == 1) ? kMaxPanel : M.n - j0;
    const int tiles = (int)((N + tc::BN - 1) / tc::BN);
    const int groups = (tiles + tpc - 1) / tpc;
    tc::LimbJob J;
    J.C = (kind == 1) ? M.E : M.A + j0;
    J.ldc = (kind == 1) ? kMaxPanel : M.n;
    J.m = M.m;
    J.N = N;
    J.rb = l / groups;
    J.t0 = (l % groups) * tpc;
    J.t1 = min(tiles, J.t0 + tpc);
    J.a_row0 = M.el_row0;
    J.a_plane = M.m_pad;
    J.b_row0 = (kind == 1) ? M.bx_row0 : M.bs_row0;
    J.k = *M.panel_k;
    J.overwrite = (kind == 1) ? 1 : 0;
    J.redc = M.redc;
    J.f.p = M.p;
    J.f.mu = M.mu;
    J.pinv = M.pinv;
    J.w = M.w;
    J.off = M.off;
    J.err = err;
    J.status = status;
    if (J.redc) tc::limb_cta<tc::EPI_REDC>(J, &tmA, &tmB);
    else tc::limb_cta<tc::EPI_BARRETT>(J, &tmA, &tmB);
}

static __global__ void batch_check_kernel(const BatchMat* mats, const int* active, int step) {
    const BatchMat& M = mats[active[blockIdx.y]];
    const int64_t j0 = (int64_t)step * kMaxPanel;
    const int bw = (int)((M.n - j0) < kMaxPanel ? (M.n - j0) : kMaxPanel);
    check_missed_body(M.A, M.n, M.m, j0, bw, M.row_used, M.pivmask, M.missed_any);
}

// order pivots by column, then write the RREF rows and the pivot outputs
static __global__ void __launch_bounds__(1024) batch_finalize_kernel(const BatchMat* mats) {
    const BatchMat& M = mats[blockIdx.x];
    __shared__ int s_warp[32];
    __shared__ int s_base, s_total;
    const int64_t rank = *M.rank;
    for (int64_t c = threadIdx.x; c < M.n; c += blockDim.x) M.col_row[c] = -1;
    __syncthreads();
    for (int64_t i = threadIdx.x; i < rank; i += blockDim.x) M.col_row[M.piv_col[i]] = M.piv_row[i];
    if (threadIdx.x == 0) s_base = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int64_t c0 = 0; c0 < M.n; c0 += blockDim.x) {
        const int64_t c = c0 + threadIdx.x;
        const int32_t r = (c < M.n) ? M.col_row[c] : -1;
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
            M.piv_row[pos] = r;
            M.piv_col[pos] = c;
        }
        __syncthreads();
        if (threadIdx.x == 0) s_base += s_total;
        __syncthreads();
    }
    const int64_t kmax = min(M.m, M.n);
    for (int64_t i = threadIdx.x; i < kmax; i += blockDim.x)
        if (M.out_piv) M.out_piv[i] = (i < rank) ? M.piv_col[i] : -1;
    if (threadIdx.x == 0 && M.out_rank) *M.out_rank = rank;
}

static __global__ void batch_gather_out_kernel(const BatchMat* mats) {
    const BatchMat& M = mats[blockIdx.y];
    const int64_t rank = *M.rank;
    for (int64_t r = blockIdx.x; r < M.m; r += gridDim.x) {
        uint32_t* dst = M.out + r * M.ldo;
        if (r < rank) {
            const uint32_t* src = M.A + (int64_t)M.piv_row[r] * M.n;
            for (int64_t c = threadIdx.x; c < M.n; c += blockDim.x) dst[c] = src[c];
        } else {
            for (int64_t c = threadIdx.x; c < M.n; c += blockDim.x) dst[c] = 0u;
        }
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
int tc_make_map_bf16(CUtensorMap* map, void* base, uint64_t inner, uint64_t outer, uint32_t box_inner,
                     uint32_t box_outer);
int rref_device_dispatch(int dtype, int64_t m, int64_t n, uint64_t p, double tol, void* work, int64_t ldw,
                         void* out, int64_t ldo, int64_t* dev_piv, int64_t* dev_rank, cudaStream_t s, int flags);

static size_t al256(size_t x) { return (x + 255) / 256 * 256; }

struct BatchPlan {
    int device = -1;
    int64_t count = 0;
    std::vector<lnc_batch_matrix> mats;
    std::vector<BatchMat> host_desc;
    void* arena = nullptr;
    size_t arena_bytes = 0;
    BatchMat* d_desc = nullptr;
    int* d_prefix = nullptr;
    int* d_words = nullptr;  // err, status
    int* d_missed = nullptr;  // per matrix: a candidate panel missed a pivot
    // per step: offset into d_prefix of the active-matrix list (largest n
    // first) and its length; offsets into d_items of the work lists (gather,
    // E = G X, A += E A_P) and their lengths (the grid sizes)
    std::vector<int> active_off, active_cnt, offg, off1, off2;
    std::vector<int> itemsg, items1, items2;
    int2* d_items = nullptr;
    int steps = 0;
    int tpc = 16;
    int smax = kCandRows;
    int max_tiles = 0;
    int64_t max_rows = 0;
    int64_t max_n = 0;
    bool has_class[3] = {false, false, false};
    CUtensorMap mapA, mapB;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t launches_per_run = 0;
    std::vector<int> host_missed;
};

static int record_batch(BatchPlan& P, cudaStream_t s) {
    const int nmat = (int)P.count;
    __nv_bfloat16* EL = nullptr;
    __nv_bfloat16* BS = nullptr;
    {
        unsigned char* base = (unsigned char*)P.arena;
        EL = (__nv_bfloat16*)base;
        size_t el_bytes = 0;
        for (auto& d : P.host_desc) el_bytes += (size_t)4 * d.m_pad * tc::KMAX * 2;
        BS = (__nv_bfloat16*)(base + al256(el_bytes));
    }
    int64_t launches = 0;
    const unsigned gy = (unsigned)nmat;  // once-per-run kernels: one CTA row per matrix
    const unsigned gx_rows = (unsigned)std::min<int64_t>(std::max<int64_t>(1, (P.max_rows * 128 + 255) / 256), 64);
    batch_prepare_kernel<<<dim3(64, gy), 256, 0, s>>>(P.d_desc);
    ++launches;
    const size_t cand_smem = (size_t)(P.smax | 1) * kMaxPanel * 4 + 2 * kMaxPanel * 4 + 256 * 4;
    for (int q = 0; q < P.steps; ++q) {
        const int na = P.active_cnt[q];
        const int* act = P.d_prefix + P.active_off[q];
        if (P.has_class[1]) {
            batch_cand_kernel<ArithSmall, 1><<<na, kCandThreads, cand_smem, s>>>(P.d_desc, act, q, P.smax);
            ++launches;
        }
        if (P.has_class[2]) {
            batch_cand_kernel<ArithMont, 2><<<na, kCandThreads, cand_smem, s>>>(P.d_desc, act, q, P.smax);
            ++launches;
        }
        if (P.has_class[0]) {
            batch_cand_kernel<ArithTwo, 0><<<na, kCandThreads, cand_smem, s>>>(P.d_desc, act, q, P.smax);
            ++launches;
        }
        const dim3 g_rows(gx_rows, (unsigned)na);
        batch_split_g_kernel<<<g_rows, 256, 0, s>>>(P.d_desc, act, q, EL);
        batch_gather_b_kernel<<<P.itemsg[q], 256, 0, s>>>(P.d_desc, P.d_items + P.offg[q], q, BS);
        if (P.items1[q] > 0)
            batch_gemm_kernel<<<P.items1[q], tc::THREADS, tc::SMEM_BYTES, s>>>(
                P.mapA, P.mapB, P.d_desc, P.d_items + P.off1[q], q, 1, P.tpc, P.d_words, P.d_words + 1);
        batch_split_e_kernel<<<g_rows, 256, 0, s>>>(P.d_desc, act, EL);
        if (P.items2[q] > 0)
            batch_gemm_kernel<<<P.items2[q], tc::THREADS, tc::SMEM_BYTES, s>>>(
                P.mapA, P.mapB, P.d_desc, P.d_items + P.off2[q], q, 2, P.tpc, P.d_words, P.d_words + 1);
        batch_check_kernel<<<g_rows, 256, 0, s>>>(P.d_desc, act, q);
        launches += 4 + (P.items1[q] > 0) + (P.items2[q] > 0);
    }
    batch_finalize_kernel<<<nmat, 1024, 0, s>>>(P.d_desc);
    batch_gather_out_kernel<<<dim3(64, gy), 256, 0, s>>>(P.d_desc);
    launches += 2;
    P.launches_per_run = launches;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_status(e, "batched RREF launch");
    return LNC_OK;
}

static int plan_create(const lnc_batch_matrix* mats, int64_t count, int tpc, int smax, cudaStream_t s,
                       BatchPlan** out) {
    if (count <= 0) { set_error("empty batch"); return LNC_ERR_INVALID; }
    if (count > 65535) { set_error("batch of %lld matrices exceeds 65535", (long long)count); return LNC_ERR_UNSUPPORTED; }
    if (!trailing_tc_u32_available()) { set_error("the batched path needs the tcgen05 tensor cores"); return LNC_ERR_UNSUPPORTED; }
    BatchPlan* P = new BatchPlan();
    P->count = count;
    P->mats.assign(mats, mats + count);
    P->tpc = (tpc >= 1 && tpc <= 64) ? tpc : 16;
    P->smax = (smax >= 32 && smax <= kCandRows) ? smax : kCandRows;
    LNC_CUDA(cudaGetDevice(&P->device));
    // ---- layout
    size_t el_rows = 0, bs_rows = 0, bytes = 0;
    std::vector<size_t> mat_off(count);
    P->host_desc.resize(count);
    for (int64_t i = 0; i < count; ++i) {
        const auto& mm = mats[i];
        if (mm.m <= 0 || mm.n <= 0 || mm.ld_in < mm.n || mm.ld_out < mm.n || mm.p < 2 || mm.p > 0xFFFFFFFFull ||
            !is_prime_u64(mm.p)) {
            delete P;
            set_error("batch matrix %lld: invalid shape or non-prime modulus", (long long)i);
            return LNC_ERR_INVALID;
        }
        BatchMat& d = P->host_desc[i];
        d.m = mm.m;
        d.n = mm.n;
        d.m_pad = tc_m_pad(mm.m);
        d.bs_tiles = std::max<int>(kMaxPanel / tc::BN, (int)((mm.n + tc::BN - 1) / tc::BN));
        d.el_row0 = (int)el_rows;
        d.bs_row0 = (int)bs_rows;
        d.bx_row0 = (int)(bs_rows + (size_t)d.bs_tiles * tc::B_ROWS);
        el_rows += (size_t)4 * d.m_pad;
        bs_rows += (size_t)(d.bs_tiles + kMaxPanel / tc::BN) * tc::B_ROWS;
        P->steps = std::max<int>(P->steps, (int)((mm.n + kMaxPanel - 1) / kMaxPanel));
        P->max_tiles = std::max<int>(P->max_tiles, (int)((mm.n + tc::BN - 1) / tc::BN));
        P->max_rows = std::max<int64_t>(P->max_rows, mm.m);
        P->max_n = std::max<int64_t>(P->max_n, mm.n);
        P->has_class[arith_class((uint32_t)mm.p)] = true;
        const int64_t kmax = std::min(mm.m, mm.n);
        mat_off[i] = bytes;
        bytes += al256((size_t)mm.m * mm.n * 4)          // A
                 + al256((size_t)mm.m)                   // row_used
                 + al256((size_t)kmax * 4)               // piv_row
                 + al256((size_t)kmax * 8)               // piv_col
                 + 256                                   // scalars
                 + al256(kMaxPanel * 4) * 2              // panel rows / cols
                 + al256((size_t)mm.m * 4)               // panel_mark
                 + al256(kMaxPanel * kMaxPanel * 4)      // X
                 + al256((size_t)mm.m * kMaxPanel * 4)   // E
                 + al256(256 * 4)                        // candidates
                 + al256((size_t)mm.n * 4);              // col_row
    }
    if (el_rows > 0x7fffffffull || bs_rows > 0x7fffffffull) {
        delete P;
        set_error("batch too large for one digit tensor");
        return LNC_ERR_UNSUPPORTED;
    }
    const size_t el_bytes = al256(el_rows * tc::KMAX * 2);
    const size_t bs_bytes = al256(bs_rows * tc::KMAX * 2);
    P->arena_bytes = el_bytes + bs_bytes + bytes + 1024;
    cudaError_t e = cudaMallocAsync(&P->arena, P->arena_bytes, s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        delete P;
        set_error("batch scratch of %zu bytes: %s", (size_t)el_bytes + bs_bytes + bytes, cudaGetErrorString(e));
        return LNC_ERR_OOM;
    }
    unsigned char* base = (unsigned char*)P->arena;
    unsigned char* mats_base = base + el_bytes + bs_bytes;
    for (int64_t i = 0; i < count; ++i) {
        const auto& mm = mats[i];
        BatchMat& d = P->host_desc[i];
        unsigned char* q = mats_base + mat_off[i];
        auto take = [&](size_t b) { void* r = q; q += al256(b); return r; };
        const int64_t kmax = std::min(mm.m, mm.n);
        d.A = (uint32_t*)take((size_t)mm.m * mm.n * 4);
        d.row_used = (uint8_t*)take((size_t)mm.m);
        d.piv_row = (int32_t*)take((size_t)kmax * 4);
        d.piv_col = (int64_t*)take((size_t)kmax * 8);
        unsigned char* sc = (unsigned char*)take(256);
        d.rank = (int64_t*)sc;
        d.panel_k = (int32_t*)(sc + 8);
        d.cand_n = (int32_t*)(sc + 12);
        d.next_row = (int32_t*)(sc + 16);
        d.missed = (int*)(sc + 20);
        d.pivmask = (uint32_t*)(sc + 32);
        d.panel_rows = (int32_t*)take(kMaxPanel * 4);
        d.panel_cols = (int32_t*)take(kMaxPanel * 4);
        d.panel_mark = (int32_t*)take((size_t)mm.m * 4);
        d.X = (uint32_t*)take(kMaxPanel * kMaxPanel * 4);
        d.E = (uint32_t*)take((size_t)mm.m * kMaxPanel * 4);
        d.cand = (int32_t*)take(256 * 4);
        d.col_row = (int32_t*)take((size_t)mm.n * 4);
        d.in = (const uint32_t*)mm.dev_in;
        d.ldi = mm.ld_in;
        d.out = (uint32_t*)mm.dev_out;
        d.ldo = mm.ld_out;
        d.out_piv = mm.dev_pivot_cols;
        d.out_rank = mm.dev_rank;
        const uint32_t p = (uint32_t)mm.p;
        d.p = p;
        d.mu = ~0ull / p;
        uint32_t x = p;
        for (int t = 0; t < 5; ++t) x *= 2u - p * x;
        d.pinv = 0u - x;
        d.r2 = (uint32_t)((((unsigned __int128)1) << 64) % p);
        const tc::LimbConstants lc = tc::limb_constants(p);
        d.redc = lc.redc;
        for (int g = 0; g < tc::GROUPS; ++g) d.w[g] = lc.w[g];
        d.off = lc.off;
    }
    // ---- per-step active lists and work lists (static: they depend on the shapes only)
    std::vector<int> order(count);
    for (int64_t i = 0; i < count; ++i) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(),
                     [&](int x, int y) { return P->host_desc[x].n > P->host_desc[y].n; });
    std::vector<int> prefix;
    std::vector<int2> items;
    for (int q = 0; q < P->steps; ++q) {
        const int64_t j0 = (int64_t)q * kMaxPanel;
        P->active_off.push_back((int)prefix.size());
        int na = 0;
        for (int i : order)
            if (P->host_desc[i].n > j0) { prefix.push_back(i); ++na; }
        P->active_cnt.push_back(na);
        for (int list = 0; list < 3; ++list) {  // 0: gather tiles, 1: E = G X, 2: A += E A_P
            (list == 0 ? P->offg : list == 1 ? P->off1 : P->off2).push_back((int)items.size());
            int cnt = 0;
            for (int a = 0; a < na; ++a) {
                const int i = prefix[P->active_off[q] + a];
                const BatchMat& d = P->host_desc[i];
                const int64_t N = (list == 1) ? kMaxPanel : d.n - j0;
                const int tiles = (int)((N + tc::BN - 1) / tc::BN);
                const int c = (list == 0) ? kMaxPanel / tc::BN + tiles
                                          : (d.m_pad / tc::BM) * ((tiles + P->tpc - 1) / P->tpc);
                for (int l = 0; l < c; ++l) items.push_back(make_int2(i, l));
                cnt += c;
            }
            (list == 0 ? P->itemsg : list == 1 ? P->items1 : P->items2).push_back(cnt);
        }
    }
    const size_t desc_bytes = al256(sizeof(BatchMat) * (size_t)count);
    const size_t pre_bytes = al256(sizeof(int) * prefix.size());
    const size_t item_bytes = al256(sizeof(int2) * items.size());
    e = cudaMallocAsync((void**)&P->d_desc,
                        desc_bytes + pre_bytes + 256 + al256(sizeof(int) * (size_t)count) + item_bytes, s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        cudaFreeAsync(P->arena, s);
        delete P;
        set_error("batch descriptors: %s", cudaGetErrorString(e));
        return LNC_ERR_OOM;
    }
    P->d_prefix = (int*)((unsigned char*)P->d_desc + desc_bytes);
    P->d_words = (int*)((unsigned char*)P->d_desc + desc_bytes + pre_bytes);
    P->d_missed = (int*)((unsigned char*)P->d_desc + desc_bytes + pre_bytes + 256);
    P->d_items = (int2*)((unsigned char*)P->d_missed + al256(sizeof(int) * (size_t)count));
    for (int64_t i = 0; i < count; ++i) P->host_desc[i].missed_any = P->d_missed + i;
    LNC_CUDA(cudaMemcpyAsync(P->d_desc, P->host_desc.data(), sizeof(BatchMat) * (size_t)count, cudaMemcpyHostToDevice, s));
    LNC_CUDA(cudaMemcpyAsync(P->d_prefix, prefix.data(), sizeof(int) * prefix.size(), cudaMemcpyHostToDevice, s));
    if (!items.empty())
        LNC_CUDA(cudaMemcpyAsync(P->d_items, items.data(), sizeof(int2) * items.size(), cudaMemcpyHostToDevice, s));
    LNC_CUDA(cudaMemsetAsync(P->d_words, 0, 256, s));
    int rc = tc_make_map_bf16(&P->mapA, base, tc::KMAX, el_rows, tc::KC, tc::BM);
    if (!rc) rc = tc_make_map_bf16(&P->mapB, base + el_bytes, tc::KMAX, bs_rows, tc::KC, tc::B_ROWS);
    if (rc) {
        cudaFreeAsync(P->d_desc, s);
        cudaFreeAsync(P->arena, s);
        delete P;
        return rc;
    }
    // ---- capture the whole batch into one graph
    const size_t cand_smem = (size_t)(P->smax | 1) * kMaxPanel * 4 + 2 * kMaxPanel * 4 + 256 * 4;
    for (const void* k : {(const void*)batch_cand_kernel<ArithSmall, 1>, (const void*)batch_cand_kernel<ArithMont, 2>,
                          (const void*)batch_cand_kernel<ArithTwo, 0>}) {
        const int rc0 = allow_dynamic_smem(k, cand_smem);
        if (rc0) {
            cudaFreeAsync(P->d_desc, s);
            cudaFreeAsync(P->arena, s);
            delete P;
            return rc0;
        }
    }
    LNC_CUDA(cudaFuncSetAttribute(batch_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc::SMEM_BYTES));
    LNC_CUDA(cudaStreamSynchronize(s));
    cudaStream_t cs;
    LNC_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    LNC_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    rc = record_batch(*P, cs);
    cudaGraph_t g = nullptr;
    cudaError_t ee = cudaStreamEndCapture(cs, &g);
    cudaStreamDestroy(cs);
    if (rc == LNC_OK && ee != cudaSuccess) rc = cuda_status(ee, "graph capture");
    if (rc == LNC_OK) {
        ee = cudaGraphInstantiate(&P->exec, g, 0);
        if (ee != cudaSuccess) rc = cuda_status(ee, "graph instantiate");
    }
    P->graph = g;
    if (rc) {
        if (P->exec) cudaGraphExecDestroy(P->exec);
        if (g) cudaGraphDestroy(g);
        cudaFree(P->d_desc);
        cudaFree(P->arena);
        delete P;
        return rc;
    }
    *out = P;
    return LNC_OK;
}

int batch_run(BatchPlan* P, cudaStream_t s) {
    LNC_CUDA(cudaMemsetAsync(P->d_words, 0, 8, s));
    {
        ScopedKernelTimer kt(KC_BATCH, s);
        LNC_CUDA(cudaGraphLaunch(P->exec, s));
    }
    for (int64_t i = 0; i < P->launches_per_run; ++i) count_launch();
    return LNC_OK;
}

// Matrices whose candidate panels missed a pivot are redone exhaustively from
// their input; returns how many.
int batch_finish(BatchPlan* P, cudaStream_t s, int64_t* n_redo) {
    std::vector<BatchMat>& D = P->host_desc;
    P->host_missed.assign(P->count, 0);
    int words[2] = {0, 0};
    LNC_CUDA(cudaMemcpyAsync(words, P->d_words, 8, cudaMemcpyDeviceToHost, s));
    LNC_CUDA(cudaMemcpyAsync(P->host_missed.data(), P->d_missed, sizeof(int) * (size_t)P->count,
                             cudaMemcpyDeviceToHost, s));
    LNC_CUDA(cudaStreamSynchronize(s));
    if (words[0] != 0) {
        set_error("a bounded device-side wait timed out in the batched RREF (status %d)", words[0]);
        return LNC_ERR_TIMEOUT;
    }
    int64_t redo = 0;
    for (int64_t i = 0; i < P->count; ++i) {
        if (!P->host_missed[i]) continue;
        ++redo;
        const auto& mm = P->mats[i];
        // exhaustive path on a fresh copy of the input (the working copy is in the arena)
        LNC_CUDA(cudaMemcpy2DAsync(D[i].A, mm.n * 4, mm.dev_in, mm.ld_in * 4, mm.n * 4, mm.m, cudaMemcpyDeviceToDevice, s));
        int rc = rref_device_dispatch(LNC_U32, mm.m, mm.n, mm.p, 0.0, D[i].A, mm.n, mm.dev_out, mm.ld_out,
                                      mm.dev_pivot_cols, mm.dev_rank, s, LNC_FLAG_ROBUST_PANEL);
        if (rc) return rc;
    }
    if (n_redo) *n_redo = redo;
    if (redo) LNC_CUDA(cudaStreamSynchronize(s));
    return LNC_OK;
}

// One graph over several plans: every plan's graph becomes a child graph of
// the group, behind a memset node that clears that plan's error words, with
// no dependency between plans, so one launch runs all of them and the GPU
// overlaps their steps (one plan's last steps, which hold few large
// matrices, run beside the other plans' work).
struct BatchGroup {
    std::vector<BatchPlan*> plans;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t launches_per_run = 0;
};

int batch_group_create(BatchPlan* const* plans, int64_t count, BatchGroup** out) {
    if (count <= 0) { set_error("empty plan group"); return LNC_ERR_INVALID; }
    BatchGroup* G = new BatchGroup();
    int rc = LNC_OK;
    cudaError_t e = cudaGraphCreate(&G->graph, 0);
    for (int64_t i = 0; e == cudaSuccess && i < count; ++i) {
        BatchPlan* P = plans[i];
        if (!P || !P->graph) { rc = LNC_ERR_INVALID; set_error("plan %lld of the group is not a batch plan", (long long)i); break; }
        cudaMemsetParams mp = {};
        mp.dst = P->d_words;
        mp.value = 0;
        mp.elementSize = 4;
        mp.width = 2;
        mp.height = 1;
        mp.pitch = 0;
        cudaGraphNode_t ms = nullptr, child = nullptr;
        e = cudaGraphAddMemsetNode(&ms, G->graph, nullptr, 0, &mp);
        if (e == cudaSuccess) e = cudaGraphAddChildGraphNode(&child, G->graph, &ms, 1, P->graph);
        G->plans.push_back(P);
        G->launches_per_run += P->launches_per_run;
    }
    if (!rc && e == cudaSuccess) e = cudaGraphInstantiate(&G->exec, G->graph, 0);
    if (!rc && e != cudaSuccess) rc = cuda_status(e, "plan group graph");
    if (rc) {
        if (G->exec) cudaGraphExecDestroy(G->exec);
        if (G->graph) cudaGraphDestroy(G->graph);
        delete G;
        return rc;
    }
    *out = G;
    return LNC_OK;
}

int batch_group_run(BatchGroup* G, cudaStream_t s) {
    {
        ScopedKernelTimer kt(KC_BATCH, s);
        LNC_CUDA(cudaGraphLaunch(G->exec, s));
    }
    for (int64_t i = 0; i < G->launches_per_run; ++i) count_launch();
    return LNC_OK;
}

void batch_group_destroy(BatchGroup* G) {
    if (!G) return;
    if (G->exec) cudaGraphExecDestroy(G->exec);
    if (G->graph) cudaGraphDestroy(G->graph);
    delete G;
}

void batch_destroy(BatchPlan* P) {
    if (!P) return;
    if (P->exec) cudaGraphExecDestroy(P->exec);
    if (P->graph) cudaGraphDestroy(P->graph);
    if (P->d_desc) cudaFree(P->d_desc);
    if (P->arena) cudaFree(P->arena);
    delete P;
}

size_t batch_plan_bytes(BatchPlan* P) { return P ? P->arena_bytes : 0; }

int batch_plan_create(const lnc_batch_matrix* mats, int64_t count, int tpc, int smax, cudaStream_t s,
                      BatchPlan** out) {
    return plan_create(mats, count, tpc, smax, s, out);
}

}  // namespace lnc
