// Internal declarations shared by rref.cu and trailing_tc.cu.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"
#include "field.cuh"
#include "sync.cuh"

namespace lnc {

struct RrefPlan {
    int G = 0;             // CTAs of the cooperative panel kernel
    int rows_per_cta = 0;  // panel rows held by each CTA
    int b = 0;             // panel width (columns)
    size_t smem = 0;
    bool lookahead_ok = false;  // the candidate-panel path can look ahead (tensor-core update present)
    bool lookahead = false;     // ... and does: next panel overlaps the trailing update
};

template <class F>
struct PanelArgs {
    F f;
    typename F::T* A;
    int64_t lda;
    int64_t m;
    int64_t j0;
    int bw;                 // width of this panel
    int b;                  // nominal panel width (E / exchange leading dims)
    uint8_t* row_used;      // 1 once a row is a pivot row
    int64_t* rank;          // pivots found before this panel (updated)
    int32_t* piv_row;       // physical row of pivot t
    int64_t* piv_col;       // column of pivot t
    int32_t* panel_k;       // pivots found in this panel
    int32_t* panel_rows;    // their physical rows
    typename F::T* E;       // m x ldE transform columns (may be null)
    int64_t ldE;
    typename F::Key* cand_key;  // [2][G] per-CTA proposals
    int64_t* cand_row;          // [2][G]
    typename F::T* cand_vals;   // [2][G][b] proposed rows
    GridBarrier bar;
    int rows_per_cta;
    const int* run_if;      // optional: the kernel does nothing unless *run_if != 0
    // float path, mixed precision: set *uncertain when a column's best pivot
    // candidate has magnitude in (band_lo, band_hi] (a rank decision the
    // reduced-precision updates could have tipped)
    int* uncertain = nullptr;
    double band_lo = 0.0, band_hi = 0.0;
};

// Multiply-accumulate policy of the SIMT trailing update, per field.
template <class F> struct GemmOps;

template <> struct GemmOps<FieldU32> {
    using Acc = uint64_t;
    static __device__ __forceinline__ Acc acc_zero(const FieldU32&) { return 0ull; }
    static __device__ __forceinline__ uint32_t b_zero(const FieldU32&) { return 0u; }
    static __device__ __forceinline__ uint32_t prep_b(const FieldU32&, uint32_t v) { return v; }
    // lazy accumulation: the caller folds after LAZY products (LAZY = 4 for
    // p < 2^31 keeps acc < p + 4 (p-1)^2 < 2^64)
    static __device__ __forceinline__ Acc mac(const FieldU32&, Acc acc, uint32_t a, uint32_t b) {
        return acc + (uint64_t)a * b;
    }
    static __device__ __forceinline__ Acc fold(const FieldU32& f, Acc acc) { return f.reduce64(acc); }
    static __device__ __forceinline__ uint32_t finish(const FieldU32& f, Acc acc, uint32_t c) {
        return f.add(c, f.reduce64(acc));
    }
};

template <> struct GemmOps<FieldU64> {
    using Acc = uint64_t;
    static __device__ __forceinline__ Acc acc_zero(const FieldU64&) { return 0ull; }
    static __device__ __forceinline__ uint64_t b_zero(const FieldU64&) { return 0ull; }
    // the B operand is kept in Montgomery form so that one REDC per product
    // yields the ordinary residue
    static __device__ __forceinline__ uint64_t prep_b(const FieldU64& f, uint64_t v) { return f.to_mont(v); }
    static __device__ __forceinline__ Acc mac(const FieldU64& f, Acc acc, uint64_t a, uint64_t b) {
        return f.add(acc, f.montmul(a, b));
    }
    static __device__ __forceinline__ Acc fold(const FieldU64&, Acc acc) { return acc; }
    static __device__ __forceinline__ uint64_t finish(const FieldU64& f, Acc acc, uint64_t c) {
        return f.add(c, acc);
    }
};

template <> struct GemmOps<FieldF64> {
    using Acc = double;
    static __device__ __forceinline__ Acc acc_zero(const FieldF64&) { return 0.0; }
    static __device__ __forceinline__ double b_zero(const FieldF64&) { return 0.0; }
    static __device__ __forceinline__ double prep_b(const FieldF64&, double v) { return v; }
    static __device__ __forceinline__ Acc mac(const FieldF64&, Acc acc, double a, double b) {
        return fma(a, b, acc);
    }
    static __device__ __forceinline__ Acc fold(const FieldF64&, Acc acc) { return acc; }
    static __device__ __forceinline__ double finish(const FieldF64&, Acc acc, double c) { return c + acc; }
};

template <> struct GemmOps<FieldC128> {
    using Acc = c128;
    static __device__ __forceinline__ Acc acc_zero(const FieldC128& f) { return f.zero(); }
    static __device__ __forceinline__ c128 b_zero(const FieldC128& f) { return f.zero(); }
    static __device__ __forceinline__ c128 prep_b(const FieldC128&, c128 v) { return v; }
    static __device__ __forceinline__ Acc mac(const FieldC128&, Acc acc, c128 a, c128 b) {
        acc.x = fma(a.x, b.x, acc.x);
        acc.x = fma(-a.y, b.y, acc.x);
        acc.y = fma(a.x, b.y, acc.y);
        acc.y = fma(a.y, b.x, acc.y);
        return acc;
    }
    static __device__ __forceinline__ Acc fold(const FieldC128&, Acc acc) { return acc; }
    static __device__ __forceinline__ c128 finish(const FieldC128&, Acc acc, c128 c) {
        c.x += acc.x;
        c.y += acc.y;
        return c;
    }
};

__device__ __forceinline__ double scale_real(double x, double s) { return x / s; }
__device__ __forceinline__ c128 scale_real(c128 x, double s) {
    c128 r;
    r.x = x.x / s;
    r.y = x.y / s;
    return r;
}

// Everything a trailing-update implementation needs for one panel.
template <class F>
struct TrailingCtx {
    F f;
    int64_t m = 0, n = 0;
    typename F::T* A = nullptr;
    int64_t lda = 0;
    const typename F::T* E = nullptr;  // m x ldE, transform columns
    int64_t ldE = 0;
    const typename F::T* Bm = nullptr; // k x ldb, pivot rows' trailing part
    int64_t ldb = 0;
    const int32_t* panel_k = nullptr;
    const int32_t* panel_rows = nullptr;  // physical rows of this panel's pivots
    int* err = nullptr;                // call-wide error word
    int* status = nullptr;             // module status word
    void* extra = nullptr;             // scratch reserved by trailing_extra_scratch
    int b = 0;
    int64_t j1 = 0, N = 0;             // trailing columns [j1, j1 + N)
    bool force_simt = false;
    bool predicated = false;           // runs only if the panel before it found pivots (fallback)
    void* fx = nullptr;                // float path: fixed-point tensor-core update scratch (mixed precision)
};

template <class F>
int trailing_update_simt(const TrailingCtx<F>& t, cudaStream_t s);

// Tensor-core trailing update for 32-bit residues (trailing_tc.cu).
int trailing_update_tc_u32(const TrailingCtx<FieldU32>& t, cudaStream_t s);
size_t trailing_tc_u32_scratch(int64_t m, int64_t n, int b);
bool trailing_tc_u32_available();

// Tiles per CTA of a limb contraction over row_blocks x n_tiles tiles: the
// grid's waves (CTAs over the SM count) times the tiles each CTA runs plus
// its fixed start-up (E digits load, TMEM allocation; about 0.6 tile),
// minimised over 4 .. 48 (trailing_tc.cu).
int limb_tiles_per_cta(int n_tiles, int row_blocks);

// Reusable tensor-core pieces (trailing_tc.cu)
size_t tc_el_bytes(int64_t m);
size_t tc_bs_bytes(int64_t n);
int tc_m_pad(int64_t m);
int tc_split_e(const uint32_t* E, int64_t ldE, int b, int64_t m, uint32_t p, const int32_t* k_ptr, void* EL,
               cudaStream_t s, int max_grid = 0);
int tc_gather_split_b(uint32_t* C, int64_t ldc, int64_t N, const int32_t* rows, const int32_t* k_ptr, uint32_t p,
                      void* BS, bool zero_src, cudaStream_t s);
int tc_limb_gemm(const FieldU32& f, uint32_t* C, int64_t ldc, int64_t m, int64_t N, const int32_t* k_ptr,
                 bool overwrite, const void* EL, const void* BS, int64_t n_map, int* err, int* status,
                 cudaStream_t s, bool count_work = true, int tiles_per_cta = 0);

// Candidate-block panel for F_p with 32-bit residues (cand_panel.cu)
constexpr int kCandThreads = 512;
constexpr int kCandRows = 160;  // candidate rows per panel (panel width + 32)
struct CandMont {
    uint32_t p, pinv, r2;
    uint64_t mu;
};
struct CandArgs {
    const void* A;        // residues (uint32, or uint64 for the 64-bit panel)
    int64_t lda;
    int64_t m;
    int64_t j0;
    int bw;
    int smax;
    uint8_t* row_used;
    int32_t* cand;      // [256] current candidate rows
    int32_t* cand_n;
    int32_t* next_row;  // rows >= next_row have not been candidates yet
    int64_t* rank;
    int32_t* piv_row;
    int64_t* piv_col;
    int32_t* panel_k;
    int32_t* panel_rows;
    int32_t* panel_cols;
    int32_t* panel_mark;  // (gen << 8) | (t + 1) for the pivot rows of panel `gen`
    int gen;
    void* X;              // [PW][PW] inverse of the pivot block (residue words)
    uint32_t* pivmask;    // [4] pivot columns of the panel
    int* missed;
    struct {
        uint32_t p, pinv, r2;
        uint64_t mu;
    } M;
    FieldU64 f64;         // 64-bit panel: the field's Montgomery constants
};
int launch_cand_panel(const CandArgs& a, cudaStream_t s);
int launch_split_g(const uint32_t* A, int64_t lda, int64_t m, int64_t j0, uint32_t p, const int32_t* panel_k,
                   const int32_t* panel_cols, const int32_t* panel_mark, int gen, void* EL, cudaStream_t s);
int launch_check_missed(const uint32_t* A, int64_t lda, int64_t m, int64_t j0, int bw, const uint8_t* row_used,
                        const uint32_t* pivmask, int* missed, cudaStream_t s);
// 64-bit residues: candidate panel of 64 columns and its miss check (cand_panel.cu)
constexpr int kPanelU64 = 64;
int launch_cand_panel64(const CandArgs& a, cudaStream_t s);
int launch_check_missed64(const uint64_t* A, int64_t lda, int64_t m, int64_t j0, int bw, const uint8_t* row_used,
                          const uint32_t* pivmask, int* missed, cudaStream_t s);

// Tensor-core trailing update for 64-bit residues (trailing_tc64.cu); panels of <= 64 columns
int trailing_update_tc_u64(const TrailingCtx<FieldU64>& t, cudaStream_t s);
size_t trailing_tc_u64_scratch(int64_t m, int64_t n);
bool trailing_tc_u64_available();
constexpr int kMaxPanelU64Tc = 64;
int tc64_split_e(const uint64_t* E, int64_t ldE, int64_t m, uint64_t p, const int32_t* k_ptr, void* EL,
                 cudaStream_t s, int max_grid = 0);
int tc64_split_g(const uint64_t* A, int64_t lda, int64_t m, int64_t j0, uint64_t p, const int32_t* k_ptr,
                 const int32_t* panel_cols, const int32_t* panel_mark, int gen, void* EL, cudaStream_t s);
int tc64_gather_split_b(uint64_t* C, int64_t ldc, int64_t N, const int32_t* rows, const int32_t* k_ptr, uint64_t p,
                        void* BS, bool zero_src, cudaStream_t s);
int tc64_limb_gemm(const FieldU64& f, uint64_t* C, int64_t ldc, int64_t m, int64_t N, const int32_t* k_ptr,
                   bool overwrite, const void* EL, const void* BS, int* err, int* status, cudaStream_t s,
                   bool count_work, int kwork, int tiles_per_cta = 0);
void* tc64_bs_base(void* extra, int64_t m);  // B digit tiles inside the 64-bit update's scratch
size_t tc64_el_bytes(int64_t m);             // E digit planes of m rows
size_t tc64_bs_bytes(int64_t n);             // B digit tiles of n columns

template <class F>
inline size_t trailing_extra_scratch(int64_t m, int64_t n, const RrefPlan& pl) {
    if constexpr (F::kDtype == 1) return trailing_tc_u32_scratch(m, n, pl.b);
    if constexpr (F::kDtype == 2) return trailing_tc_u64_available() ? trailing_tc_u64_scratch(m, n) : 0;
    return 0;
}

// Fixed-point tensor-core trailing update of the float path (trailing_fx.cu)
template <class F>
int trailing_update_fx(const TrailingCtx<F>& t, cudaStream_t s);
size_t trailing_fx_scratch(int64_t m, int64_t n, bool cplx);
// FP64 refinement kernels (trailing_fx.cu)
template <class T>
int refine_narrow_gemm(int64_t m, int q, int64_t K, const int32_t* k_ptr, const T* A, int64_t lda, const T* B,
                       int64_t ldb, T* C, int64_t ldc, cudaStream_t s);
template <class T>
int refine_build_z(int64_t n, int q, const int32_t* colmap, const int32_t* Nc, const T* R, int64_t ldr, T* Z,
                   cudaStream_t s);
template <class T>
int refine_apply(int64_t rank, int q, const int32_t* piv_row, const int32_t* Nc, const T* D, T* R, int64_t ldr,
                 unsigned long long* stats, cudaStream_t s, bool apply = true);

template <class F>
inline int trailing_update(const TrailingCtx<F>& t, cudaStream_t s) {
    if constexpr (F::kDtype == 1) {
        if (!t.force_simt && trailing_tc_u32_available()) return trailing_update_tc_u32(t, s);
    }
    if constexpr (F::kDtype == 2) {
        if (!t.force_simt && t.b <= kMaxPanelU64Tc && trailing_tc_u64_available()) return trailing_update_tc_u64(t, s);
    }
    if constexpr (F::kDtype == 3 || F::kDtype == 4) {
        if (t.fx) return trailing_update_fx<F>(t, s);
    }
    return trailing_update_simt<F>(t, s);
}

int rref_device_dispatch(int dtype, int64_t m, int64_t n, uint64_t p, double tol, void* work,
                         int64_t ldw, void* out, int64_t ldo, int64_t* dev_piv, int64_t* dev_rank,
                         cudaStream_t s, int flags);
int rref_read_and_clear_status(int* status);
size_t rref_device_scratch(int dtype, int64_t m, int64_t n);
int mixed_report(int* iterations, double* last_correction, int* redone);
double mixed_error_estimate();
// every matrix of a batch through the single-matrix path on `workers` concurrent streams (float_batch.cu)
int concurrent_batch(int dtype, const lnc_batch_matrix* mats, int64_t count, double tol, int flags, int workers,
                     lnc_mixed_result* reports);

}  // namespace lnc
