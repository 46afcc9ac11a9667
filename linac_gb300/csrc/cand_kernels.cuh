// Candidate-block panel kernels (device code shared by cand_panel.cu and
// batch.cu).  See cand_panel.cu for the method.
#pragma once

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

// Arithmetic policies of the candidate panel.  `prep` / `aux` turn a
// normalised pivot-row value v into the form(s) the update uses, and
// `mulsub(x, f, prep(v), aux(v))` is x - f v mod p; `mul` multiplies two
// ordinary residues.
struct ArithSmall {  // odd p < 2^31: 32-bit Montgomery, reductions by unsigned min
    Mont32 M;
    __device__ ArithSmall(const decltype(CandArgs::M)& c) : M(c) {}
    __device__ __forceinline__ uint32_t red(uint64_t t) const {
        const uint32_t lo = (uint32_t)t, hi = (uint32_t)(t >> 32);
        const uint32_t mh = __umulhi(lo * M.pinv, M.p);
        const uint32_t u = hi + mh + (lo != 0u ? 1u : 0u);  // < 2p < 2^32
        return min(u, u - M.p);
    }
    __device__ __forceinline__ uint32_t montmul(uint32_t a, uint32_t b) const { return red((uint64_t)a * b); }
    __device__ __forceinline__ uint32_t prep(uint32_t v) const { return v; }
    // Shoup's constant of a fixed multiplier v < p: floor(v 2^32 / p), by Barrett division with
    // mu = floor((2^64 - 1) / p): the estimate falls short by at most two (integer pipe only;
    // this part's FP64 rate is far too low for a per-column quotient)
    __device__ __forceinline__ uint32_t aux(uint32_t v) const {
        const uint64_t x = (uint64_t)v << 32;
        uint64_t q = __umul64hi(x, M.mu);
        uint64_t r = x - q * (uint64_t)M.p;
        if (r >= M.p) { ++q; r -= M.p; }
        if (r >= M.p) ++q;
        return (uint32_t)q;
    }
    // x - f v mod p with v's Shoup constant vs: q = floor(f vs / 2^32) undershoots f v / p by at
    // most 1, so f v - q p lies in [0, 2p) (computed mod 2^32; 2p < 2^32)
    __device__ __forceinline__ uint32_t mulsub(uint32_t x, uint32_t f, uint32_t v, uint32_t vs) const {
        const uint32_t q = __umulhi(f, vs);
        uint32_t r = f * v - q * M.p;
        r = min(r, r - M.p);
        const uint32_t d = x - r;
        return min(d, d + M.p);
    }
    __device__ __forceinline__ uint32_t mul(uint32_t a, uint32_t b) const { return montmul(montmul(a, b), M.r2); }
    __device__ __forceinline__ uint32_t sub(uint32_t a, uint32_t b) const {
        const uint32_t d = a - b;
        return min(d, d + M.p);
    }
    __device__ __forceinline__ uint32_t inverse(uint32_t a) const { return inv_binary<uint32_t>(a, M.p); }
    // fraction-free step  a x - f v  with both fixed factors prepared (value, Shoup constant)
    using Pre = uint2;
    __device__ __forceinline__ uint32_t neg(uint32_t f) const { return f ? M.p - f : 0u; }
    __device__ __forceinline__ Pre pre_ff(uint32_t v) const { return make_uint2(v, aux(v)); }
    __device__ __forceinline__ uint32_t shoup(uint32_t x, uint2 w) const {  // x w mod p, any 32-bit x
        const uint32_t q = __umulhi(x, w.y);
        const uint32_t r = x * w.x - q * M.p;
        return min(r, r - M.p);
    }
    __device__ __forceinline__ uint32_t ffsub(uint32_t x, uint2 a, uint32_t f, uint2 v) const {
        const uint32_t d = shoup(x, a) - shoup(f, v);
        return min(d, d + M.p);
    }
};
struct ArithMont {  // odd p >= 2^31
    Mont32 M;
    __device__ ArithMont(const decltype(CandArgs::M)& c) : M(c) {}
    __device__ __forceinline__ uint32_t prep(uint32_t v) const { return M.to_mont(v); }
    __device__ __forceinline__ uint32_t aux(uint32_t) const { return 0u; }
    __device__ __forceinline__ uint32_t mulsub(uint32_t x, uint32_t f, uint32_t vp, uint32_t) const {
        return M.sub(x, M.montmul(f, vp));
    }
    __device__ __forceinline__ uint32_t mul(uint32_t a, uint32_t b) const { return M.montmul(M.to_mont(a), b); }
    __device__ __forceinline__ uint32_t sub(uint32_t a, uint32_t b) const { return M.sub(a, b); }
    __device__ __forceinline__ uint32_t inverse(uint32_t a) const { return inv_binary<uint32_t>(a, M.p); }
    using Pre = uint32_t;  // Montgomery form
    __device__ __forceinline__ uint32_t neg(uint32_t f) const { return f ? M.p - f : 0u; }
    __device__ __forceinline__ Pre pre_ff(uint32_t v) const { return M.to_mont(v); }
    __device__ __forceinline__ uint32_t ffsub(uint32_t x, Pre a, uint32_t f, Pre v) const {
        return M.sub(M.montmul(x, a), M.montmul(f, v));
    }
};
struct ArithTwo {  // p = 2
    Mont32 M;
    __device__ ArithTwo(const decltype(CandArgs::M)& c) : M(c) {}
    __device__ __forceinline__ uint32_t prep(uint32_t v) const { return v; }
    __device__ __forceinline__ uint32_t aux(uint32_t) const { return 0u; }
    __device__ __forceinline__ uint32_t mulsub(uint32_t x, uint32_t f, uint32_t vp, uint32_t) const {
        return M.sub(x, M.barrett((uint64_t)f * vp));
    }
    __device__ __forceinline__ uint32_t mul(uint32_t a, uint32_t b) const { return M.barrett((uint64_t)a * b); }
    __device__ __forceinline__ uint32_t sub(uint32_t a, uint32_t b) const { return M.sub(a, b); }
    __device__ __forceinline__ uint32_t inverse(uint32_t) const { return 1u; }
    using Pre = uint32_t;
    __device__ __forceinline__ uint32_t neg(uint32_t f) const { return f; }  // -1 = 1 mod 2
    __device__ __forceinline__ Pre pre_ff(uint32_t v) const { return v; }
    __device__ __forceinline__ uint32_t ffsub(uint32_t x, Pre a, uint32_t f, Pre v) const {
        return (x & a) ^ (f & v);  // residues 0 / 1
    }
};

struct Arith64 {  // 64-bit residues (odd p < 2^64): Montgomery with R = 2^64
    FieldU64 F;
    __device__ Arith64(const CandArgs& a) : F(a.f64) {}
    __device__ __forceinline__ uint64_t prep(uint64_t v) const { return F.to_mont(v); }
    __device__ __forceinline__ uint64_t aux(uint64_t) const { return 0ull; }
    __device__ __forceinline__ uint64_t mulsub(uint64_t x, uint64_t f, uint64_t vp, uint64_t) const {
        return F.sub(x, F.montmul(f, vp));  // f (v R) R^-1 = f v
    }
    __device__ __forceinline__ uint64_t mul(uint64_t a, uint64_t b) const { return F.mul(a, b); }
    __device__ __forceinline__ uint64_t inverse(uint64_t a) const { return inv_binary<uint64_t>(a, F.p); }
    using Pre = uint64_t;  // Montgomery form
    __device__ __forceinline__ uint64_t neg(uint64_t f) const { return f ? F.p - f : 0ull; }
    __device__ __forceinline__ Pre pre_ff(uint64_t v) const { return F.to_mont(v); }
    __device__ __forceinline__ uint64_t ffsub(uint64_t x, Pre a, uint64_t f, Pre v) const {
        return F.sub(F.montmul(x, a), F.montmul(f, v));
    }
};

// arithmetic policies are built from the panel arguments
template <class Arith>
__device__ __forceinline__ Arith make_arith(const CandArgs& a) { return Arith(a.M); }
template <>
__device__ __forceinline__ Arith64 make_arith<Arith64>(const CandArgs& a) { return Arith64(a); }

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

// dynamic shared memory of the candidate panel for word type W and panel width PW
template <class W, int PW>
__host__ __device__ constexpr size_t cand_smem(int smax) {
    return ((size_t)(smax | 1) * PW + 2 * PW + 256) * sizeof(W);
}

// W: residue word (uint32_t, or uint64_t for 64-bit primes); PW: panel width
template <class Arith, class W = uint32_t, int PW = kMaxPanel>
__device__ __forceinline__ void cand_body(const CandArgs& a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int bw = a.bw;
    // column-major block, odd pitch: a column (fixed c, consecutive rows) and a
    // row (fixed i, consecutive columns) are both free of bank conflicts
    const int LDT = a.smax | 1;
    W* tile = (W*)smem_raw;                   // [bw][LDT]
    W* nprM = tile + (size_t)LDT * PW;        // [PW]
    W* fcol = nprM + PW;                      // [256]
    W* nprS = fcol + 256;                     // [PW] aux(v) of the pivot row
    __shared__ int s_cand[256];
    __shared__ uint8_t s_isp[256];
    __shared__ int s_pr[PW], s_pc[PW];
    __shared__ int s_warp[32];
    __shared__ int s_n, s_total, s_next;
    __shared__ int s_npi;           // look-ahead: pivot row of the next column (-1: none)
    __shared__ W s_ninv;            // and the inverse of its entry
    const Arith ar = make_arith<Arith>(a);
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
        const W* src = (const W*)a.A + (int64_t)s_cand[i] * a.lda + a.j0;
        for (int c = lane; c < bw; c += 32) tile[(size_t)c * LDT + i] = src[c];
    }
    for (int i = tid; i < 256; i += blockDim.x) s_isp[i] = 0;
    __syncthreads();

    // ---- Gauss-Jordan on the block, transform kept in the pivot columns.
    // Look-ahead: while warps 1.. eliminate column c's pivot from the rest of the
    // block, warp 0 first brings column c+1 up to date, picks its pivot row and
    // computes the inverse, so the serial inverse overlaps the bulk update.
    // Lanes run over rows, so each lane keeps its rows' multipliers in registers.
    constexpr int RPL = (kCandRows + 31) / 32;  // rows per lane (n <= kCandRows)
    auto pick_pivot = [&](int col, int exclude) {
        // warp 0: first candidate row, not a pivot row and not `exclude`, with a
        // non-zero entry in column `col`; lane 0 then computes its inverse
        int found = -1;
        const W* colp = tile + (size_t)col * LDT;
        for (int base = 0; base < n && found < 0; base += 32) {
            const int i = base + lane;
            const bool ok = i < n && !s_isp[i] && i != exclude && colp[i] != 0;
            const unsigned b = __ballot_sync(0xffffffffu, ok);
            if (b) found = base + __ffs(b) - 1;
        }
        if (lane == 0) {
            s_npi = found;
            s_ninv = (found >= 0) ? ar.inverse(colp[found]) : (W)0;
        }
    };
    if (warp == 0) pick_pivot(0, -1);
    __syncthreads();
    int k = 0;
    for (int c = 0; c < bw; ++c) {
        const int pi = s_npi;
        const W inv = s_ninv;
        if (pi < 0) {
            // column c has no pivot: nothing changes, look at column c + 1
            __syncthreads();
            if (warp == 0 && c + 1 < bw) pick_pivot(c + 1, -1);
            __syncthreads();
            continue;
        }
        // normalised pivot row (its column c holds the inverse: the transform) and
        // the multipliers of every other row
        for (int cc = tid; cc < bw; cc += blockDim.x) {
            W* e = tile + (size_t)cc * LDT + pi;
            const W v = (cc == c) ? inv : ar.mul(*e, inv);
            nprM[cc] = ar.prep(v);
            nprS[cc] = ar.aux(v);
            *e = v;
        }
        for (int i = tid; i < n; i += blockDim.x) fcol[i] = (i == pi) ? (W)0 : tile[(size_t)c * LDT + i];
        __syncthreads();
        // this lane's rows and their multipliers (0 for the pivot row and absent rows)
        W fr[RPL];
#pragma unroll
        for (int j = 0; j < RPL; ++j) {
            const int i = lane + 32 * j;
            fr[j] = (i < n) ? fcol[i] : (W)0;
        }
        if (warp == 0) {
            if (c + 1 < bw) {
                W* colp = tile + (size_t)(c + 1) * LDT;
                const W vp = nprM[c + 1], vs = nprS[c + 1];
#pragma unroll
                for (int j = 0; j < RPL; ++j) {
                    const int i = lane + 32 * j;
                    if (fr[j] != 0) colp[i] = ar.mulsub(colp[i], fr[j], vp, vs);
                }
                __syncwarp();
                pick_pivot(c + 1, pi);
            }
        } else {
            // target columns: right of c + 1, then the transform columns (earlier
            // pivot columns and c).  Earlier columns without a pivot are zero in the
            // pivot row and stay as they are.
            const int nright = bw - c - 2 > 0 ? bw - c - 2 : 0;
            const int ntarget = nright + k + 1;
            for (int t = warp - 1; t < ntarget; t += NW - 1) {
                const int cc = (t < nright) ? c + 2 + t : ((t - nright < k) ? s_pc[t - nright] : c);
                W* colp = tile + (size_t)cc * LDT;
                const W vp = nprM[cc], vs = nprS[cc];
                const bool zero_first = (cc == c);
#pragma unroll
                for (int j = 0; j < RPL; ++j) {
                    const int i = lane + 32 * j;
                    if (fr[j] != 0) {
                        const W x = zero_first ? (W)0 : colp[i];
                        colp[i] = ar.mulsub(x, fr[j], vp, vs);
                    }
                }
            }
        }
        __syncthreads();
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
    W* X = (W*)a.X;  // [PW][PW]
    for (int idx = tid; idx < PW * PW; idx += blockDim.x) {
        const int t = idx / PW, u = idx % PW;
        X[idx] = (t < k && u < k) ? tile[(size_t)s_pc[u] * LDT + s_pr[t]] : (W)0;
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

template <class Arith, class W = uint32_t, int PW = kMaxPanel>
static __global__ void __launch_bounds__(kCandThreads, 1) cand_panel_kernel(const __grid_constant__ CandArgs a) {
    cand_body<Arith, W, PW>(a);
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

__device__ __forceinline__ void split_g_body(const uint32_t* A, int64_t lda, int64_t m, int m_pad, int64_t j0,
                                             uint32_t p, const int32_t* panel_k, const int32_t* panel_cols,
                                             const int32_t* panel_mark, int gen, __nv_bfloat16* EL) {
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
template <class W = uint32_t>
__device__ __forceinline__ void check_missed_body(const W* A, int64_t lda, int64_t m, int64_t j0, int bw,
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
        const W* row = A + r * lda + j0;
        for (int c = lane; c < bw; c += 32)
            if (!((s_mask[c >> 5] >> (c & 31)) & 1u) && row[c] != 0) bad = 1;
    }
    if (__any_sync(0xffffffffu, bad) && lane == 0) atomicExch(missed, 1);
}

static __global__ void split_g_kernel(const uint32_t* A, int64_t lda, int64_t m, int m_pad, int64_t j0, uint32_t p,
                                      const int32_t* panel_k, const int32_t* panel_cols, const int32_t* panel_mark,
                                      int gen, __nv_bfloat16* EL) {
    split_g_body(A, lda, m, m_pad, j0, p, panel_k, panel_cols, panel_mark, gen, EL);
}

template <class W = uint32_t>
static __global__ void check_missed_kernel(const W* A, int64_t lda, int64_t m, int64_t j0, int bw,
                                           const uint8_t* row_used, const uint32_t* pivmask, int* missed) {
    check_missed_body<W>(A, lda, m, j0, bw, row_used, pivmask, missed);
}

}  // namespace lnc
