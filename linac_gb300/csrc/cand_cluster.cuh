// Candidate-block panel on a thread-block cluster (device code).
//
// The single-CTA panel (cand_body) runs the whole 160-row candidate block on
// one SM; its per-column chain (pivot row, inverse, normalisation, update of
// 127 columns) is bound by that SM's issue rate.  Here CL CTAs of one cluster
// split the panel's columns (CTA r holds columns [r CW, r CW + CW) of every
// candidate row in its shared memory) and exchange, per pivot step, only
// what the step needs: the pivot row index, the pivot value and the pivot
// column's entries (the multipliers), pushed by the owner of that column into
// every CTA's shared memory (distributed shared memory, double-buffered by
// step parity) and released at a cluster barrier.
//
// The elimination is fraction-free, so no inverse sits on the per-column
// chain: step s with pivot row p, pivot value a and multipliers f updates
// every other row as  x <- a x - f_i v  (v: the pivot row's entry in that
// column) and leaves row p as it is.  The pivot column itself becomes the
// transform column (-f_i, and 1 in row p), and earlier transform columns are
// updated like any other column.  For the product T of the step matrices,
// the column of pivot u then holds T[:, p_u] / S_u with S_u = a_0 ... a_(u-1)
// (row p_u was scaled by every earlier step before it became a pivot row),
// and T A[P, Q] is diagonal with entries d_t = a_t a_(t+1) ... a_(k-1), so the
// pivot block's inverse is
//     X[t][u] = col_u[p_t] S_u / d_t = col_u[p_t] S_u S_t / (a_0 ... a_(k-1)):
// one inverse per panel (of the product of all pivots) replaces one per
// column.  Pivot choice (first candidate row, in candidate order, with a
// non-zero entry) and therefore every output equal the single-CTA panel's:
// fraction-free values are non-zero multiples of the normalised ones.
//
// Look-ahead: while the other warps apply step s, warp 0 of the CTA owning
// column s + 1 updates that column first, picks its pivot row, pushes step
// s + 1's data and arrives at the cluster barrier with release semantics; the
// other threads arrive (relaxed) as soon as they have read step s's slot, and
// every thread waits at the start of the next step.  All threads alternate
// arrive and wait the same number of times (one full barrier before the
// loop, one phase per column, one full barrier at the end); no CTA returns
// early.
#pragma once

#include "cand_kernels.cuh"

namespace lnc {
namespace ccl {

__device__ __forceinline__ uint32_t cta_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
// every thread of every CTA of the cluster; orders distributed shared-memory stores
__device__ __forceinline__ void cluster_sync() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// split phases: a thread arrives once it no longer needs what the next phase's
// producers overwrite, and waits only when it needs what they produce
__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.release;" ::: "memory"); }
// arrival that publishes nothing (the thread only signals that it has read a slot)
__device__ __forceinline__ void cluster_arrive_relaxed() { asm volatile("barrier.cluster.arrive.relaxed;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire;" ::: "memory"); }
__device__ __forceinline__ uint32_t map_rank(const void* p, uint32_t rank) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
    return r;
}
__device__ __forceinline__ void st_remote(uint32_t addr, uint32_t v) {
    asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
}
__device__ __forceinline__ void st_remote(uint32_t addr, uint64_t v) {
    asm volatile("st.shared::cluster.u64 [%0], %1;" ::"r"(addr), "l"(v) : "memory");
}

}  // namespace ccl

constexpr int kCandClusterThreads = 256;
constexpr int kCandFcolPitch = 168;  // >= kCandRows, multiple of 8

// dynamic shared memory of one CTA: its column slice of the block, column-major, odd pitch
template <class W, int PW, int CL>
__host__ __device__ constexpr size_t cand_cluster_smem(int smax) {
    return (size_t)(smax | 1) * (PW / CL) * sizeof(W);
}

template <class Arith, class W, int PW, int CL>
__device__ __forceinline__ void cand_cluster_body(const CandArgs& a) {
    constexpr int CW = PW / CL;  // columns per CTA
    constexpr int NW = kCandClusterThreads / 32;
    constexpr int RPL = (kCandRows + 31) / 32;  // candidate rows per lane
    using Pre = typename Arith::Pre;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int LDT = a.smax | 1;
    W* tile = (W*)smem_raw;  // [CW][LDT]: local column cl = global column base + cl

    __shared__ __align__(16) W s_f[2][kCandFcolPitch];  // step multipliers (pushed by the step's owner)
    __shared__ int s_spi[2];                            // step pivot row (-1: none)
    __shared__ W s_sa[2];                               // step pivot value
    __shared__ int s_cand[256];
    __shared__ uint8_t s_isp[256];
    __shared__ int s_pr[PW], s_pc[PW];
    __shared__ W s_pa[PW];    // pivot values in step order
    __shared__ W s_scale[PW + 1];  // S_t, then S_t / P
    __shared__ int s_opc[CW];  // this CTA's pivot columns (global), in step order
    __shared__ int s_ko;
    __shared__ int s_warp[32];
    __shared__ int s_n, s_total, s_next;

    const Arith ar = make_arith<Arith>(a);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int rank = (int)ccl::cta_rank();
    const int base = rank * CW;
    const int bw = a.bw;
    auto owner = [&](int c) { return c / CW; };

    // ---- candidate rows (every CTA derives the same list from the same global state)
    if (tid == 0) {
        if (rank == 0) *a.missed = 0;
        s_next = *a.next_row;
        s_ko = 0;
    }
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
        const int b0 = s_next;
        const int r = b0 + tid;
        const int e = (r < a.m) ? !a.row_used[r] : 0;
        const int pos = block_scan_flag(e, s_warp, &s_total);
        const int need = a.smax - s_n;
        if (e && pos < need) s_cand[s_n + pos] = r;
        if (e && pos == need - 1) s_next = r + 1;
        __syncthreads();
        if (tid == 0) {
            if (s_total < need) {
                s_n += s_total;
                s_next = min((int64_t)b0 + (int64_t)blockDim.x, a.m);
            } else {
                s_n += need;
            }
        }
        __syncthreads();
    }
    const int n = s_n;
    // ---- this CTA's columns of the block
    for (int i = warp; i < n; i += NW) {
        const W* src = (const W*)a.A + (int64_t)s_cand[i] * a.lda + a.j0 + base;
        for (int cl = lane; cl < CW; cl += 32)
            if (base + cl < bw) tile[(size_t)cl * LDT + i] = src[cl];
    }
    for (int i = tid; i < 256; i += blockDim.x) s_isp[i] = 0;
    // remote addresses of every CTA's step slots (lanes of warp 0 push)
    uint32_t r_f[CL], r_pi[CL], r_a[CL];
#pragma unroll
    for (int q = 0; q < CL; ++q) {
        r_f[q] = ccl::map_rank(&s_f[0][0], (uint32_t)q);
        r_pi[q] = ccl::map_rank(&s_spi[0], (uint32_t)q);
        r_a[q] = ccl::map_rank(&s_sa[0], (uint32_t)q);
    }
    __syncthreads();

    // warp 0 of the owner of column c: first non-pivot candidate row with a non-zero entry, and
    // the push of step c's row, value and multipliers into slot `slot` of every CTA
    auto pick_and_push = [&](int c, int slot) {
        const W* colp = tile + (size_t)(c - base) * LDT;
        int found = -1;
        W v[RPL];
#pragma unroll
        for (int j = 0; j < RPL; ++j) {  // independent loads and ballots
            const int i = lane + 32 * j;
            v[j] = (i < n) ? colp[i] : (W)0;
            const unsigned bal = __ballot_sync(0xffffffffu, i < n && !s_isp[i] && v[j] != 0);
            if (found < 0 && bal) found = 32 * j + __ffs(bal) - 1;
        }
        if (found >= 0) {
#pragma unroll
            for (int j = 0; j < RPL; ++j) {
                const int i = lane + 32 * j;
                if (i < n) {
#pragma unroll
                    for (int q = 0; q < CL; ++q)
                        ccl::st_remote(r_f[q] + (uint32_t)((slot * kCandFcolPitch + i) * sizeof(W)), v[j]);
                }
            }
        }
        if (lane < CL) {
            ccl::st_remote(r_pi[lane] + (uint32_t)(slot * sizeof(int)), (uint32_t)found);
            ccl::st_remote(r_a[lane] + (uint32_t)(slot * sizeof(W)), found >= 0 ? colp[found] : (W)0);
        }
    };

    ccl::cluster_sync();  // every CTA resident and initialised before the first push
    if (bw > 0 && owner(0) == rank && warp == 0) pick_and_push(0, 0);
    ccl::cluster_arrive();

    // Each step: wait for its data, read it, arrive (so the next-but-one producer may reuse the
    // slot; the producer of the next step arrives after its push), then update.  A CTA's warps
    // meet at __syncthreads before the look-ahead touches the tile again.
    int k = 0;
    for (int c = 0; c < bw; ++c) {
        const int slot = c & 1;
        ccl::cluster_wait();
        const int pi = s_spi[slot];
        const W av = s_sa[slot];
        const bool mine = owner(c) == rank;
        const bool la_owner = (c + 1 < bw) && owner(c + 1) == rank;
        W fr[RPL];
#pragma unroll
        for (int j = 0; j < RPL; ++j) {
            const int i = lane + 32 * j;
            fr[j] = (pi >= 0 && i < n) ? s_f[slot][i] : (W)0;
        }
        if (tid == 0 && pi >= 0) {
            s_pr[k] = pi;
            s_pc[k] = c;
            s_pa[k] = av;
            s_isp[pi] = 1;
            if (mine) s_opc[s_ko++] = c;
        }
        __syncthreads();
        const int kop = s_ko - ((mine && pi >= 0) ? 1 : 0);  // earlier transform columns of this CTA
        const Pre A = ar.pre_ff(av);
        if (la_owner && warp == 0) {
            if (pi >= 0) {
                W* colp = tile + (size_t)(c + 1 - base) * LDT;
                const Pre V = ar.pre_ff(colp[pi]);
#pragma unroll
                for (int j = 0; j < RPL; ++j) {
                    const int i = lane + 32 * j;
                    if (i < n && i != pi) colp[i] = ar.ffsub(colp[i], A, fr[j], V);
                }
                __syncwarp();
            }
            pick_and_push(c + 1, slot ^ 1);
            ccl::cluster_arrive();
        } else {
            ccl::cluster_arrive_relaxed();
            if (pi >= 0) {
                // this CTA's targets: columns right of c (c + 1 excepted when warp 0 has it), the
                // earlier transform columns, and column c itself when it is here
                const int lo = max(c + 1 + (la_owner ? 1 : 0), base);
                const int hi = min(base + CW, bw);
                const int nright = hi > lo ? hi - lo : 0;
                const int ntarget = nright + kop + (mine ? 1 : 0);
                const int w0 = la_owner ? 1 : 0;
                for (int t = warp - w0; t < ntarget; t += NW - w0) {
                    const int cc = (t < nright) ? lo + t : ((t - nright < kop) ? s_opc[t - nright] : c);
                    W* colp = tile + (size_t)(cc - base) * LDT;
                    if (cc == c) {
                        // transform column of this step: -f in every other row, 1 in the pivot row
#pragma unroll
                        for (int j = 0; j < RPL; ++j) {
                            const int i = lane + 32 * j;
                            if (i < n) colp[i] = (i == pi) ? (W)1 : ar.neg(fr[j]);
                        }
                    } else {
                        const Pre V = ar.pre_ff(colp[pi]);  // the pivot row's entry (row pi is not written)
#pragma unroll
                        for (int j = 0; j < RPL; ++j) {
                            const int i = lane + 32 * j;
                            if (i < n && i != pi) colp[i] = ar.ffsub(colp[i], A, fr[j], V);
                        }
                    }
                }
            }
        }
        if (pi >= 0) ++k;
    }
    ccl::cluster_wait();  // pairs the last arrive: every CTA is done with the slots
    __syncthreads();

    // ---- X = A[P, Q]^-1 from the transform columns: X[t][u] = T[p_t, p_u] S_u S_t / P
    if (warp == 0) {
        // inclusive prefix products of the pivot values (PW / 32 per lane), S_0 = 1
        constexpr int PL = PW / 32;
        W loc[PL];
        W run = (W)1;
#pragma unroll
        for (int j = 0; j < PL; ++j) {
            const int t = lane * PL + j;
            const W v = (t < k) ? s_pa[t] : (W)1;
            run = (j == 0) ? v : ar.mul(run, v);
            loc[j] = run;
        }
        W incl = run;  // product of this lane's chunk -> inclusive scan over lanes
        for (int o = 1; o < 32; o <<= 1) {
            const W up = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl = ar.mul(incl, up);
        }
        W excl = __shfl_up_sync(0xffffffffu, incl, 1);
        if (lane == 0) excl = (W)1;
        const W total = __shfl_sync(0xffffffffu, incl, 31);
        const W tinv = (k > 0) ? ar.inverse(total) : (W)1;
#pragma unroll
        for (int j = 0; j < PL; ++j) {
            const int t = lane * PL + j;
            // S_t = product of a_0 .. a_(t-1): the exclusive prefix
            const W st = (j == 0) ? excl : ar.mul(excl, loc[j - 1]);
            s_scale[t] = st;  // S_t (column factor)
            if (t < PW) s_pa[t] = ar.mul(st, tinv);  // S_t / P (row factor), reuses s_pa
        }
    }
    __syncthreads();
    W* X = (W*)a.X;  // [PW][PW]
    for (int idx = tid; idx < PW * PW; idx += blockDim.x) {
        const int t = idx / PW, u = idx % PW;
        if (u < k) {
            const int q = s_pc[u];
            if (owner(q) != rank) continue;
            X[idx] = (t < k) ? ar.mul(ar.mul(tile[(size_t)(q - base) * LDT + s_pr[t]], s_scale[u]), s_pa[t]) : (W)0;
        } else if (rank == 0) {
            X[idx] = (W)0;
        }
    }
    const int64_t rank0 = *a.rank;
    if (rank == 0) {
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
    }
    {
        const int keep = (tid < n) ? !s_isp[tid] : 0;
        const int pos = block_scan_flag(keep, s_warp, &s_total);
        if (rank == 0) {
            if (keep) a.cand[pos] = s_cand[tid];
            if (tid == 0) {
                *a.cand_n = s_total;
                *a.next_row = s_next;
                *a.panel_k = k;
                *a.rank = rank0 + k;
            }
        }
    }
    ccl::cluster_sync();
}

}  // namespace lnc
