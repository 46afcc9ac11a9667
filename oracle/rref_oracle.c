/*
 * CPU oracle for the dense RREF and monomial-loader path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA library is
 * compared against: only tests/, __graft_entry__.smoke() and bench.py (its
 * cpu_baseline leg and its `--impl reference` arm) may load it.  Nothing in the
 * linac_gb300 package links or calls it.
 *
 * It restates, in plain C, the algorithm of linac's CPU `row_reduce`
 * (linac/row_reduce.py:16-78) and the CPU branch of `load_matrices`
 * (linac/pycuda_matrix_loader.py:220-225).  It is pinned against the
 * reference itself by tests/golden/ (fixtures produced by importing the
 * reference's Python in the build container, plus the reference's stored
 * golden vector tests/test_data/known_result_4096_4097_2to32m19.npy).
 *
 * Finite fields: row_reduce(A, pivoting=1, scaling=False, threshold=0,
 * prime=p).  The reference computes over numpy int64 (exact for p < 2^31.5);
 * this restatement is exact for every p < 2^64 by using 128-bit products, so it
 * also serves the 2^61-1 cases where the reference's int64 path overflows.
 * The RREF over a field is unique, so the pivot choice (largest residue, as in
 * row_reduce.py:45-47) does not change the result.
 *
 * Reals / complex: row_reduce(A, pivoting=1, scaling=True, threshold=1e-9)
 * in double / double complex, operation for operation (row_reduce.py:32-34,
 * 45-47, 60-70); compiled with -ffp-contract=off so that no FMA changes the
 * rounding relative to numpy.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <complex.h>

typedef unsigned __int128 u128;
typedef __int128 i128;

/* ------------------------------------------------------------------ */
/* modular arithmetic                                                  */
/* ------------------------------------------------------------------ */

/* Barrett constant for p < 2^32: mu = floor((2^64-1)/p). */
typedef struct { uint64_t p; uint64_t mu; int small; } modp_t;

static modp_t modp_make(uint64_t p) {
    modp_t r; r.p = p; r.small = (p < (1ull << 32)); r.mu = r.small ? (~0ull) / p : 0; return r;
}

/* x mod p for x < 2^64 (small p) */
static inline uint64_t modp_red64(const modp_t *M, uint64_t x) {
    uint64_t q = (uint64_t)(((u128)x * M->mu) >> 64);
    uint64_t r = x - q * M->p;
    while (r >= M->p) r -= M->p;
    return r;
}

static inline uint64_t modp_mul(const modp_t *M, uint64_t a, uint64_t b) {
    if (M->small) return modp_red64(M, a * b);
    return (uint64_t)(((u128)a * b) % M->p);
}

static inline uint64_t modp_sub(const modp_t *M, uint64_t a, uint64_t b) {
    return a >= b ? a - b : a + (M->p - b);
}

/* Extended Euclid (the textbook algorithm behind
 * pyadic.finite_field.extended_euclidean_algorithm, used at row_reduce.py:62):
 * returns s with a*s = gcd (mod p), and the gcd. */
static uint64_t ext_euclid_inverse(uint64_t a, uint64_t p, uint64_t *gcd_out) {
    i128 old_r = (i128)a, r = (i128)p;
    i128 old_s = 1, s = 0;
    while (r != 0) {
        i128 q = old_r / r;
        i128 t = old_r - q * r; old_r = r; r = t;
        t = old_s - q * s; old_s = s; s = t;
    }
    *gcd_out = (uint64_t)old_r;
    i128 v = old_s % (i128)p;
    if (v < 0) v += (i128)p;
    return (uint64_t)v;
}

/* ------------------------------------------------------------------ */
/* F_p RREF, in place, row-major A (m x n, leading dimension lda).     */
/* Returns 0 on success, -2 if an inverse does not exist (non-prime p, */
/* the reference raises ZeroDivisionError at row_reduce.py:63-64).     */
/* pivcols[0..rank) receives the pivot columns.                       */
/* ------------------------------------------------------------------ */
int oracle_rref_modp(uint64_t *A, int64_t m, int64_t n, int64_t lda, uint64_t p,
                     int64_t *pivcols, int64_t *rank_out, int nthreads) {
    if (p < 2) return -1;
    modp_t M = modp_make(p);
    /* the reference reduces every column it has passed (row_reduce.py:75-76);
       reducing the input once up front gives the same residues */
    for (int64_t r = 0; r < m; ++r)
        for (int64_t c = 0; c < n; ++c) A[r * lda + c] %= p;
    int64_t i = 0, j = 0;
    uint64_t *tmp = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(n > 0 ? n : 1));
    if (!tmp) return -3;
    while (i < m && j < n) {
        /* partial pivoting: first row with the largest residue (row_reduce.py:45-47) */
        int64_t prow = i; uint64_t best = A[i * lda + j];
        for (int64_t r = i + 1; r < m; ++r) {
            uint64_t v = A[r * lda + j];
            if (v > best) { best = v; prow = r; }
        }
        if (prow != i) {
            memcpy(tmp, A + i * lda, sizeof(uint64_t) * (size_t)n);
            memcpy(A + i * lda, A + prow * lda, sizeof(uint64_t) * (size_t)n);
            memcpy(A + prow * lda, tmp, sizeof(uint64_t) * (size_t)n);
        }
        if (A[i * lda + j] != 0) {
            uint64_t g;
            uint64_t s = ext_euclid_inverse(A[i * lda + j], p, &g);
            if (g != 1) { free(tmp); return -2; }
            uint64_t *pr = A + i * lda;
            for (int64_t c = j; c < n; ++c) pr[c] = modp_mul(&M, pr[c], s);
            /* eliminate below and above (row_reduce.py:68-70) */
            #pragma omp parallel for schedule(static) num_threads(nthreads) if(nthreads > 1 && (m - 1) * (n - j) > 65536)
            for (int64_t r = 0; r < m; ++r) {
                if (r == i) continue;
                uint64_t *rr = A + r * lda;
                uint64_t f = rr[j];
                if (f == 0) continue;
                for (int64_t c = j; c < n; ++c) rr[c] = modp_sub(&M, rr[c], modp_mul(&M, f, pr[c]));
            }
            if (pivcols) pivcols[i] = j;
            ++i; ++j;
        } else {
            ++j;
        }
    }
    free(tmp);
    if (rank_out) *rank_out = i;
    return 0;
}

/* Same algorithm, stopping after `max_pivots` pivot steps; used to time a
 * bounded sample of a large elimination.  Returns the number of pivots done. */
int64_t oracle_rref_modp_partial(uint64_t *A, int64_t m, int64_t n, int64_t lda, uint64_t p,
                                 int64_t max_pivots, int nthreads) {
    modp_t M = modp_make(p);
    int64_t i = 0, j = 0;
    uint64_t *tmp = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(n > 0 ? n : 1));
    if (!tmp) return -3;
    while (i < m && j < n && i < max_pivots) {
        int64_t prow = i; uint64_t best = A[i * lda + j];
        for (int64_t r = i + 1; r < m; ++r) { uint64_t v = A[r * lda + j]; if (v > best) { best = v; prow = r; } }
        if (prow != i) {
            memcpy(tmp, A + i * lda, sizeof(uint64_t) * (size_t)n);
            memcpy(A + i * lda, A + prow * lda, sizeof(uint64_t) * (size_t)n);
            memcpy(A + prow * lda, tmp, sizeof(uint64_t) * (size_t)n);
        }
        if (A[i * lda + j] != 0) {
            uint64_t g; uint64_t s = ext_euclid_inverse(A[i * lda + j], p, &g);
            if (g != 1) { free(tmp); return -2; }
            uint64_t *pr = A + i * lda;
            for (int64_t c = j; c < n; ++c) pr[c] = modp_mul(&M, pr[c], s);
            #pragma omp parallel for schedule(static) num_threads(nthreads) if(nthreads > 1)
            for (int64_t r = 0; r < m; ++r) {
                if (r == i) continue;
                uint64_t *rr = A + r * lda; uint64_t f = rr[j];
                if (f == 0) continue;
                for (int64_t c = j; c < n; ++c) rr[c] = modp_sub(&M, rr[c], modp_mul(&M, f, pr[c]));
            }
            ++i; ++j;
        } else ++j;
    }
    free(tmp);
    return i;
}

/* ------------------------------------------------------------------ */
/* Real RREF: row_reduce(A, pivoting=1, scaling=True, threshold=thr)   */
/* ------------------------------------------------------------------ */
int oracle_rref_f64(double *A, int64_t m, int64_t n, int64_t lda, double threshold, int scaling,
                    int64_t *pivcols, int64_t *rank_out) {
    if (scaling) { /* row_reduce.py:32-34: divide each row by max |a| */
        for (int64_t r = 0; r < m; ++r) {
            double s = 0.0;
            for (int64_t c = 0; c < n; ++c) { double v = fabs(A[r * lda + c]); if (v > s) s = v; }
            for (int64_t c = 0; c < n; ++c) A[r * lda + c] = A[r * lda + c] / s;
        }
    }
    double *tmp = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    double *prow_copy = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    int64_t i = 0, j = 0;
    while (i < m && j < n) {
        int64_t prow = i; double best = fabs(A[i * lda + j]);
        for (int64_t r = i + 1; r < m; ++r) { double v = fabs(A[r * lda + j]); if (v > best) { best = v; prow = r; } }
        if (prow != i) {
            memcpy(tmp, A + i * lda, sizeof(double) * (size_t)n);
            memcpy(A + i * lda, A + prow * lda, sizeof(double) * (size_t)n);
            memcpy(A + prow * lda, tmp, sizeof(double) * (size_t)n);
        }
        if (fabs(A[i * lda + j]) > threshold) {
            double h = A[i * lda + j];
            double *pr = A + i * lda;
            for (int64_t c = 0; c < n; ++c) pr[c] = pr[c] / h;   /* row_reduce.py:67 */
            for (int64_t c = 0; c < n; ++c) prow_copy[c] = pr[c];
            for (int64_t r = 0; r < m; ++r) {                    /* row_reduce.py:68-70 */
                if (r == i) continue;
                double *rr = A + r * lda; double f = rr[j];
                for (int64_t c = j; c < n; ++c) rr[c] = rr[c] - f * prow_copy[c];
            }
            if (pivcols) pivcols[i] = j;
            ++i; ++j;
        } else ++j;
    }
    free(tmp); free(prow_copy);
    if (rank_out) *rank_out = i;
    return 0;
}

/* numpy's complex division (npymath: Smith's method variant used by
 * numpy's `/` for complex128) so that the oracle rounds like numpy. */
static inline double complex npy_cdiv(double complex a, double complex b) {
    double ar = creal(a), ai = cimag(a), br = creal(b), bi = cimag(b);
    double abs_br = fabs(br), abs_bi = fabs(bi);
    if (abs_br >= abs_bi) {
        if (abs_br == 0 && abs_bi == 0) {
            return CMPLX(ar / abs_br, ai / abs_bi);
        }
        double rat = bi / br;
        double scl = 1.0 / (br + bi * rat);
        return CMPLX((ar + ai * rat) * scl, (ai - ar * rat) * scl);
    } else {
        double rat = br / bi;
        double scl = 1.0 / (bi + br * rat);
        return CMPLX((ar * rat + ai) * scl, (ai * rat - ar) * scl);
    }
}

static inline double complex npy_cmul(double complex a, double complex b) {
    double ar = creal(a), ai = cimag(a), br = creal(b), bi = cimag(b);
    return CMPLX(ar * br - ai * bi, ar * bi + ai * br);
}

int oracle_rref_c128(double complex *A, int64_t m, int64_t n, int64_t lda, double threshold, int scaling,
                     int64_t *pivcols, int64_t *rank_out) {
    if (scaling) {
        for (int64_t r = 0; r < m; ++r) {
            double s = 0.0;
            for (int64_t c = 0; c < n; ++c) { double v = cabs(A[r * lda + c]); if (v > s) s = v; }
            for (int64_t c = 0; c < n; ++c) A[r * lda + c] = npy_cdiv(A[r * lda + c], CMPLX(s, 0.0));
        }
    }
    double complex *tmp = (double complex *)malloc(sizeof(double complex) * (size_t)(n > 0 ? n : 1));
    double complex *prow_copy = (double complex *)malloc(sizeof(double complex) * (size_t)(n > 0 ? n : 1));
    int64_t i = 0, j = 0;
    while (i < m && j < n) {
        int64_t prow = i; double best = cabs(A[i * lda + j]);
        for (int64_t r = i + 1; r < m; ++r) { double v = cabs(A[r * lda + j]); if (v > best) { best = v; prow = r; } }
        if (prow != i) {
            memcpy(tmp, A + i * lda, sizeof(double complex) * (size_t)n);
            memcpy(A + i * lda, A + prow * lda, sizeof(double complex) * (size_t)n);
            memcpy(A + prow * lda, tmp, sizeof(double complex) * (size_t)n);
        }
        if (cabs(A[i * lda + j]) > threshold) {
            double complex h = A[i * lda + j];
            double complex *pr = A + i * lda;
            for (int64_t c = 0; c < n; ++c) pr[c] = npy_cdiv(pr[c], h);
            for (int64_t c = 0; c < n; ++c) prow_copy[c] = pr[c];
            for (int64_t r = 0; r < m; ++r) {
                if (r == i) continue;
                double complex *rr = A + r * lda; double complex f = rr[j];
                for (int64_t c = j; c < n; ++c) rr[c] = rr[c] - npy_cmul(f, prow_copy[c]);
            }
            if (pivcols) pivcols[i] = j;
            ++i; ++j;
        } else ++j;
    }
    free(tmp); free(prow_copy);
    if (rank_out) *rank_out = i;
    return 0;
}

/* ------------------------------------------------------------------ */
/* Monomial loader (CPU branch of load_matrices,                       */
/* linac/pycuda_matrix_loader.py:221-225): out[r, c] is the left fold  */
/* of the products basis[r, lind[c, t]], reduced mod p after each      */
/* product for finite fields; a single factor is returned as is.       */
/* ------------------------------------------------------------------ */
void oracle_load_modp(const uint64_t *bases, int64_t n_rows, int64_t basis_len,
                      const uint32_t *lind, int64_t n_cols, int64_t degree,
                      uint64_t p, uint64_t *out) {
    modp_t M = modp_make(p);
    for (int64_t r = 0; r < n_rows; ++r) {
        const uint64_t *b = bases + r * basis_len;
        for (int64_t c = 0; c < n_cols; ++c) {
            const uint32_t *ix = lind + c * degree;
            uint64_t acc = b[ix[0]];
            for (int64_t t = 1; t < degree; ++t) {
                uint64_t x = b[ix[t]];
                if (M.small) acc = (uint64_t)(((u128)acc * x) % p);  /* operands may exceed p */
                else acc = (uint64_t)(((u128)acc * x) % p);
            }
            out[r * n_cols + c] = acc;
        }
    }
}

void oracle_load_f64(const double *bases, int64_t n_rows, int64_t basis_len,
                     const uint32_t *lind, int64_t n_cols, int64_t degree, double *out) {
    for (int64_t r = 0; r < n_rows; ++r)
        for (int64_t c = 0; c < n_cols; ++c) {
            const uint32_t *ix = lind + c * degree;
            double acc = bases[r * basis_len + ix[0]];
            for (int64_t t = 1; t < degree; ++t) acc = acc * bases[r * basis_len + ix[t]];
            out[r * n_cols + c] = acc;
        }
}

void oracle_load_c128(const double complex *bases, int64_t n_rows, int64_t basis_len,
                      const uint32_t *lind, int64_t n_cols, int64_t degree, double complex *out) {
    for (int64_t r = 0; r < n_rows; ++r)
        for (int64_t c = 0; c < n_cols; ++c) {
            const uint32_t *ix = lind + c * degree;
            double complex acc = bases[r * basis_len + ix[0]];
            for (int64_t t = 1; t < degree; ++t) acc = npy_cmul(acc, bases[r * basis_len + ix[t]]);
            out[r * n_cols + c] = acc;
        }
}

/* The RREF as a function of the loader's output: a product of matrices mod p,
 * used to build rank-deficient inputs B.C (exact, 128-bit accumulation). */
void oracle_matmul_modp(const uint64_t *B, const uint64_t *C, int64_t m, int64_t k, int64_t n,
                        uint64_t p, uint64_t *out, int nthreads) {
    #pragma omp parallel for schedule(static) num_threads(nthreads) if(nthreads > 1)
    for (int64_t r = 0; r < m; ++r) {
        for (int64_t c = 0; c < n; ++c) out[r * n + c] = 0;
        for (int64_t t = 0; t < k; ++t) {
            uint64_t b = B[r * k + t] % p;
            if (!b) continue;
            for (int64_t c = 0; c < n; ++c)
                out[r * n + c] = (uint64_t)(((u128)b * (C[t * n + c] % p) + out[r * n + c]) % p);
        }
    }
}

/* ------------------------------------------------------------------ */
/* Reference solutions of float systems (tests only)                   */
/* ------------------------------------------------------------------ */
/* out = B - A X (A m x k, X k x q, B and out m x q; row-major, real or
 * complex as interleaved pairs) with every product split exactly by fma
 * (Dekker/Kahan TwoProduct) and every sum carried in double-double (Knuth's
 * TwoSum), rounded once at the end.  Iterating X += A^-1 (B - A X) with this
 * residual converges to the exact solution of the stored system to FP64
 * accuracy (Wilkinson's refinement with an extended-precision residual);
 * the tests compare the mixed-precision GPU result against that solution.
 * The explicit fma calls are unaffected by -ffp-contract=off. */
static inline void two_sum(double a, double b, double *s, double *e) {
    double x = a + b, bv = x - a;
    *e = (a - (x - bv)) + (b - bv);
    *s = x;
}

static inline void dd_acc(double *hi, double *lo, double p, double pe) {
    double s, e;
    two_sum(*hi, p, &s, &e);
    *hi = s;
    *lo += e + pe;
}

void oracle_residual_f64(const double *A, const double *X, const double *B, int64_t m, int64_t k, int64_t q,
                         double *out, int nthreads) {
    #pragma omp parallel for schedule(static) num_threads(nthreads) if(nthreads > 1)
    for (int64_t r = 0; r < m; ++r) {
        double *hi = (double *)malloc(sizeof(double) * (size_t)(2 * q));
        double *lo = hi + q;
        for (int64_t c = 0; c < q; ++c) { hi[c] = B[r * q + c]; lo[c] = 0.0; }
        for (int64_t t = 0; t < k; ++t) {
            const double a = -A[r * k + t];
            if (a == 0.0) continue;
            for (int64_t c = 0; c < q; ++c) {
                const double x = X[t * q + c], p = a * x;
                dd_acc(&hi[c], &lo[c], p, fma(a, x, -p));
            }
        }
        for (int64_t c = 0; c < q; ++c) out[r * q + c] = hi[c] + lo[c];
        free(hi);
    }
}

void oracle_residual_c128(const double *A, const double *X, const double *B, int64_t m, int64_t k, int64_t q,
                          double *out, int nthreads) {
    #pragma omp parallel for schedule(static) num_threads(nthreads) if(nthreads > 1)
    for (int64_t r = 0; r < m; ++r) {
        double *acc = (double *)malloc(sizeof(double) * (size_t)(4 * q));  /* re hi, re lo, im hi, im lo */
        for (int64_t c = 0; c < q; ++c) {
            acc[4 * c] = B[2 * (r * q + c)]; acc[4 * c + 1] = 0.0;
            acc[4 * c + 2] = B[2 * (r * q + c) + 1]; acc[4 * c + 3] = 0.0;
        }
        for (int64_t t = 0; t < k; ++t) {
            const double ar = -A[2 * (r * k + t)], ai = -A[2 * (r * k + t) + 1];
            if (ar == 0.0 && ai == 0.0) continue;
            for (int64_t c = 0; c < q; ++c) {
                const double xr = X[2 * (t * q + c)], xi = X[2 * (t * q + c) + 1];
                double p;
                p = ar * xr; dd_acc(&acc[4 * c], &acc[4 * c + 1], p, fma(ar, xr, -p));
                p = -(ai * xi); dd_acc(&acc[4 * c], &acc[4 * c + 1], p, fma(-ai, xi, -p));
                p = ar * xi; dd_acc(&acc[4 * c + 2], &acc[4 * c + 3], p, fma(ar, xi, -p));
                p = ai * xr; dd_acc(&acc[4 * c + 2], &acc[4 * c + 3], p, fma(ai, xr, -p));
            }
        }
        for (int64_t c = 0; c < q; ++c) {
            out[2 * (r * q + c)] = acc[4 * c] + acc[4 * c + 1];
            out[2 * (r * q + c) + 1] = acc[4 * c + 2] + acc[4 * c + 3];
        }
        free(acc);
    }
}
