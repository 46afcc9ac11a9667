// Field arithmetic for the RREF kernels: F_p with 32-bit and 64-bit residues,
// the reals (double) and the complex numbers (double2).
//
// linac's kernels reduce every product with a wide `%`
// (linac/row_reduce.cu:107-114: 64-bit for uint32, 128-bit for uint64) and
// invert by Fermat (row_reduce.cu:92-105).  Here:
//   * 32-bit residues (p < 2^32): Barrett reduction of the 64-bit product with
//     mu = floor((2^64-1)/p); at most two conditional subtractions.
//   * 64-bit residues (odd p < 2^64): Montgomery multiplication with R = 2^64;
//     `mul` returns the ordinary product by a second multiplication by R^2.
//   * inverses by Fermat's little theorem (p is validated prime on the host).
// Each field exposes the same small interface, used by the templated panel,
// trailing-update and gather kernels:
//   T, Key                     element and pivot-preference key types
//   mul, sub, add, zero, one   arithmetic
//   inv(a)                     multiplicative inverse of a pivot
//   scale(x, piv, inv)         x / piv (pivot-row normalisation)
//   key(a), is_pivot(key)      partial-pivot key (largest first) and head test
//   reduce_input(a)            canonical representative of an input entry
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace lnc {

struct c128 {
    double x, y;
};

// ----------------------------------------------------------------------------
// F_p, 32-bit residues
// ----------------------------------------------------------------------------
// Multiplicative inverse of a (0 < a < p, p prime) by the binary extended
// Euclidean algorithm: invariants x1 a = u, x2 a = v (mod p); halving x mod p
// is x / 2 or (x + p) / 2 = x/2 + p/2 + 1 for odd x (no overflow for any
// p < 2^64).  About 2 log2(p) short dependent steps, several times shorter
// than Fermat's log2(p) modular squarings on the pivot's critical path.
template <class W>
__device__ __forceinline__ W inv_binary(W a, W p) {
    if (a == 1) return 1;  // also the only case for p = 2
    W u = a, v = p, x1 = 1, x2 = 0;
    const W half = (p >> 1) + 1;
    while (u != 1 && v != 1) {
        while (!(u & 1)) {
            u >>= 1;
            x1 = (x1 & 1) ? (x1 >> 1) + half : (x1 >> 1);
        }
        while (!(v & 1)) {
            v >>= 1;
            x2 = (x2 & 1) ? (x2 >> 1) + half : (x2 >> 1);
        }
        if (u >= v) {
            u -= v;
            x1 = (x1 >= x2) ? x1 - x2 : x1 + (p - x2);
        } else {
            v -= u;
            x2 = (x2 >= x1) ? x2 - x1 : x2 + (p - x1);
        }
    }
    return (u == 1) ? x1 : x2;
}

struct FieldU32 {
    using T = uint32_t;
    using Key = uint64_t;
    static constexpr int kDtype = 1;
    uint32_t p;
    uint64_t mu;  // floor((2^64 - 1) / p)

    static FieldU32 make(uint64_t prime) {
        FieldU32 f;
        f.p = (uint32_t)prime;
        f.mu = ~0ull / prime;
        return f;
    }
    __device__ __forceinline__ T reduce64(uint64_t x) const {
        uint64_t q = __umul64hi(x, mu);
        uint64_t r = x - q * (uint64_t)p;
        r = (r >= p) ? r - p : r;
        r = (r >= p) ? r - p : r;
        return (T)r;
    }
    __device__ __forceinline__ T mul(T a, T b) const { return reduce64((uint64_t)a * b); }
    __device__ __forceinline__ T add(T a, T b) const {
        uint64_t s = (uint64_t)a + b;
        return (T)(s >= p ? s - p : s);
    }
    __device__ __forceinline__ T sub(T a, T b) const { return a >= b ? a - b : a + (p - b); }
    __device__ __forceinline__ T zero() const { return 0u; }
    __device__ __forceinline__ T one() const { return 1u; }
    __device__ __forceinline__ T pow(T a, uint64_t e) const {
        T r = 1u, x = a;
        while (e) {
            if (e & 1) r = mul(r, x);
            x = mul(x, x);
            e >>= 1;
        }
        return r;
    }
    __device__ __forceinline__ T inv(T a) const { return inv_binary<uint32_t>(a, p); }
    __device__ __forceinline__ T scale(T x, T /*piv*/, T pinv) const { return mul(x, pinv); }
    __device__ __forceinline__ Key key(T a) const { return (Key)a; }
    __device__ __forceinline__ bool is_pivot(Key k) const { return k != 0; }
    __device__ __forceinline__ bool nonzero(T a) const { return a != 0; }
    __device__ __forceinline__ T reduce_input(T a) const { return a >= p ? a % p : a; }
};

// ----------------------------------------------------------------------------
// F_p, 64-bit residues (odd p), Montgomery with R = 2^64
// ----------------------------------------------------------------------------
struct FieldU64 {
    using T = uint64_t;
    using Key = uint64_t;
    static constexpr int kDtype = 2;
    uint64_t p;
    uint64_t pinv;  // -p^{-1} mod 2^64
    uint64_t r2;    // 2^128 mod p
    uint64_t r1;    // 2^64 mod p (Montgomery form of 1)

    static FieldU64 make(uint64_t prime) {
        FieldU64 f;
        f.p = prime;
        uint64_t x = prime;  // Newton iteration for p^{-1} mod 2^64 (p odd)
        for (int i = 0; i < 6; ++i) x *= 2 - prime * x;
        f.pinv = (uint64_t)0 - x;
        unsigned __int128 R = ((unsigned __int128)1 << 64) % prime;
        f.r1 = (uint64_t)R;
        f.r2 = (uint64_t)((R * R) % prime);
        return f;
    }
    // REDC of (hi:lo) < p * 2^64
    __device__ __forceinline__ T redc(uint64_t lo, uint64_t hi) const {
        uint64_t m = lo * pinv;
        uint64_t mp_hi = __umul64hi(m, p);
        uint64_t carry = (lo != 0) ? 1ull : 0ull;  // lo + m*p == 0 (mod 2^64)
        uint64_t t = hi + mp_hi;
        bool of = t < hi;
        uint64_t t2 = t + carry;
        of |= t2 < t;
        if (of || t2 >= p) t2 -= p;
        return t2;
    }
    __device__ __forceinline__ T montmul(T a, T b) const { return redc(a * b, __umul64hi(a, b)); }
    __device__ __forceinline__ T to_mont(T a) const { return montmul(a, r2); }
    __device__ __forceinline__ T from_mont(T a) const { return redc(a, 0); }
    __device__ __forceinline__ T mul(T a, T b) const { return montmul(montmul(a, b), r2); }
    __device__ __forceinline__ T add(T a, T b) const {
        uint64_t s = a + b;
        return (s < a || s >= p) ? s - p : s;
    }
    __device__ __forceinline__ T sub(T a, T b) const { return a >= b ? a - b : a + (p - b); }
    __device__ __forceinline__ T zero() const { return 0ull; }
    __device__ __forceinline__ T one() const { return 1ull; }
    __device__ __forceinline__ T inv(T a) const { return inv_binary<uint64_t>(a, p); }
    __device__ __forceinline__ T scale(T x, T /*piv*/, T pinv_) const { return mul(x, pinv_); }
    __device__ __forceinline__ Key key(T a) const { return a; }
    __device__ __forceinline__ bool is_pivot(Key k) const { return k != 0; }
    __device__ __forceinline__ bool nonzero(T a) const { return a != 0; }
    __device__ __forceinline__ T reduce_input(T a) const { return a >= p ? a % p : a; }
};

// ----------------------------------------------------------------------------
// reals: partial pivoting by |a|, head test |a| > tol (linac/row_reduce.cu:55,
// 404-418)
// ----------------------------------------------------------------------------
struct FieldF64 {
    using T = double;
    using Key = double;
    static constexpr int kDtype = 3;
    double tol;

    static FieldF64 make(double tol_) { FieldF64 f; f.tol = tol_; return f; }
    __device__ __forceinline__ T mul(T a, T b) const { return a * b; }
    __device__ __forceinline__ T add(T a, T b) const { return a + b; }
    __device__ __forceinline__ T sub(T a, T b) const { return a - b; }
    __device__ __forceinline__ T zero() const { return 0.0; }
    __device__ __forceinline__ T one() const { return 1.0; }
    __device__ __forceinline__ T inv(T a) const { return 1.0 / a; }
    __device__ __forceinline__ T scale(T x, T piv, T /*pinv*/) const { return x / piv; }
    __device__ __forceinline__ Key key(T a) const { return fabs(a); }
    __device__ __forceinline__ bool is_pivot(Key k) const { return k > tol; }
    __device__ __forceinline__ bool nonzero(T a) const { return a != 0.0; }
    __device__ __forceinline__ T reduce_input(T a) const { return a; }
};

// ----------------------------------------------------------------------------
// complex numbers
// ----------------------------------------------------------------------------
struct FieldC128 {
    using T = c128;
    using Key = double;
    static constexpr int kDtype = 4;
    double tol;

    static FieldC128 make(double tol_) { FieldC128 f; f.tol = tol_; return f; }
    __device__ __forceinline__ T mk(double x, double y) const { T r; r.x = x; r.y = y; return r; }
    __device__ __forceinline__ T mul(T a, T b) const {
        return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
    }
    __device__ __forceinline__ T add(T a, T b) const { return mk(a.x + b.x, a.y + b.y); }
    __device__ __forceinline__ T sub(T a, T b) const { return mk(a.x - b.x, a.y - b.y); }
    __device__ __forceinline__ T zero() const { return mk(0.0, 0.0); }
    __device__ __forceinline__ T one() const { return mk(1.0, 0.0); }
    // Smith's algorithm for a / b
    __device__ __forceinline__ T div(T a, T b) const {
        if (fabs(b.x) >= fabs(b.y)) {
            double rat = b.y / b.x, scl = 1.0 / (b.x + b.y * rat);
            return mk((a.x + a.y * rat) * scl, (a.y - a.x * rat) * scl);
        } else {
            double rat = b.x / b.y, scl = 1.0 / (b.y + b.x * rat);
            return mk((a.x * rat + a.y) * scl, (a.y * rat - a.x) * scl);
        }
    }
    __device__ __forceinline__ T inv(T a) const { return div(one(), a); }
    __device__ __forceinline__ T scale(T x, T piv, T /*pinv*/) const { return div(x, piv); }
    __device__ __forceinline__ Key key(T a) const { return hypot(a.x, a.y); }
    __device__ __forceinline__ bool is_pivot(Key k) const { return k > tol; }
    __device__ __forceinline__ bool nonzero(T a) const { return a.x != 0.0 || a.y != 0.0; }
    __device__ __forceinline__ T reduce_input(T a) const { return a; }
};

}  // namespace lnc
