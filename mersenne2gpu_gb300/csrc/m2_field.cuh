// m2_field.cuh -- device arithmetic of the squaring chain.
//
// Dual-field element: GF(P61^2) (a + b i, P61 = 2^61-1) and GF(P31^2)
// (c + d i, P31 = 2^31-1).  Both primes are 3 mod 4, so i = sqrt(-1) spans the
// quadratic extension, and 2 has order 61 (resp. 31), so the IBDWT weights
// 2^(k/n) are powers of two and weighting is a bit rotation.
//
// Value convention: a GF(P61) coordinate is any representative in
// [0, 2^61 + 7] (a 64-bit word at most 8 above P61: one fold of any sum or
// product lands there, so no helper spends a second fold); a GF(P31)
// coordinate is in [0, P31].  Twiddles are stored canonical ([0, P61]).
// Helpers accept and return these ranges unless stated otherwise; rotl61 and
// the CRT need [0, P61] and get it from full61 / fold61.
//
// Built twice: with M2_DUAL = 1 (the default, namespace m2d) for both fields,
// and with M2_DUAL = 0 (namespace m2d61) for the GF(P61^2)-only layout, where
// every GF(P31^2) coordinate is the constant 0: loads, stores, shuffles and
// products of that half compile away (kDual).
#pragma once
#include <cstdint>

#ifndef M2_DUAL
#define M2_DUAL 1
#endif
#if M2_DUAL
#define M2D_NS m2d
#else
#define M2D_NS m2d61
#endif

namespace M2D_NS {

// false in the GF(P61^2)-only build: the GF(P31^2) half is not computed
constexpr bool kDual = M2_DUAL != 0;
// a GF(P31^2) coordinate as the build carries it
__device__ __forceinline__ unsigned int g31(unsigned int v) { return kDual ? v : 0u; }

typedef unsigned long long u64;
typedef unsigned int u32;
typedef long long i64;
typedef unsigned __int128 u128;
typedef __int128 i128;

constexpr u64 P61 = (1ull << 61) - 1;
constexpr u32 P31 = (1u << 31) - 1;

struct E { u64 a, b; u32 c, d; };   // 24-byte dual element

// ---------------- GF(P61) ----------------
// 2 P61 and 4 P61: subtrahend offsets (multiples of P61 above every operand)
constexpr u64 K2_61 = 2 * P61;
constexpr u64 K4_61 = 4 * P61;
// fold: any t < 2^64 -> [0, 2^61 + 7]; t <= 2^61 + 7 -> [0, P61]
__device__ __forceinline__ u64 fold61(u64 t) { return (t & P61) + (t >> 61); }
__device__ __forceinline__ u64 add61(u64 a, u64 b) { return fold61(a + b); }
__device__ __forceinline__ u64 sub61(u64 a, u64 b) { return fold61(a + (K2_61 - b)); }
// [0, 2^61 + 7] -> [0, P61 - 1]: the unique canonical representative
__device__ __forceinline__ u64 full61(u64 x) { x = fold61(x); return x == P61 ? 0 : x; }

// reduce a 128-bit value x < 2^124 (hi, lo): x >> 61 < 2^63, so the first sum
// stays below 2^64, and one fold leaves at most P61 + 5
__device__ __forceinline__ u64 red61(u64 lo, u64 hi) {
    const u64 s = (lo & P61) + ((hi << 3) | (lo >> 61));
    return fold61(s);
}
__device__ __forceinline__ u64 mul61(u64 a, u64 b) {
    const u64 lo = a * b, hi = __umul64hi(a, b);
    return red61(lo, hi);
}
// x * 2^s for x in [0, P61] (not the full range), s in [0, 60]: a rotation of
// the 61-bit word
__device__ __forceinline__ u64 rotl61(u64 x, u32 s) {
    return ((x << s) & P61) | (x >> (61u - s));
}

// ---------------- GF(P31) ----------------
__device__ __forceinline__ u32 fold31(u32 t) { return (t & P31) + (t >> 31); }
// a + b and a - b for a, b in [0, P31]: the unsigned minimum of the sum and the
// sum less P31 (the difference and the difference plus P31) is the reduced
// value -- the wrong candidate has wrapped around to a larger number
__device__ __forceinline__ u32 add31(u32 a, u32 b) { const u32 s = a + b; return min(s, s - P31); }
__device__ __forceinline__ u32 sub31(u32 a, u32 b) { const u32 s = a - b; return min(s, s + P31); }
// reduce x < 2^64 to [0, P31]
__device__ __forceinline__ u32 red31(u64 x) {
    u64 r = (x & P31) + (x >> 31);             // < 2^34
    u32 s = (u32)((r & P31) + (r >> 31));      // <= P31 + 7
    return min(s, s - P31);
}
__device__ __forceinline__ u32 rotl31(u32 x, u32 s) {
    return ((x << s) & P31) | (x >> (31u - s));
}

// ---------------- complex products ----------------
// (a0 + a1 i)(b0 + b1 i) in GF(P61^2) with three 64x64->128-bit products
// (Karatsuba): p0 = a0 b0, p1 = a1 b1, k = (a0 + a1)(b0 + b1); the real part
// is p0 - p1, taken as p0 + (C - p1) with C = P61 2^62 above every p1, the
// imaginary part k - p0 - p1 = a0 b1 + a1 b0 is exact.  The integer pipe runs
// each 128-bit product as four wide multiplies on the multiply-add pipe, the
// busier of the two; the extra 128-bit additions go to the ALU pipe.  With
// a in [0, 2^61 + 7] and b in [0, P61] both results stay below 2^124, the bound
// of red61.
__device__ __forceinline__ u128 mul128(u64 a, u64 b) { return (u128)a * b; }
constexpr u128 KM61 = (u128)P61 << 62;
__device__ __forceinline__ void cmul61(u64 a0, u64 a1, u64 b0, u64 b1, u64& r0, u64& r1) {
    const u128 p0 = mul128(a0, b0), p1 = mul128(a1, b1), k = mul128(a0 + a1, b0 + b1);
    const u128 re = p0 + (KM61 - p1);
    const u128 im = k - p0 - p1;
    r0 = red61((u64)re, (u64)(re >> 64));
    r1 = red61((u64)im, (u64)(im >> 64));
}
// (a0 + a1 i) * conj(b0 + b1 i): the real part p0 + p1; the imaginary part
// a1 b0 - a0 b1 as (a0 + a1)(b0 + P61 - b1) - p0 + p1, which adds the
// multiple (a0 + a1) P61 and so is never negative, and stays below 2^124
__device__ __forceinline__ void cmulconj61(u64 a0, u64 a1, u64 b0, u64 b1, u64& r0, u64& r1) {
    const u128 p0 = mul128(a0, b0), p1 = mul128(a1, b1), k = mul128(a0 + a1, b0 + (P61 - b1));
    const u128 re = p0 + p1;
    const u128 im = k - p0 + p1;
    r0 = red61((u64)re, (u64)(re >> 64));
    r1 = red61((u64)im, (u64)(im >> 64));
}
__device__ __forceinline__ void csqr61(u64 a0, u64 a1, u64& r0, u64& r1) {
    const u128 re = (u128)a0 * a0 + (u128)a1 * (K2_61 - a1);
    const u128 im = ((u128)a0 * a1) << 1;
    r0 = red61((u64)re, (u64)(re >> 64));
    r1 = red61((u64)im, (u64)(im >> 64));
}
// GF(P31^2): the real part a0 b0 - a1 b1 as a0 b0 + a1 (P31 - b1), a chain of
// two 32x32->64 multiply-adds below 2^63
__device__ __forceinline__ void cmul31(u32 a0, u32 a1, u32 b0, u32 b1, u32& r0, u32& r1) {
    r0 = red31((u64)a0 * b0 + (u64)a1 * (P31 - b1));
    r1 = red31((u64)a0 * b1 + (u64)a1 * b0);
}
__device__ __forceinline__ void cmulconj31(u32 a0, u32 a1, u32 b0, u32 b1, u32& r0, u32& r1) {
    r0 = red31((u64)a0 * b0 + (u64)a1 * b1);
    r1 = red31((u64)a1 * b0 + (u64)a0 * (P31 - b1));
}
__device__ __forceinline__ void csqr31(u32 a0, u32 a1, u32& r0, u32& r1) {
    r0 = red31((u64)a0 * a0 + (u64)a1 * (P31 - a1));
    r1 = red31(((u64)a0 * a1) << 1);
}

// ---------------- dual element ops ----------------
__device__ __forceinline__ E eadd(const E& x, const E& y) { return E{add61(x.a, y.a), add61(x.b, y.b), add31(x.c, y.c), add31(x.d, y.d)}; }
__device__ __forceinline__ E esub(const E& x, const E& y) { return E{sub61(x.a, y.a), sub61(x.b, y.b), sub31(x.c, y.c), sub31(x.d, y.d)}; }
// x + i y, x - i y
__device__ __forceinline__ E eaddi(const E& x, const E& y) { return E{sub61(x.a, y.b), add61(x.b, y.a), sub31(x.c, y.d), add31(x.d, y.c)}; }
__device__ __forceinline__ E esubi(const E& x, const E& y) { return E{add61(x.a, y.b), sub61(x.b, y.a), add31(x.c, y.d), sub31(x.d, y.c)}; }
// x + conj(y), x - conj(y), conj(x - y)
__device__ __forceinline__ E eaddconj(const E& x, const E& y) { return E{add61(x.a, y.a), sub61(x.b, y.b), add31(x.c, y.c), sub31(x.d, y.d)}; }
__device__ __forceinline__ E esubconj(const E& x, const E& y) { return E{sub61(x.a, y.a), add61(x.b, y.b), sub31(x.c, y.c), add31(x.d, y.d)}; }
__device__ __forceinline__ E econjsub(const E& x, const E& y) { return E{sub61(x.a, y.a), sub61(y.b, x.b), sub31(x.c, y.c), sub31(y.d, x.d)}; }
__device__ __forceinline__ E emul(const E& x, const E& w) {
    E r;
    cmul61(x.a, x.b, w.a, w.b, r.a, r.b);
    if (kDual) cmul31(x.c, x.d, w.c, w.d, r.c, r.d);
    else r.c = r.d = 0;
    return r;
}
__device__ __forceinline__ E emulconj(const E& x, const E& w) {
    E r;
    cmulconj61(x.a, x.b, w.a, w.b, r.a, r.b);
    if (kDual) cmulconj31(x.c, x.d, w.c, w.d, r.c, r.d);
    else r.c = r.d = 0;
    return r;
}
__device__ __forceinline__ E esqr(const E& x) {
    E r;
    csqr61(x.a, x.b, r.a, r.b);
    if (kDual) csqr31(x.c, x.d, r.c, r.d);
    else r.c = r.d = 0;
    return r;
}

// ---------------- butterflies ----------------
// Forward radix-4 step of the per-block-twiddle transform: the block holds a
// polynomial mod X^(4m) - c; with r^4 = c the outputs are its residues mod
// X^m - r, X^m + r, X^m - i r, X^m + i r (bit-reversed order of the roots).
//
// The GF(P61) half folds once per output, not once per add: the first layer's
// sums and differences stay unfolded (below 3 2^61 + 8, differences offset by
// 2 P61), the second layer offsets its differences by 4 P61 (sums below
// 7 2^61 + 8 < 2^64) and folds.  The GF(P31) half folds every step (32-bit).
struct L61 { u64 a, b; };   // unfolded GF(P61^2) intermediate
__device__ __forceinline__ L61 ladd(u64 xa, u64 xb, u64 ya, u64 yb) { return L61{xa + ya, xb + yb}; }
__device__ __forceinline__ L61 lsub(u64 xa, u64 xb, u64 ya, u64 yb) { return L61{xa + (K2_61 - ya), xb + (K2_61 - yb)}; }
__device__ __forceinline__ u64 fadd(u64 x, u64 y) { return fold61(x + y); }
__device__ __forceinline__ u64 fsub(u64 x, u64 y) { return fold61(x + (K4_61 - y)); }

__device__ __forceinline__ void dif4(E& x0, E& x1, E& x2, E& x3, const E& r1, const E& r2, const E& r3) {
    const E u1 = emul(x1, r1), u2 = emul(x2, r2), u3 = emul(x3, r3);
    const L61 v0 = ladd(x0.a, x0.b, u2.a, u2.b), v1 = ladd(u1.a, u1.b, u3.a, u3.b);
    const L61 v2 = lsub(x0.a, x0.b, u2.a, u2.b), v3 = lsub(u1.a, u1.b, u3.a, u3.b);
    const u32 c0 = add31(x0.c, u2.c), d0 = add31(x0.d, u2.d), c1 = add31(u1.c, u3.c), d1 = add31(u1.d, u3.d);
    const u32 c2 = sub31(x0.c, u2.c), d2 = sub31(x0.d, u2.d), c3 = sub31(u1.c, u3.c), d3 = sub31(u1.d, u3.d);
    x0 = E{fadd(v0.a, v1.a), fadd(v0.b, v1.b), add31(c0, c1), add31(d0, d1)};
    x1 = E{fsub(v0.a, v1.a), fsub(v0.b, v1.b), sub31(c0, c1), sub31(d0, d1)};
    x2 = E{fsub(v2.a, v3.b), fadd(v2.b, v3.a), sub31(c2, d3), add31(d2, c3)};   // v2 + i v3
    x3 = E{fadd(v2.a, v3.b), fsub(v2.b, v3.a), add31(c2, d3), sub31(d2, c3)};   // v2 - i v3
}
// Exact inverse of dif4 up to the factor 4.
__device__ __forceinline__ void dit4(E& x0, E& x1, E& x2, E& x3, const E& r1, const E& r2, const E& r3) {
    const L61 v0 = ladd(x0.a, x0.b, x1.a, x1.b), v1 = lsub(x0.a, x0.b, x1.a, x1.b);
    const L61 v2 = ladd(x2.a, x2.b, x3.a, x3.b), v3 = lsub(x3.a, x3.b, x2.a, x2.b);
    const u32 c0 = add31(x0.c, x1.c), d0 = add31(x0.d, x1.d), c1 = sub31(x0.c, x1.c), d1 = sub31(x0.d, x1.d);
    const u32 c2 = add31(x2.c, x3.c), d2 = add31(x2.d, x3.d), c3 = sub31(x3.c, x2.c), d3 = sub31(x3.d, x2.d);
    const E y0 = E{fadd(v0.a, v2.a), fadd(v0.b, v2.b), add31(c0, c2), add31(d0, d2)};
    const E s2 = E{fsub(v0.a, v2.a), fsub(v0.b, v2.b), sub31(c0, c2), sub31(d0, d2)};
    const E s1 = E{fsub(v1.a, v3.b), fadd(v1.b, v3.a), sub31(c1, d3), add31(d1, c3)};   // v1 + i v3
    const E s3 = E{fadd(v1.a, v3.b), fsub(v1.b, v3.a), add31(c1, d3), sub31(d1, c3)};   // v1 - i v3
    x0 = y0;
    x1 = emulconj(s1, r1);
    x2 = emulconj(s2, r2);
    x3 = emulconj(s3, r3);
}
// dif4 / dit4 of the transform's first level (one block, root 1): no products
__device__ __forceinline__ void dif4_1(E& x0, E& x1, E& x2, E& x3) {
    const L61 v0 = ladd(x0.a, x0.b, x2.a, x2.b), v1 = ladd(x1.a, x1.b, x3.a, x3.b);
    const L61 v2 = lsub(x0.a, x0.b, x2.a, x2.b), v3 = lsub(x1.a, x1.b, x3.a, x3.b);
    const u32 c0 = add31(x0.c, x2.c), d0 = add31(x0.d, x2.d), c1 = add31(x1.c, x3.c), d1 = add31(x1.d, x3.d);
    const u32 c2 = sub31(x0.c, x2.c), d2 = sub31(x0.d, x2.d), c3 = sub31(x1.c, x3.c), d3 = sub31(x1.d, x3.d);
    x0 = E{fadd(v0.a, v1.a), fadd(v0.b, v1.b), add31(c0, c1), add31(d0, d1)};
    x1 = E{fsub(v0.a, v1.a), fsub(v0.b, v1.b), sub31(c0, c1), sub31(d0, d1)};
    x2 = E{fsub(v2.a, v3.b), fadd(v2.b, v3.a), sub31(c2, d3), add31(d2, c3)};
    x3 = E{fadd(v2.a, v3.b), fsub(v2.b, v3.a), add31(c2, d3), sub31(d2, c3)};
}
__device__ __forceinline__ void dit4_1(E& x0, E& x1, E& x2, E& x3) {
    const L61 v0 = ladd(x0.a, x0.b, x1.a, x1.b), v1 = lsub(x0.a, x0.b, x1.a, x1.b);
    const L61 v2 = ladd(x2.a, x2.b, x3.a, x3.b), v3 = lsub(x3.a, x3.b, x2.a, x2.b);
    const u32 c0 = add31(x0.c, x1.c), d0 = add31(x0.d, x1.d), c1 = sub31(x0.c, x1.c), d1 = sub31(x0.d, x1.d);
    const u32 c2 = add31(x2.c, x3.c), d2 = add31(x2.d, x3.d), c3 = sub31(x3.c, x2.c), d3 = sub31(x3.d, x2.d);
    const E y0 = E{fadd(v0.a, v2.a), fadd(v0.b, v2.b), add31(c0, c2), add31(d0, d2)};
    const E y2 = E{fsub(v0.a, v2.a), fsub(v0.b, v2.b), sub31(c0, c2), sub31(d0, d2)};
    const E y1 = E{fsub(v1.a, v3.b), fadd(v1.b, v3.a), sub31(c1, d3), add31(d1, c3)};
    const E y3 = E{fadd(v1.a, v3.b), fsub(v1.b, v3.a), add31(c1, d3), sub31(d1, c3)};
    x0 = y0; x1 = y1; x2 = y2; x3 = y3;
}
__device__ __forceinline__ void dif2(E& x0, E& x1, const E& r) {
    const E u1 = emul(x1, r);
    const E y0 = eadd(x0, u1), y1 = esub(x0, u1);
    x0 = y0; x1 = y1;
}
__device__ __forceinline__ void dit2(E& x0, E& x1, const E& r) {
    const E y0 = eadd(x0, x1), y1 = emulconj(esub(x0, x1), r);
    x0 = y0; x1 = y1;
}

// Centre of the real-packed squaring for an (even position k, mirror mk) pair
// with root zeta at k: Z(k) holds E + iO, conj(Z(mk)) holds E - iO; the square
// of the real sequence is E^2 + zeta O^2 (even part) and 2 E O (odd part),
// scaled by 4 here.
__device__ __forceinline__ void centre_pair(E& zk, E& zmk, const E& zeta) {
    const E u0 = eaddconj(zk, zmk), u1 = esubconj(zk, zmk);
    const E v0 = esub(esqr(u0), emul(esqr(u1), zeta));
    const E v1 = emul(u0, eadd(u1, u1));
    zk = eadd(v0, v1);
    zmk = econjsub(v0, v1);
}
// Positions 0 (root 1) and 1 (root -1) are their own mirrors.
__device__ __forceinline__ void centre_zero(E& z0, E& z1) {
    const E u0 = eaddconj(z0, z0), u1 = esubconj(z0, z0);
    const E v0 = esub(esqr(u0), esqr(u1));
    const E v1 = emul(u0, eadd(u1, u1));
    z0 = eadd(v0, v1);
    const E t = eadd(z1, z1);
    z1 = esqr(t);
}

// ---------------- lane exchanges ----------------
// dual element from lane (this lane ^ m); every lane of the warp takes part
__device__ __forceinline__ E shfl_xor_e(const E& v, int m) {
    E r;
    r.a = __shfl_xor_sync(0xffffffffu, v.a, m);
    r.b = __shfl_xor_sync(0xffffffffu, v.b, m);
    r.c = kDual ? __shfl_xor_sync(0xffffffffu, v.c, m) : 0u;
    r.d = kDual ? __shfl_xor_sync(0xffffffffu, v.d, m) : 0u;
    return r;
}

// ---------------- digits <-> field ----------------
__device__ __forceinline__ u64 digit_to61(i64 d) { return d >= 0 ? (u64)d : P61 - (u64)(-d); }
// d + P31 2^32 (a multiple of P31, 2^63 - 2^32) is a non-negative 64-bit
// value for every digit and pending carry (|d| < 2^62), so one reduction
// gives d mod P31 without the sign branches
__device__ __forceinline__ u32 digit_to31(i64 d) { return red31((u64)d + ((u64)P31 << 32)); }
__device__ __forceinline__ u64 canon61(u64 x) { return x == P61 ? 0 : x; }
__device__ __forceinline__ u32 canon31(u32 x) { return x == P31 ? 0 : x; }

// Garner: the signed value z with z == r61 (mod P61), z == r31 (mod P31),
// |z| < P61 P31 / 2.
__device__ __forceinline__ i128 crt_signed(u64 r61, u32 r31) {
    r61 = full61(r61); r31 = canon31(r31);
    u64 u = full61(sub61(r61, (u64)r31));
    u = add61(u, rotl61(u, 31));                          // u (2^31 + 1) == u / P31 (mod P61)
    u = full61(u);
    const u128 L = ((u128)u << 31) - u + r31;             // u P31 + r31 < P61 P31
    const u128 M = (u128)P61 * P31;
    return (L > (M >> 1)) ? (i128)L - (i128)M : (i128)L;
}

// width of digit j, ceil(p (j+1) / n) - ceil(p j / n) with n = 2^ln: for
// j >= 1 it is q + [((p j - 1) mod n) + (p mod n) >= n], the remainder taken
// in 32-bit arithmetic (its low ln bits are exact); digit 0 has q + [p mod n != 0]
__device__ __forceinline__ u32 width_of(u32 p, int ln, u64 j) {
    const u32 nm = (1u << ln) - 1u, pm = p & nm, q = p >> ln;
    if (j == 0) return q + (pm != 0u);
    const u32 r = ((u32)j * pm - 1u) & nm;
    return q + ((r + pm) >> ln);
}
// One digit of the carry: z = the signed convolution word with z == r61
// (mod P61), z == r31 (mod P31), |z| < P61 P31 / 2 (Garner), then
// t = mul z + c + 2^(w-1), digit = (t mod 2^w) - 2^(w-1), carry out t >> w.
// The carry out is below 2^62 in magnitude for every exponent of the table,
// so it is formed from the 128-bit t by a 64-bit funnel shift.  1 <= w <= 63.
__device__ __forceinline__ i64 crt_digit(u64 r61, u32 r31, u32 w, u32 mul, i64 sub, i64& c, u32& bad, bool gf61) {
    // r61 in [0, P61], r31 in [0, P31]: either may be the non-canonical zero
    u64 lo, hi;
    if (gf61) {
        // GF(P61^2)-only layout: the word is the residue in (-P61/2, P61/2]
        r61 = (r61 == P61) ? 0 : r61;
        const bool neg = r61 > (P61 >> 1);
        lo = neg ? r61 - P61 : r61;
        hi = neg ? ~0ull : 0ull;
    } else {
    u64 u = fold61(r61 + (P61 - r31));             // (r61 - r31) mod P61 in [0, P61] (the sum is below 2 P61)
    u = fold61(u + (((u << 31) & P61) | (u >> 30)));   // u (2^31 + 1) mod P61 in [0, P61]: + u 2^31, a 61-bit rotation
    // L = u P31 + r31 = u 2^31 - u + r31 <= P61 P31 + P31: a value of L at or
    // above M = P61 P31 leaves L - M in [0, P31] below, the same word
    lo = u << 31; hi = u >> 33;
    const u64 lo2 = lo - u;
    hi -= (lo2 > lo);
    lo = lo2 + r31;
    hi += (lo < lo2);
    // signed: z = L - M when L > M/2 (M = P61 P31 = 2^92 - 2^61 - 2^31 + 1)
    constexpr u64 MLO = 0xdfffffff80000001ull, MHI = 0x000000000fffffffull;   // M
    constexpr u64 HLO = 0xefffffffc0000000ull, HHI = 0x0000000007ffffffull;   // (M - 1) / 2
    if (hi > HHI || (hi == HHI && lo > HLO)) {
        const u64 l2 = lo - MLO;
        hi = hi - MHI - (l2 > lo);
        lo = l2;
    }
    }
    // t = mul z + c + half  (two's complement in hi:lo)
    if (mul == 3) {
        const u64 l3 = lo * 3;
        hi = hi * 3 + __umul64hi(lo, 3);
        lo = l3;
    }
    const i64 add = c - sub + ((i64)1 << (w - 1));
    const u64 l4 = lo + (u64)add;
    hi += (l4 < lo) + (u64)(add >> 63);            // sign-extend add into the high word
    lo = l4;
    // t >> w fits in 64 bits iff the high word above bit w-1 is pure sign
    const i64 top = (i64)hi >> (w - 1);
    bad |= (u32)(top != 0 && top != -1);
    c = (i64)((hi << (64 - w)) | (lo >> w));
    return (i64)(lo & ((1ull << w) - 1)) - ((i64)1 << (w - 1));
}

// Balanced split of t at width w: t = d + c 2^w with d in [-2^(w-1), 2^(w-1)).
__device__ __forceinline__ i64 split_balanced(i128 t, u32 w, i128& c) {
    if (w == 0) { c = t; return 0; }
    const i128 half = (i128)1 << (w - 1);
    c = (t + half) >> w;
    return (i64)(t - (c << w));
}
__device__ __forceinline__ i64 split_balanced64(i64 t, u32 w, i64& c) {
    if (w == 0) { c = t; return 0; }
    const i64 half = (i64)1 << (w - 1);
    c = (t + half) >> w;
    return t - (c << w);
}

}  // namespace M2D_NS
