// m2_field.cuh -- device arithmetic of the squaring chain.
//
// Dual-field element: GF(P61^2) (a + b i, P61 = 2^61-1) and GF(P31^2)
// (c + d i, P31 = 2^31-1).  Both primes are 3 mod 4, so i = sqrt(-1) spans the
// quadratic extension, and 2 has order 61 (resp. 31), so the IBDWT weights
// 2^(k/n) are powers of two and weighting is a bit rotation.
//
// Value convention: every stored coordinate is in [0, P61] (resp. [0, P31]);
// P itself is an alternative representative of 0.  All helpers accept and
// return that range.
#pragma once
#include <cstdint>

namespace m2d {

typedef unsigned long long u64;
typedef unsigned int u32;
typedef long long i64;
typedef unsigned __int128 u128;
typedef __int128 i128;

constexpr u64 P61 = (1ull << 61) - 1;
constexpr u32 P31 = (1u << 31) - 1;

struct E { u64 a, b; u32 c, d; };   // 24-byte dual element

// ---------------- GF(P61) ----------------
// fold: t <= 2 P61 + 1  ->  [0, P61]
__device__ __forceinline__ u64 fold61(u64 t) { return (t & P61) + (t >> 61); }
__device__ __forceinline__ u64 add61(u64 a, u64 b) { return fold61(a + b); }
// P61 - b == P61 ^ b for b <= P61
__device__ __forceinline__ u64 sub61(u64 a, u64 b) { return fold61(a + (P61 ^ b)); }
__device__ __forceinline__ u64 neg61(u64 b) { return P61 ^ b; }

// reduce a 128-bit value x < 2^125 (hi, lo) to [0, P61]
__device__ __forceinline__ u64 red61(u64 lo, u64 hi) {
    u64 s = (lo & P61) + ((hi << 3) | (lo >> 61));   // < 2^61 + 2^64 / 2 ... < 2^64
    s = (s & P61) + (s >> 61);                          // <= P61 + 7
    return fold61(s);
}
__device__ __forceinline__ u64 mul61(u64 a, u64 b) {
    const u64 lo = a * b, hi = __umul64hi(a, b);
    return red61(lo, hi);
}
// x * 2^s for x in [0, P61], s in [0, 60]: a rotation of the 61-bit word
__device__ __forceinline__ u64 rotl61(u64 x, u32 s) {
    return ((x << s) & P61) | (x >> (61u - s));
}

// ---------------- GF(P31) ----------------
__device__ __forceinline__ u32 fold31(u32 t) { return (t & P31) + (t >> 31); }
__device__ __forceinline__ u32 add31(u32 a, u32 b) { return fold31(a + b); }
__device__ __forceinline__ u32 sub31(u32 a, u32 b) { return fold31(a + (P31 ^ b)); }
// reduce x < 2^64 to [0, P31]
__device__ __forceinline__ u32 red31(u64 x) {
    u64 r = (x & P31) + (x >> 31);             // < 2^34
    u32 s = (u32)((r & P31) + (r >> 31));      // <= P31 + 7
    return fold31(s);
}
__device__ __forceinline__ u32 rotl31(u32 x, u32 s) {
    return ((x << s) & P31) | (x >> (31u - s));
}

// ---------------- complex products ----------------
// (a0 + a1 i)(b0 + b1 i) in GF(P61^2): the real part is accumulated as
// a0 b0 + (2^122 - 1 - a1 b1), which is a0 b0 - a1 b1 modulo P61 because
// 2^122 - 1 = (2^61 - 1)(2^61 + 1).
__device__ __forceinline__ void cmul61(u64 a0, u64 a1, u64 b0, u64 b1, u64& r0, u64& r1) {
    const u128 ac = (u128)a0 * b0, bd = (u128)a1 * b1;
    const u128 ad = (u128)a0 * b1, bc = (u128)a1 * b0;
    const u128 m122 = ((u128)1 << 122) - 1;
    const u128 re = ac + (m122 - bd);
    const u128 im = ad + bc;
    r0 = red61((u64)re, (u64)(re >> 64));
    r1 = red61((u64)im, (u64)(im >> 64));
}
// (a0 + a1 i) * conj(b0 + b1 i)
__device__ __forceinline__ void cmulconj61(u64 a0, u64 a1, u64 b0, u64 b1, u64& r0, u64& r1) {
    const u128 ac = (u128)a0 * b0, bd = (u128)a1 * b1;
    const u128 ad = (u128)a0 * b1, bc = (u128)a1 * b0;
    const u128 m122 = ((u128)1 << 122) - 1;
    const u128 re = ac + bd;
    const u128 im = bc + (m122 - ad);
    r0 = red61((u64)re, (u64)(re >> 64));
    r1 = red61((u64)im, (u64)(im >> 64));
}
__device__ __forceinline__ void csqr61(u64 a0, u64 a1, u64& r0, u64& r1) {
    const u128 aa = (u128)a0 * a0, bb = (u128)a1 * a1, ab = (u128)a0 * a1;
    const u128 m122 = ((u128)1 << 122) - 1;
    const u128 re = aa + (m122 - bb);
    const u128 im = ab << 1;
    r0 = red61((u64)re, (u64)(re >> 64));
    r1 = red61((u64)im, (u64)(im >> 64));
}
// GF(P31^2): real part a0 b0 + (2^62 - 1 - a1 b1), 2^62 - 1 = (2^31-1)(2^31+1)
__device__ __forceinline__ void cmul31(u32 a0, u32 a1, u32 b0, u32 b1, u32& r0, u32& r1) {
    const u64 m62 = (1ull << 62) - 1;
    r0 = red31((u64)a0 * b0 + (m62 - (u64)a1 * b1));
    r1 = red31((u64)a0 * b1 + (u64)a1 * b0);
}
__device__ __forceinline__ void cmulconj31(u32 a0, u32 a1, u32 b0, u32 b1, u32& r0, u32& r1) {
    const u64 m62 = (1ull << 62) - 1;
    r0 = red31((u64)a0 * b0 + (u64)a1 * b1);
    r1 = red31((u64)a1 * b0 + (m62 - (u64)a0 * b1));
}
__device__ __forceinline__ void csqr31(u32 a0, u32 a1, u32& r0, u32& r1) {
    const u64 m62 = (1ull << 62) - 1;
    r0 = red31((u64)a0 * a0 + (m62 - (u64)a1 * a1));
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
    cmul31(x.c, x.d, w.c, w.d, r.c, r.d);
    return r;
}
__device__ __forceinline__ E emulconj(const E& x, const E& w) {
    E r;
    cmulconj61(x.a, x.b, w.a, w.b, r.a, r.b);
    cmulconj31(x.c, x.d, w.c, w.d, r.c, r.d);
    return r;
}
__device__ __forceinline__ E esqr(const E& x) {
    E r;
    csqr61(x.a, x.b, r.a, r.b);
    csqr31(x.c, x.d, r.c, r.d);
    return r;
}

// ---------------- butterflies ----------------
// Forward radix-4 step of the per-block-twiddle transform: the block holds a
// polynomial mod X^(4m) - c; with r^4 = c the outputs are its residues mod
// X^m - r, X^m + r, X^m - i r, X^m + i r (bit-reversed order of the roots).
__device__ __forceinline__ void dif4(E& x0, E& x1, E& x2, E& x3, const E& r1, const E& r2, const E& r3) {
    const E u1 = emul(x1, r1), u2 = emul(x2, r2), u3 = emul(x3, r3);
    const E v0 = eadd(x0, u2), v1 = eadd(u1, u3), v2 = esub(x0, u2), v3 = esub(u1, u3);
    x0 = eadd(v0, v1); x1 = esub(v0, v1); x2 = eaddi(v2, v3); x3 = esubi(v2, v3);
}
// Exact inverse of dif4 up to the factor 4.
__device__ __forceinline__ void dit4(E& x0, E& x1, E& x2, E& x3, const E& r1, const E& r2, const E& r3) {
    const E v0 = eadd(x0, x1), v1 = esub(x0, x1), v2 = eadd(x2, x3), v3 = esub(x3, x2);
    const E y0 = eadd(v0, v2);
    const E y2 = emulconj(esub(v0, v2), r2);
    const E y1 = emulconj(eaddi(v1, v3), r1);
    const E y3 = emulconj(esubi(v1, v3), r3);
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

// ---------------- digits <-> field ----------------
__device__ __forceinline__ u64 digit_to61(i64 d) { return d >= 0 ? (u64)d : P61 - (u64)(-d); }
__device__ __forceinline__ u32 digit_to31(i64 d) {
    const u64 m = (u64)(d >= 0 ? d : -d);
    const u32 r = red31(m);
    return d >= 0 ? r : (P31 ^ r);
}
__device__ __forceinline__ u64 canon61(u64 x) { return x == P61 ? 0 : x; }
__device__ __forceinline__ u32 canon31(u32 x) { return x == P31 ? 0 : x; }

// Garner: the signed value z with z == r61 (mod P61), z == r31 (mod P31),
// |z| < P61 P31 / 2.
__device__ __forceinline__ i128 crt_signed(u64 r61, u32 r31) {
    r61 = canon61(r61); r31 = canon31(r31);
    u64 u = sub61(r61, (u64)r31);
    u = add61(u, rotl61(canon61(u), 31));                 // u (2^31 + 1) == u / P31 (mod P61)
    u = canon61(u);
    const u128 L = ((u128)u << 31) - u + r31;             // u P31 + r31 < P61 P31
    const u128 M = (u128)P61 * P31;
    return (L > (M >> 1)) ? (i128)L - (i128)M : (i128)L;
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

}  // namespace m2d
