// m2_host.cpp -- host-side tables, roots and exact state conversion.
#include "m2_host.hpp"

#include <algorithm>
#include <cmath>
#include <stdexcept>

namespace m2 {

using u128 = unsigned __int128;
using i128 = __int128;

// ---------------- host field arithmetic ----------------
static inline u64 add61(u64 a, u64 b) { u64 t = a + b; return t >= P61 ? t - P61 : t; }
static inline u64 sub61(u64 a, u64 b) { return a >= b ? a - b : a + P61 - b; }
static inline u64 mul61(u64 a, u64 b) {
    u128 t = (u128)a * b;
    u64 r = ((u64)t & P61) + (u64)(t >> 61);
    r = (r & P61) + (r >> 61);
    return r >= P61 ? r - P61 : r;
}
static inline u32 add31(u32 a, u32 b) { u32 t = a + b; return t >= P31 ? t - P31 : t; }
static inline u32 sub31(u32 a, u32 b) { return a >= b ? a - b : a + P31 - b; }
static inline u32 mul31(u32 a, u32 b) {
    u64 t = (u64)a * b;
    u64 r = (t & P31) + (t >> 31);
    r = (r & P31) + (r >> 31);
    return (u32)(r >= P31 ? r - P31 : r);
}

struct G61 { u64 a, b; };
struct G31 { u32 a, b; };
static inline G61 mul(G61 x, G61 y) {
    return { sub61(mul61(x.a, y.a), mul61(x.b, y.b)), add61(mul61(x.a, y.b), mul61(x.b, y.a)) };
}
static inline G31 mul(G31 x, G31 y) {
    return { sub31(mul31(x.a, y.a), mul31(x.b, y.b)), add31(mul31(x.a, y.b), mul31(x.b, y.a)) };
}
template <class G> static G gpow(G x, u64 e, G one) {
    G r = one;
    while (e) { if (e & 1) r = mul(r, x); x = mul(x, x); e >>= 1; }
    return r;
}

// Generator of the Sylow 2-subgroup (order 2^62 resp. 2^32): the first x = a + b i
// (b = 1, 2, ...; a = 1, 2, ...) whose power x^((q^2-1)/2^k) has full order,
// replaced by its cube if its order-4 power is -i (so that w_4 = +i).
static G61 gen61() {
    static G61 g = [] {
        const G61 one{1, 0};
        for (u64 b = 1; b < 64; ++b)
            for (u64 a = 1; a < 64; ++a) {
                G61 y = gpow(G61{a, b}, (u64(1) << 60) - 1, one);     // (P61^2-1)/2^62 = 2^60-1
                G61 t = gpow(y, u64(1) << 61, one);
                if (t.a == 1 && t.b == 0) continue;                  // order < 2^62
                G61 w4 = gpow(y, u64(1) << 60, one);
                if (w4.a == 0 && w4.b == P61 - 1) y = mul(mul(y, y), y);
                return y;
            }
        throw std::runtime_error("no GF(P61^2) generator found");
    }();
    return g;
}
static G31 gen31() {
    static G31 g = [] {
        const G31 one{1, 0};
        for (u32 b = 1; b < 64; ++b)
            for (u32 a = 1; a < 64; ++a) {
                G31 y = gpow(G31{a, b}, (u64(1) << 30) - 1, one);     // (P31^2-1)/2^32 = 2^30-1
                G31 t = gpow(y, u64(1) << 31, one);
                if (t.a == 1 && t.b == 0) continue;
                G31 w4 = gpow(y, u64(1) << 30, one);
                if (w4.a == 0 && w4.b == P31 - 1) y = mul(mul(y, y), y);
                return y;
            }
        throw std::runtime_error("no GF(P31^2) generator found");
    }();
    return g;
}

Dual root_of_unity(u64 order) {
    if (order == 0 || (order & (order - 1)) || order > (u64(1) << 32)) throw std::invalid_argument("root order");
    G61 x = gpow(gen61(), (u64(1) << 62) / order, G61{1, 0});
    G31 y = gpow(gen31(), (u64(1) << 32) / order, G31{1, 0});
    return Dual{x.a, x.b, y.a, y.b};
}

static inline Dual dmul(const Dual& x, const Dual& y) {
    G61 a = mul(G61{x.a, x.b}, G61{y.a, y.b});
    G31 b = mul(G31{x.c, x.d}, G31{y.c, y.d});
    return Dual{a.a, a.b, b.a, b.b};
}

static inline u64 bitrev(u64 i, int bits) {
    u64 r = 0;
    for (int k = 0; k < bits; ++k, i >>= 1) r = (r << 1) | (i & 1);
    return r;
}

// ---------------- layout ----------------
int transform_log2(u64 p, int bound) {
    int ln = 2;
    u64 w;
    do { ++ln; w = p >> ln; } while (u64(ln) + 2 * (w + 1) >= u64(bound));
    return ln;
}

Layout make_layout(u32 p, int bound) {
    Layout L;
    L.p = p;
    L.ln = transform_log2(p, bound);
    L.n = u64(1) << L.ln;
    L.h = L.n / 2;
    L.q = u32(p >> L.ln);
    L.width.assign(L.n, 0);
    L.w61.assign(L.n, 0);
    L.w31.assign(L.n, 0);
    L.bitpos.assign(L.n + 1, 0);
    const u64 n = L.n;
    // lr = n^-1 mod 61 (resp. 31); 2^60 == 1 mod 61 and 2^30 == 1 mod 31
    const u64 lr61 = ((u64(1) << 60) / n) % 61, lr31 = ((u64(1) << 30) / n) % 31;
    for (u64 j = 0; j <= n; ++j) {
        u64 pj = u64(p) * j;
        L.bitpos[j] = j ? ((pj - 1) >> L.ln) + 1 : 0;         // ceil(p j / n)
        if (j > 0) L.width[j - 1] = uint8_t(L.bitpos[j] - L.bitpos[j - 1]);
        if (j > 0 && j < n) {
            u64 r = pj & (n - 1);
            L.w61[j] = uint8_t((lr61 * (n - r)) % 61);
            L.w31[j] = uint8_t((lr31 * (n - r)) % 31);
        }
    }
    return L;
}

// ---------------- twiddles ----------------
Twiddles make_twiddles(u64 h) {
    Twiddles T;
    int lh = 0;
    while ((u64(1) << lh) < h) ++lh;
    // radix-4 steps: S = 1, 4, 16, ... while 4S <= h
    u64 smax = 0;
    for (u64 S = 1; 4 * S <= h; S *= 4) smax = S;
    T.tw4.assign(smax ? 3 * 2 * smax : 3, Dual{0, 0, 0, 0});
    for (u64 S = 1; 4 * S <= h; S *= 4) {
        int bits = 0;
        while ((u64(1) << bits) < S) ++bits;
        Dual w = root_of_unity(4 * S);
        std::vector<Dual> pw(S);
        pw[0] = Dual{1, 0, 1, 0};
        for (u64 e = 1; e < S; ++e) pw[e] = dmul(pw[e - 1], w);
        for (u64 j = 0; j < S; ++j) {
            Dual r = pw[bitrev(j, bits)];
            Dual r2 = dmul(r, r), r3 = dmul(r2, r);
            T.tw4[3 * (S + j) + 0] = r;
            T.tw4[3 * (S + j) + 1] = r2;
            T.tw4[3 * (S + j) + 2] = r3;
        }
    }
    // centre / radix-2 twiddles: tc[j] = w_h^{br_{h/2}(j)}
    const u64 hh = std::max<u64>(h / 2, 1);
    T.tc.assign(hh, Dual{1, 0, 1, 0});
    if (h >= 2) {
        Dual w = root_of_unity(h);
        std::vector<Dual> pw(hh);
        pw[0] = Dual{1, 0, 1, 0};
        for (u64 e = 1; e < hh; ++e) pw[e] = dmul(pw[e - 1], w);
        for (u64 j = 0; j < hh; ++j) T.tc[j] = pw[bitrev(j, lh - 1)];
    }
    return T;
}

int carry_span(const Layout& L) {
    // |z| <= n * 2^(2q+1) * (1+eps) for balanced digits (|d| <= 2^(w-1) + small);
    // steady-state segment carries are below 2^(ln+q+3).  Propagating such a carry
    // through k digits of width >= q leaves at most c_k, c_{k+1} = (2^q + c_k)/2^q + 1.
    if (L.q == 0) return 1 << 30;   // tiny exponents: only the whole-vector path
    double c = std::ldexp(1.0, L.ln + int(L.q) + 3);
    const double half = std::ldexp(1.0, int(L.q));
    int k = 0;
    while (c > 4.0 && k < 64) { c = (half + c) / std::ldexp(1.0, int(L.q)) + 1.0; ++k; }
    return std::max(k, 1);
}

// ---------------- state conversion ----------------
static std::vector<u64> normalize(const Layout& L, const std::vector<i128>& t);

std::vector<u64> canonical_digits(const Layout& L, const std::vector<i64>& d,
                                  const std::vector<i64>& carry, u64 seg_digits) {
    const u64 n = L.n;
    std::vector<i128> t(n);
    for (u64 j = 0; j < n; ++j) t[j] = d[j];
    if (seg_digits) {
        for (u64 s = 0; s < carry.size(); ++s) t[((s + 1) * seg_digits) % n] += carry[s];
    }
    return normalize(L, t);
}

std::vector<u64> canonical_from_unsigned(const Layout& L, const u64* d) {
    std::vector<i128> t(L.n);
    for (u64 j = 0; j < L.n; ++j) t[j] = (i128)d[j];
    return normalize(L, t);
}

// Exact carry propagation of arbitrary signed digit words to [0, 2^w_j) with
// the top carry re-entering at digit 0 (2^p == 1 mod M_p).
static std::vector<u64> normalize(const Layout& L, const std::vector<i128>& t) {
    const u64 n = L.n;
    std::vector<u64> out(n);
    i128 c = 0;
    for (u64 j = 0; j < n; ++j) {
        const int w = L.width[j];
        i128 v = t[j] + c;
        // floor division by 2^w
        i128 qv = v >> w;            // arithmetic shift == floor for signed
        out[j] = (u64)(v - (qv << w));
        c = qv;
    }
    // 2^p == 1 (mod M_p): the carry out of the top re-enters at digit 0.
    for (int pass = 0; c != 0 && pass < 64; ++pass) {
        for (u64 j = 0; j < n && c != 0; ++j) {
            const int w = L.width[j];
            i128 v = (i128)out[j] + c;
            i128 qv = v >> w;
            out[j] = (u64)(v - (qv << w));
            c = qv;
        }
    }
    if (c != 0) throw std::runtime_error("canonical_digits: carry did not settle");
    bool ones = true;
    for (u64 j = 0; j < n && ones; ++j) ones = (out[j] == ((u64(1) << L.width[j]) - 1));
    if (ones) std::fill(out.begin(), out.end(), 0);
    return out;
}

std::vector<i64> balanced_digits(const Layout& L, const std::vector<u64>& canon) {
    const u64 n = L.n;
    std::vector<i64> out(n);
    i64 c = 0;
    for (u64 j = 0; j < n; ++j) {
        const int w = L.width[j];
        i64 v = i64(canon[j]) + c;
        if (w == 0) { out[j] = 0; c = v; continue; }
        i64 qv = (v + (i64(1) << (w - 1))) >> w;
        out[j] = v - (qv << w);
        c = qv;
    }
    out[0] += c;   // wrap-around (2^p == 1)
    return out;
}

std::vector<u64> digits_of_small(const Layout& L, u64 x) {
    std::vector<u64> out(L.n, 0);
    for (u64 j = 0; j < L.n && x; ++j) {
        const int w = L.width[j];
        if (w == 0) continue;
        out[j] = x & ((u64(1) << w) - 1);
        x = (w >= 64) ? 0 : (x >> w);
    }
    return out;
}

u64 res64_of(const Layout& L, const std::vector<u64>& canon) {
    u64 r = 0;
    for (u64 j = 0; j < L.n && L.bitpos[j] < 64; ++j) r |= canon[j] << L.bitpos[j];
    return r;
}

bool equals_small(const Layout& L, const std::vector<u64>& canon, u64 v) {
    if (L.p < 64) v %= (u64(1) << L.p) - 1;   // canonical residue of v
    return digits_of_small(L, v) == canon;
}

}  // namespace m2
