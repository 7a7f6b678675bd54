/*
 * m2_oracle.c -- CPU oracle for the Lucas-Lehmer / PRP squaring chain.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py may load this library, and only as the checker
 * (or as the timed CPU restatement).  The product path (libm2gpu.so and the
 * mersenne2 CLI) never links or calls it.
 *
 * This is a plain-C restatement of the algorithm of cherubrock-seb/mersenne2GPU
 * (mersenne2_gpu.cpp, "M2" below), driven the way M2's generic launch plan
 * drives its kernels (M2:4327-4765), one work-item at a time:
 *
 *   transformsize                M2:286-293
 *   digit widths, IBDWT shifts   M2:3921-3944
 *   twiddle table                M2:3911-3919 (root_nth M2:202/237, bitrev M2:278-282)
 *   field arithmetic             M2:75-261 (host), M2:337-444 (device)
 *   weight                       M2:517-520
 *   forward4 / forward2          M2:732-747 / M2:571-578
 *   square_half                  M2:856-870
 *   backward2 / backward4        M2:580-587 / M2:951-963
 *   unweight_norm                M2:1975-1980
 *   Garner CRT                   M2:2018-2030
 *   digit add-with-carry         M2:1982-1993
 *   block prepare + carry drain  M2:2097-2123, 2922-3004 (restated as one
 *                                sequential pass over all digits with the
 *                                carry out of the top digit re-entering digit 0,
 *                                repeated until the carry is zero: the same
 *                                fully propagated result the block scheme reaches)
 *   LL subtract 2                M2:3006-3024
 *   PRP check (== 9)             M2:3051-3076
 *   PRP x3 variant               gf61_ntt_prp_opencl_inplace_nobitrev_fused.cpp:508-531
 *
 * Parity is pinned against (a) GMP (tests/golden/gmp_chain.c) and (b) the
 * reference's own kernel source compiled for the CPU (oracle/build_ref.py ->
 * oracle/_ref/), see tests/test_oracle.py.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef uint64_t u64;
typedef uint32_t u32;
typedef unsigned __int128 u128;

#define P61 ((((u64)1) << 61) - 1)
#define P31 ((((u32)1) << 31) - 1)

/* ---- field arithmetic: GF(P61^2) x GF(P31^2) (M2:75-261, 337-444) ---- */
static inline u64 add61(u64 a, u64 b) { u64 t = a + b; return t >= P61 ? t - P61 : t; }
static inline u64 sub61(u64 a, u64 b) { return a >= b ? a - b : a + P61 - b; }
static inline u64 mul61(u64 a, u64 b) {
    u128 t = (u128)a * b;
    u64 r = ((u64)t & P61) + (u64)(t >> 61);
    r = (r & P61) + (r >> 61);
    return r >= P61 ? r - P61 : r;
}
static inline u64 shl61(u64 x, unsigned s) {          /* x * 2^s mod P61, M2:363-368 */
    s %= 61u;
    if (s == 0) return x;
    u64 r = ((x << s) & P61) + (x >> (61 - s));
    return r >= P61 ? r - P61 : r;
}
static inline u64 shr61(u64 x, unsigned s) { s %= 61u; return s ? shl61(x, 61u - s) : x; }

static inline u32 add31(u32 a, u32 b) { u32 t = a + b; return t >= P31 ? t - P31 : t; }
static inline u32 sub31(u32 a, u32 b) { return a >= b ? a - b : a + P31 - b; }
static inline u32 mul31(u32 a, u32 b) {
    u64 t = (u64)a * b;
    u64 r = (t & P31) + (t >> 31);
    r = (r & P31) + (r >> 31);
    return (u32)(r >= P31 ? r - P31 : r);
}
static inline u32 shl31(u32 x, unsigned s) {
    s %= 31u;
    if (s == 0) return x;
    u64 r = (((u64)x << s) & P31) + ((u64)x >> (31 - s));
    return (u32)(r >= P31 ? r - P31 : r);
}
static inline u32 shr31(u32 x, unsigned s) { s %= 31u; return s ? shl31(x, 31u - s) : x; }

typedef struct { u64 s0, s1; u32 t0, t1; } gf;   /* M2:299 element layout */

static inline gf gf_add(gf a, gf b) { gf r = { add61(a.s0, b.s0), add61(a.s1, b.s1), add31(a.t0, b.t0), add31(a.t1, b.t1) }; return r; }
static inline gf gf_sub(gf a, gf b) { gf r = { sub61(a.s0, b.s0), sub61(a.s1, b.s1), sub31(a.t0, b.t0), sub31(a.t1, b.t1) }; return r; }
/* a + i*b and a - i*b */
static inline gf gf_addi(gf a, gf b) { gf r = { sub61(a.s0, b.s1), add61(a.s1, b.s0), sub31(a.t0, b.t1), add31(a.t1, b.t0) }; return r; }
static inline gf gf_subi(gf a, gf b) { gf r = { add61(a.s0, b.s1), sub61(a.s1, b.s0), add31(a.t0, b.t1), sub31(a.t1, b.t0) }; return r; }
/* a + conj(b), a - conj(b), conj(a - b) */
static inline gf gf_addconj(gf a, gf b) { gf r = { add61(a.s0, b.s0), sub61(a.s1, b.s1), add31(a.t0, b.t0), sub31(a.t1, b.t1) }; return r; }
static inline gf gf_subconj(gf a, gf b) { gf r = { sub61(a.s0, b.s0), add61(a.s1, b.s1), sub31(a.t0, b.t0), add31(a.t1, b.t1) }; return r; }
static inline gf gf_conjsub(gf a, gf b) { gf r = { sub61(a.s0, b.s0), sub61(b.s1, a.s1), sub31(a.t0, b.t0), sub31(b.t1, a.t1) }; return r; }
static inline gf gf_mul(gf a, gf b) {
    gf r = { sub61(mul61(a.s0, b.s0), mul61(a.s1, b.s1)), add61(mul61(a.s0, b.s1), mul61(a.s1, b.s0)),
             sub31(mul31(a.t0, b.t0), mul31(a.t1, b.t1)), add31(mul31(a.t0, b.t1), mul31(a.t1, b.t0)) };
    return r;
}
/* a * conj(b) */
static inline gf gf_mulconj(gf a, gf b) {
    gf r = { add61(mul61(a.s0, b.s0), mul61(a.s1, b.s1)), sub61(mul61(a.s1, b.s0), mul61(a.s0, b.s1)),
             add31(mul31(a.t0, b.t0), mul31(a.t1, b.t1)), sub31(mul31(a.t1, b.t0), mul31(a.t0, b.t1)) };
    return r;
}
static inline gf gf_sqr(gf a) { return gf_mul(a, a); }

static gf gf_pow(gf a, u64 e) {
    gf r = { 1, 0, 1, 0 };
    while (e) { if (e & 1) r = gf_mul(r, a); a = gf_mul(a, a); e >>= 1; }
    return r;
}

/* Generators of the 2-Sylow subgroups: order 2^62 in GF(P61^2) and 2^32 in
 * GF(P31^2) (M2:173-174, 208-209).  root_nth(n) = H^(ORDER/n) (M2:202, 237). */
static gf root_nth(u64 n) {
    gf h61 = { 264036120304204ull, 4677669021635377ull, 0, 0 };
    gf h31 = { 0, 0, 7735u, 748621u };
    gf a = gf_pow(h61, ((u64)1 << 62) / n), b = gf_pow(h31, ((u64)1 << 32) / n);
    gf r = { a.s0, a.s1, b.t0, b.t1 };
    return r;
}

static u64 bitrev(u64 i, u64 n) {                       /* M2:278-282 */
    u64 r = 0;
    for (; n > 1; n >>= 1, i >>= 1) r = (r << 1) | (i & 1);
    return r;
}

/* ---- tables ---- */

/* Smallest ln >= 3 with ln + 2((p >> ln) + 1) < 92 (M2:286-293). */
int o_transformsize(u64 p) {
    int ln = 2;
    u64 w;
    do { ++ln; w = p >> ln; } while ((u64)ln + 2 * (w + 1) >= 61 + 31);
    return ln;
}

typedef struct {
    u32 p; int mode; int ln; u64 n, h;
    u32 iter;
    unsigned char* width;      /* n digit widths (M2:3929-3934) */
    unsigned char* w61;        /* n IBDWT shifts, GF61 (M2:3936-3939) */
    unsigned char* w31;        /* n IBDWT shifts, GF31 */
    gf* tw;                    /* n twiddles (M2:3911-3919) */
    gf* z;                     /* h elements */
    u64* digit;                /* n canonical digits (the state) */
} o_ctx;

/* digit widths and shifts: width_j = ceil(p(j+1)/n) - ceil(pj/n);
 * shift_j = lr2 * (n - (p j mod n)) mod 61 (resp. 31), shift_0 = 0, with
 * lr2 = (2^60 / n) mod 61 and (2^30 / n) mod 31 (M2:203, 238, 3921-3944). */
static void build_weights(o_ctx* c) {
    u64 n = c->n, p = c->p;
    unsigned lr61 = (unsigned)((((u64)1) << 60) / n % 61), lr31 = (unsigned)((((u64)1) << 30) / n % 31);
    u64 prev = 0;
    for (u64 j = 1; j <= n; ++j) {
        u64 pj = p * j;
        u64 cj = ((pj - 1) >> c->ln) + 1;      /* ceil(pj/n) */
        c->width[j - 1] = (unsigned char)(cj - prev);
        prev = cj;
        if (j < n) {
            u64 r = pj & (n - 1);
            c->w61[j] = (unsigned char)((lr61 * (n - r)) % 61);
            c->w31[j] = (unsigned char)((lr31 * (n - r)) % 31);
        }
    }
    c->w61[0] = 0; c->w31[0] = 0;
}

/* tw[s+j] = root(2s)^bitrev(j,s), s = 1..n/4; tw[n/2+s+j] = tw[s+j]*tw[2(s+j)] (M2:3911-3919) */
static void build_twiddles(o_ctx* c) {
    u64 n = c->n;
    memset(c->tw, 0, sizeof(gf) * n);
    for (u64 s = 1; s <= n / 4; s <<= 1) {
        gf r = root_nth(2 * s);
        for (u64 j = 0; j < s; ++j) c->tw[s + j] = gf_pow(r, bitrev(j, s));
    }
    for (u64 s = 1; s <= n / 4; s <<= 1)
        for (u64 j = 0; j < s; ++j) c->tw[n / 2 + s + j] = gf_mul(c->tw[s + j], c->tw[2 * (s + j)]);
}

/* ---- one squaring (M2 generic plan, M2:4327-4765) ---- */

static void o_square(o_ctx* c) {
    gf* z = c->z; gf* w = c->tw;
    u64 n = c->n, h = c->h;
    /* load digits into GF elements: z[k] = (d_2k, d_2k+1) in both fields (M2:2116, 3908) */
    for (u64 k = 0; k < h; ++k) {
        u64 a = c->digit[2 * k], b = c->digit[2 * k + 1];
        gf e = { a % P61, b % P61, (u32)(a % P31), (u32)(b % P31) };
        z[k] = e;
    }
    /* weight (M2:517-520) */
    for (u64 k = 0; k < h; ++k) {
        z[k].s0 = shl61(z[k].s0, c->w61[2 * k]); z[k].s1 = shl61(z[k].s1, c->w61[2 * k + 1]);
        z[k].t0 = shl31(z[k].t0, c->w31[2 * k]); z[k].t1 = shl31(z[k].t1, c->w31[2 * k + 1]);
    }
    /* forward radix-4 DIF (M2:732-747), s blocks of 4m */
    u64 cur = n / 4, s = 1;
    for (; cur > 1; cur /= 4, s *= 4) {
        u64 m = cur / 2;
        for (u64 j = 0; j < s; ++j) {
            u64 b = j * 4 * m;
            gf w2 = w[2 * (s + j)], w1 = w[s + j], w3 = w[n / 2 + s + j];
            for (u64 i = 0; i < m; ++i) {
                gf u0 = z[b + i], u1 = gf_mul(z[b + m + i], w2), u2 = gf_mul(z[b + 2 * m + i], w1), u3 = gf_mul(z[b + 3 * m + i], w3);
                gf v0 = gf_add(u0, u2), v1 = gf_add(u1, u3), v2 = gf_sub(u0, u2), v3 = gf_sub(u1, u3);
                z[b + i] = gf_add(v0, v1); z[b + m + i] = gf_sub(v0, v1);
                z[b + 2 * m + i] = gf_addi(v2, v3); z[b + 3 * m + i] = gf_subi(v2, v3);
            }
        }
    }
    u64 n4 = h / 2;
    int odd = (cur == 1);
    if (odd) {                                            /* forward2 (M2:571-578) */
        for (u64 j = 0; j < n4; ++j) {
            gf u0 = z[2 * j], u1 = gf_mul(z[2 * j + 1], w[n4 + j]);
            z[2 * j] = gf_add(u0, u1); z[2 * j + 1] = gf_sub(u0, u1);
        }
    }
    /* square_half (M2:856-870): mirror pairs k, mk = 3*2^floor(log2 k) - k - 1 */
    for (u64 j = 0; j < n4; ++j) {
        u64 k = 2 * j, mk = 0;
        if (k) { u64 e = 63 - __builtin_clzll(k); mk = (3ull << e) - k - 1; }
        gf zk = z[k], zmk = z[mk];
        gf u0 = gf_addconj(zk, zmk), u1 = gf_subconj(zk, zmk);
        gf v0 = gf_sub(gf_sqr(u0), gf_mul(gf_sqr(u1), w[n4 + j]));
        gf v1 = gf_mul(u0, gf_add(u1, u1));
        z[k] = gf_add(v0, v1);
        if (k == 0) z[1] = gf_sqr(gf_add(z[1], z[1]));
        else z[mk] = gf_conjsub(v0, v1);
    }
    if (odd) {                                            /* backward2 (M2:580-587) */
        for (u64 j = 0; j < n4; ++j) {
            gf u0 = z[2 * j], u1 = z[2 * j + 1];
            z[2 * j] = gf_add(u0, u1); z[2 * j + 1] = gf_mulconj(gf_sub(u0, u1), w[n4 + j]);
        }
    }
    /* inverse radix-4 DIT (M2:951-963), mirror order */
    for (u64 bm = odd ? 4 : 2, bs = s / 4; bs >= 1; bm *= 4, bs /= 4) {
        u64 m = bm / 2;
        for (u64 j = 0; j < bs; ++j) {
            u64 b = j * 4 * m;
            gf w2 = w[2 * (bs + j)], w1 = w[bs + j], w3 = w[n / 2 + bs + j];
            for (u64 i = 0; i < m; ++i) {
                gf u0 = z[b + i], u1 = z[b + m + i], u2 = z[b + 2 * m + i], u3 = z[b + 3 * m + i];
                gf v0 = gf_add(u0, u1), v1 = gf_sub(u0, u1), v2 = gf_add(u2, u3), v3 = gf_sub(u3, u2);
                z[b + i] = gf_add(v0, v2);
                z[b + 2 * m + i] = gf_mulconj(gf_sub(v0, v2), w1);
                z[b + m + i] = gf_mulconj(gf_addi(v1, v3), w2);
                z[b + 3 * m + i] = gf_mulconj(gf_subi(v1, v3), w3);
            }
        }
        if (bs == 1) break;
    }
    /* unweight: z * 2^-(shift + ln + 1), the 1/(2n) scale included (M2:1975-1980) */
    unsigned l1 = (unsigned)c->ln + 1;
    for (u64 k = 0; k < h; ++k) {
        z[k].s0 = shr61(z[k].s0, c->w61[2 * k] + l1); z[k].s1 = shr61(z[k].s1, c->w61[2 * k + 1] + l1);
        z[k].t0 = shr31(z[k].t0, c->w31[2 * k] + l1); z[k].t1 = shr31(z[k].t1, c->w31[2 * k + 1] + l1);
    }
}

/* Garner: L = u*P31 + r31 with u = (r61 - r31) * (2^31 + 1) mod P61, L < P61*P31 (M2:2018-2030) */
static inline u128 garner(u64 r61, u32 r31) {
    u64 u = mul61(sub61(r61, (u64)r31), (((u64)1) << 31) + 1);
    return (u128)u * P31 + r31;
}

/* carry with full propagation and wrap-around (M2:1982-1993, 2097-2123, 2922-3004);
 * mul3 = 1 applies the x3 of the PRP-3 variant before the carry. */
static void o_carry(o_ctx* c, int mul3) {
    u64 n = c->n;
    u128 carry = 0;
    for (u64 k = 0; k < c->h; ++k) {
        u128 L[2] = { garner(c->z[k].s0, c->z[k].t0), garner(c->z[k].s1, c->z[k].t1) };
        for (int e = 0; e < 2; ++e) {
            u64 j = 2 * k + e;
            u128 t = L[e] * (mul3 ? 3u : 1u) + carry;
            unsigned wd = c->width[j];
            c->digit[j] = (u64)(t & ((((u128)1) << wd) - 1));
            carry = t >> wd;
        }
    }
    while (carry) {                                       /* 2^p == 1: top carry re-enters digit 0 */
        for (u64 j = 0; j < n && carry; ++j) {
            u128 t = (u128)c->digit[j] + carry;
            unsigned wd = c->width[j];
            c->digit[j] = (u64)(t & ((((u128)1) << wd) - 1));
            carry = t >> wd;
        }
    }
}

/* x <- x - a with wrapping borrow (M2:3006-3024) */
static void o_sub(o_ctx* c, u32 a) {
    u32 borrow = a;
    while (borrow) {
        for (u64 j = 0; j < c->n && borrow; ++j) {
            u64 d = c->digit[j];
            if (d >= borrow) { c->digit[j] = d - borrow; borrow = 0; }
            else { c->digit[j] = d + (((u64)1) << c->width[j]) - borrow; borrow = 1; }
        }
    }
}

/* ---- C-ABI used by the tests (ctypes) ---- */

enum { O_LL = 0, O_PRP = 1, O_PRP3 = 2 };

o_ctx* o_create(u32 p, int mode) {
    if (p < 3 || mode < 0 || mode > 2) return NULL;
    o_ctx* c = (o_ctx*)calloc(1, sizeof(o_ctx));
    c->p = p; c->mode = mode; c->ln = o_transformsize(p);
    c->n = (u64)1 << c->ln; c->h = c->n / 2;
    c->width = (unsigned char*)calloc(c->n, 1);
    c->w61 = (unsigned char*)calloc(c->n, 1);
    c->w31 = (unsigned char*)calloc(c->n, 1);
    c->tw = (gf*)calloc(c->n, sizeof(gf));
    c->z = (gf*)calloc(c->h, sizeof(gf));
    c->digit = (u64*)calloc(c->n, sizeof(u64));
    build_weights(c);
    build_twiddles(c);
    /* initial value: 4 for LL, 3 for PRP (M2:3908), spread over the low digits */
    u64 x0 = (mode == O_LL) ? 4 : 3;
    for (u64 j = 0; j < c->n && x0; ++j) {
        unsigned wd = c->width[j];
        c->digit[j] = wd >= 64 ? x0 : (x0 & ((((u64)1) << wd) - 1));
        x0 = wd >= 64 ? 0 : (x0 >> wd);
    }
    return c;
}

void o_destroy(o_ctx* c) {
    if (!c) return;
    free(c->width); free(c->w61); free(c->w31); free(c->tw); free(c->z); free(c->digit); free(c);
}

void o_iterate(o_ctx* c, u32 k) {
    for (u32 i = 0; i < k; ++i) {
        o_square(c);
        o_carry(c, c->mode == O_PRP3);
        if (c->mode == O_LL) o_sub(c, 2);
        c->iter++;
    }
}

int o_ln(const o_ctx* c) { return c->ln; }
u64 o_n(const o_ctx* c) { return c->n; }
u32 o_iter(const o_ctx* c) { return c->iter; }
void o_widths(const o_ctx* c, unsigned char* out) { memcpy(out, c->width, c->n); }
void o_shifts(const o_ctx* c, unsigned char* w61, unsigned char* w31) { memcpy(w61, c->w61, c->n); memcpy(w31, c->w31, c->n); }
void o_twiddles(const o_ctx* c, u64* out /* 4 words per entry: s0, s1, t0, t1 */) {
    for (u64 i = 0; i < c->n; ++i) {
        out[4 * i] = c->tw[i].s0; out[4 * i + 1] = c->tw[i].s1; out[4 * i + 2] = c->tw[i].t0; out[4 * i + 3] = c->tw[i].t1;
    }
}

/* canonical digits: the all-ones vector (== M_p) maps to all zeros (M2:3035-3042) */
static int is_all_ones(const o_ctx* c) {
    for (u64 j = 0; j < c->n; ++j) if (c->digit[j] != ((((u64)1) << c->width[j]) - 1)) return 0;
    return 1;
}
void o_get_digits(const o_ctx* c, u64* out) {
    if (is_all_ones(c)) { memset(out, 0, sizeof(u64) * c->n); return; }
    memcpy(out, c->digit, sizeof(u64) * c->n);
}
void o_set_digits(o_ctx* c, const u64* in, u32 iter) { memcpy(c->digit, in, sizeof(u64) * c->n); c->iter = iter; }

u64 o_res64(const o_ctx* c) {
    if (is_all_ones(c)) return 0;
    u64 r = 0; unsigned pos = 0;
    for (u64 j = 0; j < c->n && pos < 64; ++j) { r |= c->digit[j] << pos; pos += c->width[j]; }
    return r;
}

/* 1 = prime / probable prime (M2:4865-4868, 3051-3076; PRP-3: == 3) */
int o_verdict(const o_ctx* c) {
    u64 want = (c->mode == O_LL) ? 0 : (c->mode == O_PRP ? 9 : 3);
    if (c->p < 64) want %= (((u64)1) << c->p) - 1;     /* 9 mod 7 = 2 for p = 3 */
    if (is_all_ones(c)) return want == 0;
    u64 r = 0; unsigned pos = 0;
    for (u64 j = 0; j < c->n; ++j) {
        if (pos >= 64) { if (c->digit[j]) return 0; }
        else r |= c->digit[j] << pos;
        pos += c->width[j];
    }
    return r == want;
}
