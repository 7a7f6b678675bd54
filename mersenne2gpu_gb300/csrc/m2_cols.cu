// m2_cols.cu -- column passes of the three-pass path for R = 1024 rows (n =
// 2^21, 2^22) and R = 256 rows with rows of 1024 or 2048 (n = 2^19, 2^20), C =
// 4 columns per CTA, with the radix-16 passes spread over lane quads as in the
// row pass.  R = 256 has four levels (passes A and B) and copies between
// shared and global memory where R = 1024 runs pass C.
//
// k_cols_fwd_q (one CTA per group of 4 columns; 512 threads for R = 1024,
// 128 for R = 256):
//   row stage  each thread takes whole rows: applies the segment carry that
//              the previous k_cols_inv_q left for the row's 8 digits (the carry
//              of the segment before it), converts to both fields and weights;
//   pass A     levels 1-2 of the columns (radix 16 in a lane quad);
//   pass B     levels 3-4;
//   pass C     level 5 on groups of 4 consecutive rows, stored to global memory.
// k_cols_inv_q runs pass C (from global), B and A inverse, then the row stage
// unweights, recombines (CRT) and carries each row segment of 8 digits,
// writing digits and the segment's carry out.
//
// Shared memory: 6 arrays of 32-bit words, element (row r, column c) at
// r C + c through an XOR swizzle of the low five address bits (by bits 5-11)
// that keeps every warp access of these stages on 32 distinct banks.
#include "m2_field.cuh"
#include "m2_kernels.cuh"

using namespace M2D_NS;

namespace M2K_NS {

namespace {

constexpr int CC = 4;
// threads of a CTA for R = CR rows: 8 elements each
template <int CR> struct ColShape { static constexpr int CNT = CR * CC / 8; };

__device__ __forceinline__ u32 swzc(u32 e) {
    u32 x = 0;
    x ^= (0u - ((e >> 5) & 1u)) & 26u;
    x ^= (0u - ((e >> 6) & 1u)) & 31u;
    x ^= (0u - ((e >> 7) & 1u)) & 18u;
    x ^= (0u - ((e >> 8) & 1u)) & 25u;
    x ^= (0u - ((e >> 9) & 1u)) & 14u;
    x ^= (0u - ((e >> 10) & 1u)) & 10u;
    x ^= (0u - ((e >> 11) & 1u)) & 31u;
    return e ^ x;
}

// The swizzle is linear over GF(2), so for an index a + b with a and b on
// disjoint bits swzc(a + b) = swzc(a) ^ swzc(b): the passes swizzle a thread's
// base once and reach each element with one XOR by a compile-time constant
// (ldp/stp take swizzled indices).
struct S6c {
    u32 *al, *ah, *bl, *bh, *c, *d;
    __device__ __forceinline__ E ldp(u32 p) const {
        return E{(u64)al[p] | ((u64)ah[p] << 32), (u64)bl[p] | ((u64)bh[p] << 32), kDual ? c[p] : 0u, kDual ? d[p] : 0u};
    }
    __device__ __forceinline__ void stp(u32 p, const E& v) const {
        al[p] = (u32)v.a; ah[p] = (u32)(v.a >> 32); bl[p] = (u32)v.b; bh[p] = (u32)(v.b >> 32);
        if (kDual) { c[p] = v.c; d[p] = v.d; }
    }
    __device__ __forceinline__ E ld(u32 e) const { return ldp(swzc(e)); }
    __device__ __forceinline__ void st(u32 e, const E& v) const { stp(swzc(e), v); }
};
__device__ __forceinline__ S6c make_s6c(unsigned char* base, u32 ne) {
    u32* w = reinterpret_cast<u32*>(base);
    return S6c{w, w + ne, w + 2 * ne, w + 3 * ne, w + 4 * ne, w + 5 * ne};
}

__device__ __forceinline__ E ldw(const DTw* t, u64 i) {
    const u64* q = reinterpret_cast<const u64*>(t + i);
    const u64 a = __ldg(q), b = __ldg(q + 1), cd = kDual ? __ldg(q + 2) : 0ull;
    return E{a, b, (u32)cd, (u32)(cd >> 32)};
}
struct Tri { E r1, r2, r3; };
__device__ __forceinline__ Tri tri(const DTw* tw4, u64 S, u64 J) {
    const u64 base = 3 * (S + J);
    return Tri{ldw(tw4, base), ldw(tw4, base + 1), ldw(tw4, base + 2)};
}

__device__ __forceinline__ E weigh(i64 d0, i64 d1, u32 s061, u32 s161, u32 s031, u32 s131) {
    return E{rotl61(digit_to61(d0), s061), rotl61(digit_to61(d1), s161), g31(rotl31(digit_to31(d0), s031)), g31(rotl31(digit_to31(d1), s131))};
}

// the 16-element sub-column passes over the columns (rows i + stride k of a
// block; base < stride, so base and stride k sit on disjoint bits).  Lane l of
// the quad loads k = l + 4m, runs the first level, and hands its outputs on
// through the same slots: after a warp barrier it reads k = 4l + m, runs the
// second level and stores there (no other quad touches the 16 slots).
__device__ __forceinline__ void colpass_fwd(const S6c& z, u32 base, u32 stride, u32 l, const DTw* tw4, u64 SA_, u64 JA, u64 JB0) {
    const u32 pb = swzc(base), pl = pb ^ swzc(stride * l), p4l = pb ^ swzc(stride * 4 * l);
    E x[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) x[m] = z.ldp(pl ^ swzc(stride * 4 * m));
    if (SA_ == 1) dif4_1(x[0], x[1], x[2], x[3]);   // the first level: root 1
    else { const Tri A = tri(tw4, SA_, JA); dif4(x[0], x[1], x[2], x[3], A.r1, A.r2, A.r3); }
#pragma unroll
    for (int m = 0; m < 4; ++m) z.stp(pl ^ swzc(stride * 4 * m), x[m]);
    __syncwarp();
#pragma unroll
    for (int m = 0; m < 4; ++m) x[m] = z.ldp(p4l ^ swzc(stride * m));
    { const Tri Bt = tri(tw4, 4 * SA_, JB0 + l); dif4(x[0], x[1], x[2], x[3], Bt.r1, Bt.r2, Bt.r3); }
#pragma unroll
    for (int m = 0; m < 4; ++m) z.stp(p4l ^ swzc(stride * m), x[m]);
}
__device__ __forceinline__ void colpass_inv(const S6c& z, u32 base, u32 stride, u32 l, const DTw* tw4, u64 SA_, u64 JA, u64 JB0) {
    const u32 pb = swzc(base), pl = pb ^ swzc(stride * l), p4l = pb ^ swzc(stride * 4 * l);
    E x[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) x[m] = z.ldp(p4l ^ swzc(stride * m));
    { const Tri Bt = tri(tw4, 4 * SA_, JB0 + l); dit4(x[0], x[1], x[2], x[3], Bt.r1, Bt.r2, Bt.r3); }
#pragma unroll
    for (int m = 0; m < 4; ++m) z.stp(p4l ^ swzc(stride * m), x[m]);
    __syncwarp();
#pragma unroll
    for (int m = 0; m < 4; ++m) x[m] = z.ldp(pl ^ swzc(stride * 4 * m));
    if (SA_ == 1) dit4_1(x[0], x[1], x[2], x[3]);   // the first level: root 1
    else { const Tri A = tri(tw4, SA_, JA); dit4(x[0], x[1], x[2], x[3], A.r1, A.r2, A.r3); }
#pragma unroll
    for (int m = 0; m < 4; ++m) z.stp(pl ^ swzc(stride * 4 * m), x[m]);
}

// element (row r, column c) of the CTA's column group lives at r*CC + c

// ---- stages shared by the three column kernels ----

// forward row stage: pending carry (the carry out of the segment before this
// row's segment), fields, weights.  Digits come from global memory, or from
// the CTA's own shared slots (the fused kernel), where each element slot of a
// row holds its two digits in the al/ah and bl/bh words.
template <int CR, bool FROM_SMEM>
__device__ __forceinline__ void fwd_row_stage(const S6c& z, const LargePlan& P, const LargeBufs& bf, u32 g) {
    constexpr int CNT = ColShape<CR>::CNT;
    const u32 B = P.B, G = P.G, tid = threadIdx.x;
    const u64 RG = (u64)CR * G;
    const u32 p = P.p;
    const int ln = P.ln;
#pragma unroll 1
    for (u32 r = tid; r < (u32)CR; r += CNT) {
        const u64 s = (u64)r * G + g;
        const u64 sp = s ? s - 1 : RG - 1;   // the segment before (the last one for segment 0)
        i64 c = FROM_SMEM ? (i64)__ldcg(reinterpret_cast<const long long*>(bf.carries + sp)) : bf.carries[sp];
        const u64 j0 = 2 * ((u64)r * B + (u64)g * CC);
        i64 d[2 * CC];
        if (FROM_SMEM) {
#pragma unroll
            for (int u = 0; u < CC; ++u) {
                const u32 q = swzc(r * CC) ^ (u32)u;
                d[2 * u] = (i64)((u64)z.al[q] | ((u64)z.ah[q] << 32));
                d[2 * u + 1] = (i64)((u64)z.bl[q] | ((u64)z.bh[q] << 32));
            }
        } else {
            const longlong2* src = reinterpret_cast<const longlong2*>(bf.digits + j0);
#pragma unroll
            for (int u = 0; u < CC; ++u) { const longlong2 v = src[u]; d[2 * u] = v.x; d[2 * u + 1] = v.y; }
        }
#pragma unroll
        for (int u = 0; u < 2 * CC; ++u) {
            if (u < P.span) d[u] = split_balanced64(d[u] + c, width_of(p, ln, j0 + u), c);
            else if (u == P.span) d[u] += c;
        }
        const uchar4* w61 = reinterpret_cast<const uchar4*>(bf.w61 + j0);
        const uchar4* w31 = reinterpret_cast<const uchar4*>(bf.w31 + j0);
#pragma unroll
        for (int h2 = 0; h2 < 2; ++h2) {
            const uchar4 a = w61[h2], b = w31[h2];
            const u32 pr = swzc(r * CC);
            z.stp(pr ^ (u32)(2 * h2), weigh(d[4 * h2], d[4 * h2 + 1], a.x, a.y, b.x, b.y));
            z.stp(pr ^ (u32)(2 * h2 + 1), weigh(d[4 * h2 + 2], d[4 * h2 + 3], a.z, a.w, b.z, b.w));
        }
    }
}

// forward passes A (levels 1-2) and B (levels 3-4) in shared memory, then for
// R = 1024 pass C (level 5, blocks of 4 rows) on the way to global memory, for
// R = 256 (4 levels) a plain copy to global memory
template <int CR>
__device__ __forceinline__ void fwd_passes(const S6c& z, const LargePlan& P, const LargeBufs& bf, u32 g) {
    constexpr int CNT = ColShape<CR>::CNT;
    constexpr u32 MB = CR / 16, SB = (CR >= 256) ? CR / 256 : 1;   // pass B block rows and stride
    const u32 B = P.B, tid = threadIdx.x, l = tid & 3u;
    // pass A: levels 1-2 (blocks of CR and CR/4 rows)
#pragma unroll 1
    for (u32 L = tid; L < (u32)(CC * CR / 4); L += CNT) {
        const u32 sc = L >> 2, c = sc % CC, i = sc / CC;
        colpass_fwd(z, i * CC + c, (CR / 16) * CC, l, bf.tw4, 1, 0, 0);
    }
    __syncthreads();
    // pass B: levels 3-4 (blocks of CR/16 and CR/64 rows)
#pragma unroll 1
    for (u32 L = tid; L < (u32)(CC * CR / 4); L += CNT) {
        const u32 sc = L >> 2, c = sc % CC, rest = sc / CC, jb = rest / SB, ib = rest % SB;
        colpass_fwd(z, (jb * MB + ib) * CC + c, SB * CC, l, bf.tw4, 16, jb, 4 * jb);
    }
    __syncthreads();
    if (CR == 1024) {
        // pass C: level 5 (blocks of 4 rows), to global memory
#pragma unroll 1
        for (u32 Gq = tid; Gq < (u32)(CC * CR / 4); Gq += CNT) {
            const u32 c = Gq % CC, J = Gq / CC;
            const u32 pj = swzc(4 * J * CC + c);     // swzc((4J + b) CC + c) = pj ^ b CC
            E x[4];
#pragma unroll
            for (int b = 0; b < 4; ++b) x[b] = z.ldp(pj ^ (u32)(b * CC));
            const Tri t = tri(bf.tw4, 256, J);
            dif4(x[0], x[1], x[2], x[3], t.r1, t.r2, t.r3);
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const u64 e = (u64)(4 * J + b) * B + (u64)g * CC + c;
                bf.za[e] = make_ulonglong2(x[b].a, x[b].b);
                if (kDual) bf.zb[e] = make_uint2(x[b].c, x[b].d);
            }
        }
    } else {
#pragma unroll 1
        for (u32 e = tid; e < (u32)(CC * CR); e += CNT) {
            const E v = z.ld(e);
            const u64 o = (u64)(e / CC) * B + (u64)g * CC + e % CC;
            bf.za[o] = make_ulonglong2(v.a, v.b);
            if (kDual) bf.zb[o] = make_uint2(v.c, v.d);
        }
    }
}

// inverse passes: for R = 1024 pass C (level 5) from global memory, for R =
// 256 a plain copy from global memory; then B and A
template <int CR>
__device__ __forceinline__ void inv_passes(const S6c& z, const LargePlan& P, const LargeBufs& bf, u32 g) {
    constexpr int CNT = ColShape<CR>::CNT;
    constexpr u32 MB = CR / 16, SB = (CR >= 256) ? CR / 256 : 1;
    const u32 B = P.B, tid = threadIdx.x, l = tid & 3u;
    if (CR == 1024) {
#pragma unroll 1
        for (u32 Gq = tid; Gq < (u32)(CC * CR / 4); Gq += CNT) {
            const u32 c = Gq % CC, J = Gq / CC;
            E x[4];
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const u64 e = (u64)(4 * J + b) * B + (u64)g * CC + c;
                const ulonglong2 va = bf.za[e];
                const uint2 vb = kDual ? bf.zb[e] : make_uint2(0u, 0u);
                x[b] = E{va.x, va.y, vb.x, vb.y};
            }
            const Tri t = tri(bf.tw4, 256, J);
            dit4(x[0], x[1], x[2], x[3], t.r1, t.r2, t.r3);
            const u32 pj = swzc(4 * J * CC + c);
#pragma unroll
            for (int b = 0; b < 4; ++b) z.stp(pj ^ (u32)(b * CC), x[b]);
        }
    } else {
#pragma unroll 1
        for (u32 e = tid; e < (u32)(CC * CR); e += CNT) {
            const u64 o = (u64)(e / CC) * B + (u64)g * CC + e % CC;
            const ulonglong2 va = bf.za[o];
            const uint2 vb = kDual ? bf.zb[o] : make_uint2(0u, 0u);
            z.st(e, E{va.x, va.y, vb.x, vb.y});
        }
    }
    __syncthreads();
#pragma unroll 1
    for (u32 L = tid; L < (u32)(CC * CR / 4); L += CNT) {
        const u32 sc = L >> 2, c = sc % CC, rest = sc / CC, jb = rest / SB, ib = rest % SB;
        colpass_inv(z, (jb * MB + ib) * CC + c, SB * CC, l, bf.tw4, 16, jb, 4 * jb);
    }
    __syncthreads();
#pragma unroll 1
    for (u32 L = tid; L < (u32)(CC * CR / 4); L += CNT) {
        const u32 sc = L >> 2, c = sc % CC, i = sc / CC;
        colpass_inv(z, i * CC + c, (CR / 16) * CC, l, bf.tw4, 1, 0, 0);
    }
}

// inverse row stage: unweight (rotations from the per-element table), CRT,
// carry within the row segment of 8 digits;
// the digits go to global memory or back into the row's own shared slots, the
// segment's carry out to global memory
template <int CR, bool TO_SMEM>
__device__ __forceinline__ void inv_row_stage(const S6c& z, const LargePlan& P, const LargeBufs& bf, u32 g) {
    constexpr int CNT = ColShape<CR>::CNT;
    const u32 B = P.B, G = P.G, tid = threadIdx.x;
#pragma unroll 1
    for (u32 r = tid; r < (u32)CR; r += CNT) {
        const u64 e0 = (u64)r * B + (u64)g * CC, j0 = 2 * e0;
        const u32 mul = (P.mode == PRP3) ? 3u : 1u;
        i64 c = 0;
        u32 bad = 0;
        i64 d[2 * CC];
#pragma unroll
        for (int cc = 0; cc < CC; ++cc) {
            // the element's unweighting rotations and digit widths
            const uint2 t = bf.aux[e0 + cc];
            const E v = z.ldp(swzc(r * CC) ^ (u32)cc);
            const u64 x0 = rotl61(fold61(v.a), t.x & 0xffu), x1 = rotl61(fold61(v.b), (t.x >> 8) & 0xffu);
            const u32 y0 = rotl31(v.c, (t.x >> 16) & 0xffu), y1 = rotl31(v.d, t.x >> 24);
            const i64 sub = (P.mode == LL && j0 + 2 * cc == 0) ? 2 : 0;
            d[2 * cc] = crt_digit(x0, y0, t.y & 0xffu, mul, sub, c, bad, !kDual || P.gf61 != 0);
            d[2 * cc + 1] = crt_digit(x1, y1, (t.y >> 8) & 0xffu, mul, 0, c, bad, !kDual || P.gf61 != 0);
        }
        if (TO_SMEM) {
#pragma unroll
            for (int u = 0; u < CC; ++u) {
                const u32 q = swzc(r * CC) ^ (u32)u;
                z.al[q] = (u32)(u64)d[2 * u]; z.ah[q] = (u32)((u64)d[2 * u] >> 32);
                z.bl[q] = (u32)(u64)d[2 * u + 1]; z.bh[q] = (u32)((u64)d[2 * u + 1] >> 32);
            }
        } else {
            longlong2* dst = reinterpret_cast<longlong2*>(bf.digits + j0);
#pragma unroll
            for (int u = 0; u < CC; ++u) dst[u] = make_longlong2(d[2 * u], d[2 * u + 1]);
        }
        if (bad) atomicOr(bf.status, ST_CARRY_RANGE);
        bf.carries[(u64)r * G + g] = c;
    }
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* a) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(a) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long ld_acquire64(const unsigned long long* a) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(a) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned* a, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" :: "l"(a), "r"(v) : "memory");
}

}  // namespace

// register budget 64 at every shape: two 512-thread CTAs (R = 1024) or eight
// 128-thread CTAs (R = 256) per SM
template <int CR>
__global__ void __launch_bounds__(ColShape<CR>::CNT, 65536 / (64 * ColShape<CR>::CNT)) k_cols_fwd_q(LargePlan P, LargeBufs bf) {
    extern __shared__ __align__(16) unsigned char smem[];
    const S6c z = make_s6c(smem, CR * CC);
    fwd_row_stage<CR, false>(z, P, bf, blockIdx.x);
    __syncthreads();
    fwd_passes<CR>(z, P, bf, blockIdx.x);
}

template <int CR>
__global__ void __launch_bounds__(ColShape<CR>::CNT, 65536 / (64 * ColShape<CR>::CNT)) k_cols_inv_q(LargePlan P, LargeBufs bf) {
    extern __shared__ __align__(16) unsigned char smem[];
    const S6c z = make_s6c(smem, CR * CC);
    inv_passes<CR>(z, P, bf, blockIdx.x);
    __syncthreads();
    inv_row_stage<CR, false>(z, P, bf, blockIdx.x);
}

// The inverse column pass of one squaring fused with the forward column pass
// of the next: the digits never leave the CTA; only the segment carries go
// through global memory, from CTA g-1 to CTA g (CTA G-1 to CTA 0 for the row
// before).  Every CTA publishes its carries, raises its flag to this launch's
// epoch (one more than its value at entry; every launch raises every flag
// once, so all flags are equal between launches) and waits, bounded, for its
// predecessor's flag; a wait that runs out sets ST_WAIT_TIMEOUT and the CTA
// goes on.
//  * TK = false: launched cooperatively, all G CTAs resident, CTA g is group g.
//    With P.mid_barrier the CTA then also waits until all G groups have
//    published (a count of arrivals): a CTA alone on its SM then no longer
//    starts its forward half while CTAs that share an SM are still in their
//    inverse halves, and those get the SM's issue slots to themselves.
//  * TK = true: G CTAs that need not all fit at once (G = 512 at n = 2^22).
//    Each CTA takes its group from a 64-bit ticket counter in arrival order
//    (ticket t of a launch is group t mod G: every launch draws exactly G).
//    The CTA of group g >= 1 then waits only on a CTA that arrived before it,
//    is resident, and publishes before it waits itself; only group 0 waits on
//    a later arrival (group G-1), which gets a slot as the others finish.
template <int CR, bool TK>
__global__ void __launch_bounds__(ColShape<CR>::CNT, 65536 / (64 * ColShape<CR>::CNT)) k_cols_mid_q(LargePlan P, LargeBufs bf) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ unsigned s_epoch;
    const S6c z = make_s6c(smem, CR * CC);
    const u32 G = P.G;
    u32 g = blockIdx.x;
    if (TK) {
        __shared__ unsigned s_g;
        if (threadIdx.x == 0) {
            s_g = (unsigned)(atomicAdd(bf.ticket, 1ull) % G);
            s_epoch = bf.flags[s_g] + 1u;
        }
        __syncthreads();
        g = s_g;
    } else if (threadIdx.x == 0) {
        s_epoch = bf.flags[g] + 1u;
    }
    inv_passes<CR>(z, P, bf, g);
    __syncthreads();
    inv_row_stage<CR, true>(z, P, bf, g);
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned ep = s_epoch;
        st_release(bf.flags + g, ep);
        if (!TK && P.mid_barrier) {
            // phase barrier (cooperative launch, all G CTAs resident): wait
            // until every group has published.  Every launch adds G, so the
            // count reaches a multiple of G.
            const unsigned long long old = atomicAdd(bf.phase, 1ull), target = (old / G + 1) * G;
            unsigned it = 0;
            while ((long long)(ld_acquire64(bf.phase) - target) < 0) {
                if (++it > (1u << 20)) { atomicOr(bf.status, ST_WAIT_TIMEOUT); break; }
                __nanosleep(128);
            }
        }
        const unsigned* prev = bf.flags + (g + G - 1) % G;
        unsigned it = 0;
        while ((int)(ld_acquire(prev) - ep) < 0) {
            if (++it > (1u << 20)) { atomicOr(bf.status, ST_WAIT_TIMEOUT); break; }
            __nanosleep(64);
        }
    }
    __syncthreads();
    // cooperative launch with R = 1024 (every CTA resident): the row pass, a
    // programmatic dependent that waits for this grid's completion before it
    // reads, may now take the SMs' free slots.  Measured: n = 2^21 0.2%
    // faster; with R = 256 and rows of 2048 (n = 2^20) the early row CTAs
    // crowded onto the few SMs with room, and the squaring took 36% longer.
    if (!TK && CR == 1024) asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    fwd_row_stage<CR, true>(z, P, bf, g);
    __syncthreads();
    fwd_passes<CR>(z, P, bf, g);
}

// R = 256 only with rows of 1024 or more: below that (G <= 128 CTAs of 128
// threads) the generic kernels' larger CTAs measured faster
bool cols_q_supported(const LargePlan& P) {
    return (P.R == 1024u || (P.R == 256u && P.B >= 1024u)) && P.C == (u32)CC && P.span < 2 * CC;
}

namespace {
template <int CR>
cudaError_t setup_shape() {
    const int sm = (int)(24ull * CR * CC);
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(k_cols_fwd_q<CR>, cudaFuncAttributePreferredSharedMemoryCarveout, 100))) return e;
    if ((e = cudaFuncSetAttribute(k_cols_inv_q<CR>, cudaFuncAttributePreferredSharedMemoryCarveout, 100))) return e;
    if ((e = cudaFuncSetAttribute(k_cols_mid_q<CR, false>, cudaFuncAttributePreferredSharedMemoryCarveout, 100))) return e;
    if ((e = cudaFuncSetAttribute(k_cols_mid_q<CR, true>, cudaFuncAttributePreferredSharedMemoryCarveout, 100))) return e;
    if ((e = cudaFuncSetAttribute(k_cols_mid_q<CR, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm))) return e;
    if ((e = cudaFuncSetAttribute(k_cols_fwd_q<CR>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm))) return e;
    if ((e = cudaFuncSetAttribute(k_cols_inv_q<CR>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm))) return e;
    return cudaFuncSetAttribute(k_cols_mid_q<CR, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
}
template <int CR>
bool mid_fits(const LargePlan& P) {
    int dev = 0, sms = 0, per = 0, coop = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop) return false;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return false;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_cols_mid_q<CR, false>, ColShape<CR>::CNT, 24ull * CR * CC) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return (long long)per * sms >= (long long)P.G;
}
template <int CR>
cudaError_t launch_mid(const LargePlan& P, const LargeBufs& b, cudaStream_t s) {
    if (P.mid_tickets) {
        k_cols_mid_q<CR, true><<<P.G, ColShape<CR>::CNT, 24ull * CR * CC, s>>>(P, b);
        return cudaGetLastError();
    }
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(P.G);
    cfg.blockDim = dim3(ColShape<CR>::CNT);
    cfg.dynamicSmemBytes = 24ull * CR * CC;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_cols_mid_q<CR, false>, P, b);
}
}  // namespace

cudaError_t cols_q_setup(const LargePlan& P) { return P.R == 1024u ? setup_shape<1024>() : setup_shape<256>(); }

// the fused kernel serves every plan of the quad-shuffle column kernels: with
// a cooperative launch when all G CTAs fit on the device at once, else with
// groups by arrival ticket
bool cols_mid_supported(const LargePlan& P) { return cols_q_supported(P); }
bool cols_mid_cooperative(const LargePlan& P) {
#if M2_DUAL
    if (P.gf61) return m2k_g61::cols_mid_cooperative(P);
#endif
    if (!cols_q_supported(P)) return false;
    return P.R == 1024u ? mid_fits<1024>(P) : mid_fits<256>(P);
}

cudaError_t launch_cols_q(const LargePlan& P, const LargeBufs& b, bool inverse, cudaStream_t s) {
    if (P.R == 1024u) {
        constexpr int CR = 1024;
        if (inverse) k_cols_inv_q<CR><<<P.G, ColShape<CR>::CNT, 24ull * CR * CC, s>>>(P, b);
        else k_cols_fwd_q<CR><<<P.G, ColShape<CR>::CNT, 24ull * CR * CC, s>>>(P, b);
    } else {
        constexpr int CR = 256;
        if (inverse) k_cols_inv_q<CR><<<P.G, ColShape<CR>::CNT, 24ull * CR * CC, s>>>(P, b);
        else k_cols_fwd_q<CR><<<P.G, ColShape<CR>::CNT, 24ull * CR * CC, s>>>(P, b);
    }
    return cudaGetLastError();
}

cudaError_t launch_cols_mid(const LargePlan& P, const LargeBufs& b, cudaStream_t s) {
    return P.R == 1024u ? launch_mid<1024>(P, b, s) : launch_mid<256>(P, b, s);
}

}  // namespace M2K_NS
