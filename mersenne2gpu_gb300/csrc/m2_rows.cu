// m2_rows.cu -- row pass of the three-pass path for row lengths B = 1024 and
// 2048: radix-16 passes spread over lane quads.
//
// One CTA owns a pair of mirror rows (t0, t1): every position of row t1 is the
// mirror (inverse root) of a position of row t0, so the centre square pairs
// them.  Per CTA:
//   pass A  levels 1-2 of the row: a 16-element sub-column lives in a quad of
//           lanes (4 elements each), loaded straight from global memory; one
//           radix-4 level, then the quad hands its elements over through the
//           sub-column's own shared-memory slots (store k = l + 4m, warp
//           barrier, load k = 4l + m), the second radix-4 level, then a store
//           to shared memory;
//   pass B  levels 3-4 the same way, shared memory in and out;
//   tail    the last level (groups of 4, or radix 4 + radix 2 on groups of 8
//           when log2 B is odd), the centre square and the first inverse
//           level: a lane holds a group of row t0, its partner lane the mirror
//           group of row t1, and the centre pairs swap the odd positions
//           through shuffles;
//   then pass B and pass A inverse, the last one storing to global memory.
// Four shared-memory round trips and four barriers per CTA; each lane keeps
// at most 8 elements, so the code stays small and the occupancy high.
//
// Twiddles of row t1 are not loaded: the block of t1 mirroring block J of t0
// has root r' = i conj(r_J) at a radix-4 level (r'^2 = -conj(r_J^2),
// r'^3 = -i conj(r_J^3)) and r' = -conj(r_J) at the radix-2 level, since mirror
// positions hold inverse roots.  The CTA of rows 0 and 1 (each its own mirror)
// loads all its twiddles and runs the tail with per-position centre pairs.
//
// Shared memory holds 6 arrays of 32-bit words (GF(P61) low/high words of the
// two coordinates, GF(P31) coordinates) indexed through an XOR swizzle of the
// low five address bits by bits 5-11, chosen so that every warp access of the
// passes and the tail touches 32 distinct banks.
#include "m2_field.cuh"
#include "m2_kernels.cuh"

using namespace M2D_NS;

namespace M2K_NS {

namespace {

__device__ __forceinline__ u32 swz(u32 e) {
    u32 x = 0;
    x ^= (0u - ((e >> 5) & 1u)) & 30u;
    x ^= (0u - ((e >> 6) & 1u)) & 23u;
    x ^= (0u - ((e >> 7) & 1u)) & 12u;
    x ^= (0u - ((e >> 8) & 1u)) & 21u;
    x ^= (0u - ((e >> 9) & 1u)) & 24u;
    x ^= (0u - ((e >> 10) & 1u)) & 23u;
    x ^= (0u - ((e >> 11) & 1u)) & 10u;
    return e ^ x;
}

// The swizzle is linear over GF(2) (it XORs masks selected by bits 5-11 into
// bits 0-4), so for an index a + b with a and b on disjoint bits swz(a + b) =
// swz(a) ^ swz(b): the passes swizzle a thread's base once and reach each
// element with one XOR by a compile-time constant (ldp/stp take swizzled
// indices).
struct S6 {
    u32 *al, *ah, *bl, *bh, *c, *d;
    __device__ __forceinline__ E ldp(u32 p) const {
        return E{(u64)al[p] | ((u64)ah[p] << 32), (u64)bl[p] | ((u64)bh[p] << 32), kDual ? c[p] : 0u, kDual ? d[p] : 0u};
    }
    __device__ __forceinline__ void stp(u32 p, const E& v) const {
        al[p] = (u32)v.a; ah[p] = (u32)(v.a >> 32); bl[p] = (u32)v.b; bh[p] = (u32)(v.b >> 32);
        if (kDual) { c[p] = v.c; d[p] = v.d; }
    }
    __device__ __forceinline__ E ld(u32 e) const { return ldp(swz(e)); }
    __device__ __forceinline__ void st(u32 e, const E& v) const { stp(swz(e), v); }
};
__device__ __forceinline__ S6 make_s6(unsigned char* base, u32 ne) {
    u32* w = reinterpret_cast<u32*>(base);
    return S6{w, w + ne, w + 2 * ne, w + 3 * ne, w + 4 * ne, w + 5 * ne};
}

__device__ __forceinline__ E ldw(const DTw* t, u64 i) {
    const u64* q = reinterpret_cast<const u64*>(t + i);
    const u64 a = __ldg(q), b = __ldg(q + 1), cd = kDual ? __ldg(q + 2) : 0ull;
    return E{a, b, (u32)cd, (u32)(cd >> 32)};
}
__device__ __forceinline__ u64 neg61(u64 x) { return P61 - x; }
__device__ __forceinline__ u32 neg31(u32 x) { return g31(P31 - x); }
// mirror-block twiddles (inputs canonical, outputs in [0, P61] / [0, P31])
__device__ __forceinline__ E mir1(const E& r) { return E{r.b, r.a, r.d, r.c}; }                                 // i conj(r)
__device__ __forceinline__ E mir2(const E& r) { return E{neg61(r.a), r.b, neg31(r.c), r.d}; }                  // -conj(r^2)
__device__ __forceinline__ E mir3(const E& r) { return E{neg61(r.b), neg61(r.a), neg31(r.d), neg31(r.c)}; }    // -i conj(r^3)
__device__ __forceinline__ E mirp(const E& r) { return E{neg61(r.a), r.b, neg31(r.c), r.d}; }                  // -conj(r), radix 2
__device__ __forceinline__ E times_i(const E& r) { return E{neg61(r.b), r.a, neg31(r.d), r.c}; }               // i r

struct Tri { E r1, r2, r3; };
// triple of block J at the radix-4 step with S blocks; mirrored when `mir`
__device__ __forceinline__ Tri tri(const DTw* tw4, u64 S, u64 J, bool mir) {
    const u64 base = 3 * (S + J);
    const E a = ldw(tw4, base), b = ldw(tw4, base + 1), c = ldw(tw4, base + 2);
    if (!mir) return Tri{a, b, c};
    return Tri{mir1(a), mir2(b), mir3(c)};
}

__device__ __forceinline__ E gload(const LargeBufs& bf, u64 e) {
    const ulonglong2 va = bf.za[e];
    const uint2 vb = kDual ? bf.zb[e] : make_uint2(0u, 0u);
    return E{va.x, va.y, vb.x, vb.y};
}
__device__ __forceinline__ void gstore(const LargeBufs& bf, u64 e, const E& v) {
    bf.za[e] = make_ulonglong2(v.a, v.b);
    if (kDual) bf.zb[e] = make_uint2(v.c, v.d);
}


// A radix-16 pass on one sub-column of 16 elements e(k) = base + stride k,
// spread over a quad: lane l loads k = l + 4m (load(m)), runs the first
// radix-4 level (block JA at SA_ blocks), transposes, runs the second level
// (block JB0 + l, or JB0 + 3 - l when mirrored, at 4 SA_ blocks) and stores
// k = 4l + m (store(m, v)).  The inverse loads k = 4l + m, runs the same steps
// backwards and stores k = l + 4m.
// The quad's exchange between the two levels goes through the sub-column's
// own shared-memory slots: the first level's outputs are stored where k = l + 4m
// lies (xst(m, v)), and after a warp barrier each lane reads k = 4l + m
// (xld(m)).  No other quad touches those 16 slots during the pass.
template <class LOAD, class STORE, class XST, class XLD>
__device__ __forceinline__ void pass16_fwd(LOAD&& load, STORE&& store, XST&& xst, XLD&& xld, u32 l, const DTw* tw4, u64 SA_,
                                           u64 JA, u64 JB0, bool mir) {
    E x[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) x[m] = load(m);
    {
        const Tri A = tri(tw4, SA_, JA, mir);
        dif4(x[0], x[1], x[2], x[3], A.r1, A.r2, A.r3);
    }
#pragma unroll
    for (int m = 0; m < 4; ++m) xst(m, x[m]);
    __syncwarp();
#pragma unroll
    for (int m = 0; m < 4; ++m) x[m] = xld(m);
    {
        const Tri Bt = tri(tw4, 4 * SA_, JB0 + (mir ? 3 - l : l), mir);
        dif4(x[0], x[1], x[2], x[3], Bt.r1, Bt.r2, Bt.r3);
    }
#pragma unroll
    for (int m = 0; m < 4; ++m) store(m, x[m]);
}
// the inverse: loads k = 4l + m, exchanges through xst (k = 4l + m) and xld
// (k = l + 4m), stores k = l + 4m
template <class LOAD, class STORE, class XST, class XLD>
__device__ __forceinline__ void pass16_inv(LOAD&& load, STORE&& store, XST&& xst, XLD&& xld, u32 l, const DTw* tw4, u64 SA_,
                                           u64 JA, u64 JB0, bool mir) {
    E x[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) x[m] = load(m);
    {
        const Tri Bt = tri(tw4, 4 * SA_, JB0 + (mir ? 3 - l : l), mir);
        dit4(x[0], x[1], x[2], x[3], Bt.r1, Bt.r2, Bt.r3);
    }
#pragma unroll
    for (int m = 0; m < 4; ++m) xst(m, x[m]);
    __syncwarp();
#pragma unroll
    for (int m = 0; m < 4; ++m) x[m] = xld(m);
    {
        const Tri A = tri(tw4, SA_, JA, mir);
        dit4(x[0], x[1], x[2], x[3], A.r1, A.r2, A.r3);
    }
#pragma unroll
    for (int m = 0; m < 4; ++m) store(m, x[m]);
}

}  // namespace

template <int B>
// two CTAs per SM at both row lengths: for B = 2048 the 64-register limit
// spills about 1.2 KiB per thread, and still measured 3% faster than one CTA
// per SM at 128 registers
__global__ void __launch_bounds__(512, 2) k_rows_q(LargePlan P, LargeBufs bf) {
    constexpr int T = (B == 2048) ? 8 : 4;      // tail group
    constexpr int NT = 512;
    constexpr int PER = B / 16;                // sub-columns per row
    constexpr int SA = B / 16;                 // pass A stride
    constexpr int MB = B / 16, SB = B / 256;   // pass B block and stride
    constexpr int QIT = (2 * PER * 4) / NT;    // quad-lane roles per thread per pass
    // launched as a programmatic dependent of the previous column pass: the CTA
    // may be resident before that grid has finished, and waits here until its
    // writes are complete and visible
    asm volatile("griddepcontrol.wait;" ::: "memory");
    extern __shared__ __align__(16) unsigned char smem[];
    const S6 z = make_s6(smem, 2 * B);
    const u32 pi = blockIdx.x, tid = threadIdx.x;
    u32 t0, t1;
    if (pi == 0) { t0 = 0; t1 = 1; }
    else {
        const u32 e = 32u - __clz(pi);
        const u32 a = pi - (1u << (e - 1));
        t0 = (1u << e) + a;
        t1 = (2u << e) - 1u - a;
    }
    const bool general = (pi != 0);
    const u64 R = P.R;
    const u32 l = tid & 3u;

    // ---------------- pass A: levels 1-2 ----------------
#pragma unroll 1
    for (int it = 0; it < QIT; ++it) {
        const u32 sc = (tid >> 2) + (u32)it * (NT / 4);     // sub-column in [0, 2 PER)
        const u32 sl = sc / PER, i = sc % PER;
        const u32 trow = sl ? t1 : t0;
        const bool mir = general && sl;
        const u32 tsrc = mir ? t0 : trow;
        const u32 pb = swz(sl * B + i), ps = pb ^ swz(SA * 4 * l), pk = pb ^ swz(SA * l);   // k = 4l + m; k = l + 4m
        pass16_fwd([&](int m) { return gload(bf, (u64)trow * B + i + (u64)SA * (l + 4 * m)); },
                   [&](int m, const E& v) { z.stp(ps ^ swz(SA * m), v); },
                   [&](int m, const E& v) { z.stp(pk ^ swz(SA * 4 * m), v); }, [&](int m) { return z.ldp(ps ^ swz(SA * m)); },
                   l, bf.tw4, R, tsrc, 4ull * tsrc, mir);
    }
    __syncthreads();
    // ---------------- pass B: levels 3-4 ----------------
#pragma unroll 1
    for (int it = 0; it < QIT; ++it) {
        const u32 sc = (tid >> 2) + (u32)it * (NT / 4);
        const u32 sl = sc / PER, q = sc % PER, jb = q / SB, ib = q % SB;
        const bool mir = general && sl;
        const u32 tsrc = mir ? t0 : (sl ? t1 : t0);
        const u64 jj = mir ? 15 - jb : jb;
        const u32 base = sl * B + jb * MB + ib;
        const u32 pb = swz(base), pl = pb ^ swz(SB * l), p4l = pb ^ swz(SB * 4 * l);
        pass16_fwd([&](int m) { return z.ldp(pl ^ swz(SB * 4 * m)); }, [&](int m, const E& v) { z.stp(p4l ^ swz(SB * m), v); },
                   [&](int m, const E& v) { z.stp(pl ^ swz(SB * 4 * m), v); }, [&](int m) { return z.ldp(p4l ^ swz(SB * m)); },
                   l, bf.tw4, 16 * R, 16ull * tsrc + jj, 64ull * tsrc + 4 * jj, mir);
    }
    __syncthreads();
    // ---------------- tail: last level(s) + centre + first inverse level(s) ----------------
    const u64 S5 = 256 * R;                    // blocks at the last radix-4 step (h/4 or h/8)
    if (general) {
        // lane pair: even lane = group J of row t0, odd lane = its mirror group of row t1
        const u32 J = tid >> 1, s = tid & 1u;
        const u32 G = s ? (B / T - 1 - J) : J;
        const u32 ebase = s * B + G * T;
        E x[T];
        const u32 pe = swz(ebase);                 // ebase is a multiple of T: swz(ebase + b) = pe ^ b
#pragma unroll
        for (int b = 0; b < T; ++b) x[b] = z.ldp(pe ^ (u32)b);
        const Tri r0 = tri(bf.tw4, S5, (u64)t0 * (B / T) + J, false);
        const Tri r = s ? Tri{mir1(r0.r1), mir2(r0.r2), mir3(r0.r3)} : r0;
        if (T == 4) {
            dif4(x[0], x[1], x[2], x[3], r.r1, r.r2, r.r3);
            E y1 = shfl_xor_e(x[1], 1), y3 = shfl_xor_e(x[3], 1);
            centre_pair(x[0], y3, r.r1);
            centre_pair(x[2], y1, times_i(r.r1));
            x[1] = shfl_xor_e(y1, 1);
            x[3] = shfl_xor_e(y3, 1);
            dit4(x[0], x[1], x[2], x[3], r.r1, r.r2, r.r3);
        } else {
            E p[4];
            const u64 pbase = (u64)t0 * (B / 2) + 4ull * J;
#pragma unroll
            for (int b = 0; b < 4; ++b) p[b] = ldw(bf.tc, pbase + (s ? 3 - b : b));
            if (s) {
#pragma unroll
                for (int b = 0; b < 4; ++b) p[b] = mirp(p[b]);
            }
#pragma unroll
            for (int u = 0; u < 2; ++u) dif4(x[u], x[u + 2], x[u + 4], x[u + 6], r.r1, r.r2, r.r3);
#pragma unroll
            for (int b = 0; b < 4; ++b) dif2(x[2 * b], x[2 * b + 1], p[b]);
            E y[4];
#pragma unroll
            for (int b = 0; b < 4; ++b) y[b] = shfl_xor_e(x[2 * b + 1], 1);     // partner's odd positions
#pragma unroll
            for (int b = 0; b < 4; ++b) centre_pair(x[2 * b], y[3 - b], p[b]);    // mirror of 2b is 7 - 2b
#pragma unroll
            for (int b = 0; b < 4; ++b) x[2 * b + 1] = shfl_xor_e(y[b], 1);
#pragma unroll
            for (int b = 0; b < 4; ++b) dit2(x[2 * b], x[2 * b + 1], p[b]);
#pragma unroll
            for (int u = 0; u < 2; ++u) dit4(x[u], x[u + 2], x[u + 4], x[u + 6], r.r1, r.r2, r.r3);
        }
#pragma unroll
        for (int b = 0; b < T; ++b) z.stp(pe ^ (u32)b, x[b]);
    } else {
        // rows 0 and 1: each row its own mirror; per-group steps with table twiddles,
        // then per-position centre pairs
        for (u32 G = tid; G < (u32)(2 * B / T); G += NT) {
            const u32 s = G / (B / T), J = G % (B / T);
            const u32 tr = s ? t1 : t0;
            E g[T];
#pragma unroll
            for (int b = 0; b < T; ++b) g[b] = z.ld(s * B + J * T + b);
            const Tri r = tri(bf.tw4, S5, (u64)tr * (B / T) + J, false);
            if (T == 4) {
                dif4(g[0], g[1], g[2], g[3], r.r1, r.r2, r.r3);
            } else {
#pragma unroll
                for (int u = 0; u < 2; ++u) dif4(g[u], g[u + 2], g[u + 4], g[u + 6], r.r1, r.r2, r.r3);
#pragma unroll
                for (int b = 0; b < 4; ++b) dif2(g[2 * b], g[2 * b + 1], ldw(bf.tc, (u64)tr * (B / 2) + 4ull * J + b));
            }
#pragma unroll
            for (int b = 0; b < T; ++b) z.st(s * B + J * T + b, g[b]);
        }
        __syncthreads();
        for (u32 b = tid; b < (u32)B; b += NT) {
            const u32 s = b / (B / 2), i = 2 * (b % (B / 2));
            const u64 k = (u64)(s ? t1 : t0) * B + i;
            if (k == 0) {
                E a0 = z.ld(0), a1 = z.ld(1);
                centre_zero(a0, a1);
                z.st(0, a0); z.st(1, a1);
            } else {
                const u32 e = 63u - (u32)__clzll((long long)k);
                const u64 mk = (3ull << e) - k - 1ull;
                const u32 li = s * B + i, lm = s * B + (u32)(mk % B);
                E zk = z.ld(li), zm = z.ld(lm);
                centre_pair(zk, zm, ldw(bf.tc, k >> 1));
                z.st(li, zk); z.st(lm, zm);
            }
        }
        __syncthreads();
        for (u32 G = tid; G < (u32)(2 * B / T); G += NT) {
            const u32 s = G / (B / T), J = G % (B / T);
            const u32 tr = s ? t1 : t0;
            E g[T];
#pragma unroll
            for (int b = 0; b < T; ++b) g[b] = z.ld(s * B + J * T + b);
            const Tri r = tri(bf.tw4, S5, (u64)tr * (B / T) + J, false);
            if (T == 4) {
                dit4(g[0], g[1], g[2], g[3], r.r1, r.r2, r.r3);
            } else {
#pragma unroll
                for (int b = 0; b < 4; ++b) dit2(g[2 * b], g[2 * b + 1], ldw(bf.tc, (u64)tr * (B / 2) + 4ull * J + b));
#pragma unroll
                for (int u = 0; u < 2; ++u) dit4(g[u], g[u + 2], g[u + 4], g[u + 6], r.r1, r.r2, r.r3);
            }
#pragma unroll
            for (int b = 0; b < T; ++b) z.st(s * B + J * T + b, g[b]);
        }
    }
    __syncthreads();
    // ---------------- pass B inverse ----------------
#pragma unroll 1
    for (int it = 0; it < QIT; ++it) {
        const u32 sc = (tid >> 2) + (u32)it * (NT / 4);
        const u32 sl = sc / PER, q = sc % PER, jb = q / SB, ib = q % SB;
        const bool mir = general && sl;
        const u32 tsrc = mir ? t0 : (sl ? t1 : t0);
        const u64 jj = mir ? 15 - jb : jb;
        const u32 base = sl * B + jb * MB + ib;
        const u32 pb = swz(base), pl = pb ^ swz(SB * l), p4l = pb ^ swz(SB * 4 * l);
        pass16_inv([&](int m) { return z.ldp(p4l ^ swz(SB * m)); }, [&](int m, const E& v) { z.stp(pl ^ swz(SB * 4 * m), v); },
                   [&](int m, const E& v) { z.stp(p4l ^ swz(SB * m), v); }, [&](int m) { return z.ldp(pl ^ swz(SB * 4 * m)); },
                   l, bf.tw4, 16 * R, 16ull * tsrc + jj, 64ull * tsrc + 4 * jj, mir);
    }
    __syncthreads();
    // ---------------- pass A inverse ----------------
#pragma unroll 1
    for (int it = 0; it < QIT; ++it) {
        const u32 sc = (tid >> 2) + (u32)it * (NT / 4);
        const u32 sl = sc / PER, i = sc % PER;
        const u32 trow = sl ? t1 : t0;
        const bool mir = general && sl;
        const u32 tsrc = mir ? t0 : trow;
        const u32 pb = swz(sl * B + i), pl = pb ^ swz(SA * 4 * l), pk = pb ^ swz(SA * l);   // k = 4l + m; k = l + 4m
        pass16_inv([&](int m) { return z.ldp(pl ^ swz(SA * m)); },
                   [&](int m, const E& v) { gstore(bf, (u64)trow * B + i + (u64)SA * (l + 4 * m), v); },
                   [&](int m, const E& v) { z.stp(pl ^ swz(SA * m), v); }, [&](int m) { return z.ldp(pk ^ swz(SA * 4 * m)); },
                   l, bf.tw4, R, tsrc, 4ull * tsrc, mir);
    }
}

bool rows_q_supported(const LargePlan& P) { return P.B == 1024 || P.B == 2048; }

cudaError_t rows_q_setup(const LargePlan& P) {
    const int sm = (int)(24ull * 2 * P.B);
    cudaError_t e;
    if (P.B == 1024) {
        if ((e = cudaFuncSetAttribute(k_rows_q<1024>, cudaFuncAttributePreferredSharedMemoryCarveout, 100))) return e;
        return cudaFuncSetAttribute(k_rows_q<1024>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    }
    if (P.B == 2048) {
        if ((e = cudaFuncSetAttribute(k_rows_q<2048>, cudaFuncAttributePreferredSharedMemoryCarveout, 100))) return e;
        return cudaFuncSetAttribute(k_rows_q<2048>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_rows_q(const LargePlan& P, const LargeBufs& b, cudaStream_t s) {
    // programmatic dependent launch: scheduling overlaps the previous kernel's
    // tail; the kernel's griddepcontrol.wait orders the data
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(P.R / 2);
    cfg.blockDim = dim3(512);
    cfg.dynamicSmemBytes = 24ull * 2 * P.B;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    if (P.B == 1024) return cudaLaunchKernelEx(&cfg, k_rows_q<1024>, P, b);
    if (P.B == 2048) return cudaLaunchKernelEx(&cfg, k_rows_q<2048>, P, b);
    return cudaErrorInvalidValue;
}

}  // namespace M2K_NS
