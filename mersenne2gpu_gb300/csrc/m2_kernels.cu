// m2_kernels.cu -- sm_103a kernels of the squaring chain x <- x^2 (-2) mod 2^p - 1.
//
// State between iterations: n balanced signed digits d_j (|d_j| <~ 2^(w_j-1),
// widths w_j = ceil(p(j+1)/n) - ceil(pj/n)), in natural order, as int64.
// One squaring is an IBDWT over GF(P61^2) x GF(P31^2):
//   weight (rotate by the IBDWT shift) -> forward transform (in-place DIF with
//   per-block twiddles, natural in, bit-reversed out) -> real-packed centre
//   square -> inverse transform -> unweight (includes the 1/(2n) scale) ->
//   Garner CRT to a signed 92-bit word -> balanced carry.
//
// Two execution shapes:
//  * k_small: one CTA owns one whole test (state in shared memory) and loops
//    over iterations on-chip.  Used for a lone test up to n = 2048, and by the
//    batched engine and the server up to n = 16384 (one CTA per test, many
//    tests per launch).
//  * three-pass path, h = R x B elements (these generic kernels serve every
//    plan; m2_cols.cu and m2_rows.cu hold faster ones for R = 1024 / B = 1024,
//    2048 and the fused inverse + forward column pass):
//      k_cols_fwd: apply pending segment carries, weight, first log2 R levels
//                  down the columns (C adjacent columns per CTA)
//      k_rows:     last log2 B levels, centre square, first inverse levels on a
//                  pair of mirror rows per CTA
//      k_cols_inv: last inverse levels on the columns, unweight, CRT, carry
//                  within each row segment of C elements; the segment's carry
//                  out is applied by the next k_cols_fwd.
#include "m2_kernels.cuh"
#include "m2_field.cuh"

using namespace M2D_NS;

namespace M2K_NS {

namespace {

struct SE {
    u64* a; u64* b; u32* c; u32* d;
    __device__ __forceinline__ E ld(u32 i) const { return E{a[i], b[i], kDual ? c[i] : 0u, kDual ? d[i] : 0u}; }
    __device__ __forceinline__ void st(u32 i, const E& e) const {
        a[i] = e.a; b[i] = e.b;
        if (kDual) { c[i] = e.c; d[i] = e.d; }
    }
};
__device__ __forceinline__ SE make_se(unsigned char* base, u32 ne) {
    return SE{(u64*)base, (u64*)base + ne, (u32*)(base + 16ull * ne), (u32*)(base + 16ull * ne) + ne};
}

// The one-CTA kernel's arrays are indexed through an XOR swizzle of the low
// four element-index bits by bits 4 and up (one IMAD, three ALU ops): chosen
// by a bank-conflict model of every access of the kernel (contiguous, radix-4
// strides 1 ... h/4, radix-2 pairs, centre mirrors, the segmented carry's lane
// stride n / (2 Tc)) for h = 64 ... 8192 and 32 ... 256 threads, which it
// leaves with 3.5% of the unswizzled layout's extra shared-memory wavefronts.
__device__ __forceinline__ u32 swsm(u32 i) { return i ^ ((((i >> 4) * 5u) ^ (i >> 8)) & 15u); }
struct SZ {
    u64* a; u64* b; u32* c; u32* d;
    __device__ __forceinline__ E ld(u32 i) const {
        const u32 q = swsm(i);
        return E{a[q], b[q], kDual ? c[q] : 0u, kDual ? d[q] : 0u};
    }
    __device__ __forceinline__ void st(u32 i, const E& e) const {
        const u32 q = swsm(i);
        a[q] = e.a; b[q] = e.b;
        if (kDual) { c[q] = e.c; d[q] = e.d; }
    }
    __device__ __forceinline__ u64& A(u32 i) const { return a[swsm(i)]; }
    __device__ __forceinline__ u64& Bv(u32 i) const { return b[swsm(i)]; }
};
__device__ __forceinline__ SZ make_sz(unsigned char* base, u32 ne) {
    return SZ{(u64*)base, (u64*)base + ne, (u32*)(base + 16ull * ne), (u32*)(base + 16ull * ne) + ne};
}

__device__ __forceinline__ E ldtw(const DTw* t, u32 i) {
    const u64* q = reinterpret_cast<const u64*>(t + i);
    const u64 a = __ldg(q), b = __ldg(q + 1), cd = kDual ? __ldg(q + 2) : 0ull;
    return E{a, b, (u32)cd, (u32)(cd >> 32)};
}


__device__ __forceinline__ E weigh(i64 d0, i64 d1, u32 s061, u32 s161, u32 s031, u32 s131) {
    return E{rotl61(digit_to61(d0), s061), rotl61(digit_to61(d1), s161), g31(rotl31(digit_to31(d0), s031)), g31(rotl31(digit_to31(d1), s131))};
}
// multiplier 2^-(s + ln + 1) as a left rotation
__device__ __forceinline__ u32 unrot61(u32 s, int ln) { const u32 t = (s + (u32)ln + 1u) % 61u; return t ? 61u - t : 0u; }
__device__ __forceinline__ u32 unrot31(u32 s, int ln) { const u32 t = (s + (u32)ln + 1u) % 31u; return t ? 31u - t : 0u; }

// unweight element k (digits 2k, 2k+1) and return the two signed convolution words
// GF(P61)-only transforms: the residue in (-P61/2, P61/2] is the word itself
__device__ __forceinline__ i128 signed61(u64 a) {
    a = full61(a);
    return (a > (P61 >> 1)) ? (i128)a - (i128)P61 : (i128)a;
}
__device__ __forceinline__ void unweigh_crt(const E& v, u64 j, const unsigned char* w61, const unsigned char* w31, int ln,
                                            int mode, int gf61_only, i128& z0, i128& z1) {
    const u64 a = rotl61(fold61(v.a), unrot61(w61[j], ln)), b = rotl61(fold61(v.b), unrot61(w61[j + 1], ln));
    if (!kDual || gf61_only) {
        z0 = signed61(a);
        z1 = signed61(b);
    } else {
        const u32 c = rotl31(v.c, unrot31(w31[j], ln)), d = rotl31(v.d, unrot31(w31[j + 1], ln));
        z0 = crt_signed(a, c);
        z1 = crt_signed(b, d);
    }
    if (mode == PRP3) { z0 *= 3; z1 *= 3; }
}


}  // namespace

// =====================================================================
// k_small: whole test in one CTA
// =====================================================================

// The fused middle of a squaring: the last forward level, the centre square and
// the first inverse level in one pass.  The last level works on blocks of q
// consecutive positions (q = 4: the last radix-4 step when log2 h is even;
// q = 2: the radix-2 step when it is odd), and the centre pairs position k
// with its mirror 3 2^e - k - 1 (2^e <= k < 2^(e+1)), which for k = q j + 2c
// (j >= 2) lies at offset q - 1 - 2c of block j' = 3 2^e' - 1 - j
// (2^e' <= j < 2^(e'+1)): blocks j and j' hold each other's mirrors, so one
// thread runs both blocks through the level, the centre and the inverse level.
// Blocks 0 and 1 are their own mirrors.  Work item w = 0 is blocks 0 and 1;
// w >= 1 is the pair j = w + 2^floor(log2 w), j' = 3 2^floor(log2 j) - 1 - j.
template <int Q>
__device__ __forceinline__ void fused_middle(const SZ& z, const SmallTest& T, u32 h, u32 s4max) {
    const u32 nb = h / Q, items = nb > 1 ? nb / 2 : 1;
    auto fwd = [&](E* x, u32 j) {
        if (Q == 4) {
            const u32 ti = 3 * (s4max + j);
            if (s4max == 1) dif4_1(x[0], x[1], x[2], x[3]);
            else dif4(x[0], x[1], x[2], x[3], ldtw(T.tw4, ti), ldtw(T.tw4, ti + 1), ldtw(T.tw4, ti + 2));
        } else {
            dif2(x[0], x[1], ldtw(T.tc, j));
        }
    };
    auto inv = [&](E* x, u32 j) {
        if (Q == 4) {
            const u32 ti = 3 * (s4max + j);
            if (s4max == 1) dit4_1(x[0], x[1], x[2], x[3]);
            else dit4(x[0], x[1], x[2], x[3], ldtw(T.tw4, ti), ldtw(T.tw4, ti + 1), ldtw(T.tw4, ti + 2));
        } else {
            dit2(x[0], x[1], ldtw(T.tc, j));
        }
    };
    for (u32 w = threadIdx.x; w < items; w += blockDim.x) {
        E x[Q], y[Q];
        if (w == 0) {
            // block 0: positions 0 and 1 are their own mirrors; with q = 4, 2 pairs with 3
#pragma unroll
            for (int c = 0; c < Q; ++c) x[c] = z.ld(c);
            fwd(x, 0);
            centre_zero(x[0], x[1]);
            if (Q == 4) centre_pair(x[2], x[3], ldtw(T.tc, 1));
            inv(x, 0);
#pragma unroll
            for (int c = 0; c < Q; ++c) z.st(c, x[c]);
            if (nb > 1) {
                // block 1: position Q + 2c pairs with Q + Q - 1 - 2c
#pragma unroll
                for (int c = 0; c < Q; ++c) y[c] = z.ld(Q + c);
                fwd(y, 1);
#pragma unroll
                for (int c = 0; c < Q / 2; ++c) centre_pair(y[2 * c], y[Q - 1 - 2 * c], ldtw(T.tc, (Q + 2 * c) / 2));
                inv(y, 1);
#pragma unroll
                for (int c = 0; c < Q; ++c) z.st(Q + c, y[c]);
            }
            continue;
        }
        const u32 j = w + (1u << (31 - __clz(w)));
        const u32 jp = (3u << (31 - __clz(j))) - 1u - j;
#pragma unroll
        for (int c = 0; c < Q; ++c) { x[c] = z.ld(Q * j + c); y[c] = z.ld(Q * jp + c); }
        fwd(x, j);
        fwd(y, jp);
#pragma unroll
        for (int c = 0; c < Q / 2; ++c) {
            centre_pair(x[2 * c], y[Q - 1 - 2 * c], ldtw(T.tc, (Q * j + 2 * c) / 2));
            centre_pair(y[2 * c], x[Q - 1 - 2 * c], ldtw(T.tc, (Q * jp + 2 * c) / 2));
        }
        inv(x, j);
        inv(y, jp);
#pragma unroll
        for (int c = 0; c < Q; ++c) { z.st(Q * j + c, x[c]); z.st(Q * jp + c, y[c]); }
    }
}

template <bool FUSE>
__device__ __forceinline__ void run_small(const SmallTest& T, u32 h, u32 iters, unsigned char* smem) {
    const SZ z = make_sz(smem, h);
    i64* cx = reinterpret_cast<i64*>(smem + 24ull * h);
    const u32 tid = threadIdx.x, nt = blockDim.x;
    const u64 n = 2ull * h;
    const int ln = T.ln;
    const u32 p = T.p;
    const int L = ln - 1;
    const bool odd = (L & 1) != 0;
    constexpr bool fuse = FUSE;
    u32 s4max = 0;
    for (u32 S = 1; 4 * S <= h; S *= 4) s4max = S;

    for (u32 k = tid; k < h; k += nt) { z.A(k) = (u64)T.digits[2 * k]; z.Bv(k) = (u64)T.digits[2 * k + 1]; }
    __syncthreads();

    for (u32 it = 0; it < iters; ++it) {
        for (u32 k = tid; k < h; k += nt) {
            const i64 d0 = (i64)z.A(k), d1 = (i64)z.Bv(k);
            z.st(k, weigh(d0, d1, T.w61[2 * k], T.w61[2 * k + 1], T.w31[2 * k], T.w31[2 * k + 1]));
        }
        __syncthreads();
        // forward radix-4 steps, S blocks of M = h/S (with the fused middle, the
        // last step of an even log2 h runs there)
        const u32 s4last = (fuse && !odd) ? s4max / 4 : s4max;
        for (u32 S = 1; S <= s4last && s4last; S *= 4) {
            // h, S and Q are powers of two: block and offset by shift and mask
            const u32 lq = (u32)L - (31u - __clz(S)) - 2u, Q = 1u << lq, M = Q << 2;
            for (u32 b = tid; b < h / 4; b += nt) {
                const u32 j = b >> lq, i = b & (Q - 1u), base = j * M + i;
                E x0 = z.ld(base), x1 = z.ld(base + Q), x2 = z.ld(base + 2 * Q), x3 = z.ld(base + 3 * Q);
                const u32 ti = 3 * (S + j);
                if (S == 1) dif4_1(x0, x1, x2, x3);   // the first level: root 1
                else dif4(x0, x1, x2, x3, ldtw(T.tw4, ti), ldtw(T.tw4, ti + 1), ldtw(T.tw4, ti + 2));
                z.st(base, x0); z.st(base + Q, x1); z.st(base + 2 * Q, x2); z.st(base + 3 * Q, x3);
            }
            __syncthreads();
        }
        if (fuse) {
            if (odd) fused_middle<2>(z, T, h, s4max);
            else fused_middle<4>(z, T, h, s4max);
            __syncthreads();
        }
        if (odd && !fuse) {
            for (u32 b = tid; b < h / 2; b += nt) {
                E x0 = z.ld(2 * b), x1 = z.ld(2 * b + 1);
                dif2(x0, x1, ldtw(T.tc, b));
                z.st(2 * b, x0); z.st(2 * b + 1, x1);
            }
            __syncthreads();
        }
        // centre: even position k with its mirror 3*2^e - k - 1
        for (u32 b = tid; b < h / 2 && !fuse; b += nt) {
            const u32 k = 2 * b;
            if (k == 0) {
                E z0 = z.ld(0), z1 = z.ld(1);
                centre_zero(z0, z1);
                z.st(0, z0); z.st(1, z1);
            } else {
                const u32 e = 31u - __clz(k);
                const u32 mk = (3u << e) - k - 1u;
                E zk = z.ld(k), zm = z.ld(mk);
                centre_pair(zk, zm, ldtw(T.tc, b));
                z.st(k, zk); z.st(mk, zm);
            }
        }
        if (!fuse) __syncthreads();
        if (odd && !fuse) {
            for (u32 b = tid; b < h / 2; b += nt) {
                E x0 = z.ld(2 * b), x1 = z.ld(2 * b + 1);
                dit2(x0, x1, ldtw(T.tc, b));
                z.st(2 * b, x0); z.st(2 * b + 1, x1);
            }
            __syncthreads();
        }
        for (u32 S = s4last; S >= 1 && s4last; S /= 4) {
            const u32 lq = (u32)L - (31u - __clz(S)) - 2u, Q = 1u << lq, M = Q << 2;
            for (u32 b = tid; b < h / 4; b += nt) {
                const u32 j = b >> lq, i = b & (Q - 1u), base = j * M + i;
                E x0 = z.ld(base), x1 = z.ld(base + Q), x2 = z.ld(base + 2 * Q), x3 = z.ld(base + 3 * Q);
                const u32 ti = 3 * (S + j);
                if (S == 1) dit4_1(x0, x1, x2, x3);
                else dit4(x0, x1, x2, x3, ldtw(T.tw4, ti), ldtw(T.tw4, ti + 1), ldtw(T.tw4, ti + 2));
                z.st(base, x0); z.st(base + Q, x1); z.st(base + 2 * Q, x2); z.st(base + 3 * Q, x3);
            }
            __syncthreads();
            if (S == 1) break;
        }
        // unweight, CRT, carry
        const int Tc = T.carry_threads;
        if (Tc == 0) {
            // tiny exponents: one thread, full normalization with wrap-around
            if (tid == 0) {
                i128 c = 0;
                for (u32 k = 0; k < h; ++k) {
                    i128 z0, z1;
                    unweigh_crt(z.ld(k), 2ull * k, T.w61, T.w31, ln, T.mode, T.gf61_only, z0, z1);
                    if (T.mode == LL && k == 0) z0 -= 2;
                    const i64 d0 = split_balanced(z0 + c, width_of(p, ln, 2ull * k), c);
                    const i64 d1 = split_balanced(z1 + c, width_of(p, ln, 2ull * k + 1), c);
                    z.A(k) = (u64)d0; z.Bv(k) = (u64)d1;
                }
                int pass = 0;
                while (c != 0 && pass < 8) {
                    for (u64 j = 0; j < n && c != 0; ++j) {
                        u64* slot = (j & 1) ? &z.Bv((u32)(j >> 1)) : &z.A((u32)(j >> 1));
                        *slot = (u64)split_balanced((i128)(i64)*slot + c, width_of(p, ln, j), c);
                    }
                    ++pass;
                }
                if (c != 0) atomicExch(T.status, ST_NORMALIZE);
            }
            __syncthreads();
        } else {
            const u32 D = (u32)(n / (u64)Tc);
            if (tid < (u32)Tc) {
                // the 64-bit two-word CRT and carry step (the column passes'):
                // a carry that would leave 64 bits flags the state
                i64 c = 0;
                u32 bad = 0;
                const u64 j0 = (u64)tid * D;
                const u32 mul = (T.mode == PRP3) ? 3u : 1u;
                const bool g61 = !kDual || T.gf61_only;
                for (u32 u = 0; u < D; u += 2) {
                    const u32 k = (u32)((j0 + u) >> 1);
                    const u64 j = 2ull * k;
                    const E v = z.ld(k);
                    const u64 x0 = rotl61(fold61(v.a), unrot61(T.w61[j], ln)), x1 = rotl61(fold61(v.b), unrot61(T.w61[j + 1], ln));
                    const u32 y0 = g61 ? 0u : rotl31(v.c, unrot31(T.w31[j], ln));
                    const u32 y1 = g61 ? 0u : rotl31(v.d, unrot31(T.w31[j + 1], ln));
                    const i64 sub = (T.mode == LL && j == 0) ? 2 : 0;
                    const i64 d0 = crt_digit(x0, y0, width_of(p, ln, j), mul, sub, c, bad, g61);
                    const i64 d1 = crt_digit(x1, y1, width_of(p, ln, j + 1), mul, 0, c, bad, g61);
                    z.A(k) = (u64)d0; z.Bv(k) = (u64)d1;
                }
                if (bad) atomicExch(T.status, ST_CARRY_RANGE);
                cx[tid] = c;
            }
            __syncthreads();
            if (tid < (u32)Tc) {
                i64 c = cx[tid ? tid - 1u : (u32)Tc - 1u];
                const u64 j0 = (u64)tid * D;
                for (int u = 0; u <= T.span; ++u) {
                    const u64 j = j0 + (u64)u;
                    u64* slot = (j & 1) ? &z.Bv((u32)(j >> 1)) : &z.A((u32)(j >> 1));
                    if (u < T.span) *slot = (u64)split_balanced64((i64)*slot + c, width_of(p, ln, j), c);
                    else *slot = (u64)((i64)*slot + c);
                }
            }
            __syncthreads();
        }
    }
    for (u32 k = tid; k < h; k += nt) { T.digits[2 * k] = (i64)z.A(k); T.digits[2 * k + 1] = (i64)z.Bv(k); }
}

// One CTA per test (queue == nullptr), or a persistent grid whose CTAs take
// test indices from *queue until all `ntests` are done.
// FUSE: the transform's middle as one pass (the tests' fuse_middle); a
// separate instantiation, so that each variant gets its own register budget
template <bool FUSE>
__global__ void __launch_bounds__(256, 2) k_small(const SmallTest* tests, int ntests, u32 h, u32 iters_override, int* queue) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_next;
    if (queue == nullptr) {
        const SmallTest T = tests[blockIdx.x];
        run_small<FUSE>(T, h, iters_override ? iters_override : T.iters, smem);
        return;
    }
    for (;;) {
        if (threadIdx.x == 0) s_next = atomicAdd(queue, 1);
        __syncthreads();
        const int idx = s_next;
        __syncthreads();
        if (idx >= ntests) break;
        const SmallTest T = tests[idx];
        run_small<FUSE>(T, h, iters_override ? iters_override : T.iters, smem);
        __syncthreads();
    }
}

// Largest dynamic shared memory a CTA of `func` may request on the current
// device: the opt-in maximum less the kernel's static shared memory.  The
// kernels' limits are set to this rather than to one plan's size: the
// attribute belongs to the kernel, and contexts of different sizes share it.
int dyn_smem_limit(const void* func) {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa{};
    if (cudaFuncGetAttributes(&fa, func) == cudaSuccess) v -= (int)fa.sharedSizeBytes;
    return v > 0 ? v : 48 * 1024;
}

int small_threads_for(unsigned int h) {
    unsigned int t = h / 4;
    if (t < 32) t = 32;
    if (t > 256) t = 256;
    return (int)t;
}
size_t small_smem_bytes(unsigned int h, int threads) { return 24ull * h + 8ull * (size_t)threads; }

namespace {
const void* small_fn(bool fuse) { return fuse ? (const void*)k_small<true> : (const void*)k_small<false>; }
}  // namespace

cudaError_t launch_small(const SmallTest* d_tests, int ntests, unsigned int h, int threads, unsigned int iters_override,
                         cudaStream_t s, bool fuse, bool gf61) {
#if M2_DUAL
    if (gf61) return m2k_g61::launch_small(d_tests, ntests, h, threads, iters_override, s, fuse, true);
#endif
    const size_t sm = small_smem_bytes(h, threads);
    cudaError_t e = cudaFuncSetAttribute(small_fn(fuse), cudaFuncAttributeMaxDynamicSharedMemorySize, dyn_smem_limit(small_fn(fuse)));
    if (e != cudaSuccess) return e;
    if (fuse) k_small<true><<<ntests, threads, sm, s>>>(d_tests, ntests, h, iters_override, nullptr);
    else k_small<false><<<ntests, threads, sm, s>>>(d_tests, ntests, h, iters_override, nullptr);
    return cudaGetLastError();
}

cudaError_t launch_small_persistent(const SmallTest* d_tests, int ntests, unsigned int h, int threads, int* d_queue,
                                    int grid, cudaStream_t s, bool fuse) {
    const size_t sm = small_smem_bytes(h, threads);
    cudaError_t e = cudaFuncSetAttribute(small_fn(fuse), cudaFuncAttributeMaxDynamicSharedMemorySize, dyn_smem_limit(small_fn(fuse)));
    if (e != cudaSuccess) return e;
    if (fuse) k_small<true><<<grid, threads, sm, s>>>(d_tests, ntests, h, 0u, d_queue);
    else k_small<false><<<grid, threads, sm, s>>>(d_tests, ntests, h, 0u, d_queue);
    return cudaGetLastError();
}

int small_ctas_per_sm(unsigned int h, int threads, bool fuse) {
    int nb = 0;
    const size_t sm = small_smem_bytes(h, threads);
    if (cudaFuncSetAttribute(small_fn(fuse), cudaFuncAttributeMaxDynamicSharedMemorySize, dyn_smem_limit(small_fn(fuse))) != cudaSuccess) return 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, small_fn(fuse), threads, sm) != cudaSuccess) return 1;
    return nb > 0 ? nb : 1;
}

// =====================================================================
// three-pass path
// =====================================================================
constexpr int LT = 256;   // threads per CTA of the row kernel
constexpr int LTC = 512;  // threads per CTA of the column kernels

template <int C>
__global__ void __launch_bounds__(LTC, 2) k_cols_fwd(LargePlan P, LargeBufs bf) {
    extern __shared__ __align__(16) unsigned char smem[];
    const u32 R = P.R, B = P.B, G = P.G, g = blockIdx.x;
    const u32 NE = (u32)C * R;
    const SE z = make_se(smem, NE);
    const u64 RG = (u64)R * G;
    const u32 p = P.p;
    const int ln = P.ln;
    for (u32 t = threadIdx.x; t < R; t += blockDim.x) {
        const u64 s = (u64)t * G + g;
        i64 c = bf.carries[s ? s - 1 : RG - 1];   // the segment before (the last one for segment 0)
        const u64 e0 = (u64)t * B + (u64)g * C;
        const u64 j0 = 2 * e0;
        i64 d[2 * C];
#pragma unroll
        for (int u = 0; u < 2 * C; ++u) d[u] = bf.digits[j0 + u];
#pragma unroll
        for (int u = 0; u < 2 * C; ++u) {
            if (u < P.span) d[u] = split_balanced64(d[u] + c, width_of(p, ln, j0 + u), c);
            else if (u == P.span) d[u] += c;
        }
#pragma unroll
        for (int cc = 0; cc < C; ++cc) {
            const u64 j = j0 + 2 * cc;
            z.st(t * C + cc, weigh(d[2 * cc], d[2 * cc + 1], bf.w61[j], bf.w61[j + 1], bf.w31[j], bf.w31[j + 1]));
        }
    }
    __syncthreads();
    for (u32 S = 1; S < R; S *= 4) {
        // R, S and Q are powers of two: block and offset by shift and mask
        const u32 M = R / S, Q = M >> 2, lq = 31u - __clz(Q);
        for (u32 b = threadIdx.x; b < NE / 4; b += blockDim.x) {
            const u32 cc = b % C, rho = b / C, j = rho >> lq, i = rho & (Q - 1u);
            const u32 r0 = j * M + i;
            const u32 i0 = r0 * C + cc, i1 = (r0 + Q) * C + cc, i2 = (r0 + 2 * Q) * C + cc, i3 = (r0 + 3 * Q) * C + cc;
            E x0 = z.ld(i0), x1 = z.ld(i1), x2 = z.ld(i2), x3 = z.ld(i3);
            const u32 ti = 3 * (S + j);
            if (S == 1) dif4_1(x0, x1, x2, x3);   // the first level: root 1
            else dif4(x0, x1, x2, x3, ldtw(bf.tw4, ti), ldtw(bf.tw4, ti + 1), ldtw(bf.tw4, ti + 2));
            z.st(i0, x0); z.st(i1, x1); z.st(i2, x2); z.st(i3, x3);
        }
        __syncthreads();
    }
    for (u32 l = threadIdx.x; l < NE; l += blockDim.x) {
        const u32 t = l / C, cc = l % C;
        const u64 e = (u64)t * B + (u64)g * C + cc;
        const E v = z.ld(l);
        bf.za[e] = make_ulonglong2(v.a, v.b);
        if (kDual) bf.zb[e] = make_uint2(v.c, v.d);
    }
}

__global__ void __launch_bounds__(LT, 4) k_rows(LargePlan P, LargeBufs bf) {
    extern __shared__ __align__(16) unsigned char smem[];
    const u32 B = P.B, NE = 2 * B, lb = 31u - __clz(B);   // B is a power of two
    const SE z = make_se(smem, NE);
    const u32 pi = blockIdx.x;
    u32 t0, t1;
    if (pi == 0) { t0 = 0; t1 = 1; }
    else {
        const u32 e = 32u - __clz(pi);                 // floor(log2 pi) + 1
        const u32 a = pi - (1u << (e - 1));
        t0 = (1u << e) + a;
        t1 = (2u << e) - 1u - a;
    }
    for (u32 l = threadIdx.x; l < NE; l += blockDim.x) {
        const u32 sl = l >> lb, col = l & (B - 1u);
        const u64 e = (u64)(sl ? t1 : t0) * B + col;
        const ulonglong2 va = bf.za[e];
        const uint2 vb = kDual ? bf.zb[e] : make_uint2(0u, 0u);
        z.st(l, E{va.x, va.y, vb.x, vb.y});
    }
    __syncthreads();
    // B, per4, Mloc and Q are powers of two: shifts and masks
    const u32 per4 = B / 4, lp4 = 31u - __clz(per4);
    u32 S = P.R, Mloc = B;
    for (; Mloc >= 4; S *= 4, Mloc /= 4) {
        const u32 Q = Mloc >> 2, nb = B / Mloc, lq = 31u - __clz(Q);
        for (u32 b = threadIdx.x; b < 2 * per4; b += blockDim.x) {
            const u32 sl = b >> lp4, rho = b & (per4 - 1u), j = rho >> lq, i = rho & (Q - 1u);
            const u32 base = sl * B + j * Mloc + i;
            const u32 J = (sl ? t1 : t0) * nb + j;
            E x0 = z.ld(base), x1 = z.ld(base + Q), x2 = z.ld(base + 2 * Q), x3 = z.ld(base + 3 * Q);
            const u64 ti = 3ull * ((u64)S + J);
            dif4(x0, x1, x2, x3, ldtw(bf.tw4, (u32)ti), ldtw(bf.tw4, (u32)ti + 1), ldtw(bf.tw4, (u32)ti + 2));
            z.st(base, x0); z.st(base + Q, x1); z.st(base + 2 * Q, x2); z.st(base + 3 * Q, x3);
        }
        __syncthreads();
    }
    const bool odd = (Mloc == 2);
    const u32 per2 = B / 2;
    if (odd) {
        for (u32 b = threadIdx.x; b < 2 * per2; b += blockDim.x) {
            const u32 sl = b / per2, rho = b % per2, base = sl * B + 2 * rho;
            const u32 J = (sl ? t1 : t0) * per2 + rho;
            E x0 = z.ld(base), x1 = z.ld(base + 1);
            dif2(x0, x1, ldtw(bf.tc, J));
            z.st(base, x0); z.st(base + 1, x1);
        }
        __syncthreads();
    }
    // centre
    for (u32 b = threadIdx.x; b < B; b += blockDim.x) {
        const u32 sl = b / per2, i = 2 * (b % per2);
        const u64 k = (u64)(sl ? t1 : t0) * B + i;
        const u32 li = sl * B + i;
        if (pi == 0) {
            if (k == 0) {
                E a0 = z.ld(0), a1 = z.ld(1);
                centre_zero(a0, a1);
                z.st(0, a0); z.st(1, a1);
            } else {
                const u32 e = 63u - (u32)__clzll((long long)k);
                const u64 mk = (3ull << e) - k - 1ull;
                const u32 lm = sl * B + (u32)(mk % B);
                E zk = z.ld(li), zm = z.ld(lm);
                centre_pair(zk, zm, ldtw(bf.tc, (u32)(k >> 1)));
                z.st(li, zk); z.st(lm, zm);
            }
        } else {
            const u32 lm = (1u - sl) * B + (B - 1u - i);
            E zk = z.ld(li), zm = z.ld(lm);
            centre_pair(zk, zm, ldtw(bf.tc, (u32)(k >> 1)));
            z.st(li, zk); z.st(lm, zm);
        }
    }
    __syncthreads();
    if (odd) {
        for (u32 b = threadIdx.x; b < 2 * per2; b += blockDim.x) {
            const u32 sl = b / per2, rho = b % per2, base = sl * B + 2 * rho;
            const u32 J = (sl ? t1 : t0) * per2 + rho;
            E x0 = z.ld(base), x1 = z.ld(base + 1);
            dit2(x0, x1, ldtw(bf.tc, J));
            z.st(base, x0); z.st(base + 1, x1);
        }
        __syncthreads();
    }
    // inverse radix-4 steps in reverse order
    for (S /= 4, Mloc = odd ? 8 : 4; Mloc <= B && S >= P.R; S /= 4, Mloc *= 4) {
        const u32 Q = Mloc >> 2, nb = B / Mloc, lq = 31u - __clz(Q);
        for (u32 b = threadIdx.x; b < 2 * per4; b += blockDim.x) {
            const u32 sl = b >> lp4, rho = b & (per4 - 1u), j = rho >> lq, i = rho & (Q - 1u);
            const u32 base = sl * B + j * Mloc + i;
            const u32 J = (sl ? t1 : t0) * nb + j;
            E x0 = z.ld(base), x1 = z.ld(base + Q), x2 = z.ld(base + 2 * Q), x3 = z.ld(base + 3 * Q);
            const u64 ti = 3ull * ((u64)S + J);
            dit4(x0, x1, x2, x3, ldtw(bf.tw4, (u32)ti), ldtw(bf.tw4, (u32)ti + 1), ldtw(bf.tw4, (u32)ti + 2));
            z.st(base, x0); z.st(base + Q, x1); z.st(base + 2 * Q, x2); z.st(base + 3 * Q, x3);
        }
        __syncthreads();
        if (S == P.R) break;
    }
    for (u32 l = threadIdx.x; l < NE; l += blockDim.x) {
        const u32 sl = l >> lb, col = l & (B - 1u);
        const u64 e = (u64)(sl ? t1 : t0) * B + col;
        const E v = z.ld(l);
        bf.za[e] = make_ulonglong2(v.a, v.b);
        if (kDual) bf.zb[e] = make_uint2(v.c, v.d);
    }
}

template <int C>
__global__ void __launch_bounds__(LTC, 2) k_cols_inv(LargePlan P, LargeBufs bf) {
    extern __shared__ __align__(16) unsigned char smem[];
    const u32 R = P.R, B = P.B, G = P.G, g = blockIdx.x;
    const u32 NE = (u32)C * R;
    const SE z = make_se(smem, NE);
    const u32 p = P.p;
    const int ln = P.ln;
    for (u32 l = threadIdx.x; l < NE; l += blockDim.x) {
        const u32 t = l / C, cc = l % C;
        const u64 e = (u64)t * B + (u64)g * C + cc;
        const ulonglong2 va = bf.za[e];
        const uint2 vb = kDual ? bf.zb[e] : make_uint2(0u, 0u);
        z.st(l, E{va.x, va.y, vb.x, vb.y});
    }
    __syncthreads();
    for (u32 S = R / 4; S >= 1; S /= 4) {
        const u32 M = R / S, Q = M >> 2, lq = 31u - __clz(Q);
        for (u32 b = threadIdx.x; b < NE / 4; b += blockDim.x) {
            const u32 cc = b % C, rho = b / C, j = rho >> lq, i = rho & (Q - 1u);
            const u32 r0 = j * M + i;
            const u32 i0 = r0 * C + cc, i1 = (r0 + Q) * C + cc, i2 = (r0 + 2 * Q) * C + cc, i3 = (r0 + 3 * Q) * C + cc;
            E x0 = z.ld(i0), x1 = z.ld(i1), x2 = z.ld(i2), x3 = z.ld(i3);
            const u32 ti = 3 * (S + j);
            if (S == 1) dit4_1(x0, x1, x2, x3);
            else dit4(x0, x1, x2, x3, ldtw(bf.tw4, ti), ldtw(bf.tw4, ti + 1), ldtw(bf.tw4, ti + 2));
            z.st(i0, x0); z.st(i1, x1); z.st(i2, x2); z.st(i3, x3);
        }
        __syncthreads();
        if (S == 1) break;
    }
    // unweight, CRT and carry over the row segment (the 64-bit step of the
    // quad-shuffle column passes; a carry that would leave 64 bits flags the state)
    const u32 mul = (P.mode == PRP3) ? 3u : 1u;
    const bool g61 = !kDual || P.gf61 != 0;
    for (u32 t = threadIdx.x; t < R; t += blockDim.x) {
        const u64 e0 = (u64)t * B + (u64)g * C;
        i64 c = 0;
        u32 bad = 0;
#pragma unroll
        for (int cc = 0; cc < C; ++cc) {
            const u64 e = e0 + cc, j = 2 * e;
            const E v = z.ld(t * C + cc);
            const u64 x0 = rotl61(fold61(v.a), unrot61(bf.w61[j], ln)), x1 = rotl61(fold61(v.b), unrot61(bf.w61[j + 1], ln));
            const u32 y0 = g61 ? 0u : rotl31(v.c, unrot31(bf.w31[j], ln));
            const u32 y1 = g61 ? 0u : rotl31(v.d, unrot31(bf.w31[j + 1], ln));
            bf.digits[j] = crt_digit(x0, y0, width_of(p, ln, j), mul, (P.mode == LL && e == 0) ? 2 : 0, c, bad, g61);
            bf.digits[j + 1] = crt_digit(x1, y1, width_of(p, ln, j + 1), mul, 0, c, bad, g61);
        }
        if (bad) atomicExch(bf.status, ST_CARRY_RANGE);
        bf.carries[(u64)t * G + g] = c;
    }
}

size_t large_smem_cols(const LargePlan& P) { return 24ull * P.C * P.R; }
size_t large_smem_rows(const LargePlan& P) { return 24ull * 2 * P.B; }

#define M2_FOR_C(X) X(4) X(8) X(16)

cudaError_t large_setup(const LargePlan& P) {
#if M2_DUAL
    if (P.gf61) return m2k_g61::large_setup(P);
#endif
    cudaError_t e;
#define M2_SET(CC)                                                                                          \
    if (P.C == CC) {                                                                                        \
        if ((e = cudaFuncSetAttribute(k_cols_fwd<CC>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn_smem_limit((const void*)k_cols_fwd<CC>)))) return e; \
        if ((e = cudaFuncSetAttribute(k_cols_inv<CC>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn_smem_limit((const void*)k_cols_inv<CC>)))) return e; \
        if ((e = cudaFuncSetAttribute(k_cols_fwd<CC>, cudaFuncAttributePreferredSharedMemoryCarveout, 100))) return e; \
        if ((e = cudaFuncSetAttribute(k_cols_inv<CC>, cudaFuncAttributePreferredSharedMemoryCarveout, 100))) return e; \
    }
    M2_FOR_C(M2_SET)
#undef M2_SET
    if (rows_q_supported(P) && (e = rows_q_setup(P))) return e;
    if (cols_q_supported(P) && (e = cols_q_setup(P))) return e;
    if ((e = cudaFuncSetAttribute(k_rows, cudaFuncAttributePreferredSharedMemoryCarveout, 100))) return e;
    return cudaFuncSetAttribute(k_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn_smem_limit((const void*)k_rows));
}

cudaError_t launch_large_stage(const LargePlan& P, const LargeBufs& b, int stage, cudaStream_t s) {
#if M2_DUAL
    if (P.gf61) return m2k_g61::launch_large_stage(P, b, stage, s);
#endif
    const size_t sc = large_smem_cols(P), sr = large_smem_rows(P);
    if (stage == STAGE_MID) return b.flags ? launch_cols_mid(P, b, s) : cudaErrorInvalidValue;
    if (stage != 1 && cols_q_supported(P)) return launch_cols_q(P, b, stage == 2, s);
    if (stage == 0) {
#define M2_FWD(CC) if (P.C == CC) k_cols_fwd<CC><<<P.G, LTC, sc, s>>>(P, b);
        M2_FOR_C(M2_FWD)
#undef M2_FWD
    } else if (stage == 1) {
        if (rows_q_supported(P)) return launch_rows_q(P, b, s);
        k_rows<<<P.R / 2, LT, sr, s>>>(P, b);
    } else {
#define M2_INV(CC) if (P.C == CC) k_cols_inv<CC><<<P.G, LTC, sc, s>>>(P, b);
        M2_FOR_C(M2_INV)
#undef M2_INV
    }
    return cudaGetLastError();
}

const char* large_stage_name(int stage) {
    static const char* names[] = {"k_cols_fwd", "k_rows", "k_cols_inv", "k_cols_mid"};
    return (stage >= 0 && stage < 4) ? names[stage] : "?";
}

// Algorithmic bytes of one launch: what the stage must read and write at least.
unsigned long long large_stage_bytes(const LargePlan& P, int stage) {
    const unsigned long long h = (unsigned long long)P.R * P.B;
    const unsigned long long carries = 8ull * P.R * P.G;
    if (stage == 0) return 16ull * h + carries + 24ull * h;   // digits + carries in, dual elements out
    if (stage == 1) return 48ull * h;                          // dual elements in and out
    if (stage == STAGE_MID) return 48ull * h + 2 * carries;    // dual elements in and out, carries out and in
    return 24ull * h + 16ull * h + carries;                    // dual elements in, digits + carries out
}

cudaError_t launch_large_iteration(const LargePlan& P, const LargeBufs& b, cudaStream_t s) {
#if M2_DUAL
    if (P.gf61) return m2k_g61::launch_large_iteration(P, b, s);
#endif
    for (int st = 0; st < LARGE_STAGES; ++st) {
        cudaError_t e = launch_large_stage(P, b, st, s);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_large_run(const LargePlan& P, const LargeBufs& b, unsigned k, bool fused, cudaStream_t s) {
#if M2_DUAL
    if (P.gf61) return m2k_g61::launch_large_run(P, b, k, fused, s);
#endif
    cudaError_t e = cudaSuccess;
    if (k == 0) return e;
    if (!fused) {
        for (unsigned i = 0; i < k && e == cudaSuccess; ++i) e = launch_large_iteration(P, b, s);
        return e;
    }
    if ((e = launch_large_stage(P, b, 0, s)) || (e = launch_large_stage(P, b, 1, s))) return e;
    for (unsigned i = 1; i < k; ++i)
        if ((e = launch_large_stage(P, b, STAGE_MID, s)) || (e = launch_large_stage(P, b, 1, s))) return e;
    return launch_large_stage(P, b, 2, s);
}

}  // namespace M2K_NS
