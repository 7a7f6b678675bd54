// m2_carry.cu -- full carry propagation on the device: relaxed signed digits
// (plus pending segment carries) -> canonical digits of the residue mod 2^p - 1.
//
// The reference resolves carries with a block-carry scheme whose last phase is
// a single work-item loop over all blocks, the top carry re-entering digit 0
// because 2^p == 1 (mersenne2_gpu.cpp:2097-2123, 2922-3004); the prototype
// kernels of gf61_ntt_prp_opencl_inplace_nobitrev_fused_powonly_blockcarry.cl
// use a summary / look-ahead carry instead.  Here the propagation is a
// parallel carry-lookahead in three launches, with no inter-CTA waiting:
//
//   k_norm_blocks  every thread owns a chunk of 8 digits and summarises it as
//                  a transfer function carry_in -> carry_out (below); a CTA
//                  scans its 256 summaries and stores the composite of its
//                  2048 digits;
//   k_norm_scan    one CTA scans the block composites, solves the wrap-around
//                  (the carry into digit 0 is the carry out of the top digit)
//                  by fixed-point iteration, and stores every block's carry-in;
//   k_norm_apply   recomputes the in-block scan, propagates each chunk with its
//                  exact carry-in and writes canonical digits.  Every chunk
//                  checks that its exact carry-out equals the carry-in assigned
//                  to the next chunk (the top one against digit 0), so a state
//                  outside the summaries' range is reported, never mis-carried.
//   k_norm_ones    the all-ones vector (== M_p) becomes zero.
//
// Transfer function of a chunk for a small carry-in c (|c| < 2^w0): with the
// chunk propagated from carry-in 0 giving digits o_j and carry-out C0, adding
// c changes digit 0's carry by r = floor((o_0 + c) / 2^w0) in {-1, 0, 1}; the
// change ripples to the chunk's carry-out only through digits that are all
// 2^w - 1 (r = 1) or all 0 (r = -1).  So carry_out(c) = out[1 + R(c)] with
// R(c) in {-1, 0, 1} decided by (o_0, w0, rest-all-max, rest-all-zero) and
// out[k] = C0 + (k - 1).  A range of chunks has the same form: the descriptor
// of its first chunk and the range's carry-out for each ripple of that chunk;
// composing ranges maps each out[] entry through the next range.
#include <cuda_runtime.h>

#include <cstdint>

#include "m2_kernels.cuh"

namespace m2k {

typedef long long i64;
typedef unsigned long long u64;
typedef unsigned int u32;

struct NormSum {
    i64 out[3];                  // carry-out for a first-chunk ripple of -1, 0, +1
    u64 o0;                      // first digit of the first chunk, from carry-in 0
    u32 w0;                      // its width
    u32 flags;                   // bit 0: rest of the first chunk all max; bit 1: all zero
};

namespace {

constexpr int NT = 256;          // threads per CTA of the block kernels
constexpr int CH = 8;            // digits per chunk
constexpr int BD = NT * CH;      // digits per block
constexpr int ST = 1024;         // threads of the scan CTA

typedef NormSum Sum;

__device__ __forceinline__ u64 bitpos(u64 p, int ln, u64 j) { return (p * j + (1ull << ln) - 1) >> ln; }

// ripple of the first chunk for carry-in c; 2 = out of the summarised range
__device__ __forceinline__ int ripple(const Sum& s, i64 c) {
    if (c == 0) return 0;
    const i64 lim = (s.w0 >= 62) ? (i64(1) << 62) : (i64(1) << s.w0);
    if (c >= lim || c <= -lim) return 2;
    if (c > 0) return ((i64)s.o0 + c >= lim && (s.flags & 1u)) ? 1 : 0;
    return ((i64)s.o0 + c < 0 && (s.flags & 2u)) ? -1 : 0;
}

constexpr i64 BAD = (i64)0x7fffffffffffffffll;   // marks an out-of-range composite entry

__device__ __forceinline__ i64 eval(const Sum& s, i64 c) {
    if (c == BAD) return BAD;
    const int r = ripple(s, c);
    return r == 2 ? BAD : s.out[r + 1];
}

// a then b
__device__ __forceinline__ Sum combine(const Sum& a, const Sum& b) {
    Sum r = a;
    for (int k = 0; k < 3; ++k) r.out[k] = eval(b, a.out[k]);
    return r;
}

__device__ __forceinline__ Sum identity_sum() {
    // carry passes through unchanged: a zero-width "digit" with both flags
    Sum s;
    s.out[0] = BAD; s.out[1] = BAD; s.out[2] = BAD;
    s.o0 = 0; s.w0 = 0; s.flags = 0xffu;
    return s;
}
__device__ __forceinline__ bool is_identity(const Sum& s) { return s.flags == 0xffu; }
__device__ __forceinline__ Sum comb(const Sum& a, const Sum& b) {
    if (is_identity(a)) return b;
    if (is_identity(b)) return a;
    return combine(a, b);
}
__device__ __forceinline__ i64 apply(const Sum& s, i64 c) { return is_identity(s) ? c : eval(s, c); }

__device__ __forceinline__ Sum shfl_up_sum(const Sum& s, int d) {
    Sum r;
    for (int k = 0; k < 3; ++k) r.out[k] = __shfl_up_sync(0xffffffffu, s.out[k], d);
    r.o0 = __shfl_up_sync(0xffffffffu, s.o0, d);
    r.w0 = __shfl_up_sync(0xffffffffu, s.w0, d);
    r.flags = __shfl_up_sync(0xffffffffu, s.flags, d);
    return r;
}

// input word of digit j: the digit plus the pending carry of the segment before
// it (segment carries enter at the first digit of the following segment)
__device__ __forceinline__ i64 input_word(const NormArgs& a, u64 j) {
    i64 t = a.digits[j];
    if (a.carries && (j % a.seg) == 0) {
        const u64 s = j / a.seg, ns = a.n / a.seg;
        t += a.carries[(s + ns - 1) % ns];
    }
    return t;
}

// the chunk of digits [j0, j0 + CH): its summary
__device__ Sum chunk_sum(const NormArgs& a, u64 j0) {
    Sum s;
    i64 c = 0;
    u32 allmax = 1, allzero = 1;
    u64 b = bitpos(a.p, a.ln, j0);
    for (int k = 0; k < CH; ++k) {
        const u64 b1 = bitpos(a.p, a.ln, j0 + k + 1);
        const u32 w = (u32)(b1 - b);
        b = b1;
        const i64 v = input_word(a, j0 + k) + c;
        const u64 o = (u64)v & ((1ull << w) - 1);
        c = v >> w;
        if (k == 0) { s.o0 = o; s.w0 = w; }
        else { allmax &= (u32)(o == (1ull << w) - 1); allzero &= (u32)(o == 0); }
    }
    s.out[0] = c - 1; s.out[1] = c; s.out[2] = c + 1;
    s.flags = allmax | (allzero << 1);
    return s;
}

// inclusive scan of one summary per thread over the CTA (NT threads);
// returns the exclusive prefix of this thread, and the CTA total in *total
__device__ Sum cta_scan(Sum s, Sum* sh, Sum* total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    Sum inc = s;
    for (int d = 1; d < 32; d <<= 1) {
        const Sum o = shfl_up_sum(inc, d);
        if (lane >= d) inc = comb(o, inc);
    }
    if (lane == 31) sh[wid] = inc;
    __syncthreads();
    if (threadIdx.x == 0) {
        Sum acc = identity_sum();
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { const Sum t = sh[w]; sh[w] = acc; acc = comb(acc, t); }
        sh[32] = acc;
    }
    __syncthreads();
    Sum ex = shfl_up_sum(inc, 1);
    if (lane == 0) ex = identity_sum();
    ex = comb(sh[wid], ex);
    *total = sh[32];
    return ex;
}

__global__ void __launch_bounds__(NT) k_norm_blocks(NormArgs a) {
    __shared__ Sum sh[33];
    const u64 j0 = ((u64)blockIdx.x * NT + threadIdx.x) * CH;
    const Sum s = (j0 < a.n) ? chunk_sum(a, j0) : identity_sum();
    Sum total;
    cta_scan(s, sh, &total);
    if (threadIdx.x == 0) a.block_sum[blockIdx.x] = total;
}

__global__ void __launch_bounds__(ST) k_norm_scan(NormArgs a, u32 nb) {
    __shared__ Sum sh[33];
    const u32 per = (nb + ST - 1) / ST;
    const u32 b0 = threadIdx.x * per;
    Sum loc = identity_sum();
    for (u32 k = 0; k < per && b0 + k < nb; ++k) loc = comb(loc, a.block_sum[b0 + k]);
    Sum total;
    const Sum ex = cta_scan(loc, sh, &total);
    // the carry into digit 0 is the carry out of the top digit: fixed point
    __shared__ i64 c_top;
    if (threadIdx.x == 0) {
        i64 c = 0;
        int it = 0;
        for (; it < 8; ++it) {
            const i64 nc = apply(total, c);
            if (nc == BAD) { c = BAD; break; }
            if (nc == c) break;
            c = nc;
        }
        if (it == 8 || c == BAD) { atomicOr(a.status, 2); c = 0; }
        c_top = c;
    }
    __syncthreads();
    i64 c = apply(ex, c_top);
    if (c == BAD) { atomicOr(a.status, 2); c = 0; }
    for (u32 k = 0; k < per && b0 + k < nb; ++k) {
        a.block_cin[b0 + k] = c;
        c = apply(a.block_sum[b0 + k], c);
        if (c == BAD) { atomicOr(a.status, 2); c = 0; }
    }
}

__global__ void __launch_bounds__(NT) k_norm_apply(NormArgs a) {
    __shared__ Sum sh[33];
    __shared__ i64 cin_next[NT];
    const u64 j0 = ((u64)blockIdx.x * NT + threadIdx.x) * CH;
    const bool mine = j0 < a.n;
    const Sum s = mine ? chunk_sum(a, j0) : identity_sum();
    Sum total;
    const Sum ex = cta_scan(s, sh, &total);
    i64 c = apply(ex, a.block_cin[blockIdx.x]);
    if (c == BAD) { atomicOr(a.status, 2); c = 0; }
    const i64 my_cin = c;
    u32 ones = 1, high_nonzero = 0;
    if (mine) {
        u64 b = bitpos(a.p, a.ln, j0);
        for (int k = 0; k < CH; ++k) {
            const u64 b1 = bitpos(a.p, a.ln, j0 + k + 1);
            const u32 w = (u32)(b1 - b);
            b = b1;
            const i64 v = input_word(a, j0 + k) + c;
            const u64 o = (u64)v & ((1ull << w) - 1);
            c = v >> w;
            a.out[j0 + k] = o;
            ones &= (u32)(o == (1ull << w) - 1);
            high_nonzero |= (u32)(o != 0 && j0 + k >= CH);
        }
    }
    // consistency: this chunk's exact carry-out is the next chunk's carry-in
    // (the top chunk's is the carry into digit 0)
    cin_next[threadIdx.x] = my_cin;
    __syncthreads();
    if (mine) {
        const u64 jn = j0 + CH;
        i64 want;
        if (jn >= a.n) want = a.block_cin[0];
        else if (threadIdx.x + 1 < NT) want = cin_next[threadIdx.x + 1];
        else want = a.block_cin[blockIdx.x + 1];
        if (c != want) atomicOr(a.status, 2);
    }
    const u32 all_ones = __syncthreads_and(mine ? ones : 1);
    const u32 any_high = __syncthreads_or(high_nonzero);
    if (threadIdx.x == 0) {
        if (!all_ones) atomicAnd(a.flags, ~1u);
        if (any_high) atomicOr(a.flags, 2u);
    }
}

__global__ void k_norm_ones(NormArgs a) {
    if ((*a.flags & 1u) == 0) return;
    for (u64 j = (u64)blockIdx.x * blockDim.x + threadIdx.x; j < a.n; j += (u64)gridDim.x * blockDim.x) a.out[j] = 0;
}

__global__ void k_norm_init(NormArgs a) {
    if (threadIdx.x == 0) *a.flags = 1u;
}

// tiny transforms (n <= 64, or digits of width < 4): one thread, the plain
// sequential propagation repeated until the wrapped carry settles; exact for
// any input words
__global__ void k_norm_tiny(NormArgs a) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    i64 c = 0;
    for (int pass = 0; pass < 66; ++pass) {
        u64 b = 0;
        for (u64 j = 0; j < a.n; ++j) {
            const u64 b1 = bitpos(a.p, a.ln, j + 1);
            const u32 w = (u32)(b1 - b);
            b = b1;
            const i64 t = (pass == 0) ? input_word(a, j) : (i64)a.out[j];
            const i64 v = t + c;
            const u64 o = (w == 0) ? 0 : ((u64)v & ((1ull << w) - 1));
            c = (w == 0) ? v : (v >> w);
            a.out[j] = o;
        }
        if (c == 0) break;
    }
    if (c != 0) atomicOr(a.status, 2);
    u32 ones = 1, high = 0;
    u64 b = 0;
    for (u64 j = 0; j < a.n; ++j) {
        const u64 b1 = bitpos(a.p, a.ln, j + 1);
        const u32 w = (u32)(b1 - b);
        b = b1;
        ones &= (u32)(a.out[j] == ((w == 0) ? 0 : (1ull << w) - 1));
        high |= (u32)(a.out[j] != 0 && j >= CH);
    }
    *a.flags = ones | (high << 1);
}

// canonical digits (each < 2^w) -> balanced relaxed digits with no pending
// carries: a digit >= 2^(w-1) gives 2^w back and a carry of one to the next
// digit (the top digit's to digit 0): every result lies in [-2^(w-1), 2^(w-1)].
// A digit at or above 2^w (not canonical) sets *bad; the caller then loads
// the state another way (the digits written here are not used).
__global__ void k_balance(const u64* canon, i64* digits, u64 p, int ln, u64 n, unsigned* bad) {
    unsigned any = 0;
    for (u64 j = (u64)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (u64)gridDim.x * blockDim.x) {
        const u64 b0 = bitpos(p, ln, j), b1 = bitpos(p, ln, j + 1);
        const u32 w = (u32)(b1 - b0);
        const u64 jp = (j == 0) ? n - 1 : j - 1;
        const u32 wprev = (u32)(bitpos(p, ln, jp + 1) - bitpos(p, ln, jp));
        i64 v = (i64)canon[j];
        any |= (u32)((canon[j] >> w) != 0);   // widths stay below 64
        if (w > 0 && canon[j] >= (1ull << (w - 1))) v -= (i64)1 << w;
        if (wprev > 0 && canon[jp] >= (1ull << (wprev - 1))) v += 1;
        digits[j] = v;
    }
    if (bad && __syncthreads_or(any) && threadIdx.x == 0) atomicOr(bad, 1u);
}

}  // namespace

size_t norm_scratch_bytes(u64 n) {
    const u64 nb = (n + BD - 1) / BD;
    return nb * sizeof(Sum) + (nb + 1) * sizeof(i64) + 64;
}

void norm_bind_scratch(NormArgs& a, void* scratch) {
    const u64 nb = (a.n + BD - 1) / BD;
    char* s = static_cast<char*>(scratch);
    a.block_sum = reinterpret_cast<NormSum*>(s);
    a.block_cin = reinterpret_cast<i64*>(s + nb * sizeof(Sum));
    a.flags = reinterpret_cast<u32*>(s + nb * sizeof(Sum) + (nb + 1) * sizeof(i64));
}

cudaError_t launch_normalize(const NormArgs& a, cudaStream_t s) {
    const u64 nb = (a.n + BD - 1) / BD;
    const u64 q = a.p >> a.ln;
    const unsigned g = (unsigned)((a.n + 255) / 256 < 1024 ? (a.n + 255) / 256 : 1024);
    if (q < 4 || a.n <= 64) {
        k_norm_tiny<<<1, 32, 0, s>>>(a);
        k_norm_ones<<<g, 256, 0, s>>>(a);
        return cudaGetLastError();
    }
    k_norm_init<<<1, 32, 0, s>>>(a);
    k_norm_blocks<<<(unsigned)nb, NT, 0, s>>>(a);
    k_norm_scan<<<1, ST, 0, s>>>(a, (u32)nb);
    k_norm_apply<<<(unsigned)nb, NT, 0, s>>>(a);
    k_norm_ones<<<g, 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_balance(const u64* canon, i64* digits, u64 p, int ln, u64 n, unsigned* bad, cudaStream_t s) {
    const unsigned g = (unsigned)((n + 255) / 256 < 2048 ? (n + 255) / 256 : 2048);
    k_balance<<<g, 256, 0, s>>>(canon, digits, p, ln, n, bad);
    return cudaGetLastError();
}

}  // namespace m2k
